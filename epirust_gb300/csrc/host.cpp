// host.cpp -- config, geography, world build, intervention triggers and outputs.
#include "host.hpp"

#include <sys/stat.h>

#include <cerrno>
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <stdexcept>
#include <unordered_map>

#include "json.hpp"

namespace epi {

namespace {

const json::Value& need(const json::Value& obj, const char* key, const char* where) {
    const json::Value* v = obj.get(key);
    if (!v) throw std::runtime_error(std::string("missing field `") + key + "` in " + where);
    return *v;
}

uint32_t as_u32(const json::Value& v, const char* what) {
    unsigned long long x = v.as_uint();
    if (x > 0xFFFFFFFFull) throw std::runtime_error(std::string(what) + " does not fit u32");
    return (uint32_t)x;
}

}  // namespace

// Config (common/src/config/mod.rs:44-58) with Population::Auto, an inline Disease,
// GeographyParameters, hours, interventions and starting_infections (default: 1 exposed,
// common/src/config/starting_infections.rs:65-69).  Two optional keys that the reference
// ignores select the random stream ("seed") and the occupancy-triggered hospital build.
int read_population_csv(const std::string& path, std::vector<uint8_t>& flags, std::string& err) {
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) { err = "Could not read population file " + path; return EPI_ERR_IO; }
    std::string text;
    char buf[1 << 16];
    size_t got;
    while ((got = std::fread(buf, 1, sizeof buf, f)) > 0) text.append(buf, got);
    std::fclose(f);
    auto split = [](const std::string& line) {
        std::vector<std::string> out;
        size_t a = 0;
        while (true) {
            size_t b = line.find(',', a);
            std::string cell = line.substr(a, b == std::string::npos ? std::string::npos : b - a);
            while (!cell.empty() && (cell.back() == '\r' || cell.back() == ' ')) cell.pop_back();
            while (!cell.empty() && cell.front() == ' ') cell.erase(cell.begin());
            out.push_back(cell);
            if (b == std::string::npos) break;
            a = b + 1;
        }
        return out;
    };
    flags.clear();
    size_t pos = 0;
    int col_work = -1, col_pt = -1;
    size_t line_no = 0;
    while (pos < text.size()) {
        size_t end = text.find('\n', pos);
        if (end == std::string::npos) end = text.size();
        const std::string line = text.substr(pos, end - pos);
        pos = end + 1;
        ++line_no;
        if (line.find_first_not_of(" \r") == std::string::npos) continue;
        const std::vector<std::string> cells = split(line);
        if (col_work < 0) {  // the header row names the PopulationRecord fields
            for (size_t c = 0; c < cells.size(); ++c) {
                if (cells[c] == "working") col_work = (int)c;
                if (cells[c] == "pub_transport") col_pt = (int)c;
            }
            if (col_work < 0 || col_pt < 0) { err = path + ": the header needs the columns working and pub_transport"; return EPI_ERR_CONFIG; }
            continue;
        }
        auto boolean = [&](int c, uint8_t bit) -> int {
            if ((size_t)c >= cells.size()) return -1;
            if (cells[c] == "True") return bit;
            if (cells[c] == "False") return 0;
            return -1;
        };
        const int w = boolean(col_work, 1), t = boolean(col_pt, 2);
        if (w < 0 || t < 0) {
            err = path + ":" + std::to_string(line_no) + ": working and pub_transport must be True or False";
            return EPI_ERR_CONFIG;
        }
        flags.push_back((uint8_t)(w | t));
    }
    if (flags.empty()) { err = path + ": no citizens"; return EPI_ERR_CONFIG; }
    return EPI_OK;
}

epi_params params_from_json(const std::string& text) {
    json::Value root = json::parse(text);
    if (root.kind != json::Value::Object) throw std::runtime_error("config must be a JSON object");
    epi_params p;
    std::memset(&p, 0, sizeof p);

    const json::Value& pop = need(root, "population", "config");
    if (const json::Value* csv = pop.get("Csv")) {
        // Population::Csv{file, cols}: the agent count is the file's row count
        const json::Value& file = need(*csv, "file", "Csv");
        if (file.kind != json::Value::String || file.text.empty() || file.text.size() >= sizeof p.population_file)
            throw std::runtime_error("Csv.file must be a path shorter than 256 bytes");
        std::memcpy(p.population_file, file.text.c_str(), file.text.size() + 1);
        p.population_source = 1;
        std::vector<uint8_t> flags;
        std::string err;
        if (read_population_csv(file.text, flags, err)) throw std::runtime_error(err);
        p.number_of_agents = (uint32_t)flags.size();
    } else {
        const json::Value& autop = need(pop, "Auto", "population");
        p.number_of_agents = as_u32(need(autop, "number_of_agents", "Auto"), "number_of_agents");
        p.public_transport_percentage = need(autop, "public_transport_percentage", "Auto").as_double();
        p.working_percentage = need(autop, "working_percentage", "Auto").as_double();
    }

    const json::Value* dis = root.get("disease");
    if (!dis || dis->kind != json::Value::Object)
        throw std::runtime_error("config has no inline `disease` (Config::get_disease unwraps it)");
    p.regular_transmission_start_day = as_u32(need(*dis, "regular_transmission_start_day", "disease"), "day");
    p.high_transmission_start_day = as_u32(need(*dis, "high_transmission_start_day", "disease"), "day");
    p.last_day = as_u32(need(*dis, "last_day", "disease"), "day");
    p.asymptomatic_last_day = as_u32(need(*dis, "asymptomatic_last_day", "disease"), "day");
    p.mild_infected_last_day = as_u32(need(*dis, "mild_infected_last_day", "disease"), "day");
    p.regular_transmission_rate = need(*dis, "regular_transmission_rate", "disease").as_double();
    p.high_transmission_rate = need(*dis, "high_transmission_rate", "disease").as_double();
    p.death_rate = need(*dis, "death_rate", "disease").as_double();
    p.percentage_asymptomatic_population = need(*dis, "percentage_asymptomatic_population", "disease").as_double();
    p.percentage_severe_infected_population = need(*dis, "percentage_severe_infected_population", "disease").as_double();
    p.exposed_duration = as_u32(need(*dis, "exposed_duration", "disease"), "hours");
    p.pre_symptomatic_duration = as_u32(need(*dis, "pre_symptomatic_duration", "disease"), "hours");

    const json::Value& geo = need(root, "geography_parameters", "config");
    p.grid_size = as_u32(need(geo, "grid_size", "geography_parameters"), "grid_size");
    p.hospital_beds_percentage = need(geo, "hospital_beds_percentage", "geography_parameters").as_double();
    p.hours = as_u32(need(root, "hours", "config"), "hours");

    const json::Value& ivs = need(root, "interventions", "config");
    if (ivs.kind != json::Value::Array) throw std::runtime_error("`interventions` must be a list");
    for (const auto& iv : ivs.items) {
        if (iv.kind != json::Value::Object || iv.members.size() != 1)
            throw std::runtime_error("each intervention is an object with one variant key");
        const std::string& kind = iv.members[0].first;
        const json::Value& body = iv.members[0].second;
        if (kind == "Vaccinate") {
            if (p.n_vaccinations >= EPI_MAX_VACCINATIONS) throw std::runtime_error("too many Vaccinate entries");
            p.vaccination_at_hour[p.n_vaccinations] = as_u32(need(body, "at_hour", "Vaccinate"), "at_hour");
            p.vaccination_percent[p.n_vaccinations] = need(body, "percent", "Vaccinate").as_double();
            p.n_vaccinations++;
        } else if (kind == "Lockdown") {
            if (!p.has_lockdown) {  // the first entry is used (lockdown.rs:35-45)
                p.has_lockdown = 1;
                p.lockdown_at_number_of_infections = as_u32(need(body, "at_number_of_infections", "Lockdown"), "count");
                p.essential_workers_population = need(body, "essential_workers_population", "Lockdown").as_double();
            }
        } else if (kind == "BuildNewHospital") {
            if (!p.has_build_new_hospital) {  // hospital.rs:34-44
                p.has_build_new_hospital = 1;
                p.spread_rate_threshold = as_u32(need(body, "spread_rate_threshold", "BuildNewHospital"), "threshold");
            }
        } else {
            throw std::runtime_error("unknown intervention variant `" + kind + "`");
        }
    }

    const json::Value* si = root.get("starting_infections");
    if (si && si->kind == json::Value::Object) {
        p.infected_mild_asymptomatic = as_u32(need(*si, "infected_mild_asymptomatic", "starting_infections"), "count");
        p.infected_mild_symptomatic = as_u32(need(*si, "infected_mild_symptomatic", "starting_infections"), "count");
        p.infected_severe = as_u32(need(*si, "infected_severe", "starting_infections"), "count");
        p.exposed = as_u32(need(*si, "exposed", "starting_infections"), "count");
    } else {
        p.exposed = 1;
    }
    if (const json::Value* s = root.get("seed")) p.seed = s->as_uint();
    if (const json::Value* t = root.get("hospital_occupancy_trigger")) p.hospital_occupancy_trigger = t->as_double();
    return p;
}

std::string validate_params(const epi_params& p) {
    auto pct = [](double v) { return v >= 0.0 && v <= 1.0; };  // validate_percentage, custom_types.rs:29-35
    if (p.number_of_agents == 0) return "population is empty (No citizens!)";
    if (p.population_source > 1) return "population_source must be 0 (Auto) or 1 (Csv)";
    if (p.number_of_agents > kMaxAgentsPerWorld) return "number_of_agents must be <= 33554431 per world";
    if (p.grid_size < 1 || p.grid_size > kMaxGrid) return "grid_size must be in [1, 16382]";
    if (p.hours > kMaxHours) return "hours must be <= 1500000 (16-bit infection day on the device)";
    if (!pct(p.public_transport_percentage) || !pct(p.working_percentage)) return "population percentages must be in [0, 1]";
    if (!pct(p.hospital_beds_percentage)) return "hospital_beds_percentage must be in [0, 1]";
    if (!pct(p.regular_transmission_rate) || !pct(p.high_transmission_rate) || !pct(p.death_rate) ||
        !pct(p.percentage_asymptomatic_population) || !pct(p.percentage_severe_infected_population))
        return "disease percentages must be in [0, 1]";
    if (p.has_lockdown && !pct(p.essential_workers_population)) return "essential_workers_population must be in [0, 1]";
    for (int k = 0; k < p.n_vaccinations; ++k)
        if (!pct(p.vaccination_percent[k])) return "vaccination percent must be in [0, 1]";
    if (p.n_vaccinations < 0 || p.n_vaccinations > EPI_MAX_VACCINATIONS) return "bad vaccination count";
    if (p.exposed_duration > 0x7FFFFFFFu) return "exposed_duration too large";
    return "";
}

static epi_area mk(int32_t x0, int32_t y0, int32_t x1, int32_t y1) {
    epi_area a;
    a.x0 = x0; a.y0 = y0; a.x1 = x1; a.y1 = y1;
    return a;
}

// define_geography (engine/src/geography/mod.rs:33-70): four vertical strips of
// ceil(0.4G), ceil(0.2G), ceil(0.2G), ceil(0.1G) columns, each spanning rows 0..=G, and
// the 2x2 / 10x10 tilings of area_factory (area.rs:95-117).
epi_geography define_geography(uint32_t grid_size) {
    const double g = (double)grid_size;
    const int32_t G = (int32_t)grid_size;
    int32_t x_transport = (int32_t)std::ceil(g * 0.4);
    int32_t x_work = x_transport + (int32_t)std::ceil(g * 0.2);
    int32_t x_hospital = x_work + (int32_t)std::ceil(g * 0.2);
    int32_t x_end = x_hospital + (int32_t)std::ceil(g * 0.1);
    epi_geography geo;
    std::memset(&geo, 0, sizeof geo);
    geo.grid_size = grid_size;
    geo.housing = mk(0, 0, x_transport - 1, G);
    geo.transport = mk(x_transport, 0, x_work - 1, G);
    geo.work = mk(x_work, 0, x_hospital - 1, G);
    geo.hospital = mk(x_hospital, 0, x_end - 1, G);
    geo.houses_x = (uint32_t)((geo.housing.x1 - geo.housing.x0 + 1) / 2);
    geo.houses_y = (uint32_t)((geo.housing.y1 - geo.housing.y0 + 1) / 2);
    geo.offices_x = (uint32_t)((geo.work.x1 - geo.work.x0 + 1) / 10);
    geo.offices_y = (uint32_t)((geo.work.y1 - geo.work.y0 + 1) / 10);
    return geo;
}

// Grid::resize_hospital (grid.rs:240-261).  Its cell count omits the +1 of an inclusive
// rectangle; kept as is.
void resize_hospital(epi_geography& g, int32_t number_of_agents, double staff_pct, double beds_pct) {
    const double n = (double)number_of_agents;
    double beds_f = n * beds_pct;
    double staff_f = n * staff_pct;
    uint32_t beds = (uint32_t)std::ceil(beds_f + staff_f);
    int32_t width = g.hospital.x1 - g.hospital.x0;
    uint32_t cells = (uint32_t)(width * (g.hospital.y1 - g.hospital.y0));
    if (beds <= cells && width > 0) g.hospital.y1 = (int32_t)(beds / (uint32_t)width);
}

// Grid::increase_hospital_size (grid.rs:233-238).
epi_area grown_hospital(const epi_geography& g) {
    return mk(g.hospital.x0, g.hospital.y0, (int32_t)g.grid_size, (int32_t)g.grid_size);
}

epi_area house_area(const epi_geography& g, uint32_t k) {
    int32_t x = g.housing.x0 + 2 * (int32_t)(k % g.houses_x);
    int32_t y = g.housing.y0 + 2 * (int32_t)(k / g.houses_x);
    return mk(x, y, x + 1, y + 1);
}

epi_area office_area(const epi_geography& g, uint32_t k) {
    int32_t x = g.work.x0 + 10 * (int32_t)(k % g.offices_x);
    int32_t y = g.work.y0 + 10 * (int32_t)(k / g.offices_x);
    return mk(x, y, x + 9, y + 9);
}

namespace {

struct WorldDraws {
    uint32_t k0, k1;
    void at(uint32_t item, uint32_t block, uint32_t out[4]) const { philox4x32(item, kWorldHour, block, 0u, k0, k1, out); }
};

inline bool bern(uint32_t u, uint64_t thr) { return (uint64_t)u < thr; }

}  // namespace

// Population build of Epidemiology::new with counter-based draws per agent
// (engine/src/geography/grid.rs:83-155, engine/src/citizen/citizen_factory.rs:31-134,
// engine/src/epidemiology_simulation.rs:85-117 and 178-192):
//   - create_citizen for agent i: house i mod H, office i mod O, working ~ B(w),
//     public transport ~ B(pt) capped by the transport points, hospital staff ~ B(0.002)
//     among workers (work_start_at 8), immunity uniform in {-2..2};
//   - starting infections: the first `total` picks of a partial Fisher-Yates shuffle of
//     the agent indices become exposed (hour 0), then asymptomatic, mild, severe (day 1);
//   - start points: a house with one agent puts it on a random cell; with k >= 2 agents
//     the k-th (by index) takes the k-th cell of the x-major product of the house's two
//     columns and two rows (Area::random_points over a 2x2 house);
//   - resize_hospital(N, 0.002, beds), then Normal workers become Essential ~ B(ess).
int world_plan(const epi_params& p, WorldPlan& plan, std::string& err, const uint8_t* flags) {
    std::string bad = validate_params(p);
    if (!bad.empty()) { err = bad; return EPI_ERR_CONFIG; }
    plan.geo = define_geography(p.grid_size);
    const epi_geography& geo = plan.geo;
    const uint32_t n = p.number_of_agents;
    plan.n = n;
    plan.houses = geo.houses_x * geo.houses_y;
    plan.offices = geo.offices_x * geo.offices_y;
    if (plan.houses == 0 || plan.offices == 0) { err = "grid too small: no houses or no offices"; return EPI_ERR_CONFIG; }
    plan.flags = flags;
    if (flags && (uint64_t)n > 4ull * plan.houses) {  // read_population, grid.rs:216-223
        err = "Cannot accommodate citizens into homes! There are " + std::to_string(n) + " citizens, but " +
              std::to_string(4ull * plan.houses) + " home points";
        return EPI_ERR_CAPACITY;
    }
    const uint64_t per_house = ((uint64_t)n + plan.houses - 1) / plan.houses;
    if (per_house > 4) {
        err = "There are " + std::to_string(per_house) + " agents assigned to a house, but house capacity is 4";
        return EPI_ERR_CAPACITY;
    }
    const uint64_t infections = (uint64_t)p.exposed + p.infected_mild_asymptomatic + p.infected_mild_symptomatic + p.infected_severe;
    if (infections > n) {
        err = "There are " + std::to_string(infections) + " people set to infect, but only " + std::to_string(n) + " agents available";
        return EPI_ERR_CAPACITY;
    }
    plan.key0 = (uint32_t)p.seed;
    plan.key1 = (uint32_t)(p.seed >> 32);
    WorldDraws wd{plan.key0, plan.key1};

    // Number of transport points: min(n_pt, |xs| * |ys|) of Area::random_points.
    const double wanted = (double)n * (p.public_transport_percentage + 0.1) * (p.working_percentage + 0.1);
    const uint64_t n_points = (uint64_t)std::ceil(wanted);
    const uint64_t side = (uint64_t)std::ceil(std::sqrt((float)n_points));
    uint64_t cols = (uint64_t)(geo.transport.x1 - geo.transport.x0 + 1);
    uint64_t rows = (uint64_t)(geo.transport.y1 - geo.transport.y0 + 1);
    cols = cols < side ? cols : side;
    rows = rows < side ? rows : side;
    plan.transport_points = cols * rows < n_points ? cols * rows : n_points;

    plan.thr_work = bernoulli_threshold(p.working_percentage);
    plan.thr_pt = bernoulli_threshold(p.public_transport_percentage);
    plan.thr_staff = bernoulli_threshold(0.002);
    plan.thr_ess = bernoulli_threshold(p.has_lockdown ? p.essential_workers_population : 0.0);

    // set_starting_infections: choose_multiple as a partial Fisher-Yates shuffle of the agent
    // indices (only the touched positions are stored), then the exposed, asymptomatic, mild
    // and severe agents in that order
    plan.infections.clear();
    if (infections) {
        std::unordered_map<uint32_t, uint32_t> moved;  // position -> agent, where not the identity
        auto at = [&](uint32_t k) { auto it = moved.find(k); return it == moved.end() ? k : it->second; };
        std::vector<uint32_t> picked((size_t)infections);
        for (uint32_t j = 0; j < (uint32_t)infections; ++j) {
            uint32_t u[4];
            wd.at(j, kBlkInfectPick, u);
            const uint32_t r = j + uniform_index(u[0], n - j);
            const uint32_t aj = at(j), ar = at(r);
            moved[j] = ar;
            moved[r] = aj;
            picked[j] = ar;
        }
        uint32_t j = 0;
        auto set = [&](uint32_t count, uint8_t state, uint32_t day) {
            for (uint32_t k = 0; k < count; ++k, ++j) plan.infections.push_back({picked[j], state, day});
        };
        set(p.exposed, EPI_E, 0);
        set(p.infected_mild_asymptomatic, EPI_I_ASYM, 1);
        set(p.infected_mild_symptomatic, EPI_I_MILD, 1);
        set(p.infected_severe, EPI_I_SEVERE, 1);
    }
    return EPI_OK;
}

int build_world(const epi_params& p, std::vector<epi_agent_record>& out, epi_geography& geo, std::string& err,
                const uint8_t* flags) {
    WorldPlan plan;
    int rc = world_plan(p, plan, err, flags);
    if (rc) return rc;
    geo = plan.geo;
    const uint32_t n = plan.n, houses = plan.houses, offices = plan.offices;
    WorldDraws wd{plan.key0, plan.key1};
    out.assign(n, epi_agent_record());
    uint64_t pt_users = 0;
    for (uint32_t i = 0; i < n; ++i) {
        uint32_t u[4];
        wd.at(i, kBlkCitizen, u);
        epi_agent_record& r = out[i];
        std::memset(&r, 0, sizeof r);
        const bool working = flags ? (flags[i] & 1u) != 0 : bern(u[0], plan.thr_work);
        const epi_area h = house_area(geo, i % houses);
        const epi_area o = office_area(geo, i % offices);
        bool pt;
        if (flags) {
            pt = (flags[i] & 2u) != 0;  // PopulationRecord::pub_transport as given
        } else {
            pt = bern(u[1], plan.thr_pt) && working && pt_users < plan.transport_points;
            if (pt) ++pt_users;
        }
        r.flags = pt ? EPI_F_PUBLIC_TRANSPORT : 0;
        r.home_x = h.x0; r.home_y = h.y0;
        if (working) {
            r.work_x = o.x0; r.work_y = o.y0;
            if (bern(u[2], plan.thr_staff)) { r.work_status = EPI_WS_HOSPITAL_STAFF; r.work_start_at = 8; }
            else r.work_status = EPI_WS_NORMAL;
        } else {
            // Auto: create_citizen keeps the house; Csv: from_record keeps the cycled office
            r.work_x = flags ? o.x0 : h.x0;
            r.work_y = flags ? o.y0 : h.y0;
            r.work_status = EPI_WS_NA;
        }
        r.immunity = (int8_t)((int32_t)uniform_index(u[3], 5u) - 2);
        r.state = EPI_S;
        r.area_x0 = h.x0; r.area_y0 = h.y0; r.area_x1 = h.x1; r.area_y1 = h.y1;
    }
    for (const auto& inf : plan.infections) {
        out[inf.agent].state = inf.state;
        out[inf.agent].infection_day = inf.day;
        out[inf.agent].at_hour = 0;
    }
    for (uint32_t i = 0; i < n; ++i) {
        const uint32_t house = i % houses, rank = i / houses;
        const uint32_t in_house = (n - 1 - house) / houses + 1;
        epi_agent_record& r = out[i];
        if (in_house == 1) {
            uint32_t u[4];
            wd.at(house, kBlkHouse, u);
            r.x = r.home_x + (int32_t)uniform_index(u[0], 2u);
            r.y = r.home_y + (int32_t)uniform_index(u[1], 2u);
        } else {
            r.x = r.home_x + (int32_t)(rank >> 1);
            r.y = r.home_y + (int32_t)(rank & 1u);
        }
    }
    resize_hospital(geo, (int32_t)n, 0.002, p.hospital_beds_percentage);
    for (uint32_t i = 0; i < n; ++i) {
        if (out[i].work_status != EPI_WS_NORMAL) continue;
        uint32_t u[4];
        wd.at(i, kBlkEssential, u);
        if (bern(u[0], plan.thr_ess)) out[i].work_status = EPI_WS_ESSENTIAL;
    }
    return EPI_OK;
}

bool is_event_hour(const epi_params& p, uint32_t hour) {
    if (hour % 24u == 0) return true;
    for (int k = 0; k < p.n_vaccinations; ++k)
        if (p.vaccination_at_hour[k] == hour) return true;
    return false;
}

uint32_t next_fixed_event(const epi_params& p, const InterventionState& st, uint32_t from) {
    uint32_t e = 0xFFFFFFFFu;
    for (int k = 0; k < p.n_vaccinations; ++k)
        if (p.vaccination_at_hour[k] >= from) e = std::min(e, p.vaccination_at_hour[k]);
    const uint64_t lift = (uint64_t)st.zero_infection_hour + 21u * 24u;  // decide_interventions' unlock hour
    if (st.locked && lift >= from && lift < e) e = (uint32_t)lift;
    return e;
}

GuardParams guard_params(const epi_params& p, const InterventionState& st, const epi_area& hospital) {
    GuardParams g;
    if (p.has_lockdown && !st.locked) {
        g.flags |= 1u;
        g.lock_threshold = p.lockdown_at_number_of_infections;
    }
    if (!st.hospital_applied) {
        if (p.has_build_new_hospital) {
            g.flags |= 2u;
            g.spread_threshold = p.spread_rate_threshold;
        }
        if (p.hospital_occupancy_trigger > 0.0) {
            // the same double product as decide_interventions; hospitalized >= x <=> >= ceil(x)
            const double cells = (double)(hospital.x1 - hospital.x0 + 1) * (double)(hospital.y1 - hospital.y0 + 1);
            const double x = std::ceil(p.hospital_occupancy_trigger * cells);
            if (x <= 4294967295.0) {
                g.flags |= 4u;
                g.occ_threshold = (uint32_t)std::max(x, 0.0);
            }
        }
    }
    return g;
}

// process_interventions triggers (engine/src/allocation_map.rs:306-337):
// VaccinateIntervention::get_vaccination_percentage (vaccination.rs:52-54; last entry of an
// hour wins like the HashMap insert), LockdownIntervention::should_apply / should_unlock
// (lockdown.rs:55-73; zero_infection_hour stays 0 in standalone mode, so a lockdown lifts at
// hour 504 exactly), BuildNewHospital::counts_updated / should_apply (hospital.rs:51-74), and
// the occupancy extension.
InterventionActions decide_interventions(const epi_params& p, InterventionState& st, const epi_counts& c,
                                         const epi_area& hospital) {
    InterventionActions a;
    const uint32_t hour = c.hour;
    int vi = -1;
    for (int k = 0; k < p.n_vaccinations; ++k)
        if (p.vaccination_at_hour[k] == hour) vi = k;
    if (vi >= 0) {
        a.vaccinate = true;
        a.vaccinate_percent = p.vaccination_percent[vi];
        a.applied |= EPI_IV_VACCINATION;
        st.reports.push_back({hour, "vaccination", "{}"});
    }
    if (!st.locked && hour % 24u == 0 && p.has_lockdown && c.infected > p.lockdown_at_number_of_infections) {
        st.locked = true;
        a.lock = true;
        a.applied |= EPI_IV_LOCKDOWN;
        st.reports.push_back({hour, "lockdown", "{\"status\":\"locked_down\"}"});
    }
    if (st.locked && hour == st.zero_infection_hour + 21u * 24u) {
        st.locked = false;
        st.zero_infection_hour = 0;
        a.unlock = true;
        a.applied |= EPI_IV_LOCKDOWN_REVOKED;
        st.reports.push_back({hour, "lockdown", "{\"status\":\"lockdown_revoked\"}"});
    }
    if (hour % 24u == 0)
        st.new_infections_in_a_day = c.infected > st.new_infections_in_a_day ? c.infected - st.new_infections_in_a_day : 0u;
    if (!st.hospital_applied && hour % 24u == 0) {
        bool grow = p.has_build_new_hospital && st.new_infections_in_a_day >= p.spread_rate_threshold;
        if (p.hospital_occupancy_trigger > 0.0) {
            double cells = (double)(hospital.x1 - hospital.x0 + 1) * (double)(hospital.y1 - hospital.y0 + 1);
            if ((double)c.hospitalized >= p.hospital_occupancy_trigger * cells) grow = true;
        }
        if (grow) {
            st.hospital_applied = true;
            a.grow_hospital = true;
            a.applied |= EPI_IV_BUILD_NEW_HOSPITAL;
            st.reports.push_back({hour, "build_new_hospital", "{}"});
        }
    }
    return a;
}

// <dir>/output/simulation_<id>_<UTC YYYY-MM-DDTHH:MM:SS>.csv and ..._interventions.json
// (engine/src/utils/util.rs:28-43, csv_service.rs:44-71, intervention_reporter.rs:52-58).
int write_outputs(const std::string& dir, const std::string& engine_id, const std::vector<epi_counts>& rows,
                  const std::vector<Report>& reports, std::string& err) {
    std::string out_dir = dir + "/output";
    if (mkdir(out_dir.c_str(), 0755) != 0 && errno != EEXIST) {
        err = "cannot create " + out_dir;
        return EPI_ERR_IO;
    }
    char stamp[32];
    std::time_t now = std::time(nullptr);
    std::tm tm_utc;
    gmtime_r(&now, &tm_utc);
    std::strftime(stamp, sizeof stamp, "%Y-%m-%dT%H:%M:%S", &tm_utc);
    std::string base = out_dir + "/simulation_" + engine_id + "_" + stamp;
    FILE* f = std::fopen((base + ".csv").c_str(), "w");
    if (!f) { err = "cannot write " + base + ".csv"; return EPI_ERR_IO; }
    std::fprintf(f, "hour,susceptible,exposed,infected,hospitalized,recovered,deceased\n");
    for (const auto& r : rows)
        std::fprintf(f, "%u,%u,%u,%u,%u,%u,%u\n", r.hour, r.susceptible, r.exposed, r.infected, r.hospitalized,
                     r.recovered, r.deceased);
    std::fclose(f);
    f = std::fopen((base + "_interventions.json").c_str(), "w");
    if (!f) { err = "cannot write " + base + "_interventions.json"; return EPI_ERR_IO; }
    std::fprintf(f, "[");
    for (size_t k = 0; k < reports.size(); ++k)
        std::fprintf(f, "%s{\"hour\":%u,\"intervention\":\"%s\",\"data\":%s}", k ? "," : "", reports[k].hour,
                     reports[k].name.c_str(), reports[k].data.c_str());
    std::fprintf(f, "]");
    std::fclose(f);
    return EPI_OK;
}

}  // namespace epi
