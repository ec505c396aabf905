// host.hpp -- host-side pieces of the engine: config, geography, world build, the
// intervention triggers and the output listeners.  No CUDA in here.
#pragma once

#include <string>
#include <vector>

#include "epi_internal.h"

namespace epi {

// Config::read equivalent; throws std::runtime_error with a message on bad input.
epi_params params_from_json(const std::string& text);
// Range checks the engine needs (percentages in [0,1], sizes, hours); "" when fine.
std::string validate_params(const epi_params& p);

epi_geography define_geography(uint32_t grid_size);
void resize_hospital(epi_geography& g, int32_t number_of_agents, double staff_pct, double beds_pct);
epi_area grown_hospital(const epi_geography& initial);

epi_area house_area(const epi_geography& g, uint32_t k);
epi_area office_area(const epi_geography& g, uint32_t k);

// Epidemiology::new world build on the host (geography, population, starting infections,
// start points, hospital resize, essential workers).  Returns EPI_OK or an error code.
// flags (Csv population, bit 0 working, bit 1 public transport) replace the Auto draws.
int build_world(const epi_params& p, std::vector<epi_agent_record>& out, epi_geography& geo, std::string& err,
                const uint8_t* flags = nullptr);
int read_population_csv(const std::string& path, std::vector<uint8_t>& flags, std::string& err);

// Everything about a world build that is not per agent: the checks of generate_population
// and set_starting_infections, the Bernoulli thresholds, the public-transport budget of
// Area::random_points and the starting infections (agent index, state, infection day) in
// the order set_starting_infections assigns them.  build_world and the device build share it.
struct WorldPlan {
    epi_geography geo{};  // before resize_hospital
    uint32_t n = 0, houses = 0, offices = 0;
    uint64_t transport_points = 0;
    uint64_t thr_work = 0, thr_pt = 0, thr_staff = 0, thr_ess = 0;
    uint32_t key0 = 0, key1 = 0;
    struct Infection { uint32_t agent; uint8_t state; uint32_t day; };
    std::vector<Infection> infections;
    const uint8_t* flags = nullptr;  // Csv population flags (not owned)
};
int world_plan(const epi_params& p, WorldPlan& plan, std::string& err, const uint8_t* flags = nullptr);

struct Report {
    uint32_t hour;
    std::string name, data;
};

// State of LockdownIntervention / BuildNewHospital / VaccinateIntervention between hours.
struct InterventionState {
    bool locked = false;
    uint32_t zero_infection_hour = 0;
    uint32_t new_infections_in_a_day = 0;
    bool hospital_applied = false;
    std::vector<Report> reports;
};

struct InterventionActions {
    bool vaccinate = false;
    double vaccinate_percent = 0.0;
    bool lock = false, unlock = false, grow_hospital = false;
    uint32_t applied = 0;  // EPI_IV_* bits
};

// Trigger logic of process_interventions for this hour's counts (updates st and
// st.reports); the caller applies the returned bulk actions to the agents in the order
// vaccinate, lock, unlock, grow (allocation_map.rs:315-336).
InterventionActions decide_interventions(const epi_params& p, InterventionState& st, const epi_counts& c,
                                         const epi_area& hospital);

// Is this hour one at which an intervention can fire (a day boundary or a vaccination
// hour)?  The run loop calls decide_interventions at these hours.
bool is_event_hour(const epi_params& p, uint32_t hour);

// The first hour >= from at which an intervention fires whatever the counts are -- a
// vaccination hour, or the lifting of a lockdown in force -- or 0xFFFFFFFF.  The run loop's
// chains end there; the data-dependent triggers are watched on the device (GuardParams).
uint32_t next_fixed_event(const epi_params& p, const InterventionState& st, uint32_t from);

// The data-dependent triggers of decide_interventions still armed, for the device guard:
// lockdown when infected > lock_threshold; a new hospital when the day's new infections >=
// spread_threshold or hospitalized >= occ_threshold (the smallest count meeting the
// occupancy fraction of the current hospital's cells).
struct GuardParams {
    uint32_t flags = 0;  // bit 0 lockdown, bit 1 spread, bit 2 occupancy
    uint32_t lock_threshold = 0, spread_threshold = 0, occ_threshold = 0;
};
GuardParams guard_params(const epi_params& p, const InterventionState& st, const epi_area& hospital);

// CsvListener + InterventionReporter output files.
int write_outputs(const std::string& dir, const std::string& engine_id, const std::vector<epi_counts>& rows,
                  const std::vector<Report>& reports, std::string& err);

}  // namespace epi
