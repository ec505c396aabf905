/*
 * oracle/o1.c -- TEST INFRASTRUCTURE ONLY.  Nothing in the product links, loads or calls
 * this file; tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it as the
 * checker.
 *
 * O1: the bit-exact scalar oracle.  A single-threaded C restatement of the EpiRust
 * single-engine tick (thoughtworks/epirust) -- rules in o_rules.h, one function per
 * reference function -- with two deliberate, documented substitutions:
 *   1. the Philox draw slots of o_common.h replace the unseeded thread_rng;
 *   2. the serial conflict resolve of allocation_map.rs:93-102 runs in agent-index order
 *      (the reference runs it in hash-map iteration order), so the lowest index wins a
 *      contested cell.
 * The previous-hour map is a dense (G+1)^2 array of agent indices (-1 = vacant); the
 * reference's FnvHashMap<Point, Citizen> answers the same two queries.  Agents are indexed
 * in creation order.  The world build restates Epidemiology::new with the same draw slots.
 */
#include <stdlib.h>

#include "o_common.h"

typedef struct {
    const int32_t* occ;    /* agent index per cell, -1 vacant */
    const citizen* agents; /* previous-hour agents */
    int32_t W;
} dense_map;

#define SNAP_T dense_map
static inline int32_t dense_index(const dense_map* m, pt p) {
    if (p.x < 0 || p.y < 0 || p.x >= m->W || p.y >= m->W) abort(); /* rules never leave [0,G]^2 */
    return p.y * m->W + p.x;
}
static inline int snap_vacant(const dense_map* m, pt p) { return m->occ[dense_index(m, p)] < 0; }
static inline const citizen* snap_get(const dense_map* m, pt p) {
    int32_t j = m->occ[dense_index(m, p)];
    return j < 0 ? NULL : &m->agents[j];
}
#include "o_rules.h"

typedef struct o1_sim {
    o_world w;
    uint32_t n;
    citizen *cur, *nxt;
    pt *pos, *npos, *tgt;
    int32_t *occ, *upc;
    o_iv_state iv;
    o_report* reports;
    uint32_t n_reports, cap_reports;
} o1_sim;

static int32_t cidx(const o1_sim* s, pt p) {
    if (p.x < 0 || p.y < 0 || p.x >= s->w.W || p.y >= s->w.W) abort();
    return p.y * s->w.W + p.x;
}

/* CitizenLocationMap::simulate, allocation_map.rs:67-129 (no travel, no citizen-state
 * listener): the map phase over the previous-hour map, then the serial first-come resolve
 * (here in index order), counts, and the swap. */
int o1_simulate(o1_sim* s, uint32_t hour, uint32_t out_counts[6]) {
    dense_map m = {s->occ, s->cur, s->w.W};
    uint32_t cnt[6] = {0, 0, 0, 0, 0, 0};
    for (uint32_t i = 0; i < s->n; ++i) {
        draws d;
        draws_init(&d, &s->w, i, hour);
        s->nxt[i] = s->cur[i];
        s->tgt[i] = routine(&s->w, &m, &s->nxt[i], s->pos[i], hour, &d);
    }
    for (uint32_t i = 0; i < s->n; ++i) {
        pt old_cell = s->pos[i], new_cell = s->tgt[i];
        int32_t ni = cidx(s, new_cell);
        if (s->upc[ni] < 0) {
            s->upc[ni] = (int32_t)i;
            s->npos[i] = new_cell;
        } else {
            s->upc[cidx(s, old_cell)] = (int32_t)i;
            s->npos[i] = old_cell;
        }
        count_agent(cnt, &s->nxt[i]);
    }
    for (uint32_t i = 0; i < s->n; ++i) s->occ[cidx(s, s->pos[i])] = -1;
    int32_t* t = s->occ; s->occ = s->upc; s->upc = t;
    citizen* tc = s->cur; s->cur = s->nxt; s->nxt = tc;
    pt* tp = s->pos; s->pos = s->npos; s->npos = tp;
    uint32_t total = 0;
    for (int k = 0; k < 6; ++k) total += cnt[k];
    if (out_counts) memcpy(out_counts, cnt, sizeof cnt);
    return total == s->n ? EPI_OK : EPI_ERR_INVARIANT; /* assert, allocation_map.rs:128 */
}

/* ---------------------------------------------------------------- interventions */
static void add_report(o1_sim* s, uint32_t hour, const char* name, const char* data) {
    if (s->n_reports == s->cap_reports) {
        s->cap_reports = s->cap_reports ? 2 * s->cap_reports : 16;
        s->reports = (o_report*)realloc(s->reports, s->cap_reports * sizeof(o_report));
    }
    o_report* r = &s->reports[s->n_reports++];
    r->hour = hour;
    strncpy(r->name, name, sizeof r->name - 1); r->name[sizeof r->name - 1] = 0;
    strncpy(r->data, data, sizeof r->data - 1); r->data[sizeof r->data - 1] = 0;
}

/* allocation_map.rs:349-356 */
void o1_lock_city(o1_sim* s) {
    for (uint32_t i = 0; i < s->n; ++i) if (s->cur[i].ws != EPI_WS_ESSENTIAL) s->cur[i].isolated = 1;
}
/* allocation_map.rs:358-365 */
void o1_unlock_city(o1_sim* s) {
    for (uint32_t i = 0; i < s->n; ++i) if (s->cur[i].isolated) s->cur[i].isolated = 0;
}
/* allocation_map.rs:381-387 */
void o1_vaccinate(o1_sim* s, uint32_t hour, double percent) {
    for (uint32_t i = 0; i < s->n; ++i) {
        if (s->cur[i].state != EPI_S) continue;
        uint32_t u[4];
        draw4(&s->w, i, hour, 3u, u);
        if (bern(u[0], percent)) s->cur[i].vaccinated = 1;
    }
}
void o1_increase_hospital_size(o1_sim* s) { o_increase_hospital_size(&s->w); }

/* CitizenLocationMap::process_interventions, allocation_map.rs:306-337. */
uint32_t o1_process_interventions(o1_sim* s, uint32_t hour, const uint32_t c[6]) {
    o_iv_actions a = o_decide_interventions(&s->w, &s->iv, hour, c);
    if (a.vaccinate) { o1_vaccinate(s, hour, a.percent); add_report(s, hour, "vaccination", "{}"); }
    if (a.lock) { o1_lock_city(s); add_report(s, hour, "lockdown", "{\"status\":\"locked_down\"}"); }
    if (a.unlock) { o1_unlock_city(s); add_report(s, hour, "lockdown", "{\"status\":\"lockdown_revoked\"}"); }
    if (a.grow) { o1_increase_hospital_size(s); add_report(s, hour, "build_new_hospital", "{}"); }
    return a.applied;
}

/* ---------------------------------------------------------------- world build */
static area house(const o_world* w, uint32_t k) {
    int32_t x = w->housing.s.x + 2 * (int32_t)(k % w->hfx), y = w->housing.s.y + 2 * (int32_t)(k / w->hfx);
    return mk_area(x, y, x + 1, y + 1);
}
static area office(const o_world* w, uint32_t k) {
    int32_t x = w->work_area.s.x + 10 * (int32_t)(k % w->ofx), y = w->work_area.s.y + 10 * (int32_t)(k / w->ofx);
    return mk_area(x, y, x + 9, y + 9);
}

static int alloc_state(o1_sim* s) {
    size_t cells = (size_t)s->w.W * (size_t)s->w.W, n = s->n ? s->n : 1;
    s->cur = (citizen*)calloc(n, sizeof(citizen));
    s->nxt = (citizen*)calloc(n, sizeof(citizen));
    s->pos = (pt*)calloc(n, sizeof(pt));
    s->npos = (pt*)calloc(n, sizeof(pt));
    s->tgt = (pt*)calloc(n, sizeof(pt));
    s->occ = (int32_t*)malloc(cells * sizeof(int32_t));
    s->upc = (int32_t*)malloc(cells * sizeof(int32_t));
    if (!s->cur || !s->nxt || !s->pos || !s->npos || !s->tgt || !s->occ || !s->upc) return EPI_ERR_CAPACITY;
    memset(s->occ, 0xff, cells * sizeof(int32_t));
    memset(s->upc, 0xff, cells * sizeof(int32_t));
    return EPI_OK;
}

static int place_agents(o1_sim* s) {
    for (uint32_t i = 0; i < s->n; ++i) {
        pt q = s->pos[i];
        if (q.x < 0 || q.y < 0 || q.x >= s->w.W || q.y >= s->w.W) return EPI_ERR_ARG;
        int32_t ci = cidx(s, q);
        if (s->occ[ci] >= 0) return EPI_ERR_ARG;
        s->occ[ci] = (int32_t)i;
    }
    return EPI_OK;
}

/* Grid::generate_population + citizen_factory + set_starting_infections +
 * set_start_locations_and_occupancies + resize_hospital + init_interventions:
 * grid.rs:83-155, citizen_factory.rs:31-134, epidemiology_simulation.rs:85-117, 178-192. */
static int build_world(o1_sim* s) {
    const o_world* w = &s->w;
    const epi_params* p = &w->p;
    uint32_t n = s->n;
    uint32_t n_houses = w->hfx * w->hfy, n_offices = w->ofx * w->ofy;
    if (n_houses == 0 || n_offices == 0) return EPI_ERR_CONFIG;
    if ((n + n_houses - 1) / n_houses > 4u) return EPI_ERR_CAPACITY; /* grid.rs:140-142 */
    /* transport_area.random_points(ceil(N (pt+0.1)(w+0.1))): only its length matters to the
     * tick (transport_location is never read by the standalone routine). area.rs:64-74 */
    double want = (double)n * (p->public_transport_percentage + 0.1) * (p->working_percentage + 0.1);
    uint64_t n_pt = (uint64_t)ceil(want);
    uint64_t nx = (uint64_t)ceilf(sqrtf((float)n_pt));
    uint64_t xs = (uint64_t)(w->transport.e.x - w->transport.s.x + 1);
    uint64_t ys = (uint64_t)(w->transport.e.y - w->transport.s.y + 1);
    if (xs > nx) xs = nx;
    if (ys > nx) ys = nx;
    uint64_t n_tl = xs * ys < n_pt ? xs * ys : n_pt;
    uint64_t cur_pt = 0;
    for (uint32_t i = 0; i < n; ++i) { /* create_citizen, citizen_factory.rs:58-88 */
        citizen* c = &s->cur[i];
        uint32_t u[4];
        draw4(w, i, WB_HOUR, 16u, u);
        int working = bern(u[0], p->working_percentage);
        c->id = i;
        c->home = house(w, i % n_houses);
        area wk = office(w, i % n_offices);
        int upt = bern(u[1], p->public_transport_percentage) && working && cur_pt < n_tl;
        if (upt) cur_pt++;
        c->uses_pt = (uint8_t)upt;
        c->work = working ? wk : c->home;
        if (working) { /* derive_work_status, citizen/mod.rs:442-450 */
            if (bern(u[2], 0.002)) { c->ws = EPI_WS_HOSPITAL_STAFF; c->work_start_at = 8u; }
            else c->ws = EPI_WS_NORMAL;
        } else c->ws = EPI_WS_NA;
        c->immunity = (int32_t)pick(u[3], 5u) - 2; /* IMMUNITY_RANGE */
        c->state = EPI_S;
        c->current = c->home;
    }
    /* set_starting_infections: choose_multiple, then exposed / asym / mild / severe in order */
    uint64_t total = (uint64_t)p->exposed + p->infected_mild_asymptomatic + p->infected_mild_symptomatic +
                     p->infected_severe;
    if (total > n) return EPI_ERR_CAPACITY;
    if (total) {
        uint32_t* idx = (uint32_t*)malloc((size_t)n * sizeof(uint32_t));
        for (uint32_t i = 0; i < n; ++i) idx[i] = i;
        for (uint32_t j = 0; j < (uint32_t)total; ++j) {
            uint32_t u[4];
            draw4(w, j, WB_HOUR, 19u, u);
            uint32_t r = j + pick(u[0], n - j);
            uint32_t t = idx[j]; idx[j] = idx[r]; idx[r] = t;
        }
        uint32_t j = 0;
        for (uint32_t k = 0; k < p->exposed; ++k, ++j) { s->cur[idx[j]].state = EPI_E; s->cur[idx[j]].at_hour = 0; }
        for (uint32_t k = 0; k < p->infected_mild_asymptomatic; ++k, ++j) { s->cur[idx[j]].state = EPI_I_ASYM; s->cur[idx[j]].day = 1; }
        for (uint32_t k = 0; k < p->infected_mild_symptomatic; ++k, ++j) { s->cur[idx[j]].state = EPI_I_MILD; s->cur[idx[j]].day = 1; }
        for (uint32_t k = 0; k < p->infected_severe; ++k, ++j) { s->cur[idx[j]].state = EPI_I_SEVERE; s->cur[idx[j]].day = 1; }
        free(idx);
    }
    /* start points: house h holds agents h, h+H, h+2H, ... in index order and takes
     * home.random_points(k) (area.rs:64-74): one agent -> a random cell; k >= 2 ->
     * choose_multiple of 2 out of 2 values keeps both in order, so the x-major product. */
    for (uint32_t i = 0; i < n; ++i) {
        uint32_t h = i % n_houses, rank = i / n_houses;
        uint32_t k = (n - 1 - h) / n_houses + 1;
        area ha = s->cur[i].home;
        pt q;
        if (k == 1) {
            uint32_t u[4];
            draw4(w, h, WB_HOUR, 18u, u);
            q.x = ha.s.x + (int32_t)pick(u[0], 2u);
            q.y = ha.s.y + (int32_t)pick(u[1], 2u);
        } else {
            q.x = ha.s.x + (int32_t)(rank / 2u);
            q.y = ha.s.y + (int32_t)(rank % 2u);
        }
        s->pos[i] = q;
    }
    o_resize_hospital(&s->w, (int32_t)n, 0.002, p->hospital_beds_percentage);
    /* init_interventions: assign_essential_worker, citizen/mod.rs:434-440 */
    double ess = p->has_lockdown ? p->essential_workers_population : 0.0;
    for (uint32_t i = 0; i < n; ++i) {
        if (s->cur[i].ws != EPI_WS_NORMAL) continue;
        uint32_t u[4];
        draw4(w, i, WB_HOUR, 17u, u);
        if (bern(u[0], ess)) s->cur[i].ws = EPI_WS_ESSENTIAL;
    }
    return place_agents(s);
}

/* ---------------------------------------------------------------- exported API */
void o1_free(o1_sim* s) {
    if (!s) return;
    free(s->cur); free(s->nxt); free(s->pos); free(s->npos); free(s->tgt); free(s->occ); free(s->upc);
    free(s->reports);
    free(s);
}

static o1_sim* o1_new(const epi_params* p, int* status) {
    o1_sim* s = (o1_sim*)calloc(1, sizeof(o1_sim));
    *status = o_world_init(&s->w, p);
    s->n = p->number_of_agents;
    if (*status) return s;
    if (p->hours > 1500000u) { *status = EPI_ERR_CONFIG; return s; }
    *status = alloc_state(s);
    return s;
}

o1_sim* o1_create(const epi_params* p, int* status) {
    o1_sim* s = o1_new(p, status);
    if (*status == EPI_OK) *status = build_world(s);
    return s;
}

void o_import_citizen(const epi_agent_record* r, uint32_t id, citizen* c, pt* pos) {
    memset(c, 0, sizeof *c);
    c->id = id;
    pos->x = r->x; pos->y = r->y;
    c->state = r->state;
    c->at_hour = r->at_hour;
    c->day = r->infection_day;
    c->immunity = r->immunity;
    c->hospitalized = (r->flags & EPI_F_HOSPITALIZED) != 0;
    c->isolated = (r->flags & EPI_F_ISOLATED) != 0;
    c->vaccinated = (r->flags & EPI_F_VACCINATED) != 0;
    c->work_quarantined = (r->flags & EPI_F_WORK_QUARANTINED) != 0;
    c->uses_pt = (r->flags & EPI_F_PUBLIC_TRANSPORT) != 0;
    c->ws = r->work_status;
    c->work_start_at = r->work_start_at;
    c->home = mk_area(r->home_x, r->home_y, r->home_x + 1, r->home_y + 1);
    /* a non-worker keeps the work area it was built with: its house (Auto, create_citizen)
       or the cycled office (Csv, Citizen::from_record) */
    c->work = (c->ws == EPI_WS_NA && r->work_x == r->home_x && r->work_y == r->home_y)
                  ? c->home
                  : mk_area(r->work_x, r->work_y, r->work_x + 9, r->work_y + 9);
    c->current = mk_area(r->area_x0, r->area_y0, r->area_x1, r->area_y1);
}

/* Start from given records (e.g. the product's world) with the initial geography. */
o1_sim* o1_create_from_records(const epi_params* p, const epi_agent_record* recs, uint32_t n, int* status) {
    epi_params q = *p;
    q.number_of_agents = n;
    o1_sim* s = o1_new(&q, status);
    if (*status) return s;
    o_resize_hospital(&s->w, (int32_t)n, 0.002, p->hospital_beds_percentage);
    for (uint32_t i = 0; i < n; ++i) o_import_citizen(&recs[i], i, &s->cur[i], &s->pos[i]);
    *status = place_agents(s);
    return s;
}

void o_export_citizen(const citizen* c, pt pos, epi_agent_record* r) {
    memset(r, 0, sizeof *r);
    r->x = pos.x; r->y = pos.y;
    r->state = c->state;
    r->flags = (uint8_t)((c->hospitalized ? EPI_F_HOSPITALIZED : 0) | (c->isolated ? EPI_F_ISOLATED : 0) |
                         (c->vaccinated ? EPI_F_VACCINATED : 0) | (c->work_quarantined ? EPI_F_WORK_QUARANTINED : 0) |
                         (c->uses_pt ? EPI_F_PUBLIC_TRANSPORT : 0));
    r->work_status = c->ws;
    r->immunity = (int8_t)c->immunity;
    r->at_hour = (c->state == EPI_E || c->state == EPI_I_PRE) ? c->at_hour : 0;
    r->infection_day = is_infected(c) ? c->day : 0;
    r->work_start_at = c->ws == EPI_WS_HOSPITAL_STAFF ? c->work_start_at : 0;
    r->home_x = c->home.s.x; r->home_y = c->home.s.y;
    r->work_x = c->work.s.x; r->work_y = c->work.s.y;
    r->area_x0 = c->current.s.x; r->area_y0 = c->current.s.y;
    r->area_x1 = c->current.e.x; r->area_y1 = c->current.e.y;
}

void o1_export(const o1_sim* s, epi_agent_record* out) {
    for (uint32_t i = 0; i < s->n; ++i) o_export_citizen(&s->cur[i], s->pos[i], &out[i]);
}

void o_world_geography(const o_world* w, epi_geography* g) {
    g->grid_size = (uint32_t)w->G;
    g->housing.x0 = w->housing.s.x; g->housing.y0 = w->housing.s.y; g->housing.x1 = w->housing.e.x; g->housing.y1 = w->housing.e.y;
    g->transport.x0 = w->transport.s.x; g->transport.y0 = w->transport.s.y; g->transport.x1 = w->transport.e.x; g->transport.y1 = w->transport.e.y;
    g->work.x0 = w->work_area.s.x; g->work.y0 = w->work_area.s.y; g->work.x1 = w->work_area.e.x; g->work.y1 = w->work_area.e.y;
    g->hospital.x0 = w->hospital.s.x; g->hospital.y0 = w->hospital.s.y; g->hospital.x1 = w->hospital.e.x; g->hospital.y1 = w->hospital.e.y;
    g->houses_x = w->hfx; g->houses_y = w->hfy; g->offices_x = w->ofx; g->offices_y = w->ofy;
}

void o1_geography(const o1_sim* s, epi_geography* g) { o_world_geography(&s->w, g); }
uint32_t o1_population(const o1_sim* s) { return s->n; }

/* Epidemiology::run_single_engine, epidemiology_simulation.rs:211-274, with the standalone
 * stop rule stop_simulation (564-575).  rows: 7 u32 per hour (hour,S,E,I,H,R,D). */
int o1_run(o1_sim* s, uint32_t first_hour, uint32_t last_hour_excl, uint32_t* rows, uint32_t* n_rows,
           int with_interventions, int with_stop) {
    uint32_t k = 0;
    for (uint32_t hour = first_hour; hour < last_hour_excl; ++hour) {
        uint32_t c[6];
        int st = o1_simulate(s, hour, c);
        if (st) { *n_rows = k; return st; }
        rows[7 * k] = hour;
        memcpy(&rows[7 * k + 1], c, sizeof c);
        ++k;
        if (with_interventions) o1_process_interventions(s, hour, c);
        if (with_stop && c[1] == 0 && c[2] == 0 && c[3] == 0) break;
    }
    *n_rows = k;
    return EPI_OK;
}

uint32_t o1_n_reports(const o1_sim* s) { return s->n_reports; }
void o1_report(const o1_sim* s, uint32_t k, uint32_t* hour, char* name, char* data) {
    *hour = s->reports[k].hour;
    strcpy(name, s->reports[k].name);
    strcpy(data, s->reports[k].data);
}

/* Building blocks that the reference pins with known-answer tests. */
double o1_transmission_rate(const epi_params* p, uint32_t day) { return transmission_rate(p, day); }
int o1_is_to_be_hospitalized(const epi_params* p, uint32_t day) {
    return transmission_rate(p, day) >= p->high_transmission_rate;
}
void o1_define_geography(uint32_t G, epi_geography* g) {
    o_world w; memset(&w, 0, sizeof w);
    w.G = (int32_t)G; w.W = w.G + 1;
    o_define_geography(&w);
    o_world_geography(&w, g);
}
void o1_resize_hospital(epi_geography* g, int32_t n, double staff, double beds) {
    o_world w; memset(&w, 0, sizeof w);
    w.G = (int32_t)g->grid_size;
    w.hospital = mk_area(g->hospital.x0, g->hospital.y0, g->hospital.x1, g->hospital.y1);
    o_resize_hospital(&w, n, staff, beds);
    g->hospital.x0 = w.hospital.s.x; g->hospital.y0 = w.hospital.s.y;
    g->hospital.x1 = w.hospital.e.x; g->hospital.y1 = w.hospital.e.y;
}
/* Grid::increase_hospital_size(grid_size), grid.rs:233-238 */
void o1_geography_increase_hospital_size(epi_geography* g, uint32_t grid_size) {
    g->hospital.x1 = (int32_t)grid_size;
    g->hospital.y1 = (int32_t)grid_size;
}
void o1_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) { orc_philox4x32_10(ctr, key, out); }
void o1_philox2x32(const uint32_t ctr[2], uint32_t key, uint32_t out[2]) { orc_philox2x32_10(ctr, key, out); }
/* Area::get_neighbors_of, area.rs:56-58 */
void o1_area_neighbors(int32_t x0, int32_t y0, int32_t x1, int32_t y1, int32_t px, int32_t py, int32_t* out, uint32_t* n) {
    area a = mk_area(x0, y0, x1, y1);
    *n = 0;
    for (int i = 0; i < 8; ++i) {
        pt q; q.x = px + NB_DX[i]; q.y = py + NB_DY[i];
        if (contains(a, q)) { out[2 * *n] = q.x; out[2 * *n + 1] = q.y; ++*n; }
    }
}
/* Area::iter, area.rs:60-62, 131-148: row-major cells */
uint32_t o1_area_cells(int32_t x0, int32_t y0, int32_t x1, int32_t y1, int32_t* out, uint32_t cap) {
    uint32_t n = 0;
    for (int32_t y = y0; y <= y1; ++y)
        for (int32_t x = x0; x <= x1; ++x) {
            if (n < cap) { out[2 * n] = x; out[2 * n + 1] = y; }
            ++n;
        }
    return n;
}
/* area_factory, area.rs:95-117 */
uint32_t o1_area_factory(int32_t sx, int32_t sy, int32_t ex, int32_t ey, uint32_t size, int32_t* out, uint32_t cap) {
    int32_t fx = (ex - sx + 1) / (int32_t)size, fy = (ey - sy + 1) / (int32_t)size;
    uint32_t n = 0;
    for (int32_t j = 0; j < fy; ++j)
        for (int32_t i = 0; i < fx; ++i) {
            if (n < cap) {
                out[4 * n] = sx + i * (int32_t)size; out[4 * n + 1] = sy + j * (int32_t)size;
                out[4 * n + 2] = sx + i * (int32_t)size + (int32_t)size - 1; out[4 * n + 3] = sy + j * (int32_t)size + (int32_t)size - 1;
            }
            ++n;
        }
    return n;
}
