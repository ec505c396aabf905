/*
 * oracle/o_common.h -- TEST INFRASTRUCTURE ONLY (shared by the two CPU oracles, never
 * linked into the product).
 *
 * Types and helpers of the reference model (thoughtworks/epirust) restated in C: points,
 * inclusive areas, the citizen record, the grid layout, and the Philox draw slots.
 *
 * Randomness.  The reference draws from an unseeded thread_rng
 * (common/src/utils/random_wrapper.rs:27-30).  Here every draw is a fixed word of a
 * counter-based Philox block.  The movement words come from Philox2x32-10 keyed by the
 * world's movement key (word 0 of the Philox4x32-10 block (0, 0xFFFFFFFF, 20, 0) of the
 * world key):
 *   point    counter = (agent | 1 << 25, hour): u0,u1 = random point x,y
 *   choice   counter = (agent, hour): u2 = Moore choice (move_agent_from) or death draw
 *            (hour 23)
 * The rest come from Philox4x32-10 keyed by the world key, counter = (agent, hour, block, 0):
 *   block 1  disease: Susceptible neighbours 0-3; Exposed u0 = jitter, u1 = symptoms;
 *            Pre u0 = severe
 *   block 2  Susceptible neighbours 4-7
 *   block 3  vaccination (hour = the vaccination hour)
 * World build uses hour = 0xFFFFFFFF with blocks 16 (citizen), 17 (essential worker),
 * 18 (house start point, counter word 0 = house index), 19 (starting-infection sampling
 * step).  gen_bool(p) is u < floor(p * 2^32) (always true for p >= 1); gen_range/choose
 * over k values is (u * k) >> 32 (rand 0.8.5's own integer mapping is not reproduced: its
 * stream is unseeded, so only the distributions carry over).
 */
#ifndef ORACLE_COMMON_H
#define ORACLE_COMMON_H

#include <math.h>
#include <stdint.h>
#include <string.h>

#include "../include/epi_engine.h"
#include "philox.h"

#define WB_HOUR 0xFFFFFFFFu

typedef struct { int32_t x, y; } pt;
typedef struct { pt s, e; } area; /* inclusive corners, engine/src/geography/area.rs:30-35 */

/* engine/src/citizen/mod.rs:48-63 (id = creation index) */
typedef struct {
    uint32_t id;
    uint8_t state;          /* EPI_S .. EPI_D */
    uint32_t at_hour;       /* Exposed / Pre */
    uint32_t day;           /* Infected */
    int32_t immunity;
    area home, work;
    uint8_t vaccinated, uses_pt, hospitalized, isolated, work_quarantined;
    area current;
    uint8_t ws;             /* EPI_WS_* */
    uint32_t work_start_at; /* HospitalStaff */
} citizen;

/* engine/src/geography/grid.rs:36-50 plus the config and the random key */
typedef struct {
    epi_params p;
    int32_t G, W;           /* grid size, plane width G+1 */
    area housing, transport, work_area, hospital;
    uint32_t hfx, hfy, ofx, ofy;
    uint32_t key[2];
    uint32_t move_key;      /* key of the Philox2x32 movement draws */
} o_world;

static inline void draw4(const o_world* w, uint32_t c0, uint32_t c1, uint32_t c2, uint32_t out[4]) {
    uint32_t ctr[4] = {c0, c1, c2, 0u};
    orc_philox4x32_10(ctr, w->key, out);
}

/* Bernoulli(p) of rand's gen_bool, as an integer threshold on a 32-bit word. */
static inline int bern(uint32_t u, double p) {
    uint64_t thr = p >= 1.0 ? (1ull << 32) : (p > 0.0 ? (uint64_t)(p * 4294967296.0) : 0ull);
    return (uint64_t)u < thr;
}

static inline uint32_t pick(uint32_t u, uint32_t k) { return (uint32_t)(((uint64_t)u * k) >> 32); }

static inline int32_t rng_range(uint32_t u, int32_t lo, int32_t hi) {
    return lo + (int32_t)pick(u, (uint32_t)(hi - lo + 1));
}

static inline area mk_area(int32_t x0, int32_t y0, int32_t x1, int32_t y1) {
    area a; a.s.x = x0; a.s.y = y0; a.e.x = x1; a.e.y = y1; return a;
}

/* Area::contains, engine/src/geography/area.rs:83-88 */
static inline int contains(area a, pt p) {
    return a.s.x <= p.x && a.e.x >= p.x && a.s.y <= p.y && a.e.y >= p.y;
}

/* Area PartialEq compares the offsets only, area.rs:37-43 */
static inline int area_eq(area a, area b) {
    return a.s.x == b.s.x && a.s.y == b.s.y && a.e.x == b.e.x && a.e.y == b.e.y;
}

/* Area::get_random_point, area.rs:76-81 (x drawn first, then y) */
static inline pt random_point(area a, uint32_t ux, uint32_t uy) {
    pt r; r.x = rng_range(ux, a.s.x, a.e.x); r.y = rng_range(uy, a.s.y, a.e.y); return r;
}

/* CitizenLocationMap::is_point_in_grid, allocation_map.rs:156-159 */
static inline int in_grid(const o_world* w, pt p) { return p.x >= 0 && p.y >= 0 && p.x < w->G && p.y < w->G; }

/* NeighborIterator offsets, engine/src/geography/point.rs:59 */
static const int32_t NB_DX[8] = {-1, 0, 1, -1, 1, -1, 0, 1};
static const int32_t NB_DY[8] = {-1, -1, -1, 0, 0, 1, 1, 1};

/* Disease::get_current_transmission_rate, common/src/disease/mod.rs:88-95 */
static inline double transmission_rate(const epi_params* p, uint32_t day) {
    if (p->regular_transmission_start_day < day && day <= p->high_transmission_start_day)
        return p->regular_transmission_rate;
    if (p->high_transmission_start_day < day && day <= p->last_day) return p->high_transmission_rate;
    return 0.0;
}

static inline int is_infected(const citizen* c) { return c->state >= EPI_I_PRE && c->state <= EPI_I_SEVERE; }
/* DiseaseStateMachine::is_symptomatic, disease_state_machine.rs:96-98 */
static inline int is_symptomatic(const citizen* c) { return c->state == EPI_I_MILD || c->state == EPI_I_SEVERE; }
/* Citizen::can_move, citizen/mod.rs:452-454 */
static inline int can_move(const citizen* c) {
    return !(is_symptomatic(c) || c->hospitalized || c->state == EPI_D || c->isolated);
}
static inline int is_working(const citizen* c) { return c->ws != EPI_WS_NA; }

/* lazily materialised Philox blocks of one agent-hour; "block 0" words 0,1 are the point
   draw and word 2 the choice draw (Philox2x32), blocks 1, 2 are Philox4x32 */
typedef struct { const o_world* w; uint32_t agent, hour; int have[3], have_point, have_choice; uint32_t blk[3][4];
                 uint32_t point[2], choice; } draws;
static inline void draws_init(draws* d, const o_world* w, uint32_t agent, uint32_t hour) {
    d->w = w; d->agent = agent; d->hour = hour;
    d->have[0] = d->have[1] = d->have[2] = 0;
    d->have_point = d->have_choice = 0;
}
static inline uint32_t dr(draws* d, int b, int k) {
    if (b == 0) {
        if (k < 2) {
            if (!d->have_point) {
                const uint32_t ctr[2] = {d->agent | (1u << 25), d->hour};
                orc_philox2x32_10(ctr, d->w->move_key, d->point);
                d->have_point = 1;
            }
            return d->point[k];
        }
        if (!d->have_choice) {
            const uint32_t ctr[2] = {d->agent, d->hour};
            uint32_t out[2];
            orc_philox2x32_10(ctr, d->w->move_key, out);
            d->choice = out[0];
            d->have_choice = 1;
        }
        return d->choice;
    }
    if (!d->have[b]) { draw4(d->w, d->agent, d->hour, (uint32_t)b, d->blk[b]); d->have[b] = 1; }
    return d->blk[b][k];
}

/* Counts::update_counts, engine/src/models/events/counts.rs:126-140 (S,E,I,H,R,D) */
static inline void count_agent(uint32_t cnt[6], const citizen* c) {
    switch (c->state) {
    case EPI_S: cnt[0]++; break;
    case EPI_E: cnt[1]++; break;
    case EPI_R: cnt[4]++; break;
    case EPI_D: cnt[5]++; break;
    default: if (c->hospitalized) cnt[3]++; else cnt[2]++; break;
    }
}

/* ---------------------------------------------------------------- intervention triggers */
typedef struct { uint32_t hour; char name[24]; char data[40]; } o_report;

typedef struct {
    int locked;
    uint32_t zero_infection_hour;
    uint32_t new_infections_in_a_day;
    int hospital_applied;
} o_iv_state;

typedef struct { int vaccinate; double percent; int lock, unlock, grow; uint32_t applied; } o_iv_actions;

/* process_interventions triggers, allocation_map.rs:306-337: VaccinateIntervention
 * (vaccination.rs:52-54; the HashMap keeps the last entry of an hour), LockdownIntervention
 * (lockdown.rs:55-89; zero_infection_hour stays 0 in standalone mode), BuildNewHospital
 * (hospital.rs:51-74) and the occupancy extension.  c = {S,E,I,H,R,D}. */
static inline o_iv_actions o_decide_interventions(const o_world* w, o_iv_state* st, uint32_t hour, const uint32_t c[6]) {
    const epi_params* p = &w->p;
    o_iv_actions a;
    memset(&a, 0, sizeof a);
    int vi = -1;
    for (int k = 0; k < p->n_vaccinations; ++k) if (p->vaccination_at_hour[k] == hour) vi = k;
    if (vi >= 0) { a.vaccinate = 1; a.percent = p->vaccination_percent[vi]; a.applied |= EPI_IV_VACCINATION; }
    if (!st->locked && hour % 24u == 0 && p->has_lockdown && c[2] > p->lockdown_at_number_of_infections) {
        st->locked = 1; a.lock = 1; a.applied |= EPI_IV_LOCKDOWN;
    }
    /* unlock_hour = zero_infection_hour + round(14 * 1.5) * 24 (lockdown.rs:69-73) */
    if (st->locked && hour == st->zero_infection_hour + 21u * 24u) {
        st->locked = 0; st->zero_infection_hour = 0; a.unlock = 1; a.applied |= EPI_IV_LOCKDOWN_REVOKED;
    }
    if (hour % 24u == 0) {
        uint32_t inf = c[2];
        st->new_infections_in_a_day = inf > st->new_infections_in_a_day ? inf - st->new_infections_in_a_day : 0;
    }
    if (!st->hospital_applied && hour % 24u == 0) {
        int grow = p->has_build_new_hospital && st->new_infections_in_a_day >= p->spread_rate_threshold;
        if (p->hospital_occupancy_trigger > 0.0) {
            double cells = (double)(w->hospital.e.x - w->hospital.s.x + 1) * (double)(w->hospital.e.y - w->hospital.s.y + 1);
            if ((double)c[3] >= p->hospital_occupancy_trigger * cells) grow = 1;
        }
        if (grow) { st->hospital_applied = 1; a.grow = 1; a.applied |= EPI_IV_BUILD_NEW_HOSPITAL; }
    }
    return a;
}

/* Grid::increase_hospital_size, grid.rs:233-238 */
static inline void o_increase_hospital_size(o_world* w) {
    w->hospital = mk_area(w->hospital.s.x, w->hospital.s.y, w->G, w->G);
}

/* define_geography, engine/src/geography/mod.rs:33-70 */
static inline void o_define_geography(o_world* w) {
    int32_t G = w->G;
    int32_t home_width = (int32_t)ceil((double)G * 0.4);
    int32_t transport_end = home_width + (int32_t)ceil((double)G * 0.2);
    int32_t work_end = transport_end + (int32_t)ceil((double)G * 0.2);
    int32_t hospital_end = work_end + (int32_t)ceil((double)G * 0.1);
    w->housing = mk_area(0, 0, home_width - 1, G);
    w->transport = mk_area(home_width, 0, transport_end - 1, G);
    w->work_area = mk_area(transport_end, 0, work_end - 1, G);
    w->hospital = mk_area(work_end, 0, hospital_end - 1, G);
    /* area_factory, area.rs:95-117 */
    w->hfx = (uint32_t)((w->housing.e.x - w->housing.s.x + 1) / 2);
    w->hfy = (uint32_t)((w->housing.e.y - w->housing.s.y + 1) / 2);
    w->ofx = (uint32_t)((w->work_area.e.x - w->work_area.s.x + 1) / 10);
    w->ofy = (uint32_t)((w->work_area.e.y - w->work_area.s.y + 1) / 10);
}

/* Grid::resize_hospital, grid.rs:240-261 (get_number_of_cells omits the +1) */
static inline void o_resize_hospital(o_world* w, int32_t n, double staff_pct, double beds_pct) {
    uint32_t beds = (uint32_t)ceil((double)n * beds_pct + (double)n * staff_pct);
    int32_t width = w->hospital.e.x - w->hospital.s.x;
    uint32_t cells = (uint32_t)(width * (w->hospital.e.y - w->hospital.s.y));
    if (beds <= cells && width > 0) {
        int32_t end_y = (int32_t)(beds / (uint32_t)width);
        w->hospital = mk_area(w->hospital.s.x, w->hospital.s.y, w->hospital.e.x, end_y);
    }
}

static inline int o_world_init(o_world* w, const epi_params* p) {
    memset(w, 0, sizeof *w);
    w->p = *p;
    w->G = (int32_t)p->grid_size;
    w->W = w->G + 1;
    w->key[0] = (uint32_t)p->seed;
    w->key[1] = (uint32_t)(p->seed >> 32);
    {
        uint32_t mk[4];
        draw4(w, 0u, WB_HOUR, 20u, mk);
        w->move_key = mk[0];
    }
    if (p->grid_size < 1 || p->grid_size > 16382 || p->number_of_agents == 0) return EPI_ERR_CONFIG;
    o_define_geography(w);
    return EPI_OK;
}

#endif
