/*
 * oracle/o_rules.h -- TEST INFRASTRUCTURE ONLY (the per-agent rules of both CPU oracles).
 *
 * One C function per reference function of the hourly routine, reading the previous-hour
 * map through two functions the including file defines for its map type SNAP_T:
 *   static int snap_vacant(const SNAP_T* m, pt p);             is_cell_vacant
 *   static const citizen* snap_get(const SNAP_T* m, pt p);     get_agent_for (NULL if none)
 * Each rule works on a private copy of the agent (the reference's `*agent` copy in the
 * parallel map, allocation_map.rs:84-90) and returns the proposed cell.
 */
#ifndef ORACLE_RULES_H
#define ORACLE_RULES_H

#ifndef SNAP_T
#error "define SNAP_T, snap_vacant and snap_get before including o_rules.h"
#endif

/* CitizenLocationMap::move_agent, allocation_map.rs:136-142 */
static inline pt move_agent(const SNAP_T* m, pt old_cell, pt new_cell) {
    return snap_vacant(m, new_cell) ? new_cell : old_cell;
}

/* Citizen::move_agent_from, citizen/mod.rs:415-432 */
static pt move_agent_from(const o_world* w, const SNAP_T* m, const citizen* c, pt cell, draws* d) {
    if (!can_move(c)) return cell;
    pt cur = cell;
    if (!contains(c->current, cell)) cur = random_point(c->current, dr(d, 0, 0), dr(d, 0, 1));
    pt cand[8];
    uint32_t k = 0;
    for (int i = 0; i < 8; ++i) {
        pt q; q.x = cur.x + NB_DX[i]; q.y = cur.y + NB_DY[i];
        if (contains(c->current, q) && in_grid(w, q) && snap_vacant(m, q)) cand[k++] = q;
    }
    pt nc = k ? cand[pick(dr(d, 0, 2), k)] : cell;
    return move_agent(m, cell, nc);
}

/* Citizen::goto_area, citizen/mod.rs:367-395 */
static pt goto_area(const o_world* w, const SNAP_T* m, const citizen* c, area target, pt cell, draws* d) {
    int override_movement = 0;
    if (c->ws == EPI_WS_NORMAL || c->ws == EPI_WS_ESSENTIAL) {
        if (contains(c->work, cell) && area_eq(target, c->home) &&
            (c->state == EPI_I_MILD || c->state == EPI_I_SEVERE))
            override_movement = 1;
    }
    if (!can_move(c) && !override_movement) return cell;
    if (is_working(c)) {
        pt nc = random_point(target, dr(d, 0, 0), dr(d, 0, 1));
        if (!snap_vacant(m, nc)) nc = cell;
        return move_agent(m, cell, nc);
    }
    return move_agent_from(w, m, c, cell, d);
}

/* DiseaseHandler for Disease: on_susceptible / on_exposed / on_infected,
 * engine/src/state_machine/default_disease_handler.rs:41-86, dispatched by
 * DiseaseStateMachine::next, engine/src/disease_state_machine.rs:53-70. */
static void update_infection_dynamics(const o_world* w, const SNAP_T* m, citizen* c, pt cell, uint32_t hour, draws* d) {
    const epi_params* p = &w->p;
    switch (c->state) {
    case EPI_S:
        if (!c->work_quarantined && !c->vaccinated) {
            for (int i = 0; i < 8; ++i) {
                pt q; q.x = cell.x + NB_DX[i]; q.y = cell.y + NB_DY[i];
                if (!contains(c->current, q) || !in_grid(w, q)) continue;
                const citizen* nb = snap_get(m, q); /* occupant in the previous-hour map */
                if (!nb || !is_infected(nb) || nb->hospitalized) continue;
                uint32_t nday = (uint32_t)((int32_t)nb->day + nb->immunity); /* citizen/mod.rs:184 */
                uint32_t u = i < 4 ? dr(d, 1, i) : dr(d, 2, i - 4);
                if (bern(u, transmission_rate(p, nday))) {
                    c->state = EPI_E;
                    c->at_hour = hour;
                    break;
                }
            }
        }
        break;
    case EPI_E: {
        int32_t jitter = (int32_t)pick(dr(d, 1, 0), 3u) - 1;             /* RANGE_FOR_EXPOSED */
        uint32_t need = (uint32_t)((int32_t)p->exposed_duration + jitter); /* ddh:55, wraps */
        if (hour - c->at_hour >= need) {
            int symptoms = bern(dr(d, 1, 1), 1.0 - p->percentage_asymptomatic_population);
            c->day = 0;
            if (symptoms) { c->state = EPI_I_PRE; c->at_hour = hour; }
            else c->state = EPI_I_ASYM;
        }
        break;
    }
    case EPI_I_PRE:
        if (hour - c->at_hour >= p->pre_symptomatic_duration)
            c->state = bern(dr(d, 1, 0), p->percentage_severe_infected_population) ? EPI_I_SEVERE : EPI_I_MILD;
        break;
    default:
        break;
    }
}

/* Citizen::perform_movements, citizen/mod.rs:257-349 */
static pt perform_movements(const o_world* w, const SNAP_T* m, citizen* c, pt cell, uint32_t hod, uint32_t hour, draws* d) {
    pt nc = cell;
    switch (c->ws) {
    case EPI_WS_NORMAL:
    case EPI_WS_ESSENTIAL:
        if (hod == 7 || hod == 17) {
            if (c->uses_pt) { nc = goto_area(w, m, c, w->transport, cell, d); c->current = w->transport; }
            else nc = move_agent_from(w, m, c, cell, d);
        } else if (hod == 8) {
            nc = goto_area(w, m, c, c->work, cell, d); c->current = c->work;
        } else if (hod == 16) {
            nc = goto_area(w, m, c, c->home, cell, d); c->current = c->home;
        } else {
            nc = move_agent_from(w, m, c, cell, d);
        }
        update_infection_dynamics(w, m, c, nc, hour, d);
        break;
    case EPI_WS_HOSPITAL_STAFF: {
        uint32_t since = hour >= c->work_start_at ? hour - c->work_start_at : 0; /* saturating_sub */
        if (since == 24u * 14u) { c->work_quarantined = 1; return nc; }
        if (since == 24u * 14u * 2u) {
            nc = goto_area(w, m, c, c->home, cell, d);
            c->current = c->home;
            c->work_start_at = hour + 24u * 14u;
            return nc;
        }
        if (hod == 8) {
            if (!area_eq(c->current, w->hospital) && c->work_start_at <= hour) {
                nc = goto_area(w, m, c, w->hospital, cell, d);
                c->current = w->hospital;
                c->work_start_at = hour;
            }
            c->work_quarantined = 0;
        } else if (hod == 16) {
            c->work_quarantined = 1;
        } else {
            if (!c->work_quarantined && can_move(c)) nc = move_agent_from(w, m, c, cell, d);
        }
        update_infection_dynamics(w, m, c, nc, hour, d);
        break;
    }
    default: /* NA */
        if (hod == 8) {
            nc = goto_area(w, m, c, w->housing, cell, d); c->current = w->housing;
        } else if (hod == 12) {
            nc = goto_area(w, m, c, c->home, cell, d); c->current = c->home;
        } else {
            nc = move_agent_from(w, m, c, cell, d);
        }
        update_infection_dynamics(w, m, c, nc, hour, d);
        break;
    }
    return nc;
}

/* Citizen::hospitalize + CitizenLocationMap::goto_hospital + is_to_be_hospitalize,
 * citizen/mod.rs:351-365, allocation_map.rs:144-150, ddh:32-39 */
static pt hospitalize(const o_world* w, const SNAP_T* m, citizen* c, pt cell, draws* d) {
    pt nc = cell;
    if (c->hospitalized || c->state != EPI_I_SEVERE) return nc;
    uint32_t dday = (uint32_t)((int32_t)c->day + c->immunity);
    if (!(transmission_rate(&w->p, dday) >= w->p.high_transmission_rate)) return nc;
    /* hospital_area.iter().find(vacant): AreaIterator order, y outer / x inner (area.rs:131-148) */
    for (int32_t y = w->hospital.s.y; y <= w->hospital.e.y; ++y) {
        for (int32_t x = w->hospital.s.x; x <= w->hospital.e.x; ++x) {
            pt q; q.x = x; q.y = y;
            if (snap_vacant(m, q)) {
                c->hospitalized = 1;
                return move_agent(m, cell, q);
            }
        }
    }
    c->hospitalized = 0;
    return move_agent(m, cell, random_point(c->home, dr(d, 0, 0), dr(d, 0, 1)));
}

/* Citizen::deceased + on_routine_end, citizen/mod.rs:397-413, ddh:88-102 */
static pt deceased(const o_world* w, const SNAP_T* m, citizen* c, pt cell, draws* d) {
    pt nc = cell;
    if (c->state == EPI_I_ASYM && c->day == 9u) c->state = EPI_R;        /* ASYMPTOMATIC_LAST_DAY */
    else if (c->state == EPI_I_MILD && c->day == 12u) c->state = EPI_R;  /* MILD_INFECTED_LAST_DAY */
    else if (c->state == EPI_I_SEVERE && c->day == w->p.last_day)
        c->state = bern(dr(d, 0, 2), w->p.death_rate) ? EPI_D : EPI_R;
    if (c->state == EPI_R) nc = move_agent(m, cell, random_point(c->home, dr(d, 0, 0), dr(d, 0, 1)));
    if ((c->state == EPI_R || c->state == EPI_D) && c->hospitalized) c->hospitalized = 0;
    return nc;
}

/* Citizen::routine, citizen/mod.rs:227-255 */
static pt routine(const o_world* w, const SNAP_T* m, citizen* c, pt cell, uint32_t hour, draws* d) {
    uint32_t hod = hour % 24u;
    if (hod == 0) {
        if (is_infected(c)) c->day += 1; /* increment_infection_day, disease_state_machine.rs:104-106, state.rs:69-73 */
        return hospitalize(w, m, c, cell, d);
    }
    if (hod >= 1 && hod <= 6) {
        if (c->ws != EPI_WS_HOSPITAL_STAFF) c->current = c->home;
        return cell;
    }
    if (hod == 23) return deceased(w, m, c, cell, d);
    return perform_movements(w, m, c, cell, hod, hour, d);
}

#endif
