// tick.cuh -- the per-agent hourly rules as sm_103a device code.
//
// One thread owns one agent for one hour.  It reads the agent's packed words and the
// previous-hour occupancy plane (never another agent's record), proposes a target cell,
// updates its own disease state, and claims the target with atomicMin on the claim plane.
// The rules follow engine/src/citizen/mod.rs:215-454,
// engine/src/state_machine/default_disease_handler.rs:31-103 and
// engine/src/allocation_map.rs:136-163; random draws are fixed words of per-agent-hour
// Philox blocks (movement: Philox2x32, counter = agent | which, hour; disease: Philox4x32,
// counter = agent, hour, block, 0).
//
// Moore neighbourhoods are evaluated as bit masks: the byte plane carries a one-cell border,
// so the 3x3 block around any cell of [0, G]^2 is in bounds; each of its three rows comes in
// as two aligned 32-bit loads and a funnel shift, and SWAR tests turn the nine bytes into
// 8-bit masks (bit k = k-th neighbour in NeighborIterator order) of occupied, infectious and
// high-rate neighbours.  The area and grid filters of get_neighbors_of / is_point_in_grid
// become a second mask built from six comparisons.  A per-cell count of infectious
// neighbours (maintained by k_commit) lets a susceptible agent skip the exposure block when
// it is zero.
#pragma once

#include "epi_internal.h"

namespace epi {

// Moore offsets in NeighborIterator order (engine/src/geography/point.rs:59), packed as
// 2-bit (d + 1) fields: k-th neighbour = (x + dx(k), y + dy(k)) with dx(k) + 1 the k-th field
// of kMooreDx and dy(k) + 1 that of kMooreDy.
constexpr uint32_t kMooreDx = 0x9224u, kMooreDy = 0xA940u;

struct PlaneView {
    const uint8_t* __restrict__ cells;  // padded plane: cell (x, y) at (y + 1) * WP + (x + 1)
    int32_t G, WP;
    int* err;
    // Per cell, the number of infectious agents (class >= 2) on its 8 neighbours, same
    // layout as cells; nullptr when the caller keeps none (the 3x3 is then read instead).
    const uint8_t* __restrict__ danger;
    // Cells outside [0, G]^2 are never addressed by construction; if one were, it is
    // reported through err and treated as occupied instead of being dereferenced.
    __device__ __forceinline__ bool inside(int32_t x, int32_t y) const {
        return (uint32_t)x <= (uint32_t)G && (uint32_t)y <= (uint32_t)G;
    }
    __device__ __forceinline__ uint32_t at(int32_t x, int32_t y) const {
        if (!inside(x, y)) {
            atomicOr(err, 1);
            return 1u;
        }
        return __ldg(cells + (size_t)(y + 1) * (size_t)WP + (size_t)(x + 1));
    }
    __device__ __forceinline__ bool vacant(int32_t x, int32_t y) const { return at(x, y) == 0u; }
    __device__ __forceinline__ uint32_t danger_at(int32_t x, int32_t y) const {
        if (!inside(x, y)) {
            atomicOr(err, 1);
            return 0u;
        }
        return __ldg(danger + (size_t)(y + 1) * (size_t)WP + (size_t)(x + 1));
    }
    // Bytes of (x-1, y), (x, y), (x+1, y) in bits 0-7, 8-15, 16-23 (bits 24-31: the next
    // byte of the row, which no caller reads).
    __device__ __forceinline__ uint32_t row3(int32_t x, int32_t y) const {
        const uintptr_t a = (uintptr_t)(cells + (size_t)(y + 1) * (size_t)WP + (size_t)x);
        const uint32_t* w = (const uint32_t*)(a & ~(uintptr_t)3);
        const uint32_t lo = __ldg(w), hi = __ldg(w + 1);
        return __funnelshift_r(lo, hi, (uint32_t)(a & 3u) * 8u);
    }
};

// The eight neighbour bytes of a 3x3 block in NeighborIterator order, as two words: bytes of
// lo = neighbours 0-3 (row 0 bytes 0-2, row 1 byte 0), bytes of hi = neighbours 4-7 (row 1
// byte 2, row 2 bytes 0-2).  Two byte permutes; byte 3 of a row is never selected.
struct Nb8 {
    uint32_t lo, hi;
};
__device__ __forceinline__ Nb8 neighbour_bytes(uint32_t r0, uint32_t r1, uint32_t r2) {
    return Nb8{__byte_perm(r0, r1, 0x4210u), __byte_perm(r1, r2, 0x6542u)};
}
// Bit 0 of each byte of f (other bits zero) -> 4 bits, byte k to bit k: the product spreads
// byte k's bit to bit 24 + k with no carries (the other partial products land on distinct
// bits below 24 or beyond bit 31).
__device__ __forceinline__ uint32_t pack4(uint32_t f) { return (f * 0x01020408u) >> 24; }
__device__ __forceinline__ uint32_t pack8(uint32_t flo, uint32_t fhi) { return pack4(flo) | (pack4(fhi) << 4); }

// The three rows of the 3x3 block around (x, y); a cell outside [0, G]^2 reads as a
// block of occupied, non-infectious cells (and is reported).
struct Rows3 {
    uint32_t r0, r1, r2;
};
__device__ __forceinline__ Rows3 rows_around(const PlaneView& pl, int32_t x, int32_t y) {
    if (!pl.inside(x, y)) {
        atomicOr(pl.err, 1);
        return Rows3{0x010101u, 0x010101u, 0x010101u};
    }
    return Rows3{pl.row3(x, y - 1), pl.row3(x, y), pl.row3(x, y + 1)};
}

// Plane bytes are 0..3: occupied <=> bit0|bit1, infectious <=> bit1, high rate <=> bit0&bit1.
// Masks are 8 bits in NeighborIterator order.
__device__ __forceinline__ uint32_t occupied_mask(const Rows3& r) {
    const Nb8 b = neighbour_bytes(r.r0, r.r1, r.r2);
    const uint32_t m = 0x01010101u;
    return pack8((b.lo | (b.lo >> 1)) & m, (b.hi | (b.hi >> 1)) & m);
}
// Any infectious byte among the nine (the centre is vacant or the agent's own, never infectious).
__device__ __forceinline__ bool any_infectious(const Rows3& r) { return ((r.r0 | r.r1 | r.r2) & 0x020202u) != 0u; }
__device__ __forceinline__ uint32_t infectious_mask(const Rows3& r) {
    const Nb8 b = neighbour_bytes(r.r0, r.r1, r.r2);
    const uint32_t m = 0x01010101u;
    return pack8((b.lo >> 1) & m, (b.hi >> 1) & m);
}
__device__ __forceinline__ uint32_t high_mask(const Rows3& r) {
    const Nb8 b = neighbour_bytes(r.r0, r.r1, r.r2);
    const uint32_t m = 0x01010101u;
    return pack8(b.lo & (b.lo >> 1) & m, b.hi & (b.hi >> 1) & m);
}

// Neighbours of (x, y) inside area a and the grid (Area::get_neighbors_of filtered by
// is_point_in_grid), as a mask in NeighborIterator order: three column and three row tests
// (each one unsigned range compare) combined row by row.
__device__ __forceinline__ uint32_t valid_neighbours(const Rect& a, int32_t G, int32_t x, int32_t y) {
    const int32_t lx = max(a.x0, 0), hx = min(a.x1, G - 1), ly = max(a.y0, 0), hy = min(a.y1, G - 1);
    if (hx < lx || hy < ly) return 0u;
    const uint32_t wx = (uint32_t)(hx - lx), wy = (uint32_t)(hy - ly);
    const uint32_t dx = (uint32_t)(x - 1 - lx), dy = (uint32_t)(y - 1 - ly);
    const uint32_t C = (uint32_t)(dx <= wx) | ((uint32_t)(dx + 1u <= wx) << 1) | ((uint32_t)(dx + 2u <= wx) << 2);
    const uint32_t top = (dy <= wy) ? C : 0u, bot = (dy + 2u <= wy) ? C : 0u;
    const uint32_t mid = (dy + 1u <= wy) ? ((C & 1u) | ((C >> 1) & 2u)) : 0u;
    return top | (mid << 3) | (bot << 5);
}

// Moore step of the j-th set bit of an 8-bit neighbour mask, as (dx + 1) | (dy + 1) << 2,
// for every mask and j < popc(mask): one table read instead of the bit search.
struct StepTable {
    uint8_t v[256][8];
};
constexpr StepTable make_step_table() {
    StepTable t{};
    for (int m = 0; m < 256; ++m) {
        int j = 0;
        for (int k = 0; k < 8; ++k)
            if ((m >> k) & 1) {
                const int dx = (int)((kMooreDx >> (2 * k)) & 3u), dy = (int)((kMooreDy >> (2 * k)) & 3u);
                t.v[m][j++] = (uint8_t)(dx | (dy << 2));
            }
    }
    return t;
}
__device__ const StepTable kStepTable = make_step_table();

// Lazily materialised Philox blocks of one agent-hour: m(0), m(1) the random-point words
// and m(2) the choice word (Philox2x32 each), d(), d2() the disease blocks (Philox4x32).
struct Draws {
    uint32_t agent, hour, k0, k1, mk;
    uint32_t have = 0;
    uint32_t pt[2], ch[2], b1[4], b2[4];
    __device__ __forceinline__ uint32_t m(int w) {
        if (w < 2) {
            if (!(have & 1u)) { philox2x32(agent | kMovePoint, hour, mk, pt); have |= 1u; }
            return pt[w];
        }
        if (!(have & 8u)) { philox2x32(agent | kMoveChoice, hour, mk, ch); have |= 8u; }
        return ch[0];
    }
    // One movement block chosen per lane (the point block when go, else the choice block),
    // computed before a work-status branch so that a warp whose lanes take both arms runs
    // the Philox rounds once instead of once per arm; the words are the ones m() returns.
    __device__ __forceinline__ void prime(bool go) {
        uint32_t o[2];
        philox2x32(agent | (go ? kMovePoint : kMoveChoice), hour, mk, o);
        if (go) { pt[0] = o[0]; pt[1] = o[1]; have |= 1u; }
        else { ch[0] = o[0]; ch[1] = o[1]; have |= 8u; }
    }
    __device__ __forceinline__ uint32_t d(int w) {
        if (!(have & 2u)) { philox4x32(agent, hour, kBlkDisease, 0u, k0, k1, b1); have |= 2u; }
        return b1[w];
    }
    __device__ __forceinline__ uint32_t d2(int w) {
        if (!(have & 4u)) { philox4x32(agent, hour, kBlkDisease2, 0u, k0, k1, b2); have |= 4u; }
        return b2[w];
    }
};

struct Cell { int32_t x, y; };

__device__ __forceinline__ Cell random_point(const Rect& a, uint32_t ux, uint32_t uy) {
    Cell c;
    c.x = a.x0 + (int32_t)uniform_index(ux, (uint32_t)(a.x1 - a.x0 + 1));
    c.y = a.y0 + (int32_t)uniform_index(uy, (uint32_t)(a.y1 - a.y0 + 1));
    return c;
}

__device__ __forceinline__ Rect home_rect(uint32_t home) {
    int32_t x = unpack_x(home), y = unpack_y(home);
    return Rect{x, y, x + 1, y + 1};
}
__device__ __forceinline__ Rect office_rect(uint32_t work) {
    int32_t x = unpack_x(work), y = unpack_y(work);
    return Rect{x, y, x + 9, y + 9};
}
__device__ __forceinline__ Rect area_rect(const DevParams& P, uint32_t code, uint32_t home, uint32_t work) {
    if (code == kHome) return home_rect(home);
    if (code == kWork) return office_rect(work);
    return P.area[code];
}

// Citizen::can_move, citizen/mod.rs:452-454
__device__ __forceinline__ bool can_move(uint32_t s) {
    uint32_t v = s & kStateMask;
    return !(v == EPI_I_MILD || v == EPI_I_SEVERE || v == EPI_D || (s & (kHosp | kIso)));
}

// Plane byte of an occupied cell: 1 + transmission-rate class of an infectious occupant.
__device__ __forceinline__ uint32_t cell_class(const DevParams& P, uint32_t s) {
    if (!infected(s) || (s & kHosp)) return 1u;
    uint32_t d = (uint32_t)((int32_t)st_day(s) + st_imm(s));  // (day as i32 + immunity) as Day
    return 1u + rate_class(P.reg_start, P.high_start, P.last_day, d);
}

// Citizen::move_agent_from, citizen/mod.rs:415-432: uniform choice among the vacant
// neighbours (of the cell, or of a random point of the area when outside it).
__device__ __forceinline__ Cell move_agent_from(const PlaneView& pl, uint32_t s, const Rect& cur, Cell cell, Draws& dr) {
    if (!can_move(s)) return cell;
    Cell c = cell;
    if (!rect_has(cur, cell.x, cell.y)) c = random_point(cur, dr.m(0), dr.m(1));
    const Rows3 rows = rows_around(pl, c.x, c.y);
    // The choice word is drawn before the rows are used, so that its Philox rounds run while
    // the row loads are in flight (it is needed unless every neighbour is taken).
    const uint32_t u = dr.m(2);
    const uint32_t cand = valid_neighbours(cur, pl.G, c.x, c.y) & ~occupied_mask(rows);
    if (!cand) return cell;
    const uint32_t j = uniform_index(u, (uint32_t)__popc(cand));
    const uint32_t e = __ldg(&kStepTable.v[cand][j]);
    return Cell{c.x + (int32_t)(e & 3u) - 1, c.y + (int32_t)(e >> 2) - 1};  // vacant by construction: move_agent keeps it
}

// Citizen::goto_area, citizen/mod.rs:367-395
__device__ __forceinline__ Cell goto_area(const PlaneView& pl, uint32_t s, const Rect& cur, const Rect& target,
                                          uint32_t home, uint32_t work, Cell cell, Draws& dr) {
    const uint32_t ws = st_ws(s), v = s & kStateMask;
    bool override_movement = false;
    if (ws == EPI_WS_NORMAL || ws == EPI_WS_ESSENTIAL) {
        if (rect_has(office_rect(work), cell.x, cell.y) && rect_eq(target, home_rect(home)) &&
            (v == EPI_I_MILD || v == EPI_I_SEVERE))
            override_movement = true;
    }
    if (!can_move(s) && !override_movement) return cell;
    if (ws != EPI_WS_NA) {
        Cell q = random_point(target, dr.m(0), dr.m(1));
        return pl.vacant(q.x, q.y) ? q : cell;
    }
    return move_agent_from(pl, s, cur, cell, dr);
}

// One lane of an hour whose arms mix a jump and a walk, as one code path: jump lanes take
// goto_area of a worker (Normal or Essential: a random point of the target area, kept when
// vacant), walk lanes move_agent_from over the current area.  Both read the plane row through
// their centre cell in the same pass (a jump tests its centre byte); walkers also read the
// rows above and below.  Same words and outcomes as the two calls, without a warp running the
// two arms' loads one after the other.  Used for hour 8 (workers to the office, the others a
// walk): its k_decide went from 25.9 to 23.6 us at 1M agents.  In hours 7, 16 and 17 the two
// plain calls were measured as fast.
__device__ __forceinline__ Cell jump_or_walk(const PlaneView& pl, uint32_t s, bool jump, const Rect& cur,
                                             const Rect& target, uint32_t home, uint32_t work, Cell cell, Draws& dr) {
    bool act = can_move(s);
    if (jump && !act) {  // goto_area's symptomatic override of a worker going home from the office
        const uint32_t v = s & kStateMask;
        act = rect_has(office_rect(work), cell.x, cell.y) && rect_eq(target, home_rect(home)) &&
              (v == EPI_I_MILD || v == EPI_I_SEVERE);
    }
    if (!act) return cell;
    Cell c = cell;
    if (jump || !rect_has(cur, cell.x, cell.y)) c = random_point(jump ? target : cur, dr.m(0), dr.m(1));
    if (!pl.inside(c.x, c.y)) {  // reads as occupied (and is reported), as rows_around and vacant do
        atomicOr(pl.err, 1);
        return cell;
    }
    const uint32_t r1 = pl.row3(c.x, c.y);
    uint32_t r0 = 0u, r2 = 0u;
    if (!jump) {
        r0 = pl.row3(c.x, c.y - 1);
        r2 = pl.row3(c.x, c.y + 1);
    }
    if (jump) return ((r1 >> 8) & 0xFFu) == 0u ? c : cell;
    const uint32_t u = dr.m(2);
    const uint32_t cand = valid_neighbours(cur, pl.G, c.x, c.y) & ~occupied_mask(Rows3{r0, r1, r2});
    if (!cand) return cell;
    const uint32_t j = uniform_index(u, (uint32_t)__popc(cand));
    const uint32_t e = __ldg(&kStepTable.v[cand][j]);
    return Cell{c.x + (int32_t)(e & 3u) - 1, c.y + (int32_t)(e >> 2) - 1};
}

// DiseaseStateMachine::next with the default DiseaseHandler (ddh:41-86) for the hour's
// proposed cell; at is the Exposed/Pre at_hour word.
// (The agent's current area, needed only when an infectious neighbour exists, is decoded from
// its code and home / work corners here rather than by the caller.)
__device__ __forceinline__ void infection_dynamics(const DevParams& P, const PlaneView& pl, uint32_t& s, uint32_t& at,
                                                   uint32_t home, uint32_t work, Cell cell, uint32_t hour, Draws& dr) {
    const uint32_t v = s & kStateMask;
    if (v == EPI_S) {
        if (s & (kWq | kVacc)) return;
        // no infectious neighbour: no draw can succeed (the centre is vacant or the agent's own)
        if (pl.danger && pl.danger_at(cell.x, cell.y) == 0u) return;
        const Rows3 rows = rows_around(pl, cell.x, cell.y);
        if (!any_infectious(rows)) return;
        const Rect cur = area_rect(P, st_area(s), home, work);
        const uint32_t cand = valid_neighbours(cur, pl.G, cell.x, cell.y) & infectious_mask(rows);
        if (!cand) return;
        const uint32_t high = high_mask(rows);
        const uint64_t thr_reg = P.thr_rate[1], thr_high = P.thr_rate[2];
        // neighbours in NeighborIterator order; the first successful Bernoulli exposes
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            if (!((cand >> k) & 1u)) continue;
            const uint32_t u = k < 4 ? dr.d(k) : dr.d2(k - 4);
            if ((uint64_t)u < (((high >> k) & 1u) ? thr_high : thr_reg)) {
                s = with_state(s, EPI_E);
                at = hour;
                return;
            }
        }
    } else if (v == EPI_E) {
        int32_t jitter = (int32_t)uniform_index(dr.d(0), 3u) - 1;
        uint32_t need = (uint32_t)((int32_t)P.exposed_duration + jitter);
        if (hour - at >= need) {
            bool symptoms = (uint64_t)dr.d(1) < P.thr_symptoms;
            s = with_day(s, 0u);
            if (symptoms) { s = with_state(s, EPI_I_PRE); at = hour; }
            else s = with_state(s, EPI_I_ASYM);
        }
    } else if (v == EPI_I_PRE) {
        if (hour - at >= P.pre_duration)
            s = with_state(s, (uint64_t)dr.d(0) < P.thr_severe ? EPI_I_SEVERE : EPI_I_MILD);
    }
}

// Hour-of-day classes of the routine (constants.rs:27-36); the kernels are specialised per
// class so that each launch carries only the branches its hour can take.
enum HourClass : int {
    kHcStart = 0,     // 0: ROUTINE_START_TIME
    kHcEnd = 1,       // 23: ROUTINE_END_TIME
    kHcMove = 2,      // 9-11, 13-15, 18-22: everyone but hospital staff walks (move_agent_from)
    kHcTransport = 3, // 7, 17: ROUTINE_TRAVEL_START/END_TIME
    kHcWork = 4,      // 8: ROUTINE_WORK_TIME
    kHcNoon = 5,      // 12: NON_WORKING_TRAVEL_END_TIME
    kHcHome = 6,      // 16: ROUTINE_WORK_END_TIME
    kHcSleep = 7      // 1-6: SLEEP_START_TIME..=SLEEP_END_TIME
};

__host__ __device__ constexpr int hour_class(uint32_t hod) {
    return hod == 0u ? kHcStart
         : hod == 23u ? kHcEnd
         : (hod >= 1u && hod <= 6u) ? kHcSleep
         : (hod == 7u || hod == 17u) ? kHcTransport
         : hod == 8u ? kHcWork
         : hod == 12u ? kHcNoon
         : hod == 16u ? kHcHome
         : kHcMove;
}

// The HospitalStaff arm of Citizen::perform_movements (citizen/mod.rs:292-328).  Returns
// false when the hour ends before the infection update (the two early returns).
__device__ __forceinline__ bool staff_movements(const DevParams& P, const PlaneView& pl, uint32_t& s, uint32_t& wsa,
                                                uint32_t home, uint32_t work, Cell cell, Cell& nc, uint32_t hod,
                                                uint32_t hour, Draws& dr) {
    const Rect cur = area_rect(P, st_area(s), home, work);
    const uint32_t since = hour >= wsa ? hour - wsa : 0u;  // saturating_sub
    if (since == 24u * 14u) {
        s |= kWq;
        return false;
    }
    if (since == 24u * 14u * 2u) {
        nc = goto_area(pl, s, cur, home_rect(home), home, work, cell, dr);
        s = with_area(s, kHome);
        wsa = hour + 24u * 14u;
        return false;
    }
    if (hod == 8u) {
        const Rect hosp = P.area[P.hosp_code];
        if (!rect_eq(cur, hosp) && wsa <= hour) {
            nc = goto_area(pl, s, cur, hosp, home, work, cell, dr);
            s = with_area(s, P.hosp_code);
            wsa = hour;
        }
        s &= ~kWq;
    } else if (hod == 16u) {
        s |= kWq;
    } else if (!(s & kWq) && can_move(s)) {
        nc = move_agent_from(pl, s, cur, cell, dr);
    }
    return true;
}

// Citizen::perform_movements, citizen/mod.rs:257-349, for the movement classes (hours 7..22):
// the work-status arms (Normal|Essential, HospitalStaff, NA) at hour class HC.  Returns the
// proposed cell; infect is cleared when the hour ends before the infection update of
// DiseaseStateMachine::next, which the caller runs on the proposed cell otherwise.
template <int HC>
__device__ __forceinline__ Cell perform_movements(const DevParams& P, const PlaneView& pl, uint32_t& s, uint32_t& wsa,
                                                  uint32_t home, uint32_t work, Cell cell, uint32_t hod, uint32_t hour,
                                                  Draws& dr, bool& infect) {
    const uint32_t ws = st_ws(s);
    Cell nc = cell;
    infect = true;
    if (ws == EPI_WS_HOSPITAL_STAFF) {
        infect = staff_movements(P, pl, s, wsa, home, work, cell, nc, hod, hour, dr);
    } else {
        const Rect cur = area_rect(P, st_area(s), home, work);
        const bool worker = ws != EPI_WS_NA;  // Normal or Essential here
        // The arms of each class, as goto_area / move_agent_from calls of the reference.  A
        // non-worker's goto_area is move_agent_from over its current area (work status NA), so
        // a class's arms are a jump of some workers and a walk of everyone else (at noon, a
        // walk of everyone: one call).  Where lanes differ, each computes its one Philox block
        // before the branch, the point block for a jump and the choice block for a walk, so a
        // warp runs the rounds once.
        if (HC == kHcMove) {
            nc = move_agent_from(pl, s, cur, cell, dr);
        } else if (HC == kHcTransport) {
            // worker with public transport: goto_area(transport); others: move_agent_from
            const bool jump = worker && (s & kPt);
            dr.prime(jump);
            if (jump) {
                nc = goto_area(pl, s, cur, P.area[kTransport], home, work, cell, dr);
                s = with_area(s, kTransport);
            } else {
                nc = move_agent_from(pl, s, cur, cell, dr);
            }
        } else if (HC == kHcWork) {
            // worker: goto_area(office); non-worker: goto_area(housing), a walk
            dr.prime(worker);
            nc = jump_or_walk(pl, s, worker, cur, office_rect(work), home, work, cell, dr);
            s = with_area(s, worker ? kWork : kHousing);
        } else if (HC == kHcNoon) {
            // worker: move_agent_from; non-worker: goto_area(home), a walk
            nc = move_agent_from(pl, s, cur, cell, dr);
            if (!worker) s = with_area(s, kHome);
        } else {  // kHcHome
            // worker: goto_area(home); non-worker: move_agent_from
            dr.prime(worker);
            if (worker) {
                nc = goto_area(pl, s, cur, home_rect(home), home, work, cell, dr);
                s = with_area(s, kHome);
            } else {
                nc = move_agent_from(pl, s, cur, cell, dr);
            }
        }
    }
    return nc;
}

// Hour 0 of the day: increment_infection_day, then Citizen::hospitalize
// (citizen/mod.rs:240-243, 351-365; allocation_map.rs:144-150).  hosp_first is the first
// vacant hospital cell of the snapshot in area-iterator order (packed) or kNoAction.
__device__ __forceinline__ bool wants_hospital(const DevParams& P, uint32_t s) {
    if ((s & kHosp) || (s & kStateMask) != EPI_I_SEVERE) return false;
    uint32_t d = (uint32_t)((int32_t)st_day(s) + st_imm(s));
    return (P.hosp_if_class >> rate_class(P.reg_start, P.high_start, P.last_day, d)) & 1u;
}

__device__ __forceinline__ Cell routine_start(const DevParams& P, const PlaneView& pl, uint32_t& s, uint32_t home,
                                              Cell cell, uint32_t hosp_first, Draws& dr) {
    if (infected(s)) s = with_day(s, st_day(s) + 1u);
    if (!wants_hospital(P, s)) return cell;
    if (hosp_first != kNoAction) {
        s |= kHosp;
        return Cell{unpack_x(hosp_first), unpack_y(hosp_first)};
    }
    Cell q = random_point(home_rect(home), dr.m(0), dr.m(1));
    return pl.vacant(q.x, q.y) ? q : cell;
}

// Hour 23: Citizen::deceased with on_routine_end (citizen/mod.rs:397-413, ddh:88-102).
__device__ __forceinline__ Cell routine_end(const DevParams& P, const PlaneView& pl, uint32_t& s, uint32_t home,
                                            Cell cell, Draws& dr) {
    const uint32_t v = s & kStateMask, day = st_day(s);
    if (v == EPI_I_ASYM && day == 9u) s = with_state(s, EPI_R);          // ASYMPTOMATIC_LAST_DAY
    else if (v == EPI_I_MILD && day == 12u) s = with_state(s, EPI_R);    // MILD_INFECTED_LAST_DAY
    else if (v == EPI_I_SEVERE && day == P.last_day)
        s = with_state(s, (uint64_t)dr.m(2) < P.thr_death ? EPI_D : EPI_R);
    Cell nc = cell;
    const uint32_t nv = s & kStateMask;
    if (nv == EPI_R) {
        Cell q = random_point(home_rect(home), dr.m(0), dr.m(1));
        if (pl.vacant(q.x, q.y)) nc = q;
    }
    if (nv == EPI_R || nv == EPI_D) s &= ~kHosp;
    return nc;
}

// Counts::update_counts bin (counts.rs:126-140): 0 S, 1 E, 2 I, 3 H, 4 R, 5 D.
__device__ __forceinline__ uint32_t count_bin(uint32_t s) {
    uint32_t v = s & kStateMask;
    if (v == EPI_S) return 0u;
    if (v == EPI_E) return 1u;
    if (v == EPI_R) return 4u;
    if (v == EPI_D) return 5u;
    return (s & kHosp) ? 3u : 2u;
}

// tgt word: target x | y << 16 (14 bits each, grids up to 16,383) with the new plane class
// in bits 15 (low) and 31 (high) and the class before the hour in bits 14 and 30.
__device__ __forceinline__ uint32_t encode_target(Cell c, uint32_t cls, uint32_t old_cls) {
    return pack_xy(c.x, c.y) | ((cls & 1u) << 15) | ((cls >> 1) << 31) | ((old_cls & 1u) << 14) | ((old_cls >> 1) << 30);
}
__device__ __forceinline__ uint32_t target_xy(uint32_t t) { return t & 0x3FFF3FFFu; }
__device__ __forceinline__ uint32_t target_class(uint32_t t) { return ((t >> 15) & 1u) | ((t >> 30) & 2u); }
__device__ __forceinline__ uint32_t target_old_class(uint32_t t) { return ((t >> 14) & 1u) | ((t >> 29) & 2u); }

// Add delta (+1 / -1) to the infectious-neighbour count of the 8 cells around the padded
// plane index c (atomically, on the 32-bit words holding the bytes; counts stay in 0..8).
__device__ __forceinline__ void danger_add(uint8_t* danger, size_t c, uint32_t WP, int delta) {
    const size_t nb[8] = {c - WP - 1, c - WP, c - WP + 1, c - 1, c + 1, c + WP - 1, c + WP, c + WP + 1};
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const uintptr_t a = (uintptr_t)(danger + nb[k]);
        uint32_t* w = (uint32_t*)(a & ~(uintptr_t)3);
        const uint32_t one = 1u << ((a & 3u) * 8u);
        if (delta > 0) atomicAdd(w, one);
        else atomicSub(w, one);
    }
}

}  // namespace epi
