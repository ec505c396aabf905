// epi_internal.h -- layouts shared by the host world builder and the sm_103a kernels.
//
// Agent state lives on the device as struct-of-arrays of packed 32-bit words:
//   pos[i]   x | y << 16                     (x, y in [0, G]; 15 bits each)
//   st[i].x  disease state, flags, current-area code, work status, immunity, infection day
//   st[i].y  at_hour of Exposed / Infected-Pre
//   home[i]  start corner of the 2x2 house  (packed like pos)
//   work[i]  start corner of the 10x10 office (packed like pos; the house for non-workers)
//   wsa[i]   work_start_at of hospital staff (read only for staff)
// The occupancy plane is one byte per cell of the (G+1) x (G+1) plane (the reference's
// areas reach row and column G, engine/src/geography/mod.rs:42-48), stored with a one-cell
// border of zeros (pitch and height G+3, cell (x, y) at (y+1) * (G+3) + x+1):
//   0 = vacant, 1 = occupied and not infectious, 2 = infectious at the regular rate,
//   3 = infectious at the high rate.
// A u32 claim plane of (G+1) x (G+1) resolves cell conflicts (lowest agent index wins).
#pragma once

#include <stdint.h>

#include "../../include/epi_engine.h"

#if defined(__CUDACC__)
#define EPI_HD __host__ __device__ __forceinline__
#else
#define EPI_HD inline
#endif

namespace epi {

// ---- st.x bit fields
constexpr uint32_t kStateMask = 0x7u;
constexpr uint32_t kHosp = 1u << 3;
constexpr uint32_t kIso = 1u << 4;
constexpr uint32_t kVacc = 1u << 5;
constexpr uint32_t kWq = 1u << 6;
constexpr uint32_t kPt = 1u << 7;
constexpr int kAreaShift = 8;  // 3 bits
constexpr int kWsShift = 11;   // 2 bits
constexpr int kImmShift = 13;  // 3 bits, immunity + 2
constexpr int kDayShift = 16;  // 16 bits
constexpr uint32_t kAreaMask = 0x7u << kAreaShift;
constexpr uint32_t kWsMask = 0x3u << kWsShift;
constexpr uint32_t kDayMask = 0xFFFFu << kDayShift;

// current_area codes; HOME/WORK decode through the agent's home/work corner
enum AreaCode : uint32_t { kHome = 0, kWork = 1, kTransport = 2, kHousing = 3, kHosp0 = 4, kHosp1 = 5, kNumAreas = 6 };

constexpr uint32_t kNoAction = 0xFFFFFFFFu;  // tgt[i]: nothing to commit
constexpr uint32_t kNoClaim = 0xFFFFFFFFu;   // claim plane: free (larger than any key)
// Claim keys: (127 - hour mod 128) << 25 | agent.  Within a window of 128 hours that starts
// at a multiple of 128 a later hour has a smaller key, so atomicMin lets this hour's claims
// replace stale ones and the lowest agent index win among them; the plane is cleared at the
// start of every window and after any rewind of the hour.
constexpr uint32_t kClaimAgentBits = 25;
constexpr uint32_t kMaxAgentsPerWorld = (1u << kClaimAgentBits) - 1u;  // 33,554,431
constexpr uint32_t kClaimWindow = 128;
EPI_HD uint32_t claim_key(uint32_t hour, uint32_t agent) {
    return ((kClaimWindow - 1u - (hour & (kClaimWindow - 1u))) << kClaimAgentBits) | agent;
}
constexpr uint32_t kMaxGrid = 16382;          // coordinates fit 14 bits of a target word (never all ones)
constexpr uint32_t kWorldHour = 0xFFFFFFFFu; // Philox counter word 1 of world-build draws
constexpr uint32_t kMaxHours = 1500000u;     // infection day fits 16 bits

EPI_HD uint32_t st_state(uint32_t s) { return s & kStateMask; }
EPI_HD uint32_t st_area(uint32_t s) { return (s >> kAreaShift) & 7u; }
EPI_HD uint32_t st_ws(uint32_t s) { return (s >> kWsShift) & 3u; }
EPI_HD int32_t st_imm(uint32_t s) { return (int32_t)((s >> kImmShift) & 7u) - 2; }
EPI_HD uint32_t st_day(uint32_t s) { return s >> kDayShift; }
EPI_HD uint32_t with_area(uint32_t s, uint32_t a) { return (s & ~kAreaMask) | (a << kAreaShift); }
EPI_HD uint32_t with_ws(uint32_t s, uint32_t w) { return (s & ~kWsMask) | (w << kWsShift); }
EPI_HD uint32_t with_state(uint32_t s, uint32_t v) { return (s & ~kStateMask) | v; }
EPI_HD uint32_t with_day(uint32_t s, uint32_t d) { return (s & ~kDayMask) | (d << kDayShift); }
EPI_HD bool infected(uint32_t s) { uint32_t v = s & kStateMask; return v >= EPI_I_PRE && v <= EPI_I_SEVERE; }

EPI_HD uint32_t pack_xy(int32_t x, int32_t y) { return (uint32_t)x | ((uint32_t)y << 16); }
EPI_HD int32_t unpack_x(uint32_t p) { return (int32_t)(p & 0x7FFFu); }
EPI_HD int32_t unpack_y(uint32_t p) { return (int32_t)((p >> 16) & 0x7FFFu); }

struct Rect { int32_t x0, y0, x1, y1; };

EPI_HD bool rect_has(const Rect& r, int32_t x, int32_t y) { return r.x0 <= x && x <= r.x1 && r.y0 <= y && y <= r.y1; }
EPI_HD bool rect_eq(const Rect& a, const Rect& b) { return a.x0 == b.x0 && a.y0 == b.y0 && a.x1 == b.x1 && a.y1 == b.y1; }

// Per-engine constants, in device global memory (read through a const __restrict__ pointer).
struct DevParams {
    uint32_t n;                 // agents
    int32_t G;                  // grid size
    int32_t W;                  // claim-plane width G + 1
    int32_t WP;                 // byte-plane pitch G + 3 (one-cell border on each side)
    uint32_t hosp_code;         // kHosp0 or kHosp1: the current hospital_area
    Rect area[kNumAreas];       // global areas by code (HOME/WORK slots unused)
    uint32_t key0, key1;        // Philox key = seed
    uint32_t move_key;          // key of the Philox2x32 movement draws
    uint32_t reg_start, high_start, last_day;
    uint32_t exposed_duration, pre_duration;
    uint32_t hosp_if_class;     // bit c: rate of class c >= high rate (c = 0 none, 1 reg, 2 high)
    uint64_t thr_rate[3];       // Bernoulli thresholds of the rate classes
    uint64_t thr_death, thr_symptoms, thr_severe;
    // placement of this world among the replicates sharing the device arrays
    uint32_t agent_off;         // first agent slot (a multiple of the 256-slot chunk)
    uint32_t active;            // 0 once the run of this replicate has ended
    uint64_t plane_off;         // byte offset of its bordered plane
    uint64_t claim_off;         // word offset of its claim plane
    // day-boundary guard of the run loop: the data-dependent intervention triggers still armed
    uint32_t guard_flags;       // kGuard* bits
    uint32_t lock_threshold;    // lockdown when infected > this
    uint32_t spread_threshold;  // new hospital when the day's new infections >= this
    uint32_t occ_threshold;     // new hospital when hospitalized >= this
};

constexpr uint32_t kGuardLock = 1u, kGuardSpread = 2u, kGuardOccupancy = 4u;

// Code of an agent record's current_area: its house, its office (workers), or the global area
// with the same rectangle; ok = false when it is none of them.
EPI_HD uint32_t area_code_of(const DevParams& hp, const epi_agent_record& r, bool* ok) {
    const Rect a{r.area_x0, r.area_y0, r.area_x1, r.area_y1};
    *ok = true;
    if (rect_eq(a, Rect{r.home_x, r.home_y, r.home_x + 1, r.home_y + 1})) return kHome;
    if (r.work_status != EPI_WS_NA && rect_eq(a, Rect{r.work_x, r.work_y, r.work_x + 9, r.work_y + 9})) return kWork;
    for (uint32_t c = kTransport; c < kNumAreas; ++c)
        if (rect_eq(a, hp.area[c])) return c;
    *ok = false;
    return kHome;
}

// The SoA words of one agent record (the host layout), with the checks that
// epi_engine_create_from_records documents.  Returns 0 when packed, 1 when a field is out of
// range (a cell outside [0, G], a house, office or current area reaching outside the plane, a
// state, work status, immunity or infection day beyond its field), 2 when the current area is
// none of the agent's areas.
struct AgentWords {
    uint32_t pos, s, at, home, work, wsa;
};
EPI_HD bool rect_in_plane(int32_t G, int32_t x0, int32_t y0, int32_t x1, int32_t y1) {
    return x0 >= 0 && y0 >= 0 && x1 <= G && y1 <= G && x0 <= x1 && y0 <= y1;
}
EPI_HD int record_words(const DevParams& hp, const epi_agent_record& a, AgentWords& w) {
    const int32_t G = hp.G;
    if (a.x < 0 || a.y < 0 || a.x > G || a.y > G || a.state > EPI_D || a.work_status > EPI_WS_NA ||
        a.immunity < -2 || a.immunity > 2 || a.infection_day > 0xFFFFu ||
        !rect_in_plane(G, a.home_x, a.home_y, a.home_x + 1, a.home_y + 1) ||
        (a.work_status != EPI_WS_NA && !rect_in_plane(G, a.work_x, a.work_y, a.work_x + 9, a.work_y + 9)) ||
        !rect_in_plane(G, a.area_x0, a.area_y0, a.area_x1, a.area_y1))
        return 1;
    bool ok = true;
    const uint32_t code = area_code_of(hp, a, &ok);
    if (!ok) return 2;
    uint32_t s = (uint32_t)a.state;
    if (a.flags & EPI_F_HOSPITALIZED) s |= kHosp;
    if (a.flags & EPI_F_ISOLATED) s |= kIso;
    if (a.flags & EPI_F_VACCINATED) s |= kVacc;
    if (a.flags & EPI_F_WORK_QUARANTINED) s |= kWq;
    if (a.flags & EPI_F_PUBLIC_TRANSPORT) s |= kPt;
    s |= code << kAreaShift;
    s |= (uint32_t)a.work_status << kWsShift;
    s |= (uint32_t)(a.immunity + 2) << kImmShift;
    s |= a.infection_day << kDayShift;
    w = AgentWords{pack_xy(a.x, a.y), s, a.at_hour, pack_xy(a.home_x, a.home_y), pack_xy(a.work_x, a.work_y),
                   a.work_start_at};
    return 0;
}

constexpr uint32_t kChunk = 256;  // agent slots per chunk; replicates start on chunk boundaries

// Bernoulli(p) as a threshold on a uniform 32-bit word: gen_bool(p) <=> u < thr.
inline uint64_t bernoulli_threshold(double p) {
    if (!(p > 0.0)) return 0ull;
    if (p >= 1.0) return 1ull << 32;
    return (uint64_t)(p * 4294967296.0);
}

// Uniform index in [0, k) from one 32-bit word (multiply-high).
EPI_HD uint32_t uniform_index(uint32_t u, uint32_t k) { return (uint32_t)(((uint64_t)u * (uint64_t)k) >> 32); }

// Rate class of get_current_transmission_rate(day), common/src/disease/mod.rs:88-95.
EPI_HD uint32_t rate_class(uint32_t reg_start, uint32_t high_start, uint32_t last_day, uint32_t day) {
    if (reg_start < day && day <= high_start) return 1u;
    if (high_start < day && day <= last_day) return 2u;
    return 0u;
}

// Philox4x32-10 (Salmon et al., SC'11): ten rounds of two 32x32->64 multiplies whose
// halves are crossed with the odd counter words and the round key; key += Weyl constants.
EPI_HD void philox4x32(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1,
                       uint32_t out[4]) {
    for (int r = 0; r < 10; ++r) {
#if defined(__CUDA_ARCH__)
        uint32_t hi_a = __umulhi(0xD2511F53u, c0), lo_a = 0xD2511F53u * c0;
        uint32_t hi_b = __umulhi(0xCD9E8D57u, c2), lo_b = 0xCD9E8D57u * c2;
#else
        uint64_t pa = 0xD2511F53ull * c0, pb = 0xCD9E8D57ull * c2;
        uint32_t hi_a = (uint32_t)(pa >> 32), lo_a = (uint32_t)pa;
        uint32_t hi_b = (uint32_t)(pb >> 32), lo_b = (uint32_t)pb;
#endif
        uint32_t t0 = hi_b ^ c1 ^ k0;
        uint32_t t2 = hi_a ^ c3 ^ k1;
        c0 = t0; c1 = lo_b; c2 = t2; c3 = lo_a;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

// Philox2x32-10 (same paper): (R0, R1) -> (hi(M R0) ^ key ^ R1, lo(M R0)), key += Weyl.
EPI_HD void philox2x32(uint32_t c0, uint32_t c1, uint32_t key, uint32_t out[2]) {
    for (int r = 0; r < 10; ++r) {
#if defined(__CUDA_ARCH__)
        const uint32_t hi = __umulhi(0xD256D193u, c0), lo = 0xD256D193u * c0;
#else
        const uint64_t pr = 0xD256D193ull * c0;
        const uint32_t hi = (uint32_t)(pr >> 32), lo = (uint32_t)pr;
#endif
        c0 = hi ^ key ^ c1;
        c1 = lo;
        key += 0x9E3779B9u;
    }
    out[0] = c0;
    out[1] = c1;
}

// Movement draws: Philox2x32-10 keyed by DevParams::move_key (word 0 of the Philox4x32
// block (0, kWorldHour, kBlkMoveKey, 0) of the seed), counter (agent | which, hour):
constexpr uint32_t kMoveChoice = 0u;        // word 0: Moore choice (movement) / death (hour 23)
constexpr uint32_t kMovePoint = 1u << 25;   // words 0,1: random point x, y

// Draw-block ids of the Philox4x32 counter word 2 (the layout every consumer shares).
enum DrawBlock : uint32_t {
    kBlkDisease = 1,  // Susceptible neighbours 0-3 | Exposed jitter, symptoms | Pre severe
    kBlkDisease2 = 2, // Susceptible neighbours 4-7
    kBlkVaccine = 3,
    kBlkCitizen = 16, // world build: working, public transport, hospital staff, immunity
    kBlkEssential = 17,
    kBlkHouse = 18,   // counter word 0 = house index
    kBlkInfectPick = 19,
    kBlkMoveKey = 20  // counter word 2 of the movement key's block
};

}  // namespace epi
