// world.cuh -- the Auto-population world build on the device, equal to the host build
// (host.cpp:build_world) and to the oracle's, byte for byte.
//
// generate_population / create_citizen (engine/src/geography/grid.rs:83-123,
// engine/src/citizen/citizen_factory.rs:58-88): agent i lives in house i mod houses and works
// (if it works) in office i mod offices; its Philox block (i, world hour, citizen block)
// decides working, public transport, hospital staff and immunity.  Everything is per agent
// except the public-transport budget -- the first transport_points eligible agents in index
// order get it -- which is a prefix count: per-chunk counts, one exclusive scan over the
// chunks, and a rank within the chunk.  The starting infections (a partial Fisher-Yates
// shuffle over a few agents) come from the host plan as a list.
#pragma once

#include "kernels.cuh"

namespace epi {
namespace kern {

// One world's build constants (WorldPlan in device form).
struct WorldDev {
    uint32_t n, agent_off, first_chunk;
    uint32_t houses, houses_x, offices, offices_x;
    int32_t hx0, hy0, ox0, oy0;  // housing and work-area origins
    uint32_t key0, key1;
    uint32_t transport_points;
    uint32_t csv;  // 1: working and public transport come from the population flags
    uint64_t thr_work, thr_pt, thr_staff, thr_ess;
};

// Citizens of every world (one 256-agent chunk per block iteration).  elig[slot] = 1 for
// agents that would take public transport if the budget allowed; chunk_elig[c] counts them.
// flags[slot] (bit 0 working, bit 1 public transport) replace the draws of Csv worlds.
__global__ void __launch_bounds__(kThreads) k_world_citizens(const WorldDev* __restrict__ W,
                                                             const uint32_t* __restrict__ chunk_rep, uint32_t n_chunks,
                                                             uint32_t* __restrict__ pos, uint2* __restrict__ st,
                                                             uint32_t* __restrict__ home, uint32_t* __restrict__ work,
                                                             uint32_t* __restrict__ wsa, uint32_t* __restrict__ elig,
                                                             uint32_t* __restrict__ chunk_elig,
                                                             const uint8_t* __restrict__ flags) {
    for (uint32_t c = blockIdx.x; c < n_chunks; c += gridDim.x) {
        const WorldDev& w = W[chunk_rep ? chunk_rep[c] : 0u];
        const uint32_t slot = c * kChunk + threadIdx.x;
        const uint32_t i = slot - w.agent_off;
        bool e = false;
        if (i < w.n) {
            uint32_t u[4];
            philox4x32(i, kWorldHour, kBlkCitizen, 0u, w.key0, w.key1, u);
            const uint32_t fl = w.csv ? flags[slot] : 0u;
            const bool working = w.csv ? (fl & 1u) != 0u : (uint64_t)u[0] < w.thr_work;
            const uint32_t house = i % w.houses, office = i % w.offices;
            const int32_t hx = w.hx0 + 2 * (int32_t)(house % w.houses_x), hy = w.hy0 + 2 * (int32_t)(house / w.houses_x);
            const int32_t ox = w.ox0 + 10 * (int32_t)(office % w.offices_x), oy = w.oy0 + 10 * (int32_t)(office / w.offices_x);
            e = !w.csv && working && (uint64_t)u[1] < w.thr_pt;
            // Auto: a non-worker's work area is its house; Csv (from_record): the cycled office
            uint32_t ws = EPI_WS_NA, start = 0u, wk = w.csv ? pack_xy(ox, oy) : pack_xy(hx, hy);
            if (working) {
                wk = pack_xy(ox, oy);
                if ((uint64_t)u[2] < w.thr_staff) {
                    ws = EPI_WS_HOSPITAL_STAFF;
                    start = 8u;
                } else {
                    uint32_t v[4];  // essential workers among the normal ones (lockdown only)
                    philox4x32(i, kWorldHour, kBlkEssential, 0u, w.key0, w.key1, v);
                    ws = (uint64_t)v[0] < w.thr_ess ? EPI_WS_ESSENTIAL : EPI_WS_NORMAL;
                }
            }
            const uint32_t imm = uniform_index(u[3], 5u);  // immunity + 2
            // place in the house: alone -> a random cell of the 2x2, else by rank
            const uint32_t rank = i / w.houses, in_house = (w.n - 1u - house) / w.houses + 1u;
            int32_t x = hx + (int32_t)(rank >> 1), y = hy + (int32_t)(rank & 1u);
            if (in_house == 1u) {
                uint32_t h[4];
                philox4x32(house, kWorldHour, kBlkHouse, 0u, w.key0, w.key1, h);
                x = hx + (int32_t)uniform_index(h[0], 2u);
                y = hy + (int32_t)uniform_index(h[1], 2u);
            }
            pos[slot] = pack_xy(x, y);
            home[slot] = pack_xy(hx, hy);
            work[slot] = wk;
            wsa[slot] = start;
            st[slot] = make_uint2((uint32_t)EPI_S | (kHome << kAreaShift) | (ws << kWsShift) | (imm << kImmShift) |
                                      ((fl & 2u) ? kPt : 0u),
                                  0u);
        }
        elig[slot] = e ? 1u : 0u;
        const int cnt = __syncthreads_count(e);
        if (threadIdx.x == 0) chunk_elig[c] = (uint32_t)cnt;
    }
}

// In-place exclusive prefix sum of v[0..n) by one block (tiles of blockDim.x, carried).
__global__ void k_world_scan(uint32_t* __restrict__ v, uint32_t n) {
    __shared__ uint32_t warp_sum[32];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (uint32_t base = 0; base < n; base += blockDim.x) {
        const uint32_t k = base + threadIdx.x;
        const uint32_t x = k < n ? v[k] : 0u;
        uint32_t incl = x;  // inclusive scan within the warp
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= (uint32_t)o) incl += y;
        }
        if (lane == 31) warp_sum[wid] = incl;
        __syncthreads();
        if (wid == 0) {
            uint32_t ws = lane < nw ? warp_sum[lane] : 0u, wi = ws;
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, wi, o);
                if (lane >= (uint32_t)o) wi += y;
            }
            if (lane < nw) warp_sum[lane] = wi - ws;  // exclusive warp offsets
        }
        __syncthreads();
        const uint32_t total_before = carry;
        if (k < n) v[k] = total_before + warp_sum[wid] + incl - x;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry = total_before + warp_sum[wid] + incl;
        __syncthreads();
    }
}

// Public transport for the first transport_points eligible agents of every world.
__global__ void __launch_bounds__(kThreads) k_world_pt(const WorldDev* __restrict__ W, const uint32_t* __restrict__ chunk_rep,
                                                       uint32_t n_chunks, const uint32_t* __restrict__ elig,
                                                       const uint32_t* __restrict__ chunk_prefix, uint2* __restrict__ st) {
    __shared__ uint32_t warp_cnt[kThreads / 32];
    const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
    for (uint32_t c = blockIdx.x; c < n_chunks; c += gridDim.x) {
        const WorldDev& w = W[chunk_rep ? chunk_rep[c] : 0u];
        const uint32_t slot = c * kChunk + threadIdx.x;
        const bool e = elig[slot] != 0u;
        const uint32_t m = __ballot_sync(0xFFFFFFFFu, e);
        if (lane == 0) warp_cnt[wid] = (uint32_t)__popc(m);
        __syncthreads();
        uint32_t before = 0;
        for (uint32_t k = 0; k < wid; ++k) before += warp_cnt[k];
        before += (uint32_t)__popc(m & ((1u << lane) - 1u));
        const uint32_t rank = chunk_prefix[c] - chunk_prefix[w.first_chunk] + before;
        if (e && rank < w.transport_points) st[slot].x |= kPt;
        __syncthreads();
    }
}

// Starting infections {slot, state, infection day}.
__global__ void k_world_infect(const uint4* __restrict__ list, uint32_t count, uint2* __restrict__ st) {
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
        const uint4 f = list[k];
        uint2 s = st[f.x];
        s.x = with_day(with_state(s.x, f.y), f.z);
        s.y = 0u;
        st[f.x] = s;
    }
}

// Caller-supplied agent records (the host layout, copied to the device as they are, record i
// of replicate r at slot agent_off(r) + i) into the SoA words, one slot per thread; slots past
// a replicate's agents are zeroed.  A record that fails record_words leaves slot << 1 |
// (kind - 1) in *bad by atomicMin, so *bad names the first bad record in (replicate, index)
// order.
__global__ void __launch_bounds__(kThreads) k_pack_records(const DevParams* __restrict__ Pall,
                                                           const uint32_t* __restrict__ chunk_rep, uint32_t n_slots,
                                                           const epi_agent_record* __restrict__ recs,
                                                           uint32_t* __restrict__ pos, uint2* __restrict__ st,
                                                           uint32_t* __restrict__ home, uint32_t* __restrict__ work,
                                                           uint32_t* __restrict__ wsa, unsigned long long* __restrict__ bad) {
    for (uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x; slot < n_slots; slot += gridDim.x * blockDim.x) {
        const DevParams& P = Pall[chunk_rep ? chunk_rep[slot / kChunk] : 0u];
        AgentWords w{0u, 0u, 0u, 0u, 0u, 0u};
        if (slot - P.agent_off < P.n) {
            const int kind = record_words(P, recs[slot], w);
            if (kind) {
                atomicMin(bad, ((unsigned long long)slot << 1) | (unsigned long long)(kind - 1));
                w = AgentWords{0u, 0u, 0u, 0u, 0u, 0u};
            }
        }
        pos[slot] = w.pos;
        st[slot] = make_uint2(w.s, w.at);
        home[slot] = w.home;
        work[slot] = w.work;
        wsa[slot] = w.wsa;
    }
}

}  // namespace kern
}  // namespace epi
