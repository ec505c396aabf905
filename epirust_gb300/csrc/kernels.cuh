// kernels.cuh -- the sm_103a kernels of the hourly tick, over one or many replicates.
//
// Agent slots of all replicates are concatenated; each replicate starts on a 256-slot chunk
// boundary, so a chunk belongs to one replicate (chunk_rep[c]; absent when there is one).
// The counting kernels walk chunks with a grid-stride loop, stage the chunk's replicate
// parameters in shared memory and flush their per-block histogram whenever the replicate
// changes; the commit kernel runs one thread per slot.  Philox counters and claim values use
// the agent's index within its replicate, so a replicate evolves exactly as a lone engine
// with the same parameters would.
//
// Per simulated hour (CitizenLocationMap::simulate, engine/src/allocation_map.rs:67-129):
//   hours 1..6 of a day   k_sleep   current_area = home (non-staff), counts
//   other hours           k_decide  per-agent rules on the previous-hour plane, proposals,
//                                   atomicMin claims on the target cells, counts
//                         k_commit  lowest claimant moves, losers stay, plane bytes updated;
//                                   claims stay (a later hour's keys are smaller, see claim_key)
#pragma once

#include "tick.cuh"

namespace epi {
namespace kern {

constexpr int kThreads = (int)kChunk;

// Programmatic dependent launch: the hour kernels are launched so that the next kernel's
// launch is set up while the one before it runs.  dep_wait() returns once every earlier
// kernel of the stream has completed and its writes are visible (a no-op for a normal
// launch), so each hour kernel calls it before its first global access.  The kernels signal
// nothing early: blocks of the next kernel resident (and waiting) beside the running one were
// measured 1.7 % slower per hour than letting them start at its completion.
__device__ __forceinline__ void dep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Warp-aggregated 6-bin histogram into shared memory: three ballots carry the bits of each
// lane's bin (invalid lanes vote bin 7), and lane b (< 6) counts the lanes whose bits spell b.
__device__ __forceinline__ void count_into(uint32_t* sh, bool valid, uint32_t bin) {
    const uint32_t v = valid ? bin : 7u;
    const uint32_t b0 = __ballot_sync(0xFFFFFFFFu, v & 1u), b1 = __ballot_sync(0xFFFFFFFFu, v & 2u),
                   b2 = __ballot_sync(0xFFFFFFFFu, v & 4u);
    const uint32_t lane = threadIdx.x & 31u;
    if (lane < 6u) {
        const uint32_t m = ((lane & 1u) ? b0 : ~b0) & ((lane & 2u) ? b1 : ~b1) & ((lane & 4u) ? b2 : ~b2);
        const uint32_t c = (uint32_t)__popc(m);
        if (c) atomicAdd(&sh[lane], c);
    }
}

// Consecutive chunks a block takes per grid-stride step.  An ensemble block that strides one
// chunk at a time switches replicate at nearly every step (a parameter reload and a
// histogram flush); groups of 8 made the 256-replicate ensemble 10 % faster.  A single world
// keeps 1: the plain stride, where the resident blocks sweep one contiguous band of agents,
// was measured fastest (groups of 2, 4, 8 were 2, 8, 15 % slower, a scattered chunk order
// 6 % slower).
constexpr uint32_t kEnsembleChunkGroup = 8;
constexpr uint32_t kWorldChunkGroup = 1;

// Block-uniform bookkeeping of the replicate a block is working on.
struct BlockRep {
    uint32_t r = 0xFFFFFFFFu;
};

// Hours run in chains of captured pieces (a piece ends at a day boundary) launched back to
// back; the chain's counts rows are [hour - first][replicate][8], words 0-5 the bins and
// word 6 the halt mark of the run loop's guard.  The hour of a launch is read on the device,
// so one captured piece serves every day.
struct SegDev {
    uint32_t hour_base;  // first hour of the piece now running (advanced by k_piece_end)
    uint32_t first;      // first hour of the chain
};
struct HourArgs {
    SegDev* seg;
    uint32_t* counts;    // the chain's rows
    uint32_t row_words;  // R * 8
    uint32_t offset;     // hour within the piece
    uint32_t prev_back;  // hours back to the previous computed row (0: the stop rule is off)
};
// The hour of a launch and its row in the chain.  The row pointers are recomputed where they
// are used (from kernel parameters) rather than held in registers across the kernel.
struct HourRow {
    uint32_t hour, row;
};
__device__ __forceinline__ HourRow hour_row(const HourArgs& a) {
    const uint32_t hour = a.seg->hour_base + a.offset;
    return HourRow{hour, hour - a.seg->first};
}
__device__ __forceinline__ uint32_t* row_ptr(const HourArgs& a, uint32_t row) {
    return a.counts + (size_t)row * a.row_words;
}
// The previous computed row: nullptr for the first hour of a chain and outside the run loop.
__device__ __forceinline__ const uint32_t* prev_ptr(const HourArgs& a, uint32_t row) {
    return (a.prev_back && row >= a.prev_back) ? a.counts + (size_t)(row - a.prev_back) * a.row_words : nullptr;
}

// The stop rule of run_single_engine (epidemiology_simulation.rs:564-575): a replicate whose
// last computed counts row (prev, [replicate][8]) has no exposed, infected or hospitalized
// agent has ended, and the later hours of the chain leave it untouched; so do they after a
// row the guard marked (an intervention fires there, and the host takes over).
__device__ __forceinline__ bool run_ended(const uint32_t* prev, uint32_t r) {
    if (!prev) return false;
    const uint32_t* c = prev + (size_t)r * 8u;
    return (c[1] | c[2] | c[3]) == 0u || c[6] != 0u;
}

// Switch the block to replicate r: flush the histogram of the previous one into its counts
// row (counts[r * 8 + bin]), stage r's parameters, clear the histogram.  Block-uniform.
__device__ __forceinline__ void switch_rep(BlockRep& br, uint32_t r, const DevParams* __restrict__ Pall, DevParams& sP,
                                           uint32_t* sh, uint32_t* counts) {
    __syncthreads();
    if (br.r != 0xFFFFFFFFu && threadIdx.x < 6 && sh[threadIdx.x]) atomicAdd(&counts[br.r * 8 + threadIdx.x], sh[threadIdx.x]);
    __syncthreads();
    for (uint32_t k = threadIdx.x; k < sizeof(DevParams) / 4; k += blockDim.x)
        reinterpret_cast<uint32_t*>(&sP)[k] = reinterpret_cast<const uint32_t*>(Pall + r)[k];
    if (threadIdx.x < 8) sh[threadIdx.x] = 0;
    __syncthreads();
    br.r = r;
}

__device__ __forceinline__ void flush_rep(const BlockRep& br, uint32_t* sh, uint32_t* counts) {
    __syncthreads();
    if (br.r != 0xFFFFFFFFu && threadIdx.x < 6 && sh[threadIdx.x]) atomicAdd(&counts[br.r * 8 + threadIdx.x], sh[threadIdx.x]);
}

// First vacant hospital cell of the snapshot in AreaIterator order (area.rs:131-148), found
// by the whole block; kNoAction when the hospital is full.
__device__ uint32_t block_first_vacant(const DevParams& P, const PlaneView& pl) {
    __shared__ uint32_t best;
    const Rect h = P.area[P.hosp_code];
    const uint32_t w = (uint32_t)(h.x1 - h.x0 + 1), total = w * (uint32_t)(h.y1 - h.y0 + 1);
    if (threadIdx.x == 0) best = kNoAction;
    __syncthreads();
    for (uint32_t base = 0; base < total; base += blockDim.x) {
        const uint32_t c = base + threadIdx.x;
        bool vac = false;
        if (c < total) vac = pl.vacant(h.x0 + (int32_t)(c % w), h.y0 + (int32_t)(c / w));
        if (vac) atomicMin(&best, c);
        if (__syncthreads_or(vac)) break;
    }
    const uint32_t c = best;
    __syncthreads();
    if (c == kNoAction) return kNoAction;
    return pack_xy(h.x0 + (int32_t)(c % w), h.y0 + (int32_t)(c / w));
}

// Hours 1..6 (SLEEP_START_TIME..=SLEEP_END_TIME, citizen/mod.rs:244-248).  A single world
// takes its chunks kSleepBatch at a time with all their state loads in flight together (the
// kernel is one load and a compare per agent, so one load round per chunk set its time).
constexpr uint32_t kSleepBatch = 4;

__device__ __forceinline__ void sleep_agent(uint2* __restrict__ st, uint32_t slot, bool valid, uint32_t s, uint32_t* sh) {
    if (valid && st_ws(s) != EPI_WS_HOSPITAL_STAFF && st_area(s) != kHome) st[slot].x = with_area(s, kHome);
    count_into(sh, valid, count_bin(s));
}

__global__ void __launch_bounds__(kThreads) k_sleep(const DevParams* __restrict__ Pall, const uint32_t* __restrict__ chunk_rep,
                                                    uint32_t n_chunks, uint2* __restrict__ st, HourArgs ha) {
    __shared__ uint32_t sh[8];
    __shared__ DevParams sP;
    dep_wait();
    const HourRow hr = hour_row(ha);
    BlockRep br;
    bool ended = false;  // run_ended of the block's replicate (its prev row is fixed during the launch)
    if (!chunk_rep) {
        if (blockIdx.x < n_chunks) {
            switch_rep(br, 0u, Pall, sP, sh, row_ptr(ha, hr.row));
            ended = run_ended(prev_ptr(ha, hr.row), 0u);
        }
        if (blockIdx.x < n_chunks && sP.active && !ended) {
            for (uint32_t c0 = blockIdx.x; c0 < n_chunks; c0 += kSleepBatch * gridDim.x) {
                uint32_t sv[kSleepBatch];
#pragma unroll
                for (uint32_t q = 0; q < kSleepBatch; ++q) {
                    const uint32_t c = c0 + q * gridDim.x, slot = c * kChunk + threadIdx.x;
                    sv[q] = (c < n_chunks && slot < sP.n) ? st[slot].x : 0u;  // slot = agent (agent_off 0)
                }
#pragma unroll
                for (uint32_t q = 0; q < kSleepBatch; ++q) {
                    const uint32_t c = c0 + q * gridDim.x, slot = c * kChunk + threadIdx.x;
                    if (c >= n_chunks) break;  // block-uniform
                    sleep_agent(st, slot, slot < sP.n, sv[q], sh);
                }
            }
        }
        flush_rep(br, sh, row_ptr(ha, hr.row));
        return;
    }
    const uint32_t grp = kEnsembleChunkGroup;  // chunks per stride step
    for (uint32_t c = blockIdx.x * grp, k = 0; c < n_chunks;
         c = (++k < grp) ? c + 1u : c + (gridDim.x - 1u) * grp + 1u, k = (k < grp) ? k : 0u) {
        const uint32_t r = chunk_rep ? chunk_rep[c] : 0u;
        if (r != br.r) {
            switch_rep(br, r, Pall, sP, sh, row_ptr(ha, hr.row));
            ended = run_ended(prev_ptr(ha, hr.row), r);
        }
        if (!sP.active || ended) continue;
        const uint32_t slot = c * kChunk + threadIdx.x;
        const bool valid = slot - sP.agent_off < sP.n;
        sleep_agent(st, slot, valid, valid ? st[slot].x : 0u, sh);
    }
    flush_rep(br, sh, row_ptr(ha, hr.row));
}

// The rules of one agent for the hour (slot valid): proposal, claim, infection update, state
// and target words.  Returns the agent's counts bin.  FULL (a lone world with two plane
// buffers, the hours whose commit rebuilds the plane): every agent's target word names its
// cell and class.
template <int HC, bool FULL = false>
__device__ __forceinline__ uint32_t decide_agent(const DevParams& P, const PlaneView& pl, uint32_t* __restrict__ rclaim,
                                                 uint32_t* __restrict__ wsa, uint2* __restrict__ st,
                                                 uint32_t* __restrict__ tgt, uint32_t* __restrict__ lost, uint32_t slot,
                                                 uint32_t i, uint32_t s, uint32_t at, uint32_t p, uint32_t hm, uint32_t wk,
                                                 uint32_t hour, uint32_t hod, uint32_t hosp_first, int* err) {
    const uint32_t s0 = s, at0 = at;
    const Cell cell{unpack_x(p), unpack_y(p)};
    Draws dr{i, hour, P.key0, P.key1, P.move_key};
    Cell nc;
    bool infect = false;
    if (HC == kHcStart) {
        nc = routine_start(P, pl, s, hm, cell, hosp_first, dr);
    } else if (HC == kHcEnd) {
        nc = routine_end(P, pl, s, hm, cell, dr);
    } else {
        const bool staff = st_ws(s) == EPI_WS_HOSPITAL_STAFF;
        uint32_t w0 = staff ? wsa[slot] : 0u, w = w0;
        nc = perform_movements<HC>(P, pl, s, w, hm, wk, cell, hod, hour, dr, infect);
        if (staff && w != w0) wsa[slot] = w;
    }
    bool moving = nc.x != cell.x || nc.y != cell.y;
    if (moving && ((uint32_t)nc.x > (uint32_t)P.G || (uint32_t)nc.y > (uint32_t)P.G)) {
        atomicOr(err, 4);  // unreachable for validated worlds; never write outside the plane
        moving = false;
        nc = cell;
    }
    // The claim goes out before the infection update so that its round trip overlaps it.
    const uint32_t key = claim_key(hour, i);
    const uint32_t old = moving ? atomicMin(&rclaim[(size_t)nc.y * P.W + nc.x], key) : kNoClaim;
    if (infect) infection_dynamics(P, pl, s, at, hm, wk, nc, hour, dr);
    if (moving) {
        // The claim that atomicMin finds names an agent this one competes with: of the two
        // the higher index loses.  Every claimant but the cell's lowest is named so, by
        // itself or by the claimant that displaced it, so the loss marks settle the cell
        // without a second read of the claim plane.
        if (lost && old != kNoClaim && (old >> kClaimAgentBits) == (key >> kClaimAgentBits)) {
            const uint32_t j = old & kMaxAgentsPerWorld;
            if (j < i) {
                moving = false;
                nc = cell;
            } else {
                lost[P.agent_off + j] = hour;
            }
        }
    }
    // the plane byte changes when the agent moves or its class changes (s == s0 keeps it)
    uint32_t t = kNoAction;
    if (moving || s != s0 || FULL) {
        const uint32_t cls0 = cell_class(P, s0), cls = s == s0 ? cls0 : cell_class(P, s);
        if (moving || cls != cls0 || FULL) t = encode_target(nc, cls, cls0);
    }
    tgt[slot] = t;
    if (s != s0 || at != at0) st[slot] = make_uint2(s, at);
    return count_bin(s);
}

// One hour of per-agent rules (hour of day 0, 7..22 or 23), specialised per hour class HC,
// over one world (ENS false: slot = agent, the parameters staged once) or the chunks of many
// replicates (ENS true: chunk_rep names each chunk's replicate).  The body is shared by two
// kernels that differ in their launch bounds: k_decide for a single world (registers left to
// the compiler) and k_decide_ens for ensembles (at least kEnsembleMinBlocks resident blocks:
// 48 registers), whose per-chunk replicate switches favour occupancy; each was measured
// faster on its own workload.
constexpr int kEnsembleMinBlocks = 5;

template <int HC, bool ENS, bool FULL = false>
__device__ __forceinline__ void decide_body(const DevParams* __restrict__ Pall, const uint32_t* __restrict__ chunk_rep,
                                            uint32_t n_chunks, const uint32_t* __restrict__ pos, uint2* __restrict__ st,
                                            const uint32_t* __restrict__ home, const uint32_t* __restrict__ work,
                                            uint32_t* __restrict__ wsa, const uint8_t* __restrict__ plane,
                                            const uint8_t* __restrict__ danger, uint32_t* __restrict__ claim,
                                            uint32_t* __restrict__ tgt, uint32_t* __restrict__ lost, const HourArgs& ha,
                                            int* err) {
    __shared__ uint32_t sh[8];
    __shared__ DevParams sP;
    const DevParams& P = sP;
    dep_wait();
    const HourRow hr = hour_row(ha);
    const uint32_t hour = hr.hour;
    const uint32_t hod = hour % 24u;
    BlockRep br;
    uint32_t hosp_first = kNoAction;
    bool hosp_known = false;
    if (!ENS) {
        if (blockIdx.x >= n_chunks) return;  // block-uniform: nothing to do or count
        switch_rep(br, 0u, Pall, sP, sh, row_ptr(ha, hr.row));
        if (P.active && !run_ended(prev_ptr(ha, hr.row), 0u)) {
            const PlaneView pl{plane + P.plane_off, P.G, P.WP, err, danger ? danger + P.plane_off : nullptr};
            uint32_t* rclaim = claim + P.claim_off;
            const uint32_t n = P.n;
            for (uint32_t c = blockIdx.x; c < n_chunks; c += gridDim.x) {
                const uint32_t slot = c * kChunk + threadIdx.x;  // = agent index (a lone world starts at slot 0)
                const bool valid = slot < n;
                uint32_t s = 0, at = 0, p = 0;
                if (valid) {
                    const uint2 sv = st[slot];
                    s = sv.x;
                    at = sv.y;
                    p = pos[slot];
                }
                if (HC == kHcStart) {
                    const bool need = valid && wants_hospital(P, infected(s) ? with_day(s, st_day(s) + 1u) : s);
                    if (__syncthreads_or(need) && !hosp_known) {
                        hosp_first = block_first_vacant(P, pl);
                        hosp_known = true;
                    }
                }
                const uint32_t bin = valid ? decide_agent<HC, FULL>(P, pl, rclaim, wsa, st, tgt, lost, slot, slot, s, at, p,
                                                                    home[slot], work[slot], hour, hod, hosp_first, err)
                                           : 0u;
                count_into(sh, valid, bin);
            }
        }
        flush_rep(br, sh, row_ptr(ha, hr.row));
        return;
    }
    bool ended = false;
    const uint32_t grp = kEnsembleChunkGroup;  // chunks per stride step
    // The replicate of the next chunk is read one chunk ahead, and a chunk's agent words are
    // read before its replicate is known (every chunk of an ensemble is whole in the slot
    // arrays), so neither waits on the other.
    auto next_chunk = [&](uint32_t c, uint32_t k) { return k + 1u < grp ? c + 1u : c + (gridDim.x - 1u) * grp + 1u; };
    uint32_t r_next = blockIdx.x * grp < n_chunks ? chunk_rep[blockIdx.x * grp] : 0u;
    for (uint32_t c = blockIdx.x * grp, k = 0; c < n_chunks; c = next_chunk(c, k), k = (k + 1u < grp) ? k + 1u : 0u) {
        const uint32_t r = r_next;
        const uint32_t cn = next_chunk(c, k);
        r_next = cn < n_chunks ? chunk_rep[cn] : 0u;
        const uint32_t slot = c * kChunk + threadIdx.x;
        const uint2 sv = st[slot];
        const uint32_t pw = pos[slot], hw = home[slot], ww = work[slot];
        if (r != br.r) {
            switch_rep(br, r, Pall, sP, sh, row_ptr(ha, hr.row));
            hosp_known = false;
            ended = run_ended(prev_ptr(ha, hr.row), r);  // an earlier row: fixed during the launch
        }
        if (!P.active || ended) continue;
        const PlaneView pl{plane + P.plane_off, P.G, P.WP, err, danger ? danger + P.plane_off : nullptr};
        uint32_t* rclaim = claim + P.claim_off;
        const uint32_t i = slot - P.agent_off;  // index within the replicate
        const bool valid = i < P.n;
        const uint32_t s = valid ? sv.x : 0u, at = valid ? sv.y : 0u, p = valid ? pw : 0u;
        if (HC == kHcStart) {
            const bool need = valid && wants_hospital(P, infected(s) ? with_day(s, st_day(s) + 1u) : s);
            if (__syncthreads_or(need) && !hosp_known) {
                hosp_first = block_first_vacant(P, pl);
                hosp_known = true;
            }
        }
        const uint32_t bin = valid ? decide_agent<HC>(P, pl, rclaim, wsa, st, tgt, lost, slot, i, s, at, p, hw, ww, hour,
                                                      hod, hosp_first, err)
                                   : 0u;
        count_into(sh, valid, bin);
    }
    flush_rep(br, sh, row_ptr(ha, hr.row));
}

#define EPI_DECIDE_PARAMS                                                                                              \
    const DevParams *__restrict__ Pall, const uint32_t *__restrict__ chunk_rep, uint32_t n_chunks,                    \
        const uint32_t *__restrict__ pos, uint2 *__restrict__ st, const uint32_t *__restrict__ home,                  \
        const uint32_t *__restrict__ work, uint32_t *__restrict__ wsa, const uint8_t *__restrict__ plane,             \
        const uint8_t *__restrict__ danger, uint32_t *__restrict__ claim, uint32_t *__restrict__ tgt,                 \
        uint32_t *__restrict__ lost, HourArgs ha, int *err
template <int HC, bool FULL = false>
__global__ void __launch_bounds__(kThreads) k_decide(EPI_DECIDE_PARAMS) {
    decide_body<HC, false, FULL>(Pall, chunk_rep, n_chunks, pos, st, home, work, wsa, plane, danger, claim, tgt, lost, ha,
                                 err);
}
template <int HC>
__global__ void __launch_bounds__(kThreads, kEnsembleMinBlocks) k_decide_ens(EPI_DECIDE_PARAMS) {
    decide_body<HC, true>(Pall, chunk_rep, n_chunks, pos, st, home, work, wsa, plane, danger, claim, tgt, lost, ha, err);
}
#undef EPI_DECIDE_PARAMS

// Resolve the claims of the hour: the lowest index that claimed a cell moves there
// (the serial resolve of allocation_map.rs:93-102 in index order), others keep their cell.
// With loss marks (lost != nullptr) a mover wins unless k_decide marked it beaten this
// hour; without them the winner is read from the claim plane.  Each thread takes S slots a
// block-width apart (S chosen by the launch-shape autotuner), issuing all their independent
// loads first; the grid covers every slot once (a grid-stride loop here measured 1 % slower).
// SPARSE (hours of day 0 and 23, where a few agents in a million move or change class) reads
// the target words first and the position and loss mark only of the slots that act: about
// 5 us per launch at 1M agents instead of 9-10 us.
// REBUILD (a lone world with two plane buffers, the hours of day 7..22): `plane` is the other
// buffer, all zero, and every agent writes its final cell's byte there (one scattered store
// per agent instead of a cleared and a set byte per mover; k_decide then names every agent's
// cell and class in its target word).  The launch then zeroes `spent`, the buffer the hour
// read (clear_words 16-byte words), which the next rebuilding hour fills: nothing reads it
// any more.
constexpr int kCommitSlots = 4;   // default S
constexpr int kMaxCommitSlots = 8;

template <int S, bool SPARSE = false, bool REBUILD = false>
__global__ void __launch_bounds__(kThreads) k_commit(const DevParams* __restrict__ Pall, const uint32_t* __restrict__ chunk_rep,
                                                     uint32_t n_slots, uint32_t* __restrict__ pos,
                                                     const uint32_t* __restrict__ tgt, uint8_t* __restrict__ plane,
                                                     uint8_t* __restrict__ danger, uint32_t* __restrict__ claim,
                                                     const uint32_t* __restrict__ lost, HourArgs ha, uint64_t clear_cells,
                                                     uint4* __restrict__ spent, uint32_t clear_words) {
    dep_wait();
    const HourRow hr = hour_row(ha);
    const uint32_t* prev = prev_ptr(ha, hr.row);
    const uint32_t hour = hr.hour;
    // a single world's parameters once per thread; an ensemble looks each slot's replicate up
    const bool one = chunk_rep == nullptr;
    const uint32_t off0 = one ? Pall[0].agent_off : 0u, wp0 = one ? (uint32_t)Pall[0].WP : 0u;
    const bool halted0 = one && (!Pall[0].active || run_ended(prev, 0u));  // the world does nothing this hour
    {
        const uint32_t base = blockIdx.x * (blockDim.x * S) + threadIdx.x;
        uint32_t t[S], p[S], l[S];
#pragma unroll
        for (int k = 0; k < S; ++k) {
            const uint32_t slot = base + k * blockDim.x;
            t[k] = slot < n_slots ? tgt[slot] : kNoAction;
            p[k] = !SPARSE && slot < n_slots ? pos[slot] : 0u;
            l[k] = !SPARSE && lost && slot < n_slots ? lost[slot] : 0u;
        }
#pragma unroll(SPARSE ? 1 : S)
        for (int k = 0; k < S; ++k) {
            if (t[k] == kNoAction) continue;
            const uint32_t slot = base + k * blockDim.x;
            const uint32_t pk = SPARSE ? pos[slot] : p[k];
            const uint32_t lk = SPARSE ? (lost ? lost[slot] : 0u) : l[k];
            uint32_t r = 0u, off = off0, WP = wp0;
            uint64_t plane_off = 0u;
            bool halted = halted0;
            if (!one) {
                r = chunk_rep[slot / kChunk];
                const DevParams& P = Pall[r];
                off = P.agent_off;
                WP = (uint32_t)P.WP;
                plane_off = P.plane_off;
                halted = !P.active || run_ended(prev, r);
            }
            if (halted) continue;
            const uint32_t xy = target_xy(t[k]), cls = target_class(t[k]), cls0 = target_old_class(t[k]);
            bool win = false;
            if (xy != pk) {
                if (lost) {
                    win = lk != hour;
                } else {
                    const DevParams& P = Pall[r];
                    win = claim[P.claim_off + (size_t)unpack_y(xy) * (uint32_t)P.W + unpack_x(xy)] ==
                          claim_key(hour, slot - off);
                }
            }
            uint8_t* rplane = plane + plane_off;
            const size_t old_cell = (size_t)(unpack_y(pk) + 1) * WP + (unpack_x(pk) + 1);
            size_t new_cell = old_cell;
            if (win) {
                new_cell = (size_t)(unpack_y(xy) + 1) * WP + (unpack_x(xy) + 1);
                pos[slot] = xy;
            }
            if (REBUILD) {
                rplane[new_cell] = (uint8_t)cls;
            } else if (win) {
                rplane[old_cell] = 0;
                rplane[new_cell] = (uint8_t)cls;
            } else if (cls != cls0) {  // a beaten mover whose class held keeps its byte as it is
                rplane[old_cell] = (uint8_t)cls;
            }
            // infectious-neighbour counts follow infectious agents that move or stop or start
            // being infectious (rare: a few agents per hour)
            const bool inf0 = cls0 >= 2u, inf1 = cls >= 2u;
            if (danger && (inf0 || inf1) && (inf0 != inf1 || new_cell != old_cell)) {
                uint8_t* rd = danger + plane_off;
                if (inf0) danger_add(rd, old_cell, WP, -1);
                if (inf1) danger_add(rd, new_cell, WP, +1);
            }
        }
    }
    // the spent buffer of a rebuilding hour (not when the world did nothing: it still holds the plane)
    if (REBUILD && !halted0)
        for (uint32_t w = blockIdx.x * blockDim.x + threadIdx.x; w < clear_words; w += gridDim.x * blockDim.x)
            spent[w] = make_uint4(0u, 0u, 0u, 0u);
    // A new claim window (kClaimWindow hours) opens before the next hour that claims (hour of
    // day 0 claims next at 7): every claim plane is reset for it.  Only with loss marks, where
    // this kernel reads no claim.
    if (clear_cells && lost) {
        const uint32_t next = hour % 24u == 0u ? hour + 7u : hour + 1u;
        if (next / kClaimWindow != hour / kClaimWindow)
            for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < clear_cells; i += (size_t)gridDim.x * blockDim.x)
                claim[i] = kNoClaim;
    }
}

// End of a piece: the run loop's guard at a day boundary (row `guard_offset` of the piece;
// kNoGuard for none), then the piece's hours are added to the chain's hour base.  The guard
// evaluates the data-dependent triggers of process_interventions -- lockdown when infected >
// its threshold, a new hospital when the day's new infections (infected minus the previous
// boundary's figure, floored at 0) reach the spread threshold or hospitalized reaches the
// occupancy threshold -- for every replicate whose row ran, keeping the new-infections figure
// per replicate in ivn; if any fires, the row of every replicate gets the halt mark, and the
// rest of the chain does nothing.  One block.
constexpr uint32_t kNoGuard = 0xFFFFFFFFu;

__global__ void k_piece_end(const DevParams* __restrict__ Pall, uint32_t R, SegDev* seg, uint32_t* counts,
                            uint32_t row_words, uint32_t guard_offset, uint32_t advance, uint32_t* __restrict__ ivn) {
    __shared__ int fire;
    if (threadIdx.x == 0) fire = 0;
    __syncthreads();
    if (guard_offset != kNoGuard) {
        uint32_t* rows = counts + (size_t)(seg->hour_base + guard_offset - seg->first) * row_words;
        for (uint32_t r = threadIdx.x; r < R; r += blockDim.x) {
            const DevParams& P = Pall[r];
            const uint32_t* c = rows + (size_t)r * 8u;
            if (!P.active || (c[0] | c[1] | c[2] | c[3] | c[4] | c[5]) == 0u) continue;  // the hour did not run
            const uint32_t infected = c[2], hospitalized = c[3];
            const uint32_t fresh = infected > ivn[r] ? infected - ivn[r] : 0u;
            ivn[r] = fresh;
            const bool f = ((P.guard_flags & kGuardLock) && infected > P.lock_threshold) ||
                           ((P.guard_flags & kGuardSpread) && fresh >= P.spread_threshold) ||
                           ((P.guard_flags & kGuardOccupancy) && hospitalized >= P.occ_threshold);
            if (f) fire = 1;
        }
        __syncthreads();
        if (fire)
            for (uint32_t r = threadIdx.x; r < R; r += blockDim.x) rows[(size_t)r * 8u + 6u] = 1u;
    }
    __syncthreads();
    if (advance && threadIdx.x == 0) seg->hour_base += advance;
}

// Plane bytes of every agent of every replicate (world upload).
__global__ void k_build_plane(const DevParams* __restrict__ Pall, const uint32_t* __restrict__ chunk_rep, uint32_t n_slots,
                              const uint32_t* __restrict__ pos, const uint2* __restrict__ st, uint8_t* __restrict__ plane,
                              uint8_t* __restrict__ danger, int* err) {
    for (uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x; slot < n_slots; slot += gridDim.x * blockDim.x) {
        const DevParams& P = Pall[chunk_rep ? chunk_rep[slot / kChunk] : 0u];
        if (slot - P.agent_off >= P.n) continue;
        const uint32_t p = pos[slot];
        const int32_t x = unpack_x(p), y = unpack_y(p);
        if (x > P.G || y > P.G) { atomicOr(err, 2); continue; }
        const size_t c = (size_t)(y + 1) * P.WP + (x + 1);
        const uint32_t cls = cell_class(P, st[slot].x);
        plane[P.plane_off + c] = (uint8_t)cls;
        if (danger && cls >= 2u) danger_add(danger + P.plane_off, c, (uint32_t)P.WP, +1);
    }
}

// LockdownIntervention apply / revoke (allocation_map.rs:349-365) on slots [off, off + n).
__global__ void k_lock(uint2* __restrict__ st, uint32_t off, uint32_t n, int on) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t s = st[off + i].x;
        uint32_t ns = on ? (st_ws(s) != EPI_WS_ESSENTIAL ? (s | kIso) : s) : (s & ~kIso);
        if (ns != s) st[off + i].x = ns;
    }
}

// vaccinate (allocation_map.rs:381-387): susceptible agents with Philox block 3 word 0 < thr.
__global__ void k_vaccinate(uint2* __restrict__ st, uint32_t off, uint32_t n, uint32_t key0, uint32_t key1,
                            uint32_t hour, uint64_t thr) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t s = st[off + i].x;
        if ((s & kStateMask) != EPI_S) continue;
        uint32_t u[4];
        philox4x32(i, hour, kBlkVaccine, 0u, key0, key1, u);
        if ((uint64_t)u[0] < thr) st[off + i].x = s | kVacc;
    }
}

// Invariants: each agent's cell holds its class.
__global__ void k_check_agents(const DevParams* __restrict__ Pall, const uint32_t* __restrict__ chunk_rep,
                               uint32_t n_slots, const uint32_t* __restrict__ pos, const uint2* __restrict__ st,
                               const uint8_t* __restrict__ plane, unsigned long long* bad) {
    for (uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x; slot < n_slots; slot += gridDim.x * blockDim.x) {
        const DevParams& P = Pall[chunk_rep ? chunk_rep[slot / kChunk] : 0u];
        if (slot - P.agent_off >= P.n) continue;
        const uint32_t p = pos[slot];
        const int32_t x = unpack_x(p), y = unpack_y(p);
        if (x > P.G || y > P.G || plane[P.plane_off + (size_t)(y + 1) * P.WP + (x + 1)] != cell_class(P, st[slot].x))
            atomicAdd(bad, 1ull);
    }
}

// Citizen-state stream: one byte per agent for the hour -- bits 0-3 the step taken since the
// previous hour (0 none, 1 + k for the k-th Moore neighbour in NeighborIterator order, 15 a
// jump recorded as an exception {agent, x | y << 16}), bits 4-6 the state letter
// (CitizenState::state_str, models/events/citizen_state.rs:33-44: s e i r d = 0..4).
// prev holds each agent's cell at the previous record.  Single world (slot = agent).
__device__ __forceinline__ uint32_t state_letter(uint32_t s) {
    const uint32_t v = s & kStateMask;
    return v == EPI_S ? 0u : v == EPI_E ? 1u : v == EPI_R ? 3u : v == EPI_D ? 4u : 2u;
}

__global__ void k_state_delta(uint32_t n, const uint32_t* __restrict__ pos, const uint2* __restrict__ st,
                              uint32_t* __restrict__ prev, uint8_t* __restrict__ codes, uint2* __restrict__ exc,
                              uint32_t* __restrict__ exc_count) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < n;
    uint32_t code = 0u, p = 0u;
    bool jump = false;
    if (valid) {
        p = pos[i];
        const uint32_t q = prev[i];
        const int32_t dx = unpack_x(p) - unpack_x(q), dy = unpack_y(p) - unpack_y(q);
        uint32_t step = 0u;
        if (dx != 0 || dy != 0) {
            if (dx >= -1 && dx <= 1 && dy >= -1 && dy <= 1) {
                const int k9 = (dy + 1) * 3 + (dx + 1);     // row-major 3x3 index, centre 4
                step = 1u + (uint32_t)(k9 < 4 ? k9 : k9 - 1);  // NeighborIterator order
            } else {
                step = 15u;
                jump = true;
            }
            prev[i] = p;
        }
        code = step | (state_letter(st[i].x) << 4);
        codes[i] = (uint8_t)code;
    }
    // exceptions: one atomic per warp, lanes in order
    const uint32_t lane = threadIdx.x & 31u, m = __ballot_sync(0xFFFFFFFFu, jump);
    if (m) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(exc_count, (uint32_t)__popc(m));
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if (jump) exc[base + (uint32_t)__popc(m & ((1u << lane) - 1u))] = make_uint2(i, p);
    }
}

// Cells of [0, G]^2 whose infectious-neighbour count differs from the 3x3 of the plane
// (replicates r = blockIdx.y, blockIdx.y + gridDim.y, ...).
__global__ void k_check_danger(const DevParams* __restrict__ Pall, uint32_t R, const uint8_t* __restrict__ plane,
                               const uint8_t* __restrict__ danger, unsigned long long* bad) {
    unsigned long long b = 0;
    for (uint32_t r = blockIdx.y; r < R; r += gridDim.y) {
        const DevParams& P = Pall[r];
        const uint32_t side = (uint32_t)P.G + 1u, cells = side * side, WP = (uint32_t)P.WP;
        const uint8_t* pl = plane + P.plane_off;
        const uint8_t* dg = danger + P.plane_off;
        for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < cells; q += gridDim.x * blockDim.x) {
            const size_t c = (size_t)(q / side + 1) * WP + (q % side + 1);
            const uint32_t n = (pl[c - WP - 1] >= 2u) + (pl[c - WP] >= 2u) + (pl[c - WP + 1] >= 2u) +
                               (pl[c - 1] >= 2u) + (pl[c + 1] >= 2u) + (pl[c + WP - 1] >= 2u) + (pl[c + WP] >= 2u) +
                               (pl[c + WP + 1] >= 2u);
            b += n != dg[c];
        }
    }
    if (b) atomicAdd(bad, b);
}

// Occupied plane bytes over the whole buffer (borders and slack included: they must be 0).
__global__ void k_check_plane(size_t plane_bytes, const uint8_t* __restrict__ plane, unsigned long long* occupied) {
    unsigned long long o = 0;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < plane_bytes; k += stride) o += plane[k] != 0;
    for (int off = 16; off; off >>= 1) o += __shfl_down_sync(0xFFFFFFFFu, o, off);
    if ((threadIdx.x & 31) == 0 && o) atomicAdd(occupied, o);
}

}  // namespace kern
}  // namespace epi
