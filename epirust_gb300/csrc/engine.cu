// engine.cu -- the engine handle and the C ABI of the GB300 tick.
//
// An engine holds R worlds ("replicates") on one device: their agents are concatenated in
// 256-slot chunks, their bordered byte planes and claim planes laid end to end, and every
// kernel of kernels.cuh serves all of them in one launch per hour.  The single-engine API
// (epi_engine_*) is the R = 1 case; the ensemble API (epi_ensemble_*) runs many replicates
// of uneven population and grid size in lockstep.  Hour segments between intervention
// points run as one captured CUDA graph, replayed with the first hour read on the device.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <utility>
#include <vector>

#include "../../include/epi_surrogate.h"
#include "host.hpp"
#include "kernels.cuh"
#include "world.cuh"

using namespace epi;
using namespace epi::kern;

enum KernelKind { kKDecide = 0, kKCommit, kKSleep, kKLock, kKVaccinate, kKBuildPlane, kKCheck, kKindCount };
static const char* kKernelNames[kKindCount] = {"k_decide", "k_commit", "k_sleep", "k_lock", "k_vaccinate", "k_build_plane", "k_check"};

// A timed kernel launch: its kind and the events recorded around it.
struct TimedLaunch {
    int kind;
    cudaEvent_t begin, end;
    bool pooled;  // the pair returns to the engine's pool once read
};

// One world on the device.
struct Replica {
    epi_params p{};
    epi_geography geo0{}, geo{};
    DevParams hp{};
    uint32_t n = 0;
    InterventionState iv;
    std::vector<epi_counts> rows;
    bool active = true;
    // checkpoint of the host-side state (epi_engine_save_state)
    InterventionState s_iv;
    epi_geography s_geo{};
    uint32_t s_hosp_code = kHosp0;
    bool s_active = true;
    std::vector<epi_counts> s_rows;
};

struct epi_engine {
    std::vector<Replica> reps;
    uint32_t slots = 0;        // agent slots (chunk-padded replicates)
    size_t plane_bytes = 0;    // all bordered byte planes
    size_t claim_cells = 0;    // all claim planes
    int grid_blocks = 0;       // grid of the counting kernels (k_decide, k_sleep)
    int commit_slots = kCommitSlots;  // slots per k_commit thread and round (1 .. 8)
    int commit_blocks = 0;
    int resident_blocks = 0;   // SMs x resident k_decide blocks per SM
    // device
    DevParams* d_params = nullptr;
    uint32_t* d_chunk_rep = nullptr;  // null for a single replicate
    uint32_t *d_pos = nullptr, *d_home = nullptr, *d_work = nullptr, *d_wsa = nullptr, *d_tgt = nullptr;
    uint32_t* d_lost = nullptr;  // per slot: the hour in which the agent's claim was beaten
    uint2* d_st = nullptr;
    // Byte planes of all replicates (plane_bytes).  A lone world keeps two (two_planes): the
    // hours of day 7..22 rebuild the plane in the other one, and plane_par names the one
    // holding the current state.
    uint8_t* d_plane = nullptr;
    bool two_planes = false;
    uint32_t plane_par = 0;
    uint8_t* d_danger = nullptr;  // infectious-neighbour counts, same layout as d_plane
    uint32_t* d_claim = nullptr;
    uint32_t* d_counts = nullptr;  // [hour of segment][replicate][8]
    SegDev* d_seg = nullptr;       // hour base of the running piece and first hour of the chain
    uint32_t* d_ivn = nullptr;     // per replicate: the guard's new-infections figure
    int* d_err = nullptr;
    unsigned long long* d_scratch = nullptr;
    uint32_t counts_capacity = 0;  // hours
    // host
    uint32_t* h_counts = nullptr;  // pinned mirror of d_counts
    SegDev* h_seg = nullptr;       // pinned staging of d_seg and d_ivn
    uint32_t* h_ivn = nullptr;
    int halt_row = -1;             // chain offset of the row the guard marked in the last chain
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    // piece graphs by (first hour mod 24, hours, profiling | stream << 1 | run loop << 2); a
    // profiling graph carries an event-record node before and after each kernel
    struct HourGraph {
        cudaGraphExec_t exec = nullptr;
        std::vector<TimedLaunch> events;
    };
    std::map<std::tuple<uint32_t, uint32_t, uint32_t>, HourGraph> graphs;
    std::string err;
    bool profiling = false;
    uint32_t launches[kKindCount] = {};
    double total_ms[kKindCount] = {};
    std::vector<TimedLaunch> pending;          // launches whose events are not read yet
    std::vector<cudaEvent_t> event_pool;
    std::vector<TimedLaunch>* capture = nullptr;  // set while a profiling graph is captured
    uint64_t kernels_launched = 0;
    int64_t last_claim_hour = -1;  // latest hour whose claims may sit in the claim plane (-1: clean)
    bool stop_rule = false;        // inside the run loop: hours after a replicate's stop do nothing
    uint32_t loop_hour = 0;        // next hour of a paused run loop (0: none in progress)
    uint32_t s_loop_hour = 0;      // ... at the last save_state
    const uint8_t* init_flags = nullptr;  // during creation: Csv population flags of replicate 0
    // citizen-state stream (single world): per-hour codes written by k_state_delta
    FILE* stream_file = nullptr;
    uint32_t* d_prev = nullptr;     // cell of every agent at the previous record
    uint8_t* d_codes = nullptr;     // kStreamChunk x slots
    uint2* d_exc = nullptr;         // kStreamChunk x slots (worst case: everyone jumps)
    uint32_t* d_exc_n = nullptr;    // kStreamChunk
    uint8_t* h_codes = nullptr;     // pinned mirrors
    uint2* h_exc = nullptr;
    uint32_t* h_exc_n = nullptr;
    // device-side checkpoint
    uint32_t *s_pos = nullptr, *s_wsa = nullptr;
    uint2* s_st = nullptr;
    uint8_t* s_plane = nullptr;
    uint32_t s_plane_par = 0;
    uint8_t* s_danger = nullptr;
    bool saved = false;

    uint32_t R() const { return (uint32_t)reps.size(); }
};

struct epi_ensemble {
    epi_engine core;
};

static thread_local std::string g_create_error;

#define CK(call)                                                                             \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess) {                                                             \
            h->err = std::string(#call) + ": " + cudaGetErrorString(e_);                     \
            return EPI_ERR_CUDA;                                                             \
        }                                                                                    \
    } while (0)

static Rect to_rect(const epi_area& a) { return Rect{a.x0, a.y0, a.x1, a.y1}; }

#ifndef EPI_DEPENDENT_LAUNCH
#define EPI_DEPENDENT_LAUNCH 1
#endif

// Launch of an hour kernel with programmatic stream serialisation: its blocks may be
// scheduled before the previous kernel of the stream has finished and wait on the device
// (dep_wait) for it, which hides the launch gap between the hour's kernels.  Captured into
// the hour graphs as programmatic edges.
template <typename... KArgs, typename... Args>
static cudaError_t launch_hour_kernel(void (*kern)(KArgs...), uint32_t blocks, cudaStream_t s, Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(blocks);
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = EPI_DEPENDENT_LAUNCH;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...);
}

// Device parameters of one world: areas, random key, disease thresholds.
static DevParams make_dev_params(const epi_params& p, const epi_geography& geo0, uint32_t n) {
    DevParams d;
    std::memset(&d, 0, sizeof d);
    d.n = n;
    d.G = (int32_t)p.grid_size;
    d.W = d.G + 1;
    d.WP = d.G + 3;
    d.hosp_code = kHosp0;
    d.area[kTransport] = to_rect(geo0.transport);
    d.area[kHousing] = to_rect(geo0.housing);
    d.area[kHosp0] = to_rect(geo0.hospital);
    d.area[kHosp1] = to_rect(grown_hospital(geo0));
    d.key0 = (uint32_t)p.seed;
    d.key1 = (uint32_t)(p.seed >> 32);
    uint32_t mk[4];
    philox4x32(0u, kWorldHour, kBlkMoveKey, 0u, d.key0, d.key1, mk);
    d.move_key = mk[0];
    d.reg_start = p.regular_transmission_start_day;
    d.high_start = p.high_transmission_start_day;
    d.last_day = p.last_day;
    d.exposed_duration = p.exposed_duration;
    d.pre_duration = p.pre_symptomatic_duration;
    const double rates[3] = {0.0, p.regular_transmission_rate, p.high_transmission_rate};
    for (int c = 0; c < 3; ++c) {
        d.thr_rate[c] = bernoulli_threshold(rates[c]);
        if (rates[c] >= p.high_transmission_rate) d.hosp_if_class |= 1u << c;  // is_to_be_hospitalized
    }
    d.thr_death = bernoulli_threshold(p.death_rate);
    d.thr_symptoms = bernoulli_threshold(1.0 - p.percentage_asymptomatic_population);
    d.thr_severe = bernoulli_threshold(p.percentage_severe_infected_population);
    d.active = 1;
    return d;
}

// ------------------------------------------------------------------ launch bookkeeping
// Eagerly launched kernels take their event pair from the pool and return it once read;
// kernels captured into a profiling graph get a pair of their own, recorded as external
// event nodes, which the graph keeps and re-records at every replay.
static int record_launch_begin(epi_engine* h, int kind, cudaEvent_t* out_end) {
    if (!h->profiling) return EPI_OK;
    cudaEvent_t a, b;
    if (h->capture) {
        CK(cudaEventCreate(&a));
        CK(cudaEventCreate(&b));
        CK(cudaEventRecordWithFlags(a, h->stream, cudaEventRecordExternal));
        h->capture->push_back({kind, a, b, false});
    } else {
        if (h->event_pool.size() >= 2) {
            a = h->event_pool.back(); h->event_pool.pop_back();
            b = h->event_pool.back(); h->event_pool.pop_back();
        } else {
            CK(cudaEventCreate(&a));
            CK(cudaEventCreate(&b));
        }
        CK(cudaEventRecord(a, h->stream));
        h->pending.push_back({kind, a, b, true});
    }
    *out_end = b;
    return EPI_OK;
}

static int record_launch_end(epi_engine* h, cudaEvent_t end) {
    if (!h->profiling) return EPI_OK;
    if (h->capture) CK(cudaEventRecordWithFlags(end, h->stream, cudaEventRecordExternal));
    else CK(cudaEventRecord(end, h->stream));
    return EPI_OK;
}

// Read the pending launches' durations (the stream has been synchronised).
static int harvest_events(epi_engine* h) {
    for (auto& pe : h->pending) {
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, pe.begin, pe.end));
        h->launches[pe.kind]++;
        h->total_ms[pe.kind] += ms;
        if (pe.pooled) {
            h->event_pool.push_back(pe.begin);
            h->event_pool.push_back(pe.end);
        }
    }
    h->pending.clear();
    return EPI_OK;
}

static void destroy_graphs(epi_engine* h) {
    for (auto& g : h->graphs) {
        cudaGraphExecDestroy(g.second.exec);
        for (auto& t : g.second.events) { cudaEventDestroy(t.begin); cudaEventDestroy(t.end); }
    }
    h->graphs.clear();
}

#define LAUNCH(kind, ...)                                                                    \
    do {                                                                                     \
        cudaEvent_t end_ = nullptr;                                                          \
        int rc_ = record_launch_begin(h, kind, &end_);                                       \
        if (rc_) return rc_;                                                                 \
        __VA_ARGS__;                                                                         \
        CK(cudaGetLastError());                                                              \
        rc_ = record_launch_end(h, end_);                                                    \
        if (rc_) return rc_;                                                                 \
    } while (0)

static int push_params(epi_engine* h) {
    std::vector<DevParams> all(h->R());
    for (uint32_t r = 0; r < h->R(); ++r) {
        Replica& rep = h->reps[r];
        const GuardParams g = guard_params(rep.p, rep.iv, rep.geo.hospital);
        rep.hp.guard_flags = g.flags;
        rep.hp.lock_threshold = g.lock_threshold;
        rep.hp.spread_threshold = g.spread_threshold;
        rep.hp.occ_threshold = g.occ_threshold;
        all[r] = rep.hp;
    }
    CK(cudaMemcpyAsync(h->d_params, all.data(), all.size() * sizeof(DevParams), cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return EPI_OK;
}

static int ensure_counts(epi_engine* h, uint32_t hours_needed) {
    if (hours_needed <= h->counts_capacity) return EPI_OK;
    uint32_t cap = std::max<uint32_t>(hours_needed, 48);
    if (h->d_counts) CK(cudaFree(h->d_counts));
    if (h->h_counts) CK(cudaFreeHost(h->h_counts));
    h->d_counts = nullptr;
    h->h_counts = nullptr;
    const size_t words = (size_t)cap * h->R() * 8;
    CK(cudaMalloc(&h->d_counts, words * sizeof(uint32_t)));
    CK(cudaMallocHost(&h->h_counts, words * sizeof(uint32_t)));
    h->counts_capacity = cap;
    destroy_graphs(h);  // they reference the old buffer
    return EPI_OK;
}

// ------------------------------------------------------------------ the hour loop
using DecideKernel = void (*)(const DevParams*, const uint32_t*, uint32_t, const uint32_t*, uint2*, const uint32_t*,
                              const uint32_t*, uint32_t*, const uint8_t*, const uint8_t*, uint32_t*, uint32_t*, uint32_t*,
                              HourArgs, int*);

// Hours 2..6 of a day change nothing once hour 1 has sent everyone but hospital staff home
// (routine, citizen/mod.rs:244-248, sets current_area = home_location and nothing else), so
// when the previous hour ran in the same chain the hour's kernel is skipped and its counts
// row repeats the previous one.  (A piece that starts at hours 2..6 always starts a chain.)
static bool sleep_hour_skipped(uint32_t first_hour, uint32_t k) {
    const uint32_t hod = (first_hour + k) % 24u;
    return k > 0 && hod >= 2u && hod <= 6u;
}

// The k_decide instance of an hour of the day.
// The k_decide (single world) or k_decide_ens (ensemble) instance of an hour of the day.
static DecideKernel decide_kernel(uint32_t hod, bool ensemble = false, bool full = false) {
#define EPI_PICK(HC)                                                                                                 \
    (ensemble ? (DecideKernel)k_decide_ens<HC> : full ? (DecideKernel)k_decide<HC, true> : (DecideKernel)k_decide<HC>)
    switch (hour_class(hod)) {
        case kHcStart: return EPI_PICK(kHcStart);
        case kHcEnd: return EPI_PICK(kHcEnd);
        case kHcTransport: return EPI_PICK(kHcTransport);
        case kHcWork: return EPI_PICK(kHcWork);
        case kHcNoon: return EPI_PICK(kHcNoon);
        case kHcHome: return EPI_PICK(kHcHome);
        default: return EPI_PICK(kHcMove);
    }
#undef EPI_PICK
}

// The hours of day 7..22 of a lone world rebuild its plane in the other buffer (k_commit
// REBUILD), 16 a day, so the buffer that holds the state after hour x is the parity of the
// number of such hours among 1..x: a function of x mod 24.  The other hours update the
// current buffer in place.
static bool rebuild_hour(uint32_t hod) { return hod >= 7u && hod <= 22u; }
static uint32_t plane_parity(uint32_t hod) { return (hod >= 7u ? std::min(hod, 22u) - 6u : 0u) & 1u; }
static uint8_t* plane_buf(const epi_engine* h, uint32_t par) {
    return h->d_plane + (h->two_planes ? (size_t)par * h->plane_bytes : 0u);
}

static int commit_blocks_for(uint32_t slots, int per_thread = kCommitSlots) {
    const uint32_t per_block = kThreads * (uint32_t)per_thread;
    return (int)std::max<uint32_t>(1u, (slots + per_block - 1) / per_block);
}

// k_commit with S slots per thread and round; the sparse instance for the hours of day 0 and
// 23, where hardly any agent acts.
using CommitKernel = void (*)(const DevParams*, const uint32_t*, uint32_t, uint32_t*, const uint32_t*, uint8_t*,
                              uint8_t*, uint32_t*, const uint32_t*, HourArgs, uint64_t, uint4*, uint32_t);
static CommitKernel commit_kernel(int slots_per_thread, bool sparse = false, bool rebuild = false) {
#define EPI_PICK(S)                                                                                                  \
    (sparse ? (CommitKernel)k_commit<S, true> : rebuild ? (CommitKernel)k_commit<S, false, true> : (CommitKernel)k_commit<S, false>)
    switch (slots_per_thread) {
        case 1: return EPI_PICK(1);
        case 2: return EPI_PICK(2);
        case 3: return EPI_PICK(3);
        case 4: return EPI_PICK(4);
        case 5: return EPI_PICK(5);
        case 6: return EPI_PICK(6);
        case 7: return EPI_PICK(7);
        default: return EPI_PICK(8);
    }
#undef EPI_PICK
}

// k_commit grid for S slots per thread: every slot once.  (Capping it at one wave of
// resident blocks that loop over the rest was measured slower: the block scheduler's later
// waves keep more loads in flight than a second round of the same threads.)
static int commit_grid(epi_engine* h, int S, int* out) {
    *out = commit_blocks_for(h->slots, S);
    return EPI_OK;
}

// Kernels of one piece: hours first_hour .. first_hour + nh - 1 of a chain; the hour base is
// read on the device, so a captured piece serves every start hour with the same hour of the
// day.  A piece that does not end its chain ends after an hour of day 0.  In the run loop a
// guard follows every hour of day 0.
static int enqueue_piece(epi_engine* h, uint32_t first_hour, uint32_t nh) {
    const uint32_t row_words = h->R() * 8u;
    const uint32_t n_chunks = h->slots / kChunk;
    int last_row = -1;  // the latest hour of the piece whose counts the kernels computed
    for (uint32_t k = 0; k < nh; ++k) {
        const uint32_t hod = (first_hour + k) % 24u;
        // rows back to the previous computed hour: within the piece, or the hour before it
        // (a day boundary, computed) unless the piece starts the chain (checked on the device)
        const uint32_t prev_back = !h->stop_rule ? 0u : (last_row >= 0 ? k - (uint32_t)last_row : 1u);
        const HourArgs ha{h->d_seg, h->d_counts, row_words, k, prev_back};
        if (h->stream_file && k > 0) {  // record the previous hour's end state before this hour changes it
            const uint32_t n = h->reps[0].n;
            k_state_delta<<<(n + kThreads - 1) / kThreads, kThreads, 0, h->stream>>>(
                n, h->d_pos, h->d_st, h->d_prev, h->d_codes + (size_t)(k - 1) * h->slots,
                h->d_exc + (size_t)(k - 1) * h->slots, h->d_exc_n + (k - 1));
            CK(cudaGetLastError());
        }
        if (sleep_hour_skipped(first_hour, k)) continue;
        last_row = (int)k;
        if (hod >= 1u && hod <= 6u) {
            LAUNCH(kKSleep, CK(launch_hour_kernel(k_sleep, h->grid_blocks, h->stream, (const DevParams*)h->d_params,
                                                  (const uint32_t*)h->d_chunk_rep, n_chunks, h->d_st, ha)));
        } else {
            // the plane of the previous hour, and (a lone world's rebuilding hours) the other
            // buffer, all zero, which k_commit fills before it zeroes the one the hour read
            const bool rebuild = h->two_planes && rebuild_hour(hod);
            uint8_t* read_plane = plane_buf(h, plane_parity((hod + 23u) % 24u));
            uint8_t* next_plane = plane_buf(h, plane_parity(hod));
            const DecideKernel decide = decide_kernel(hod, h->R() > 1, rebuild);
            LAUNCH(kKDecide, CK(launch_hour_kernel(
                                  decide, h->grid_blocks, h->stream, (const DevParams*)h->d_params,
                                  (const uint32_t*)h->d_chunk_rep, n_chunks, (const uint32_t*)h->d_pos, h->d_st,
                                  (const uint32_t*)h->d_home, (const uint32_t*)h->d_work, h->d_wsa,
                                  (const uint8_t*)read_plane, (const uint8_t*)h->d_danger, h->d_claim, h->d_tgt, h->d_lost,
                                  ha, h->d_err)));
            const CommitKernel commit = commit_kernel(h->commit_slots, hod == 0u || hod == 23u, rebuild);
            LAUNCH(kKCommit, CK(launch_hour_kernel(commit, h->commit_blocks, h->stream, (const DevParams*)h->d_params,
                                                   (const uint32_t*)h->d_chunk_rep, h->slots, h->d_pos,
                                                   (const uint32_t*)h->d_tgt, next_plane, h->d_danger, h->d_claim,
                                                   (const uint32_t*)h->d_lost, ha, (uint64_t)h->claim_cells,
                                                   rebuild ? reinterpret_cast<uint4*>(read_plane) : (uint4*)nullptr,
                                                   (uint32_t)(rebuild ? h->plane_bytes / 16u : 0u))));
        }
        // the run loop's guard after every day boundary but the piece's last hour (the piece
        // end below takes that one)
        if (h->stop_rule && hod == 0u && k + 1 < nh) {
            k_piece_end<<<1, kThreads, 0, h->stream>>>(h->d_params, h->R(), h->d_seg, h->d_counts, row_words, k, 0u, h->d_ivn);
            CK(cudaGetLastError());
        }
    }
    if (h->stream_file) {
        const uint32_t n = h->reps[0].n;
        k_state_delta<<<(n + kThreads - 1) / kThreads, kThreads, 0, h->stream>>>(
            n, h->d_pos, h->d_st, h->d_prev, h->d_codes + (size_t)(nh - 1) * h->slots, h->d_exc + (size_t)(nh - 1) * h->slots,
            h->d_exc_n + (nh - 1));
        CK(cudaGetLastError());
    }
    const bool guard_last = h->stop_rule && (first_hour + nh - 1) % 24u == 0u;
    k_piece_end<<<1, kThreads, 0, h->stream>>>(h->d_params, h->R(), h->d_seg, h->d_counts, row_words,
                                               guard_last ? nh - 1 : kNoGuard, nh, h->d_ivn);
    CK(cudaGetLastError());
    return EPI_OK;
}

// Kernel launches of a piece, for the launch counter.
static uint64_t piece_launches(const epi_engine* h, uint32_t first_hour, uint32_t nh) {
    uint64_t n = 1;  // k_piece_end
    for (uint32_t k = 0; k < nh; ++k) {
        const uint32_t hod = (first_hour + k) % 24u;
        if (h->stream_file) n += 1;  // k_state_delta
        if (h->stop_rule && hod == 0u && k + 1 < nh) n += 1;
        if (sleep_hour_skipped(first_hour, k)) continue;
        n += (hod >= 1u && hod <= 6u) ? 1u : 2u;
    }
    return n;
}

// The graph of a piece (captured on first use).
static int piece_graph(epi_engine* h, uint32_t first_hour, uint32_t nh, cudaGraphExec_t* out,
                       std::vector<TimedLaunch>** events) {
    auto key = std::make_tuple(first_hour % 24u, nh,
                               (h->profiling ? 1u : 0u) | (h->stream_file ? 2u : 0u) | (h->stop_rule ? 4u : 0u));
    auto it = h->graphs.find(key);
    if (it == h->graphs.end()) {
        epi_engine::HourGraph hg;
        cudaGraph_t g;
        CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
        h->capture = &hg.events;
        int rc = enqueue_piece(h, first_hour, nh);
        h->capture = nullptr;
        cudaError_t ce = cudaStreamEndCapture(h->stream, &g);
        if (rc == EPI_OK && ce == cudaSuccess) {
            ce = cudaGraphInstantiate(&hg.exec, g, 0);
            cudaGraphDestroy(g);
        }
        if (rc != EPI_OK || ce != cudaSuccess) {
            for (auto& t : hg.events) { cudaEventDestroy(t.begin); cudaEventDestroy(t.end); }
            if (rc) return rc;
            h->err = std::string("hour graph: ") + cudaGetErrorString(ce);
            return EPI_ERR_CUDA;
        }
        it = h->graphs.emplace(key, std::move(hg)).first;
    }
    *out = it->second.exec;
    *events = &it->second.events;
    return EPI_OK;
}

static int check_error_flag(epi_engine* h);

// Longest piece (one captured graph): two days.  Back-to-back pieces cost nothing measurable
// on the device, while every new engine captures its pieces once: two-day pieces made a
// fresh engine's 1M-agent 4,800-hour run 1.5 % faster than eight-day ones, at equal speed once warm.
constexpr uint32_t kPieceHours = 24u * 2u;

// Simulate hours first_hour .. first_hour + nh - 1 for every active replicate as one chain:
// pieces of whole days, launched back to back with one host synchronisation at the end
// (after each piece when profiling, whose events are read per launch).  The
// counts of hour k of replicate r land in h_counts[(k * R + r) * 8 ..]; in the run loop,
// h->halt_row is the chain offset of a row the guard marked, or -1.
static int run_hours_chunk(epi_engine* h, uint32_t first_hour, uint32_t nh) {
    h->halt_row = -1;
    if (nh == 0) return EPI_OK;
    if ((uint64_t)first_hour + nh > 0xFFFFFFFFull) { h->err = "hour out of range"; return EPI_ERR_ARG; }
    int rc = ensure_counts(h, nh);
    if (rc) return rc;
    // claims left by an earlier hour of another window, or by a later hour, must go first
    if (h->last_claim_hour >= 0 &&
        ((int64_t)first_hour <= h->last_claim_hour || first_hour / kClaimWindow != (uint64_t)h->last_claim_hour / kClaimWindow))
        CK(cudaMemsetAsync(h->d_claim, 0xFF, h->claim_cells * sizeof(uint32_t), h->stream));
    if (h->last_claim_hour >= (int64_t)first_hour)  // loss marks of hours about to run again
        CK(cudaMemsetAsync(h->d_lost, 0xFF, (size_t)h->slots * sizeof(uint32_t), h->stream));
    h->last_claim_hour = (int64_t)first_hour + nh - 1;
    if (h->two_planes) {  // the chain reads the state after first_hour - 1 from its parity's buffer
        const uint32_t need = plane_parity((first_hour + 23u) % 24u);
        if (need != h->plane_par) {  // and the other buffer zero, as a rebuilding hour wants it
            CK(cudaMemcpyAsync(plane_buf(h, need), plane_buf(h, h->plane_par), h->plane_bytes, cudaMemcpyDeviceToDevice,
                               h->stream));
            CK(cudaMemsetAsync(plane_buf(h, h->plane_par), 0, h->plane_bytes, h->stream));
            h->plane_par = need;
        }
    }
    const bool ran = h->reps[0].active;  // a lone world whose run has ended runs no hour kernel
    const size_t row_words = (size_t)h->R() * 8;
    CK(cudaMemsetAsync(h->d_counts, 0, (size_t)nh * row_words * sizeof(uint32_t), h->stream));
    if (h->stream_file) CK(cudaMemsetAsync(h->d_exc_n, 0, (size_t)nh * sizeof(uint32_t), h->stream));
    h->h_seg->hour_base = first_hour;
    h->h_seg->first = first_hour;
    CK(cudaMemcpyAsync(h->d_seg, h->h_seg, sizeof(SegDev), cudaMemcpyHostToDevice, h->stream));
    // pieces: at most kPieceHours, ending after an hour of day 0 unless they end the chain, so
    // that a chain of whole days replays one graph; the stream's chunks stay whole (their
    // code buffers are indexed by the hour)
    for (uint32_t k0 = 0; k0 < nh;) {
        uint32_t len = nh - k0;
        if (!h->stream_file && len > kPieceHours) {
            const uint32_t head = (24u - (first_hour + k0) % 24u) % 24u + 1u;  // through the next hour of day 0
            len = head + (kPieceHours - std::min(head, kPieceHours)) / 24u * 24u;
        }
        cudaGraphExec_t exec;
        std::vector<TimedLaunch>* events;
        rc = piece_graph(h, first_hour + k0, len, &exec, &events);
        if (rc) return rc;
        CK(cudaGraphLaunch(exec, h->stream));
        h->kernels_launched += piece_launches(h, first_hour + k0, len);
        if (h->profiling) {  // the piece's event nodes hold this launch's times until its next launch
            h->pending.insert(h->pending.end(), events->begin(), events->end());
            CK(cudaStreamSynchronize(h->stream));
            rc = harvest_events(h);
            if (rc) return rc;
        }
        k0 += len;
    }
    CK(cudaMemcpyAsync(h->h_counts, h->d_counts, (size_t)nh * row_words * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                       h->stream));
    CK(cudaStreamSynchronize(h->stream));
    for (uint32_t k = 1; k < nh; ++k)
        if (sleep_hour_skipped(first_hour, k))
            std::memcpy(h->h_counts + (size_t)k * row_words, h->h_counts + (size_t)(k - 1) * row_words,
                        row_words * sizeof(uint32_t));
    rc = check_error_flag(h);
    if (rc) return rc;
    std::vector<uint8_t> ended(h->R(), 0);  // stop rule met at an earlier hour of this chain
    int end_row = -1;                       // the first such row (later hours ran no kernel)
    for (uint32_t k = 0; k < nh && h->halt_row < 0; ++k) {
        for (uint32_t r = 0; r < h->R(); ++r) {
            if (!h->reps[r].active || ended[r]) continue;
            const uint32_t* c = h->h_counts + ((size_t)k * h->R() + r) * 8;
            if (h->stop_rule && c[1] == 0 && c[2] == 0 && c[3] == 0) {
                ended[r] = 1;
                if (end_row < 0) end_row = (int)k;
            }
            const uint64_t total = (uint64_t)c[0] + c[1] + c[2] + c[3] + c[4] + c[5];
            if (total != h->reps[r].n) {  // assert_eq!(csv_record.total(), current_population), allocation_map.rs:128
                h->err = "replicate " + std::to_string(r) + ": counts total " + std::to_string(total) + " != population " +
                         std::to_string(h->reps[r].n);
                return EPI_ERR_INVARIANT;
            }
        }
        if (h->stop_rule && h->h_counts[(size_t)k * row_words + 6] != 0u) h->halt_row = (int)k;  // later rows did not run
    }
    if (h->two_planes && ran) {  // the buffer of the last hour whose kernels ran
        uint32_t last = nh - 1;
        if (h->halt_row >= 0) last = std::min(last, (uint32_t)h->halt_row);
        if (end_row >= 0) last = std::min(last, (uint32_t)end_row);
        h->plane_par = plane_parity((first_hour + last) % 24u);
    }
    return EPI_OK;
}

static int check_error_flag(epi_engine* h) {
    int e = 0;
    CK(cudaMemcpyAsync(&e, h->d_err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    if (e) {
        h->err = "device invariant violated (flag " + std::to_string(e) + "): a rule addressed a cell outside the plane";
        return EPI_ERR_INVARIANT;
    }
    return EPI_OK;
}

// ------------------------------------------------------------------ citizen-state stream
constexpr uint32_t kStreamChunk = 24;  // hours per stream buffer fill

// Append hours first_hour .. first_hour + m - 1 of the stream buffers to the file: per hour
// {hour, agents, exceptions} (u32 each), the agents' code bytes, then the exceptions
// {agent, x | y << 16} in agent order.
static int stream_write(epi_engine* h, uint32_t first_hour, uint32_t m) {
    const uint32_t n = h->reps[0].n;
    CK(cudaMemcpyAsync(h->h_exc_n, h->d_exc_n, m * sizeof(uint32_t), cudaMemcpyDeviceToHost, h->stream));
    for (uint32_t k = 0; k < m; ++k)
        CK(cudaMemcpyAsync(h->h_codes + (size_t)k * h->slots, h->d_codes + (size_t)k * h->slots, n,
                           cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    for (uint32_t k = 0; k < m; ++k) {
        const uint32_t ne = std::min(h->h_exc_n[k], n);
        if (ne) CK(cudaMemcpy(h->h_exc, h->d_exc + (size_t)k * h->slots, ne * sizeof(uint2), cudaMemcpyDeviceToHost));
        std::sort(h->h_exc, h->h_exc + ne, [](const uint2& a, const uint2& b) { return a.x < b.x; });
        const uint32_t head[3] = {first_hour + k, n, ne};
        if (std::fwrite(head, sizeof head, 1, h->stream_file) != 1 ||
            std::fwrite(h->h_codes + (size_t)k * h->slots, 1, n, h->stream_file) != n ||
            (ne && std::fwrite(h->h_exc, sizeof(uint2), ne, h->stream_file) != ne)) {
            h->err = "citizen-state stream: write failed";
            return EPI_ERR_IO;
        }
    }
    return EPI_OK;
}

// Hours first_hour .. first_hour + nh - 1 (see run_hours_chunk); with the stream open they run
// in chunks of at most kStreamChunk hours, each written out before the next.
static int run_hours(epi_engine* h, uint32_t first_hour, uint32_t nh) {
    if (h->stop_rule) {  // the guard's new-infections figures as the host has them (the chunks carry them on)
        CK(cudaStreamSynchronize(h->stream));  // the pinned staging may still feed an earlier copy
        for (uint32_t r = 0; r < h->R(); ++r) h->h_ivn[r] = h->reps[r].iv.new_infections_in_a_day;
        CK(cudaMemcpyAsync(h->d_ivn, h->h_ivn, h->R() * sizeof(uint32_t), cudaMemcpyHostToDevice, h->stream));
    }
    if (!h->stream_file) return run_hours_chunk(h, first_hour, nh);
    int rc = ensure_counts(h, std::max(nh, kStreamChunk));
    if (rc) return rc;
    const size_t row = (size_t)h->R() * 8;
    std::vector<uint32_t> all((size_t)nh * row, 0u);
    int halt = -1;
    for (uint32_t k0 = 0; k0 < nh; k0 += kStreamChunk) {
        const uint32_t m = std::min(kStreamChunk, nh - k0);
        rc = run_hours_chunk(h, first_hour + k0, m);
        if (rc) return rc;
        // in the run loop the record ends with the hour the stop rule fires (the reference
        // publishes no later hour), or with a row the guard marked (the hours after it did
        // not run; the run loop runs them again)
        // (each chunk is a chain of its own, so the host, not the device, ends the run here)
        uint32_t keep = m;
        bool over = false;
        if (h->stop_rule)
            for (uint32_t k = 0; k < m; ++k) {
                const uint32_t* c = h->h_counts + (size_t)k * row;
                if ((c[1] | c[2] | c[3]) == 0u) { keep = k + 1; over = true; break; }
            }
        if (h->halt_row >= 0 && (uint32_t)h->halt_row < keep) {
            keep = (uint32_t)h->halt_row + 1;
            halt = (int)(k0 + (uint32_t)h->halt_row);
            over = true;
        }
        rc = stream_write(h, first_hour + k0, keep);
        if (rc) return rc;
        std::memcpy(all.data() + (size_t)k0 * row, h->h_counts, (size_t)keep * row * sizeof(uint32_t));
        if (over) break;
    }
    std::memcpy(h->h_counts, all.data(), all.size() * sizeof(uint32_t));
    h->halt_row = halt;
    return EPI_OK;
}

static void stream_free(epi_engine* h) {
    if (h->stream_file) std::fclose(h->stream_file);
    h->stream_file = nullptr;
    cudaFree(h->d_prev); cudaFree(h->d_codes); cudaFree(h->d_exc); cudaFree(h->d_exc_n);
    if (h->h_codes) cudaFreeHost(h->h_codes);
    if (h->h_exc) cudaFreeHost(h->h_exc);
    if (h->h_exc_n) cudaFreeHost(h->h_exc_n);
    h->d_prev = nullptr; h->d_codes = nullptr; h->d_exc = nullptr; h->d_exc_n = nullptr;
    h->h_codes = nullptr; h->h_exc = nullptr; h->h_exc_n = nullptr;
}

static epi_counts counts_of(const epi_engine* h, uint32_t k, uint32_t r, uint32_t hour) {
    const uint32_t* c = h->h_counts + ((size_t)k * h->R() + r) * 8;
    epi_counts o;
    o.hour = hour;
    o.susceptible = c[0];
    o.exposed = c[1];
    o.infected = c[2];
    o.hospitalized = c[3];
    o.recovered = c[4];
    o.deceased = c[5];
    return o;
}

// ------------------------------------------------------------------ interventions
static int bulk_done(epi_engine* h) {
    CK(cudaStreamSynchronize(h->stream));
    h->kernels_launched += 1;
    return harvest_events(h);
}

static int blocks_for(uint32_t n) { return (int)std::max<uint32_t>(1u, std::min<uint32_t>((n + kThreads - 1) / kThreads, 4096u)); }

static int lock_city(epi_engine* h, uint32_t r, int on) {
    const Replica& rep = h->reps[r];
    LAUNCH(kKLock, (k_lock<<<blocks_for(rep.n), kThreads, 0, h->stream>>>(h->d_st, rep.hp.agent_off, rep.n, on)));
    return bulk_done(h);
}

static int vaccinate(epi_engine* h, uint32_t r, uint32_t hour, double percent) {
    const Replica& rep = h->reps[r];
    const uint64_t thr = bernoulli_threshold(percent);
    LAUNCH(kKVaccinate, (k_vaccinate<<<blocks_for(rep.n), kThreads, 0, h->stream>>>(h->d_st, rep.hp.agent_off, rep.n,
                                                                                    rep.hp.key0, rep.hp.key1, hour, thr)));
    return bulk_done(h);
}

static void grow_hospital(epi_engine* h, uint32_t r) {
    Replica& rep = h->reps[r];
    const epi_area grown = grown_hospital(rep.geo0);
    rep.geo.hospital = grown;
    rep.hp.hosp_code = rect_eq(to_rect(grown), rep.hp.area[kHosp0]) ? kHosp0 : kHosp1;
}

// process_interventions of one replicate; returns EPI_IV_* bits in *applied.  Parameter
// changes (the hospital, and the device guard's armed triggers after any action) are left
// for the caller to push.
static int process_interventions(epi_engine* h, uint32_t r, const epi_counts& c, uint32_t* applied, bool* params_dirty) {
    Replica& rep = h->reps[r];
    InterventionActions a = decide_interventions(rep.p, rep.iv, c, rep.geo.hospital);
    int rc = EPI_OK;
    if (a.vaccinate && (rc = vaccinate(h, r, c.hour, a.vaccinate_percent))) return rc;
    if (a.lock && (rc = lock_city(h, r, 1))) return rc;
    if (a.unlock && (rc = lock_city(h, r, 0))) return rc;
    if (a.grow_hospital) grow_hospital(h, r);
    if (a.applied) *params_dirty = true;
    if (applied) *applied = a.applied;
    return EPI_OK;
}

// run_single_engine for every replicate in lockstep: segments end at any replicate's
// intervention point or final hour; after each segment every active replicate takes its
// rows, its interventions and its stop rule (epidemiology_simulation.rs:223-269, 564-575).
static int set_all_active(epi_engine* h) {
    for (auto& rep : h->reps) {
        rep.active = true;
        rep.hp.active = 1;
    }
    return push_params(h);
}

static int run_loop_body(epi_engine* h, uint32_t until);

// The run loop through hour `until` (all of it for 0xFFFFFFFF), starting at hour 1 or where a
// paused run stopped.  Replicates drop out of the lockstep loop as their runs end; once the
// run is over all of them are active again, so that direct hour calls keep working on every
// world (a paused run keeps its flags for the continuation).
static int run_loop(epi_engine* h, uint32_t until = 0xFFFFFFFFu) {
    h->stop_rule = true;
    int rc = run_loop_body(h, until);
    h->stop_rule = false;
    if (rc) h->loop_hour = 0;  // a failed run cannot be continued
    if (h->loop_hour != 0 && !rc) return EPI_OK;
    int rc2 = set_all_active(h);
    return rc ? rc : rc2;
}

// Longest chain of the run loop: a chain that the guard halts early has launched its later
// pieces for nothing (their kernels see the mark and return at once), so the cap bounds that
// waste while the host synchronises once per chain instead of once per day.
constexpr uint32_t kChainHours = 24u * 8u;

static int run_loop_body(epi_engine* h, uint32_t until) {
    uint32_t last = 0;  // last simulated hour over all replicates
    if (h->loop_hour == 0) {  // a fresh run
        for (auto& rep : h->reps) {
            rep.rows.clear();
            rep.active = rep.p.hours >= 2;
            rep.hp.active = rep.active ? 1u : 0u;
        }
        h->loop_hour = 1;
    }
    for (const auto& rep : h->reps)
        if (rep.p.hours >= 2) last = std::max(last, rep.p.hours - 1);
    uint32_t hour = h->loop_hour;
    bool dirty = true;
    while (hour <= last && hour <= until) {
        bool any = false;
        for (auto& rep : h->reps) any |= rep.active;
        if (!any) break;
        if (dirty) {
            int rc = push_params(h);
            if (rc) return rc;
            dirty = false;
        }
        // the chain ends at the first hour where the host must act whatever the counts are: a
        // replicate's final hour or fixed intervention; data-dependent triggers halt it on
        // the device at the day boundary where they fire
        uint64_t end = std::min<uint64_t>(std::min(last, until), (uint64_t)hour + kChainHours - 1);
        for (const auto& rep : h->reps) {
            if (!rep.active) continue;
            end = std::min<uint64_t>(end, rep.p.hours - 1);
            end = std::min<uint64_t>(end, next_fixed_event(rep.p, rep.iv, hour));
        }
        const uint32_t nh = (uint32_t)end - hour + 1;
        int rc = run_hours(h, hour, nh);
        if (rc) return rc;
        uint32_t next = (uint32_t)end + 1;
        for (uint32_t k = 0; k < nh; ++k) {
            const uint32_t hr = hour + k;
            bool acted = false;
            for (uint32_t r = 0; r < h->R(); ++r) {
                Replica& rep = h->reps[r];
                if (!rep.active) continue;
                const epi_counts c = counts_of(h, k, r, hr);
                rep.rows.push_back(c);
                if (is_event_hour(rep.p, hr)) {
                    uint32_t applied = 0;
                    rc = process_interventions(h, r, c, &applied, &dirty);
                    if (rc) return rc;
                    acted |= applied != 0u;
                }
                const bool stop = c.exposed == 0 && c.infected == 0 && c.hospitalized == 0;
                if (stop || hr + 1 >= rep.p.hours) {
                    rep.active = false;
                    rep.hp.active = 0;
                    dirty = true;
                }
            }
            const bool halted = h->halt_row == (int)k;
            if (acted && !halted && k + 1 < nh) {
                // an intervention the device guard did not see: the later hours ran without it
                h->err = "run loop: an intervention fired at hour " + std::to_string(hr) +
                         " inside a chain without the device guard's mark";
                return EPI_ERR_INVARIANT;
            }
            if (acted || halted) {
                next = hr + 1;
                break;
            }
        }
        hour = next;
    }
    bool any = false;
    for (const auto& rep : h->reps) any |= rep.active;
    h->loop_hour = (any && hour <= last) ? hour : 0u;
    if (dirty) return push_params(h);
    return EPI_OK;
}

// ------------------------------------------------------------------ create / destroy
static void free_device(epi_engine* h) {
    destroy_graphs(h);
    stream_free(h);
    cudaFree(h->d_params); cudaFree(h->d_chunk_rep); cudaFree(h->d_pos); cudaFree(h->d_home); cudaFree(h->d_work);
    cudaFree(h->d_wsa); cudaFree(h->d_tgt); cudaFree(h->d_lost); cudaFree(h->d_st); cudaFree(h->d_plane); cudaFree(h->d_danger); cudaFree(h->d_claim);
    cudaFree(h->d_counts); cudaFree(h->d_seg); cudaFree(h->d_ivn); cudaFree(h->d_err); cudaFree(h->d_scratch);
    cudaFree(h->s_pos); cudaFree(h->s_wsa); cudaFree(h->s_st); cudaFree(h->s_plane); cudaFree(h->s_danger);
    if (h->h_counts) cudaFreeHost(h->h_counts);
    if (h->h_seg) cudaFreeHost(h->h_seg);
    if (h->h_ivn) cudaFreeHost(h->h_ivn);
    for (auto& pe : h->pending)
        if (pe.pooled) { cudaEventDestroy(pe.begin); cudaEventDestroy(pe.end); }
    for (auto e : h->event_pool) cudaEventDestroy(e);
    if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
}

static size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

static int finish_upload(epi_engine* h);

// World build on the device (world.cuh) for every replicate, from the host plan.
static int build_on_device(epi_engine* h) {
    const uint32_t R = h->R(), n_chunks = h->slots / kChunk;
    std::vector<WorldDev> W(R);
    std::vector<uint4> infections;
    std::vector<WorldPlan> plans(R);
    std::vector<int> status(R, EPI_OK);
    std::vector<std::string> errs(R);
    const unsigned workers = std::max(1u, std::min<unsigned>(R, std::thread::hardware_concurrency()));
    std::vector<std::thread> pool;
    for (unsigned w = 0; w < workers; ++w)
        pool.emplace_back([&, w] {
            for (uint32_t r = w; r < R; r += workers) {
                const bool csv = h->reps[r].p.population_source == 1;
                if (csv && (R != 1 || !h->init_flags)) {
                    status[r] = EPI_ERR_ARG;
                    errs[r] = "a Csv population comes with its rows (epi_engine_create_population, single engines)";
                    continue;
                }
                status[r] = world_plan(h->reps[r].p, plans[r], errs[r], csv ? h->init_flags : nullptr);
            }
        });
    for (auto& t : pool) t.join();
    for (uint32_t r = 0; r < R; ++r) {
        if (status[r]) {
            h->err = (R > 1 ? "replicate " + std::to_string(r) + ": " : std::string()) + errs[r];
            return status[r];
        }
        const WorldPlan& pl = plans[r];
        const Replica& rep = h->reps[r];
        WorldDev& d = W[r];
        d.n = pl.n;
        d.agent_off = rep.hp.agent_off;
        d.first_chunk = rep.hp.agent_off / kChunk;
        d.houses = pl.houses;
        d.houses_x = pl.geo.houses_x;
        d.offices = pl.offices;
        d.offices_x = pl.geo.offices_x;
        d.hx0 = pl.geo.housing.x0; d.hy0 = pl.geo.housing.y0;
        d.ox0 = pl.geo.work.x0; d.oy0 = pl.geo.work.y0;
        d.key0 = pl.key0; d.key1 = pl.key1;
        d.transport_points = (uint32_t)std::min<uint64_t>(pl.transport_points, 0xFFFFFFFFull);
        d.csv = pl.flags ? 1u : 0u;
        d.thr_work = pl.thr_work; d.thr_pt = pl.thr_pt; d.thr_staff = pl.thr_staff; d.thr_ess = pl.thr_ess;
        for (const auto& f : pl.infections) infections.push_back(make_uint4(rep.hp.agent_off + f.agent, f.state, f.day, 0u));
    }
    WorldDev* d_w = nullptr;
    uint4* d_inf = nullptr;
    uint8_t* d_flags = nullptr;
    CK(cudaMalloc(&d_w, R * sizeof(WorldDev)));
    if (h->init_flags) {  // single Csv world: slot = agent
        CK(cudaMalloc(&d_flags, h->slots));
        CK(cudaMemsetAsync(d_flags, 0, h->slots, h->stream));
        CK(cudaMemcpyAsync(d_flags, h->init_flags, h->reps[0].n, cudaMemcpyHostToDevice, h->stream));
    }
    if (!infections.empty()) CK(cudaMalloc(&d_inf, infections.size() * sizeof(uint4)));
    int rc = EPI_OK;
    cudaError_t e = cudaMemcpyAsync(d_w, W.data(), R * sizeof(WorldDev), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess && d_inf)
        e = cudaMemcpyAsync(d_inf, infections.data(), infections.size() * sizeof(uint4), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) {
        // scratch: d_lost holds the eligibility flags, d_tgt the per-chunk counts (both reset after)
        const int blocks = (int)std::min<uint64_t>(n_chunks, (uint64_t)h->resident_blocks * 2);
        k_world_citizens<<<blocks, kThreads, 0, h->stream>>>(d_w, h->d_chunk_rep, n_chunks, h->d_pos, h->d_st, h->d_home,
                                                             h->d_work, h->d_wsa, h->d_lost, h->d_tgt, d_flags);
        k_world_scan<<<1, 1024, 0, h->stream>>>(h->d_tgt, n_chunks);
        k_world_pt<<<blocks, kThreads, 0, h->stream>>>(d_w, h->d_chunk_rep, n_chunks, h->d_lost, h->d_tgt, h->d_st);
        if (d_inf)
            k_world_infect<<<(int)std::min<size_t>((infections.size() + kThreads - 1) / kThreads, 1024), kThreads, 0,
                             h->stream>>>(d_inf, (uint32_t)infections.size(), h->d_st);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
        h->kernels_launched += d_inf ? 4 : 3;
    }
    if (e != cudaSuccess) {
        h->err = std::string("device world build: ") + cudaGetErrorString(e);
        rc = EPI_ERR_CUDA;
    }
    cudaFree(d_w);
    cudaFree(d_inf);
    cudaFree(d_flags);
    return rc;
}

// Lay out and upload R worlds given as per-replicate record arrays (nullptr: build them on
// the device).
static int engine_init(epi_engine* h, const epi_params* params, const epi_agent_record* const* recs, uint32_t R) {
    if (R == 0) { h->err = "no replicates"; return EPI_ERR_ARG; }
    h->reps.resize(R);
    uint64_t slots = 0, plane = 0, claim = 0;
    for (uint32_t r = 0; r < R; ++r) {
        Replica& rep = h->reps[r];
        rep.p = params[r];
        const std::string bad = validate_params(rep.p);
        if (!bad.empty()) { h->err = "replicate " + std::to_string(r) + ": " + bad; return EPI_ERR_CONFIG; }
        rep.n = rep.p.number_of_agents;
        rep.geo0 = define_geography(rep.p.grid_size);
        resize_hospital(rep.geo0, (int32_t)rep.n, 0.002, rep.p.hospital_beds_percentage);
        rep.geo = rep.geo0;
        rep.hp = make_dev_params(rep.p, rep.geo0, rep.n);
        rep.hp.agent_off = (uint32_t)slots;
        rep.hp.plane_off = plane;
        rep.hp.claim_off = claim;
        const uint64_t side = (uint64_t)rep.p.grid_size + 1;
        slots += align_up(rep.n, kChunk);
        plane += align_up((side + 2) * (side + 2) + 16, 256);
        claim += side * side;
        if (slots >= 0xFFFFFFFFull - kChunk) { h->err = "too many agents for one engine"; return EPI_ERR_CAPACITY; }
    }
    h->slots = (uint32_t)slots;
    h->plane_bytes = plane;
    h->claim_cells = claim;
    int dev = 0, sms = 0, per_sm = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void*)decide_kernel(9u, R > 1), kThreads, 0));
    per_sm = std::max(per_sm, 1);
    const uint64_t n_chunks = slots / kChunk;
    h->resident_blocks = sms * per_sm;
    h->grid_blocks = (int)std::min<uint64_t>(n_chunks, (uint64_t)h->resident_blocks);
    {
        const int rc = commit_grid(h, h->commit_slots, &h->commit_blocks);
        if (rc) return rc;
    }
    CK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    h->own_stream = true;
    CK(cudaMalloc(&h->d_params, R * sizeof(DevParams)));
    if (R > 1) {
        std::vector<uint32_t> chunk_rep(n_chunks);
        for (uint32_t r = 0; r < R; ++r) {
            const uint64_t c0 = h->reps[r].hp.agent_off / kChunk, c1 = c0 + align_up(h->reps[r].n, kChunk) / kChunk;
            for (uint64_t c = c0; c < c1; ++c) chunk_rep[c] = r;
        }
        CK(cudaMalloc(&h->d_chunk_rep, n_chunks * sizeof(uint32_t)));
        CK(cudaMemcpyAsync(h->d_chunk_rep, chunk_rep.data(), n_chunks * sizeof(uint32_t), cudaMemcpyHostToDevice, h->stream));
        CK(cudaStreamSynchronize(h->stream));
    }
    CK(cudaMalloc(&h->d_pos, slots * sizeof(uint32_t)));
    CK(cudaMalloc(&h->d_home, slots * sizeof(uint32_t)));
    CK(cudaMalloc(&h->d_work, slots * sizeof(uint32_t)));
    CK(cudaMalloc(&h->d_wsa, slots * sizeof(uint32_t)));
    CK(cudaMalloc(&h->d_tgt, slots * sizeof(uint32_t)));
    CK(cudaMalloc(&h->d_lost, slots * sizeof(uint32_t)));
    CK(cudaMalloc(&h->d_st, slots * sizeof(uint2)));
    h->two_planes = R == 1;
    CK(cudaMalloc(&h->d_plane, h->plane_bytes * (h->two_planes ? 2u : 1u)));
    CK(cudaMalloc(&h->d_danger, h->plane_bytes));
    CK(cudaMalloc(&h->d_claim, h->claim_cells * sizeof(uint32_t)));
    CK(cudaMalloc(&h->d_seg, sizeof(SegDev)));
    CK(cudaMalloc(&h->d_ivn, R * sizeof(uint32_t)));
    CK(cudaMemset(h->d_ivn, 0, R * sizeof(uint32_t)));
    CK(cudaMalloc(&h->d_err, sizeof(int)));
    CK(cudaMalloc(&h->d_scratch, 4 * sizeof(unsigned long long)));
    CK(cudaMallocHost(&h->h_seg, sizeof(SegDev)));
    CK(cudaMallocHost(&h->h_ivn, R * sizeof(uint32_t)));
    int rc = ensure_counts(h, 48);
    if (rc) return rc;
    if (!recs) {
        rc = build_on_device(h);
        if (rc) return rc;
        return finish_upload(h);
    }
    // The records go to the device as they are (replicate r's at slot agent_off(r)) and
    // k_pack_records checks and packs them there; the first bad one is reported.
    rc = push_params(h);
    if (rc) return rc;
    struct DeviceBuffer {
        void* p = nullptr;
        ~DeviceBuffer() { if (p) cudaFree(p); }
    } stage;
    CK(cudaMalloc(&stage.p, slots * sizeof(epi_agent_record)));
    epi_agent_record* d_recs = static_cast<epi_agent_record*>(stage.p);
    for (uint32_t r = 0; r < R; ++r)
        CK(cudaMemcpyAsync(d_recs + h->reps[r].hp.agent_off, recs[r], (size_t)h->reps[r].n * sizeof(epi_agent_record),
                           cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemsetAsync(h->d_scratch, 0xFF, sizeof(unsigned long long), h->stream));
    k_pack_records<<<blocks_for(h->slots), kThreads, 0, h->stream>>>(h->d_params, h->d_chunk_rep, h->slots, d_recs,
                                                                     h->d_pos, h->d_st, h->d_home, h->d_work, h->d_wsa,
                                                                     h->d_scratch);
    CK(cudaGetLastError());
    unsigned long long bad = ~0ull;
    CK(cudaMemcpyAsync(&bad, h->d_scratch, sizeof bad, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    if (bad != ~0ull) {  // the replicate holding the slot, and the record's index within it
        const uint64_t slot = bad >> 1;
        uint32_t r = 0;
        while (r + 1 < R && h->reps[r + 1].hp.agent_off <= slot) ++r;
        h->err = "replicate " + std::to_string(r) + ": agent record " + std::to_string(slot - h->reps[r].hp.agent_off) +
                 ((bad & 1u) ? ": current area is not one of its areas" : " out of range");
        return EPI_ERR_ARG;
    }
    return finish_upload(h);
}

// Everything after the agent arrays are on the device: scratch words, planes, parameters.
static int finish_upload(epi_engine* h) {
    const size_t slots = h->slots;
    CK(cudaMemsetAsync(h->d_tgt, 0xFF, slots * sizeof(uint32_t), h->stream));
    CK(cudaMemsetAsync(h->d_lost, 0xFF, slots * sizeof(uint32_t), h->stream));
    CK(cudaMemsetAsync(h->d_plane, 0, h->plane_bytes * (h->two_planes ? 2u : 1u), h->stream));
    CK(cudaMemsetAsync(h->d_danger, 0, h->plane_bytes, h->stream));
    h->plane_par = 0;
    CK(cudaMemsetAsync(h->d_claim, 0xFF, h->claim_cells * sizeof(uint32_t), h->stream));
    CK(cudaMemsetAsync(h->d_err, 0, sizeof(int), h->stream));
    int rc = push_params(h);
    if (rc) return rc;
    LAUNCH(kKBuildPlane, (k_build_plane<<<blocks_for(h->slots), kThreads, 0, h->stream>>>(
                              h->d_params, h->d_chunk_rep, h->slots, h->d_pos, h->d_st, h->d_plane, h->d_danger,
                              h->d_err)));
    CK(cudaStreamSynchronize(h->stream));
    rc = harvest_events(h);
    if (rc) return rc;
    return check_error_flag(h);
}

static int snapshot_replica(epi_engine* h, uint32_t r, epi_agent_record* out, size_t n) {
    const Replica& rep = h->reps[r];
    if (!out || n != rep.n) return EPI_ERR_ARG;
    const size_t off = rep.hp.agent_off;
    std::vector<uint32_t> pos(n), home(n), work(n), wsa(n);
    std::vector<uint2> st(n);
    CK(cudaMemcpyAsync(pos.data(), h->d_pos + off, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(home.data(), h->d_home + off, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(work.data(), h->d_work + off, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(wsa.data(), h->d_wsa + off, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(st.data(), h->d_st + off, n * sizeof(uint2), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    for (size_t i = 0; i < n; ++i) {
        epi_agent_record& a = out[i];
        std::memset(&a, 0, sizeof a);
        const uint32_t s = st[i].x, v = s & kStateMask;
        a.x = unpack_x(pos[i]);
        a.y = unpack_y(pos[i]);
        a.state = (uint8_t)v;
        a.flags = (uint8_t)(((s & kHosp) ? EPI_F_HOSPITALIZED : 0) | ((s & kIso) ? EPI_F_ISOLATED : 0) |
                            ((s & kVacc) ? EPI_F_VACCINATED : 0) | ((s & kWq) ? EPI_F_WORK_QUARANTINED : 0) |
                            ((s & kPt) ? EPI_F_PUBLIC_TRANSPORT : 0));
        a.work_status = (uint8_t)st_ws(s);
        a.immunity = (int8_t)st_imm(s);
        a.at_hour = (v == EPI_E || v == EPI_I_PRE) ? st[i].y : 0u;
        a.infection_day = infected(s) ? st_day(s) : 0u;
        a.work_start_at = st_ws(s) == EPI_WS_HOSPITAL_STAFF ? wsa[i] : 0u;
        a.home_x = unpack_x(home[i]);
        a.home_y = unpack_y(home[i]);
        a.work_x = unpack_x(work[i]);
        a.work_y = unpack_y(work[i]);
        const uint32_t code = st_area(s);
        Rect ar = code == kHome ? Rect{a.home_x, a.home_y, a.home_x + 1, a.home_y + 1}
                  : code == kWork ? Rect{a.work_x, a.work_y, a.work_x + 9, a.work_y + 9}
                                  : rep.hp.area[code < kNumAreas ? code : kHome];
        a.area_x0 = ar.x0; a.area_y0 = ar.y0; a.area_x1 = ar.x1; a.area_y1 = ar.y1;
    }
    return EPI_OK;
}

static int check_all(epi_engine* h) {
    CK(cudaMemsetAsync(h->d_scratch, 0, 4 * sizeof(unsigned long long), h->stream));
    LAUNCH(kKCheck, (k_check_agents<<<blocks_for(h->slots), kThreads, 0, h->stream>>>(
                         h->d_params, h->d_chunk_rep, h->slots, h->d_pos, h->d_st, plane_buf(h, h->plane_par),
                         h->d_scratch)));
    LAUNCH(kKCheck, (k_check_plane<<<h->grid_blocks, kThreads, 0, h->stream>>>(h->plane_bytes, plane_buf(h, h->plane_par),
                                                                                h->d_scratch + 1)));
    LAUNCH(kKCheck, (k_check_danger<<<dim3(64, std::min<uint32_t>(h->R(), 4096u)), kThreads, 0, h->stream>>>(
                         h->d_params, h->R(), plane_buf(h, h->plane_par), h->d_danger, h->d_scratch + 2)));
    unsigned long long v[4] = {0, 0, 0, 0};
    CK(cudaMemcpyAsync(v, h->d_scratch, sizeof v, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    int rc = harvest_events(h);
    if (rc) return rc;
    uint64_t population = 0;
    for (const auto& rep : h->reps) population += rep.n;
    if (v[0] || v[1] != population || v[2]) {
        h->err = "invariants: " + std::to_string(v[0]) + " agents off their cell class, " + std::to_string(v[1]) +
                 " occupied cells for " + std::to_string(population) + " agents, " + std::to_string(v[2]) +
                 " cells with a wrong infectious-neighbour count";
        return EPI_ERR_INVARIANT;
    }
    return EPI_OK;
}

static int save_state(epi_engine* h);
static int restore_state(epi_engine* h);

static int set_launch_shape(epi_engine* h, uint32_t decide_blocks, uint32_t commit_slots) {
    const uint32_t n_chunks = h->slots / kChunk;
    if (decide_blocks == 0 || decide_blocks > n_chunks || commit_slots == 0 || commit_slots > (uint32_t)kMaxCommitSlots) {
        h->err = "launch shape: k_decide blocks in [1, " + std::to_string(n_chunks) + "], k_commit slots in [1, " +
                 std::to_string(kMaxCommitSlots) + "]";
        return EPI_ERR_ARG;
    }
    CK(cudaStreamSynchronize(h->stream));
    h->grid_blocks = (int)decide_blocks;
    h->commit_slots = (int)commit_slots;
    {
        const int rc = commit_grid(h, h->commit_slots, &h->commit_blocks);
        if (rc) return rc;
    }
    destroy_graphs(h);  // they bake the launch shapes in
    return EPI_OK;
}

// Launch-shape autotuner: times hours 1..hours of the engine's current world under each
// candidate (k_decide grid: the resident grid, twice it, one chunk per block; k_commit: 1, 2
// or 4 slots per thread), restarting every candidate from the same state, and keeps the
// fastest.  Results do not depend on the shape; the state, the run's rows and the launch
// counter are restored afterwards (the saved checkpoint is replaced).
static int autotune(epi_engine* h, uint32_t hours, epi_launch_shape* out) {
    if (hours == 0 || hours > 24u * 7u) { h->err = "autotune hours must be in [1, 168]"; return EPI_ERR_ARG; }
    const uint32_t n_chunks = h->slots / kChunk;
    std::vector<uint32_t> grids;
    // three quarters of the resident grid too: fewer warps per SM share the L1 that holds the
    // plane rows their agents read
    const uint64_t cand[4] = {(uint64_t)h->resident_blocks * 3u / 4u, (uint64_t)h->resident_blocks,
                              2ull * (uint64_t)h->resident_blocks, (uint64_t)n_chunks};
    for (uint64_t g : cand) {
        const uint32_t v = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(g, n_chunks));
        if (std::find(grids.begin(), grids.end(), v) == grids.end()) grids.push_back(v);
    }
    const uint32_t slot_cands[3] = {1u, 2u, 4u};
    const bool prof = h->profiling;
    const uint64_t launched = h->kernels_launched;
    h->profiling = false;
    int rc = save_state(h);
    if (rc) return rc;
    double best = 1e300;
    uint32_t best_g = (uint32_t)h->grid_blocks, best_c = (uint32_t)h->commit_slots;
    for (uint32_t g : grids) {
        for (uint32_t c : slot_cands) {
            rc = set_launch_shape(h, g, c);
            double t_min = 1e300;
            for (int rep = 0; rep < 5 && !rc; ++rep) {  // the first pass captures the graphs
                rc = restore_state(h);
                if (rc) break;
                const auto t0 = std::chrono::steady_clock::now();
                rc = run_hours(h, 1, hours);
                const double t = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
                if (rep > 0) t_min = std::min(t_min, t);
            }
            if (rc) break;
            if (t_min < best) { best = t_min; best_g = g; best_c = c; }
        }
        if (rc) break;
    }
    h->profiling = prof;
    int rc2 = set_launch_shape(h, best_g, best_c);
    if (!rc2) rc2 = restore_state(h);
    h->kernels_launched = launched;
    if (rc) return rc;
    if (rc2) return rc2;
    if (out) {
        out->decide_blocks = best_g;
        out->commit_slots = best_c;
        out->hour_us = best * 1e6 / hours;
    }
    return EPI_OK;
}

static int save_state(epi_engine* h) {
    const size_t n = h->slots;
    if (!h->s_pos) {
        CK(cudaMalloc(&h->s_pos, n * sizeof(uint32_t)));
        CK(cudaMalloc(&h->s_wsa, n * sizeof(uint32_t)));
        CK(cudaMalloc(&h->s_st, n * sizeof(uint2)));
        CK(cudaMalloc(&h->s_plane, h->plane_bytes));
        CK(cudaMalloc(&h->s_danger, h->plane_bytes));
    }
    CK(cudaMemcpyAsync(h->s_pos, h->d_pos, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, h->stream));
    CK(cudaMemcpyAsync(h->s_wsa, h->d_wsa, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, h->stream));
    CK(cudaMemcpyAsync(h->s_st, h->d_st, n * sizeof(uint2), cudaMemcpyDeviceToDevice, h->stream));
    CK(cudaMemcpyAsync(h->s_plane, plane_buf(h, h->plane_par), h->plane_bytes, cudaMemcpyDeviceToDevice, h->stream));
    h->s_plane_par = h->plane_par;
    CK(cudaMemcpyAsync(h->s_danger, h->d_danger, h->plane_bytes, cudaMemcpyDeviceToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    for (auto& rep : h->reps) {
        rep.s_iv = rep.iv;
        rep.s_geo = rep.geo;
        rep.s_hosp_code = rep.hp.hosp_code;
        rep.s_active = rep.active;
        rep.s_rows = rep.rows;
    }
    h->s_loop_hour = h->loop_hour;
    h->saved = true;
    return EPI_OK;
}

static int restore_state(epi_engine* h) {
    if (!h->saved) { h->err = "no saved state"; return EPI_ERR_ARG; }
    const size_t n = h->slots;
    CK(cudaMemcpyAsync(h->d_pos, h->s_pos, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, h->stream));
    CK(cudaMemcpyAsync(h->d_wsa, h->s_wsa, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, h->stream));
    CK(cudaMemcpyAsync(h->d_st, h->s_st, n * sizeof(uint2), cudaMemcpyDeviceToDevice, h->stream));
    CK(cudaMemcpyAsync(plane_buf(h, h->s_plane_par), h->s_plane, h->plane_bytes, cudaMemcpyDeviceToDevice, h->stream));
    if (h->two_planes) CK(cudaMemsetAsync(plane_buf(h, 1u - h->s_plane_par), 0, h->plane_bytes, h->stream));
    h->plane_par = h->s_plane_par;
    CK(cudaMemcpyAsync(h->d_danger, h->s_danger, h->plane_bytes, cudaMemcpyDeviceToDevice, h->stream));
    CK(cudaMemsetAsync(h->d_tgt, 0xFF, n * sizeof(uint32_t), h->stream));
    CK(cudaMemsetAsync(h->d_lost, 0xFF, n * sizeof(uint32_t), h->stream));
    CK(cudaMemsetAsync(h->d_claim, 0xFF, h->claim_cells * sizeof(uint32_t), h->stream));
    h->last_claim_hour = -1;
    for (auto& rep : h->reps) {
        rep.iv = rep.s_iv;
        rep.geo = rep.s_geo;
        rep.hp.hosp_code = rep.s_hosp_code;
        rep.active = rep.s_active;
        rep.hp.active = rep.s_active ? 1u : 0u;
        rep.rows = rep.s_rows;
    }
    h->loop_hour = h->s_loop_hour;
    return push_params(h);
}

static int create_engine(const epi_params* params, const epi_agent_record* const* recs, uint32_t R, epi_engine** out) {
    epi_engine* h = new epi_engine();
    int rc = engine_init(h, params, recs, R);
    if (rc) {
        g_create_error = h->err;
        free_device(h);
        delete h;
        return rc;
    }
    *out = h;
    return EPI_OK;
}

// ------------------------------------------------------------------ C ABI: config, geography, world
extern "C" {

int epi_params_from_json(const char* json_text, epi_params* out, char* err, size_t errlen) {
    if (!json_text || !out) return EPI_ERR_ARG;
    try {
        *out = params_from_json(json_text);
    } catch (const std::exception& e) {
        if (err && errlen) { std::snprintf(err, errlen, "%s", e.what()); }
        return EPI_ERR_CONFIG;
    }
    std::string bad = validate_params(*out);
    if (!bad.empty()) {
        if (err && errlen) std::snprintf(err, errlen, "%s", bad.c_str());
        return EPI_ERR_CONFIG;
    }
    return EPI_OK;
}

int epi_define_geography(uint32_t grid_size, epi_geography* out) {
    if (!out || grid_size < 1 || grid_size > 32766) return EPI_ERR_ARG;
    *out = define_geography(grid_size);
    return EPI_OK;
}

int epi_resize_hospital(epi_geography* geo, int32_t number_of_agents, double staff, double beds) {
    if (!geo) return EPI_ERR_ARG;
    resize_hospital(*geo, number_of_agents, staff, beds);
    return EPI_OK;
}

int epi_geography_increase_hospital_size(epi_geography* geo, uint32_t grid_size) {
    if (!geo || grid_size > 32766) return EPI_ERR_ARG;
    epi_geography g = *geo;
    g.grid_size = grid_size;
    geo->hospital = grown_hospital(g);
    return EPI_OK;
}

int epi_interventions_replay(const epi_params* p, const epi_counts* rows, uint32_t n, uint32_t* applied,
                             uint8_t* guard) {
    if (!p || (n && (!rows || !applied))) return EPI_ERR_ARG;
    const std::string bad = validate_params(*p);
    if (!bad.empty()) { g_create_error = bad; return EPI_ERR_CONFIG; }
    epi_geography geo = define_geography(p->grid_size);
    resize_hospital(geo, (int32_t)p->number_of_agents, 0.002, p->hospital_beds_percentage);
    const epi_geography geo0 = geo;
    InterventionState st;
    uint32_t ivn = 0;  // the device guard's new-infections figure
    for (uint32_t k = 0; k < n; ++k) {
        const epi_counts& c = rows[k];
        if (guard) {  // k_piece_end's verdict on this row, from the thresholds pushed before it
            uint8_t fire = 0;
            if (c.hour % 24u == 0u) {
                const GuardParams g = guard_params(*p, st, geo.hospital);
                const uint32_t fresh = c.infected > ivn ? c.infected - ivn : 0u;
                ivn = fresh;
                fire = ((g.flags & 1u) && c.infected > g.lock_threshold) || ((g.flags & 2u) && fresh >= g.spread_threshold) ||
                       ((g.flags & 4u) && c.hospitalized >= g.occ_threshold);
            }
            guard[k] = fire;
        }
        const InterventionActions a = decide_interventions(*p, st, c, geo.hospital);
        if (a.grow_hospital) geo.hospital = grown_hospital(geo0);
        applied[k] = a.applied;
    }
    return EPI_OK;
}

int epi_outputs_write(const char* dir, const char* engine_id, const epi_params* p, const epi_counts* rows, uint32_t n) {
    if (!dir || !engine_id || !p || (n && !rows)) return EPI_ERR_ARG;
    const std::string bad = validate_params(*p);
    if (!bad.empty()) { g_create_error = bad; return EPI_ERR_CONFIG; }
    epi_geography geo = define_geography(p->grid_size);
    resize_hospital(geo, (int32_t)p->number_of_agents, 0.002, p->hospital_beds_percentage);
    const epi_geography geo0 = geo;
    InterventionState st;
    for (uint32_t k = 0; k < n; ++k)
        if (decide_interventions(*p, st, rows[k], geo.hospital).grow_hospital) geo.hospital = grown_hospital(geo0);
    std::string err;
    const int rc = write_outputs(dir, engine_id, std::vector<epi_counts>(rows, rows + n), st.reports, err);
    if (rc) g_create_error = err;
    return rc;
}

double epi_disease_transmission_rate(const epi_params* p, uint32_t day) {
    switch (rate_class(p->regular_transmission_start_day, p->high_transmission_start_day, p->last_day, day)) {
        case 1: return p->regular_transmission_rate;
        case 2: return p->high_transmission_rate;
        default: return 0.0;
    }
}

int epi_disease_is_to_be_hospitalized(const epi_params* p, uint32_t day) {
    return epi_disease_transmission_rate(p, day) >= p->high_transmission_rate;
}

int epi_population_read_csv(const char* path, uint8_t* flags, uint32_t cap, uint32_t* n) {
    if (!path || !n) return EPI_ERR_ARG;
    std::vector<uint8_t> f;
    std::string err;
    int rc = read_population_csv(path, f, err);
    if (rc) { g_create_error = err; return rc; }
    *n = (uint32_t)f.size();
    if (flags) std::memcpy(flags, f.data(), std::min<size_t>(f.size(), cap));
    return EPI_OK;
}

int epi_world_build_population(const epi_params* p, const uint8_t* flags, uint32_t n, epi_agent_record* out,
                               epi_geography* geo) {
    if (!p || !flags || !out || n != p->number_of_agents) return EPI_ERR_ARG;
    std::vector<epi_agent_record> recs;
    epi_geography g;
    std::string err;
    int rc = build_world(*p, recs, g, err, flags);
    if (rc) { g_create_error = err; return rc; }
    std::memcpy(out, recs.data(), (size_t)n * sizeof(epi_agent_record));
    if (geo) *geo = g;
    return EPI_OK;
}

int epi_engine_create_population(const epi_params* params, const uint8_t* flags, uint32_t n, epi_engine** out) {
    if (!params || !flags || !out || n != params->number_of_agents) return EPI_ERR_ARG;
    *out = nullptr;
    epi_params p = *params;
    p.population_source = 1;
    epi_engine* h = new epi_engine();
    h->init_flags = flags;
    int rc = engine_init(h, &p, nullptr, 1);
    h->init_flags = nullptr;
    if (rc) {
        g_create_error = h->err;
        free_device(h);
        delete h;
        return rc;
    }
    *out = h;
    return EPI_OK;
}

int epi_world_build(const epi_params* p, epi_agent_record* out, size_t n, epi_geography* geo) {
    if (!p || !out || n != p->number_of_agents) return EPI_ERR_ARG;
    if (p->population_source == 1) { g_create_error = "Csv population: use epi_world_build_population"; return EPI_ERR_ARG; }
    std::vector<epi_agent_record> recs;
    epi_geography g;
    std::string err;
    int rc = build_world(*p, recs, g, err);
    if (rc) { g_create_error = err; return rc; }
    std::memcpy(out, recs.data(), n * sizeof(epi_agent_record));
    if (geo) *geo = g;
    return EPI_OK;
}

// ------------------------------------------------------------------ C ABI: single engine
int epi_engine_create_from_records(const epi_params* params, const epi_agent_record* recs, size_t n, epi_engine** out) {
    if (!params || !recs || !out) return EPI_ERR_ARG;
    *out = nullptr;
    if (n != params->number_of_agents || n == 0 || n >= 0xFFFFFFFFull) {
        g_create_error = "record count != number_of_agents";
        return EPI_ERR_ARG;
    }
    const epi_agent_record* one[1] = {recs};
    return create_engine(params, one, 1, out);
}

int epi_engine_create(const epi_params* params, epi_engine** out) {
    if (!params || !out) return EPI_ERR_ARG;
    *out = nullptr;
    return create_engine(params, nullptr, 1, out);
}

int epi_engine_create_json(const char* config_json, uint64_t seed, epi_engine** out) {
    if (!out) return EPI_ERR_ARG;
    *out = nullptr;
    epi_params p;
    char msg[512] = {0};
    int rc = epi_params_from_json(config_json, &p, msg, sizeof msg);
    if (rc) { g_create_error = msg; return rc; }
    p.seed = seed;
    if (p.population_source == 1) {  // Population::Csv: read the rows of its file
        std::vector<uint8_t> flags;
        std::string err;
        rc = read_population_csv(p.population_file, flags, err);
        if (rc) { g_create_error = err; return rc; }
        return epi_engine_create_population(&p, flags.data(), (uint32_t)flags.size(), out);
    }
    return epi_engine_create(&p, out);
}

void epi_engine_destroy(epi_engine* h) {
    if (!h) return;
    free_device(h);
    delete h;
}

const char* epi_engine_last_error(const epi_engine* h) { return h ? h->err.c_str() : g_create_error.c_str(); }

int epi_engine_set_stream(epi_engine* h, void* cuda_stream) {
    if (!h) return EPI_ERR_ARG;
    CK(cudaStreamSynchronize(h->stream));
    if (h->own_stream) CK(cudaStreamDestroy(h->stream));
    if (cuda_stream) {
        h->stream = (cudaStream_t)cuda_stream;
        h->own_stream = false;
    } else {
        CK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
        h->own_stream = true;
    }
    return EPI_OK;
}

int epi_engine_simulate_hours(epi_engine* h, uint32_t first_hour, uint32_t n, epi_counts* out) {
    if (!h || (!out && n)) return EPI_ERR_ARG;
    int rc = run_hours(h, first_hour, n);
    if (rc) return rc;
    for (uint32_t k = 0; k < n; ++k) out[k] = counts_of(h, k, 0, first_hour + k);
    return EPI_OK;
}

int epi_engine_simulate(epi_engine* h, uint32_t hour, epi_counts* out) {
    if (!h || !out) return EPI_ERR_ARG;
    return epi_engine_simulate_hours(h, hour, 1, out);
}

int epi_engine_lock_city(epi_engine* h) { return h ? lock_city(h, 0, 1) : EPI_ERR_ARG; }
int epi_engine_unlock_city(epi_engine* h) { return h ? lock_city(h, 0, 0) : EPI_ERR_ARG; }

int epi_engine_vaccinate(epi_engine* h, uint32_t hour, double percent) {
    if (!h || !(percent >= 0.0 && percent <= 1.0)) return EPI_ERR_ARG;
    return vaccinate(h, 0, hour, percent);
}

int epi_engine_increase_hospital_size(epi_engine* h) {
    if (!h) return EPI_ERR_ARG;
    grow_hospital(h, 0);
    return push_params(h);
}

int epi_engine_process_interventions(epi_engine* h, const epi_counts* counts, uint32_t* applied) {
    if (!h || !counts) return EPI_ERR_ARG;
    bool dirty = false;
    int rc = process_interventions(h, 0, *counts, applied, &dirty);
    if (rc) return rc;
    return dirty ? push_params(h) : EPI_OK;
}

int epi_engine_run(epi_engine* h, epi_counts* rows, uint32_t max_rows, uint32_t* n_rows) {
    if (!h || !n_rows) return EPI_ERR_ARG;
    *n_rows = 0;
    int rc = run_loop(h);
    if (rc) return rc;
    const std::vector<epi_counts>& got = h->reps[0].rows;
    const uint32_t nr = (uint32_t)got.size();
    if (rows) {
        if (max_rows < nr) { h->err = "rows buffer too small"; return EPI_ERR_ARG; }
        std::memcpy(rows, got.data(), nr * sizeof(epi_counts));
    }
    *n_rows = nr;
    return EPI_OK;
}

int epi_engine_run_until(epi_engine* h, uint32_t last_hour, epi_counts* rows, uint32_t max_rows, uint32_t* n_rows,
                         uint32_t* next_hour) {
    if (!h || !n_rows || !next_hour) return EPI_ERR_ARG;
    *n_rows = 0;
    *next_hour = 0;
    int rc = run_loop(h, last_hour);
    if (rc) return rc;
    const std::vector<epi_counts>& got = h->reps[0].rows;
    const uint32_t nr = (uint32_t)got.size();
    if (rows) {
        if (max_rows < nr) { h->err = "rows buffer too small"; return EPI_ERR_ARG; }
        std::memcpy(rows, got.data(), nr * sizeof(epi_counts));
    }
    *n_rows = nr;
    *next_hour = h->loop_hour;
    return EPI_OK;
}

}  // extern "C"

// ---- checkpoint file
namespace {
constexpr uint32_t kCheckpointMagic = 0x4B435045u;  // "EPCK"
constexpr uint32_t kCheckpointVersion = 1;

uint64_t fnv1a64(const std::vector<uint8_t>& b) {  // FNV-1a (Fowler, Noll, Vo), 64-bit
    uint64_t x = 0xCBF29CE484222325ull;
    for (uint8_t c : b) {
        x ^= c;
        x *= 0x100000001B3ull;
    }
    return x;
}
template <typename T>
void put(std::vector<uint8_t>& b, const T& v) {
    const uint8_t* p = reinterpret_cast<const uint8_t*>(&v);
    b.insert(b.end(), p, p + sizeof(T));
}
void put_bytes(std::vector<uint8_t>& b, const void* p, size_t n) {
    b.insert(b.end(), static_cast<const uint8_t*>(p), static_cast<const uint8_t*>(p) + n);
}
void put_string(std::vector<uint8_t>& b, const std::string& s) {
    put(b, (uint32_t)s.size());
    put_bytes(b, s.data(), s.size());
}
struct Reader {
    const std::vector<uint8_t>& b;
    size_t at = 0;
    bool ok = true;
    bool bytes(void* dst, size_t n) {
        if (!ok || n > b.size() - at) return ok = false;
        std::memcpy(dst, b.data() + at, n);
        at += n;
        return true;
    }
    template <typename T>
    bool get(T& v) { return bytes(&v, sizeof(T)); }
    bool string(std::string& s) {
        uint32_t n = 0;
        if (!get(n) || n > b.size() - at) return ok = false;
        s.assign(reinterpret_cast<const char*>(b.data() + at), n);
        at += n;
        return true;
    }
};
}  // namespace

extern "C" {

int epi_engine_checkpoint_write(epi_engine* h, const char* path) {
    if (!h || !path) return EPI_ERR_ARG;
    if (h->R() != 1) { h->err = "checkpoints are for single engines"; return EPI_ERR_ARG; }
    const Replica& rep = h->reps[0];
    std::vector<epi_agent_record> recs(rep.n);
    int rc = snapshot_replica(h, 0, recs.data(), recs.size());
    if (rc) return rc;
    std::vector<uint8_t> b;
    for (uint32_t v : {kCheckpointMagic, kCheckpointVersion, (uint32_t)sizeof(epi_params), (uint32_t)sizeof(epi_geography),
                       (uint32_t)sizeof(epi_agent_record), (uint32_t)sizeof(epi_counts), rep.n, h->loop_hour,
                       (uint32_t)rep.rows.size(), (uint32_t)rep.iv.reports.size(), rep.active ? 1u : 0u,
                       rep.iv.locked ? 1u : 0u, rep.iv.zero_infection_hour, rep.iv.new_infections_in_a_day,
                       rep.iv.hospital_applied ? 1u : 0u})
        put(b, v);
    put(b, rep.p);
    put(b, rep.geo);
    put_bytes(b, rep.rows.data(), rep.rows.size() * sizeof(epi_counts));
    for (const Report& r : rep.iv.reports) {
        put(b, r.hour);
        put_string(b, r.name);
        put_string(b, r.data);
    }
    put_bytes(b, recs.data(), recs.size() * sizeof(epi_agent_record));
    put(b, fnv1a64(b));
    FILE* f = std::fopen(path, "wb");
    if (!f) { h->err = std::string("checkpoint: cannot write ") + path; return EPI_ERR_IO; }
    const bool ok = std::fwrite(b.data(), 1, b.size(), f) == b.size();
    if (std::fclose(f) != 0 || !ok) { h->err = std::string("checkpoint: write failed: ") + path; return EPI_ERR_IO; }
    return EPI_OK;
}

int epi_engine_create_from_checkpoint(const char* path, epi_engine** out) {
    if (!path || !out) return EPI_ERR_ARG;
    *out = nullptr;
    auto fail = [](const std::string& m) {
        g_create_error = "checkpoint: " + m;
        return EPI_ERR_IO;
    };
    std::vector<uint8_t> b;
    {
        FILE* f = std::fopen(path, "rb");
        if (!f) return fail(std::string("cannot read ") + path);
        uint8_t buf[1 << 16];
        size_t k;
        while ((k = std::fread(buf, 1, sizeof buf, f)) > 0) b.insert(b.end(), buf, buf + k);
        std::fclose(f);
    }
    if (b.size() < 15 * 4 + 8) return fail("truncated file");
    uint64_t sum = 0;
    std::memcpy(&sum, b.data() + b.size() - 8, 8);
    b.resize(b.size() - 8);
    if (fnv1a64(b) != sum) return fail("checksum mismatch (truncated or corrupt file)");
    Reader rd{b};
    uint32_t hdr[15];
    for (uint32_t& v : hdr) rd.get(v);
    if (hdr[0] != kCheckpointMagic) return fail("not a checkpoint file");
    if (hdr[1] != kCheckpointVersion) return fail("unsupported version " + std::to_string(hdr[1]));
    if (hdr[2] != sizeof(epi_params) || hdr[3] != sizeof(epi_geography) || hdr[4] != sizeof(epi_agent_record) ||
        hdr[5] != sizeof(epi_counts))
        return fail("written by a build with other struct layouts");
    const uint32_t n = hdr[6], loop_hour = hdr[7], n_rows = hdr[8], n_reports = hdr[9];
    epi_params p;
    epi_geography geo;
    rd.get(p);
    rd.get(geo);
    if (!rd.ok || p.number_of_agents != n || n == 0) return fail("inconsistent header");
    if ((uint64_t)n_rows * sizeof(epi_counts) > b.size()) return fail("truncated file");
    std::vector<epi_counts> rows(n_rows);
    rd.bytes(rows.data(), rows.size() * sizeof(epi_counts));
    std::vector<Report> reports(std::min<uint32_t>(n_reports, 1u << 20));
    for (Report& r : reports) {
        rd.get(r.hour);
        rd.string(r.name);
        rd.string(r.data);
    }
    if ((uint64_t)n * sizeof(epi_agent_record) > b.size()) return fail("truncated file");
    std::vector<epi_agent_record> recs(n);
    rd.bytes(recs.data(), recs.size() * sizeof(epi_agent_record));
    if (!rd.ok || rd.at != b.size() || reports.size() != n_reports) return fail("truncated or malformed file");
    const std::string bad = validate_params(p);
    if (!bad.empty()) return fail(bad);
    epi_engine* h = nullptr;
    const epi_agent_record* one[1] = {recs.data()};
    int rc = create_engine(&p, one, 1, &h);
    if (rc) return rc;
    Replica& rep = h->reps[0];
    rep.geo = geo;
    rep.hp.hosp_code = rect_eq(to_rect(geo.hospital), rep.hp.area[kHosp0]) ? kHosp0 : kHosp1;
    rep.iv.locked = hdr[11] != 0;
    rep.iv.zero_infection_hour = hdr[12];
    rep.iv.new_infections_in_a_day = hdr[13];
    rep.iv.hospital_applied = hdr[14] != 0;
    rep.iv.reports = std::move(reports);
    rep.rows = std::move(rows);
    rep.active = hdr[10] != 0;
    rep.hp.active = rep.active ? 1u : 0u;
    h->loop_hour = loop_hour;
    rc = push_params(h);
    if (rc) {
        g_create_error = h->err;
        epi_engine_destroy(h);
        return rc;
    }
    *out = h;
    return EPI_OK;
}

int epi_engine_write_outputs(epi_engine* h, const char* dir, const char* engine_id) {
    if (!h || !dir || !engine_id) return EPI_ERR_ARG;
    return write_outputs(dir, engine_id, h->reps[0].rows, h->reps[0].iv.reports, h->err);
}

int epi_engine_population(const epi_engine* h, uint32_t* out) {
    if (!h || !out) return EPI_ERR_ARG;
    *out = h->reps[0].n;
    return EPI_OK;
}

int epi_engine_geography(const epi_engine* h, epi_geography* out) {
    if (!h || !out) return EPI_ERR_ARG;
    *out = h->reps[0].geo;
    return EPI_OK;
}

int epi_engine_snapshot(epi_engine* h, epi_agent_record* out, size_t n) {
    if (!h) return EPI_ERR_ARG;
    return snapshot_replica(h, 0, out, n);
}

int epi_engine_check(epi_engine* h) { return h ? check_all(h) : EPI_ERR_ARG; }
int epi_engine_save_state(epi_engine* h) { return h ? save_state(h) : EPI_ERR_ARG; }
int epi_engine_restore_state(epi_engine* h) { return h ? restore_state(h) : EPI_ERR_ARG; }

int epi_engine_autotune(epi_engine* h, uint32_t hours, epi_launch_shape* chosen) {
    if (!h) return EPI_ERR_ARG;
    if (h->stream_file) { h->err = "autotune: close the citizen-state stream first"; return EPI_ERR_ARG; }
    return autotune(h, hours, chosen);
}

// Citizen-state stream file: "EPCS", version 1, agents, grid (u32 each); the keyframe (per
// agent x, y as u16, then every agent's state letter byte); then hour records (stream_write).
int epi_engine_state_stream_open(epi_engine* h, const char* path) {
    if (!h || !path) return EPI_ERR_ARG;
    if (h->R() != 1) { h->err = "the citizen-state stream is for single engines"; return EPI_ERR_ARG; }
    if (h->stream_file) { h->err = "citizen-state stream already open"; return EPI_ERR_ARG; }
    const uint32_t n = h->reps[0].n;
    std::vector<epi_agent_record> recs(n);
    int rc = snapshot_replica(h, 0, recs.data(), n);
    if (rc) return rc;
    FILE* f = std::fopen(path, "wb");
    if (!f) { h->err = std::string("cannot open ") + path; return EPI_ERR_IO; }
    const uint32_t head[4] = {0x53435045u /* "EPCS" */, 1u, n, h->reps[0].p.grid_size};
    std::vector<uint16_t> xy((size_t)n * 2);
    std::vector<uint8_t> letters(n);
    for (uint32_t i = 0; i < n; ++i) {
        xy[2 * i] = (uint16_t)recs[i].x;
        xy[2 * i + 1] = (uint16_t)recs[i].y;
        const uint32_t v = recs[i].state;
        letters[i] = (uint8_t)(v == EPI_S ? 0 : v == EPI_E ? 1 : v == EPI_R ? 3 : v == EPI_D ? 4 : 2);
    }
    if (std::fwrite(head, sizeof head, 1, f) != 1 || std::fwrite(xy.data(), sizeof(uint16_t), xy.size(), f) != xy.size() ||
        std::fwrite(letters.data(), 1, n, f) != n) {
        std::fclose(f);
        h->err = "citizen-state stream: write failed";
        return EPI_ERR_IO;
    }
    h->stream_file = f;
    const size_t cap = (size_t)kStreamChunk * h->slots;
    CK(cudaMalloc(&h->d_prev, (size_t)h->slots * sizeof(uint32_t)));
    CK(cudaMalloc(&h->d_codes, cap));
    CK(cudaMalloc(&h->d_exc, cap * sizeof(uint2)));
    CK(cudaMalloc(&h->d_exc_n, kStreamChunk * sizeof(uint32_t)));
    CK(cudaMallocHost(&h->h_codes, cap));
    CK(cudaMallocHost(&h->h_exc, (size_t)h->slots * sizeof(uint2)));
    CK(cudaMallocHost(&h->h_exc_n, kStreamChunk * sizeof(uint32_t)));
    CK(cudaMemcpyAsync(h->d_prev, h->d_pos, (size_t)h->slots * sizeof(uint32_t), cudaMemcpyDeviceToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    destroy_graphs(h);  // hour graphs now carry the encoding kernel
    return EPI_OK;
}

int epi_engine_state_stream_close(epi_engine* h) {
    if (!h) return EPI_ERR_ARG;
    if (!h->stream_file) return EPI_OK;
    const int bad = std::fflush(h->stream_file);
    stream_free(h);
    destroy_graphs(h);
    if (bad) { h->err = "citizen-state stream: flush failed"; return EPI_ERR_IO; }
    return EPI_OK;
}

int epi_engine_set_launch_shape(epi_engine* h, const epi_launch_shape* shape) {
    if (!h || !shape) return EPI_ERR_ARG;
    return set_launch_shape(h, shape->decide_blocks, shape->commit_slots);
}

int epi_engine_launch_shape(const epi_engine* h, epi_launch_shape* out) {
    if (!h || !out) return EPI_ERR_ARG;
    out->decide_blocks = (uint32_t)h->grid_blocks;
    out->commit_slots = (uint32_t)h->commit_slots;
    out->hour_us = 0.0;
    return EPI_OK;
}

int epi_engine_kernels_launched(const epi_engine* h, uint64_t* out) {
    if (!h || !out) return EPI_ERR_ARG;
    *out = h->kernels_launched;
    return EPI_OK;
}

int epi_engine_set_profiling(epi_engine* h, int on) {
    if (!h) return EPI_ERR_ARG;
    h->profiling = on != 0;
    for (int k = 0; k < kKindCount; ++k) { h->launches[k] = 0; h->total_ms[k] = 0.0; }
    return EPI_OK;
}

int epi_engine_kernel_stats(const epi_engine* h, uint32_t* launches, double* total_ms, int n) {
    if (!h || !launches || !total_ms) return EPI_ERR_ARG;
    for (int k = 0; k < n && k < kKindCount; ++k) { launches[k] = h->launches[k]; total_ms[k] = h->total_ms[k]; }
    return EPI_OK;
}

const char* epi_engine_kernel_name(int k) { return (k >= 0 && k < kKindCount) ? kKernelNames[k] : ""; }
int epi_engine_kernel_kinds(void) { return kKindCount; }

size_t epi_abi_struct_size(const char* name) {
    if (!name) return 0;
    if (!std::strcmp(name, "epi_params")) return sizeof(epi_params);
    if (!std::strcmp(name, "epi_agent_record")) return sizeof(epi_agent_record);
    if (!std::strcmp(name, "epi_counts")) return sizeof(epi_counts);
    if (!std::strcmp(name, "epi_geography")) return sizeof(epi_geography);
    if (!std::strcmp(name, "epi_mlp_config")) return sizeof(epi_mlp_config);
    return 0;
}

// Algorithmic bytes of one hour over all replicates (the roofline numerator): the agent
// words the hour's kernels must read and write plus one pass over each plane.
//   movement hours and hours 0/23: decide reads pos 4 + st 8 + home 4 + work 4, writes st 8 +
//   tgt 4; commit reads tgt 4 + pos 4 + lost 4, writes pos 4; the occupancy plane and the
//   infectious-neighbour counts, (G+1)^2 bytes each, read once.
//   hour 1: st.x read 4 + write 4; hours 2-6 of a segment move no data.
int epi_engine_hour_bytes(const epi_engine* h, uint32_t hour, double* bytes) {
    if (!h || !bytes) return EPI_ERR_ARG;
    const uint32_t hod = hour % 24u;
    double b = 0.0;
    for (const auto& rep : h->reps) {
        const double n = (double)rep.n, side = (double)rep.p.grid_size + 1.0;
        if (hod >= 1u && hod <= 6u) b += hod == 1u ? n * 8.0 : 0.0;
        else b += n * 48.0 + 2.0 * side * side;
    }
    *bytes = b;
    return EPI_OK;
}

// ------------------------------------------------------------------ C ABI: ensemble
int epi_ensemble_create(const epi_params* params, uint32_t replicates, epi_ensemble** out) {
    if (!params || !out || replicates == 0) return EPI_ERR_ARG;
    *out = nullptr;
    epi_ensemble* e = new epi_ensemble();
    int rc = engine_init(&e->core, params, nullptr, replicates);
    if (rc) {
        g_create_error = e->core.err;
        free_device(&e->core);
        delete e;
        return rc;
    }
    *out = e;
    return EPI_OK;
}

void epi_ensemble_destroy(epi_ensemble* e) {
    if (!e) return;
    free_device(&e->core);
    delete e;
}

const char* epi_ensemble_last_error(const epi_ensemble* e) { return e ? e->core.err.c_str() : g_create_error.c_str(); }

int epi_ensemble_set_stream(epi_ensemble* e, void* cuda_stream) {
    return e ? epi_engine_set_stream(&e->core, cuda_stream) : EPI_ERR_ARG;
}

int epi_ensemble_run(epi_ensemble* e, epi_counts* rows, uint32_t max_rows_per_replicate, uint32_t* n_rows) {
    if (!e || !n_rows) return EPI_ERR_ARG;
    epi_engine* h = &e->core;
    int rc = run_loop(h);
    if (rc) return rc;
    for (uint32_t r = 0; r < h->R(); ++r) {
        const std::vector<epi_counts>& got = h->reps[r].rows;
        n_rows[r] = (uint32_t)got.size();
        if (rows) {
            if (got.size() > max_rows_per_replicate) { h->err = "rows buffer too small"; return EPI_ERR_ARG; }
            std::memcpy(rows + (size_t)r * max_rows_per_replicate, got.data(), got.size() * sizeof(epi_counts));
        }
    }
    return EPI_OK;
}

int epi_ensemble_replicates(const epi_ensemble* e, uint32_t* out) {
    if (!e || !out) return EPI_ERR_ARG;
    *out = e->core.R();
    return EPI_OK;
}

int epi_ensemble_snapshot(epi_ensemble* e, uint32_t replicate, epi_agent_record* out, size_t n) {
    if (!e || replicate >= e->core.R()) return EPI_ERR_ARG;
    return snapshot_replica(&e->core, replicate, out, n);
}

int epi_ensemble_check(epi_ensemble* e) { return e ? check_all(&e->core) : EPI_ERR_ARG; }
int epi_ensemble_save_state(epi_ensemble* e) { return e ? save_state(&e->core) : EPI_ERR_ARG; }
int epi_ensemble_restore_state(epi_ensemble* e) { return e ? restore_state(&e->core) : EPI_ERR_ARG; }
int epi_ensemble_set_profiling(epi_ensemble* e, int on) { return e ? epi_engine_set_profiling(&e->core, on) : EPI_ERR_ARG; }

int epi_ensemble_kernel_stats(const epi_ensemble* e, uint32_t* launches, double* total_ms, int n) {
    return e ? epi_engine_kernel_stats(&e->core, launches, total_ms, n) : EPI_ERR_ARG;
}

int epi_ensemble_autotune(epi_ensemble* e, uint32_t hours, epi_launch_shape* chosen) {
    return e ? autotune(&e->core, hours, chosen) : EPI_ERR_ARG;
}

int epi_ensemble_kernels_launched(const epi_ensemble* e, uint64_t* out) {
    return e ? epi_engine_kernels_launched(&e->core, out) : EPI_ERR_ARG;
}

int epi_ensemble_hour_bytes(const epi_ensemble* e, uint32_t hour, double* bytes) {
    return e ? epi_engine_hour_bytes(&e->core, hour, bytes) : EPI_ERR_ARG;
}

}  // extern "C"

// ------------------------------------------------------------------ no-allocation hour
// epi_tick_hour_noalloc: one simulated hour on device arrays the caller owns, for callers
// that cannot allocate device memory (see include/epi_engine.h).  Its scratch -- the
// parameter block, the hour word, the error word, the per-agent proposal buffer and the
// (G+1)^2 claim plane -- lives in the file-scope array below, which every GPU that loads
// this library holds until the process exits.  All calls share it: calls whose work overlaps
// on the GPU (two streams, two host threads) race on it and must be serialised by the caller.
namespace {

constexpr size_t kNoAllocScratchBytes = size_t(48) << 20;  // 48 MiB
constexpr size_t kNoAllocParamsOff = 0;                     // DevParams
constexpr size_t kNoAllocHourOff = 256;                     // SegDev {hour, hour}
constexpr size_t kNoAllocErrOff = 264;                      // int error flags
constexpr size_t kNoAllocTgtOff = 512;                      // u32 per agent
static_assert(sizeof(DevParams) <= kNoAllocHourOff, "parameter block must fit its slot");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

struct NoAllocDevice {
    unsigned char* base = nullptr;  // device address of g_noalloc_scratch on this device
    int grid_blocks = 0;            // resident grid of k_decide / k_sleep
};
constexpr int kNoAllocMaxDevices = 64;
NoAllocDevice g_noalloc_devices[kNoAllocMaxDevices];
std::mutex g_noalloc_mutex;

size_t align256(size_t v) { return (v + 255) & ~size_t(255); }

DevParams noalloc_params(const epi_params& p, uint32_t hospital_grown) {
    epi_geography g = define_geography(p.grid_size);
    resize_hospital(g, (int32_t)p.number_of_agents, 0.002, p.hospital_beds_percentage);
    DevParams d = make_dev_params(p, g, p.number_of_agents);
    d.hosp_code = (hospital_grown && !rect_eq(d.area[kHosp1], d.area[kHosp0])) ? kHosp1 : kHosp0;
    return d;
}

int noalloc_fail(int rc, const std::string& msg) {
    g_create_error = msg;
    return rc;
}

#define NOALLOC_CK(call)                                                                     \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess) return noalloc_fail(EPI_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// Once per device, with that device current: the device address of the scratch array (the
// host-side symbol is only a stand-in) and the launch shape.
int noalloc_setup(int dev, NoAllocDevice** out) {
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    NoAllocDevice& d = g_noalloc_devices[dev];
    if (!d.base) {
        void* ptr = nullptr;
        NOALLOC_CK(cudaGetSymbolAddress(&ptr, g_noalloc_scratch));
        int sms = 0, per_sm = 0;
        NOALLOC_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        NOALLOC_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void*)decide_kernel(9u), kThreads, 0));
        d.grid_blocks = sms * std::max(per_sm, 1);
        d.base = static_cast<unsigned char*>(ptr);
    }
    *out = &d;
    return EPI_OK;
}

}  // namespace

extern "C" int epi_tick_hour_noalloc(const epi_params* params, uint32_t hour, uint32_t hospital_grown, uint32_t* pos,
                                     uint32_t* state, const uint32_t* home, const uint32_t* work, uint32_t* work_start_at,
                                     uint8_t* plane, uint32_t* counts, void* cuda_stream) {
    if (!params || !pos || !state || !home || !work || !work_start_at || !plane || !counts)
        return noalloc_fail(EPI_ERR_ARG, "epi_tick_hour_noalloc: null pointer argument");
    if (reinterpret_cast<uintptr_t>(state) % 8 != 0)
        return noalloc_fail(EPI_ERR_ARG, "epi_tick_hour_noalloc: state must be 8-byte aligned (two words per agent)");
    // the neighbourhood reads take each plane row in aligned 32-bit words; the per-agent
    // arrays and the counts are read and written as 32-bit words
    if (reinterpret_cast<uintptr_t>(plane) % 4 != 0)
        return noalloc_fail(EPI_ERR_ARG, "epi_tick_hour_noalloc: plane must be 4-byte aligned");
    for (const void* w : {(const void*)pos, (const void*)home, (const void*)work, (const void*)work_start_at,
                          (const void*)counts})
        if (reinterpret_cast<uintptr_t>(w) % 4 != 0)
            return noalloc_fail(EPI_ERR_ARG,
                                "epi_tick_hour_noalloc: pos, home, work, work_start_at and counts must be 4-byte aligned");
    const std::string bad = validate_params(*params);
    if (!bad.empty()) return noalloc_fail(EPI_ERR_CONFIG, bad);
    const uint32_t n = params->number_of_agents;
    const size_t side = (size_t)params->grid_size + 1;
    const size_t claim_off = align256(kNoAllocTgtOff + (size_t)n * sizeof(uint32_t));
    const size_t claim_bytes = side * side * sizeof(uint32_t);
    if (claim_off + claim_bytes > kNoAllocScratchBytes)
        return noalloc_fail(EPI_ERR_CAPACITY,
                            "epi_tick_hour_noalloc: " + std::to_string(n) + " agents on a grid of " +
                                std::to_string(params->grid_size) + " need " + std::to_string(claim_off + claim_bytes) +
                                " bytes of scratch; the fixed maximum is " + std::to_string(kNoAllocScratchBytes));
    int dev = 0;
    NOALLOC_CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNoAllocMaxDevices) return noalloc_fail(EPI_ERR_ARG, "epi_tick_hour_noalloc: device index too large");
    NoAllocDevice* d = nullptr;
    int rc = noalloc_setup(dev, &d);
    if (rc) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
    const DevParams hp = noalloc_params(*params, hospital_grown);
    DevParams* d_params = reinterpret_cast<DevParams*>(d->base + kNoAllocParamsOff);
    SegDev* d_hour = reinterpret_cast<SegDev*>(d->base + kNoAllocHourOff);
    const SegDev seg{hour, hour};
    const HourArgs ha{d_hour, counts, 8u, 0u, 0u};
    int* d_err = reinterpret_cast<int*>(d->base + kNoAllocErrOff);
    uint32_t* d_tgt = reinterpret_cast<uint32_t*>(d->base + kNoAllocTgtOff);
    uint32_t* d_claim = reinterpret_cast<uint32_t*>(d->base + claim_off);
    // every call starts from clean scratch: the claim plane free, the error word zero
    NOALLOC_CK(cudaMemcpyAsync(d_params, &hp, sizeof hp, cudaMemcpyHostToDevice, s));
    NOALLOC_CK(cudaMemcpyAsync(d_hour, &seg, sizeof seg, cudaMemcpyHostToDevice, s));
    NOALLOC_CK(cudaMemsetAsync(d_err, 0, sizeof(int), s));
    NOALLOC_CK(cudaMemsetAsync(counts, 0, 8 * sizeof(uint32_t), s));
    uint2* st = reinterpret_cast<uint2*>(state);
    const uint32_t n_chunks = (n + kChunk - 1) / kChunk;
    const int blocks = (int)std::min<uint64_t>(n_chunks, (uint64_t)d->grid_blocks);
    const uint32_t hod = hour % 24u;
    if (hod >= 1u && hod <= 6u) {
        k_sleep<<<blocks, kThreads, 0, s>>>(d_params, nullptr, n_chunks, st, ha);
    } else {
        NOALLOC_CK(cudaMemsetAsync(d_claim, 0xFF, claim_bytes, s));
        const DecideKernel decide = decide_kernel(hod);
        decide<<<blocks, kThreads, 0, s>>>(d_params, nullptr, n_chunks, pos, st, home, work, work_start_at, plane, nullptr,
                                           d_claim, d_tgt, nullptr, ha, d_err);
        k_commit<kCommitSlots><<<commit_blocks_for(n), kThreads, 0, s>>>(d_params, nullptr, n, pos, d_tgt, plane, nullptr,
                                                                         d_claim, nullptr, ha, 0ull, nullptr, 0u);
    }
    NOALLOC_CK(cudaGetLastError());
    int err = 0;
    NOALLOC_CK(cudaMemcpyAsync(&err, d_err, sizeof err, cudaMemcpyDeviceToHost, s));
    NOALLOC_CK(cudaStreamSynchronize(s));
    if (err) return noalloc_fail(EPI_ERR_INVARIANT, "epi_tick_hour_noalloc: a rule addressed a cell outside the plane");
    return EPI_OK;
}
