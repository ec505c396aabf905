// engine.cu -- the GB300 engine tick: kernels, the engine handle and the C ABI.
//
// Per simulated hour (CitizenLocationMap::simulate, engine/src/allocation_map.rs:67-129):
//   hours 1..6 of a day   k_sleep   current_area = home (non-staff), counts
//   other hours           k_decide  per-agent rules on the previous-hour plane, proposals,
//                                   atomicMin claims on the target cells, counts
//                         k_commit  lowest claimant moves, losers stay, plane bytes updated,
//                                   claims released
// Hour segments between intervention points run as one captured CUDA graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "host.hpp"
#include "tick.cuh"

using namespace epi;

// ------------------------------------------------------------------ kernels
namespace {

constexpr int kThreads = 256;

// Warp-aggregated 6-bin histogram into shared memory, then one atomic per bin per block.
__device__ __forceinline__ void count_into(uint32_t* sh, bool valid, uint32_t bin) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (uint32_t b = 0; b < 6; ++b) {
        uint32_t c = __popc(__ballot_sync(0xFFFFFFFFu, valid && bin == b));
        if (lane == 0 && c) atomicAdd(&sh[b], c);
    }
}

__device__ __forceinline__ void flush_counts(uint32_t* sh, uint32_t* row) {
    __syncthreads();
    if (threadIdx.x < 6 && sh[threadIdx.x]) atomicAdd(&row[threadIdx.x], sh[threadIdx.x]);
}

// Hours 1..6 (SLEEP_START_TIME..=SLEEP_END_TIME, citizen/mod.rs:244-248).
__global__ void __launch_bounds__(kThreads) k_sleep(const DevParams* __restrict__ Pp, uint2* __restrict__ st,
                                                    uint32_t* __restrict__ counts_row) {
    __shared__ uint32_t sh[8];
    if (threadIdx.x < 8) sh[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t n = Pp->n;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
        const uint32_t i = base + threadIdx.x;
        const bool valid = i < n;
        uint32_t s = 0;
        if (valid) {
            s = st[i].x;
            if (st_ws(s) != EPI_WS_HOSPITAL_STAFF && st_area(s) != kHome) {
                s = with_area(s, kHome);
                st[i].x = s;
            }
        }
        count_into(sh, valid, count_bin(s));
    }
    flush_counts(sh, counts_row);
}

// First vacant hospital cell of the snapshot in AreaIterator order (area.rs:221-237), found
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

// One hour of per-agent rules (hour of day 0, 7..22 or 23).
__global__ void __launch_bounds__(kThreads) k_decide(const DevParams* __restrict__ Pp, const uint32_t* __restrict__ pos,
                                                     uint2* __restrict__ st, const uint32_t* __restrict__ home,
                                                     const uint32_t* __restrict__ work, uint32_t* __restrict__ wsa,
                                                     const uint8_t* __restrict__ plane, uint32_t* __restrict__ claim,
                                                     uint32_t* __restrict__ tgt, uint32_t* __restrict__ counts_row,
                                                     const uint32_t* __restrict__ hour_base, uint32_t hour_offset,
                                                     int* err) {
    __shared__ uint32_t sh[8];
    __shared__ DevParams sP;  // the parameter block, staged once per block
    if (threadIdx.x < 8) sh[threadIdx.x] = 0;
    for (uint32_t k = threadIdx.x; k < sizeof(DevParams) / 4; k += blockDim.x)
        reinterpret_cast<uint32_t*>(&sP)[k] = reinterpret_cast<const uint32_t*>(Pp)[k];
    __syncthreads();
    const DevParams& P = sP;
    const uint32_t hour = *hour_base + hour_offset;
    const uint32_t hod = hour % 24u;
    const PlaneView pl{plane, P.G, P.WP, err};
    const uint32_t n = P.n;
    const uint32_t stride = gridDim.x * blockDim.x;
    uint32_t hosp_first = kNoAction;
    bool hosp_known = false;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
        const uint32_t i = base + threadIdx.x;
        const bool valid = i < n;
        uint32_t s = 0, at = 0, p = 0;
        if (valid) {
            const uint2 sv = st[i];
            s = sv.x;
            at = sv.y;
            p = pos[i];
        }
        if (hod == 0u) {
            const bool need = valid && wants_hospital(P, infected(s) ? with_day(s, st_day(s) + 1u) : s);
            if (__syncthreads_or(need) && !hosp_known) {
                hosp_first = block_first_vacant(P, pl);
                hosp_known = true;
            }
        }
        uint32_t bin = 0;
        if (valid) {
            const uint32_t s0 = s, at0 = at;
            const uint32_t hm = home[i], wk = work[i];
            const Cell cell{unpack_x(p), unpack_y(p)};
            Draws dr{i, hour, P.key0, P.key1};
            Cell nc;
            if (hod == 0u) {
                nc = routine_start(P, pl, s, hm, cell, hosp_first, dr);
            } else if (hod == 23u) {
                nc = routine_end(P, pl, s, hm, cell, dr);
            } else {
                const bool staff = st_ws(s) == EPI_WS_HOSPITAL_STAFF;
                uint32_t w0 = staff ? wsa[i] : 0u, w = w0;
                nc = perform_movements(P, pl, s, at, w, hm, wk, cell, hod, hour, dr);
                if (staff && w != w0) wsa[i] = w;
            }
            bool moving = nc.x != cell.x || nc.y != cell.y;
            if (moving && ((uint32_t)nc.x > (uint32_t)P.G || (uint32_t)nc.y > (uint32_t)P.G)) {
                atomicOr(err, 4);  // unreachable for validated worlds; never write outside the plane
                moving = false;
                nc = cell;
            }
            const uint32_t cls = cell_class(P, s);
            if (moving) atomicMin(&claim[(size_t)nc.y * P.W + nc.x], i);
            tgt[i] = (moving || cls != cell_class(P, s0)) ? encode_target(nc, cls) : kNoAction;
            if (s != s0 || at != at0) st[i] = make_uint2(s, at);
            bin = count_bin(s);
        }
        count_into(sh, valid, bin);
    }
    flush_counts(sh, counts_row);
}

// Resolve the claims of the hour: the lowest index that claimed a cell moves there
// (the serial resolve of allocation_map.rs:93-102 in index order), others keep their cell.
__global__ void __launch_bounds__(kThreads) k_commit(const DevParams* __restrict__ Pp, uint32_t* __restrict__ pos,
                                                     const uint32_t* __restrict__ tgt, uint8_t* __restrict__ plane,
                                                     uint32_t* __restrict__ claim) {
    const uint32_t n = Pp->n, W = (uint32_t)Pp->W, WP = (uint32_t)Pp->WP;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint32_t t = tgt[i];
        if (t == kNoAction) continue;
        const uint32_t p = pos[i];
        const uint32_t xy = target_xy(t), cls = target_class(t);
        const size_t old_cell = (size_t)(unpack_y(p) + 1) * WP + (unpack_x(p) + 1);
        if (xy != p) {
            const size_t claim_cell = (size_t)unpack_y(xy) * W + unpack_x(xy);
            if (claim[claim_cell] == i) {
                claim[claim_cell] = kNoClaim;
                plane[old_cell] = 0;
                plane[(size_t)(unpack_y(xy) + 1) * WP + (unpack_x(xy) + 1)] = (uint8_t)cls;
                pos[i] = xy;
                continue;
            }
        }
        plane[old_cell] = (uint8_t)cls;
    }
}

__global__ void k_build_plane(const DevParams* __restrict__ Pp, const uint32_t* __restrict__ pos,
                              const uint2* __restrict__ st, uint8_t* __restrict__ plane, int* err) {
    const uint32_t n = Pp->n;
    const int32_t G = Pp->G, WP = Pp->WP;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t p = pos[i];
        const int32_t x = unpack_x(p), y = unpack_y(p);
        if (x > G || y > G) { atomicOr(err, 2); continue; }
        plane[(size_t)(y + 1) * WP + (x + 1)] = (uint8_t)cell_class(*Pp, st[i].x);
    }
}

// LockdownIntervention apply / revoke (allocation_map.rs:349-365).
__global__ void k_lock(const DevParams* __restrict__ Pp, uint2* __restrict__ st, int on) {
    const uint32_t n = Pp->n;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t s = st[i].x;
        uint32_t ns = on ? (st_ws(s) != EPI_WS_ESSENTIAL ? (s | kIso) : s) : (s & ~kIso);
        if (ns != s) st[i].x = ns;
    }
}

// vaccinate (allocation_map.rs:381-387): susceptible agents with Philox block 3 word 0 < thr.
__global__ void k_vaccinate(const DevParams* __restrict__ Pp, uint2* __restrict__ st, uint32_t hour, uint64_t thr) {
    const uint32_t n = Pp->n;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t s = st[i].x;
        if ((s & kStateMask) != EPI_S) continue;
        uint32_t u[4];
        philox4x32(i, hour, kBlkVaccine, 0u, Pp->key0, Pp->key1, u);
        if ((uint64_t)u[0] < thr) st[i].x = s | kVacc;
    }
}

// Invariants: each agent's cell holds its class; occupied cells == n; claims all free.
__global__ void k_check_agents(const DevParams* __restrict__ Pp, const uint32_t* __restrict__ pos,
                               const uint2* __restrict__ st, const uint8_t* __restrict__ plane,
                               unsigned long long* bad) {
    const uint32_t n = Pp->n;
    const int32_t G = Pp->G, WP = Pp->WP;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t p = pos[i];
        const int32_t x = unpack_x(p), y = unpack_y(p);
        if (x > G || y > G || plane[(size_t)(y + 1) * WP + (x + 1)] != cell_class(*Pp, st[i].x)) atomicAdd(bad, 1ull);
    }
}

__global__ void k_check_plane(size_t plane_bytes, const uint8_t* __restrict__ plane, size_t claim_cells,
                              const uint32_t* __restrict__ claim, unsigned long long* occupied,
                              unsigned long long* claimed) {
    unsigned long long o = 0, c = 0;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < plane_bytes; k += stride) o += plane[k] != 0;
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < claim_cells; k += stride) c += claim[k] != kNoClaim;
    for (int off = 16; off; off >>= 1) {
        o += __shfl_down_sync(0xFFFFFFFFu, o, off);
        c += __shfl_down_sync(0xFFFFFFFFu, c, off);
    }
    if ((threadIdx.x & 31) == 0) {
        if (o) atomicAdd(occupied, o);
        if (c) atomicAdd(claimed, c);
    }
}

}  // namespace

// ------------------------------------------------------------------ engine handle
enum KernelKind { kKDecide = 0, kKCommit, kKSleep, kKLock, kKVaccinate, kKBuildPlane, kKCheck, kKindCount };
static const char* kKernelNames[kKindCount] = {"k_decide", "k_commit", "k_sleep", "k_lock", "k_vaccinate", "k_build_plane", "k_check"};

struct epi_engine {
    epi_params p{};
    epi_geography geo0{}, geo{};
    DevParams hp{};
    uint32_t n = 0;
    size_t plane_bytes = 0;  // padded byte plane (G+3)^2 + slack
    size_t claim_cells = 0;  // (G+1)^2
    int grid_blocks = 0;    // resident grid of the counting kernels (grid-stride loops)
    int commit_blocks = 0;  // one thread per agent
    // device
    DevParams* d_params = nullptr;
    uint32_t *d_pos = nullptr, *d_home = nullptr, *d_work = nullptr, *d_wsa = nullptr, *d_tgt = nullptr;
    uint2* d_st = nullptr;
    uint8_t* d_plane = nullptr;
    uint32_t* d_claim = nullptr;
    uint32_t* d_counts = nullptr;
    uint32_t* d_hour_base = nullptr;
    int* d_err = nullptr;
    unsigned long long* d_scratch = nullptr;
    uint32_t counts_capacity = 0;
    // host
    uint32_t* h_counts = nullptr;  // pinned
    uint32_t* h_hour_base = nullptr;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::map<std::pair<uint32_t, uint32_t>, cudaGraphExec_t> graphs;  // (first hour mod 24, hours)
    InterventionState iv;
    std::vector<epi_counts> rows;
    std::string err;
    bool profiling = false;
    uint32_t launches[kKindCount] = {};
    double total_ms[kKindCount] = {};
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> pending;
    std::vector<cudaEvent_t> event_pool;
    uint64_t kernels_launched = 0;
    // device-side checkpoint (epi_engine_save_state / epi_engine_restore_state)
    uint32_t *s_pos = nullptr, *s_wsa = nullptr;
    uint2* s_st = nullptr;
    uint8_t* s_plane = nullptr;
    bool saved = false;
    InterventionState s_iv;
    uint32_t s_hosp_code = kHosp0;
    epi_geography s_geo{};
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

static uint32_t area_code_of(const epi_engine* h, const epi_agent_record& r, bool* ok) {
    Rect a{r.area_x0, r.area_y0, r.area_x1, r.area_y1};
    *ok = true;
    if (rect_eq(a, Rect{r.home_x, r.home_y, r.home_x + 1, r.home_y + 1})) return kHome;
    if (r.work_status != EPI_WS_NA && rect_eq(a, Rect{r.work_x, r.work_y, r.work_x + 9, r.work_y + 9})) return kWork;
    for (uint32_t c = kTransport; c < kNumAreas; ++c)
        if (rect_eq(a, h->hp.area[c])) return c;
    *ok = false;
    return kHome;
}

static Rect to_rect(const epi_area& a) { return Rect{a.x0, a.y0, a.x1, a.y1}; }

static void fill_dev_params(epi_engine* h) {
    DevParams& d = h->hp;
    std::memset(&d, 0, sizeof d);
    const epi_params& p = h->p;
    d.n = h->n;
    d.G = (int32_t)p.grid_size;
    d.W = d.G + 1;
    d.WP = d.G + 3;
    d.hosp_code = kHosp0;
    d.area[kTransport] = to_rect(h->geo0.transport);
    d.area[kHousing] = to_rect(h->geo0.housing);
    d.area[kHosp0] = to_rect(h->geo0.hospital);
    d.area[kHosp1] = to_rect(grown_hospital(h->geo0));
    d.key0 = (uint32_t)p.seed;
    d.key1 = (uint32_t)(p.seed >> 32);
    d.reg_start = p.regular_transmission_start_day;
    d.high_start = p.high_transmission_start_day;
    d.last_day = p.last_day;
    d.exposed_duration = p.exposed_duration;
    d.pre_duration = p.pre_symptomatic_duration;
    const double rates[3] = {0.0, p.regular_transmission_rate, p.high_transmission_rate};
    d.hosp_if_class = 0;
    for (int c = 0; c < 3; ++c) {
        d.thr_rate[c] = bernoulli_threshold(rates[c]);
        if (rates[c] >= p.high_transmission_rate) d.hosp_if_class |= 1u << c;  // is_to_be_hospitalized
    }
    d.thr_death = bernoulli_threshold(p.death_rate);
    d.thr_symptoms = bernoulli_threshold(1.0 - p.percentage_asymptomatic_population);
    d.thr_severe = bernoulli_threshold(p.percentage_severe_infected_population);
}

static int record_launch_begin(epi_engine* h, int kind, cudaEvent_t* out_end) {
    if (!h->profiling) return EPI_OK;
    cudaEvent_t a, b;
    if (h->event_pool.size() >= 2) {
        a = h->event_pool.back(); h->event_pool.pop_back();
        b = h->event_pool.back(); h->event_pool.pop_back();
    } else {
        CK(cudaEventCreate(&a));
        CK(cudaEventCreate(&b));
    }
    CK(cudaEventRecord(a, h->stream));
    h->pending.push_back({kind, {a, b}});
    *out_end = b;
    return EPI_OK;
}

static int record_launch_end(epi_engine* h, cudaEvent_t end) {
    if (!h->profiling) return EPI_OK;
    CK(cudaEventRecord(end, h->stream));
    return EPI_OK;
}

static int harvest_events(epi_engine* h) {
    for (auto& pe : h->pending) {
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, pe.second.first, pe.second.second));
        h->launches[pe.first]++;
        h->total_ms[pe.first] += ms;
        h->event_pool.push_back(pe.second.first);
        h->event_pool.push_back(pe.second.second);
    }
    h->pending.clear();
    return EPI_OK;
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

static int ensure_counts(epi_engine* h, uint32_t rows_needed) {
    if (rows_needed <= h->counts_capacity) return EPI_OK;
    uint32_t cap = std::max<uint32_t>(rows_needed, 64);
    if (h->d_counts) CK(cudaFree(h->d_counts));
    if (h->h_counts) CK(cudaFreeHost(h->h_counts));
    h->d_counts = nullptr;
    h->h_counts = nullptr;
    CK(cudaMalloc(&h->d_counts, (size_t)cap * 8 * sizeof(uint32_t)));
    CK(cudaMallocHost(&h->h_counts, (size_t)cap * 8 * sizeof(uint32_t)));
    h->counts_capacity = cap;
    // cached graphs reference the old counts buffer
    for (auto& g : h->graphs) cudaGraphExecDestroy(g.second);
    h->graphs.clear();
    return EPI_OK;
}

// Issue the kernels of hours hour_base .. hour_base + n - 1 (hour_base read on the device).
static int enqueue_hours(epi_engine* h, uint32_t first_hour, uint32_t nh) {
    CK(cudaMemsetAsync(h->d_counts, 0, (size_t)nh * 8 * sizeof(uint32_t), h->stream));
    const int blocks = h->grid_blocks;
    for (uint32_t k = 0; k < nh; ++k) {
        const uint32_t hod = (first_hour + k) % 24u;
        uint32_t* row = h->d_counts + (size_t)k * 8;
        if (hod >= 1u && hod <= 6u) {
            LAUNCH(kKSleep, (k_sleep<<<blocks, kThreads, 0, h->stream>>>(h->d_params, h->d_st, row)));
        } else {
            LAUNCH(kKDecide, (k_decide<<<blocks, kThreads, 0, h->stream>>>(
                                  h->d_params, h->d_pos, h->d_st, h->d_home, h->d_work, h->d_wsa, h->d_plane, h->d_claim,
                                  h->d_tgt, row, h->d_hour_base, k, h->d_err)));
            LAUNCH(kKCommit, (k_commit<<<h->commit_blocks, kThreads, 0, h->stream>>>(h->d_params, h->d_pos, h->d_tgt, h->d_plane,
                                                                           h->d_claim)));
        }
    }
    CK(cudaMemcpyAsync(h->h_counts, h->d_counts, (size_t)nh * 8 * sizeof(uint32_t), cudaMemcpyDeviceToHost, h->stream));
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

static int run_hours(epi_engine* h, uint32_t first_hour, uint32_t nh, epi_counts* out) {
    if (nh == 0) return EPI_OK;
    if ((uint64_t)first_hour + nh > 0xFFFFFFFFull) { h->err = "hour out of range"; return EPI_ERR_ARG; }
    int rc = ensure_counts(h, nh);
    if (rc) return rc;
    *h->h_hour_base = first_hour;
    CK(cudaMemcpyAsync(h->d_hour_base, h->h_hour_base, sizeof(uint32_t), cudaMemcpyHostToDevice, h->stream));
    if (h->profiling) {
        rc = enqueue_hours(h, first_hour, nh);
        if (rc) return rc;
    } else {
        auto key = std::make_pair(first_hour % 24u, nh);
        auto it = h->graphs.find(key);
        if (it == h->graphs.end()) {
            cudaGraph_t g;
            CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
            rc = enqueue_hours(h, first_hour, nh);
            cudaError_t ce = cudaStreamEndCapture(h->stream, &g);
            if (rc) return rc;
            if (ce != cudaSuccess) { h->err = std::string("graph capture: ") + cudaGetErrorString(ce); return EPI_ERR_CUDA; }
            cudaGraphExec_t ge;
            ce = cudaGraphInstantiate(&ge, g, 0);
            cudaGraphDestroy(g);
            if (ce != cudaSuccess) { h->err = std::string("graph instantiate: ") + cudaGetErrorString(ce); return EPI_ERR_CUDA; }
            it = h->graphs.emplace(key, ge).first;
        }
        CK(cudaGraphLaunch(it->second, h->stream));
    }
    CK(cudaStreamSynchronize(h->stream));
    for (uint32_t k = 0; k < nh; ++k) {
        const uint32_t hod = (first_hour + k) % 24u;
        h->kernels_launched += (hod >= 1u && hod <= 6u) ? 1u : 2u;
    }
    rc = harvest_events(h);
    if (rc) return rc;
    rc = check_error_flag(h);
    if (rc) return rc;
    for (uint32_t k = 0; k < nh; ++k) {
        const uint32_t* c = h->h_counts + (size_t)k * 8;
        epi_counts& o = out[k];
        o.hour = first_hour + k;
        o.susceptible = c[0];
        o.exposed = c[1];
        o.infected = c[2];
        o.hospitalized = c[3];
        o.recovered = c[4];
        o.deceased = c[5];
        uint64_t total = (uint64_t)c[0] + c[1] + c[2] + c[3] + c[4] + c[5];
        if (total != h->n) {  // assert_eq!(csv_record.total(), current_population), allocation_map.rs:128
            h->err = "counts total " + std::to_string(total) + " != population " + std::to_string(h->n);
            return EPI_ERR_INVARIANT;
        }
    }
    return EPI_OK;
}

static void free_device(epi_engine* h) {
    for (auto& g : h->graphs) cudaGraphExecDestroy(g.second);
    h->graphs.clear();
    cudaFree(h->d_params); cudaFree(h->d_pos); cudaFree(h->d_home); cudaFree(h->d_work); cudaFree(h->d_wsa);
    cudaFree(h->d_tgt); cudaFree(h->d_st); cudaFree(h->d_plane); cudaFree(h->d_claim); cudaFree(h->d_counts);
    cudaFree(h->d_hour_base); cudaFree(h->d_err); cudaFree(h->d_scratch);
    cudaFree(h->s_pos); cudaFree(h->s_wsa); cudaFree(h->s_st); cudaFree(h->s_plane);
    if (h->h_counts) cudaFreeHost(h->h_counts);
    if (h->h_hour_base) cudaFreeHost(h->h_hour_base);
    for (auto& pe : h->pending) { cudaEventDestroy(pe.second.first); cudaEventDestroy(pe.second.second); }
    for (auto e : h->event_pool) cudaEventDestroy(e);
    if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
}

static int upload_world(epi_engine* h, const epi_agent_record* recs) {
    const uint32_t n = h->n;
    std::vector<uint32_t> pos(n), home(n), work(n), wsa(n);
    std::vector<uint2> st(n);
    for (uint32_t i = 0; i < n; ++i) {
        const epi_agent_record& r = recs[i];
        const int32_t G = (int32_t)h->p.grid_size;
        auto inside = [G](int32_t x0, int32_t y0, int32_t x1, int32_t y1) {
            return x0 >= 0 && y0 >= 0 && x1 <= G && y1 <= G && x0 <= x1 && y0 <= y1;
        };
        if (r.x < 0 || r.y < 0 || r.x > G || r.y > G || r.state > EPI_D || r.work_status > EPI_WS_NA ||
            r.immunity < -2 || r.immunity > 2 || r.infection_day > 0xFFFFu ||
            !inside(r.home_x, r.home_y, r.home_x + 1, r.home_y + 1) ||
            (r.work_status != EPI_WS_NA && !inside(r.work_x, r.work_y, r.work_x + 9, r.work_y + 9)) ||
            !inside(r.area_x0, r.area_y0, r.area_x1, r.area_y1)) {
            h->err = "agent record " + std::to_string(i) + " out of range";
            return EPI_ERR_ARG;
        }
        bool ok = true;
        uint32_t code = area_code_of(h, r, &ok);
        if (!ok) { h->err = "agent record " + std::to_string(i) + ": current area is not one of its areas"; return EPI_ERR_ARG; }
        uint32_t s = (uint32_t)r.state;
        if (r.flags & EPI_F_HOSPITALIZED) s |= kHosp;
        if (r.flags & EPI_F_ISOLATED) s |= kIso;
        if (r.flags & EPI_F_VACCINATED) s |= kVacc;
        if (r.flags & EPI_F_WORK_QUARANTINED) s |= kWq;
        if (r.flags & EPI_F_PUBLIC_TRANSPORT) s |= kPt;
        s |= code << kAreaShift;
        s |= (uint32_t)r.work_status << kWsShift;
        s |= (uint32_t)(r.immunity + 2) << kImmShift;
        s |= r.infection_day << kDayShift;
        st[i] = make_uint2(s, r.at_hour);
        pos[i] = pack_xy(r.x, r.y);
        home[i] = pack_xy(r.home_x, r.home_y);
        work[i] = pack_xy(r.work_x, r.work_y);
        wsa[i] = r.work_start_at;
    }
    CK(cudaMemcpyAsync(h->d_pos, pos.data(), n * sizeof(uint32_t), cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->d_home, home.data(), n * sizeof(uint32_t), cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->d_work, work.data(), n * sizeof(uint32_t), cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->d_wsa, wsa.data(), n * sizeof(uint32_t), cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->d_st, st.data(), n * sizeof(uint2), cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemsetAsync(h->d_plane, 0, h->plane_bytes, h->stream));
    CK(cudaMemsetAsync(h->d_claim, 0xFF, h->claim_cells * sizeof(uint32_t), h->stream));
    CK(cudaMemsetAsync(h->d_err, 0, sizeof(int), h->stream));
    LAUNCH(kKBuildPlane, (k_build_plane<<<h->grid_blocks, kThreads, 0, h->stream>>>(h->d_params, h->d_pos, h->d_st,
                                                                                      h->d_plane, h->d_err)));
    CK(cudaStreamSynchronize(h->stream));  // host vectors go out of scope
    int rc = harvest_events(h);
    if (rc) return rc;
    return check_error_flag(h);
}

static int engine_init(epi_engine* h, const epi_params& p, const epi_agent_record* recs, size_t n) {
    h->p = p;
    std::string bad = validate_params(p);
    if (!bad.empty()) { h->err = bad; return EPI_ERR_CONFIG; }
    if (n != p.number_of_agents || n == 0 || n >= 0xFFFFFFFFull) { h->err = "record count != number_of_agents"; return EPI_ERR_ARG; }
    h->n = (uint32_t)n;
    h->geo0 = define_geography(p.grid_size);
    resize_hospital(h->geo0, (int32_t)n, 0.002, p.hospital_beds_percentage);
    h->geo = h->geo0;
    fill_dev_params(h);
    const size_t W = (size_t)p.grid_size + 1;
    h->claim_cells = W * W;
    h->plane_bytes = (W + 2) * (W + 2) + 16;  // border of one cell, 16 B slack for the row loads
    int dev = 0, sms = 0, per_sm = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_decide, kThreads, 0));
    per_sm = std::max(per_sm, 1);
    const uint64_t need_blocks = ((uint64_t)n + kThreads - 1) / kThreads;
    h->grid_blocks = (int)std::min<uint64_t>(need_blocks, (uint64_t)sms * per_sm);
    h->commit_blocks = (int)need_blocks;
    CK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    h->own_stream = true;
    CK(cudaMalloc(&h->d_params, sizeof(DevParams)));
    CK(cudaMalloc(&h->d_pos, n * sizeof(uint32_t)));
    CK(cudaMalloc(&h->d_home, n * sizeof(uint32_t)));
    CK(cudaMalloc(&h->d_work, n * sizeof(uint32_t)));
    CK(cudaMalloc(&h->d_wsa, n * sizeof(uint32_t)));
    CK(cudaMalloc(&h->d_tgt, n * sizeof(uint32_t)));
    CK(cudaMalloc(&h->d_st, n * sizeof(uint2)));
    CK(cudaMalloc(&h->d_plane, h->plane_bytes));
    CK(cudaMalloc(&h->d_claim, h->claim_cells * sizeof(uint32_t)));
    CK(cudaMalloc(&h->d_hour_base, sizeof(uint32_t)));
    CK(cudaMalloc(&h->d_err, sizeof(int)));
    CK(cudaMalloc(&h->d_scratch, 4 * sizeof(unsigned long long)));
    CK(cudaMallocHost(&h->h_hour_base, sizeof(uint32_t)));
    CK(cudaMemcpyAsync(h->d_params, &h->hp, sizeof(DevParams), cudaMemcpyHostToDevice, h->stream));
    int rc = ensure_counts(h, 48);
    if (rc) return rc;
    return upload_world(h, recs);
}

static int push_params(epi_engine* h) {
    CK(cudaMemcpyAsync(h->d_params, &h->hp, sizeof(DevParams), cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return EPI_OK;
}

static int finish_bulk(epi_engine* h) {
    CK(cudaStreamSynchronize(h->stream));
    h->kernels_launched += 1;
    return harvest_events(h);
}

// ------------------------------------------------------------------ C ABI
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

int epi_world_build(const epi_params* p, epi_agent_record* out, size_t n, epi_geography* geo) {
    if (!p || !out || n != p->number_of_agents) return EPI_ERR_ARG;
    std::vector<epi_agent_record> recs;
    epi_geography g;
    std::string err;
    int rc = build_world(*p, recs, g, err);
    if (rc) { g_create_error = err; return rc; }
    std::memcpy(out, recs.data(), n * sizeof(epi_agent_record));
    if (geo) *geo = g;
    return EPI_OK;
}

int epi_engine_create_from_records(const epi_params* params, const epi_agent_record* recs, size_t n, epi_engine** out) {
    if (!params || !recs || !out) return EPI_ERR_ARG;
    *out = nullptr;
    epi_engine* h = new epi_engine();
    int rc = engine_init(h, *params, recs, n);
    if (rc) {
        g_create_error = h->err;
        free_device(h);
        delete h;
        return rc;
    }
    *out = h;
    return EPI_OK;
}

int epi_engine_create(const epi_params* params, epi_engine** out) {
    if (!params || !out) return EPI_ERR_ARG;
    *out = nullptr;
    std::vector<epi_agent_record> recs;
    epi_geography g;
    std::string err;
    int rc = build_world(*params, recs, g, err);
    if (rc) { g_create_error = err; return rc; }
    return epi_engine_create_from_records(params, recs.data(), recs.size(), out);
}

int epi_engine_create_json(const char* config_json, uint64_t seed, epi_engine** out) {
    if (!out) return EPI_ERR_ARG;
    *out = nullptr;
    epi_params p;
    char msg[512] = {0};
    int rc = epi_params_from_json(config_json, &p, msg, sizeof msg);
    if (rc) { g_create_error = msg; return rc; }
    p.seed = seed;
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

int epi_engine_simulate(epi_engine* h, uint32_t hour, epi_counts* out) {
    if (!h || !out) return EPI_ERR_ARG;
    return run_hours(h, hour, 1, out);
}

int epi_engine_simulate_hours(epi_engine* h, uint32_t first_hour, uint32_t n, epi_counts* out) {
    if (!h || (!out && n)) return EPI_ERR_ARG;
    return run_hours(h, first_hour, n, out);
}

int epi_engine_lock_city(epi_engine* h) {
    if (!h) return EPI_ERR_ARG;
    LAUNCH(kKLock, (k_lock<<<h->grid_blocks, kThreads, 0, h->stream>>>(h->d_params, h->d_st, 1)));
    return finish_bulk(h);
}

int epi_engine_unlock_city(epi_engine* h) {
    if (!h) return EPI_ERR_ARG;
    LAUNCH(kKLock, (k_lock<<<h->grid_blocks, kThreads, 0, h->stream>>>(h->d_params, h->d_st, 0)));
    return finish_bulk(h);
}

int epi_engine_vaccinate(epi_engine* h, uint32_t hour, double percent) {
    if (!h || !(percent >= 0.0 && percent <= 1.0)) return EPI_ERR_ARG;
    const uint64_t thr = bernoulli_threshold(percent);
    LAUNCH(kKVaccinate, (k_vaccinate<<<h->grid_blocks, kThreads, 0, h->stream>>>(h->d_params, h->d_st, hour, thr)));
    return finish_bulk(h);
}

int epi_engine_increase_hospital_size(epi_engine* h) {
    if (!h) return EPI_ERR_ARG;
    const epi_area grown = grown_hospital(h->geo0);
    h->geo.hospital = grown;
    h->hp.hosp_code = rect_eq(to_rect(grown), h->hp.area[kHosp0]) ? kHosp0 : kHosp1;
    return push_params(h);
}

int epi_engine_process_interventions(epi_engine* h, const epi_counts* counts, uint32_t* applied) {
    if (!h || !counts) return EPI_ERR_ARG;
    InterventionActions a = decide_interventions(h->p, h->iv, *counts, h->geo.hospital);
    int rc = EPI_OK;
    if (a.vaccinate && (rc = epi_engine_vaccinate(h, counts->hour, a.vaccinate_percent))) return rc;
    if (a.lock && (rc = epi_engine_lock_city(h))) return rc;
    if (a.unlock && (rc = epi_engine_unlock_city(h))) return rc;
    if (a.grow_hospital && (rc = epi_engine_increase_hospital_size(h))) return rc;
    if (applied) *applied = a.applied;
    return EPI_OK;
}

int epi_engine_run(epi_engine* h, epi_counts* rows, uint32_t max_rows, uint32_t* n_rows) {
    if (!h || !n_rows) return EPI_ERR_ARG;
    *n_rows = 0;
    h->rows.clear();
    const uint32_t hours = h->p.hours;
    std::vector<epi_counts> seg;
    uint32_t hour = 1;
    bool stop = false;
    while (hour < hours && !stop) {
        uint32_t end = hour;  // last hour of the segment: next intervention point or the last hour
        while (end + 1 < hours && !is_event_hour(h->p, end)) ++end;
        const uint32_t nh = end - hour + 1;
        seg.resize(nh);
        int rc = run_hours(h, hour, nh, seg.data());
        if (rc) return rc;
        for (uint32_t k = 0; k < nh; ++k) {
            h->rows.push_back(seg[k]);
            // interventions can only fire at the segment's last hour (an event hour)
            if (k + 1 == nh) {
                rc = epi_engine_process_interventions(h, &seg[k], nullptr);
                if (rc) return rc;
            }
            // stop_simulation, epidemiology_simulation.rs:564-575 (standalone)
            if (seg[k].exposed == 0 && seg[k].infected == 0 && seg[k].hospitalized == 0) { stop = true; break; }
        }
        hour = end + 1;
    }
    const uint32_t nr = (uint32_t)h->rows.size();
    if (rows) {
        if (max_rows < nr) { h->err = "rows buffer too small"; return EPI_ERR_ARG; }
        std::memcpy(rows, h->rows.data(), nr * sizeof(epi_counts));
    }
    *n_rows = nr;
    return EPI_OK;
}

int epi_engine_write_outputs(epi_engine* h, const char* dir, const char* engine_id) {
    if (!h || !dir || !engine_id) return EPI_ERR_ARG;
    return write_outputs(dir, engine_id, h->rows, h->iv.reports, h->err);
}

int epi_engine_population(const epi_engine* h, uint32_t* out) {
    if (!h || !out) return EPI_ERR_ARG;
    *out = h->n;
    return EPI_OK;
}

int epi_engine_geography(const epi_engine* h, epi_geography* out) {
    if (!h || !out) return EPI_ERR_ARG;
    *out = h->geo;
    return EPI_OK;
}

int epi_engine_snapshot(epi_engine* h, epi_agent_record* out, size_t n) {
    if (!h || !out || n != h->n) return EPI_ERR_ARG;
    std::vector<uint32_t> pos(n), home(n), work(n), wsa(n);
    std::vector<uint2> st(n);
    CK(cudaMemcpyAsync(pos.data(), h->d_pos, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(home.data(), h->d_home, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(work.data(), h->d_work, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(wsa.data(), h->d_wsa, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(st.data(), h->d_st, n * sizeof(uint2), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    for (size_t i = 0; i < n; ++i) {
        epi_agent_record& r = out[i];
        std::memset(&r, 0, sizeof r);
        const uint32_t s = st[i].x, v = s & kStateMask;
        r.x = unpack_x(pos[i]);
        r.y = unpack_y(pos[i]);
        r.state = (uint8_t)v;
        r.flags = (uint8_t)(((s & kHosp) ? EPI_F_HOSPITALIZED : 0) | ((s & kIso) ? EPI_F_ISOLATED : 0) |
                            ((s & kVacc) ? EPI_F_VACCINATED : 0) | ((s & kWq) ? EPI_F_WORK_QUARANTINED : 0) |
                            ((s & kPt) ? EPI_F_PUBLIC_TRANSPORT : 0));
        r.work_status = (uint8_t)st_ws(s);
        r.immunity = (int8_t)st_imm(s);
        r.at_hour = (v == EPI_E || v == EPI_I_PRE) ? st[i].y : 0u;
        r.infection_day = infected(s) ? st_day(s) : 0u;
        r.work_start_at = st_ws(s) == EPI_WS_HOSPITAL_STAFF ? wsa[i] : 0u;
        r.home_x = unpack_x(home[i]);
        r.home_y = unpack_y(home[i]);
        r.work_x = unpack_x(work[i]);
        r.work_y = unpack_y(work[i]);
        const uint32_t code = st_area(s);
        Rect a = code == kHome ? Rect{r.home_x, r.home_y, r.home_x + 1, r.home_y + 1}
                 : code == kWork ? Rect{r.work_x, r.work_y, r.work_x + 9, r.work_y + 9}
                                 : h->hp.area[code < kNumAreas ? code : kHome];
        r.area_x0 = a.x0; r.area_y0 = a.y0; r.area_x1 = a.x1; r.area_y1 = a.y1;
    }
    return EPI_OK;
}

int epi_engine_check(epi_engine* h) {
    if (!h) return EPI_ERR_ARG;
    CK(cudaMemsetAsync(h->d_scratch, 0, 4 * sizeof(unsigned long long), h->stream));
    LAUNCH(kKCheck, (k_check_agents<<<h->grid_blocks, kThreads, 0, h->stream>>>(h->d_params, h->d_pos, h->d_st, h->d_plane,
                                                                                 h->d_scratch)));
    LAUNCH(kKCheck, (k_check_plane<<<h->grid_blocks, kThreads, 0, h->stream>>>(h->plane_bytes, h->d_plane, h->claim_cells, h->d_claim,
                                                                                h->d_scratch + 1, h->d_scratch + 2)));
    unsigned long long v[4] = {0, 0, 0, 0};
    CK(cudaMemcpyAsync(v, h->d_scratch, sizeof v, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    int rc = harvest_events(h);
    if (rc) return rc;
    if (v[0] || v[1] != h->n || v[2]) {
        h->err = "invariants: " + std::to_string(v[0]) + " agents off their cell class, " + std::to_string(v[1]) +
                 " occupied cells for " + std::to_string(h->n) + " agents, " + std::to_string(v[2]) + " stale claims";
        return EPI_ERR_INVARIANT;
    }
    return EPI_OK;
}

int epi_engine_save_state(epi_engine* h) {
    if (!h) return EPI_ERR_ARG;
    const size_t n = h->n;
    if (!h->s_pos) {
        CK(cudaMalloc(&h->s_pos, n * sizeof(uint32_t)));
        CK(cudaMalloc(&h->s_wsa, n * sizeof(uint32_t)));
        CK(cudaMalloc(&h->s_st, n * sizeof(uint2)));
        CK(cudaMalloc(&h->s_plane, h->plane_bytes));
    }
    CK(cudaMemcpyAsync(h->s_pos, h->d_pos, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, h->stream));
    CK(cudaMemcpyAsync(h->s_wsa, h->d_wsa, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, h->stream));
    CK(cudaMemcpyAsync(h->s_st, h->d_st, n * sizeof(uint2), cudaMemcpyDeviceToDevice, h->stream));
    CK(cudaMemcpyAsync(h->s_plane, h->d_plane, h->plane_bytes, cudaMemcpyDeviceToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    h->s_iv = h->iv;
    h->s_hosp_code = h->hp.hosp_code;
    h->s_geo = h->geo;
    h->saved = true;
    return EPI_OK;
}

int epi_engine_restore_state(epi_engine* h) {
    if (!h) return EPI_ERR_ARG;
    if (!h->saved) { h->err = "no saved state"; return EPI_ERR_ARG; }
    const size_t n = h->n;
    CK(cudaMemcpyAsync(h->d_pos, h->s_pos, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, h->stream));
    CK(cudaMemcpyAsync(h->d_wsa, h->s_wsa, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, h->stream));
    CK(cudaMemcpyAsync(h->d_st, h->s_st, n * sizeof(uint2), cudaMemcpyDeviceToDevice, h->stream));
    CK(cudaMemcpyAsync(h->d_plane, h->s_plane, h->plane_bytes, cudaMemcpyDeviceToDevice, h->stream));
    h->iv = h->s_iv;
    h->geo = h->s_geo;
    if (h->hp.hosp_code != h->s_hosp_code) {
        h->hp.hosp_code = h->s_hosp_code;
        CK(cudaMemcpyAsync(h->d_params, &h->hp, sizeof(DevParams), cudaMemcpyHostToDevice, h->stream));
    }
    CK(cudaStreamSynchronize(h->stream));
    h->rows.clear();
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
    return 0;
}

// Algorithmic bytes of one hour (the roofline numerator): the agent words the hour's
// kernels must read and write plus one pass over the occupancy plane.
//   movement hours and hours 0/23:  decide reads pos 4 + st 8 + home 4 + work 4, writes
//   st 8 + tgt 4; commit reads tgt 4 + pos 4, writes pos 4; plane (G+1)^2 bytes read once.
//   sleep hours: st.x read 4 (+ write 4 on the first sleep hour).
int epi_engine_hour_bytes(const epi_engine* h, uint32_t hour, double* bytes) {
    if (!h || !bytes) return EPI_ERR_ARG;
    const uint32_t hod = hour % 24u;
    const double n = (double)h->n;
    if (hod >= 1u && hod <= 6u) *bytes = n * (hod == 1u ? 8.0 : 4.0);
    else *bytes = n * 44.0 + (double)h->claim_cells;
    return EPI_OK;
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
constexpr size_t kNoAllocHourOff = 256;                     // u32 hour
constexpr size_t kNoAllocErrOff = 260;                      // int error flags
constexpr size_t kNoAllocTgtOff = 512;                      // u32 per agent
static_assert(sizeof(DevParams) <= kNoAllocHourOff, "parameter block must fit its slot");

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

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
    DevParams d;
    std::memset(&d, 0, sizeof d);
    d.n = p.number_of_agents;
    d.G = (int32_t)p.grid_size;
    d.W = d.G + 1;
    d.WP = d.G + 3;
    d.area[kTransport] = to_rect(g.transport);
    d.area[kHousing] = to_rect(g.housing);
    d.area[kHosp0] = to_rect(g.hospital);
    d.area[kHosp1] = to_rect(grown_hospital(g));
    d.hosp_code = (hospital_grown && !rect_eq(d.area[kHosp1], d.area[kHosp0])) ? kHosp1 : kHosp0;
    d.key0 = (uint32_t)p.seed;
    d.key1 = (uint32_t)(p.seed >> 32);
    d.reg_start = p.regular_transmission_start_day;
    d.high_start = p.high_transmission_start_day;
    d.last_day = p.last_day;
    d.exposed_duration = p.exposed_duration;
    d.pre_duration = p.pre_symptomatic_duration;
    const double rates[3] = {0.0, p.regular_transmission_rate, p.high_transmission_rate};
    for (int c = 0; c < 3; ++c) {
        d.thr_rate[c] = bernoulli_threshold(rates[c]);
        if (rates[c] >= p.high_transmission_rate) d.hosp_if_class |= 1u << c;
    }
    d.thr_death = bernoulli_threshold(p.death_rate);
    d.thr_symptoms = bernoulli_threshold(1.0 - p.percentage_asymptomatic_population);
    d.thr_severe = bernoulli_threshold(p.percentage_severe_infected_population);
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
        NOALLOC_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_decide, kThreads, 0));
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
    uint32_t* d_hour = reinterpret_cast<uint32_t*>(d->base + kNoAllocHourOff);
    int* d_err = reinterpret_cast<int*>(d->base + kNoAllocErrOff);
    uint32_t* d_tgt = reinterpret_cast<uint32_t*>(d->base + kNoAllocTgtOff);
    uint32_t* d_claim = reinterpret_cast<uint32_t*>(d->base + claim_off);
    // every call starts from clean scratch: the claim plane free, the error word zero
    NOALLOC_CK(cudaMemcpyAsync(d_params, &hp, sizeof hp, cudaMemcpyHostToDevice, s));
    NOALLOC_CK(cudaMemcpyAsync(d_hour, &hour, sizeof hour, cudaMemcpyHostToDevice, s));
    NOALLOC_CK(cudaMemsetAsync(d_err, 0, sizeof(int), s));
    NOALLOC_CK(cudaMemsetAsync(counts, 0, 8 * sizeof(uint32_t), s));
    uint2* st = reinterpret_cast<uint2*>(state);
    const int blocks = (int)std::min<uint64_t>(((uint64_t)n + kThreads - 1) / kThreads, (uint64_t)d->grid_blocks);
    const uint32_t hod = hour % 24u;
    if (hod >= 1u && hod <= 6u) {
        k_sleep<<<blocks, kThreads, 0, s>>>(d_params, st, counts);
    } else {
        NOALLOC_CK(cudaMemsetAsync(d_claim, 0xFF, claim_bytes, s));
        k_decide<<<blocks, kThreads, 0, s>>>(d_params, pos, st, home, work, work_start_at, plane, d_claim, d_tgt, counts,
                                             d_hour, 0u, d_err);
        k_commit<<<(int)(((uint64_t)n + kThreads - 1) / kThreads), kThreads, 0, s>>>(d_params, pos, d_tgt, plane, d_claim);
    }
    NOALLOC_CK(cudaGetLastError());
    int err = 0;
    NOALLOC_CK(cudaMemcpyAsync(&err, d_err, sizeof err, cudaMemcpyDeviceToHost, s));
    NOALLOC_CK(cudaStreamSynchronize(s));
    if (err) return noalloc_fail(EPI_ERR_INVARIANT, "epi_tick_hour_noalloc: a rule addressed a cell outside the plane");
    return EPI_OK;
}
