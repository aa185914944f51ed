// Batched execution of many light queries: one persistent launch per plan
// step over a packed multi-query history, replayed as a CUDA graph.
//
// The batch holds up to max_queries queries of up to max_steps patterns each,
// every query starting from a constant (Engine::const_to_unknown,
// core/engine.hpp:96-122) and continuing with known_to_unknown /
// known_to_known / known_to_const steps (core/engine.hpp:126-225).  A query
// with fewer patterns passes its table through the remaining steps.
//
// Packed layout (device, per step, ping-pong A/B):
//   row_off[q]  first row of query q in the step's global row order (Q+1)
//   int_off[q]  first int32 of query q's table in the packed buffer
//   cols[q]     column count of query q's table
// Step kernels:
//   batch_count : per (query,row): probe with the query's own predicate
//                 (lanes of one warp may probe different segments), output
//                 row count (degree, or 0/1 for a filter, 1 for a pass),
//                 per-tile sums and per-query sums (warp-aggregated atomics)
//   batch_scan  : one block: exclusive scan of tile sums and of per-query
//                 output rows / ints -> next step's layout; capacity check
//   batch_write : per tile: block scan of the counts, then every output row
//                 written at out_int_off[q] + pos_in_q * width; rows whose
//                 output exceeds `split` ints are written warp-cooperatively,
//                 the rest thread-per-row
// The three phases run either as three kernels per step or as one
// cooperative persistent kernel per step (batch_step_kernel) whose blocks
// meet at two grid barriers -- after the count and after the scan, which
// block 0 runs -- each wait bounded; the autotuner picks the faster.  Every
// size lives in device memory and every grid is persistent, so the launch
// sequence of a batch never depends on its data: it is captured once into a
// CUDA graph and replayed for each new batch.  Each query's rows come out in
// exactly the order the query produces alone.
#include <algorithm>
#include <cstring>
#include <unordered_map>
#include <vector>

#include "wk_probe.cuh"
#include "wk_runtime.h"

namespace wk {
namespace dev {

#define FULL 0xffffffffu

enum { BK_K2U = 0, BK_K2K = 1, BK_K2C = 2, BK_C2U = 3, BK_NOP = 4 };

struct StepDesc {
    int32_t kind, pid, dir, scol, ecol, cst;   // cst: constant start (c2u) or constant end (k2c)
};

struct BatchTune {
    int blocks_per_sm;   // persistent grid = SMs x blocks_per_sm
    int rounds;          // rows per warp per tile = 32 * rounds
    int split;           // output ints above which a row is written by a whole warp
    int fused;           // 1: one cooperative kernel per step; 0: count, scan and write kernels
    int bt;              // threads per block of the step kernels: 128 or 256
};

constexpr int kErrBarrier = 1 << 4;         // flags[0]: a grid-barrier wait ran out
constexpr long kBarrierIters = 1l << 24;    // polls of a grid-barrier wait (about 1 s with the back-off)

constexpr int kBTMin = 128;                 // the smaller of the two block sizes (128, 256 threads)
constexpr int kMaxQ = 4096;                 // queries per batch (shared-memory row offsets)

__device__ __forceinline__ int find_query(const int64_t *s_off, int Q, int64_t g) {
    int lo = 0, hi = Q - 1;   // largest q with s_off[q] <= g
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (s_off[mid] <= g) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ bool b_contains(const int32_t *e, uint32_t n, int32_t v) {
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(e + mid) < v) lo = mid + 1;
        else hi = mid;
    }
    return lo < n && __ldg(e + lo) == v;
}

struct StepIO {
    const int32_t *hist;
    int32_t *out;
    const int64_t *in_row_off, *in_int_off;
    const int32_t *in_cols;
    int64_t *out_row_off, *out_int_off;
    int32_t *out_cols;
    const StepDesc *desc;     // [Q]
    const PredView *pvs;      // [num_ids + 1]
    uint32_t *cnt, *off;      // per input row
    unsigned long long *tile_sum;   // per tile
    unsigned long long *q_rows;     // per query output rows (zeroed by the scan)
    int *flags;               // [0] error bits, [1] overflow
    int64_t cap_ints, cap_rows;
    int Q;
};

// count: per (query, row) output counts, per-tile and per-query sums (BT
// threads a block, a tile of BT x rounds rows)
template <int BT>
__device__ __forceinline__ void count_phase(const StepIO &io, int rounds, const int64_t *s_off) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int tile_rows = (BT / 32) * 32 * rounds;
    const int64_t total = s_off[io.Q];
    const int64_t ntiles = (total + tile_rows - 1) / tile_rows;
    __shared__ unsigned long long s_sum[BT / 32];
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        unsigned long long my = 0ull;
        for (int rd = 0; rd < rounds; ++rd) {
            const int64_t g = tile * tile_rows + (int64_t)warp * 32 * rounds + rd * 32 + lane;
            const bool valid = g < total;
            int q = 0;
            StepDesc d{BK_NOP, 0, 0, 0, 0, 0};
            if (valid) { q = find_query(s_off, io.Q, g); d = io.desc[q]; }
            PredView pv{};
            int32_t vid = -1;
            bool probe = valid && d.kind != BK_NOP;
            int32_t target = 0;
            if (probe) {
                pv = io.pvs[d.pid];
                if (d.kind == BK_C2U) {
                    vid = d.cst;
                } else {
                    const int64_t r = g - s_off[q];
                    const int32_t *row = io.hist + io.in_int_off[q] + r * io.in_cols[q];
                    vid = __ldg(row + d.scol);
                    target = d.kind == BK_K2K ? __ldg(row + d.ecol) : d.cst;
                }
            }
            uint32_t o = 0u, deg = 0u;
            if (__any_sync(FULL, probe))
                probe_warp_multi(pv, (uint32_t)d.pid, probe, vid, (uint32_t)d.dir, o, deg, io.flags);
            uint32_t c = 0u;
            if (valid) {
                if (d.kind == BK_NOP) c = 1u;
                else if (d.kind == BK_K2U || d.kind == BK_C2U) c = deg;
                else c = (deg > 0u && b_contains(pv.edges + o, deg, target)) ? 1u : 0u;
                io.cnt[g] = c;
                io.off[g] = o;
            }
            // per-query sums, one atomic per distinct query in the warp
            const unsigned grp = __match_any_sync(FULL, valid ? q : -1);
            unsigned long long qs = c;
            // sum within the group: lanes of a group are contiguous (rows of one query)
            for (int sh = 16; sh > 0; sh >>= 1) {
                const unsigned long long v = __shfl_down_sync(FULL, qs, sh);
                if (lane + sh < 32 && ((grp >> (lane + sh)) & 1u)) qs += v;
            }
            // after the down-sweep the lowest lane of each contiguous group holds its total
            if (valid && (__ffs(grp) - 1) == lane && qs) atomicAdd(&io.q_rows[q], qs);
            my += c;
        }
        for (int o2 = 16; o2 > 0; o2 >>= 1) my += __shfl_xor_sync(FULL, my, o2);
        if (lane == 0) s_sum[warp] = my;
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned long long t = 0ull;
            for (int w = 0; w < BT / 32; ++w) t += s_sum[w];
            io.tile_sum[tile] = t;
        }
        __syncthreads();
    }
}

template <int BT>
__global__ void __launch_bounds__(BT)
batch_count_kernel(StepIO io, int rounds) {
    extern __shared__ int64_t s_off[];   // Q + 1
    if (io.flags[1]) return;
    for (int i = threadIdx.x; i <= io.Q; i += blockDim.x) s_off[i] = io.in_row_off[i];
    __syncthreads();
    count_phase<BT>(io, rounds, s_off);
}

// One block (any multiple of 32 threads up to 1024): tile prefix sums,
// per-query output layout, capacity check.  BT: the count's block size.
template <int BT>
__device__ __forceinline__ void scan_phase(const StepIO &io, int rounds) {
    __shared__ unsigned long long ws[32], wi[32];
    const int nt = blockDim.x, nw = nt >> 5;
    const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
    const int tile_rows = (BT / 32) * 32 * rounds;
    const int64_t total = io.in_row_off[io.Q];
    const int64_t n = (total + tile_rows - 1) / tile_rows;
    // (1) exclusive scan of the tile sums, in place
    {
        const int64_t per = (n + nt - 1) / nt, a = (int64_t)t * per, b = a + per < n ? a + per : n;
        unsigned long long ls = 0ull;
        for (int64_t i = a; i < b; ++i) ls += io.tile_sum[i];
        unsigned long long is = ls;
        for (int o = 1; o < 32; o <<= 1) { const unsigned long long v = __shfl_up_sync(FULL, is, o); if (lane >= o) is += v; }
        if (lane == 31) ws[wid] = is;
        __syncthreads();
        if (wid == 0) {
            unsigned long long x = lane < nw ? ws[lane] : 0ull;
            for (int o = 1; o < 32; o <<= 1) { const unsigned long long v = __shfl_up_sync(FULL, x, o); if (lane >= o) x += v; }
            ws[lane] = x;
        }
        __syncthreads();
        unsigned long long es = is - ls + (wid ? ws[wid - 1] : 0ull);
        for (int64_t i = a; i < b; ++i) { const unsigned long long v = io.tile_sum[i]; io.tile_sum[i] = es; es += v; }
        __syncthreads();
    }
    // (2) per-query output rows and ints (Q <= 4096: four per thread of 1024)
    {
        const int Q = io.Q, per = (Q + nt - 1) / nt, a = t * per, b = a + per < Q ? a + per : Q;
        unsigned long long lr = 0ull, li = 0ull;
        for (int q = a; q < b; ++q) {
            const StepDesc d = io.desc[q];
            const int w = (d.kind == BK_K2U) ? io.in_cols[q] + 1 : (d.kind == BK_C2U ? 1 : io.in_cols[q]);
            lr += io.q_rows[q];
            li += io.q_rows[q] * (unsigned long long)w;
        }
        unsigned long long ir = lr, ii = li;
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long v = __shfl_up_sync(FULL, ir, o), x = __shfl_up_sync(FULL, ii, o);
            if (lane >= o) { ir += v; ii += x; }
        }
        if (lane == 31) { ws[wid] = ir; wi[wid] = ii; }
        __syncthreads();
        if (wid == 0) {
            unsigned long long x = lane < nw ? ws[lane] : 0ull, y = lane < nw ? wi[lane] : 0ull;
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned long long v = __shfl_up_sync(FULL, x, o), u = __shfl_up_sync(FULL, y, o);
                if (lane >= o) { x += v; y += u; }
            }
            ws[lane] = x;
            wi[lane] = y;
        }
        __syncthreads();
        unsigned long long er = ir - lr + (wid ? ws[wid - 1] : 0ull);
        unsigned long long ei = ii - li + (wid ? wi[wid - 1] : 0ull);
        for (int q = a; q < b; ++q) {
            const StepDesc d = io.desc[q];
            const int w = (d.kind == BK_K2U) ? io.in_cols[q] + 1 : (d.kind == BK_C2U ? 1 : io.in_cols[q]);
            const unsigned long long r = io.q_rows[q];
            io.out_row_off[q] = (int64_t)er;
            io.out_int_off[q] = (int64_t)ei;
            io.out_cols[q] = w;
            io.q_rows[q] = 0ull;   // the next step's count kernel accumulates afresh
            er += r;
            ei += r * (unsigned long long)w;
        }
        if (t == nt - 1) {
            io.out_row_off[Q] = (int64_t)er;
            if ((int64_t)er > io.cap_rows || (int64_t)ei > io.cap_ints) io.flags[1] = 1;
        }
    }
}

template <int BT>
__global__ void __launch_bounds__(1024)
batch_scan_kernel(StepIO io, int rounds) {
    if (io.flags[1]) return;
    scan_phase<BT>(io, rounds);
}

// Per tile: block scan of the counts, then write.  Rows with more than
// `split` output ints are queued and written by whole warps.
template <int BT>
__device__ __forceinline__ void write_phase(const StepIO &io, int rounds, int split, const int64_t *s_off) {
    __shared__ unsigned long long s_w[BT / 32];
    __shared__ int s_nq;
    __shared__ int s_big[BT * 8];        // queued rows (local index), rounds <= 8
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int tile_rows = BT * rounds;
    const int64_t total = s_off[io.Q];
    const int64_t ntiles = (total + tile_rows - 1) / tile_rows;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        if (threadIdx.x == 0) s_nq = 0;
        // thread t owns rows tile*tile_rows + t*rounds .. + rounds-1
        const int64_t g0 = tile * tile_rows + (int64_t)threadIdx.x * rounds;
        unsigned long long my = 0ull;
        for (int k = 0; k < rounds; ++k) my += (g0 + k < total) ? io.cnt[g0 + k] : 0u;
        unsigned long long inc = my;
        for (int o = 1; o < 32; o <<= 1) { const unsigned long long v = __shfl_up_sync(FULL, inc, o); if (lane >= o) inc += v; }
        if (lane == 31) s_w[warp] = inc;
        __syncthreads();
        unsigned long long pos = io.tile_sum[tile] + inc - my;
        for (int w = 0; w < warp; ++w) pos += s_w[w];
        for (int k = 0; k < rounds; ++k) {
            const int64_t g = g0 + k;
            if (g >= total) break;
            const uint32_t c = io.cnt[g];
            if (c == 0u) continue;
            const int q = find_query(s_off, io.Q, g);
            const StepDesc d = io.desc[q];
            const int cin = io.in_cols[q];
            const int w = (d.kind == BK_K2U) ? cin + 1 : (d.kind == BK_C2U ? 1 : cin);
            if ((int64_t)c * w > split) {
                const int slot = atomicAdd(&s_nq, 1);
                s_big[slot] = (int)(g - tile * tile_rows);
                // its output position is recomputed by the warp below
            } else {
                const int32_t *row = io.hist + io.in_int_off[q] + (g - s_off[q]) * cin;
                int32_t *dst = io.out + io.out_int_off[q] + ((int64_t)pos - io.out_row_off[q]) * w;
                if (d.kind == BK_K2U || d.kind == BK_C2U) {
                    const int32_t *e = io.pvs[d.pid].edges + io.off[g];
                    for (uint32_t x = 0; x < c; ++x) {
                        if (d.kind == BK_K2U) for (int cc = 0; cc < cin; ++cc) dst[cc] = __ldg(row + cc);
                        dst[w - 1] = __ldg(e + x);
                        dst += w;
                    }
                } else {
                    for (int cc = 0; cc < cin; ++cc) dst[cc] = __ldg(row + cc);
                }
            }
            pos += c;
        }
        __syncthreads();
        // queued rows: one warp per row, lanes stride over the row's output ints
        const int nq = s_nq;
        for (int i = warp; i < nq; i += BT / 32) {
            const int lr = s_big[i];
            const int64_t g = tile * tile_rows + lr;
            // output position of row g: tile base + counts of the rows before it in the tile
            unsigned long long before = 0ull;
            for (int j = lane; j < lr; j += 32) before += io.cnt[tile * tile_rows + j];
            for (int o = 16; o > 0; o >>= 1) before += __shfl_xor_sync(FULL, before, o);
            const unsigned long long p = io.tile_sum[tile] + before;
            const int q = find_query(s_off, io.Q, g);
            const StepDesc d = io.desc[q];
            const int cin = io.in_cols[q];
            const int w = (d.kind == BK_K2U) ? cin + 1 : (d.kind == BK_C2U ? 1 : cin);
            const uint32_t c = io.cnt[g];
            const int32_t *row = io.hist + io.in_int_off[q] + (g - s_off[q]) * cin;
            int32_t *dst = io.out + io.out_int_off[q] + ((int64_t)p - io.out_row_off[q]) * w;
            const int32_t *e = (d.kind == BK_K2U || d.kind == BK_C2U) ? io.pvs[d.pid].edges + io.off[g] : nullptr;
            const int64_t nw = (int64_t)c * w;
            for (int64_t x = lane; x < nw; x += 32) {
                const int64_t r = x / w;
                const int cc = (int)(x - r * w);
                int32_t v;
                if (d.kind == BK_K2U) v = (cc < cin) ? __ldg(row + cc) : __ldg(e + r);
                else if (d.kind == BK_C2U) v = __ldg(e + r);
                else v = __ldg(row + cc);
                dst[x] = v;
            }
        }
        __syncthreads();
    }
}

template <int BT>
__global__ void __launch_bounds__(BT)
batch_write_kernel(StepIO io, int rounds, int split) {
    extern __shared__ int64_t s_off[];   // Q+1 input row offsets
    if (io.flags[1]) return;
    for (int i = threadIdx.x; i <= io.Q; i += blockDim.x) s_off[i] = io.in_row_off[i];
    __syncthreads();
    write_phase<BT>(io, rounds, split, s_off);
}

__device__ __forceinline__ unsigned int ld_acquire(const unsigned int *p) {
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release(unsigned int *p, unsigned int v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Grid barrier of a cooperative launch: bar[0] counts arrivals, bar[1] is the
// generation.  The block arriving last resets the count and advances the
// generation; the others poll the generation with a back-off,
// at most kBarrierIters times -- a wait that runs out sets kErrBarrier and
// returns false in every thread of the block (the caller then leaves; every
// other block's wait ends the same way, so the launch ends).
__device__ __forceinline__ bool grid_barrier(unsigned int *bar, int *flags) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned int gen = ld_acquire(bar + 1);
        __threadfence();   // this block's writes before its arrival
        int ok = 1;
        if (atomicAdd(bar, 1u) + 1u == gridDim.x) {
            atomicExch(bar, 0u);
            __threadfence();
            st_release(bar + 1, gen + 1u);
        } else {
            long it = 0;
            while (ld_acquire(bar + 1) == gen) {
                if (++it > kBarrierIters) {
                    ok = 0;
                    atomicOr(flags, kErrBarrier);
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// One step in one cooperative launch: count, barrier, scan (block 0),
// barrier, write.  Launched with at most as many blocks as fit on the device
// at once (the cooperative launch refuses more).
template <int BT>
__global__ void __launch_bounds__(BT)
batch_step_kernel(StepIO io, int rounds, int split, unsigned int *bar) {
    extern __shared__ int64_t s_off[];   // Q + 1 input row offsets
    if (io.flags[1]) return;             // set before the launch: the same in every block
    for (int i = threadIdx.x; i <= io.Q; i += blockDim.x) s_off[i] = io.in_row_off[i];
    __syncthreads();
    count_phase<BT>(io, rounds, s_off);
    if (!grid_barrier(bar, io.flags)) return;
    if (blockIdx.x == 0) scan_phase<BT>(io, rounds);
    if (!grid_barrier(bar, io.flags)) return;
    if (*(volatile int *)(io.flags + 1)) return;   // this step's scan found the batch over capacity
    write_phase<BT>(io, rounds, split, s_off);
}

// step-0 layout: every query has one virtual row and no columns
__global__ void batch_init_kernel(int Q, int64_t *row_off, int64_t *int_off, int32_t *cols,
                                  unsigned long long *q_rows, int *flags) {
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q <= Q; q += gridDim.x * blockDim.x) {
        row_off[q] = q;
        if (q < Q) { int_off[q] = 0; cols[q] = 0; q_rows[q] = 0ull; }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) { flags[0] = 0; flags[1] = 0; }
}

}  // namespace dev
}  // namespace wk

using namespace wk;
using namespace wk::dev;

struct wk_batch {
    wk_ctx *ctx = nullptr;
    cudaStream_t stream = nullptr;          // the batch's own stream (batches overlap)
    cudaEvent_t done = nullptr;
    int32_t max_q = 0, max_steps = 0;
    int64_t cap_ints = 0, cap_rows = 0;
    int sms = 0;
    BatchTune tune{4, 4, 64, 0, 256};
    // device
    PredView *d_pvs = nullptr;
    StepDesc *d_desc = nullptr;             // [max_steps][max_q]
    int64_t *d_row_off[2] = {}, *d_int_off[2] = {};
    int32_t *d_cols[2] = {};
    int32_t *d_hist[2] = {};
    uint32_t *d_cnt = nullptr, *d_off = nullptr;
    unsigned long long *d_tile = nullptr, *d_qrows = nullptr;
    int *d_flags = nullptr;
    unsigned int *d_bar = nullptr;          // grid barrier of the one-kernel steps (count, generation)
    // host (pinned)
    StepDesc *h_desc = nullptr;
    int64_t *h_layout = nullptr;            // row_off (Q+1), int_off (Q), cols as int64 (Q)
    int *h_flags = nullptr;
    // graph
    // executable graphs by batch size (a serving loop's batch sizes vary from
    // batch to batch; each size is captured once), all for graph_tune
    std::unordered_map<int, cudaGraphExec_t> graphs;
    BatchTune graph_tune{0, 0, 0, 0, 0};
    cudaGraphExec_t gexec = nullptr;   // the last one launched
    int32_t last_q = 0;
    int final_buf = 0;
    double form_best_ms[2] = {-1.0, -1.0};   // the last autotune's best per step form (-1: none ran)
    int64_t kernels = 0;
};

namespace {

// A batch's stream has the device's highest priority: batches are short runs
// of small persistent kernels, and when they share the GPU with a large query
// (a serving loop's heavy requests) the block scheduler then places their
// blocks ahead of the large kernels' remaining blocks.
cudaError_t create_priority_stream(cudaStream_t *st) {
    int least = 0, greatest = 0;
    cudaError_t e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
    if (e != cudaSuccess) return e;
    return cudaStreamCreateWithPriority(st, cudaStreamNonBlocking, greatest);
}

// tiles of the smallest shape (kBTMin threads x rounds rows): the tile-sum
// buffer holds any tuning's
int64_t max_tiles(const wk_batch *b, int rounds) {
    const int64_t tr = (int64_t)kBTMin * rounds;
    return (b->cap_rows + tr - 1) / tr + 1;
}

void free_batch(wk_batch *b) {
    cudaSetDevice(b->ctx->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    for (auto &kv : b->graphs) cudaGraphExecDestroy(kv.second);
    b->graphs.clear();
    if (b->done) cudaEventDestroy(b->done);
    if (b->stream) cudaStreamDestroy(b->stream);
    cudaFree(b->d_pvs); cudaFree(b->d_desc);
    for (int i = 0; i < 2; ++i) { cudaFree(b->d_row_off[i]); cudaFree(b->d_int_off[i]); cudaFree(b->d_cols[i]); cudaFree(b->d_hist[i]); }
    cudaFree(b->d_cnt); cudaFree(b->d_off); cudaFree(b->d_tile); cudaFree(b->d_qrows); cudaFree(b->d_flags);
    cudaFree(b->d_bar);
    if (b->h_desc) cudaFreeHost(b->h_desc);
    if (b->h_layout) cudaFreeHost(b->h_layout);
    if (b->h_flags) cudaFreeHost(b->h_flags);
    delete b;
}

StepIO make_io(wk_batch *b, int s, int Q) {
    StepIO io;
    const int in = s & 1, out = in ^ 1;
    io.hist = b->d_hist[in];
    io.out = b->d_hist[out];
    io.in_row_off = b->d_row_off[in];
    io.in_int_off = b->d_int_off[in];
    io.in_cols = b->d_cols[in];
    io.out_row_off = b->d_row_off[out];
    io.out_int_off = b->d_int_off[out];
    io.out_cols = b->d_cols[out];
    io.desc = b->d_desc + (size_t)s * b->max_q;
    io.pvs = b->d_pvs;
    io.cnt = b->d_cnt;
    io.off = b->d_off;
    io.tile_sum = b->d_tile;
    io.q_rows = b->d_qrows;
    io.flags = b->d_flags;
    io.cap_ints = b->cap_ints;
    io.cap_rows = b->cap_rows;
    io.Q = Q;
    return io;
}

// the max_steps steps of a batch with BT-thread blocks: three kernels per
// step, or one cooperative kernel
template <int BT>
int enqueue_steps(wk_batch *b, int Q, const BatchTune &t, unsigned grid, size_t sm_off, cudaStream_t st) {
    if (t.fused) {
        // every block of a cooperative launch must be resident at once
        int occ = 0;
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, batch_step_kernel<BT>, BT, sm_off);
        if (e != cudaSuccess) return cuda_fail(e, "batch step occupancy");
        if (occ < 1) return set_error(WK_EDEVICE, "batch step kernel: no block fits on an SM");
        const unsigned gf = (unsigned)std::min<int64_t>(grid, (int64_t)occ * b->sms);
        // the barrier words start at zero in every batch (a wait that ran out leaves them unbalanced)
        if ((e = cudaMemsetAsync(b->d_bar, 0, 2 * sizeof(unsigned int), st)) != cudaSuccess)
            return cuda_fail(e, "batch barrier reset");
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeCooperative;
        attr[0].val.cooperative = 1;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(gf);
        cfg.blockDim = dim3(BT);
        cfg.dynamicSmemBytes = sm_off;
        cfg.stream = st;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        for (int s = 0; s < b->max_steps; ++s) {
            StepIO io = make_io(b, s, Q);
            if ((e = cudaLaunchKernelEx(&cfg, batch_step_kernel<BT>, io, t.rounds, t.split, b->d_bar)) != cudaSuccess)
                return cuda_fail(e, "batch step launch");
        }
    } else {
        for (int s = 0; s < b->max_steps; ++s) {
            StepIO io = make_io(b, s, Q);
            batch_count_kernel<BT><<<grid, BT, sm_off, st>>>(io, t.rounds);
            batch_scan_kernel<BT><<<1, 1024, 0, st>>>(io, t.rounds);
            batch_write_kernel<BT><<<grid, BT, sm_off, st>>>(io, t.rounds, t.split);
        }
    }
    return WK_OK;
}

// kernels of one batch: the layout init, then per step three kernels or one
int64_t batch_kernels(const wk_batch *b, const BatchTune &t) {
    return 1 + (t.fused ? 1 : 3) * (int64_t)b->max_steps;
}

// the whole batch: descriptor upload, layout init, max_steps x (count, scan,
// write) as three kernels or as one cooperative kernel
int enqueue(wk_batch *b, int Q, const BatchTune &t, cudaStream_t st) {
    // the Q descriptors of each step (step s's start at s * max_q)
    for (int s = 0; s < b->max_steps; ++s) {
        const size_t at = (size_t)s * b->max_q;
        cudaError_t e = cudaMemcpyAsync(b->d_desc + at, b->h_desc + at, sizeof(StepDesc) * (size_t)Q,
                                        cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) return cuda_fail(e, "batch descriptors");
    }
    batch_init_kernel<<<(Q + 256) / 256, 256, 0, st>>>(Q, b->d_row_off[0], b->d_int_off[0], b->d_cols[0], b->d_qrows,
                                                       b->d_flags);
    // The step kernels loop over tiles, so any grid gives the same rows.  A
    // small batch gets a grid in proportion to its queries (at least a
    // quarter of the SMs): beside a large query on another stream, a few
    // light queries then hold a few SMs, not all of them.
    const int64_t full = (int64_t)b->sms * t.blocks_per_sm;
    const unsigned grid = (unsigned)std::min<int64_t>(full, std::max<int64_t>(b->sms / 4, 2 * (int64_t)Q));
    const size_t sm_off = sizeof(int64_t) * (size_t)(Q + 1);
    const int st2 = t.bt == 128 ? enqueue_steps<128>(b, Q, t, grid, sm_off, st) : enqueue_steps<256>(b, Q, t, grid, sm_off, st);
    if (st2) return st2;
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "batch launch");
    b->kernels += batch_kernels(b, t);
    return WK_OK;
}

}  // namespace

extern "C" int wk_batch_create(wk_ctx *ctx, int32_t max_queries, int32_t max_steps, int64_t capacity_ints,
                               wk_batch **out) {
    if (!ctx || !out || max_queries < 1 || max_queries > kMaxQ || max_steps < 1 || max_steps > 16 ||
        capacity_ints < 1)
        return set_error(WK_EINVAL, "wk_batch_create: bad arguments (1..%d queries, 1..16 steps)", kMaxQ);
    if (!ctx->store) return set_error(WK_ENOSTORE, "wk_batch_create: no store built");
    if (ctx->device < 0) return set_error(WK_EDEVICE, "wk_batch_create: host-only context");
    if (ctx->store->pool) return set_error(WK_EINVAL, "wk_batch_create: batches need a resident store");
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    wk_batch *b = new wk_batch();
    b->ctx = ctx;
    b->max_q = max_queries;
    b->max_steps = max_steps;
    b->cap_ints = capacity_ints;
    b->cap_rows = capacity_ints;   // every row holds at least one int
    cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, ctx->device);
    const size_t npv = ctx->store->views.size();
    const int64_t tiles = max_tiles(b, 1);
    bool ok = cudaMalloc(&b->d_pvs, sizeof(PredView) * npv) == cudaSuccess &&
              cudaMalloc(&b->d_desc, sizeof(StepDesc) * (size_t)max_queries * max_steps) == cudaSuccess &&
              cudaMalloc(&b->d_cnt, 4 * (size_t)b->cap_rows) == cudaSuccess &&
              cudaMalloc(&b->d_off, 4 * (size_t)b->cap_rows) == cudaSuccess &&
              cudaMalloc(&b->d_tile, 8 * (size_t)tiles) == cudaSuccess &&
              cudaMalloc(&b->d_qrows, 8 * (size_t)max_queries) == cudaSuccess &&
              cudaMalloc(&b->d_flags, 64) == cudaSuccess &&
              cudaMalloc(&b->d_bar, 2 * sizeof(unsigned int)) == cudaSuccess &&
              cudaHostAlloc((void **)&b->h_desc, sizeof(StepDesc) * (size_t)max_queries * max_steps, 0) == cudaSuccess &&
              cudaHostAlloc((void **)&b->h_layout, 8 * (size_t)(3 * max_queries + 1), 0) == cudaSuccess &&
              cudaHostAlloc((void **)&b->h_flags, 64, 0) == cudaSuccess &&
              create_priority_stream(&b->stream) == cudaSuccess &&
              cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming) == cudaSuccess;
    for (int i = 0; ok && i < 2; ++i)
        ok = cudaMalloc(&b->d_row_off[i], 8 * (size_t)(max_queries + 1)) == cudaSuccess &&
             cudaMalloc(&b->d_int_off[i], 8 * (size_t)max_queries) == cudaSuccess &&
             cudaMalloc(&b->d_cols[i], 4 * (size_t)max_queries) == cudaSuccess &&
             cudaMalloc(&b->d_hist[i], 4 * (size_t)capacity_ints) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        free_batch(b);
        return set_error(WK_ENOMEM, "wk_batch_create: allocation failed (capacity %lld ints)", (long long)capacity_ints);
    }
    e = cudaMemcpy(b->d_pvs, ctx->store->views.data(), sizeof(PredView) * npv, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(b->d_flags, 0, 64);
    if (e == cudaSuccess) e = cudaMemset(b->d_bar, 0, 2 * sizeof(unsigned int));
    if (e != cudaSuccess) { int r = cuda_fail(e, "wk_batch_create"); free_batch(b); return r; }
    *out = b;
    return WK_OK;
}

extern "C" int wk_batch_destroy(wk_batch *b) {
    if (b) free_batch(b);
    return WK_OK;
}

extern "C" int wk_batch_set_tuning(wk_batch *b, int32_t blocks_per_sm, int32_t rows_per_warp, int32_t split_ints) {
    if (!b || blocks_per_sm < 1 || blocks_per_sm > 16 || rows_per_warp < 32 || rows_per_warp > 256 ||
        rows_per_warp % 32 || split_ints < 1)
        return set_error(WK_EINVAL, "wk_batch_set_tuning: blocks/SM 1..16, rows/warp 32..256 (x32), split >= 1");
    b->tune = BatchTune{blocks_per_sm, rows_per_warp / 32, split_ints, b->tune.fused, b->tune.bt};
    return WK_OK;
}

extern "C" int wk_batch_set_fused(wk_batch *b, int32_t fused) {
    if (!b || (fused != 0 && fused != 1)) return set_error(WK_EINVAL, "wk_batch_set_fused: 0 or 1");
    b->tune.fused = fused;
    return WK_OK;
}

extern "C" int wk_batch_get_fused(wk_batch *b) { return b ? b->tune.fused : 0; }

extern "C" int wk_batch_set_block_threads(wk_batch *b, int32_t threads) {
    if (!b || (threads != 128 && threads != 256)) return set_error(WK_EINVAL, "wk_batch_set_block_threads: 128 or 256");
    b->tune.bt = threads;
    return WK_OK;
}

extern "C" int wk_batch_get_block_threads(wk_batch *b) { return b ? b->tune.bt : 0; }

extern "C" int wk_batch_get_tuning(wk_batch *b, int32_t *blocks_per_sm, int32_t *rows_per_warp, int32_t *split_ints) {
    if (!b || !blocks_per_sm || !rows_per_warp || !split_ints) return set_error(WK_EINVAL, "wk_batch_get_tuning: null");
    *blocks_per_sm = b->tune.blocks_per_sm;
    *rows_per_warp = b->tune.rounds * 32;
    *split_ints = b->tune.split;
    return WK_OK;
}

// Fill the step descriptors from the queries.  A query starts from a
// constant vertex or from an index: a type index [c, type, IN, -1] is the list
// of key [0|c|IN] and a predicate index [p, 0, d, -1] the list of key [0|p|d]
// (core/gstore.hpp:546-560), so both run as a constant start at vertex 0.
static int fill_desc(wk_batch *b, const int64_t *cmd, const int32_t *npat, int32_t Q) {
    int64_t at = 0;
    const int num_ids = b->ctx->store->hs->num_ids;
    for (int q = 0; q < Q; ++q) {
        const int n = npat[q];
        if (n < 1 || n > b->max_steps) return set_error(WK_EINVAL, "wk_batch_run: query %d has %d patterns (1..%d)", q, n, b->max_steps);
        int col = 0;
        for (int s = 0; s < b->max_steps; ++s) {
            StepDesc &d = b->h_desc[(size_t)s * b->max_q + q];
            if (s >= n) { d = StepDesc{BK_NOP, 1, 0, 0, 0, 0}; continue; }
            const int64_t st = cmd[at + 4 * s], pid = cmd[at + 4 * s + 1], dir = cmd[at + 4 * s + 2], en = cmd[at + 4 * s + 3];
            if (s == 0 && st > 1 && st < WK_VID_BASE) {   // index start
                const bool ok = en == -1 && st <= num_ids &&
                                ((pid == WK_TYPE_ID && dir == WK_DIR_IN) || (pid == WK_PREDICATE_ID && (dir == 0 || dir == 1)));
                if (!ok) return set_error(WK_EINVAL, "wk_batch_run: query %d: bad index start", q);
                d = StepDesc{BK_C2U, (int32_t)st, (int32_t)dir, 0, 0, 0};
                col = 1;
                continue;
            }
            if (pid < 1 || pid > num_ids || (dir != 0 && dir != 1))
                return set_error(WK_EINVAL, "wk_batch_run: query %d step %d: predicate %lld / direction %lld", q, s,
                                 (long long)pid, (long long)dir);
            const bool start_known = st < 0 && -st <= col, end_unknown = en < 0 && -en > col, end_known = en < 0 && -en <= col;
            if (s == 0) {
                if (st < WK_VID_BASE || st > 0x7fffffffll || en != -1)
                    return set_error(WK_EINVAL, "wk_batch_run: query %d must start from a constant vertex or an index, binding -1", q);
                d = StepDesc{BK_C2U, (int32_t)pid, (int32_t)dir, 0, 0, (int32_t)st};
                col = 1;
            } else if (start_known && end_unknown) {
                if (-en - 1 != col) return set_error(WK_EINVAL, "wk_batch_run: query %d step %d skips a column", q, s);
                d = StepDesc{BK_K2U, (int32_t)pid, (int32_t)dir, (int32_t)(-st - 1), 0, 0};
                ++col;
            } else if (start_known && end_known) {
                d = StepDesc{BK_K2K, (int32_t)pid, (int32_t)dir, (int32_t)(-st - 1), (int32_t)(-en - 1), 0};
            } else if (start_known && en >= 0 && en <= 0x7fffffffll) {
                d = StepDesc{BK_K2C, (int32_t)pid, (int32_t)dir, (int32_t)(-st - 1), 0, (int32_t)en};
            } else {
                return set_error(WK_EINVAL, "wk_batch_run: query %d step %d: unsupported pattern shape", q, s);
            }
        }
        at += 4 * n;
    }
    return WK_OK;
}

extern "C" int wk_batch_launch(wk_batch *b, const int64_t *cmd_chains, const int32_t *n_patterns, int32_t nq,
                               int32_t use_graph) {
    if (!b || !cmd_chains || !n_patterns || nq < 1 || nq > b->max_q)
        return set_error(WK_EINVAL, "wk_batch_launch: bad arguments (1..%d queries)", b ? b->max_q : 0);
    wk_ctx *ctx = b->ctx;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    // the pinned descriptors may still be read by a previous launch
    if ((e = cudaEventSynchronize(b->done)) != cudaSuccess) return cuda_fail(e, "batch previous launch");
    int st = fill_desc(b, cmd_chains, n_patterns, nq);
    if (st) return st;
    cudaStream_t s = b->stream;
    if (use_graph) {
        if (std::memcmp(&b->graph_tune, &b->tune, sizeof(BatchTune)) != 0 || b->graphs.size() >= 512) {
            for (auto &kv : b->graphs) cudaGraphExecDestroy(kv.second);
            b->graphs.clear();
            b->graph_tune = b->tune;
        }
        auto it = b->graphs.find(nq);
        if (it == b->graphs.end()) {
            cudaGraph_t g;
            if ((e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
                return cuda_fail(e, "batch capture");
            st = enqueue(b, nq, b->tune, s);
            e = cudaStreamEndCapture(s, &g);
            if (st) { if (e == cudaSuccess) cudaGraphDestroy(g); return st; }
            if (e != cudaSuccess) return cuda_fail(e, "batch capture end");
            cudaGraphExec_t ge = nullptr;
            e = cudaGraphInstantiate(&ge, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) return cuda_fail(e, "batch graph instantiate");
            it = b->graphs.emplace(nq, ge).first;
            b->kernels -= batch_kernels(b, b->tune);   // capture does not launch
        }
        b->gexec = it->second;
        if ((e = cudaGraphLaunch(b->gexec, s)) != cudaSuccess) return cuda_fail(e, "batch graph launch");
        b->kernels += batch_kernels(b, b->tune);
    } else {
        if ((st = enqueue(b, nq, b->tune, s))) return st;
    }
    ctx->launches += batch_kernels(b, b->tune);
    b->last_q = nq;
    b->final_buf = b->max_steps & 1;
    // layout of the final tables + flags, then the completion event
    const int fb = b->final_buf;
    if ((e = cudaMemcpyAsync(b->h_flags, b->d_flags, 8, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(b->h_layout, b->d_row_off[fb], 8 * (size_t)(nq + 1), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(b->h_layout + nq + 1, b->d_int_off[fb], 8 * (size_t)nq, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(reinterpret_cast<int32_t *>(b->h_layout + 2 * nq + 1), b->d_cols[fb], 4 * (size_t)nq,
                             cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaEventRecord(b->done, s)) != cudaSuccess)
        return cuda_fail(e, "batch layout readback");
    return WK_OK;
}

// 1 when the last launch has finished, 0 while it runs
extern "C" int wk_batch_ready(wk_batch *b) {
    if (!b) return 1;
    return cudaEventQuery(b->done) == cudaSuccess ? 1 : 0;
}

extern "C" int wk_batch_wait(wk_batch *b) {
    if (!b) return set_error(WK_EINVAL, "wk_batch_wait: null");
    cudaError_t e = cudaEventSynchronize(b->done);
    if (e != cudaSuccess) return cuda_fail(e, "batch wait");
    if (b->h_flags[1]) return set_error(WK_EOVERFLOW, "wk_batch: a step exceeded the batch capacity of %lld ints",
                                        (long long)b->cap_ints);
    if (b->h_flags[0] & kErrBarrier)
        return set_error(WK_ETIMEDOUT, "wk_batch: a grid-barrier wait of the one-kernel step ran out");
    if (b->h_flags[0]) return set_error(WK_EDEVICE, "wk_batch: corrupt overflow chain in the store");
    return WK_OK;
}

extern "C" int wk_batch_run(wk_batch *b, const int64_t *cmd_chains, const int32_t *n_patterns, int32_t nq,
                            int32_t use_graph) {
    int st = wk_batch_launch(b, cmd_chains, n_patterns, nq, use_graph);
    return st ? st : wk_batch_wait(b);
}

extern "C" int wk_batch_result(wk_batch *b, int32_t q, int64_t *rows, int32_t *cols, int64_t *int_offset) {
    if (!b || q < 0 || q >= b->last_q || !rows || !cols || !int_offset) return set_error(WK_EINVAL, "wk_batch_result");
    const int nq = b->last_q;
    const int32_t *c = reinterpret_cast<const int32_t *>(b->h_layout + 2 * nq + 1);
    *rows = b->h_layout[q + 1] - b->h_layout[q];
    *cols = c[q];
    *int_offset = b->h_layout[nq + 1 + q];
    return WK_OK;
}

extern "C" int wk_batch_layouts(wk_batch *b, int32_t nq, int64_t *rows, int32_t *cols, int64_t *int_offsets) {
    if (!b || nq != b->last_q || (nq > 0 && (!rows || !cols || !int_offsets)))
        return set_error(WK_EINVAL, "wk_batch_layouts: bad arguments (the last run had %d queries)", b ? b->last_q : 0);
    const int32_t *c = reinterpret_cast<const int32_t *>(b->h_layout + 2 * nq + 1);
    for (int q = 0; q < nq; ++q) {
        rows[q] = b->h_layout[q + 1] - b->h_layout[q];
        cols[q] = c[q];
        int_offsets[q] = b->h_layout[nq + 1 + q];
    }
    return WK_OK;
}

extern "C" int wk_batch_download(wk_batch *b, int32_t *host, int64_t cap, int64_t *total_ints) {
    if (!b || !total_ints) return set_error(WK_EINVAL, "wk_batch_download: null");
    const int nq = b->last_q;
    const int32_t *c = reinterpret_cast<const int32_t *>(b->h_layout + 2 * nq + 1);
    const int64_t tot = nq ? b->h_layout[nq + 1 + nq - 1] + (b->h_layout[nq] - b->h_layout[nq - 1]) * c[nq - 1] : 0;
    *total_ints = tot;
    if (!host) return WK_OK;
    if (cap < tot) return set_error(WK_EOVERFLOW, "wk_batch_download: %lld ints, room for %lld", (long long)tot, (long long)cap);
    cudaError_t e;
    if (tot && (e = cudaMemcpyAsync(host, b->d_hist[b->final_buf], 4 * (size_t)tot, cudaMemcpyDeviceToHost,
                                    b->stream)) != cudaSuccess)
        return cuda_fail(e, "wk_batch_download");
    if ((e = cudaStreamSynchronize(b->stream)) != cudaSuccess) return cuda_fail(e, "wk_batch_download sync");
    return WK_OK;
}

// Autotuner: time the batch with every candidate (three kernels or one per
// step, 128 or 256 threads a block, blocks/SM, rows/warp, split) on the given
// queries (CUDA events, best of `reps` after a warm run) and keep the fastest.  A one-kernel candidate
// the device refuses (its cooperative launch, or its capture into a graph) is
// skipped.  Writes the chosen candidate's time.
extern "C" int wk_batch_autotune(wk_batch *b, const int64_t *cmd_chains, const int32_t *n_patterns, int32_t nq,
                                 int32_t reps, double *best_ms) {
    if (!b || reps < 1) return set_error(WK_EINVAL, "wk_batch_autotune: bad arguments");
    static const int kBlocks[] = {2, 4, 8};
    static const int kRows[] = {32, 64, 128};
    static const int kSplit[] = {16, 64, 256};
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
        return set_error(WK_EDEVICE, "wk_batch_autotune: events");
    double best = 1e30;
    BatchTune keep = b->tune;
    b->form_best_ms[0] = b->form_best_ms[1] = -1.0;
    for (int fu = 0; fu < 2; ++fu)
    for (int bt : {256, 128})
    for (int bl : kBlocks)
        for (int rw : kRows)
            for (int sp : kSplit) {
                b->tune = BatchTune{bl, rw / 32, sp, fu, bt};
                int st = wk_batch_run(b, cmd_chains, n_patterns, nq, 1);   // builds the graph
                if (st && fu && st != WK_EOVERFLOW && st != WK_ETIMEDOUT) {
                    cudaGetLastError();
                    continue;
                }
                if (st) { cudaEventDestroy(e0); cudaEventDestroy(e1); b->tune = keep; return st; }
                double tbest = 1e30;
                for (int r = 0; r < reps; ++r) {
                    cudaEventRecord(e0, b->stream);
                    cudaGraphLaunch(b->gexec, b->stream);
                    cudaEventRecord(e1, b->stream);
                    cudaEventSynchronize(e1);
                    float ms = 0.f;
                    cudaEventElapsedTime(&ms, e0, e1);
                    tbest = std::min(tbest, (double)ms);
                }
                if (tbest < best) { best = tbest; keep = b->tune; }
                if (b->form_best_ms[fu] < 0.0 || tbest < b->form_best_ms[fu]) b->form_best_ms[fu] = tbest;
            }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->tune = keep;
    if (best_ms) *best_ms = best;
    return wk_batch_run(b, cmd_chains, n_patterns, nq, 1);
}

extern "C" int64_t wk_batch_kernel_launches(wk_batch *b) { return b ? b->kernels : 0; }

extern "C" int wk_batch_autotune_forms(wk_batch *b, double *three_kernel_ms, double *one_kernel_ms) {
    if (!b || !three_kernel_ms || !one_kernel_ms) return set_error(WK_EINVAL, "wk_batch_autotune_forms: null");
    *three_kernel_ms = b->form_best_ms[0];
    *one_kernel_ms = b->form_best_ms[1];
    return WK_OK;
}
