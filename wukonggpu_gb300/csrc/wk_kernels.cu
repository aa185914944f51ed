// Expansion kernels of the per-pattern operator (sm_103a).
//
// Every op is integer work bounded by HBM: random 64 B bucket reads for the
// probe, then streaming reads of history/adjacency and streaming writes of the
// new table.  No tensor cores are involved.
//
//   k2u     : count (probe; per-row degree and edge offset; per-block output
//             count; per-group sums of output rows and of slices, a slice
//             being at most kSliceRows output rows of one block) -> the host
//             adds up the group sums, sizes the output and passes the groups'
//             prefixes -> expand (one CTA per slice: finds its block from the
//             group prefixes and the group's block counts, the block's local
//             scan, the slice's rows written)
//   k2k/k2c : probe + membership (per-row ballot masks; per-block count; op
//             total) -> filtered copy (per input block: output prefix by
//             look-back, selected rows copied)
//
// The filter's look-back never waits: the first kernel of the op has written
// every block's count before the second kernel starts, so a block finds its
// output prefix by adding its predecessors' counts back to the nearest
// predecessor that has already published its inclusive prefix (or to block 0).
//
// Result order equals the reference CPU engine's (core/engine.hpp:126-225):
// output rows follow input row order, and for k2u each input row's block of
// output rows follows adjacency order.
#include "wk_kernels.h"
#include "wk_probe.cuh"

namespace wk {
namespace dev {

#define FULL 0xffffffffu

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
    return v;
}

// block-wide sum of (u64, u32) pairs; result valid in thread 0
__device__ __forceinline__ void block_sum2(unsigned long long &a, unsigned int &b) {
    __shared__ unsigned long long sa[32];
    __shared__ unsigned int sb[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    a = warp_sum(a);
    b = warp_sum(b);
    if (lane == 0) { sa[wid] = a; sb[wid] = b; }
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        a = lane < nw ? sa[lane] : 0ull;
        b = lane < nw ? sb[lane] : 0u;
        a = warp_sum(a);
        b = warp_sum(b);
    }
}

// --------------------------------------------------------------- k2u count
// A block's output rows are written by slices_of(count) expansion CTAs (none
// for an empty block), so a block that holds hub rows is spread over many
// CTAs and an op with few input blocks but a large fan-out still fills the
// GPU.  The + 3 covers the 16 B alignment lead of the block's first row.
__device__ __forceinline__ unsigned long long slices_of(unsigned long long t) {
    return t == 0ull ? 0ull : (t + 3ull + kSliceRows - 1) / kSliceRows;
}

// Programmatic dependent launch: a count kernel is launched so that its CTAs
// may be placed while the previous op's expansion finishes its last wave, and
// the publish kernel so that its CTA is in place when the count finishes.
// Each CTA of such a kernel first waits (in hardware) until the previous grid
// has completed and its writes are visible; expansion and count CTAs allow
// the dependent launch as soon as they run.
__device__ __forceinline__ void wait_prior_grid() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void allow_dependent_grid() { asm volatile("griddepcontrol.launch_dependents;"); }

// A warp owns kRounds * 32 consecutive rows.  Their start vertices are loaded
// first (kRounds independent coalesced loads), then each round of 32 rows is
// probed, so the history read does not sit in front of every bucket read.
constexpr int kRounds = kRowsPerBlock / (kThreads / 32) / 32;

// blk_sum[b] = the block's output rows, added into its group's sums.  Err bit
// 1 when a block's output count reaches 2^31 (the expansion keeps block-local
// positions in 32 bits).  FUNC (a direction whose lists hold at most one
// vertex): deg receives the neighbour itself as an int32, or -1 for no match,
// and off is unused.  DENSE (the direction is an offsets array): a warp
// issues the lookups of all its rounds phase by phase -- every round's start
// vertex, then every round's offsets or neighbour -- and a lane looks up its
// own key (no shuffles).  BPC blocks per CTA: 2 for a large dense op, so each
// warp keeps eight rounds of loads in flight and a CTA's fixed costs
// (reduction, exit) are shared by 2048 rows; 1 otherwise, so a small op still
// spreads over many CTAs.
template <bool FUNC, bool DENSE, int BPC>
__global__ void __launch_bounds__(kThreads, (DENSE && FUNC) ? 8 : 6)
k2u_count_kernel(const int32_t *__restrict__ hist, int64_t R, int C, int scol, uint32_t dir, PredView pv, uint32_t *__restrict__ deg, uint32_t *__restrict__ off,
                 unsigned long long *__restrict__ blk_sum, unsigned long long *__restrict__ group_sums, int *err,
                 unsigned long long *__restrict__ clear, int64_t nclear) {
    constexpr int NR = kRounds * BPC;   // rounds of 32 rows per warp
    wait_prior_grid();   // before anything is read or cleared
    allow_dependent_grid();   // the publish kernel behind it
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t b0 = (int64_t)blockIdx.x * BPC;
    // the other sums buffer, read by the previous op's expansion, is cleared
    // for the next op (a few hundred words at most)
    for (int64_t w = (int64_t)blockIdx.x * kThreads + threadIdx.x; w < nclear; w += (int64_t)gridDim.x * kThreads)
        clear[w] = 0ull;
    const int64_t nblk = (R + kRowsPerBlock - 1) / kRowsPerBlock;
    // round rd: block b0 + rd / kRounds, the warp's rows 32 (rd % kRounds) + lane
    auto row_at = [&](int rd) -> int64_t {
        return (b0 + rd / kRounds) * kRowsPerBlock + (int64_t)warp * (kRounds * 32) + (rd % kRounds) * 32 + lane;
    };
    int32_t v[NR];
#pragma unroll
    for (int rd = 0; rd < NR; ++rd) {
        const int64_t r = row_at(rd);
        v[rd] = r < R ? __ldg(hist + r * C + scol) : -1;
    }
    unsigned long long my_sum[BPC];
#pragma unroll
    for (int j = 0; j < BPC; ++j) my_sum[j] = 0ull;
    if constexpr (DENSE) {
        const uint32_t vmin = dir ? pv.vmin[1] : pv.vmin[0], dn = dir ? pv.dn[1] : pv.dn[0];
        if constexpr (FUNC) {
            // a dense functional direction keeps the neighbour per id: one 4 B read
            const int32_t *nba = dir ? pv.nb[1] : pv.nb[0];
            int32_t g[NR];
#pragma unroll
            for (int rd = 0; rd < NR; ++rd) {
                const int32_t vid = v[rd];
                const uint32_t x = (uint32_t)vid - vmin;   // wraps above dn below vmin
                g[rd] = (vid > 0 && x < dn) ? __ldg(nba + x) : -1;
                if (vid == 0) atomicOr(err, 8);   // an index key: the op reruns unspecialised
            }
#pragma unroll
            for (int rd = 0; rd < NR; ++rd) {
                const int64_t r = row_at(rd);
                if (r < R) {
                    reinterpret_cast<int32_t *>(deg)[r] = g[rd];
                    my_sum[rd / kRounds] += g[rd] >= 0 ? 1ull : 0ull;
                }
            }
        } else {
            const uint32_t *rp = dir ? pv.rp[1] : pv.rp[0];
            uint32_t a[NR], e[NR];
#pragma unroll
            for (int rd = 0; rd < NR; ++rd) {
                const int32_t vid = v[rd];
                a[rd] = e[rd] = 0u;
                const uint32_t x = (uint32_t)vid - vmin;   // wraps above dn below vmin
                if (vid > 0 && x < dn) {
                    a[rd] = __ldg(rp + x);
                    e[rd] = __ldg(rp + x + 1);
                } else if (vid == 0) {   // index key: the hash table
                    e[rd] = probe_seg(pv.buckets, pv.nmain, pv.nover, seg_key(0u, dir), &a[rd], err);
                    e[rd] += a[rd];
                }
            }
#pragma unroll
            for (int rd = 0; rd < NR; ++rd) {
                const int64_t r = row_at(rd);
                const uint32_t d = e[rd] - a[rd];
                if (r < R) {
                    deg[r] = d;
                    off[r] = a[rd];
                    my_sum[rd / kRounds] += d;
                }
            }
        }
    } else {
        // hashed: runs of equal keys probed once (probe_warp), a round at a time
#pragma unroll
        for (int rd = 0; rd < NR; ++rd) {
            const int64_t r = row_at(rd);
            if (r - lane >= R) break;   // warp-uniform
            uint32_t o, d;
            probe_warp(pv, v[rd], dir, o, d, err);
            if (r < R) {
                if constexpr (FUNC) {
                    reinterpret_cast<int32_t *>(deg)[r] = d ? __ldg(pv.edges + o) : -1;
                    if (d > 1u) atomicOr(err, 8);   // an index list: the op reruns unspecialised
                    // at most one output row per input row, so a block's output never
                    // exceeds its rows even before the rerun
                    my_sum[rd / kRounds] += d ? 1u : 0u;
                } else {
                    deg[r] = d;
                    off[r] = o;
                    my_sum[rd / kRounds] += d;
                }
            }
        }
    }
    // each block's output rows: a warp reduction (one REDUX instruction while the
    // partial sums are small, as every valid block's are) and one barrier
    __shared__ unsigned long long s_part[BPC][kThreads / 32];
#pragma unroll
    for (int j = 0; j < BPC; ++j) {
        unsigned long long ws;
        if (!__any_sync(FULL, my_sum[j] >= (1ull << 26))) ws = __reduce_add_sync(FULL, (unsigned int)my_sum[j]);
        else ws = warp_sum(my_sum[j]);
        if (lane == 0) s_part[j][warp] = ws;
    }
    __syncthreads();
    if (threadIdx.x < BPC) {
        const int j = threadIdx.x;
        const int64_t b = b0 + j;
        unsigned long long sum = 0ull;
#pragma unroll
        for (int w = 0; w < kThreads / 32; ++w) sum += s_part[j][w];
        if (b < nblk) {
            blk_sum[b] = sum;
            // group sums spread the atomics over many addresses (256 blocks each);
            // the host adds them up for the op totals, so no address takes one per block
            if (sum) {
                unsigned long long *gs = group_sums + 2 * (b >> kGroupShift);
                atomicAdd(gs, sum);
                atomicAdd(gs + 1, slices_of(sum));
            }
            if (sum >> 31) atomicOr(err, 2);
        }
    }
}

// One CTA, stream-ordered behind a count kernel: copies the op's error word
// and group sums into pinned host memory, fences them system-wide, then writes
// the sequence number the host waits for.
__global__ void __launch_bounds__(kThreads) publish_kernel(const Publish pub) {
    wait_prior_grid();   // the count kernel's sums are complete
    for (long long w = threadIdx.x; w < pub.n; w += blockDim.x) pub.dst[2 + w] = __ldcg(pub.src + w);
    __threadfence_system();
    __syncthreads();
    if (threadIdx.x == 0) *(volatile unsigned long long *)pub.dst = pub.seq;
}

// ------------------------------------------------------- k2u slice location
static_assert(kThreads == (1 << kGroupShift), "one thread per group and per block of a group");

// inclusive scan of (x, y) pairs over the CTA's threads; sw is free again
// after the caller's next barrier
__device__ __forceinline__ void cta_scan2(unsigned long long &x, unsigned long long &y,
                                          unsigned long long (&sw)[2][kThreads / 32]) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int sh = 1; sh < 32; sh <<= 1) {
        const unsigned long long ax = __shfl_up_sync(FULL, x, sh), ay = __shfl_up_sync(FULL, y, sh);
        if (lane >= sh) { x += ax; y += ay; }
    }
    if (lane == 31) { sw[0][wid] = x; sw[1][wid] = y; }
    __syncthreads();
#pragma unroll
    for (int w = 0; w < kThreads / 32 - 1; ++w)
        if (w < wid) { x += sw[0][w]; y += sw[1][w]; }
}

struct SliceLoc {
    int64_t b;              // the input block
    unsigned long long P;   // output rows of the blocks before it
    uint32_t T;             // its output rows
    uint32_t slice;         // the slice's index within the block
};

// Where expansion CTA k works: the group whose slices cover k, then the
// block within it (a scan of the group's 256 block counts).  The group comes
// from the host's table when the op has one (a uniform binary search, every
// read a broadcast from the parameter bank), else from a scan of the count
// kernel's group sums, 256 groups per pass.  Every non-empty block has
// slices_of(count) slices, in block order.  b is -1 if k is not below the
// op's slice total.
__device__ __forceinline__ SliceLoc locate_slice(unsigned long long k, const unsigned long long *__restrict__ blk_sum,
                                                 const unsigned long long *__restrict__ group_sums, int64_t ngroups,
                                                 int64_t nblk, const GroupTable &gt) {
    __shared__ unsigned long long sw[2][kThreads / 32];
    __shared__ unsigned long long s_tot[2];
    __shared__ int64_t s_g;
    __shared__ SliceLoc s_loc;
    const int t = threadIdx.x;
    SliceLoc none;
    none.b = -1;
    if (t == 0) s_loc.b = -1;
    int64_t g;
    unsigned long long opg, spg;
    if (gt.n > 0) {
        if (k >= gt.sl[gt.n]) return none;   // the same in every thread
        int lo = 0, hi = gt.n - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (gt.sl[mid] <= k) lo = mid;
            else hi = mid - 1;
        }
        g = lo;
        opg = gt.out[lo];
        spg = gt.sl[lo];
    } else {
        unsigned long long op = 0ull, sp = 0ull;   // sums of the groups before the pass
        for (int64_t g0 = 0;; g0 += kThreads) {
            const int64_t gi = g0 + t;
            const unsigned long long x0 = gi < ngroups ? group_sums[2 * gi] : 0ull;
            const unsigned long long y0 = gi < ngroups ? group_sums[2 * gi + 1] : 0ull;
            unsigned long long x = x0, y = y0;
            cta_scan2(x, y, sw);
            if (t == kThreads - 1) { s_tot[0] = x; s_tot[1] = y; }
            // the groups that end at or before slice k are a prefix of the pass
            const int before = __syncthreads_count(gi < ngroups && sp + y <= k);
            if (before < kThreads) {
                if (t == before) {
                    s_tot[0] = op + x - x0;
                    s_tot[1] = sp + y - y0;
                    s_g = gi < ngroups ? gi : -1;
                }
                __syncthreads();
                break;
            }
            op += s_tot[0];
            sp += s_tot[1];
            __syncthreads();   // s_tot and sw are written again by the next pass
        }
        g = s_g;
        if (g < 0) return none;   // the same in every thread
        opg = s_tot[0];
        spg = s_tot[1];
    }
    const unsigned long long kk = k - spg;
    const int64_t bi = (g << kGroupShift) + t;
    const unsigned long long x0 = bi < nblk ? blk_sum[bi] : 0ull;
    const unsigned long long y0 = slices_of(x0);
    unsigned long long x = x0, y = y0;
    cta_scan2(x, y, sw);
    const int before = __syncthreads_count(bi < nblk && y <= kk);
    if (t == before && bi < nblk) {
        s_loc.b = bi;
        s_loc.P = opg + x - x0;
        s_loc.T = (uint32_t)x0;   // below 2^31 (the count kernel flags larger blocks)
        s_loc.slice = (uint32_t)(kk - (y - y0));
    }
    __syncthreads();
    return s_loc;
}

// -------------------------------------------------------------- k2u expand
// last entry k in [0, n) with pos[k] <= j; pos is non-decreasing with pos[0] =
// 0 (n >= 1), so for j below the block's total that entry's list covers j
__device__ __forceinline__ int row_of(const uint32_t *pos, int n, uint32_t j) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (pos[mid] <= j) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// The block's input rows whose list is not empty, compacted in order:
// entry k is block row row[k], its first output row pos[k] (block-local), its
// list offset minus pos[k] in erel[k] (modulo 2^32: erel + j is the entry
// index of output row j), and pos[n] = the block's total.  A sparse direction
// leaves most rows empty, so searches and walks over the entries skip them.
struct ExpandRows {
    uint32_t pos[kRowsPerBlock + 1];
    uint32_t erel[kRowsPerBlock];
    uint16_t row[kRowsPerBlock];
    int n;
};

// One group of 4 output rows.  Rows are counted locally from P - lead, the
// 16 B-aligned row at or before the block's first output row P (lead =
// P mod 4); local row u is block row j = u - lead, valid for lead <= u < span
// (span = lead + the block's count, below 2^31 + 4).  Block row j copies the
// input row of the entry k whose list covers j and appends entry j - pos[k]
// of that list.  A whole group is W 16 B stores (4 rows of W words); the
// first and last group of a block may be partial.
template <int W>
__device__ __forceinline__ void k2u_write_group(uint32_t u, uint32_t lead, uint32_t span, const ExpandRows &er_,
                                                const int32_t *__restrict__ rows, const int32_t *__restrict__ edges,
                                                int32_t *__restrict__ obase) {
    constexpr int C = W - 1;
    int k = row_of(er_.pos, er_.n, u >= lead ? u - lead : 0u);
    uint32_t nxt = er_.pos[k + 1];
    int32_t v[4 * W];
    int kp = -1;       // entry of the previous output row of the group, if valid
    uint32_t er = 0;   // erel[kp]
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const uint32_t uq = u + (uint32_t)q;
        if (uq >= lead && uq < span) {
            const uint32_t j = uq - lead;
            while (j >= nxt) nxt = er_.pos[++k + 1];   // one step per list boundary
            if (q > 0 && k == kp) {
                // the same input row as the previous output row: copied from registers
#pragma unroll
                for (int c = 0; c < C; ++c) v[q * W + c] = v[(q - 1) * W + c];
            } else {
                const int32_t *src = rows + (int)er_.row[k] * C;
#pragma unroll
                for (int c = 0; c < C; ++c) v[q * W + c] = __ldg(src + c);
                er = er_.erel[k];
            }
            v[q * W + C] = __ldg(edges + (er + j));
            kp = k;
        } else {
#pragma unroll
            for (int c = 0; c < W; ++c) v[q * W + c] = 0;
            kp = -1;
        }
    }
    int32_t *g = obase + (size_t)u * W;
    if (u >= lead && u + 4u <= span) {
#pragma unroll
        for (int k2 = 0; k2 < W; ++k2)
            reinterpret_cast<int4 *>(g)[k2] = make_int4(v[4 * k2], v[4 * k2 + 1], v[4 * k2 + 2], v[4 * k2 + 3]);
    } else {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const uint32_t uq = u + (uint32_t)q;
            if (uq >= lead && uq < span) {
#pragma unroll
                for (int c = 0; c < W; ++c) g[q * W + c] = v[q * W + c];
            }
        }
    }
}

// One CTA per slice: CTA k writes local rows [k' kSliceRows, (k' + 1)
// kSliceRows) of block b, where block b's slices are numbered from s_b (the
// slices of the blocks before it) and k' = k - s_b; locate_slice finds b, s_b
// and the block's output prefix.  W = C + 1 output columns for
// 2 <= W <= 8; W = 0 for any width (one output row per thread and step,
// scalar stores).  History rows are read through L1 (consecutive output rows
// of one input row reuse it).
// CTAs per SM the register budget is set for: the widest instantiations need
// more registers to avoid spills
template <int W>
constexpr int expand_min_ctas() { return (W >= 2 && W <= 4) || W == 0 ? 8 : (W <= 7 ? 6 : 4); }

template <int W>
__global__ void __launch_bounds__(kThreads, expand_min_ctas<W>())
k2u_expand_kernel(const int32_t *__restrict__ hist, int64_t R, int C_rt, const int32_t *__restrict__ edges,
                  const uint32_t *__restrict__ deg, const uint32_t *__restrict__ off,
                  const unsigned long long *__restrict__ blk_sum, const unsigned long long *__restrict__ group_sums,
                  int64_t ngroups, int64_t nblk, const __grid_constant__ GroupTable gt, int32_t *__restrict__ out) {
    constexpr int kRPT = kRowsPerBlock / kThreads;
    static_assert(kRPT == 4, "4 input rows per thread");
    __shared__ ExpandRows xr;
    __shared__ uint32_t s_w[2][kThreads / 32];
    const int C = W >= 2 ? W - 1 : C_rt;
    const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
    allow_dependent_grid();

    // 1. the slice's block, the block's output prefix and count
    const SliceLoc loc = locate_slice(blockIdx.x, blk_sum, group_sums, ngroups, nblk, gt);
    if (loc.b < 0) return;   // the same in every thread
    const int64_t b = loc.b;
    const uint32_t slice = loc.slice;
    const int64_t r0 = b * kRowsPerBlock;
    const int n = (int)((R - r0) < kRowsPerBlock ? (R - r0) : kRowsPerBlock);

    // 2. the block's degrees and edge offsets, 4 rows per thread; local
    //    exclusive scans of the degrees and of the non-empty rows
    const int q0 = t * kRPT;
    uint32_t d[kRPT], o[kRPT];
    if (q0 + kRPT <= n) {
        const uint4 dv = *reinterpret_cast<const uint4 *>(deg + r0 + q0);
        const uint4 ov = *reinterpret_cast<const uint4 *>(off + r0 + q0);
        d[0] = dv.x; d[1] = dv.y; d[2] = dv.z; d[3] = dv.w;
        o[0] = ov.x; o[1] = ov.y; o[2] = ov.z; o[3] = ov.w;
    } else {
#pragma unroll
        for (int q = 0; q < kRPT; ++q) {
            d[q] = q0 + q < n ? deg[r0 + q0 + q] : 0u;
            o[q] = q0 + q < n ? off[r0 + q0 + q] : 0u;
        }
    }
    const uint32_t ls = d[0] + d[1] + d[2] + d[3];
    const uint32_t lc = (d[0] != 0u) + (d[1] != 0u) + (d[2] != 0u) + (d[3] != 0u);
    uint32_t is = ls, ic = lc;
#pragma unroll
    for (int sh = 1; sh < 32; sh <<= 1) {
        const uint32_t x = __shfl_up_sync(FULL, is, sh), y = __shfl_up_sync(FULL, ic, sh);
        if (lane >= sh) { is += x; ic += y; }
    }
    if (lane == 31) { s_w[0][wid] = is; s_w[1][wid] = ic; }
    __syncthreads();
    uint32_t e = is - ls, kk = ic - lc;
#pragma unroll
    for (int w = 0; w < kThreads / 32; ++w)
        if (w < wid) { e += s_w[0][w]; kk += s_w[1][w]; }
#pragma unroll
    for (int q = 0; q < kRPT; ++q) {
        if (d[q]) {
            xr.pos[kk] = e;
            xr.erel[kk] = o[q] - e;   // modulo 2^32: erel + j is the entry's index
            xr.row[kk] = (uint16_t)(q0 + q);
            ++kk;
            e += d[q];
        }
    }
    if (t == kThreads - 1) {   // the block's totals; rows >= n have no list
        xr.pos[kk] = e;
        xr.n = (int)kk;
    }
    __syncthreads();
    const unsigned long long P = loc.P;
    const uint32_t T = loc.T;
    const int32_t *hblk = hist + r0 * C;

    // 3. the slice's share of output rows [P, P + T)
    if constexpr (W >= 2) {
        const uint32_t lead = (uint32_t)(P & 3ull), span = T + lead;
        const uint32_t u0 = slice * (uint32_t)kSliceRows;
        const uint32_t u1 = u0 >= span ? u0 : (span - u0 < (uint32_t)kSliceRows ? span : u0 + (uint32_t)kSliceRows);
        int32_t *obase = out + (P - lead) * W;
        for (uint32_t u = u0 + 4u * (uint32_t)t; u < u1; u += 4u * kThreads)
            k2u_write_group<W>(u, lead, span, xr, hblk, edges, obase);
    } else {
        const int Wd = C + 1;
        int32_t *oblk = out + P * Wd;
        const uint32_t j0 = slice * (uint32_t)kSliceRows;
        const uint32_t j1 = j0 >= T ? j0 : (T - j0 < (uint32_t)kSliceRows ? T : j0 + (uint32_t)kSliceRows);
        for (uint32_t j = j0 + (uint32_t)t; j < j1; j += kThreads) {
            const int k = row_of(xr.pos, xr.n, j);
            int32_t *dst = oblk + (size_t)j * Wd;
            const int32_t *src = hblk + (int64_t)xr.row[k] * C;
            for (int c = 0; c < C; ++c) dst[c] = __ldg(src + c);
            dst[C] = __ldg(edges + (xr.erel[k] + j));
        }
    }
}

// ------------------------------------------------- k2u expand, functional
// A direction whose lists hold at most one vertex: the expansion is a
// compaction of the matched rows with their neighbour appended.  One CTA per
// non-empty input block (its only slice).  Warp w takes rows 128 w .. 128 w +
// 127 in four passes of 32 consecutive rows, finds each matched row's output
// position by ballots, copies the row and its neighbour into shared memory
// (rows kPitch words apart, an odd pitch so the 32 lanes' rows fall in 32
// banks), and the CTA then streams the block's output words to HBM as
// aligned int4 stores.
template <int W>
__global__ void __launch_bounds__(kThreads)
k2u_expand_func_kernel(const int32_t *__restrict__ hist, int64_t R, const int32_t *__restrict__ nbr,
                       const unsigned long long *__restrict__ blk_sum,
                       const unsigned long long *__restrict__ group_sums, int64_t ngroups, int64_t nblk,
                       const __grid_constant__ GroupTable gt, int32_t *__restrict__ out) {
    constexpr int C = W - 1;
    constexpr int kPitch = W | 1;
    __shared__ int32_t rows[kRowsPerBlock * kPitch];
    __shared__ uint32_t s_w[kThreads / 32];
    const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
    allow_dependent_grid();

    // the block (every non-empty block has one slice)
    const SliceLoc loc = locate_slice(blockIdx.x, blk_sum, group_sums, ngroups, nblk, gt);
    if (loc.b < 0) return;   // the same in every thread
    const int64_t b = loc.b;
    const int64_t r0 = b * kRowsPerBlock;
    const int n = (int)((R - r0) < kRowsPerBlock ? (R - r0) : kRowsPerBlock);

    // matched rows and their block-local output positions
    int32_t x[4];
    unsigned bm[4];
    unsigned wtot = 0;
#pragma unroll
    for (int ps = 0; ps < 4; ++ps) {
        const int r = wid * 128 + ps * 32 + lane;
        x[ps] = r < n ? __ldg(nbr + r0 + r) : -1;
        bm[ps] = __ballot_sync(FULL, x[ps] >= 0);
        wtot += __popc(bm[ps]);
    }
    if (lane == 0) s_w[wid] = wtot;
    __syncthreads();
    unsigned base = 0;
#pragma unroll
    for (int w = 0; w < kThreads / 32; ++w)
        if (w < wid) base += s_w[w];
    const unsigned below = (1u << lane) - 1u;
#pragma unroll
    for (int ps = 0; ps < 4; ++ps) {
        if (x[ps] >= 0) {
            const int r = wid * 128 + ps * 32 + lane;
            const unsigned q = base + __popc(bm[ps] & below);
            const int32_t *src = hist + (r0 + r) * C;
            int32_t *dst = rows + q * kPitch;
#pragma unroll
            for (int c = 0; c < C; ++c) dst[c] = __ldg(src + c);
            dst[C] = x[ps];
        }
        base += __popc(bm[ps]);
    }
    __syncthreads();

    // output words [P W, (P + T) W): int4 stores aligned to 16 B of out
    const unsigned long long P = loc.P;
    const uint32_t T = loc.T;
    const uint32_t lead = (uint32_t)((P * W) & 3ull), words = T * W;
    int32_t *g = out + (P * W - lead);
    for (uint32_t i = (uint32_t)t; 4u * i < lead + words; i += kThreads) {
        int32_t v[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const uint32_t kk = 4u * i + j - lead;   // wraps above `words` before the lead
            v[j] = kk < words ? rows[(kk / W) * kPitch + kk % W] : 0;
        }
        if (4u * i >= lead && 4u * i + 4u <= lead + words) {
            reinterpret_cast<int4 *>(g)[i] = make_int4(v[0], v[1], v[2], v[3]);
        } else {
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const uint32_t kk = 4u * i + j - lead;
                if (kk < words) g[4u * i + j] = v[j];
            }
        }
    }
}

// ------------------------------------------------------- k2k / k2c probe
// lower_bound of `v` in the ascending list e[0..n).  Lists hold distinct ids,
// so lower_bound is also the position where the reference's linear scan
// (core/engine.hpp:172-179) stops; *scanned receives the entries that scan
// touches (position + 1 on a match, n otherwise).
__device__ __forceinline__ bool list_contains(const int32_t *__restrict__ e, uint32_t n, int32_t v,
                                              uint32_t *scanned) {
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(e + mid) < v) lo = mid + 1;
        else hi = mid;
    }
    const bool f = lo < n && __ldg(e + lo) == v;
    *scanned = f ? lo + 1 : n;
    return f;
}

// The general lookup of the filter probe: probe_warp (runs of equal keys
// probed once) where every lane takes it; in the NB kernel only a lane with an
// index key (a start value of 0) gets here, alone, and looks itself up.
template <bool NB>
__device__ __forceinline__ void probe_view_or_warp(const PredView &pv, int32_t vid, uint32_t dir, uint32_t &o,
                                                   uint32_t &d, int *err) {
    if constexpr (NB) {
        o = 0u;
        d = vid >= 0 ? probe_view(pv, (uint32_t)vid, dir, &o, err) : 0u;
    } else {
        probe_warp(pv, vid, dir, o, d, err);
    }
}

// totals[0] += adjacency entries a linear scan would touch, totals[1] += rows kept.
// NB: the direction is dense and functional, so its neighbour array answers a
// membership test with one 4 B read (the list holds that neighbour or
// nothing; a linear scan touches 1 entry or none); a start value of 0 (an
// index key, hashed) takes the general path.  All rounds' reads are issued
// before any is used.
// One CTA per block of input rows (two blocks per CTA, with eight rounds of
// loads in flight per lane, took 48 registers and ran slower).
template <bool NB>
__global__ void __launch_bounds__(kThreads, 6)
filter_probe_kernel(const int32_t *__restrict__ hist, int64_t R, int C, int scol, int ecol,
                    int32_t end_const, uint32_t dir, PredView pv,
                    uint32_t *__restrict__ mask, unsigned int *__restrict__ blk_nz,
                    unsigned long long *__restrict__ group_sums, unsigned long long *__restrict__ clear,
                    int64_t nclear, unsigned long long *__restrict__ totals, int *err) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // the other sums buffer, read by the previous op's write or expansion, is
    // cleared for the next op (a few hundred words at most)
    for (int64_t w = (int64_t)blockIdx.x * kThreads + threadIdx.x; w < nclear; w += (int64_t)gridDim.x * kThreads)
        clear[w] = 0ull;
    const int64_t b = blockIdx.x;
    const int64_t wrow0 = b * kRowsPerBlock + (int64_t)warp * (kRounds * 32);
    int32_t v[kRounds], tg[kRounds];
#pragma unroll
    for (int rd = 0; rd < kRounds; ++rd) {
        const int64_t r = wrow0 + rd * 32 + lane;
        v[rd] = r < R ? __ldg(hist + r * C + scol) : -1;
        tg[rd] = (r < R && ecol >= 0) ? __ldg(hist + r * C + ecol) : end_const;
    }
    unsigned int my_nz = 0u;   // kept rows (lane 0)
    unsigned long long my_scan = 0;
    int32_t g[kRounds];   // NB: the neighbour, or -1 (none, or not looked up here)
    if constexpr (NB) {
        const int32_t *nba = dir ? pv.nb[1] : pv.nb[0];
        const uint32_t vmin = dir ? pv.vmin[1] : pv.vmin[0], dn = dir ? pv.dn[1] : pv.dn[0];
#pragma unroll
        for (int rd = 0; rd < kRounds; ++rd) {
            const uint32_t x = (uint32_t)v[rd] - vmin;   // wraps above dn below vmin
            g[rd] = (v[rd] > 0 && x < dn) ? __ldg(nba + x) : -1;
        }
    }
#pragma unroll
    for (int rd = 0; rd < kRounds; ++rd) {
        const int64_t row0 = wrow0 + rd * 32, r = row0 + lane;
        if (row0 >= R) break;   // warp-uniform
        bool found = false;
        if (NB && v[rd] != 0) {
            found = r < R && g[rd] >= 0 && g[rd] == tg[rd];
            my_scan += (r < R && g[rd] >= 0) ? 1u : 0u;
        } else {
            uint32_t o, d;
            probe_view_or_warp<NB>(pv, v[rd], dir, o, d, err);
            if (r < R && d > 0u) {
                uint32_t sc = 0;
                found = list_contains(pv.edges + o, d, tg[rd], &sc);
                my_scan += sc;
            }
        }
        const uint32_t m = __ballot_sync(FULL, found);
        if (lane == 0) {
            mask[row0 >> 5] = m;
            my_nz += __popc(m);
        }
    }
    block_sum2(my_scan, my_nz);
    if (threadIdx.x == 0) {
        blk_nz[b] = my_nz;
        if (my_scan) atomicAdd(totals, my_scan);
        if (my_nz) {
            atomicAdd(totals + 1, (unsigned long long)my_nz);
            atomicAdd(group_sums + 2 * (b >> kGroupShift), (unsigned long long)my_nz);
        }
    }
}

// ----------------------------------------------------------- filter write
// A write CTA takes kWriteBlocks consecutive blocks of input rows, one per
// warp, all in one group of 2^kGroupShift blocks.  Their output prefixes need
// no look-back and no wait: the probe kernel added every block's kept-row
// count into its group's sum, so the prefix of the CTA's first block is the
// sum of the group sums before its group and of the block counts before it in
// the group -- one CTA reduction -- and warp w adds the counts of the CTA's
// blocks before its own.  Each warp then writes its block alone: the kept
// rows' positions from the block's 32 mask words (one per lane, a warp scan
// of their popcounts), then the block's output words [P C, (P + nb) C) as
// aligned 16 B stores where whole, each word gathered from its kept row (the
// block's rows stay in L1 and L2 while the warp copies them).
constexpr int kWriteBlocks = kThreads / 32;
static_assert(((1 << kGroupShift) % kWriteBlocks) == 0, "a write CTA's blocks share a group");

template <int CT>   // the columns, or 0 for any (C_rt)
__global__ void __launch_bounds__(kThreads)
filter_write_kernel(const int32_t *__restrict__ hist, int64_t R, int C_rt, const uint32_t *__restrict__ mask,
                    const unsigned int *__restrict__ blk_nz, const unsigned long long *__restrict__ group_sums,
                    int32_t *__restrict__ out) {
    __shared__ uint16_t sel[kWriteBlocks][kRowsPerBlock];   // each warp's kept rows, in order
    __shared__ unsigned long long s_part[kThreads / 32];
    __shared__ unsigned int s_nz[kWriteBlocks];
    const int C = CT > 0 ? CT : C_rt;
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const int64_t nblk = (R + kRowsPerBlock - 1) / kRowsPerBlock;
    const int64_t b0 = (int64_t)blockIdx.x * kWriteBlocks;
    const int64_t g = b0 >> kGroupShift;

    // 1. the prefix of block b0, and the CTA's blocks' counts
    unsigned long long x = 0ull;
    for (int64_t i = t; i < g; i += kThreads) x += group_sums[2 * i];
    for (int64_t i = (g << kGroupShift) + t; i < b0; i += kThreads) x += blk_nz[i];
    if (t < kWriteBlocks) s_nz[t] = b0 + t < nblk ? blk_nz[b0 + t] : 0u;
    x = warp_sum(x);
    if (lane == 0) s_part[w] = x;
    __syncthreads();
    unsigned long long P = 0ull;
#pragma unroll
    for (int i = 0; i < kThreads / 32; ++i) P += s_part[i];
    for (int i = 0; i < w; ++i) P += s_nz[i];
    const unsigned int nb = s_nz[w];
    if (nb == 0u) return;   // the warp's block keeps nothing (or lies past the table)

    // 2. the block's kept rows, in order
    const int64_t b = b0 + w, r0 = b * kRowsPerBlock;
    const int64_t wi = (r0 >> 5) + lane, nwords = (R + 31) >> 5;
    uint32_t m = wi < nwords ? mask[wi] : 0u;   // bits past R are 0
    const unsigned int c = __popc(m);
    unsigned int pos = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned int v = __shfl_up_sync(FULL, pos, o);
        if (lane >= o) pos += v;
    }
    pos -= c;
    uint16_t *ws = sel[w];
    while (m) {
        ws[pos++] = (uint16_t)(lane * 32 + __ffs(m) - 1);
        m &= m - 1u;
    }
    __syncwarp();

    // 3. output words [P C, (P + nb) C) as int4 stores aligned to 16 B of out
    const int32_t *hb = hist + r0 * C;
    const uint32_t words = nb * (uint32_t)C;
    const uint32_t lead = (uint32_t)((P * (unsigned long long)C) & 3ull);
    int32_t *gout = out + (P * (unsigned long long)C - lead);
    for (uint32_t u = (uint32_t)lane; 4u * u < lead + words; u += 32u) {
        int32_t v[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const uint32_t kk = 4u * u + (uint32_t)j - lead;   // wraps above `words` before the lead
            v[j] = kk < words ? __ldg(hb + (int)ws[kk / (uint32_t)C] * C + (int)(kk % (uint32_t)C)) : 0;
        }
        if (4u * u >= lead && 4u * u + 4u <= lead + words) {
            reinterpret_cast<int4 *>(gout)[u] = make_int4(v[0], v[1], v[2], v[3]);
        } else {
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const uint32_t kk = 4u * u + (uint32_t)j - lead;
                if (kk < words) gout[4u * u + j] = v[j];
            }
        }
    }
}

// ------------------------------------------------------------- list copy
__global__ void copy_list_kernel(const int32_t *__restrict__ src, int64_t n, int32_t *__restrict__ dst) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = __ldg(src + i);
}

// ============================================================== launchers
static inline unsigned int nblocks_rows(int64_t R) {
    return (unsigned int)((R + kRowsPerBlock - 1) / kRowsPerBlock);
}

void launch_k2u_count(const int32_t *hist, int64_t R, int C, int scol, uint32_t dir, PredView pv, uint32_t *deg, uint32_t *off, unsigned long long *blk_sum, unsigned long long *group_sums,
                      int *err, bool func, unsigned long long *clear, int64_t nclear, int sms, cudaStream_t st) {
    const bool dense = (dir ? pv.rp[1] : pv.rp[0]) != nullptr;
    const unsigned int nb = nblocks_rows(R);
    // two blocks per CTA once the op has enough blocks to fill the GPU with half as many CTAs
    if (sms < 1) sms = 1;
    const bool pair = dense && nb >= 16u * (unsigned int)sms;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.blockDim = dim3(kThreads);
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
#define WK_COUNT(F, D, B)                                                                                         \
    do {                                                                                                         \
        cfg.gridDim = dim3((nb + B - 1) / B);                                                                    \
        cudaLaunchKernelEx(&cfg, k2u_count_kernel<F, D, B>, hist, R, C, scol, dir, pv, deg, off, blk_sum,         \
                           group_sums, err, clear, nclear);                                                      \
    } while (0)
    if (func && dense) {
        if (pair) WK_COUNT(true, true, 2);
        else WK_COUNT(true, true, 1);
    } else if (func) {
        WK_COUNT(true, false, 1);
    } else if (dense) {
        if (pair) WK_COUNT(false, true, 2);
        else WK_COUNT(false, true, 1);
    } else {
        WK_COUNT(false, false, 1);
    }
#undef WK_COUNT
}

// launched so that its one CTA is in place when the count kernel finishes
void launch_publish(const Publish &pub, cudaStream_t st) {
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(1);
    cfg.blockDim = dim3(kThreads);
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, publish_kernel, pub);
}

void launch_k2u_expand_func(const int32_t *hist, int64_t R, int C, const int32_t *nbr,
                            const unsigned long long *blk_sum, const unsigned long long *group_sums,
                            const GroupTable &gt, unsigned long long slices, int32_t *out, cudaStream_t st) {
    if (slices == 0ull) return;
    const int64_t nblk = (R + kRowsPerBlock - 1) / kRowsPerBlock;
    const int64_t ng = (nblk + (1 << kGroupShift) - 1) >> kGroupShift;
    const unsigned int g = (unsigned int)slices;
#define WK_EXPAND_F(WC) \
    k2u_expand_func_kernel<WC><<<g, kThreads, 0, st>>>(hist, R, nbr, blk_sum, group_sums, ng, nblk, gt, out)
    switch (C + 1) {
        case 2: WK_EXPAND_F(2); break;
        case 3: WK_EXPAND_F(3); break;
        case 4: WK_EXPAND_F(4); break;
        case 5: WK_EXPAND_F(5); break;
        case 6: WK_EXPAND_F(6); break;
        case 7: WK_EXPAND_F(7); break;
        default: WK_EXPAND_F(8); break;
    }
#undef WK_EXPAND_F
}

void launch_k2u_expand(const int32_t *hist, int64_t R, int C, const int32_t *edges, const uint32_t *deg,
                       const uint32_t *off, const unsigned long long *blk_sum, const unsigned long long *group_sums,
                       const GroupTable &gt, unsigned long long slices, int32_t *out, cudaStream_t st) {
    if (slices == 0ull) return;
    const int64_t nblk = (R + kRowsPerBlock - 1) / kRowsPerBlock;
    const int64_t ng = (nblk + (1 << kGroupShift) - 1) >> kGroupShift;
    const unsigned int g = (unsigned int)slices;
#define WK_EXPAND(WC) \
    k2u_expand_kernel<WC><<<g, kThreads, 0, st>>>(hist, R, C, edges, deg, off, blk_sum, group_sums, ng, nblk, gt, \
                                                 out)
    switch (C + 1) {
        case 2: WK_EXPAND(2); break;
        case 3: WK_EXPAND(3); break;
        case 4: WK_EXPAND(4); break;
        case 5: WK_EXPAND(5); break;
        case 6: WK_EXPAND(6); break;
        case 7: WK_EXPAND(7); break;
        case 8: WK_EXPAND(8); break;
        default: WK_EXPAND(0); break;
    }
#undef WK_EXPAND
}

// Load every k2u count and expansion kernel now (with lazy module loading a
// kernel's code is otherwise loaded, and device memory taken for it, at its
// first launch).
int preload_k2u_kernels() {
    cudaFuncAttributes a;
    cudaError_t e = cudaSuccess;
    auto get = [&](const void *f) {
        if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, f);
    };
    get((const void *)k2u_count_kernel<false, false, 1>);
    get((const void *)k2u_count_kernel<false, true, 1>);
    get((const void *)k2u_count_kernel<false, true, 2>);
    get((const void *)k2u_count_kernel<true, false, 1>);
    get((const void *)k2u_count_kernel<true, true, 1>);
    get((const void *)k2u_count_kernel<true, true, 2>);
    get((const void *)publish_kernel);
    get((const void *)k2u_expand_kernel<0>);
    get((const void *)k2u_expand_kernel<2>);
    get((const void *)k2u_expand_kernel<3>);
    get((const void *)k2u_expand_kernel<4>);
    get((const void *)k2u_expand_kernel<5>);
    get((const void *)k2u_expand_kernel<6>);
    get((const void *)k2u_expand_kernel<7>);
    get((const void *)k2u_expand_kernel<8>);
    return (int)e;
}

void launch_filter_probe(const int32_t *hist, int64_t R, int C, int scol, int ecol, int32_t end_const,
                         uint32_t dir, PredView pv, uint32_t *mask, unsigned int *blk_nz,
                         unsigned long long *group_sums, unsigned long long *clear, int64_t nclear,
                         unsigned long long *totals, int *err, cudaStream_t st) {
    const unsigned int nb = nblocks_rows(R);
#define WK_PROBE(NBV) \
    filter_probe_kernel<NBV><<<nb, kThreads, 0, st>>>(hist, R, C, scol, ecol, end_const, dir, pv, mask, blk_nz, \
                                                      group_sums, clear, nclear, totals, err)
    if ((dir ? pv.nb[1] : pv.nb[0]) != nullptr) WK_PROBE(true);
    else WK_PROBE(false);
#undef WK_PROBE
}

void launch_filter_write(const int32_t *hist, int64_t R, int C, const uint32_t *mask, const unsigned int *blk_nz,
                         const unsigned long long *group_sums, int32_t *out, cudaStream_t st) {
    const unsigned int g = (nblocks_rows(R) + kWriteBlocks - 1) / kWriteBlocks;
#define WK_FWRITE(CC) filter_write_kernel<CC><<<g, kThreads, 0, st>>>(hist, R, C, mask, blk_nz, group_sums, out)
    switch (C) {
        case 1: WK_FWRITE(1); break;
        case 2: WK_FWRITE(2); break;
        case 3: WK_FWRITE(3); break;
        case 4: WK_FWRITE(4); break;
        case 5: WK_FWRITE(5); break;
        case 6: WK_FWRITE(6); break;
        case 7: WK_FWRITE(7); break;
        case 8: WK_FWRITE(8); break;
        default: WK_FWRITE(0); break;
    }
#undef WK_FWRITE
}

void launch_copy_list(const int32_t *src, int64_t n, int32_t *dst, cudaStream_t st) {
    int64_t nb = (n + 255) / 256;
    if (nb > 152 * 16) nb = 152 * 16;
    if (nb < 1) nb = 1;
    copy_list_kernel<<<(unsigned int)nb, 256, 0, st>>>(src, n, dst);
}

}  // namespace dev
}  // namespace wk
