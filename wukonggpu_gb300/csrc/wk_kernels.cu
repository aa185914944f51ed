// Expansion kernels of the per-pattern operator (sm_103a).
//
// Every op is integer work bounded by HBM: random 64 B bucket reads for the
// probe, then streaming reads of history/adjacency and streaming writes of the
// new table.  No tensor cores are involved.
//
//   k2u : probe (+ per-block sums) -> block scan -> compact -> tiled write
//   k2k/k2c : probe + membership (ballot masks) -> block scan -> filtered copy
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

// ----------------------------------------------------------------- k2u probe
// A warp owns kRounds * 32 consecutive rows.  Their start vertices are loaded
// first (kRounds independent coalesced loads), then each round of 32 rows is
// probed, so the history read does not sit in front of every bucket read.
constexpr int kRounds = kRowsPerBlock / (kThreads / 32) / 32;

__global__ void __launch_bounds__(kThreads)
k2u_probe_kernel(const int32_t *__restrict__ hist, int64_t R, int C, int scol, uint32_t dir, PredView pv,
                 uint32_t *__restrict__ deg, uint32_t *__restrict__ off,
                 unsigned long long *__restrict__ blk_sum, unsigned int *__restrict__ blk_nz, int *err) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t wrow0 = (int64_t)blockIdx.x * kRowsPerBlock + (int64_t)warp * (kRounds * 32);
    int32_t v[kRounds];
#pragma unroll
    for (int rd = 0; rd < kRounds; ++rd) {
        const int64_t r = wrow0 + rd * 32 + lane;
        v[rd] = r < R ? __ldg(hist + r * C + scol) : -1;
    }
    unsigned long long my_sum = 0;
    unsigned int my_nz = 0;
#pragma unroll
    for (int rd = 0; rd < kRounds; ++rd) {
        const int64_t row0 = wrow0 + rd * 32;
        if (row0 >= R) break;   // warp-uniform
        const int64_t r = row0 + lane;
        uint32_t o, d;
        probe_warp(pv, v[rd], dir, o, d, err);
        if (r < R) {
            deg[r] = d;
            off[r] = o;
            my_sum += d;
            my_nz += d > 0u;
        }
    }
    block_sum2(my_sum, my_nz);
    if (threadIdx.x == 0) {
        blk_sum[blockIdx.x] = my_sum;
        blk_nz[blockIdx.x] = my_nz;
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

__global__ void __launch_bounds__(kThreads)
filter_probe_kernel(const int32_t *__restrict__ hist, int64_t R, int C, int scol, int ecol,
                    int32_t end_const, uint32_t dir, PredView pv,
                    uint32_t *__restrict__ mask, unsigned long long *__restrict__ blk_sum,
                    unsigned int *__restrict__ blk_nz, int *err) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t wrow0 = (int64_t)blockIdx.x * kRowsPerBlock + (int64_t)warp * (kRounds * 32);
    int32_t v[kRounds], tg[kRounds];
#pragma unroll
    for (int rd = 0; rd < kRounds; ++rd) {
        const int64_t r = wrow0 + rd * 32 + lane;
        v[rd] = r < R ? __ldg(hist + r * C + scol) : -1;
        tg[rd] = (r < R && ecol >= 0) ? __ldg(hist + r * C + ecol) : end_const;
    }
    unsigned int my_nz = 0;
    unsigned long long my_scan = 0;   // adjacency entries a linear scan would touch
#pragma unroll
    for (int rd = 0; rd < kRounds; ++rd) {
        const int64_t row0 = wrow0 + rd * 32;
        if (row0 >= R) break;   // warp-uniform
        const int64_t r = row0 + lane;
        uint32_t o, d;
        probe_warp(pv, v[rd], dir, o, d, err);
        bool found = false;
        if (r < R && d > 0u) {
            uint32_t sc = 0;
            found = list_contains(pv.edges + o, d, tg[rd], &sc);
            my_scan += sc;
        }
        const uint32_t m = __ballot_sync(FULL, found);
        if (lane == 0) {
            mask[row0 >> 5] = m;
            my_nz += __popc(m);
        }
    }
    block_sum2(my_scan, my_nz);
    if (threadIdx.x == 0) {
        blk_sum[blockIdx.x] = my_scan;
        blk_nz[blockIdx.x] = my_nz;
    }
}

// ------------------------------------------------------------ block scan
// One block: exclusive scan of n (u64, u32) pairs in place.
__global__ void __launch_bounds__(1024)
scan_blocks_kernel(unsigned long long *__restrict__ s, unsigned int *__restrict__ z, int64_t n,
                   unsigned long long *__restrict__ totals, unsigned long long *__restrict__ cz_pos) {
    __shared__ unsigned long long ws[32];
    __shared__ unsigned int wz[32];
    const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
    const int64_t per = (n + 1023) / 1024;
    const int64_t a = (int64_t)t * per, b = a + per < n ? a + per : n;
    unsigned long long ls = 0;
    unsigned int lz = 0;
    for (int64_t i = a; i < b; ++i) { ls += s[i]; lz += z[i]; }
    // inclusive warp scan
    unsigned long long is = ls;
    unsigned int iz = lz;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long vs = __shfl_up_sync(FULL, is, o);
        const unsigned int vz = __shfl_up_sync(FULL, iz, o);
        if (lane >= o) { is += vs; iz += vz; }
    }
    if (lane == 31) { ws[wid] = is; wz[wid] = iz; }
    __syncthreads();
    if (wid == 0) {
        unsigned long long x = ws[lane];
        unsigned int y = wz[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long vs = __shfl_up_sync(FULL, x, o);
            const unsigned int vz = __shfl_up_sync(FULL, y, o);
            if (lane >= o) { x += vs; y += vz; }
        }
        ws[lane] = x;   // inclusive over warps
        wz[lane] = y;
    }
    __syncthreads();
    unsigned long long es = is - ls + (wid ? ws[wid - 1] : 0ull);
    unsigned int ez = iz - lz + (wid ? wz[wid - 1] : 0u);
    for (int64_t i = a; i < b; ++i) {
        const unsigned long long vs = s[i];
        const unsigned int vz = z[i];
        s[i] = es;
        z[i] = ez;
        es += vs;
        ez += vz;
    }
    if (t == 1023) {
        totals[0] = es;
        totals[1] = ez;
        if (cz_pos) cz_pos[ez] = es;
    }
}

// ------------------------------------------------------------ k2u compact
__global__ void __launch_bounds__(kThreads)
k2u_compact_kernel(const uint32_t *__restrict__ deg, const uint32_t *__restrict__ off, int64_t R,
                   const unsigned long long *__restrict__ blk_sum, const unsigned int *__restrict__ blk_nz,
                   int32_t *__restrict__ cz_row, unsigned long long *__restrict__ cz_pos,
                   uint32_t *__restrict__ cz_off, int32_t *__restrict__ tile_k0, int tile_rows) {
    __shared__ unsigned long long ws[kThreads / 32];
    __shared__ unsigned int wz[kThreads / 32];
    constexpr int kPer = kRowsPerBlock / kThreads;   // 4 rows per thread
    const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
    const int64_t r0 = (int64_t)blockIdx.x * kRowsPerBlock + (int64_t)t * kPer;
    uint32_t d[kPer];
    unsigned long long ls = 0;
    unsigned int lz = 0;
#pragma unroll
    for (int q = 0; q < kPer; ++q) {
        d[q] = (r0 + q < R) ? deg[r0 + q] : 0u;
        ls += d[q];
        lz += d[q] > 0u;
    }
    unsigned long long is = ls;
    unsigned int iz = lz;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long vs = __shfl_up_sync(FULL, is, o);
        const unsigned int vz = __shfl_up_sync(FULL, iz, o);
        if (lane >= o) { is += vs; iz += vz; }
    }
    if (lane == 31) { ws[wid] = is; wz[wid] = iz; }
    __syncthreads();
    unsigned long long es = blk_sum[blockIdx.x] + is - ls;
    unsigned int ez = blk_nz[blockIdx.x] + iz - lz;
    for (int w = 0; w < wid; ++w) { es += ws[w]; ez += wz[w]; }
#pragma unroll
    for (int q = 0; q < kPer; ++q) {
        if (d[q] == 0u) continue;
        const int64_t r = r0 + q;
        cz_row[ez] = (int32_t)r;
        cz_pos[ez] = es;
        cz_off[ez] = off[r];
        // every tile whose first output row falls in [es, es + d) starts at this row
        const unsigned long long T = (unsigned long long)tile_rows;
        for (unsigned long long tt = (es + T - 1) / T; tt * T < es + d[q]; ++tt) tile_k0[tt] = (int32_t)ez;
        es += d[q];
        ++ez;
    }
}

// -------------------------------------------------------------- k2u write
// One block per output tile of `tile_rows` rows.  The compacted source rows
// covering the tile are staged in shared memory; each output row finds its
// source by binary search, then the tile is written as a contiguous run of
// 16 B stores (the tile start is a multiple of 32 rows, so 16 B aligned).
// WC = output width (C + 1) when known at compile time, 0 for the generic case.
template <int WC>
__global__ void __launch_bounds__(kThreads)
k2u_write_kernel(const int32_t *__restrict__ hist, int C_rt, const int32_t *__restrict__ edges,
                 const int32_t *__restrict__ cz_row, const unsigned long long *__restrict__ cz_pos,
                 const uint32_t *__restrict__ cz_off, int64_t nz, const int32_t *__restrict__ tile_k0,
                 int64_t ntiles, int tile_rows, int64_t R_out, int32_t *__restrict__ out) {
    extern __shared__ int smem[];
    int *pos_rel = smem;                         // tile_rows + 2
    int *srow = pos_rel + tile_rows + 2;         // tile_rows + 1
    uint32_t *soff = (uint32_t *)(srow + tile_rows + 1);   // tile_rows + 1
    int *rsrc = (int *)(soff + tile_rows + 1);   // tile_rows
    const int W = WC > 0 ? WC : C_rt + 1;
    const int C = W - 1;

    const int64_t t = blockIdx.x;
    const int64_t o0 = t * (int64_t)tile_rows;
    const int nrows = (int)((R_out - o0) < tile_rows ? (R_out - o0) : tile_rows);
    const int64_t k0 = tile_k0[t];
    const int64_t k1 = (t + 1 < ntiles) ? (int64_t)tile_k0[t + 1] : nz - 1;
    const int nk = (int)(k1 - k0 + 1);
    for (int i = threadIdx.x; i < nk; i += blockDim.x) {
        pos_rel[i] = (int)((long long)cz_pos[k0 + i] - (long long)o0);
        srow[i] = cz_row[k0 + i];
        soff[i] = cz_off[k0 + i];
    }
    __syncthreads();
    for (int j = threadIdx.x; j < nrows; j += blockDim.x) {
        int lo = 0, hi = nk - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (pos_rel[mid] <= j) lo = mid;
            else hi = mid - 1;
        }
        rsrc[j] = lo;
    }
    __syncthreads();
    const int nwords = nrows * W;
    int32_t *gout = out + o0 * W;
    const int nvec = (nwords + 3) >> 2;
    for (int v = threadIdx.x; v < nvec; v += blockDim.x) {
        const int w0 = v << 2;
        int j = w0 / W, c = w0 - j * W;
        int vals[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            int x = 0;
            if (w0 + q < nwords) {
                const int i = rsrc[j];
                if (c < C) x = __ldg(hist + (int64_t)srow[i] * C + c);
                else x = __ldg(edges + soff[i] + (uint32_t)(j - pos_rel[i]));
            }
            vals[q] = x;
            if (++c == W) { c = 0; ++j; }
        }
        if (w0 + 4 <= nwords) {
            reinterpret_cast<int4 *>(gout)[v] = make_int4(vals[0], vals[1], vals[2], vals[3]);
        } else {
            for (int q = 0; q < 4 && w0 + q < nwords; ++q) gout[w0 + q] = vals[q];
        }
    }
}

// ----------------------------------------------------------- filter write
__global__ void __launch_bounds__(kThreads)
filter_write_kernel(const int32_t *__restrict__ hist, int64_t R, int C, const uint32_t *__restrict__ mask,
                    const unsigned int *__restrict__ blk_nz, int32_t *__restrict__ out) {
    __shared__ int sel[kRowsPerBlock];
    __shared__ unsigned int wbase[kRowsPerBlock / 32 + 1];
    constexpr int kPer = kRowsPerBlock / kThreads;   // 4 rows per thread
    const int64_t r0 = (int64_t)blockIdx.x * kRowsPerBlock;
    const int64_t nwords_mask = (R + 31) >> 5;
    const int t = threadIdx.x;
    if (t < 32) {
        const int64_t wi = (r0 >> 5) + t;
        const uint32_t m = wi < nwords_mask ? mask[wi] : 0u;
        unsigned int c = __popc(m), inc = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned int v = __shfl_up_sync(FULL, inc, o);
            if (t >= o) inc += v;
        }
        wbase[t] = inc - c;
        if (t == 31) wbase[32] = inc;
    }
    __syncthreads();
    {
        const int wi = (t * kPer) >> 5, bit0 = (t * kPer) & 31;
        const int64_t mwi = (r0 >> 5) + wi;
        const uint32_t m = mwi < nwords_mask ? mask[mwi] : 0u;
        unsigned int pos = wbase[wi] + __popc(m & ((1u << bit0) - 1u));
#pragma unroll
        for (int q = 0; q < kPer; ++q)
            if (m & (1u << (bit0 + q))) sel[pos++] = t * kPer + q;
    }
    __syncthreads();
    const int nsel = (int)wbase[32];
    const int64_t base = (int64_t)blk_nz[blockIdx.x] * C;
    const int64_t nwords = (int64_t)nsel * C;
    for (int64_t w = t; w < nwords; w += blockDim.x) {
        const int j = (int)(w / C), c = (int)(w - (int64_t)j * C);
        out[base + w] = __ldg(hist + (r0 + sel[j]) * C + c);
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

int k2u_tile_rows(int out_cols) {
    (void)out_cols;
    return 1024;
}

static size_t k2u_write_smem(int tile_rows) { return (size_t)(4 * tile_rows + 4) * sizeof(int); }

void launch_k2u_probe(const int32_t *hist, int64_t R, int C, int scol, uint32_t dir, PredView pv,
                      uint32_t *deg, uint32_t *off, unsigned long long *blk_sum, unsigned int *blk_nz,
                      int *err, cudaStream_t st) {
    k2u_probe_kernel<<<nblocks_rows(R), kThreads, 0, st>>>(hist, R, C, scol, dir, pv, deg, off, blk_sum,
                                                           blk_nz, err);
}

void launch_filter_probe(const int32_t *hist, int64_t R, int C, int scol, int ecol, int32_t end_const,
                         uint32_t dir, PredView pv, uint32_t *mask, unsigned long long *blk_sum,
                         unsigned int *blk_nz, int *err, cudaStream_t st) {
    filter_probe_kernel<<<nblocks_rows(R), kThreads, 0, st>>>(hist, R, C, scol, ecol, end_const, dir, pv,
                                                              mask, blk_sum, blk_nz, err);
}

void launch_scan_blocks(unsigned long long *blk_sum, unsigned int *blk_nz, int64_t nblk,
                        unsigned long long *totals, unsigned long long *cz_pos, cudaStream_t st) {
    scan_blocks_kernel<<<1, 1024, 0, st>>>(blk_sum, blk_nz, nblk, totals, cz_pos);
}

void launch_k2u_compact(const uint32_t *deg, const uint32_t *off, int64_t R,
                        const unsigned long long *blk_sum, const unsigned int *blk_nz,
                        int32_t *cz_row, unsigned long long *cz_pos, uint32_t *cz_off,
                        int32_t *tile_k0, int tile_rows, cudaStream_t st) {
    k2u_compact_kernel<<<nblocks_rows(R), kThreads, 0, st>>>(deg, off, R, blk_sum, blk_nz, cz_row, cz_pos,
                                                             cz_off, tile_k0, tile_rows);
}

void launch_k2u_write(const int32_t *hist, int C, const int32_t *edges, const int32_t *cz_row,
                      const unsigned long long *cz_pos, const uint32_t *cz_off, int64_t nz,
                      const int32_t *tile_k0, int64_t ntiles, int tile_rows, int64_t R_out,
                      int32_t *out, cudaStream_t st) {
    const unsigned int g = (unsigned int)ntiles;
    const size_t sm = k2u_write_smem(tile_rows);
#define WK_WRITE(WC)                                                                                   \
    k2u_write_kernel<WC><<<g, kThreads, sm, st>>>(hist, C, edges, cz_row, cz_pos, cz_off, nz, tile_k0, \
                                                  ntiles, tile_rows, R_out, out)
    switch (C + 1) {
        case 2: WK_WRITE(2); break;
        case 3: WK_WRITE(3); break;
        case 4: WK_WRITE(4); break;
        case 5: WK_WRITE(5); break;
        case 6: WK_WRITE(6); break;
        case 7: WK_WRITE(7); break;
        case 8: WK_WRITE(8); break;
        default: WK_WRITE(0); break;
    }
#undef WK_WRITE
}

void launch_filter_write(const int32_t *hist, int64_t R, int C, const uint32_t *mask,
                         const unsigned int *blk_nz, int32_t *out, cudaStream_t st) {
    filter_write_kernel<<<nblocks_rows(R), kThreads, 0, st>>>(hist, R, C, mask, blk_nz, out);
}

void launch_copy_list(const int32_t *src, int64_t n, int32_t *dst, cudaStream_t st) {
    int64_t nb = (n + 255) / 256;
    if (nb > 152 * 16) nb = 152 * 16;
    if (nb < 1) nb = 1;
    copy_list_kernel<<<(unsigned int)nb, 256, 0, st>>>(src, n, dst);
}

}  // namespace dev
}  // namespace wk
