// Device sort of the store build: the triples ordered by (predicate, s, o) and
// by (predicate, o, s), the two orders the store's out-lists and in-lists are
// cut from (core/dgraph.hpp:268-330 sorts per predicate with
// edge_sort_by_spo / edge_sort_by_ops, core/gstore.hpp:56-99).
//
// A stable least-significant-digit radix sort of (key, predicate) pairs,
// key = hi << 32 | lo: 8-bit digits of lo, then of hi, then of the predicate,
// skipping the digit positions above the largest value.  Each pass is three
// kernels: per-tile digit counts, one exclusive scan of the counts
// (digit-major, so equal digits of later tiles follow earlier ones), and a
// stable scatter.  A tile is 4096 pairs (256 threads x 16); each warp owns 512
// consecutive pairs, ranks its pairs per digit with __match_any_sync in
// order, and takes its digits' offsets after the warps before it.
#include "wk_runtime.h"

#include <algorithm>

namespace wk {
namespace sortdev {

constexpr int kThreads = 256;
constexpr int kPer = 16;                       // pairs per thread
constexpr int kTile = kThreads * kPer;         // 4096 pairs per tile
constexpr int kBins = 256;
constexpr int kWarps = kThreads / 32;

__device__ __forceinline__ uint32_t digit_of(uint64_t key, uint32_t pid, int shift) {
    // shift 0..56: a digit of the key; 64, 72, 80: a digit of the predicate
    return shift < 64 ? (uint32_t)(key >> shift) & 0xffu : (pid >> (shift - 64)) & 0xffu;
}

// counts[d * ntiles + tile] = pairs of the tile with digit d
__global__ void __launch_bounds__(kThreads)
hist_kernel(const uint64_t *__restrict__ key, const uint32_t *__restrict__ pid, int64_t n, int shift,
            uint32_t *__restrict__ counts, int64_t ntiles) {
    __shared__ uint32_t h[kBins];
    const int t = threadIdx.x;
    h[t] = 0u;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * kTile;
#pragma unroll 4
    for (int i = 0; i < kPer; ++i) {
        const int64_t g = base + (int64_t)i * kThreads + t;
        if (g < n) atomicAdd(&h[digit_of(key[g], pid[g], shift)], 1u);
    }
    __syncthreads();
    counts[(int64_t)t * ntiles + blockIdx.x] = h[t];
}

// Exclusive scan of m uint32 counts in place, in three steps: per-block sums,
// a scan of the block sums in one block, and the blocks' own scans.
constexpr int kScanPer = 8;
constexpr int kScanBlock = kThreads * kScanPer;   // 2048 entries per block

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t *total, uint32_t *sw) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t in = v;
#pragma unroll
    for (int sh = 1; sh < 32; sh <<= 1) {
        const uint32_t x = __shfl_up_sync(0xffffffffu, in, sh);
        if (lane >= sh) in += x;
    }
    if (lane == 31) sw[wid] = in;
    __syncthreads();
    uint32_t off = 0, all = 0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) {
        if (w < wid) off += sw[w];
        all += sw[w];
    }
    __syncthreads();
    *total = all;
    return off + in - v;
}

__global__ void __launch_bounds__(kThreads)
scan_sums_kernel(const uint32_t *__restrict__ c, int64_t m, uint32_t *__restrict__ bsum) {
    __shared__ uint32_t sw[kWarps];
    const int64_t b0 = (int64_t)blockIdx.x * kScanBlock + (int64_t)threadIdx.x * kScanPer;
    uint32_t s = 0;
#pragma unroll
    for (int i = 0; i < kScanPer; ++i)
        if (b0 + i < m) s += c[b0 + i];
    uint32_t tot;
    block_exclusive_scan(s, &tot, sw);
    if (threadIdx.x == 0) bsum[blockIdx.x] = tot;
}

// one block: exclusive scan of nb block sums (nb arbitrary; chunks of kScanBlock)
__global__ void __launch_bounds__(kThreads)
scan_top_kernel(uint32_t *__restrict__ bsum, int64_t nb) {
    __shared__ uint32_t sw[kWarps];
    uint32_t carry = 0;
    for (int64_t c0 = 0; c0 < nb; c0 += kScanBlock) {
        const int64_t b0 = c0 + (int64_t)threadIdx.x * kScanPer;
        uint32_t v[kScanPer], s = 0;
#pragma unroll
        for (int i = 0; i < kScanPer; ++i) {
            v[i] = b0 + i < nb ? bsum[b0 + i] : 0u;
            s += v[i];
        }
        uint32_t tot;
        uint32_t e = block_exclusive_scan(s, &tot, sw) + carry;
#pragma unroll
        for (int i = 0; i < kScanPer; ++i) {
            if (b0 + i < nb) bsum[b0 + i] = e;
            e += v[i];
        }
        carry += tot;
    }
}

__global__ void __launch_bounds__(kThreads)
scan_apply_kernel(uint32_t *__restrict__ c, int64_t m, const uint32_t *__restrict__ bsum) {
    __shared__ uint32_t sw[kWarps];
    const int64_t b0 = (int64_t)blockIdx.x * kScanBlock + (int64_t)threadIdx.x * kScanPer;
    uint32_t v[kScanPer], s = 0;
#pragma unroll
    for (int i = 0; i < kScanPer; ++i) {
        v[i] = b0 + i < m ? c[b0 + i] : 0u;
        s += v[i];
    }
    uint32_t tot;
    uint32_t e = block_exclusive_scan(s, &tot, sw) + bsum[blockIdx.x];
#pragma unroll
    for (int i = 0; i < kScanPer; ++i) {
        if (b0 + i < m) c[b0 + i] = e;
        e += v[i];
    }
}

// Stable scatter of one tile.  Warp w owns tile pairs [512 w, 512 w + 512),
// lane l the pairs 512 w + 32 i + l (i = 0..15, coalesced); tile order within
// a warp is i-major, then lane, so ranks taken step by step are stable.
__global__ void __launch_bounds__(kThreads)
scatter_kernel(const uint64_t *__restrict__ key, const uint32_t *__restrict__ pid, int64_t n, int shift,
               const uint32_t *__restrict__ offs, int64_t ntiles, uint64_t *__restrict__ key_out,
               uint32_t *__restrict__ pid_out) {
    __shared__ uint32_t wcnt[kWarps][kBins];   // digit counts per warp, then each warp's digit offsets
    const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
    for (int i = t; i < kWarps * kBins; i += kThreads) (&wcnt[0][0])[i] = 0u;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * kTile + (int64_t)wid * (kPer * 32);
    uint64_t k[kPer];
    uint32_t pv[kPer], d[kPer];
#pragma unroll
    for (int i = 0; i < kPer; ++i) {
        const int64_t g = base + (int64_t)i * 32 + lane;
        const bool ok = g < n;
        k[i] = ok ? key[g] : 0ull;
        pv[i] = ok ? pid[g] : 0u;
        d[i] = ok ? digit_of(k[i], pv[i], shift) : 0xffffffffu;   // past the end: no digit
    }
    // 1. this warp's count of each digit
#pragma unroll
    for (int i = 0; i < kPer; ++i) {
        const unsigned peers = __match_any_sync(0xffffffffu, d[i]);
        if (d[i] != 0xffffffffu && lane == __ffs(peers) - 1) wcnt[wid][d[i]] += __popc(peers);
    }
    __syncthreads();
    // 2. per digit: the tile's global offset, then the warps in order
    {
        const int dg = t;   // kThreads == kBins
        uint32_t o = offs[(int64_t)dg * ntiles + blockIdx.x];
#pragma unroll
        for (int w = 0; w < kWarps; ++w) {
            const uint32_t c = wcnt[w][dg];
            wcnt[w][dg] = o;
            o += c;
        }
    }
    __syncthreads();
    // 3. ranks in order; the first lane of each digit group advances the warp's offset
    const unsigned below = (1u << lane) - 1u;
#pragma unroll
    for (int i = 0; i < kPer; ++i) {
        const unsigned peers = __match_any_sync(0xffffffffu, d[i]);
        if (d[i] != 0xffffffffu) {
            const uint32_t at = wcnt[wid][d[i]] + __popc(peers & below);
            key_out[at] = k[i];
            pid_out[at] = pv[i];
        }
        __syncwarp();
        if (d[i] != 0xffffffffu && lane == __ffs(peers) - 1) wcnt[wid][d[i]] += __popc(peers);
        __syncwarp();
    }
}

// key = hi << 32 | lo with (hi, lo) = (s, o) or (o, s)
__global__ void pack_kernel(const int32_t *__restrict__ s, const int32_t *__restrict__ p,
                            const int32_t *__restrict__ o, int64_t n, int order, uint64_t *__restrict__ key,
                            uint32_t *__restrict__ pid) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t a = (uint32_t)s[i], b = (uint32_t)o[i];
        key[i] = order == 0 ? ((uint64_t)a << 32 | b) : ((uint64_t)b << 32 | a);
        pid[i] = (uint32_t)p[i];
    }
}

int bits_of(uint64_t v) {
    int b = 0;
    while (v) { ++b; v >>= 1; }
    return b;
}

}  // namespace sortdev

// Exclusive scan of m uint32 values in place on stream st (the sum of all m
// must stay below 2^32); scratch receives the block sums.
int scan_u32_device(uint32_t *x, int64_t m, DevBuf &scratch, cudaStream_t st, int64_t *launches) {
    using namespace sortdev;
    if (m <= 0) return WK_OK;
    const int64_t nb = (m + kScanBlock - 1) / kScanBlock;
    int rc = scratch.reserve((size_t)nb * 4);
    if (rc) return rc;
    scan_sums_kernel<<<(unsigned int)nb, kThreads, 0, st>>>(x, m, scratch.as<uint32_t>());
    scan_top_kernel<<<1, kThreads, 0, st>>>(scratch.as<uint32_t>(), nb);
    scan_apply_kernel<<<(unsigned int)nb, kThreads, 0, st>>>(x, m, scratch.as<uint32_t>());
    if (launches) *launches += 3;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? WK_OK : cuda_fail(e, "device scan");
}

// Stable LSD radix sort of n (key, id) pairs on stream st by (id, key): the
// key's 8-bit digits at the given bit offsets (0..56), then the id's digits
// up to id_bits.  key/id hold the input and receive the result; key_tmp and
// id_tmp are ping-pong buffers of the same sizes.
int sort_pairs_device(uint64_t *key, uint32_t *id, uint64_t *key_tmp, uint32_t *id_tmp, int64_t n,
                      const std::vector<int> &key_shifts, int id_bits, cudaStream_t st, int64_t *launches) {
    using namespace sortdev;
    if (n <= 1) return WK_OK;
    const int64_t ntiles = (n + kTile - 1) / kTile;
    const int64_t m = ntiles * kBins;
    DevBuf cnt, bs;
    int rc;
    if ((rc = cnt.reserve((size_t)m * 4))) return rc;
    std::vector<int> shifts(key_shifts);
    for (int sh = 0; sh < id_bits; sh += 8) shifts.push_back(64 + sh);
    uint64_t *kb[2] = {key, key_tmp};
    uint32_t *pb[2] = {id, id_tmp};
    int cur = 0;
    const unsigned int gt = (unsigned int)ntiles;
    for (int sh : shifts) {
        hist_kernel<<<gt, kThreads, 0, st>>>(kb[cur], pb[cur], n, sh, cnt.as<uint32_t>(), ntiles);
        if ((rc = scan_u32_device(cnt.as<uint32_t>(), m, bs, st, launches))) return rc;
        scatter_kernel<<<gt, kThreads, 0, st>>>(kb[cur], pb[cur], n, sh, cnt.as<uint32_t>(), ntiles, kb[1 - cur],
                                                pb[1 - cur]);
        if (launches) *launches += 2;
        cur = 1 - cur;
    }
    cudaError_t e = cudaSuccess;
    if (cur == 1) {   // the result is in the tmp buffers: move it back
        if ((e = cudaMemcpyAsync(key, key_tmp, (size_t)n * 8, cudaMemcpyDeviceToDevice, st)) == cudaSuccess)
            e = cudaMemcpyAsync(id, id_tmp, (size_t)n * 4, cudaMemcpyDeviceToDevice, st);
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    return e == cudaSuccess ? WK_OK : cuda_fail(e, "device sort");
}

// Pack the triples of one order (0: s << 32 | o, 1: o << 32 | s) with their
// predicates, from device copies of s, p, o.
void pack_triples_device(const int32_t *s, const int32_t *p, const int32_t *o, int64_t n, int order, uint64_t *key,
                         uint32_t *pid, cudaStream_t st) {
    sortdev::pack_kernel<<<1024, 256, 0, st>>>(s, p, o, n, order, key, pid);
}

int radix_bits(uint64_t v) { return sortdev::bits_of(v); }

}  // namespace wk
