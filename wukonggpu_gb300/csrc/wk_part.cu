// Fork-join across ranks: the device-side split of a history table by the
// rank that owns each row's start vertex, and device-to-device transfers of
// tables in and out of a context (for a collective's buffers).
//
//   wk_history_partition <-> RCache::generate_sub_query (core/rcache.hpp:964-1030)
//                            with calc_dispatched_position / history_dispatch
//                            (core/gpu_hash.cu:698-790), as GPU_Engine::
//                            generate_sub_query calls it (core/gpu_engine.hpp:293-370)
//
// The owner of a row is its start column's value modulo the number of parts,
// the rule of mymath::hash_mod (utils/mymath.hpp:55-59) applied by
// d_hash_dispatched_server_id and Engine::generate_sub_requests
// (core/engine.hpp:355-358).  The reference places rows within a part by an
// atomicAdd per row, so their order there depends on scheduling; here the
// split is stable (a part keeps the rows in their input order), which gives
// every part the same multiset of rows and a fixed order besides.
//
// Steps on the op stream, a stable counting split in two passes over the
// table:
//   1. part_count: per tile of 2048 rows, the rows of each owner (warp
//      match-any, one shared-memory add per owner and chunk of 32 rows);
//   2. one exclusive scan of those counts laid out owner by owner, tile by
//      tile: the global start of every (owner, tile) slot, so a part keeps
//      its tiles, and the rows within a tile, in input order;
//   3. part_scatter: each tile again, in order; a row's place in its part is
//      its tile slot's start, plus the rows of that owner in the tile's
//      earlier warps and earlier chunks, plus its rank among the lanes of its
//      chunk with the same owner;
//   4. the parts' bounds from the scanned slots, read back once.
#include "wk_runtime.h"

#include <algorithm>
#include <vector>

namespace wk {
int scan_u32_device(uint32_t *x, int64_t m, DevBuf &scratch, cudaStream_t st, int64_t *launches);
}

using namespace wk;

namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kMaxParts = 256;
constexpr int kTile = 2048;                 // rows per CTA
constexpr int kChunks = kTile / kThreads;   // chunks of 32 rows per warp
#define FULL 0xffffffffu

// the owner of row r, or ~0 past the table
__device__ __forceinline__ uint32_t owner_of(const int32_t *__restrict__ hist, int64_t r, int64_t R, int C, int col,
                                             uint32_t nparts) {
    return r < R ? (uint32_t)__ldg(hist + r * C + col) % nparts : FULL;
}

// row of chunk c of warp w in tile t
__device__ __forceinline__ int64_t tile_row(int64_t t, int w, int c, int lane) {
    return t * kTile + (int64_t)w * (kChunks * 32) + c * 32 + lane;
}

// cnt[p * ntiles + t] = rows of owner p in tile t
__global__ void __launch_bounds__(kThreads)
part_count_kernel(const int32_t *__restrict__ hist, int64_t R, int C, int col, uint32_t nparts, int64_t ntiles,
                  uint32_t *__restrict__ cnt) {
    __shared__ uint32_t h[kMaxParts];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (uint32_t p = threadIdx.x; p < nparts; p += kThreads) h[p] = 0u;
    __syncthreads();
    const int64_t t = blockIdx.x;
    uint32_t own[kChunks];   // every load in flight before the first match
#pragma unroll
    for (int c = 0; c < kChunks; ++c) own[c] = owner_of(hist, tile_row(t, w, c, lane), R, C, col, nparts);
#pragma unroll
    for (int c = 0; c < kChunks; ++c) {
        const uint32_t o = own[c];
        const unsigned m = __match_any_sync(FULL, o);
        if (o != FULL && lane == __ffs(m) - 1) atomicAdd(&h[o], (uint32_t)__popc(m));
    }
    __syncthreads();
    for (uint32_t p = threadIdx.x; p < nparts; p += kThreads) cnt[(int64_t)p * ntiles + t] = h[p];
}

// one row of C ints (CT = C for 1, 2 and 4 columns: one vector load and
// store; CT = 0 for any C)
template <int CT>
__device__ __forceinline__ void copy_row(const int32_t *__restrict__ src, int32_t *__restrict__ dst, int C) {
    if constexpr (CT == 4) {
        *reinterpret_cast<int4 *>(dst) = __ldg(reinterpret_cast<const int4 *>(src));
    } else if constexpr (CT == 2) {
        *reinterpret_cast<int2 *>(dst) = __ldg(reinterpret_cast<const int2 *>(src));
    } else if constexpr (CT == 1) {
        *dst = __ldg(src);
    } else {
        for (int k = 0; k < C; ++k) dst[k] = __ldg(src + k);
    }
}

// rows of tile t to their places: start[p * ntiles + t] is where owner p's
// rows of the tile begin (the scanned counts)
template <int CT>
__global__ void __launch_bounds__(kThreads)
part_scatter_kernel(const int32_t *__restrict__ hist, int64_t R, int C, int col, uint32_t nparts, int64_t ntiles,
                    const uint32_t *__restrict__ start, int32_t *__restrict__ out) {
    __shared__ uint32_t wc[kWarps][kMaxParts];   // per warp: its rows per owner, then its next place per owner
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t t = blockIdx.x;
    for (uint32_t p = threadIdx.x; p < nparts; p += kThreads)
#pragma unroll
        for (int x = 0; x < kWarps; ++x) wc[x][p] = 0u;
    __syncthreads();
    uint32_t own[kChunks];   // every load in flight before the first match
#pragma unroll
    for (int c = 0; c < kChunks; ++c) own[c] = owner_of(hist, tile_row(t, w, c, lane), R, C, col, nparts);
#pragma unroll
    for (int c = 0; c < kChunks; ++c) {
        const uint32_t o = own[c];
        const unsigned m = __match_any_sync(FULL, o);
        if (o != FULL && lane == __ffs(m) - 1) wc[w][o] += (uint32_t)__popc(m);   // this warp's row of wc only
        __syncwarp();
    }
    __syncthreads();
    // per owner: the tile's start, then the warps in order
    for (uint32_t p = threadIdx.x; p < nparts; p += kThreads) {
        uint32_t acc = start[(int64_t)p * ntiles + t];
#pragma unroll
        for (int x = 0; x < kWarps; ++x) {
            const uint32_t n = wc[x][p];
            wc[x][p] = acc;
            acc += n;
        }
    }
    __syncthreads();
    const unsigned below = (1u << lane) - 1u;
#pragma unroll
    for (int c = 0; c < kChunks; ++c) {
        const uint32_t o = own[c];
        const unsigned m = __match_any_sync(FULL, o);
        if (o != FULL) {
            const uint32_t pos = wc[w][o] + (uint32_t)__popc(m & below);
            copy_row<CT>(hist + tile_row(t, w, c, lane) * C, out + (int64_t)pos * C, C);
        }
        __syncwarp();
        if (o != FULL && lane == __ffs(m) - 1) wc[w][o] += (uint32_t)__popc(m);
        __syncwarp();
    }
}

// bound[p] = the first row of part p, bound[nparts] = R
__global__ void part_bounds_kernel(const uint32_t *__restrict__ start, int64_t ntiles, int64_t R, uint32_t nparts,
                                   int64_t *__restrict__ bound) {
    for (uint32_t p = threadIdx.x; p <= nparts; p += blockDim.x)
        bound[p] = p < nparts ? (int64_t)start[(int64_t)p * ntiles] : R;
}

}  // namespace

extern "C" int wk_history_partition(wk_ctx *ctx, const wk_history *in, int64_t start, int32_t nparts,
                                    int64_t *part_rows, wk_history *out) {
    if (!ctx || !in || !out || !part_rows) return set_error(WK_EINVAL, "wk_history_partition: null argument");
    if (ctx->device < 0) return set_error(WK_EDEVICE, "wk_history_partition: host-only context");
    if (nparts < 1 || nparts > kMaxParts)
        return set_error(WK_EINVAL, "wk_history_partition: %d parts (1..%d)", nparts, kMaxParts);
    const int C = in->col_num;
    if (start >= 0 || C <= 0 || -start - 1 >= C)
        return set_error(WK_EINVAL, "wk_history_partition: start %lld is not a bound variable of a %d-column table",
                         (long long)start, C);
    if (in->size < 0 || in->size % C != 0 || (in->size > 0 && !in->data))
        return set_error(WK_EINVAL, "wk_history_partition: bad table (size %lld, %d columns)", (long long)in->size, C);
    const int64_t R = in->size / C;
    if (R >= (int64_t)UINT32_MAX) return set_error(WK_EINVAL, "wk_history_partition: %lld rows (< 2^32 - 1)", (long long)R);
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    const int32_t *src = in->data;
    const int32_t step = in->step;
    DevBuf &ob = (src == static_cast<const int32_t *>(ctx->hbuf[0].ptr)) ? ctx->hbuf[1] : ctx->hbuf[0];
    int st = ob.reserve((size_t)in->size * 4 + 16);
    if (st) return st;
    cudaStream_t s = ctx->stream;
    DevBuf &cb = ctx->part_cnt, &sb = ctx->part_scan, &bb = ctx->part_bound;
    if ((st = bb.reserve((size_t)(kMaxParts + 1) * 8))) return st;
    std::vector<int64_t> bound((size_t)nparts + 1, 0);
    if (R > 0) {
        const int64_t ntiles = (R + kTile - 1) / kTile, m = ntiles * nparts;
        if ((st = cb.reserve((size_t)m * 4))) return st;
        const int col = (int)(-start - 1);
        part_count_kernel<<<(unsigned)ntiles, kThreads, 0, s>>>(src, R, C, col, (uint32_t)nparts, ntiles,
                                                                cb.as<uint32_t>());
        ++ctx->launches;
        if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "partition count");
        if ((st = scan_u32_device(cb.as<uint32_t>(), m, sb, s, &ctx->launches))) return st;
        // vector copies need 4 B x C aligned rows in both tables (the history
        // buffers are 256 B aligned; a caller's table may not be)
        const bool al = ((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(ob.ptr)) & 15u) == 0;
#define WK_SCATTER(CT)                                                                                               \
    part_scatter_kernel<CT><<<(unsigned)ntiles, kThreads, 0, s>>>(src, R, C, col, (uint32_t)nparts, ntiles, \
                                                                      cb.as<uint32_t>(), ob.as<int32_t>())
        if (al && C == 4) WK_SCATTER(4);
        else if (al && C == 2) WK_SCATTER(2);
        else if (C == 1) WK_SCATTER(1);
        else WK_SCATTER(0);
#undef WK_SCATTER
        part_bounds_kernel<<<1, kThreads, 0, s>>>(cb.as<uint32_t>(), ntiles, R, (uint32_t)nparts, bb.as<int64_t>());
        ctx->launches += 2;
        if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "partition scatter");
        if ((e = cudaMemcpyAsync(bound.data(), bb.ptr, bound.size() * 8, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
            return cuda_fail(e, "partition bounds readback");
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail(e, "partition sync");
    }
    for (int p = 0; p < nparts; ++p) part_rows[p] = bound[(size_t)p + 1] - bound[(size_t)p];
    out->data = ob.as<int32_t>();
    out->size = in->size;
    out->col_num = C;
    out->step = step;
    return WK_OK;
}

extern "C" int wk_history_to_device(wk_ctx *ctx, const wk_history *h, int32_t *dst, int64_t cap) {
    if (!ctx || !h || (h->size > 0 && (!dst || cap < h->size)))
        return set_error(WK_EINVAL, "wk_history_to_device: bad arguments (cap %lld < size %lld)", (long long)cap,
                         h ? (long long)h->size : 0ll);
    if (ctx->device < 0) return set_error(WK_EDEVICE, "wk_history_to_device: host-only context");
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    if (h->size > 0 &&
        (e = cudaMemcpyAsync(dst, h->data, (size_t)h->size * 4, cudaMemcpyDeviceToDevice, ctx->stream)) != cudaSuccess)
        return cuda_fail(e, "wk_history_to_device");
    if ((e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess) return cuda_fail(e, "wk_history_to_device sync");
    return WK_OK;
}

extern "C" int wk_history_from_device(wk_ctx *ctx, wk_history *h, const int32_t *src, int64_t size, int32_t col_num) {
    if (!ctx || !h || size < 0 || (size > 0 && !src) || col_num < 0 || (col_num == 0 && size != 0) ||
        (col_num > 0 && size % col_num != 0))
        return set_error(WK_EINVAL, "wk_history_from_device: bad arguments");
    if (ctx->device < 0) return set_error(WK_EDEVICE, "wk_history_from_device: host-only context");
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    DevBuf &b = ctx->hbuf[0];
    int st = b.reserve((size_t)size * 4 + 16);
    if (st) return st;
    if (size > 0 && (e = cudaMemcpyAsync(b.ptr, src, (size_t)size * 4, cudaMemcpyDeviceToDevice, ctx->stream)) != cudaSuccess)
        return cuda_fail(e, "wk_history_from_device");
    if ((e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess) return cuda_fail(e, "wk_history_from_device sync");
    h->data = static_cast<int32_t *>(b.ptr);
    h->size = size;
    h->col_num = col_num;
    return WK_OK;
}
