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
// Steps on the op stream: a key (owner << 32 | row) per row; one stable
// radix pass on the owner byte (wk_sort.cu); a gather of the rows in key
// order into the ping-pong partner of the input buffer; the parts' bounds by
// a binary search per part over the sorted keys, read back once.
#include "wk_runtime.h"

#include <algorithm>
#include <vector>

namespace wk {
int sort_pairs_device(uint64_t *key, uint32_t *id, uint64_t *key_tmp, uint32_t *id_tmp, int64_t n,
                      const std::vector<int> &key_shifts, int id_bits, cudaStream_t st, int64_t *launches);
}

using namespace wk;

namespace {

constexpr int kThreads = 256;
constexpr int kMaxParts = 256;   // the owner is one radix digit

__global__ void owner_keys_kernel(const int32_t *__restrict__ hist, int64_t R, int C, int col, uint32_t nparts,
                                  uint64_t *__restrict__ key, uint32_t *__restrict__ id) {
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < R; r += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t owner = (uint32_t)__ldg(hist + r * C + col) % nparts;
        key[r] = ((uint64_t)owner << 32) | (uint64_t)r;
        id[r] = 0u;
    }
}

// out row i = in row (low 32 bits of key[i])
template <int C>
__global__ void gather_rows_fixed_kernel(const int32_t *__restrict__ in, const uint64_t *__restrict__ key, int64_t R,
                                         int32_t *__restrict__ out) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < R; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t src = (int64_t)(uint32_t)key[i];
#pragma unroll
        for (int c = 0; c < C; ++c) out[i * C + c] = __ldg(in + src * C + c);
    }
}

__global__ void gather_rows_kernel(const int32_t *__restrict__ in, const uint64_t *__restrict__ key, int64_t R, int C,
                                   int32_t *__restrict__ out) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < R; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t src = (int64_t)(uint32_t)key[i];
        for (int c = 0; c < C; ++c) out[i * C + c] = __ldg(in + src * C + c);
    }
}

// bound[p] = the first sorted row whose owner is >= p, for p in [0, nparts]
__global__ void part_bounds_kernel(const uint64_t *__restrict__ key, int64_t R, int nparts, int64_t *__restrict__ bound) {
    for (int p = threadIdx.x; p <= nparts; p += blockDim.x) {
        int64_t lo = 0, hi = R;
        while (lo < hi) {
            const int64_t mid = (lo + hi) >> 1;
            if ((int)(key[mid] >> 32) < p) lo = mid + 1;
            else hi = mid;
        }
        bound[p] = lo;
    }
}

int launch_gather(const int32_t *in, const uint64_t *key, int64_t R, int C, int32_t *out, unsigned int g,
                  cudaStream_t st) {
    switch (C) {
    case 1: gather_rows_fixed_kernel<1><<<g, kThreads, 0, st>>>(in, key, R, out); break;
    case 2: gather_rows_fixed_kernel<2><<<g, kThreads, 0, st>>>(in, key, R, out); break;
    case 3: gather_rows_fixed_kernel<3><<<g, kThreads, 0, st>>>(in, key, R, out); break;
    case 4: gather_rows_fixed_kernel<4><<<g, kThreads, 0, st>>>(in, key, R, out); break;
    default: gather_rows_kernel<<<g, kThreads, 0, st>>>(in, key, R, C, out); break;
    }
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? WK_OK : cuda_fail(e, "partition gather");
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
    DevBuf &kb = ctx->part_key[0], &kt = ctx->part_key[1], &ib = ctx->part_id[0], &it = ctx->part_id[1];
    DevBuf &bb = ctx->part_bound;
    if ((st = bb.reserve((size_t)(kMaxParts + 1) * 8))) return st;
    if (R > 0) {
        if ((st = kb.reserve((size_t)R * 8)) || (st = kt.reserve((size_t)R * 8)) || (st = ib.reserve((size_t)R * 4)) ||
            (st = it.reserve((size_t)R * 4)))
            return st;
        const unsigned int g = (unsigned int)std::min<int64_t>((R + kThreads - 1) / kThreads, (int64_t)ctx->sms * 8);
        owner_keys_kernel<<<g, kThreads, 0, s>>>(src, R, C, (int)(-start - 1), (uint32_t)nparts, kb.as<uint64_t>(),
                                                  ib.as<uint32_t>());
        ++ctx->launches;
        if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "partition keys");
        if (nparts > 1 &&
            (st = sort_pairs_device(kb.as<uint64_t>(), ib.as<uint32_t>(), kt.as<uint64_t>(), it.as<uint32_t>(), R,
                                    std::vector<int>{32}, 0, s, &ctx->launches)))
            return st;
        if ((st = launch_gather(src, kb.as<uint64_t>(), R, C, ob.as<int32_t>(), g, s))) return st;
        part_bounds_kernel<<<1, kThreads, 0, s>>>(kb.as<uint64_t>(), R, nparts, bb.as<int64_t>());
        ctx->launches += 2;
        if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "partition bounds");
    }
    std::vector<int64_t> bound((size_t)nparts + 1, 0);
    if (R > 0) {
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
