// known_to_unknown without any allocation.
//
// Some callers cannot allocate device memory at the moment they expand a
// pattern: a host that runs this operator inside its own memory-pool
// callback or under a fixed device-memory budget, or a real-time serving
// thread that must never enter cudaMalloc/cudaFree (both can synchronise the
// whole device and stall every other stream).  This entry point serves them:
// the caller passes the input history and an output buffer it already owns,
// and every scratch array of the two-pass expansion lives in one file-scope
// device array of fixed size, so the call allocates nothing.
//
// Limits and sharing rules:
//   - at most kMaxRows input rows per call (262,144); a larger call is
//     rejected with WK_EINVAL before any device work; the output is bounded
//     only by the caller's capacity (WK_EOVERFLOW, with the row count);
//   - the array (about 2.1 MB) is loaded on a device, and its address looked
//     up, when a context is made for that device (wk_ctx_create calls
//     noalloc_prepare), together with the kernels this entry point launches:
//     with lazy module loading both would otherwise be loaded -- and device
//     memory taken -- inside the first call.  The array then stays on that
//     GPU until the process exits;
//   - every call shares it and it keeps the last call's contents: the fields
//     that must start at zero (error flags and group sums) are cleared at the
//     start of each call, everything else is fully written before it is read.
//     Calls that overlap on the GPU (from several host threads or several
//     contexts' streams at once) race on the array and must not be issued;
//   - a context keeps the address it looked up; it must not be used after a
//     reset of its device.
#include <cstdint>

#include "wk_runtime.h"

namespace {

constexpr int64_t kMaxRows = 1 << 18;                 // input rows per call
constexpr int64_t kMaxBlocks = kMaxRows / wk::dev::kRowsPerBlock;
static_assert(kMaxBlocks <= (1 << wk::dev::kGroupShift), "one k2u group sum per call");

constexpr size_t al(size_t x) { return (x + 255) & ~(size_t)255; }
// byte layout of the scratch array
constexpr size_t kOffFlags = 0;       // err (int, 16 B), the group's sums (output rows, slices)
constexpr size_t kOffDeg = al(kOffFlags + 32);
constexpr size_t kOffOff = al(kOffDeg + 4 * kMaxRows);
constexpr size_t kOffBlkSum = al(kOffOff + 4 * kMaxRows);
constexpr size_t kScratchBytes = al(kOffBlkSum + 8 * kMaxBlocks);

__device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

}  // namespace

using namespace wk;

int wk::noalloc_prepare(unsigned char **scratch) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) return cuda_fail(e == cudaSuccess ? cudaErrorInvalidSymbol : e,
                                                 "noalloc: cudaGetSymbolAddress");
    if ((e = (cudaError_t)dev::preload_k2u_kernels()) != cudaSuccess) return cuda_fail(e, "noalloc: kernel load");
    *scratch = static_cast<unsigned char *>(p);
    return WK_OK;
}

extern "C" int wk_known_to_unknown_noalloc(wk_ctx *ctx, const int32_t *hist, int64_t rows, int32_t cols,
                                           int64_t start, int32_t direction, int32_t predict, int32_t *out,
                                           int64_t out_capacity, int64_t *out_rows) {
    if (!ctx || !out_rows || rows < 0 || cols < 1 || (rows > 0 && !hist) || out_capacity < 0 ||
        (out_capacity > 0 && !out))
        return set_error(WK_EINVAL, "known_to_unknown_noalloc: bad arguments");
    *out_rows = 0;
    if (!ctx->store) return set_error(WK_ENOSTORE, "known_to_unknown_noalloc: no store built");
    if (ctx->device < 0) return set_error(WK_EDEVICE, "known_to_unknown_noalloc: host-only context");
    if (ctx->store->pool)
        return set_error(WK_EINVAL, "known_to_unknown_noalloc: needs a resident store (paging loads segments)");
    if (predict < 1 || predict > ctx->store->hs->num_ids || (direction != WK_DIR_IN && direction != WK_DIR_OUT))
        return set_error(WK_EINVAL, "known_to_unknown_noalloc: bad predicate %d / direction %d", predict, direction);
    if (start >= 0 || -start > cols)
        return set_error(WK_EINVAL, "known_to_unknown_noalloc: start %lld is not a bound column", (long long)start);
    if (rows > kMaxRows)
        return set_error(WK_EINVAL, "known_to_unknown_noalloc: %lld input rows exceed the maximum of %lld",
                         (long long)rows, (long long)kMaxRows);
    // the expansion kernel writes whole output rows as 16 B vectors
    if (((uintptr_t)out & 15u) != 0 || ((uintptr_t)hist & 3u) != 0)
        return set_error(WK_EINVAL, "known_to_unknown_noalloc: out must be 16 B aligned and hist 4 B aligned");
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    if (rows == 0) return WK_OK;
    unsigned char *sc = ctx->noalloc_scratch;   // looked up when the context was made
    if (!sc) return set_error(WK_EDEVICE, "known_to_unknown_noalloc: the context has no scratch address");
    int *err = reinterpret_cast<int *>(sc + kOffFlags);
    unsigned long long *gsum = reinterpret_cast<unsigned long long *>(sc + kOffFlags) + 2;
    uint32_t *deg = reinterpret_cast<uint32_t *>(sc + kOffDeg);
    uint32_t *off = reinterpret_cast<uint32_t *>(sc + kOffOff);
    unsigned long long *blk_sum = reinterpret_cast<unsigned long long *>(sc + kOffBlkSum);

    const PredView pv = ctx->store->views[(size_t)predict];
    const int scol = (int)(-start - 1);
    cudaStream_t s = ctx->stream;
    if ((e = cudaMemsetAsync(sc + kOffFlags, 0, 32, s)) != cudaSuccess) return cuda_fail(e, "noalloc: clear flags");
    // kMaxRows input rows are one group: its two sums are the op's totals
    dev::launch_k2u_count(hist, rows, cols, scol, (uint32_t)direction, pv, deg, off, blk_sum, gsum, err, false,
                          nullptr, 0, ctx->sms, s);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "noalloc: count launch");
    ctx->launches += 1;
    if ((e = cudaMemcpyAsync(ctx->h_scal, sc + kOffFlags, 32, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return cuda_fail(e, "noalloc: totals");
    if (ctx->h_scal[0] & 1ull)
        return set_error(WK_EDEVICE, "known_to_unknown_noalloc: corrupt overflow chain in the store");
    const int64_t R_out = (int64_t)ctx->h_scal[2];
    *out_rows = R_out;
    if (ctx->h_scal[0] & 2ull)
        return set_error(WK_EOVERFLOW, "known_to_unknown_noalloc: 1024 consecutive input rows expand to 2^31 rows or more");
    if (R_out == 0) return WK_OK;
    // R_out * (cols + 1) > out_capacity, without forming a product that could overflow
    const int64_t width = (int64_t)cols + 1;
    if (R_out > out_capacity / width)
        return set_error(WK_EOVERFLOW,
                         "known_to_unknown_noalloc: output needs %lld rows of %lld int32 elements, capacity is %lld "
                         "(*out_rows holds the row count)",
                         (long long)R_out, (long long)width, (long long)out_capacity);
    dev::GroupTable gt;
    gt.n = 1;
    gt.out[0] = 0ull;
    gt.sl[0] = 0u;
    gt.out[1] = ctx->h_scal[2];
    // the slices of at most 256 blocks: each block has ceil((count + 3) / 8192)
    // of them with count below 2^31, so fewer than 2^26 in all
    gt.sl[1] = (unsigned int)ctx->h_scal[3];
    dev::launch_k2u_expand(hist, rows, cols, pv.edges, deg, off, blk_sum, gsum, gt, ctx->h_scal[3], out, s);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "noalloc: expand launch");
    ctx->launches += 1;
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail(e, "noalloc: sync");
    return WK_OK;
}
