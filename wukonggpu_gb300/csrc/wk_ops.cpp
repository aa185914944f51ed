// The per-pattern ops and the step dispatcher.
//
//   wk_known_to_unknown  <-> RCache::known_to_unknown  (core/rcache.hpp:232-414)
//   wk_known_to_known    <-> RCache::known_to_known    (core/rcache.hpp:417-612)
//   wk_known_to_const    <-> RCache::known_to_const    (core/rcache.hpp:614-809)
//   wk_index_to_unknown  <-> RCache::index_to_unknown  (core/rcache.hpp:811-962)
//   wk_const_to_unknown  <-> Engine::const_to_unknown  (core/engine.hpp:96-122)
//   wk_execute           <-> GPU_Engine::execute_one_step / execute_request
//                            (core/gpu_engine.hpp:395-526)
//
// Differences from the reference, none of which changes a result row:
// each op needs at most one host synchronisation (to size the k2u output);
// k2k/k2c need none before their last kernel; a missing key yields an empty
// adjacency instead of the reference GPU's out-of-bounds read of slot -1
// (core/gpu_hash.cu:276-277); tables are not limited to 20 columns or to
// GPU_MAX_ELEM elements; errors are returned, never asserted.
#include "wk_runtime.h"

#include <algorithm>
#include <cstring>

using namespace wk;

namespace {

enum { KIND_K2U = 0, KIND_K2K = 1, KIND_K2C = 2, KIND_I2U = 3, KIND_C2U = 4 };

inline bool is_tpid(int64_t id) { return id > 1 && id < WK_VID_BASE; }   // core/gstore.hpp:111

int check_ctx(wk_ctx *ctx, wk_history *h, const char *what) {
    if (!ctx || !h) return set_error(WK_EINVAL, "%s: null argument", what);
    if (!ctx->store) return set_error(WK_ENOSTORE, "%s: no store built", what);
    if (ctx->device < 0) return set_error(WK_EDEVICE, "%s: host-only context", what);
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    return WK_OK;
}

int check_pid(wk_ctx *ctx, int64_t pid, int32_t dir, const char *what) {
    if (pid < 1 || pid > ctx->store->hs->num_ids)
        return set_error(WK_EINVAL, "%s: predicate %lld outside [1,%d]", what, (long long)pid, ctx->store->hs->num_ids);
    if (dir != WK_DIR_IN && dir != WK_DIR_OUT) return set_error(WK_EINVAL, "%s: direction %d", what, dir);
    return WK_OK;
}

// ---- per-op timing: a begin/end CUDA event pair around every kernel on the
// op stream, so host gaps between kernels are never counted
struct OpClock {
    wk_ctx *ctx;
    explicit OpClock(wk_ctx *c) : ctx(c) {
        ctx->tn = 0;
        ctx->tmain.clear();
        ctx->last = wk_op_stats{};
    }
    int record() {
        if (!ctx->timing) return WK_OK;
        if ((int)ctx->tev.size() <= ctx->tn) {
            cudaEvent_t ev;
            cudaError_t e = cudaEventCreate(&ev);
            if (e != cudaSuccess) return cuda_fail(e, "timing event");
            ctx->tev.push_back(ev);
        }
        cudaError_t e = cudaEventRecord(ctx->tev[(size_t)ctx->tn++], ctx->stream);
        return e == cudaSuccess ? WK_OK : cuda_fail(e, "timing record");
    }
    int begin() { return record(); }
    int end(bool is_main) {   // after the kernel's launch
        ++ctx->launches;
        ++ctx->last.kernels;
        if (!ctx->timing) return WK_OK;
        if (is_main) ctx->tmain.push_back(ctx->tn - 1);   // begin event of this pair
        return record();
    }
    // call after the stream has been synchronised
    void finish() {
        if (!ctx->timing) return;
        double tot = 0.0, main = 0.0;
        size_t m = 0;   // tmain is ascending
        for (int i = 0; i + 1 < ctx->tn; i += 2) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, ctx->tev[(size_t)i], ctx->tev[(size_t)i + 1]);
            tot += ms;
            if (m < ctx->tmain.size() && ctx->tmain[m] == i) {
                main += ms;
                ++m;
            }
        }
        ctx->last.ms = tot;
        ctx->last.ms_main = main;
        float span = 0.f;
        if (ctx->tn >= 2) cudaEventElapsedTime(&span, ctx->tev[0], ctx->tev[(size_t)ctx->tn - 1]);
        ctx->last.span_ms = span;
    }
};

int launch_check(const char *what) {
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? WK_OK : cuda_fail(e, what);
}

// output buffer: the ping-pong partner of the input
wk::DevBuf &out_buf(wk_ctx *ctx, const wk_history *h) {
    return (h->data == ctx->hbuf[0].ptr) ? ctx->hbuf[1] : ctx->hbuf[0];
}

int ensure_seg(wk_ctx *ctx, int id, PredView *pv) {
    DeviceStore &ds = *ctx->store;
    if (ds.pool) {
        std::vector<int> prot = ctx->protect;
        prot.push_back(id);
        int st = ds.ensure(id, prot, ctx->query_rest, ctx->stream, ctx->stream, nullptr);
        if (st) return st;
    }
    *pv = ds.views[(size_t)id];
    return WK_OK;
}

// Wait until the publish kernel of sequence number seq has written its copy
// into ctx->h_gs.  The wait ends with the stream's work: the stream is polled
// every 4096 reads of the word (a few microseconds; no clock is read, as a
// clock read can enter the kernel and cost the thread its core), and a stream
// that has finished (or failed) without the number there is an error.
int wait_published(wk_ctx *ctx, unsigned long long seq) {
    for (unsigned int i = 1;; ++i) {
        if (__atomic_load_n(ctx->h_gs, __ATOMIC_ACQUIRE) == seq) return WK_OK;
        if ((i & 4095u) != 0u) continue;
        const cudaError_t e = cudaStreamQuery(ctx->stream);
        if (e == cudaErrorNotReady) continue;
        if (e != cudaSuccess) return cuda_fail(e, "op sync");
        if (__atomic_load_n(ctx->h_gs, __ATOMIC_ACQUIRE) == seq) return WK_OK;
        return set_error(WK_EDEVICE, "op finished without publishing its totals");
    }
}

int fail_corrupt(wk_ctx *ctx) {
    cudaMemsetAsync(ctx->dscal.ptr, 0, 8, ctx->stream);
    return set_error(WK_EDEVICE, "probe found an overflow chain longer than the segment's overflow area (corrupt store)");
}

}  // namespace

namespace {
// The k2u sums buffers for ops of up to `groups` groups: zero when allocated
// (both), then each count kernel clears the buffer it does not add into.
int reserve_gsum(wk_ctx *ctx, int64_t groups) {
    if (groups <= ctx->gs_groups) return WK_OK;
    const int64_t want = std::max(groups, ctx->gs_groups + ctx->gs_groups / 2);
    const size_t buf_bytes = 16 + (size_t)want * 16;
    int st = ctx->gsum.reserve(2 * buf_bytes);
    if (st) return st;
    cudaError_t e = cudaMemsetAsync(ctx->gsum.ptr, 0, ctx->gsum.cap, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(e, "k2u: clear group sums");
    // every publish into the old copy has been waited for
    if (ctx->h_gs) cudaFreeHost(ctx->h_gs);
    ctx->h_gs = ctx->h_gs_dev = nullptr;
    ctx->h_gs_bytes = 0;
    e = cudaHostAlloc((void **)&ctx->h_gs, 16 + buf_bytes, cudaHostAllocMapped);
    if (e == cudaSuccess) {
        std::memset(ctx->h_gs, 0, 16 + buf_bytes);   // no sequence number yet
        e = cudaHostGetDevicePointer((void **)&ctx->h_gs_dev, ctx->h_gs, 0);
    }
    if (e != cudaSuccess) {
        if (ctx->h_gs) cudaFreeHost(ctx->h_gs);
        ctx->h_gs = ctx->h_gs_dev = nullptr;
        ctx->gs_groups = 0;
        return cuda_fail(e, "k2u: pinned group sums");
    }
    ctx->h_gs_bytes = 16 + buf_bytes;
    ctx->gs_groups = want;
    ctx->gs_par = 0;
    ctx->gs_used[0] = ctx->gs_used[1] = 0;
    return WK_OK;
}

unsigned long long *gsum_buffer(wk_ctx *ctx, int par) {
    return ctx->gsum.as<unsigned long long>() + (size_t)par * (size_t)(2 + 2 * ctx->gs_groups);
}
}  // namespace

int wk::reserve_op_scratch(wk_ctx *ctx, int64_t rows) {
    if (!ctx || rows < 0) return set_error(WK_EINVAL, "reserve_op_scratch: bad arguments");
    if (ctx->device < 0) return WK_OK;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    const int64_t nblk = (rows + dev::kRowsPerBlock - 1) / dev::kRowsPerBlock + 1;
    int st;
    if ((st = ctx->deg.reserve((size_t)rows * 4)) || (st = ctx->off.reserve((size_t)rows * 4)) ||
        (st = ctx->mask.reserve((size_t)((rows + 31) / 32) * 4)) || (st = ctx->blk_sum.reserve((size_t)nblk * 8)) ||
        (st = ctx->blk_nz.reserve((size_t)nblk * 4)) ||
        (st = reserve_gsum(ctx, (nblk + (1 << dev::kGroupShift) - 1) >> dev::kGroupShift)))
        return st;
    return WK_OK;
}

namespace {

// An op's device-buffer reservation.  A context given injected allocation
// failures (wk_ctx_inject_alloc_failure) fails its next ones with WK_ENOMEM
// here, as a failed cudaMalloc inside DevBuf::reserve would.
int take(wk_ctx *ctx, DevBuf &b, size_t bytes) {
    if (ctx->inject_alloc_fail.load(std::memory_order_relaxed) > 0 &&
        ctx->inject_alloc_fail.fetch_sub(1, std::memory_order_relaxed) > 0)
        return set_error(WK_ENOMEM, "cudaMalloc: out of memory (injected allocation failure)");
    return b.reserve(bytes);
}

// zero the op totals (dscal[1..3]) before a first pass accumulates into them
int clear_totals(wk_ctx *ctx) {
    cudaError_t e = cudaMemsetAsync(ctx->dscal.as<unsigned long long>() + 1, 0, 24, ctx->stream);
    return e == cudaSuccess ? WK_OK : cuda_fail(e, "clear totals");
}

// two-pass k2u (count -> host adds up the group sums -> expand)
int op_k2u(wk_ctx *ctx, wk_history *h, int scol, uint32_t pid, uint32_t dir) {
    const int C = h->col_num;
    const int64_t R = h->size / C;
    OpClock clk(ctx);
    ctx->last.kind = KIND_K2U;
    ctx->last.rows_in = R;
    ctx->last.cols_in = C;
    PredView pv;
    int st = ensure_seg(ctx, (int)pid, &pv);
    if (st) return st;
    DevBuf &ob = out_buf(ctx, h);
    if (R == 0) {
        if ((st = take(ctx, ob, 16))) return st;
        h->data = ob.as<int32_t>();
        h->size = 0;
        h->col_num = C + 1;
        h->step++;
        return WK_OK;
    }
    const int64_t nblk = (R + dev::kRowsPerBlock - 1) / dev::kRowsPerBlock;
    const int64_t groups = (nblk + (1 << dev::kGroupShift) - 1) >> dev::kGroupShift;
    if ((st = take(ctx, ctx->deg, (size_t)R * 4)) || (st = take(ctx, ctx->off, (size_t)R * 4)) ||
        (st = take(ctx, ctx->blk_sum, (size_t)nblk * 8)) || (st = reserve_gsum(ctx, groups)))
        return st;
    // a functional direction (at most one neighbour per vertex) expands as a
    // compaction; if a row hits an index list (vertex 0) the op reruns unspecialised
    bool func = pv.func[dir] != 0u && C + 1 <= 8;
    int errf = 0;
    unsigned long long *gs = nullptr;
    for (;;) {
        const int par = ctx->gs_par;
        gs = gsum_buffer(ctx, par);
        if ((st = clk.begin())) return st;
        // the op's error flags and group sums come to the host through pinned
        // memory (a one-CTA kernel behind the count); the host adds up the totals
        const dev::Publish pub{gs, ctx->h_gs_dev, 2 + 2 * groups, ++ctx->pub_seq};
        dev::launch_k2u_count(h->data, R, C, scol, dir, pv, ctx->deg.as<uint32_t>(), ctx->off.as<uint32_t>(),
                              ctx->blk_sum.as<unsigned long long>(), gs + 2, reinterpret_cast<int *>(gs), func,
                              gsum_buffer(ctx, par ^ 1), 2 + 2 * ctx->gs_used[par ^ 1], ctx->sms, ctx->stream);
        if ((st = launch_check("k2u count")) || (st = clk.end(false))) return st;
        // outside the count's timing events: the op's device span counts it,
        // the count kernel's time does not
        dev::launch_publish(pub, ctx->stream);
        if ((st = launch_check("k2u publish"))) return st;
        ++ctx->launches;
        ++ctx->last.kernels;
        ctx->gs_par = par ^ 1;
        ctx->gs_used[par ^ 1] = 0;
        ctx->gs_used[par] = groups;
        if ((st = wait_published(ctx, pub.seq))) return st;
        errf = (int)(ctx->h_gs[2] & 0xffffffffull);
        if (!(func && (errf & 8))) break;
        func = false;   // the next count adds into the other, cleared buffer
    }
    if (errf & 1)
        return set_error(WK_EDEVICE, "probe found an overflow chain longer than the segment's overflow area (corrupt store)");
    if (errf & 2) return set_error(WK_EOVERFLOW, "k2u: 1024 consecutive input rows expand to 2^31 rows or more");
    // the op totals, and the groups' prefixes for the expansion
    dev::GroupTable gt;
    gt.n = groups <= dev::kTableGroups ? (int)groups : 0;
    unsigned long long rows_out = 0ull, slices = 0ull;
    for (int64_t g = 0; g < groups; ++g) {
        if (gt.n) {
            gt.out[g] = rows_out;
            gt.sl[g] = (unsigned int)slices;
        }
        rows_out += ctx->h_gs[4 + 2 * g];
        slices += ctx->h_gs[5 + 2 * g];
    }
    if (slices >> 32) gt.n = 0;   // not reached: a slice holds up to 8192 of the output rows
    if (gt.n) {
        gt.out[gt.n] = rows_out;
        gt.sl[gt.n] = (unsigned int)slices;
    }
    const int64_t R_out = (int64_t)rows_out;
    if (R_out > ctx->row_limit)
        return set_error(WK_EOVERFLOW, "k2u: %lld output rows exceed the context's row limit %lld", (long long)R_out,
                         (long long)ctx->row_limit);
    ctx->last.rows_out = R_out;
    ctx->last.alg_bytes = 4 * R * C + 16 * R + 4 * R_out + 4 * R_out * (C + 1);
    if (R_out == 0) {
        if ((st = take(ctx, ob, 16))) return st;
    } else {
        if ((st = take(ctx, ob, (size_t)R_out * (C + 1) * 4))) return st;
        if ((st = clk.begin())) return st;
        if (func)
            dev::launch_k2u_expand_func(h->data, R, C, ctx->deg.as<int32_t>(), ctx->blk_sum.as<unsigned long long>(),
                                        gs + 2, gt, slices, ob.as<int32_t>(), ctx->stream);
        else
            dev::launch_k2u_expand(h->data, R, C, pv.edges, ctx->deg.as<uint32_t>(), ctx->off.as<uint32_t>(),
                                   ctx->blk_sum.as<unsigned long long>(), gs + 2, gt, slices, ob.as<int32_t>(),
                                   ctx->stream);
        if ((st = launch_check("k2u expand")) || (st = clk.end(true))) return st;
        if (ctx->timing) {
            cudaError_t e = cudaStreamSynchronize(ctx->stream);
            if (e != cudaSuccess) return cuda_fail(e, "k2u sync");
        }
    }
    clk.finish();
    h->data = ob.as<int32_t>();
    h->size = R_out * (C + 1);
    h->col_num = C + 1;
    h->step++;
    return WK_OK;
}

// two-pass k2k / k2c (probe + membership -> filtered copy); the output is
// sized by the input, so the host reads the totals only at the end
int op_filter(wk_ctx *ctx, wk_history *h, int scol, int ecol, int32_t end_const, uint32_t pid, uint32_t dir) {
    const int C = h->col_num;
    const int64_t R = h->size / C;
    OpClock clk(ctx);
    ctx->last.kind = ecol >= 0 ? KIND_K2K : KIND_K2C;
    ctx->last.rows_in = R;
    ctx->last.cols_in = C;
    PredView pv;
    int st = ensure_seg(ctx, (int)pid, &pv);
    if (st) return st;
    DevBuf &ob = out_buf(ctx, h);
    if (R == 0) {
        if ((st = take(ctx, ob, 16))) return st;
        h->data = ob.as<int32_t>();
        h->size = 0;
        h->step++;
        return WK_OK;
    }
    const int64_t nblk = (R + dev::kRowsPerBlock - 1) / dev::kRowsPerBlock;
    const int64_t groups = (nblk + (1 << dev::kGroupShift) - 1) >> dev::kGroupShift;
    if ((st = take(ctx, ctx->mask, (size_t)((R + 31) / 32) * 4)) || (st = take(ctx, ctx->blk_nz, (size_t)nblk * 4)) ||
        (st = reserve_gsum(ctx, groups)) || (st = take(ctx, ob, (size_t)R * C * 4)) || (st = clear_totals(ctx)))
        return st;
    unsigned long long *tot = ctx->dscal.as<unsigned long long>() + 1;
    int *err = ctx->dscal.as<int>();
    // the block counts' group sums go to one of the two sums buffers k2u uses,
    // and the probe clears the other
    const int par = ctx->gs_par;
    unsigned long long *gs = gsum_buffer(ctx, par) + 2;
    if ((st = clk.begin())) return st;
    dev::launch_filter_probe(h->data, R, C, scol, ecol, end_const, dir, pv, ctx->mask.as<uint32_t>(),
                             ctx->blk_nz.as<unsigned int>(), gs, gsum_buffer(ctx, par ^ 1),
                             2 + 2 * ctx->gs_used[par ^ 1], tot, err, ctx->stream);
    if ((st = launch_check("filter probe"))) return st;
    ctx->gs_par = par ^ 1;
    ctx->gs_used[par ^ 1] = 0;
    ctx->gs_used[par] = groups;
    if ((st = clk.end(true)) || (st = clk.begin())) return st;
    dev::launch_filter_write(h->data, R, C, ctx->mask.as<uint32_t>(), ctx->blk_nz.as<unsigned int>(), gs,
                             ob.as<int32_t>(), ctx->stream);
    if ((st = launch_check("filter write")) || (st = clk.end(false))) return st;
    // the error word and totals come to the host through pinned memory, as a
    // k2u op's group sums do
    const dev::Publish pub{ctx->dscal.as<unsigned long long>(), ctx->h_gs_dev, 4, ++ctx->pub_seq};
    dev::launch_publish(pub, ctx->stream);
    if ((st = launch_check("filter publish"))) return st;
    ++ctx->launches;
    ++ctx->last.kernels;
    if ((st = wait_published(ctx, pub.seq))) return st;
    if (ctx->h_gs[2] & 0xffffffffull) return fail_corrupt(ctx);
    const int64_t E = (int64_t)ctx->h_gs[3];
    const int64_t nz = (int64_t)ctx->h_gs[4];
    clk.finish();
    ctx->last.rows_out = nz;
    ctx->last.alg_bytes = 4 * R * C + 16 * R + 4 * E + 4 * nz * C;
    h->data = ob.as<int32_t>();
    h->size = nz * C;
    h->step++;
    return WK_OK;
}

// one adjacency list -> one-column table (index or constant start)
int op_list(wk_ctx *ctx, wk_history *h, uint64_t vid, uint32_t pid, uint32_t dir, int kind) {
    OpClock clk(ctx);
    ctx->last.kind = kind;
    ctx->last.rows_in = 1;
    const HostStore &hs = *ctx->store->hs;
    const int32_t *e = nullptr;
    const uint64_t deg = hs.lookup(vid, pid, dir, &e);
    DevBuf &ob = out_buf(ctx, h);
    int st;
    if ((st = take(ctx, ob, (size_t)deg * 4 + 16))) return st;
    if (deg) {
        PredView pv;
        if ((st = ensure_seg(ctx, (int)pid, &pv))) return st;
        const uint64_t off = (uint64_t)(e - (hs.edges + hs.segs[pid].edge_off));
        if ((st = clk.begin())) return st;
        dev::launch_copy_list(pv.edges + off, (int64_t)deg, ob.as<int32_t>(), ctx->stream);
        if ((st = launch_check("list copy")) || (st = clk.end(true))) return st;
        if (ctx->timing) {
            cudaError_t ce = cudaStreamSynchronize(ctx->stream);
            if (ce != cudaSuccess) return cuda_fail(ce, "list sync");
        }
    }
    clk.finish();
    ctx->last.rows_out = (int64_t)deg;
    ctx->last.alg_bytes = 16 + 8 * (int64_t)deg;
    h->data = ob.as<int32_t>();
    h->size = (int64_t)deg;
    h->col_num = 1;
    h->step++;
    return WK_OK;
}

int known_col(const wk_history *h, int64_t v, const char *what, int *col) {
    if (v >= 0 || -v > h->col_num)
        return set_error(WK_EINVAL, "%s: %lld is not a bound variable (col_num %d)", what, (long long)v, h->col_num);
    *col = (int)(-v - 1);
    return WK_OK;
}

int check_table(const wk_history *h, const char *what) {
    if (h->col_num <= 0 || h->size < 0 || h->size % h->col_num != 0 || (h->size > 0 && !h->data))
        return set_error(WK_EINVAL, "%s: malformed history (size %lld, col_num %d)", what, (long long)h->size,
                         h->col_num);
    return WK_OK;
}

}  // namespace

extern "C" int wk_known_to_unknown(wk_ctx *ctx, wk_history *h, int64_t start, int32_t direction, int32_t predict) {
    int st, scol;
    if ((st = check_ctx(ctx, h, "known_to_unknown")) || (st = check_table(h, "known_to_unknown")) ||
        (st = check_pid(ctx, predict, direction, "known_to_unknown")) ||
        (st = known_col(h, start, "known_to_unknown start", &scol)))
        return st;
    return op_k2u(ctx, h, scol, (uint32_t)predict, (uint32_t)direction);
}

extern "C" int wk_known_to_known(wk_ctx *ctx, wk_history *h, int64_t start, int32_t direction, int32_t predict,
                                 int64_t end) {
    int st, scol, ecol;
    if ((st = check_ctx(ctx, h, "known_to_known")) || (st = check_table(h, "known_to_known")) ||
        (st = check_pid(ctx, predict, direction, "known_to_known")) ||
        (st = known_col(h, start, "known_to_known start", &scol)) ||
        (st = known_col(h, end, "known_to_known end", &ecol)))
        return st;
    return op_filter(ctx, h, scol, ecol, 0, (uint32_t)predict, (uint32_t)direction);
}

extern "C" int wk_known_to_const(wk_ctx *ctx, wk_history *h, int64_t start, int32_t direction, int32_t predict,
                                 int64_t end) {
    int st, scol;
    if ((st = check_ctx(ctx, h, "known_to_const")) || (st = check_table(h, "known_to_const")) ||
        (st = check_pid(ctx, predict, direction, "known_to_const")) ||
        (st = known_col(h, start, "known_to_const start", &scol)))
        return st;
    if (end < 0 || end > 0x7fffffffll) return set_error(WK_EINVAL, "known_to_const: end %lld is not a constant", (long long)end);
    return op_filter(ctx, h, scol, -1, (int32_t)end, (uint32_t)predict, (uint32_t)direction);
}

extern "C" int wk_index_to_unknown(wk_ctx *ctx, wk_history *h, int32_t index_vertex, int32_t direction) {
    int st;
    if ((st = check_ctx(ctx, h, "index_to_unknown")) || (st = check_pid(ctx, index_vertex, direction, "index_to_unknown")))
        return st;
    if (h->col_num != 0) return set_error(WK_EINVAL, "index_to_unknown: history already has %d columns", h->col_num);
    return op_list(ctx, h, 0, (uint32_t)index_vertex, (uint32_t)direction, KIND_I2U);
}

extern "C" int wk_const_to_unknown(wk_ctx *ctx, wk_history *h, int64_t start, int32_t direction, int32_t predict) {
    int st;
    if ((st = check_ctx(ctx, h, "const_to_unknown")) || (st = check_pid(ctx, predict, direction, "const_to_unknown")))
        return st;
    if (h->col_num != 0) return set_error(WK_EINVAL, "const_to_unknown: history already has %d columns", h->col_num);
    if (start < WK_VID_BASE || start > 0xffffffffll)
        return set_error(WK_EINVAL, "const_to_unknown: start %lld is not a vertex id", (long long)start);
    return op_list(ctx, h, (uint64_t)start, (uint32_t)predict, (uint32_t)direction, KIND_C2U);
}

// GPU_Engine::execute_one_step dispatch (core/gpu_engine.hpp:395-467) with the
// variable typing of request_or_reply::variable_type (core/query.hpp:141-149).
static int vtype(int64_t v, int col_num) {   // 0 known, 1 unknown, 2 const
    if (v >= 0) return 2;
    return (-v > col_num) ? 1 : 0;
}

extern "C" int wk_execute(wk_ctx *ctx, const int64_t *cmd, int32_t n, wk_history *h, int64_t *step_rows) {
    if (!ctx || !cmd || !h || n <= 0) return set_error(WK_EINVAL, "wk_execute: bad arguments");
    if (!ctx->store) return set_error(WK_ENOSTORE, "wk_execute: no store");
    if (ctx->device < 0) return set_error(WK_EDEVICE, "wk_execute: host-only context");
    wk_history_init(h);
    ctx->protect.clear();
    ctx->query_rest.clear();
    ctx->qstats.clear();
    DeviceStore &ds = *ctx->store;
    int st = WK_OK;
    for (int i = 0; i < n && st == WK_OK; ++i) {
        const int64_t start = cmd[i * 4], pid = cmd[i * 4 + 1], d = cmd[i * 4 + 2], end = cmd[i * 4 + 3];
        if (ds.pool) {
            // the segments of steps i.. (an index start's segment is its index id)
            ctx->query_rest.clear();
            for (int k = i; k < n; ++k) {
                const int64_t sid = (k == 0 && is_tpid(cmd[0])) ? cmd[0] : cmd[k * 4 + 1];
                if (sid >= 1 && sid <= ds.hs->num_ids) ctx->query_rest.push_back((int)sid);
            }
        }
        if (ds.pool && ctx->cfg.enable_prefetch && i + 1 < n) {
            const int64_t np = cmd[(i + 1) * 4 + 1];
            const int64_t cp = (i == 0 && is_tpid(cmd[0])) ? cmd[0] : pid;
            if (np >= 1 && np <= ds.hs->num_ids && cp >= 1 && cp <= ds.hs->num_ids) {
                std::vector<int> prot{(int)cp, (int)np};
                ds.ensure((int)np, prot, ctx->query_rest, ctx->side, ctx->stream, ctx->use_ready, false);
                ctx->protect = prot;
            }
        }
        if (i == 0 && is_tpid(start)) {
            if (end != -1) return set_error(WK_EINVAL, "wk_execute: index pattern must bind variable -1");
            st = wk_index_to_unknown(ctx, h, (int32_t)start, (int32_t)d);
        } else {
            if (pid < 0) return set_error(WK_EINVAL, "wk_execute: variable predicates are not supported");
            const int ts = vtype(start, h->col_num), te = vtype(end, h->col_num);
            if (ts == 2 && te == 1) {
                if (h->col_num != 0 || end != -1)
                    return set_error(WK_EINVAL, "wk_execute: constant start must be the first pattern and bind -1");
                st = wk_const_to_unknown(ctx, h, start, (int32_t)d, (int32_t)pid);
            } else if (ts == 0 && te == 1) {
                if (-end - 1 != h->col_num)
                    return set_error(WK_EINVAL, "wk_execute: pattern %d binds %lld but the next column is %d", i,
                                     (long long)end, h->col_num);
                st = wk_known_to_unknown(ctx, h, start, (int32_t)d, (int32_t)pid);
            } else if (ts == 0 && te == 0) {
                st = wk_known_to_known(ctx, h, start, (int32_t)d, (int32_t)pid, end);
            } else if (ts == 0 && te == 2) {
                st = wk_known_to_const(ctx, h, start, (int32_t)d, (int32_t)pid, end);
            } else {
                return set_error(WK_EINVAL, "wk_execute: unsupported pattern shape at step %d (start %lld, end %lld)",
                                 i, (long long)start, (long long)end);
            }
        }
        if (st == WK_OK && step_rows) step_rows[i] = h->col_num ? h->size / h->col_num : 0;
        if (st == WK_OK && ctx->timing) ctx->qstats.push_back(ctx->last);
    }
    ctx->protect.clear();
    ctx->query_rest.clear();
    return st;
}

extern "C" int wk_ctx_inject_alloc_failure(wk_ctx *ctx, int32_t n) {
    if (!ctx || n < 0) return set_error(WK_EINVAL, "wk_ctx_inject_alloc_failure: bad arguments");
    ctx->inject_alloc_fail.store(n);
    return WK_OK;
}

extern "C" int wk_set_row_limit(wk_ctx *ctx, int64_t max_rows) {
    if (!ctx || max_rows < 0) return set_error(WK_EINVAL, "wk_set_row_limit: bad arguments");
    ctx->row_limit = max_rows ? max_rows : INT64_MAX;
    return WK_OK;
}
