// Host runtime behind the C ABI: contexts, the device store, the predicate
// segment cache, the per-pattern ops and the step dispatcher.
//
// Reference counterparts: RCache (core/rcache.hpp) for the ops and buffer
// ownership, ShardManager (core/shard_manager.hpp) for the segment cache,
// GPU_Engine::execute_one_step (core/gpu_engine.hpp:395-467) for dispatch.
#include "wk_runtime.h"

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>

namespace wk {

int cuda_fail(cudaError_t e, const char *what) {
    cudaGetLastError();
    return set_error(e == cudaErrorMemoryAllocation ? WK_ENOMEM : WK_EDEVICE, "%s: %s (%d)", what,
                     cudaGetErrorString(e), (int)e);
}

// ------------------------------------------------------------ DevBuf
int DevBuf::reserve(size_t nbytes) {
    if (nbytes <= cap) return WK_OK;
    size_t want = std::max(nbytes, cap + cap / 2);
    want = (want + 255) & ~(size_t)255;
    if (ptr) { cudaFree(ptr); ptr = nullptr; cap = 0; }
    cudaError_t e = cudaMalloc(&ptr, want);
    if (e != cudaSuccess) {
        ptr = nullptr;
        e = cudaMalloc(&ptr, (nbytes + 255) & ~(size_t)255);   // retry without slack
        if (e != cudaSuccess) { ptr = nullptr; return cuda_fail(e, "cudaMalloc"); }
        cap = (nbytes + 255) & ~(size_t)255;
        return WK_OK;
    }
    cap = want;
    return WK_OK;
}
void DevBuf::release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    cap = 0;
}

// ------------------------------------------------------- DeviceStore
DeviceStore::~DeviceStore() {
    if (d_buckets) cudaFree(d_buckets);
    if (d_rowptr) cudaFree(d_rowptr);
    if (d_edges) cudaFree(d_edges);
    if (pool) cudaFree(pool);
    for (auto &r : res)
        if (r.ev) cudaEventDestroy(r.ev);
}

static inline uint64_t align256(uint64_t x) { return (x + 255) & ~(uint64_t)255; }

int DeviceStore::upload_resident() {
    const uint64_t bbytes = hs->total_buckets * sizeof(Bucket), ebytes = hs->total_edges * 4,
                   rbytes = hs->total_rowptr * 4;
    cudaError_t e;
    if ((e = cudaMalloc(&d_buckets, bbytes ? bbytes : 16)) != cudaSuccess) { d_buckets = nullptr; return cuda_fail(e, "store upload (buckets)"); }
    if ((e = cudaMalloc(&d_edges, ebytes ? ebytes : 16)) != cudaSuccess) { d_edges = nullptr; return cuda_fail(e, "store upload (edges)"); }
    if ((e = cudaMalloc(&d_rowptr, rbytes ? rbytes : 16)) != cudaSuccess) { d_rowptr = nullptr; return cuda_fail(e, "store upload (offsets)"); }
    if (bbytes && (e = cudaMemcpy(d_buckets, hs->buckets, bbytes, cudaMemcpyHostToDevice)) != cudaSuccess)
        return cuda_fail(e, "store upload copy (buckets)");
    if (ebytes && (e = cudaMemcpy(d_edges, hs->edges, ebytes, cudaMemcpyHostToDevice)) != cudaSuccess)
        return cuda_fail(e, "store upload copy (edges)");
    if (rbytes && (e = cudaMemcpy(d_rowptr, hs->rowptr, rbytes, cudaMemcpyHostToDevice)) != cudaSuccess)
        return cuda_fail(e, "store upload copy (offsets)");
    views.assign((size_t)hs->num_ids + 1, PredView{});
    for (int id = 1; id <= hs->num_ids; ++id) {
        const PredSeg &sg = hs->segs[(size_t)id];
        views[(size_t)id] = make_view(sg, static_cast<const Bucket *>(d_buckets) + sg.bucket_off,
                                      d_rowptr + sg.rp_off, d_edges + sg.edge_off);
    }
    device_bytes = bbytes + ebytes + rbytes;
    return WK_OK;
}

int DeviceStore::init_paged(uint64_t budget) {
    cudaError_t e = cudaMalloc(&pool, budget);
    if (e != cudaSuccess) { pool = nullptr; return cuda_fail(e, "segment cache pool"); }
    pool_bytes = budget;
    free_list.clear();
    free_list[0] = budget;
    res.assign((size_t)hs->num_ids + 1, Resident());
    views.assign((size_t)hs->num_ids + 1, PredView{});
    device_bytes = budget;
    return WK_OK;
}

uint64_t DeviceStore::seg_bytes(int id) const {
    const PredSeg &sg = hs->segs[(size_t)id];
    return align256(sg.bucket_bytes()) + align256(sg.rowptr_bytes()) + align256(sg.edge_bytes());
}

bool DeviceStore::pool_alloc(uint64_t need, uint64_t *off) {
    for (auto it = free_list.begin(); it != free_list.end(); ++it) {
        if (it->second >= need) {
            *off = it->first;
            uint64_t rest = it->second - need, at = it->first + need;
            free_list.erase(it);
            if (rest) free_list[at] = rest;
            return true;
        }
    }
    return false;
}

void DeviceStore::pool_free(uint64_t off, uint64_t n) {
    auto it = free_list.emplace(off, n).first;
    // merge with the next range
    auto nx = std::next(it);
    if (nx != free_list.end() && it->first + it->second == nx->first) {
        it->second += nx->second;
        free_list.erase(nx);
    }
    // merge with the previous range
    if (it != free_list.begin()) {
        auto pv = std::prev(it);
        if (pv->first + pv->second == it->first) {
            pv->second += it->second;
            free_list.erase(it);
        }
    }
}

uint64_t DeviceStore::pool_free_bytes() const {
    uint64_t f = 0;
    for (auto &x : free_list) f += x.second;
    return f;
}

// Slide every resident segment down to the lowest offsets, in offset order,
// so that the free space becomes one range at the top of the pool.  Used when
// the pool's free bytes would hold a segment but no single free range does
// (segments kept resident, such as the current step's and the prefetched
// one, can split the free space).  Both streams are drained first, so no
// kernel or copy uses a segment while it moves; a move copies forward in
// chunks no longer than the distance moved, so no chunk overwrites bytes not
// yet copied.  The views of moved segments are updated.
int DeviceStore::compact(cudaStream_t use_st, cudaStream_t copy_st) {
    cudaError_t e;
    if ((e = cudaStreamSynchronize(copy_st)) != cudaSuccess || (e = cudaStreamSynchronize(use_st)) != cudaSuccess)
        return cuda_fail(e, "segment cache compaction (drain)");
    std::vector<int> ids;
    for (int v = 1; v <= hs->num_ids; ++v)
        if (res[(size_t)v].resident && res[(size_t)v].bytes) ids.push_back(v);
    std::sort(ids.begin(), ids.end(), [&](int a, int b) { return res[(size_t)a].off < res[(size_t)b].off; });
    char *base = static_cast<char *>(pool);
    uint64_t at = 0;
    for (int v : ids) {
        Resident &x = res[(size_t)v];
        if (x.off != at) {
            const uint64_t dist = x.off - at;   // > 0: segments never overlap and are visited in order
            for (uint64_t done = 0; done < x.bytes;) {
                const uint64_t c = std::min(dist, x.bytes - done);
                if ((e = cudaMemcpyAsync(base + at + done, base + x.off + done, c, cudaMemcpyDeviceToDevice,
                                         use_st)) != cudaSuccess)
                    return cuda_fail(e, "segment cache compaction (move)");
                done += c;
            }
            x.off = at;
            const PredSeg &sg = hs->segs[(size_t)v];
            char *sb = base + at;
            char *rb = sb + align256(sg.bucket_bytes());
            char *eb = rb + align256(sg.rowptr_bytes());
            views[(size_t)v] = make_view(sg, reinterpret_cast<const Bucket *>(sb), reinterpret_cast<const uint32_t *>(rb),
                                         reinterpret_cast<const int32_t *>(eb));
        }
        at += x.bytes;
    }
    if ((e = cudaStreamSynchronize(use_st)) != cudaSuccess) return cuda_fail(e, "segment cache compaction (sync)");
    free_list.clear();
    if (at < pool_bytes) free_list[at] = pool_bytes - at;
    ++compactions;
    return WK_OK;
}

// Make segment `id` resident (ShardManager::load_predicate,
// core/shard_manager.hpp:473-555).  Eviction never takes a protected segment.
// Like the reference, which evicts predicates outside the query first and the
// query's own last (evict_kcache_blocks / evict_vcache_blocks,
// core/shard_manager.hpp:130-295), it takes a segment that the query's
// remaining steps (`avoid`) use only when no other will do.  Among the rest it
// takes the least requested segment, the most recently used one on a tie:
// a mix that cycles through its queries then keeps a fixed set of segments
// instead of evicting each one just before it comes round again (least
// recently used would), and a skewed mix keeps its frequent segments.
// Request counts halve every 4096 requests, so past popularity fades.  The
// copy is issued on `copy_st`; `use_st` is made to wait for it.  With
// may_evict false (a prefetch) the segment loads only into free space: no
// segment is evicted or moved, and the step's own request loads it otherwise.
int DeviceStore::ensure(int id, const std::vector<int> &protect, const std::vector<int> &avoid, cudaStream_t copy_st,
                        cudaStream_t use_st, cudaEvent_t use_ready, bool may_evict) {
    if (!pool) return WK_OK;
    Resident &r = res[(size_t)id];
    if (!may_evict && r.resident) return WK_OK;   // a prefetch of a resident segment: nothing to do
    ++clock;
    if (may_evict) {   // a step's request (a prefetch is not one)
        ++requests;
        if ((requests & 4095) == 0)
            for (Resident &x : res) x.uses >>= 1;
        if (r.uses < UINT32_MAX) ++r.uses;
    }
    if (r.resident) {
        ++hits;
        r.last_use = clock;
        if (r.ev && copy_st != use_st) {
            cudaError_t e = cudaStreamWaitEvent(use_st, r.ev, 0);
            if (e != cudaSuccess) return cuda_fail(e, "segment cache wait");
        }
        return WK_OK;
    }
    const PredSeg &sg = hs->segs[(size_t)id];
    const uint64_t need = seg_bytes(id);
    if (need == 0) { r.resident = true; r.last_use = clock; return WK_OK; }
    if (need > pool_bytes)
        return set_error(WK_ENOMEM, "segment cache: id %d needs %llu bytes, pool holds %llu", id,
                         (unsigned long long)need, (unsigned long long)pool_bytes);
    uint64_t off = 0;
    while (!pool_alloc(need, &off)) {
        if (!may_evict) return WK_OK;
        // free bytes enough but split into ranges: compact rather than evict
        if (pool_free_bytes() >= need) {
            int st = compact(use_st, copy_st);
            if (st) return st;
            continue;
        }
        int victim = -1;
        bool v_needed = true;
        uint32_t v_uses = 0;
        uint64_t v_last = 0;
        for (int v = 1; v <= hs->num_ids; ++v) {
            const Resident &x = res[(size_t)v];
            if (!x.resident || x.bytes == 0) continue;
            if (std::find(protect.begin(), protect.end(), v) != protect.end()) continue;
            const bool needed = std::find(avoid.begin(), avoid.end(), v) != avoid.end();
            // order: not needed by the query's remaining steps, fewer requests, more recent use
            const bool better = victim < 0 || (needed != v_needed ? !needed
                                                                  : (x.uses != v_uses ? x.uses < v_uses
                                                                                      : x.last_use > v_last));
            if (better) {
                victim = v;
                v_needed = needed;
                v_uses = x.uses;
                v_last = x.last_use;
            }
        }
        if (victim < 0)
            return set_error(WK_ENOMEM,
                             "segment cache: cannot fit id %d (%llu bytes) beside the protected segments "
                             "(%llu bytes free; the budget must hold the largest segments a query step and "
                             "its prefetch use at once)",
                             id, (unsigned long long)need, (unsigned long long)pool_free_bytes());
        Resident &x = res[(size_t)victim];
        pool_free(x.off, x.bytes);
        x.resident = false;
        x.bytes = 0;
        views[(size_t)victim] = PredView{};
        ++evictions;
    }
    // a copy on a side stream must not overwrite memory that kernels already
    // queued on the use stream may still read
    cudaError_t e;
    if (copy_st != use_st && use_ready) {
        if ((e = cudaEventRecord(use_ready, use_st)) != cudaSuccess) return cuda_fail(e, "segment cache record");
        if ((e = cudaStreamWaitEvent(copy_st, use_ready, 0)) != cudaSuccess) return cuda_fail(e, "segment cache wait");
    }
    char *base = static_cast<char *>(pool) + off;
    const uint64_t bb = sg.bucket_bytes(), eb = sg.edge_bytes(), rb = sg.rowptr_bytes();
    if (bb && (e = cudaMemcpyAsync(base, hs->buckets + sg.bucket_off, bb, cudaMemcpyHostToDevice, copy_st)) != cudaSuccess)
        return cuda_fail(e, "segment cache copy (buckets)");
    char *rbase = base + align256(bb);
    if (rb && (e = cudaMemcpyAsync(rbase, hs->rowptr + sg.rp_off, rb, cudaMemcpyHostToDevice, copy_st)) != cudaSuccess)
        return cuda_fail(e, "segment cache copy (offsets)");
    char *ebase = rbase + align256(rb);
    if (eb && (e = cudaMemcpyAsync(ebase, hs->edges + sg.edge_off, eb, cudaMemcpyHostToDevice, copy_st)) != cudaSuccess)
        return cuda_fail(e, "segment cache copy (edges)");
    if (!r.ev && (e = cudaEventCreateWithFlags(&r.ev, cudaEventDisableTiming)) != cudaSuccess) {
        r.ev = nullptr;
        return cuda_fail(e, "segment cache event");
    }
    if ((e = cudaEventRecord(r.ev, copy_st)) != cudaSuccess) return cuda_fail(e, "segment cache record");
    if (copy_st != use_st && (e = cudaStreamWaitEvent(use_st, r.ev, 0)) != cudaSuccess)
        return cuda_fail(e, "segment cache wait");
    r.resident = true;
    r.off = off;
    r.bytes = need;
    r.last_use = clock;
    views[(size_t)id] = make_view(sg, reinterpret_cast<const Bucket *>(base), reinterpret_cast<const uint32_t *>(rbase),
                                  reinterpret_cast<const int32_t *>(ebase));
    ++loads;
    bytes_loaded += bb + rb + eb;
    return WK_OK;
}

}  // namespace wk

using namespace wk;

// ================================================================ context
static int make_current(wk_ctx *ctx) {
    if (ctx->device < 0) return set_error(WK_EDEVICE, "host-only context: no device work");
    cudaError_t e = cudaSetDevice(ctx->device);
    return e == cudaSuccess ? WK_OK : cuda_fail(e, "cudaSetDevice");
}

wk_ctx::~wk_ctx() {
    if (device < 0) return;
    cudaSetDevice(device);
    if (stream) cudaStreamSynchronize(stream);
    for (auto &b : hbuf) b.release();
    deg.release(); off.release(); mask.release(); blk_sum.release(); blk_nz.release();
    dscal.release();
    part_cnt.release();
    part_scan.release();
    part_bound.release();
    if (h_scal) cudaFreeHost(h_scal);
    if (h_gs) cudaFreeHost(h_gs);
    for (auto &e : tev) cudaEventDestroy(e);
    if (use_ready) cudaEventDestroy(use_ready);
    if (tm0) cudaEventDestroy(tm0);
    if (tm1) cudaEventDestroy(tm1);
    if (side) cudaStreamDestroy(side);
    if (stream) cudaStreamDestroy(stream);
}

extern "C" void wk_config_default(wk_config *cfg) {
    if (!cfg) return;
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->enable_prefetch = 1;
}

extern "C" int wk_device_count(int *count) {
    if (!count) return set_error(WK_EINVAL, "wk_device_count: null");
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess) { *count = 0; return cuda_fail(e, "cudaGetDeviceCount"); }
    *count = n;
    return WK_OK;
}

extern "C" int wk_ctx_create(const wk_config *cfg_in, wk_ctx **out) {
    if (!out) return set_error(WK_EINVAL, "wk_ctx_create: null out");
    *out = nullptr;
    wk_config cfg;
    if (cfg_in) cfg = *cfg_in;
    else wk_config_default(&cfg);
    if (cfg.device < 0) {   // host-only: store image, statistics and planner, no device work
        wk_ctx *hctx = new wk_ctx();
        hctx->device = -1;
        hctx->cfg = cfg;
        *out = hctx;
        return WK_OK;
    }
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n <= 0) return cuda_fail(e == cudaSuccess ? cudaErrorNoDevice : e, "wk_ctx_create: no CUDA device");
    if (cfg.device < 0 || cfg.device >= n) return set_error(WK_EINVAL, "wk_ctx_create: device %d of %d", cfg.device, n);
    wk_ctx *ctx = new wk_ctx();
    ctx->device = cfg.device;
    ctx->cfg = cfg;
    int st;
    if ((st = make_current(ctx)) != WK_OK) { delete ctx; return st; }
    if ((e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&ctx->use_ready, cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaHostAlloc((void **)&ctx->h_scal, 64, cudaHostAllocDefault)) != cudaSuccess) {
        int r = cuda_fail(e, "wk_ctx_create");
        delete ctx;
        return r;
    }
    if ((e = cudaDeviceGetAttribute(&ctx->sms, cudaDevAttrMultiProcessorCount, ctx->device)) != cudaSuccess) {
        int r = cuda_fail(e, "wk_ctx_create: SM count");
        delete ctx;
        return r;
    }
    if ((st = wk::noalloc_prepare(&ctx->noalloc_scratch)) != WK_OK) { delete ctx; return st; }
    if ((st = ctx->dscal.reserve(4096)) != WK_OK) { delete ctx; return st; }
    if ((e = cudaMemset(ctx->dscal.ptr, 0, 4096)) != cudaSuccess) { int r = cuda_fail(e, "wk_ctx_create"); delete ctx; return r; }
    const int64_t hc = cfg.history_capacity > 0 ? cfg.history_capacity : (16ll << 20);
    for (auto &b : ctx->hbuf)
        if ((st = b.reserve((size_t)hc * 4)) != WK_OK) { delete ctx; return st; }
    *out = ctx;
    return WK_OK;
}

extern "C" int wk_ctx_destroy(wk_ctx *ctx) {
    delete ctx;
    return WK_OK;
}

extern "C" int wk_sync(wk_ctx *ctx) {
    if (!ctx) return set_error(WK_EINVAL, "wk_sync: null ctx");
    if (ctx->device < 0) return WK_OK;
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    return e == cudaSuccess ? WK_OK : cuda_fail(e, "wk_sync");
}

namespace wk {
int build_store_device(wk_ctx *ctx, const int32_t *s, const int32_t *p, const int32_t *o, int64_t n, int32_t num_ids,
                       HostStore **out);
}

static int store_build(wk_ctx *ctx, const int32_t *s, const int32_t *p, const int32_t *o, int64_t n,
                       int32_t num_ids, bool on_device) {
    int st;
    if (ctx->device >= 0 && (st = make_current(ctx))) return st;
    HostStore *hs = nullptr;
    if (on_device && n > 0) {
        if (n < 0 || !s || !p || !o || num_ids < 1 || num_ids >= WK_VID_BASE)
            return set_error(WK_EINVAL, "store build: bad arguments (n=%lld, num_ids=%d)", (long long)n, num_ids);
        st = build_store_device(ctx, s, p, o, n, num_ids, &hs);
    } else {
        st = build_host_store(s, p, o, n, num_ids, &hs);
    }
    if (st != WK_OK) return st;
    auto ds = std::make_shared<DeviceStore>();
    ds->hs.reset(hs);
    ds->device = ctx->device;
    if (ctx->device < 0) {   // host-only: no device copy
        ctx->store = ds;
        return WK_OK;
    }
    if (ctx->cfg.cache_budget_mb > 0) st = ds->init_paged((uint64_t)ctx->cfg.cache_budget_mb << 20);
    else st = ds->upload_resident();
    if (st != WK_OK) return st;
    ctx->store = ds;
    return WK_OK;
}

extern "C" int wk_store_build(wk_ctx *ctx, const int32_t *s, const int32_t *p, const int32_t *o,
                              int64_t n, int32_t num_ids) {
    if (!ctx) return set_error(WK_EINVAL, "wk_store_build: null ctx");
    return store_build(ctx, s, p, o, n, num_ids, false);
}

extern "C" int wk_store_build_device(wk_ctx *ctx, const int32_t *s, const int32_t *p, const int32_t *o,
                                     int64_t n, int32_t num_ids) {
    if (!ctx) return set_error(WK_EINVAL, "wk_store_build_device: null ctx");
    if (ctx->device < 0) return set_error(WK_EDEVICE, "wk_store_build_device: host-only context");
    if (n >= (int64_t)0xffffffffll) return set_error(WK_EINVAL, "wk_store_build_device: %lld triples exceed 2^32 - 1",
                                                     (long long)n);
    return store_build(ctx, s, p, o, n, num_ids, true);
}

extern "C" int wk_store_digest(wk_ctx *ctx, uint64_t *digest) {
    if (!ctx || !digest) return set_error(WK_EINVAL, "wk_store_digest: null");
    if (!ctx->store) return set_error(WK_ENOSTORE, "wk_store_digest: no store");
    *digest = ctx->store->hs->digest();
    return WK_OK;
}

extern "C" int wk_store_build_graph(wk_ctx *ctx, const wk_graph *g) {
    if (!g) return set_error(WK_EINVAL, "wk_store_build_graph: null graph");
    return wk_store_build(ctx, wk_graph_s(g), wk_graph_p(g), wk_graph_o(g), wk_graph_size(g), wk_graph_num_ids(g));
}

extern "C" int wk_ctx_share_store(wk_ctx *ctx, wk_ctx *owner) {
    if (!ctx || !owner || !owner->store) return set_error(WK_EINVAL, "wk_ctx_share_store: bad arguments");
    if (ctx->device != owner->device) return set_error(WK_EINVAL, "wk_ctx_share_store: different devices");
    if (owner->store->pool) return set_error(WK_EINVAL, "wk_ctx_share_store: a paged store cannot be shared");
    ctx->store = owner->store;
    return WK_OK;
}

extern "C" int wk_store_get_info(wk_ctx *ctx, wk_store_info *info) {
    if (!ctx || !info) return set_error(WK_EINVAL, "wk_store_get_info: null");
    if (!ctx->store) return set_error(WK_ENOSTORE, "wk_store_get_info: no store");
    const HostStore *hs = ctx->store->hs.get();
    info->num_keys = (int64_t)hs->total_keys;
    info->num_edges = (int64_t)hs->total_edges;
    info->key_bytes = (int64_t)(hs->total_buckets * sizeof(Bucket) + hs->total_rowptr * 4);
    info->edge_bytes = (int64_t)hs->total_edges * 4;
    info->overflow_buckets = (int64_t)hs->total_over;
    info->device_bytes = (int64_t)ctx->store->device_bytes;
    info->num_ids = hs->num_ids;
    info->paged = ctx->store->pool ? 1 : 0;
    info->cache_loads = ctx->store->loads;
    info->cache_evictions = ctx->store->evictions;
    info->cache_bytes_loaded = (int64_t)ctx->store->bytes_loaded;
    info->cache_requests = ctx->store->requests;
    info->cache_hits = ctx->store->hits;
    info->cache_compactions = ctx->store->compactions;
    info->dense_dirs = 0;
    for (int id = 1; id <= hs->num_ids; ++id)
        info->dense_dirs += (hs->segs[(size_t)id].dn[0] ? 1 : 0) + (hs->segs[(size_t)id].dn[1] ? 1 : 0);
    return WK_OK;
}

extern "C" int wk_store_get_edges(wk_ctx *ctx, int64_t vid, int32_t pid, int32_t dir, int32_t *out,
                                  int64_t cap, int64_t *deg) {
    if (!ctx || !deg || (cap > 0 && !out)) return set_error(WK_EINVAL, "wk_store_get_edges: null");
    if (!ctx->store) return set_error(WK_ENOSTORE, "wk_store_get_edges: no store");
    if (vid < 0 || vid > 0xffffffffll || (dir != 0 && dir != 1)) return set_error(WK_EINVAL, "wk_store_get_edges: bad key");
    const int32_t *e = nullptr;
    uint64_t d = ctx->store->hs->lookup((uint64_t)vid, (uint32_t)pid, (uint32_t)dir, &e);
    *deg = (int64_t)d;
    if (e && cap > 0) std::memcpy(out, e, (size_t)std::min<int64_t>(cap, (int64_t)d) * 4);
    return WK_OK;
}

extern "C" int wk_store_pred_stats(wk_ctx *ctx, int32_t id, int64_t *triples, int64_t *subjects, int64_t *objects) {
    if (!ctx || !triples || !subjects || !objects) return set_error(WK_EINVAL, "wk_store_pred_stats: null");
    if (!ctx->store) return set_error(WK_ENOSTORE, "wk_store_pred_stats: no store");
    const HostStore *hs = ctx->store->hs.get();
    if (id < 1 || id > hs->num_ids) return set_error(WK_EINVAL, "wk_store_pred_stats: id %d out of range", id);
    const PredSeg &sg = hs->segs[(size_t)id];
    *triples = sg.triples;
    *subjects = sg.subjects;
    *objects = sg.objects;
    return WK_OK;
}

extern "C" int wk_store_seg_layout(wk_ctx *ctx, int32_t id, wk_seg_layout *out) {
    if (!ctx || !out) return set_error(WK_EINVAL, "wk_store_seg_layout: null");
    if (!ctx->store) return set_error(WK_ENOSTORE, "wk_store_seg_layout: no store");
    const HostStore *hs = ctx->store->hs.get();
    if (id < 1 || id > hs->num_ids) return set_error(WK_EINVAL, "wk_store_seg_layout: id %d out of range", id);
    const PredSeg &sg = hs->segs[(size_t)id];
    std::memset(out, 0, sizeof(*out));
    out->keys = (int64_t)sg.nkeys;
    out->edges = (int64_t)sg.nedges;
    out->main_buckets = (int32_t)sg.nmain;
    out->overflow_buckets = (int32_t)sg.nover;
    for (int d = 0; d < 2; ++d) {
        out->dense[d] = sg.dn[d] ? 1 : 0;
        out->functional[d] = sg.maxdeg[d] <= 1u ? 1 : 0;
        out->bitmap[d] = sg.bn[d] ? 1 : 0;
        out->max_degree[d] = (int32_t)sg.maxdeg[d];
    }
    out->device_bytes = (int64_t)ctx->store->seg_bytes(id);
    return WK_OK;
}

extern "C" int wk_enable_timing(wk_ctx *ctx, int enable) {
    if (!ctx) return set_error(WK_EINVAL, "wk_enable_timing: null");
    ctx->timing = enable != 0;
    return WK_OK;
}

extern "C" int wk_last_op_stats(wk_ctx *ctx, wk_op_stats *st) {
    if (!ctx || !st) return set_error(WK_EINVAL, "wk_last_op_stats: null");
    *st = ctx->last;
    return WK_OK;
}

extern "C" int wk_query_op_stats(wk_ctx *ctx, wk_op_stats *st, int32_t cap, int32_t *n) {
    if (!ctx || !n || cap < 0 || (cap > 0 && !st)) return set_error(WK_EINVAL, "wk_query_op_stats: bad arguments");
    const int32_t k = (int32_t)std::min<size_t>((size_t)cap, ctx->qstats.size());
    for (int32_t i = 0; i < k; ++i) st[i] = ctx->qstats[(size_t)i];
    *n = (int32_t)ctx->qstats.size();
    return WK_OK;
}

extern "C" int64_t wk_kernel_launches(wk_ctx *ctx) { return ctx ? ctx->launches : 0; }

extern "C" int wk_host_alloc(int64_t bytes, void **out) {
    if (!out || bytes < 0) return set_error(WK_EINVAL, "wk_host_alloc: bad arguments");
    *out = nullptr;
    cudaError_t e = cudaHostAlloc(out, (size_t)(bytes ? bytes : 1), cudaHostAllocPortable);
    if (e != cudaSuccess) { *out = nullptr; return cuda_fail(e, "wk_host_alloc"); }
    return WK_OK;
}

extern "C" int wk_host_free(void *p) {
    if (!p) return WK_OK;
    cudaError_t e = cudaFreeHost(p);
    return e == cudaSuccess ? WK_OK : cuda_fail(e, "wk_host_free");
}

extern "C" int wk_timer_begin(wk_ctx *ctx) {
    if (!ctx) return set_error(WK_EINVAL, "wk_timer_begin: null");
    cudaError_t e;
    for (auto *ev : {&ctx->tm0, &ctx->tm1})
        if (!*ev && (e = cudaEventCreate(ev)) != cudaSuccess) { *ev = nullptr; return cuda_fail(e, "timer event"); }
    e = cudaEventRecord(ctx->tm0, ctx->stream);
    return e == cudaSuccess ? WK_OK : cuda_fail(e, "timer record");
}

extern "C" int wk_timer_end(wk_ctx *ctx, double *ms) {
    if (!ctx || !ms || !ctx->tm0) return set_error(WK_EINVAL, "wk_timer_end: no interval begun");
    cudaError_t e = cudaEventRecord(ctx->tm1, ctx->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(ctx->tm1);
    float f = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&f, ctx->tm0, ctx->tm1);
    if (e != cudaSuccess) return cuda_fail(e, "timer");
    *ms = f;
    return WK_OK;
}

extern "C" void wk_history_init(wk_history *h) {
    if (h) std::memset(h, 0, sizeof(*h));
}

extern "C" int wk_history_upload(wk_ctx *ctx, wk_history *h, const int32_t *host, int64_t size, int32_t col_num) {
    if (!ctx || !h || size < 0 || (size > 0 && !host) || col_num < 0 || (col_num == 0 && size != 0) ||
        (col_num > 0 && size % col_num != 0))
        return set_error(WK_EINVAL, "wk_history_upload: bad arguments");
    int st = make_current(ctx);
    if (st) return st;
    DevBuf &b = ctx->hbuf[0];
    if ((st = b.reserve((size_t)size * 4 + 16)) != WK_OK) return st;
    if (size) {
        cudaError_t e = cudaMemcpyAsync(b.ptr, host, (size_t)size * 4, cudaMemcpyHostToDevice, ctx->stream);
        if (e != cudaSuccess) return cuda_fail(e, "wk_history_upload");
    }
    h->data = static_cast<int32_t *>(b.ptr);
    h->size = size;
    h->col_num = col_num;
    h->step = 0;
    return WK_OK;
}

extern "C" int wk_history_download(wk_ctx *ctx, const wk_history *h, int32_t *host, int64_t cap) {
    if (!ctx || !h || (h->size > 0 && (!host || cap < h->size)))
        return set_error(WK_EINVAL, "wk_history_download: bad arguments (cap %lld < size %lld)",
                         (long long)cap, h ? (long long)h->size : 0ll);
    int st = make_current(ctx);
    if (st) return st;
    cudaError_t e;
    if (h->size > 0 && (e = cudaMemcpyAsync(host, h->data, (size_t)h->size * 4, cudaMemcpyDeviceToHost, ctx->stream)) != cudaSuccess)
        return cuda_fail(e, "wk_history_download");
    if ((e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess) return cuda_fail(e, "wk_history_download sync");
    return WK_OK;
}
