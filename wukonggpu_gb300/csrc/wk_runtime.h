// Host runtime state behind the C ABI.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <climits>
#include <map>
#include <memory>
#include <vector>

#include "wk_internal.h"
#include "wk_kernels.h"

namespace wk {

int cuda_fail(cudaError_t e, const char *what);

// growable device buffer (grows by 1.5x, never shrinks); freed when it goes
// out of scope (the device it was allocated on must be current then)
struct DevBuf {
    void *ptr = nullptr;
    size_t cap = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
    int reserve(size_t nbytes);
    void release();
    template <class T> T *as() const { return static_cast<T *>(ptr); }
};

// The device copy of the store: either fully resident (one bucket array and
// one edge array) or paged per id through a fixed device pool
// (ShardManager, core/shard_manager.hpp:44-557).
struct DeviceStore {
    struct Resident {
        bool resident = false;
        uint64_t off = 0, bytes = 0, last_use = 0;
        uint32_t uses = 0;   // requests since load or the last halving (eviction by frequency)
        cudaEvent_t ev = nullptr;   // completion of the segment's copy
    };
    int device = 0;
    std::unique_ptr<HostStore> hs;
    std::shared_ptr<Stats> stats;   // built on first use by the planner
    std::vector<PredView> views;    // per id
    uint64_t device_bytes = 0;
    // resident mode
    void *d_buckets = nullptr;
    int32_t *d_edges = nullptr;
    uint32_t *d_rowptr = nullptr;
    // paged mode
    void *pool = nullptr;
    uint64_t pool_bytes = 0, clock = 0;
    std::map<uint64_t, uint64_t> free_list;   // offset -> size
    std::vector<Resident> res;
    int64_t loads = 0, evictions = 0, requests = 0, hits = 0, compactions = 0;
    uint64_t bytes_loaded = 0;

    ~DeviceStore();
    int upload_resident();
    int init_paged(uint64_t budget);
    uint64_t seg_bytes(int id) const;
    bool pool_alloc(uint64_t need, uint64_t *off);
    void pool_free(uint64_t off, uint64_t n);
    uint64_t pool_free_bytes() const;
    int compact(cudaStream_t use_st, cudaStream_t copy_st);
    int ensure(int id, const std::vector<int> &protect, const std::vector<int> &avoid, cudaStream_t copy_st,
               cudaStream_t use_st, cudaEvent_t use_ready, bool may_evict = true);
};

}  // namespace wk

struct wk_ctx {
    int device = 0;                  // -1: host-only context (store image, statistics, planner)
    int sms = 0;                     // the device's SM count
    wk_config cfg{};
    cudaStream_t stream = nullptr;   // op stream
    cudaStream_t side = nullptr;     // segment prefetch stream
    cudaEvent_t use_ready = nullptr;
    std::shared_ptr<wk::DeviceStore> store;

    wk::DevBuf hbuf[2];              // ping-pong history buffers (core/rcache.hpp:87-88)
    // scratch of the two-pass ops
    wk::DevBuf deg, off, mask, blk_sum, blk_nz;
    // k2u: two alternating sums buffers, each a 16 B header (the op's error
    // flags) and 16 B per group of 256 input blocks; a count kernel adds into
    // one and clears the other for the next op
    wk::DevBuf gsum;
    int64_t gs_groups = 0;           // groups per buffer
    int gs_par = 0;                  // the buffer the next count kernel adds into
    int64_t gs_used[2] = {0, 0};     // groups written into each buffer since it was cleared
    // pinned, device-mapped host words: [0] the sequence number of the last
    // count kernel that published, then a copy of its sums buffer from [2]
    unsigned long long *h_gs = nullptr;
    unsigned long long *h_gs_dev = nullptr;   // its device address
    size_t h_gs_bytes = 0;
    unsigned long long pub_seq = 0;  // the last count kernel's sequence number
    wk::DevBuf dscal;                // [0] error flags, [8..32) totals
    // wk_history_partition: rows per (owner, tile) and their scan's block
    // sums, and the parts' bounds (grown on demand, kept for the next call)
    wk::DevBuf part_cnt, part_scan, part_bound;
    unsigned long long *h_scal = nullptr;   // pinned mirror of the totals

    // timing
    bool timing = false;
    std::vector<cudaEvent_t> tev;
    std::vector<int> tmain;          // index of kernel pairs that are the op's main kernel
    int tn = 0;
    wk_op_stats last{};
    std::vector<wk_op_stats> qstats;   // every op of the last wk_execute, while timing
    int64_t launches = 0;
    int64_t row_limit = INT64_MAX;   // wk_set_row_limit
    cudaEvent_t tm0 = nullptr, tm1 = nullptr;   // wk_timer_begin / wk_timer_end

    // query-level state (segment cache protection / prefetch): segments that
    // must stay (the current step's and the prefetched one), and the segments
    // the query's remaining steps use, evicted only when nothing else can be
    std::vector<int> protect, query_rest;

    // injected allocation failures still to come (wk_ctx_inject_alloc_failure)
    std::atomic<int> inject_alloc_fail{0};

    // the no-allocation entry point's scratch array on this device, resolved
    // when the context is made (wk_noalloc.cu)
    unsigned char *noalloc_scratch = nullptr;

    ~wk_ctx();
};

namespace wk {
// The device address of the no-allocation entry point's scratch array on the
// current device, after loading the kernels that entry point launches, so
// that no later call loads a module or takes device memory (wk_noalloc.cu).
int noalloc_prepare(unsigned char **scratch);

// Reserve a context's per-op scratch (per-row degree/offset/mask, per-block
// counts and look-back words) for steps of up to `rows` input rows.
int reserve_op_scratch(wk_ctx *ctx, int64_t rows);
}  // namespace wk
