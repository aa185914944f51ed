/*
 * wukong_gpu.h - C ABI of the GB300-native graph-exploration operator library.
 *
 * The operator surface is the per-triple-pattern API of the Wukong+G GPU engine:
 * a history table of int32 vertex-id rows (row-major, `cols` columns) goes in
 * together with the pattern's start column, predicate id, direction and a
 * constant or variable end, and the expanded history comes out.  The library
 * owns the device store (packed-key hash buckets + per-predicate edge
 * segments on HBM) and the device history buffers, exactly as the reference's
 * RCache owns its store and ping-pong result buffers.
 *
 * Conventions (all entry points):
 *   - return an int status: WK_OK (0) or one of the negative WK_E* codes below;
 *     nothing aborts.  wk_last_error() gives a one-line message for the
 *     calling thread's last failure.
 *   - variable ids follow the reference encoding (core/query.hpp:141-154):
 *     a value >= 0 is a constant vertex id, a value < 0 is variable -v-1
 *     (column index); direction IN = 0, OUT = 1 (core/gstore.hpp:107).
 *   - vertex ids are >= 2^17, predicate and type ids are in [1, 2^17)
 *     (datagen/generate_data.cpp:88-98); pid 1 is rdf:type.
 *   - a wk_ctx is used by one host thread at a time (the reference's
 *     one-query-at-a-time GPU lock, core/gpu.hpp:49-61); several contexts may
 *     share one device store through wk_ctx_share_store.
 *
 * No torch or C++ types appear in these signatures.
 */
#ifndef WUKONG_GPU_H
#define WUKONG_GPU_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
enum {
    WK_OK        = 0,
    WK_EINVAL    = -1,  /* bad argument or unsupported pattern shape        */
    WK_ENOMEM    = -2,  /* device or pinned-host allocation failed          */
    WK_ETIMEDOUT = -3,  /* a bounded device-side wait gave up               */
    WK_EDEVICE   = -4,  /* CUDA runtime error (no device, launch failure)   */
    WK_ENOSTORE  = -5,  /* no store has been built/attached to the context  */
    WK_EOVERFLOW = -6,  /* a result exceeded a stated capacity               */
    WK_ECANCELED = -7,  /* a server request was cancelled before it ran      */
    WK_EREJECTED = -8   /* a server request was refused at admission         */
};

enum { WK_DIR_IN = 0, WK_DIR_OUT = 1 };
enum { WK_PREDICATE_ID = 0, WK_TYPE_ID = 1 };

typedef struct wk_ctx wk_ctx;

/*
 * Device history table, the counterpart of request_or_reply's
 * gpu_history_ptr / gpu_history_table_size / col_num (core/query.hpp:63-65,
 * :160-174).  `data` is a device pointer owned by the context (never free it);
 * `size` counts int32 elements (rows * col_num), as in the reference.
 */
typedef struct {
    int32_t *data;      /* device pointer, row-major int32               */
    int64_t  size;      /* number of int32 elements = rows * col_num     */
    int32_t  col_num;   /* number of bound columns                       */
    int32_t  step;      /* number of patterns executed so far            */
} wk_history;

/* Context configuration (the global_gpu_* knobs of core/config.hpp:66-78). */
typedef struct {
    int32_t  device;                 /* CUDA device ordinal; -1 = host-only context
                                        (store image, statistics, planner)          */
    int32_t  cache_budget_mb;        /* 0 = whole store resident; > 0 = page
                                        predicate segments from pinned host memory
                                        into a device pool of this many MiB
                                        (core/shard_manager.hpp)                    */
    int32_t  enable_prefetch;        /* page the next pattern's predicate on a side
                                        stream (global_gpu_enable_pipeline)         */
    int32_t  reserved;
    int64_t  history_capacity;       /* initial int32 capacity of each ping-pong
                                        history buffer; 0 = 16 Mi elements          */
} wk_config;

/* ------------------------------------------------------------- context */
void        wk_config_default(wk_config *cfg);
int         wk_ctx_create(const wk_config *cfg, wk_ctx **out);
int         wk_ctx_destroy(wk_ctx *ctx);
const char *wk_last_error(void);
const char *wk_status_str(int status);
int         wk_device_count(int *count);

/* -------------------------------------------------------------- store
 * Build the device store from ID-form triples (s, p, o), as the reference
 * loader does from its id_* files (core/dgraph.hpp:268-330,
 * core/gstore.hpp:600-978): duplicate triples are removed, every non-type
 * triple is stored in both directions, rdf:type triples (p == 1) become the
 * per-vertex type list plus the type index, and every predicate gets a
 * subject index [0|p|IN] and an object index [0|p|OUT].  Adjacency lists are
 * ascending by neighbour id.  `num_ids` is the number of predicate+type ids
 * (ids 1..num_ids are valid).
 */
int wk_store_build(wk_ctx *ctx, const int32_t *s, const int32_t *p, const int32_t *o,
                   int64_t n_triples, int32_t num_ids);
/* As wk_store_build, with the whole build on the context's device: the
 * checks, the sorts of the triples by (s, o) and by (o, s), deduplication,
 * list cutting, index lists, dense offsets and neighbour arrays, presence
 * bitmaps and bucket insertion (wk_build.cu); the host does per-id
 * arithmetic only and receives the finished image.  The image is
 * byte-identical to wk_store_build's.  Needs a device context and n < 2^32 - 1. */
int wk_store_build_device(wk_ctx *ctx, const int32_t *s, const int32_t *p, const int32_t *o,
                          int64_t n, int32_t num_ids);
/* FNV-1a digest of the host store image (metadata, buckets, edges, offsets
 * arrays): equal for two builds exactly when their images are identical. */
int wk_store_digest(wk_ctx *ctx, uint64_t *digest);
/* Attach the store of `owner` to `ctx` (read-only sharing, one copy on HBM). */
int wk_ctx_share_store(wk_ctx *ctx, wk_ctx *owner);

typedef struct {
    int64_t num_keys;        /* packed (vid,pid,dir) keys                     */
    int64_t num_edges;       /* int32 edge entries incl. index lists          */
    int64_t key_bytes;       /* bytes of key storage: hash buckets and dense  */
                             /* offsets arrays (all predicates)               */
    int64_t edge_bytes;      /* bytes of edge segments (all predicates)       */
    int64_t overflow_buckets;/* indirect (overflow) buckets in use            */
    int64_t device_bytes;    /* bytes of the store resident on the device     */
    int32_t num_ids;
    int32_t paged;           /* 1 if predicate segments are paged (cache mode)*/
    int64_t cache_loads;     /* segment loads (H2D) so far, paged mode        */
    int64_t cache_evictions; /* segment evictions so far, paged mode          */
    int64_t cache_bytes_loaded;
    int64_t dense_dirs;      /* (id, direction) pairs stored as dense offsets */
                             /* arrays instead of hashed keys                 */
    int64_t cache_requests;  /* segment lookups by ops and prefetches, paged  */
    int64_t cache_hits;      /* ... of which found the segment resident       */
    int64_t cache_compactions; /* times the pool was compacted (free bytes    */
                             /* enough for a segment but split into ranges)   */
} wk_store_info;
int wk_store_get_info(wk_ctx *ctx, wk_store_info *info);

/* Host-side lookup in the store's host image (no device work): the
 * counterpart of GStore::get_edges_global (core/gstore.hpp:1129).  Writes at
 * most `cap` neighbours to `out` and the true degree to *deg. */
int wk_store_get_edges(wk_ctx *ctx, int64_t vid, int32_t pid, int32_t dir,
                       int32_t *out, int64_t cap, int64_t *deg);

/* Per-predicate statistics from the built store (GStore::generate_statistic,
 * core/gstore.hpp:1010-1127): triples, distinct subjects, distinct objects
 * per id; for class ids the member count is returned in `subjects`. */
int wk_store_pred_stats(wk_ctx *ctx, int32_t id, int64_t *triples, int64_t *subjects,
                        int64_t *objects);

/* How one id's segment is laid out (this library's own HBM format; the
 * reference keeps every key in GStore's buckets, core/gstore.hpp:102-187):
 * per direction (index = WK_DIR_IN / WK_DIR_OUT), whether its vertex keys are
 * a dense offsets array, whether every vertex list holds at most one
 * neighbour (functional: a dense functional direction also keeps the
 * neighbour per id), and whether a hashed direction has a presence bitmap. */
typedef struct {
    int64_t keys;            /* keys of the id, hashed and dense               */
    int64_t edges;           /* int32 entries of its edge segment             */
    int32_t main_buckets, overflow_buckets;
    int32_t dense[2], functional[2], bitmap[2];
    int32_t max_degree[2];   /* longest vertex list (index lists excluded)    */
    int64_t device_bytes;    /* bytes the segment takes on the device (its    */
                             /* buckets, offsets arrays and edges, 256 B apart)*/
} wk_seg_layout;
int wk_store_seg_layout(wk_ctx *ctx, int32_t id, wk_seg_layout *out);

/* --------------------------------------------------- per-pattern ops
 * Counterparts of RCache::{known_to_unknown, known_to_known, known_to_const,
 * index_to_unknown} (core/rcache.hpp:232, :417, :614, :811) and of the
 * constant-start step (core/engine.hpp:96-122, done on the host by the
 * reference GPU engine at core/gpu_engine.hpp:171-189; here on the device).
 * Each op replaces h->data with a context-owned device buffer holding the
 * expanded history (ping-pong, like core/rcache.hpp:389-400), updates size and
 * col_num the way GPU_Engine does (core/gpu_engine.hpp:210-212), and bumps
 * h->step.  `start` / `end` are reference-encoded ids (negative = variable).
 */
int wk_known_to_unknown(wk_ctx *ctx, wk_history *h, int64_t start, int32_t direction,
                        int32_t predict);
int wk_known_to_known(wk_ctx *ctx, wk_history *h, int64_t start, int32_t direction,
                      int32_t predict, int64_t end);
int wk_known_to_const(wk_ctx *ctx, wk_history *h, int64_t start, int32_t direction,
                      int32_t predict, int64_t end);
int wk_index_to_unknown(wk_ctx *ctx, wk_history *h, int32_t index_vertex, int32_t direction);
int wk_const_to_unknown(wk_ctx *ctx, wk_history *h, int64_t start, int32_t direction,
                        int32_t predict);

/* known_to_unknown for callers that cannot allocate device memory while a
 * query runs (a host that calls the operator from inside its own allocator
 * or under a fixed device budget, a serving thread that must never enter
 * cudaMalloc/cudaFree).  No counterpart in the reference.  The caller passes
 * the input history (device, rows x cols int32) and an output buffer it owns
 * (out_capacity int32 elements, 16 B aligned; hist 4 B aligned, else
 * WK_EINVAL); *out_rows receives the output row count
 * (also when the output does not fit: WK_EOVERFLOW).  The call allocates
 * nothing: its scratch is one fixed device array inside the library (about
 * 2.1 MB), which wk_ctx_create loads on the context's device -- with the
 * kernels this call launches -- and looks up, so no call loads a module or
 * takes device memory; the array stays on that GPU until the process exits.
 * Limits: at most 262,144 input rows per call; the output is bounded by
 * out_capacity; needs a resident (unpaged) store.  Every call on a device
 * shares that array, so calls that overlap on the GPU race.  A context must
 * not outlive a reset of its device (the address it looked up would be
 * stale).  Returns after the output is written. */
int wk_known_to_unknown_noalloc(wk_ctx *ctx, const int32_t *hist, int64_t rows, int32_t cols,
                                int64_t start, int32_t direction, int32_t predict,
                                int32_t *out, int64_t out_capacity, int64_t *out_rows);

/* History transfer: upload a host table into the context's device buffer
 * (GPU::load_history_data, core/gpu.hpp:79-88) and download the current
 * table (the last-step D2H of core/rcache.hpp:402-408). */
int wk_history_upload(wk_ctx *ctx, wk_history *h, const int32_t *host, int64_t size,
                      int32_t col_num);
int wk_history_download(wk_ctx *ctx, const wk_history *h, int32_t *host, int64_t cap);
void wk_history_init(wk_history *h);

/* ------------------------------------------------------ fork-join across ranks
 * Split a table by the rank that owns each row's start vertex, the device
 * side of a fork-join step (RCache::generate_sub_query, core/rcache.hpp:
 * 964-1030, with calc_dispatched_position / history_dispatch,
 * core/gpu_hash.cu:698-790).  `start` is the bound variable of the next
 * pattern (column -start-1); a row goes to part value % nparts
 * (mymath::hash_mod, utils/mymath.hpp:55-59; values are vertex ids, >= 0).
 * On return *out holds the parts one after another, each in the input's
 * row order, in the ping-pong partner of the input's buffer, and
 * part_rows[0..nparts) their row counts.  1 <= nparts <= 256; fewer than
 * 2^32 - 1 rows.  `out` may be `in`. */
int wk_history_partition(wk_ctx *ctx, const wk_history *in, int64_t start, int32_t nparts,
                         int64_t *part_rows, wk_history *out);

/* Device-to-device transfers for a collective's buffers: copy the table of
 * *h to `dst` (cap int32 elements; WK_EINVAL when smaller than h->size), and
 * make *h a table of `size` elements in `col_num` columns copied from
 * `src`, in the context's first history buffer (h->step is kept).  Both
 * return after the copy is complete. */
int wk_history_to_device(wk_ctx *ctx, const wk_history *h, int32_t *dst, int64_t cap);
int wk_history_from_device(wk_ctx *ctx, wk_history *h, const int32_t *src, int64_t size, int32_t col_num);

/* ------------------------------------------------------ whole query
 * Execute every pattern of `cmd_chains` (n_patterns x {start, pid, dir, end},
 * core/query.hpp:68) with the step dispatch of GPU_Engine::execute_one_step
 * (core/gpu_engine.hpp:395-467), leaving the final table in *h.  When
 * `step_rows` is non-null it receives the row count after every step (the
 * true per-step cardinalities that the estimator trains on).
 */
int wk_execute(wk_ctx *ctx, const int64_t *cmd_chains, int32_t n_patterns, wk_history *h,
               int64_t *step_rows);

/* -------------------------------------------------- batched light queries
 * Many concurrent constant-start queries executed together: one persistent
 * launch per plan step over a packed multi-query history with per-query
 * offsets, captured once as a CUDA graph and replayed for every batch (the
 * batched counterpart of running GPU_Engine::execute_request once per query,
 * core/gpu_engine.hpp:471-526).  Every query's rows are exactly those it
 * produces alone.  Queries: 1..max_steps patterns, the first one
 * `<const> p d -1`, the others k2u / k2k / k2c; packed back to back in
 * cmd_chains with n_patterns[q] patterns each.  capacity_ints bounds every
 * step's packed table; a larger step returns WK_EOVERFLOW. */
typedef struct wk_batch wk_batch;
int wk_batch_create(wk_ctx *ctx, int32_t max_queries, int32_t max_steps, int64_t capacity_ints,
                    wk_batch **out);
int wk_batch_destroy(wk_batch *b);
int wk_batch_run(wk_batch *b, const int64_t *cmd_chains, const int32_t *n_patterns, int32_t nq,
                 int32_t use_graph);
/* Asynchronous form: launch on the batch's own stream, poll, wait (wait
 * reports WK_EOVERFLOW / WK_EDEVICE like wk_batch_run).  Two batches overlap
 * on the device. */
int wk_batch_launch(wk_batch *b, const int64_t *cmd_chains, const int32_t *n_patterns, int32_t nq,
                    int32_t use_graph);
int wk_batch_ready(wk_batch *b);
int wk_batch_wait(wk_batch *b);
/* Result of query q of the last run: rows, columns and its int32 offset in the packed result. */
int wk_batch_result(wk_batch *b, int32_t q, int64_t *rows, int32_t *cols, int64_t *int_offset);
/* The results of all nq queries of the last run at once (nq must be its
 * query count): rows, columns and int32 offsets, one entry per query. */
int wk_batch_layouts(wk_batch *b, int32_t nq, int64_t *rows, int32_t *cols, int64_t *int_offsets);
/* Copy the packed results of the last run to host memory (host may be NULL to get the size). */
int wk_batch_download(wk_batch *b, int32_t *host, int64_t cap, int64_t *total_ints);
/* Launch shape of the step kernels: persistent blocks per SM, input rows per
 * warp per tile, and the output size (ints) above which a row is written by a
 * whole warp instead of one thread. */
int wk_batch_set_tuning(wk_batch *b, int32_t blocks_per_sm, int32_t rows_per_warp, int32_t split_ints);
int wk_batch_get_tuning(wk_batch *b, int32_t *blocks_per_sm, int32_t *rows_per_warp, int32_t *split_ints);
/* Step form: 0 = three kernels per step (count, scan, write); 1 = one
 * cooperative persistent kernel per step whose blocks meet at two bounded
 * grid barriers (a wait that runs out fails the batch with WK_ETIMEDOUT).
 * wk_batch_get_fused returns the current form. */
int wk_batch_set_fused(wk_batch *b, int32_t fused);
int wk_batch_get_fused(wk_batch *b);
/* Threads per block of the step kernels: 128 or 256 (a tile is that many
 * warps' rows).  wk_batch_get_block_threads returns the current value. */
int wk_batch_set_block_threads(wk_batch *b, int32_t threads);
int wk_batch_get_block_threads(wk_batch *b);
/* Autotuner: time every candidate step form, block size and launch shape on these queries and keep the fastest. */
int wk_batch_autotune(wk_batch *b, const int64_t *cmd_chains, const int32_t *n_patterns, int32_t nq,
                      int32_t reps, double *best_ms);
int64_t wk_batch_kernel_launches(wk_batch *b);
/* The last wk_batch_autotune's best time (ms) of each step form: three
 * kernels per step, and one cooperative kernel per step; -1 where none of
 * that form ran (the device refused it, or no autotune yet). */
int wk_batch_autotune_forms(wk_batch *b, double *three_kernel_ms, double *one_kernel_ms);

/* ------------------------------------------- learned cardinality estimator
 * An MLP (48 features + 32-d predicate embedding -> 3 x 256 GELU -> 1) that
 * predicts log(1 + rows) after a plan step, trained and run by BF16
 * tensor-core kernels (FP32 accumulation, FP32 Adam over FP32 master
 * weights).  Parameters in one block: W1[256x80], W2[256x256], W3[256x256],
 * W4[1x256], b1[256], b2[256], b3[256], b4[64] (first used),
 * emb[(n_ids+1) x 32]. */
typedef struct wk_mlp wk_mlp;
int     wk_mlp_create(wk_ctx *ctx, int32_t n_ids, int32_t max_batch, uint64_t seed, wk_mlp **out);
int     wk_mlp_destroy(wk_mlp *m);
int64_t wk_mlp_num_params(wk_mlp *m);
int     wk_mlp_get_params(wk_mlp *m, float *host, int64_t n);
int     wk_mlp_set_params(wk_mlp *m, const float *host, int64_t n);
/* one forward + backward without an update: loss and every gradient */
int     wk_mlp_gradients(wk_mlp *m, const float *feats, const int32_t *pids, const float *target, int32_t n,
                         float *grads, float *loss);
int     wk_mlp_train(wk_mlp *m, const float *feats, const int32_t *pids, const float *target, int64_t n,
                     int32_t epochs, int32_t batch, float lr, uint64_t seed, float *last_loss);
int     wk_mlp_predict(wk_mlp *m, const float *feats, const int32_t *pids, int64_t n, float *out);
/* Features (n x 48) and embedding ids of every step of an executable plan;
 * true_rows (optional) = rows after each step, stats_est (optional) receives
 * the chained statistics estimate of the rows after each step. */
int     wk_featurize(wk_ctx *ctx, const int64_t *cmd_chains, int32_t n, const int64_t *true_rows, float *feats,
                     int32_t *pids, double *stats_est);
/* Held-out check: q-error = exp(|predicted - true|) in log(1 + rows) per
 * sample; the model is trusted while the 95th percentile is within
 * qerror_bound (>= 1).  A model starts trusted; an untrusted one makes the
 * learned planners fall back to the statistics planner (wk_plan). */
int     wk_mlp_validate(wk_mlp *m, const float *feats, const int32_t *pids, const float *target, int64_t n,
                        double qerror_bound, double *p95_qerror, int32_t *trusted);
int     wk_mlp_is_trusted(wk_mlp *m);
/* Plan by the model's predicted cardinalities: beam search over join orders,
 * cost = the sum of the predicted rows of every table the plan builds.  Same
 * output format as wk_plan (*n_out = 0 when no executable order exists).
 * With an untrusted model the statistics plan is returned (when wk_plan finds
 * one); *est_log_rows = log1p of the plan's cost. */
int     wk_plan_learned(wk_ctx *ctx, wk_mlp *m, const int64_t *cmd_in, int32_t n, int64_t *cmd_out,
                        int32_t *n_out, double *est_log_rows);

/* Learned plans of nq BGPs at once (every level of every query's search is
 * one model call).  cmd_in packs the queries (n_in[q] patterns each);
 * cmd_out must hold sum(n_in[q] + 1) patterns; n_out[q] = plan length.  Same
 * statistics fallback as wk_plan_learned. */
int     wk_plan_learned_batch(wk_ctx *ctx, wk_mlp *m, const int64_t *cmd_in, const int32_t *n_in, int32_t nq,
                              int64_t *cmd_out, int32_t *n_out);
/* Cap on the rows of any k2u output of this context (0 = none); a larger
 * step returns WK_EOVERFLOW before writing. */
int     wk_set_row_limit(wk_ctx *ctx, int64_t max_rows);

/* ------------------------------------------------------- request loop
 * Open-loop serving: requests carry a scheduled arrival time (seconds after
 * wk_server_start) and become visible when the server clock passes it.
 * mode 0: one query at a time through wk_execute, in arrival order.
 * mode 1: light requests (constant start, <= max_steps patterns) are packed
 * into continuous batches on two alternating batch objects; heavy requests
 * run on worker contexts sharing the store, overlapping on the device.
 * Admission: a batch takes arrived requests while their projected history
 * bytes fit light_budget_bytes.  plan = 1 plans each request with wk_plan at
 * submission (statistically empty requests complete without device work).
 * The latency of a request is its completion time minus its arrival time. */
typedef struct {
    int32_t mode;                 /* 0 query-at-a-time, 1 batched serving        */
    int32_t max_batch;            /* queries per batch (<= 4096)                  */
    int32_t max_steps;            /* patterns of a batched (light) request        */
    int32_t heavy_workers;        /* worker contexts for heavy requests (mode 1) */
    int64_t batch_capacity_ints;  /* int32 capacity of each batch step table      */
    int64_t light_budget_bytes;   /* admission budget of one batch                */
    int32_t plan;                 /* 0 run as given, 1 statistics planner          */
    int32_t keep_results;         /* 1 keep every result table on the host         */
    int32_t batch_window_us;      /* a light batch launches once its oldest request
                                     has waited this long, or it is full (0: as
                                     soon as a batch object is free)             */
    int32_t pad;
    int64_t max_request_bytes;    /* admission cap: a request whose projected
                                     history bytes exceed it is refused at
                                     submission (status WK_EREJECTED, no device
                                     work); 0 = no cap                            */
} wk_server_config;

typedef struct {
    int64_t completed, light, heavy, failed, batches;
    double  mean_batch;           /* requests per batch                           */
    double  span_s;               /* first arrival .. last completion             */
    double  qps;                  /* completed / span                             */
    double  p50_ms, p99_ms, light_p50_ms, light_p99_ms, heavy_p50_ms, heavy_p99_ms;
                                  /* percentiles by the reference Logger's rule:
                                     sorted latencies, element floor(n q)         */
    int64_t rejected, cancelled;  /* refused at admission / cancelled before they
                                     ran (neither counts as completed)            */
} wk_server_stats;

typedef struct wk_server wk_server;
void    wk_server_config_default(wk_server_config *cfg);
int     wk_server_create(wk_ctx *ctx, const wk_server_config *cfg, wk_server **out);
/* returns the request id (>= 0) or a negative status */
int64_t wk_server_submit(wk_server *s, const int64_t *cmd_chains, int32_t n_patterns, double arrival_s);
int     wk_server_start(wk_server *s);
int     wk_server_drain(wk_server *s, double timeout_s);
int     wk_server_result(wk_server *s, int64_t id, int64_t *rows, int32_t *cols, int32_t *host, int64_t cap,
                         double *latency_s, int32_t *status);
int     wk_server_get_stats(wk_server *s, wk_server_stats *out);
/* A request tagged with its query type: the index of the template it was
 * instantiated from in a weighted mix, as the reference's batch driver tags
 * each request (core/proxy.hpp:360-410, Logger::start_record).  The class
 * (light or heavy) still follows the request's shape. */
int64_t wk_server_submit_typed(wk_server *s, const int64_t *cmd_chains, int32_t n_patterns, double arrival_s,
                               int32_t type);
/* Per-type statistics of the completed requests of one type, by the
 * reference Logger's rule (core/logger.hpp:182-305: per-type sorted
 * latencies, median element n / 2, 99th element floor(0.99 n), the 25-point
 * CDF); qps is the type's completed requests over the server's span. */
typedef struct {
    int64_t completed, failed;
    double  qps, p50_ms, p99_ms;
    double  cdf_ms[25];
} wk_type_stats;
int     wk_server_type_stats(wk_server *s, int32_t type, wk_type_stats *out);
/* Cancel a request that has not started: it completes at once with status
 * WK_ECANCELED and no device work.  WK_EINVAL when it is already running or
 * finished (its result stands). */
int     wk_server_cancel(wk_server *s, int64_t id);
/* Host-side fault injection: the next n device-buffer reservations of
 * worker context `worker` (0.. the server's workers; -1 the context that
 * re-runs overflowed light requests) fail with WK_ENOMEM exactly as a failed
 * cudaMalloc would, before any kernel of the op is launched.  The request
 * that meets it fails with WK_ENOMEM; every other request is unaffected. */
int     wk_server_inject_alloc_failure(wk_server *s, int32_t worker, int32_t n);
/* Latency CDF of the completed requests (cls 0 all, 1 light, 2 heavy): the
 * reference Logger's 25 points (core/logger.hpp print_cdf), at rates 0.01,
 * 0.05 .. 0.95 by 0.05 and 0.96 .. 1.00 by 0.01, into out_ms[WK_CDF_POINTS]. */
#define WK_CDF_POINTS 25
int     wk_server_latency_cdf(wk_server *s, int32_t cls, double *out_ms);
int     wk_server_destroy(wk_server *s);

/* Per-op timing of the last op (device time from CUDA events, ms) and its
 * algorithmic bytes (input rows/cols, output rows, adjacency entries read). */
typedef struct {
    double  ms;            /* sum of device time of every kernel of the op */
    double  ms_main;       /* device time of the dominant (expansion) kernel */
    int64_t rows_in;
    int64_t rows_out;
    int32_t cols_in;
    int32_t kind;          /* 0 k2u, 1 k2k, 2 k2c, 3 i2u, 4 c2u            */
    int64_t alg_bytes;     /* algorithmic bytes per the roofline formulas   */
    int64_t kernels;       /* kernel launches of the op                     */
    double span_ms;        /* first kernel's start to last kernel's end: ms
                              plus the device's idle time between the op's
                              kernels (the host round trip of a k2u op)     */
} wk_op_stats;
int wk_enable_timing(wk_ctx *ctx, int enable);
int wk_last_op_stats(wk_ctx *ctx, wk_op_stats *st);
/* The per-op statistics of every op of the context's last wk_execute, in
 * pattern order, recorded while timing is enabled: up to `cap` entries into
 * `st`, their number in *n. */
int wk_query_op_stats(wk_ctx *ctx, wk_op_stats *st, int32_t cap, int32_t *n);
int64_t wk_kernel_launches(wk_ctx *ctx);   /* cumulative kernel launches */
int wk_sync(wk_ctx *ctx);
/* Host-side fault injection: the context's next n device-buffer reservations
 * (history and op scratch) fail with WK_ENOMEM as a failed cudaMalloc would.
 * For testing the callers' error paths; no device state is touched. */
int wk_ctx_inject_alloc_failure(wk_ctx *ctx, int32_t n);
/* ------------------------------------------------------- the planner
 * Statistics-based plan of a BGP: Planner::generate_plan
 * (core/planner.hpp:927-1028) over the statistics of
 * GStore::generate_statistic (core/gstore.hpp:1010-1127).  The input is a
 * BGP in SPARQL triple form (every pattern (subject, predicate, OUT, object),
 * any variable numbering, 1..10 patterns); a query already in executable form
 * (IN steps, an index start) gets no plan (*n_out = 0, cost +inf) and is run
 * as written.  The output
 * is the executable order (possibly starting with an inserted index pattern)
 * with variables renumbered -1, -2, ... in plan order.  *n_out holds the room
 * of cmd_out in patterns on entry and the plan's patterns on return.  When
 * the correlation statistics prove the result empty, *proved_empty is set
 * and no plan is returned (the reference's "identified empty result
 * query").  When the search finds no complete order, *n_out is 0 and the
 * cost is +inf, as the reference returns an empty plan (it happens when every
 * pattern starts from one constant); callers then run the query as written.
 * Statistics are built on first use.  Works on host-only contexts. */
int wk_plan(wk_ctx *ctx, const int64_t *cmd_in, int32_t n, int64_t *cmd_out, int32_t *n_out,
            double *est_cost, int32_t *proved_empty);
/* One statistic: which = 0 triples, 1 subjects, 2 objects, 3 type members
 * (of id a; out4[0]), 4 correlation of the pair (a, b) as {out_out, out_in,
 * in_in, in_out} in out4[0..3].  Same counts as the reference's global_*
 * maps after its gather. */
int wk_stat_get(wk_ctx *ctx, int32_t which, int32_t a, int32_t b, int64_t *out4);

/* Device-side interval on the context's stream: begin records a CUDA event,
 * end records another, synchronises and returns the elapsed milliseconds. */
int wk_timer_begin(wk_ctx *ctx);
int wk_timer_end(wk_ctx *ctx, double *ms);
/* Page-locked host memory for history uploads/downloads at full link speed. */
int wk_host_alloc(int64_t bytes, void **out);
int wk_host_free(void *p);

/* ------------------------------------------------ synthetic RDF graphs
 * Seeded generator of ID-form graphs with the id encoding of
 * datagen/generate_data.cpp:88-98.  Deterministic across x86_64 and aarch64.
 * Predicate groups: kind 0 = one-to-many with Zipf(s, cap) out-degree and
 * uniform objects; kind 1 = functional one-to-one (a bijection); kind 2 =
 * many-to-one onto a hub set of hub_frac * n_entities vertices.  Each subject
 * takes part in a predicate with probability `participation`.
 */
typedef struct {
    int32_t kind;
    int32_t count;
    double  zipf_s;
    int32_t zipf_cap;
    int32_t pad;
    double  participation;
    double  hub_frac;
} wk_pred_group;

typedef struct {
    uint64_t      seed;
    int64_t       n_entities;
    int32_t       n_classes;
    int32_t       n_groups;
    wk_pred_group groups[4];
} wk_graph_spec;

typedef struct wk_graph wk_graph;
int     wk_graph_generate(const wk_graph_spec *spec, int32_t n_threads, wk_graph **out);
int64_t wk_graph_size(const wk_graph *g);
int32_t wk_graph_num_ids(const wk_graph *g);
int32_t wk_graph_first_class(const wk_graph *g);
const int32_t *wk_graph_s(const wk_graph *g);
const int32_t *wk_graph_p(const wk_graph *g);
const int32_t *wk_graph_o(const wk_graph *g);
void    wk_graph_free(wk_graph *g);
/* Build the store straight from a generated graph (no host copies). */
int     wk_store_build_graph(wk_ctx *ctx, const wk_graph *g);

#ifdef __cplusplus
}
#endif
#endif /* WUKONG_GPU_H */
