/*
 * CPU oracle for the per-triple-pattern operator -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's store and CPU engine, used by the
 * tests as the checker and by bench.py as the timed CPU baseline.  Nothing in
 * the product (wukonggpu_gb300/) links, loads or calls it.
 *
 * Parity is pinned against the reference itself: oracle/ref_harness.cpp
 * compiles the reference's core/gstore.hpp from its own sources, and the
 * tests compare this restatement with it (and with golden fixtures made from
 * it under tests/golden/).
 */
#ifndef WK_ORACLE_H
#define WK_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_store orc_store;

typedef struct {
    int32_t *data;   /* row-major, malloc'ed */
    int64_t rows;
    int32_t cols;
    int32_t pad;
} orc_table;

/* Build the store (core/dgraph.hpp:268-330 + core/gstore.hpp:600-978). */
orc_store *orc_build(const int32_t *s, const int32_t *p, const int32_t *o, int64_t n, int32_t num_ids);
void orc_free(orc_store *st);

/* GStore::get_edges_local (core/gstore.hpp:471-481); returns the degree. */
int64_t orc_get_edges(const orc_store *st, int64_t vid, int32_t pid, int32_t dir, const int32_t **out);
int64_t orc_num_keys(const orc_store *st);
/* order-independent content digest (keys, degrees, neighbour sets) */
uint64_t orc_digest(const orc_store *st, int64_t *nkeys, int64_t *nedges);
/* i-th stored key in slot order; returns its degree, -1 past the end */
int64_t orc_key_at(const orc_store *st, int64_t i, int64_t *vid, int32_t *pid, int32_t *dir);

/* One pattern with the CPU engine's semantics (core/engine.hpp:96-255),
 * dispatched as GPU_Engine::execute_one_step (core/gpu_engine.hpp:395-467).
 * Returns 0, or -1 on an unsupported shape. */
int orc_step(const orc_store *st, orc_table *t, int is_first, int64_t start, int64_t pid, int64_t dir,
             int64_t end, int64_t *scanned);

/* Whole query; nthreads > 1 splits the first step's rows by stride like
 * Engine::index_to_unknown (core/engine.hpp:243-245) and concatenates the
 * per-thread results.  step_rows (may be NULL) receives the row count after
 * every step (summed over the threads' tables when nthreads > 1). */
int orc_execute(const orc_store *st, const int64_t *cmd, int32_t npat, int32_t nthreads, orc_table *out,
                int64_t *step_rows);

void orc_table_free(orc_table *t);
/* Order-independent digest of a rows x cols table (sum over rows of a hash of
 * each row), computed on nthreads threads. */
uint64_t orc_rows_digest(const int32_t *data, int64_t rows, int32_t cols, int32_t nthreads);
/* replace t's contents with a copy of src (rows x cols) */
int orc_table_set(orc_table *t, const int32_t *src, int64_t rows, int32_t cols);

/* Per-id statistics as GStore::generate_statistic counts them
 * (core/gstore.hpp:1010-1127). */
void orc_pred_stats(const orc_store *st, int32_t id, int64_t *triples, int64_t *subjects, int64_t *objects);

#ifdef __cplusplus
}
#endif
#endif
