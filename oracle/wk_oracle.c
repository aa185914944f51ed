/*
 * CPU oracle -- TEST INFRASTRUCTURE ONLY (see wk_oracle.h).
 *
 * Restates, in plain C:
 *   - the loader's per-predicate sort + dedup (core/dgraph.hpp:268-330 with
 *     the edge_sort_by_spo / edge_sort_by_ops orders, core/gstore.hpp:56-99);
 *   - GStore's cluster-chaining key/value store: 64-bit key {dir:1, pid:17,
 *     vid:46} (core/gstore.hpp:117-149), 64-bit pointer {size:28, off:36}
 *     (:156-176), 8-slot buckets whose last slot links to an indirect bucket
 *     (insert_key :296-343, get_vertex_local :389-409), Thomas Wang's 64-bit
 *     hash (utils/mymath.hpp:62-71), main headers split per predicate in
 *     proportion to its triple count (GStore::init :600-659);
 *   - the insert order of insert_normal (:665-833) and the index lists
 *     (record_index_info :835-870, insert_type_index_map :460-480,
 *     insert_index_map :490-524);
 *   - the CPU engine's steps (core/engine.hpp:96-255) and the step dispatch of
 *     GPU_Engine::execute_one_step (core/gpu_engine.hpp:395-467) with the
 *     variable typing of core/query.hpp:141-154.
 * The sizing of the key region is this file's own (the reference takes it
 * from a config value); it changes placement only, never content.
 */
#include "wk_oracle.h"

#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define ASSOC 8
#define VID_BASE (1 << 17)
#define TYPE_ID 1
#define DIR_IN 0
#define DIR_OUT 1

typedef struct {
    uint64_t key;   /* bit 0 dir, bits 1..17 pid, bits 18..63 vid */
    uint64_t ptr;   /* bits 0..27 size, bits 28..63 off */
} slot_t;

struct orc_store {
    int32_t num_ids;
    uint64_t num_buckets, num_buckets_ext, last_ext;
    slot_t *slots;
    int32_t *edges;
    uint64_t num_entries, last_entry;
    uint64_t *partition_sz, *main_hdr_start;
    int64_t *st_triples, *st_subjects, *st_objects;
    int64_t nkeys;
};

static inline uint64_t pack_key(uint64_t vid, uint64_t pid, uint64_t dir) {
    return (vid << 18) | (pid << 1) | dir;
}
static inline uint64_t key_vid(uint64_t k) { return k >> 18; }
static inline int is_tpid(int64_t id) { return id > 1 && id < VID_BASE; }   /* core/gstore.hpp:111 */

/* utils/mymath.hpp:62-71 */
static inline uint64_t wang_hash(uint64_t key) {
    key = (~key) + (key << 21);
    key = key ^ (key >> 24);
    key = (key + (key << 3)) + (key << 8);
    key = key ^ (key >> 14);
    key = (key + (key << 2)) + (key << 4);
    key = key ^ (key >> 28);
    key = key + (key << 31);
    return key;
}

/* ---------------------------------------------------------------- sorting */
/* LSD radix sort of u64 values, 16-bit digits */
static int radix_sort_u64(uint64_t *a, uint64_t n) {
    if (n < 2) return 0;
    uint64_t *tmp = (uint64_t *)malloc(n * sizeof(uint64_t));
    uint64_t *cnt = (uint64_t *)malloc(65536 * sizeof(uint64_t));
    if (!tmp || !cnt) { free(tmp); free(cnt); return -1; }
    uint64_t *src = a, *dst = tmp;
    for (int pass = 0; pass < 4; ++pass) {
        const int sh = pass * 16;
        memset(cnt, 0, 65536 * sizeof(uint64_t));
        for (uint64_t i = 0; i < n; ++i) cnt[(src[i] >> sh) & 0xffff]++;
        if (cnt[(src[0] >> sh) & 0xffff] == n) continue;   /* digit constant */
        uint64_t sum = 0;
        for (int d = 0; d < 65536; ++d) { uint64_t c = cnt[d]; cnt[d] = sum; sum += c; }
        for (uint64_t i = 0; i < n; ++i) dst[cnt[(src[i] >> sh) & 0xffff]++] = src[i];
        uint64_t *t = src; src = dst; dst = t;
    }
    if (src != a) memcpy(a, src, n * sizeof(uint64_t));
    free(tmp);
    free(cnt);
    return 0;
}

static uint64_t dedup_u64(uint64_t *a, uint64_t n) {   /* core/dgraph.hpp:70-84 on sorted data */
    if (n < 2) return n;
    uint64_t m = 1;
    for (uint64_t i = 1; i < n; ++i)
        if (a[i] != a[m - 1]) a[m++] = a[i];
    return m;
}

/* -------------------------------------------------------------- the store */
static int insert_key(orc_store *st, uint64_t key, uint64_t *slot_out) {   /* core/gstore.hpp:296-343 */
    const uint32_t pid = (uint32_t)((key >> 1) & 0x1ffff);
    if (st->partition_sz[pid] == 0) return -1;
    uint64_t bucket = st->main_hdr_start[pid] + wang_hash(key) % st->partition_sz[pid];
    const uint64_t nb = st->num_buckets + st->num_buckets_ext;
    for (;;) {
        uint64_t slot = bucket * ASSOC;
        for (int i = 0; i < ASSOC - 1; ++i, ++slot) {
            if (st->slots[slot].key == key) return -1;   /* duplicate key */
            if (st->slots[slot].key == 0) {
                st->slots[slot].key = key;
                *slot_out = slot;
                return 0;
            }
        }
        if (st->slots[slot].key != 0) {   /* linked to an indirect bucket */
            bucket = key_vid(st->slots[slot].key);
            continue;
        }
        if (st->last_ext >= st->num_buckets_ext) return -1;
        const uint64_t nbk = st->num_buckets + st->last_ext++;
        if (nbk >= nb) return -1;
        st->slots[slot].key = pack_key(nbk, 0, 0);
        st->slots[nbk * ASSOC].key = key;
        *slot_out = nbk * ASSOC;
        return 0;
    }
}

static int put_list(orc_store *st, uint64_t key, const int32_t *vals, uint64_t n) {
    uint64_t slot;
    if (insert_key(st, key, &slot)) return -1;
    if (st->last_entry + n > st->num_entries) return -1;
    const uint64_t off = st->last_entry;
    memcpy(st->edges + off, vals, n * sizeof(int32_t));
    st->last_entry += n;
    st->slots[slot].ptr = (n & ((1ull << 28) - 1)) | (off << 28);
    st->nkeys++;
    return 0;
}

/* groups of a sorted (hi<<32|lo) array: one key [hi|pid|dir] -> lo values */
static int put_groups(orc_store *st, const uint64_t *a, uint64_t n, uint32_t pid, uint32_t dir, int32_t *scratch,
                      int32_t *distinct_hi, uint64_t *ndistinct) {
    uint64_t i = 0, nd = 0;
    while (i < n) {
        const uint32_t hi = (uint32_t)(a[i] >> 32);
        uint64_t j = i;
        while (j < n && (uint32_t)(a[j] >> 32) == hi) { scratch[j - i] = (int32_t)(uint32_t)a[j]; ++j; }
        if (put_list(st, pack_key(hi, pid, dir), scratch, j - i)) return -1;
        if (distinct_hi) distinct_hi[nd] = (int32_t)hi;
        ++nd;
        i = j;
    }
    if (ndistinct) *ndistinct = nd;
    return 0;
}

void orc_free(orc_store *st) {
    if (!st) return;
    free(st->slots);
    free(st->edges);
    free(st->partition_sz);
    free(st->main_hdr_start);
    free(st->st_triples);
    free(st->st_subjects);
    free(st->st_objects);
    free(st);
}

orc_store *orc_build(const int32_t *s, const int32_t *p, const int32_t *o, int64_t n, int32_t num_ids) {
    if (n < 0 || num_ids < 1 || num_ids >= VID_BASE) return NULL;
    const size_t nid = (size_t)num_ids + 2;
    orc_store *st = (orc_store *)calloc(1, sizeof(orc_store));
    int64_t *cnt = (int64_t *)calloc(nid, sizeof(int64_t));
    int64_t *start = (int64_t *)calloc(nid + 1, sizeof(int64_t));
    uint64_t *spo = (uint64_t *)malloc(((size_t)n + 1) * sizeof(uint64_t));
    uint64_t *ops = (uint64_t *)malloc(((size_t)n + 1) * sizeof(uint64_t));
    int32_t *scratch = (int32_t *)malloc(((size_t)n + 1) * sizeof(int32_t));
    int32_t *dist = (int32_t *)malloc(((size_t)n + 1) * sizeof(int32_t));
    uint64_t *pend = (uint64_t *)calloc(nid, sizeof(uint64_t));   /* deduped group sizes */
    uint64_t *oend = (uint64_t *)calloc(nid, sizeof(uint64_t));
    if (!st || !cnt || !start || !spo || !ops || !scratch || !dist || !pend || !oend) goto fail;
    st->num_ids = num_ids;
    for (int64_t i = 0; i < n; ++i) {
        if (p[i] < 1 || p[i] > num_ids) goto fail;
        cnt[p[i]]++;
    }
    for (size_t i = 1; i <= nid; ++i) start[i] = start[i - 1] + cnt[i - 1];
    {
        int64_t *at = (int64_t *)malloc(nid * sizeof(int64_t));
        if (!at) goto fail;
        memcpy(at, start, nid * sizeof(int64_t));
        for (int64_t i = 0; i < n; ++i)
            spo[at[p[i]]++] = ((uint64_t)(uint32_t)s[i] << 32) | (uint32_t)o[i];
        free(at);
    }
    /* sort spo by (p,s,o) and ops by (p,o,s), dedup (core/dgraph.hpp:318-324) */
    for (int32_t id = 1; id <= num_ids; ++id) {
        uint64_t *a = spo + start[id];
        const uint64_t m = (uint64_t)cnt[id];
        if (radix_sort_u64(a, m)) goto fail;
        pend[id] = dedup_u64(a, m);
        uint64_t *b = ops + start[id];
        if (id != TYPE_ID) {
            for (uint64_t i = 0; i < pend[id]; ++i) b[i] = ((a[i] & 0xffffffffull) << 32) | (a[i] >> 32);
            if (radix_sort_u64(b, pend[id])) goto fail;
            oend[id] = pend[id];
        }
    }
    /* per-id triple counts for the main-header split (core/gstore.hpp:600-633) */
    st->partition_sz = (uint64_t *)calloc(nid, sizeof(uint64_t));
    st->main_hdr_start = (uint64_t *)calloc(nid, sizeof(uint64_t));
    st->st_triples = (int64_t *)calloc(nid, sizeof(int64_t));
    st->st_subjects = (int64_t *)calloc(nid, sizeof(int64_t));
    st->st_objects = (int64_t *)calloc(nid, sizeof(int64_t));
    uint64_t *psz = (uint64_t *)calloc(nid, sizeof(uint64_t));
    if (!st->partition_sz || !st->main_hdr_start || !st->st_triples || !st->st_subjects || !st->st_objects || !psz)
        goto fail;
    uint64_t num_edges = 0, nkeys_est = 0;
    for (int32_t id = 1; id <= num_ids; ++id) {
        const uint64_t *a = spo + start[id];
        for (uint64_t i = 0; i < pend[id]; ++i) {
            psz[id]++;
            num_edges++;
            const int64_t ob = (int64_t)(uint32_t)a[i];
            if (is_tpid(ob)) { psz[ob]++; num_edges++; }
        }
        if (id != TYPE_ID) { psz[id] += oend[id]; num_edges += oend[id]; }
        nkeys_est += 2 * pend[id] + 3;
    }
    nkeys_est += (uint64_t)num_ids + 16;
    /* key region: main headers at ~1/2 load, then indirect buckets */
    st->num_buckets = (nkeys_est * 2 + ASSOC - 2) / (ASSOC - 1) + 64;
    st->num_buckets_ext = st->num_buckets / 4 + nkeys_est / (ASSOC - 1) + 64;
    st->slots = (slot_t *)calloc((st->num_buckets + st->num_buckets_ext) * ASSOC, sizeof(slot_t));
    st->num_entries = 2 * (uint64_t)n + 2 * (uint64_t)n + 16;
    st->edges = (int32_t *)malloc(st->num_entries * sizeof(int32_t));
    if (!st->slots || !st->edges) { free(psz); goto fail; }
    {
        uint64_t main_hdr_cnt = 0;
        for (int32_t id = 1; id <= num_ids; ++id) {
            uint64_t nbk = num_edges ? (uint64_t)(((double)psz[id] / (double)num_edges) * (double)st->num_buckets) : 0;
            if (nbk == 0 && psz[id] > 0) nbk = 1;
            st->partition_sz[id] = nbk;
            st->main_hdr_start[id] = main_hdr_cnt;
            main_hdr_cnt += nbk;
        }
        if (main_hdr_cnt > st->num_buckets) {   /* rounding: widen the main region */
            st->num_buckets_ext += main_hdr_cnt - st->num_buckets;
        }
        /* indirect buckets start after the (possibly widened) main region */
        if (main_hdr_cnt > st->num_buckets) st->num_buckets = main_hdr_cnt;
    }
    free(psz);
    /* insertion: per predicate, out-lists then in-lists, then the indexes */
    {
        int32_t *type_out_s = NULL;
        for (int32_t id = 1; id <= num_ids; ++id) {
            const uint64_t *a = spo + start[id];
            uint64_t nd = 0;
            if (id == TYPE_ID) {
                if (put_groups(st, a, pend[id], id, DIR_OUT, scratch, NULL, &nd)) goto fail;
                st->st_triples[id] = (int64_t)pend[id];
                st->st_subjects[id] = (int64_t)nd;
                (void)type_out_s;
                continue;
            }
            if (!pend[id]) continue;
            uint64_t nsub = 0, nobj = 0;
            if (put_groups(st, a, pend[id], id, DIR_OUT, scratch, dist, &nsub)) goto fail;
            if (put_list(st, pack_key(0, id, DIR_IN), dist, nsub)) goto fail;       /* [0|p|IN] subjects */
            if (put_groups(st, ops + start[id], oend[id], id, DIR_IN, scratch, dist, &nobj)) goto fail;
            if (put_list(st, pack_key(0, id, DIR_OUT), dist, nobj)) goto fail;      /* [0|p|OUT] objects */
            st->st_triples[id] = (int64_t)pend[id];
            st->st_subjects[id] = (int64_t)nsub;
            st->st_objects[id] = (int64_t)nobj;
        }
        /* type index [0|c|IN]: members of every class, ascending */
        const uint64_t *a = spo + start[TYPE_ID];
        const uint64_t m = pend[TYPE_ID];
        if (m) {
            uint64_t *cs = ops + start[TYPE_ID];   /* unused region for the type predicate */
            for (uint64_t i = 0; i < m; ++i) cs[i] = ((a[i] & 0xffffffffull) << 32) | (a[i] >> 32);
            if (radix_sort_u64(cs, m)) goto fail;
            uint64_t i = 0;
            while (i < m) {
                const uint32_t c = (uint32_t)(cs[i] >> 32);
                uint64_t j = i;
                while (j < m && (uint32_t)(cs[j] >> 32) == c) { scratch[j - i] = (int32_t)(uint32_t)cs[j]; ++j; }
                if (put_list(st, pack_key(0, c, DIR_IN), scratch, j - i)) goto fail;
                st->st_subjects[c] += (int64_t)(j - i);
                st->st_triples[c] += (int64_t)(j - i);
                i = j;
            }
        }
    }
    free(cnt); free(start); free(spo); free(ops); free(scratch); free(dist); free(pend); free(oend);
    return st;
fail:
    free(cnt); free(start); free(spo); free(ops); free(scratch); free(dist); free(pend); free(oend);
    orc_free(st);
    return NULL;
}

/* core/gstore.hpp:389-409 and :471-481 */
int64_t orc_get_edges(const orc_store *st, int64_t vid, int32_t pid, int32_t dir, const int32_t **out) {
    *out = NULL;
    if (pid < 0 || pid > st->num_ids || vid < 0 || (dir != 0 && dir != 1)) return 0;
    if (st->partition_sz[pid] == 0) return 0;
    const uint64_t key = pack_key((uint64_t)vid, (uint64_t)pid, (uint64_t)dir);
    uint64_t bucket = st->main_hdr_start[pid] + wang_hash(key) % st->partition_sz[pid];
    const uint64_t nb = st->num_buckets + st->num_buckets_ext;
    for (uint64_t hops = 0; hops <= nb; ++hops) {
        for (int i = 0; i < ASSOC; ++i) {
            const slot_t *sl = &st->slots[bucket * ASSOC + i];
            if (i < ASSOC - 1) {
                if (sl->key == key) {
                    *out = st->edges + (sl->ptr >> 28);
                    return (int64_t)(sl->ptr & ((1ull << 28) - 1));
                }
            } else {
                if (sl->key == 0) return 0;
                bucket = key_vid(sl->key);
            }
        }
    }
    return 0;
}


/* Order-independent digest of the stored content: per key, the key bits, its
 * degree and the sum of mix64 over its neighbours; summed over keys.  Index
 * lists are filled by racing threads in the reference, so no order enters. */
static inline uint64_t dmix(uint64_t x) {
    x ^= x >> 31; x *= 0x7fb5d329728ea185ull; x ^= x >> 27; x *= 0x81dadef4bc2dd44dull; x ^= x >> 33;
    return x;
}
uint64_t orc_digest(const orc_store *st, int64_t *nkeys, int64_t *nedges) {
    const uint64_t nslots = (st->num_buckets + st->num_buckets_ext) * ASSOC;
    uint64_t d = 0;
    int64_t k = 0, e = 0;
    for (uint64_t i = 0; i < nslots; ++i) {
        if ((i % ASSOC) == ASSOC - 1 || st->slots[i].key == 0) continue;
        const uint64_t sz = st->slots[i].ptr & ((1ull << 28) - 1), off = st->slots[i].ptr >> 28;
        uint64_t a = 0;
        for (uint64_t j = 0; j < sz; ++j) a += dmix((uint64_t)(uint32_t)st->edges[off + j]);
        d += dmix(st->slots[i].key ^ dmix(sz) ^ dmix(a + 0x9e37));
        ++k;
        e += (int64_t)sz;
    }
    *nkeys = k;
    *nedges = e;
    return d;
}

int64_t orc_num_keys(const orc_store *st) { return st->nkeys; }

int64_t orc_key_at(const orc_store *st, int64_t i, int64_t *vid, int32_t *pid, int32_t *dir) {
    /* walk data slots in order; O(n) per call is fine for small checks, so
       callers iterate with a cursor: i is a slot cursor, not a key index */
    const uint64_t nslots = (st->num_buckets + st->num_buckets_ext) * ASSOC;
    for (uint64_t sidx = (uint64_t)i; sidx < nslots; ++sidx) {
        if ((sidx % ASSOC) == ASSOC - 1) continue;
        const slot_t *sl = &st->slots[sidx];
        if (sl->key == 0) continue;
        *vid = (int64_t)key_vid(sl->key);
        *pid = (int32_t)((sl->key >> 1) & 0x1ffff);
        *dir = (int32_t)(sl->key & 1);
        return (int64_t)sidx;
    }
    return -1;
}

void orc_pred_stats(const orc_store *st, int32_t id, int64_t *triples, int64_t *subjects, int64_t *objects) {
    if (id < 1 || id > st->num_ids) { *triples = *subjects = *objects = 0; return; }
    *triples = st->st_triples[id];
    *subjects = st->st_subjects[id];
    *objects = st->st_objects[id];
}

/* ------------------------------------------------------------- the engine */
typedef struct {
    int32_t *d;
    int64_t n, cap;
} vec_t;

static int vpush(vec_t *v, const int32_t *x, int64_t k) {
    if (v->n + k > v->cap) {
        int64_t nc = v->cap ? v->cap * 2 : 1024;
        while (nc < v->n + k) nc *= 2;
        int32_t *nd = (int32_t *)realloc(v->d, (size_t)nc * sizeof(int32_t));
        if (!nd) return -1;
        v->d = nd;
        v->cap = nc;
    }
    memcpy(v->d + v->n, x, (size_t)k * sizeof(int32_t));
    v->n += k;
    return 0;
}

static void replace(orc_table *t, vec_t *v, int32_t cols) {
    free(t->data);
    t->data = v->d;
    t->cols = cols;
    t->rows = cols ? v->n / cols : 0;
}

/* query.hpp:141-149: 0 known, 1 unknown, 2 const */
static int vtype(int64_t v, int32_t col_num) {
    if (v >= 0) return 2;
    return (-v > col_num) ? 1 : 0;
}

int orc_step(const orc_store *st, orc_table *t, int is_first, int64_t start, int64_t pid, int64_t d, int64_t end,
             int64_t *scanned) {
    vec_t out = {0, 0, 0};
    const int32_t *res;
    int64_t sz;
    const int32_t C = t->cols;
    if (scanned) *scanned = 0;
    if (is_first && is_tpid(start)) {   /* Engine::index_to_unknown, full list (:227-255) */
        if (C != 0) return -1;
        sz = orc_get_edges(st, 0, (int32_t)start, (int32_t)d, &res);
        if (sz && vpush(&out, res, sz)) return -1;
        replace(t, &out, 1);
        return 0;
    }
    if (pid < 0) return -1;
    const int ts = vtype(start, C), te = vtype(end, C);
    if (ts == 2 && te == 1) {   /* const_to_unknown (:96-122) */
        if (C != 0) return -1;
        sz = orc_get_edges(st, start, (int32_t)pid, (int32_t)d, &res);
        if (sz && vpush(&out, res, sz)) return -1;
        replace(t, &out, 1);
        return 0;
    }
    if (ts != 0) return -1;
    const int64_t sc = -start - 1;
    if (te == 1) {   /* known_to_unknown (:126-160) */
        if (-end - 1 != C) return -1;
        int32_t *row = (int32_t *)malloc((size_t)(C + 1) * sizeof(int32_t));
        if (!row) return -1;
        for (int64_t i = 0; i < t->rows; ++i) {
            const int32_t *r = t->data + i * C;
            sz = orc_get_edges(st, (int64_t)(uint32_t)r[sc], (int32_t)pid, (int32_t)d, &res);
            memcpy(row, r, (size_t)C * sizeof(int32_t));
            for (int64_t k = 0; k < sz; ++k) {
                row[C] = res[k];
                if (vpush(&out, row, C + 1)) { free(row); return -1; }
            }
        }
        free(row);
        replace(t, &out, C + 1);
        return 0;
    }
    /* known_to_known (:162-194) / known_to_const (:196-225): first match wins */
    const int64_t ec = te == 0 ? -end - 1 : -1;
    int64_t nscan = 0;
    for (int64_t i = 0; i < t->rows; ++i) {
        const int32_t *r = t->data + i * C;
        sz = orc_get_edges(st, (int64_t)(uint32_t)r[sc], (int32_t)pid, (int32_t)d, &res);
        const int32_t target = te == 0 ? r[ec] : (int32_t)end;
        int64_t k;
        for (k = 0; k < sz; ++k)
            if (res[k] == target) break;
        nscan += (k < sz) ? k + 1 : sz;
        if (k < sz && vpush(&out, r, C)) return -1;
    }
    if (scanned) *scanned = nscan;
    replace(t, &out, C);
    return 0;
}

int orc_table_set(orc_table *t, const int32_t *src, int64_t rows, int32_t cols) {
    free(t->data);
    t->data = (int32_t *)malloc((size_t)(rows * cols + 1) * sizeof(int32_t));
    if (!t->data) return -1;
    if (rows * cols) memcpy(t->data, src, (size_t)(rows * cols) * sizeof(int32_t));
    t->rows = rows;
    t->cols = cols;
    return 0;
}

void orc_table_free(orc_table *t) {
    if (!t) return;
    free(t->data);
    t->data = NULL;
    t->rows = 0;
    t->cols = 0;
}

typedef struct {
    const orc_store *st;
    const int64_t *cmd;
    int32_t npat;
    orc_table t;
    int64_t *rows;   /* rows of this thread's table after every step */
    int rc;
} mt_job;

static void *mt_run(void *arg) {
    mt_job *j = (mt_job *)arg;
    for (int32_t i = 1; i < j->npat && j->rc == 0; ++i) {
        j->rc = orc_step(j->st, &j->t, 0, j->cmd[i * 4], j->cmd[i * 4 + 1], j->cmd[i * 4 + 2], j->cmd[i * 4 + 3], NULL);
        j->rows[i] = j->t.rows;
    }
    return NULL;
}

int orc_execute(const orc_store *st, const int64_t *cmd, int32_t npat, int32_t nthreads, orc_table *out,
                int64_t *step_rows) {
    memset(out, 0, sizeof(*out));
    if (npat <= 0) return -1;
    if (orc_step(st, out, 1, cmd[0], cmd[1], cmd[2], cmd[3], NULL)) return -1;
    if (step_rows) step_rows[0] = out->rows;
    if (nthreads <= 1 || npat == 1) {
        for (int32_t i = 1; i < npat; ++i) {
            if (orc_step(st, out, 0, cmd[i * 4], cmd[i * 4 + 1], cmd[i * 4 + 2], cmd[i * 4 + 3], NULL)) return -1;
            if (step_rows) step_rows[i] = out->rows;
        }
        return 0;
    }
    /* strided split of the first step's rows (core/engine.hpp:243-245) */
    mt_job *jobs = (mt_job *)calloc((size_t)nthreads, sizeof(mt_job));
    pthread_t *th = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
    int64_t *trows = (int64_t *)calloc((size_t)nthreads * (size_t)npat, sizeof(int64_t));
    if (!jobs || !th || !trows) { free(jobs); free(th); free(trows); return -1; }
    const int32_t C = out->cols;
    for (int32_t tdx = 0; tdx < nthreads; ++tdx) {
        mt_job *j = &jobs[tdx];
        j->st = st; j->cmd = cmd; j->npat = npat;
        j->rows = trows + (size_t)tdx * (size_t)npat;
        int64_t nr = out->rows > tdx ? (out->rows - tdx + nthreads - 1) / nthreads : 0;
        j->t.data = (int32_t *)malloc((size_t)(nr * C + 1) * sizeof(int32_t));
        j->t.cols = C;
        j->t.rows = nr;
        for (int64_t k = tdx, r = 0; k < out->rows; k += nthreads, ++r)
            memcpy(j->t.data + r * C, out->data + k * C, (size_t)C * sizeof(int32_t));
    }
    for (int32_t tdx = 0; tdx < nthreads; ++tdx) pthread_create(&th[tdx], NULL, mt_run, &jobs[tdx]);
    int rc = 0;
    int64_t total = 0;
    int32_t cols = 0;
    for (int32_t tdx = 0; tdx < nthreads; ++tdx) {
        pthread_join(th[tdx], NULL);
        rc |= jobs[tdx].rc;
        total += jobs[tdx].t.rows;
        cols = jobs[tdx].t.cols;
    }
    orc_table_free(out);
    if (!rc) {
        out->data = (int32_t *)malloc((size_t)(total * cols + 1) * sizeof(int32_t));
        out->cols = cols;
        out->rows = total;
        int64_t at = 0;
        for (int32_t tdx = 0; tdx < nthreads; ++tdx) {
            memcpy(out->data + at, jobs[tdx].t.data, (size_t)(jobs[tdx].t.rows * cols) * sizeof(int32_t));
            at += jobs[tdx].t.rows * cols;
        }
    }
    /* the row count after every step is the sum over the threads' tables */
    if (!rc && step_rows)
        for (int32_t i = 1; i < npat; ++i) {
            int64_t r = 0;
            for (int32_t tdx = 0; tdx < nthreads; ++tdx) r += jobs[tdx].rows[i];
            step_rows[i] = r;
        }
    for (int32_t tdx = 0; tdx < nthreads; ++tdx) orc_table_free(&jobs[tdx].t);
    free(jobs);
    free(th);
    free(trows);
    return rc ? -1 : 0;
}

/* ------------------------------------------------------ table digests */
/* Order-independent digest of a table: the sum (mod 2^64) over rows of a
 * 64-bit hash of the row's values in column order.  Two tables with the same
 * rows in any order have the same digest; the test code compares results of
 * the strided multi-thread split and of index starts (whose order the
 * reference leaves to racing loader threads) this way, at sizes where a
 * canonical sort would take minutes. */
static inline uint64_t row_hash(const int32_t *r, int32_t cols) {
    uint64_t h = 0x243f6a8885a308d3ull ^ (uint64_t)cols;
    for (int32_t c = 0; c < cols; ++c) h = dmix(h + ((uint64_t)(uint32_t)r[c] | ((uint64_t)(c + 1) << 32)));
    return h;
}

typedef struct {
    const int32_t *data;
    int64_t r0, r1;
    int32_t cols;
    uint64_t sum;
} dg_job;

static void *dg_run(void *arg) {
    dg_job *j = (dg_job *)arg;
    uint64_t s = 0;
    for (int64_t i = j->r0; i < j->r1; ++i) s += row_hash(j->data + i * j->cols, j->cols);
    j->sum = s;
    return NULL;
}

uint64_t orc_rows_digest(const int32_t *data, int64_t rows, int32_t cols, int32_t nthreads) {
    if (rows <= 0 || cols <= 0) return 0;
    if (nthreads < 1) nthreads = 1;
    if ((int64_t)nthreads > rows / 4096 + 1) nthreads = (int32_t)(rows / 4096 + 1);
    dg_job *jobs = (dg_job *)calloc((size_t)nthreads, sizeof(dg_job));
    pthread_t *th = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
    if (!jobs || !th) {
        free(jobs);
        free(th);
        dg_job one = {data, 0, rows, cols, 0};
        dg_run(&one);
        return one.sum;
    }
    for (int32_t t = 0; t < nthreads; ++t) {
        jobs[t].data = data;
        jobs[t].cols = cols;
        jobs[t].r0 = rows * t / nthreads;
        jobs[t].r1 = rows * (t + 1) / nthreads;
        pthread_create(&th[t], NULL, dg_run, &jobs[t]);
    }
    uint64_t s = 0;
    for (int32_t t = 0; t < nthreads; ++t) {
        pthread_join(th[t], NULL);
        s += jobs[t].sum;
    }
    free(jobs);
    free(th);
    return s;
}
