// Internal declarations shared by the host runtime (.cpp) and the kernels (.cu).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstddef>
#include <functional>
#include <string>
#include <vector>

#include <vector_types.h>

#include "../../include/wukong_gpu.h"

#define WK_VID_BASE (1 << 17)      // first vertex id (datagen/generate_data.cpp:96)

// Bucket layout.  A segment (one predicate or class id) is a hash table of
// 64 B buckets, one L2 fetch each.  A bucket holds 5 slots and a link:
//   w[0..4]   slot keys: vid << 1 | dir, WK_EMPTY_KEY when unused
//   w[5]      overflow link: bucket index in the same segment, or WK_NO_LINK
//   w[6..10]  slot edge offsets, relative to the segment's edge list
//   w[11..15] slot degrees (0 in unused slots)
// The predicate is implied by the segment, so a slot key needs 32 bits; the
// full packed key of the reference (vid << 18 | pid << 1 | dir,
// core/gstore.hpp:117-149) is never stored.
//
// Dense directions.  When the vertex keys of one direction of a segment cover
// at least 1/WK_DENSE_RATIO of their id range [vmin, vmin + n), that
// direction is stored as an offsets array instead: rowptr[v - vmin] is the
// first edge of v's list and rowptr[v - vmin + 1] its end (equal for an
// absent vertex), over the same edge list, whose lists of a direction are
// already in ascending vertex order.  A probe then reads 8 B (one sector)
// instead of a 64 B bucket, the array costs 4 B per id of the range (a hash
// key costs about 26 B), and dense arrays of a few million vertices stay in
// L2.  Index keys (vid 0) always stay in the hash table.  A dense direction
// whose lists hold at most one vertex (a functional predicate) also keeps
// nb[v - vmin] = that vertex or -1, so a lookup that only needs the neighbour
// is a single 4 B read.  A hashed direction whose keys are not too sparse in
// their id range keeps a presence bitmap over it (at most 64 B per key), so a
// probe of an absent vertex -- most probes of a sparse predicate -- is one
// 4 B read instead of a 64 B bucket.
#define WK_BUCKET_WORDS 16
#define WK_BUCKET_BYTES 64
#define WK_DATA_SLOTS 5
#define WK_LINK_WORD 5
#define WK_OFF_WORD 6
#define WK_DEG_WORD 11
#define WK_EMPTY_KEY 0xffffffffu
#define WK_NO_LINK 0xffffffffu
#define WK_DENSE_RATIO 8

#if defined(__CUDACC__)
#define WK_HD __host__ __device__ __forceinline__
#else
#define WK_HD inline
#endif

namespace wk {

int set_error(int status, const char *fmt, ...);

// Segment-local slot key.  vid is a non-negative int32 (vertex ids are at
// least 2^17, index keys use 0), so the key fits 32 bits; the builder rejects
// vid = 2^31 - 1, whose OUT key would equal WK_EMPTY_KEY.
WK_HD uint32_t seg_key(uint32_t vid, uint32_t dir) { return (vid << 1) | dir; }

// Bucket hash: the 32-bit finalizer of MurmurHash3 (fmix32), then a
// multiply-high map onto [0, n).  Any good mixer works here; content, not
// placement, is what must match the reference.
WK_HD uint32_t seg_mix(uint32_t k) {
    k ^= k >> 16;
    k *= 0x85ebca6bu;
    k ^= k >> 13;
    k *= 0xc2b2ae35u;
    k ^= k >> 16;
    return k;
}

WK_HD uint32_t seg_bucket(uint32_t key, uint32_t n) {
    return (uint32_t)(((uint64_t)seg_mix(key) * (uint64_t)n) >> 32);
}

// A BGP in SPARQL triple form, the planners' input: every pattern is
// (subject, predicate, OUT, object) with a variable or a vertex as subject,
// and a variable, a vertex, or (for rdf:type) a class as object.  The
// engine's executable form (IN steps, index starts) is not triple form.
inline bool triple_form(const int64_t *cmd, int n) {
    for (int i = 0; i < n; ++i) {
        const int64_t s = cmd[4 * i], p = cmd[4 * i + 1], d = cmd[4 * i + 2], o = cmd[4 * i + 3];
        if (d != WK_DIR_OUT || p < 1) return false;
        if (s >= 0 && s < WK_VID_BASE) return false;
        if (o >= 0 && o < WK_VID_BASE && !(p == WK_TYPE_ID && o > 1)) return false;
    }
    return true;
}

struct alignas(WK_BUCKET_BYTES) Bucket {
    uint32_t w[WK_BUCKET_WORDS];
};

// One predicate/type id's segment in the host image.
struct PredSeg {
    uint64_t bucket_off = 0;   // first bucket of the segment in the host image
    uint32_t nmain = 0;        // main buckets (hash space)
    uint32_t nover = 0;        // overflow buckets appended after the main ones
    uint64_t edge_off = 0;     // first int32 in the host edge image
    uint64_t nedges = 0;       // int32 entries in this id's edge segment
    uint64_t nkeys = 0;        // all keys, hashed or dense
    // dense directions (index = dir): ids [dvmin, dvmin + dn); dn = 0 when hashed.
    // The offsets arrays of both directions are contiguous in the host
    // rowptr image from rp_off: dir IN (dn[0] + 1 entries, if dense), then OUT.
    uint32_t dvmin[2] = {0u, 0u}, dn[2] = {0u, 0u};
    uint64_t rp_off = 0;
    uint32_t maxdeg[2] = {0u, 0u};   // longest vertex list per direction (index lists excluded)
    uint32_t bvmin[2] = {0u, 0u}, bn[2] = {0u, 0u};   // presence bitmap of a hashed direction; bn = 0: none
    // statistics (GStore::generate_statistic, core/gstore.hpp:1010-1127)
    int64_t triples = 0, subjects = 0, objects = 0;
    uint64_t bucket_bytes() const { return (uint64_t)(nmain + nover) * WK_BUCKET_BYTES; }
    uint64_t edge_bytes() const { return nedges * 4; }
    uint64_t rp_entries(int dir) const { return dn[dir] ? (uint64_t)dn[dir] + 1 : 0; }
    // neighbour array of a dense functional direction, after both offsets arrays
    uint64_t nb_entries(int dir) const { return (dn[dir] && maxdeg[dir] <= 1u) ? (uint64_t)dn[dir] : 0; }
    // presence bitmap words of a hashed direction, after the neighbour arrays
    uint64_t bm_words(int dir) const { return ((uint64_t)bn[dir] + 31) / 32; }
    uint64_t rowptr_bytes() const {
        return 4 * (rp_entries(0) + rp_entries(1) + nb_entries(0) + nb_entries(1) + bm_words(0) + bm_words(1));
    }
};

struct HostStore {
    int32_t num_ids = 0;
    std::vector<PredSeg> segs;     // indexed by id, size num_ids + 1
    Bucket *buckets = nullptr;     // all segments' buckets, segment after segment
    int32_t *edges = nullptr;
    uint32_t *rowptr = nullptr;    // all dense directions' offsets arrays
    uint64_t total_buckets = 0, total_edges = 0, total_keys = 0, total_over = 0, total_rowptr = 0;
    bool pinned = false;
    ~HostStore();
    // host lookup in the image; returns degree (0 if absent) and the edge pointer
    uint64_t lookup(uint64_t vid, uint32_t pid, uint32_t dir, const int32_t **edges_out) const;
    uint64_t digest() const;   // of the whole image, for comparing two builds
    // every key of segment id: f(vid, dir, edge offset in the segment, degree)
    template <class F>
    void for_each_key(int id, F f) const {
        const PredSeg &sg = segs[(size_t)id];
        const Bucket *base = buckets + sg.bucket_off;
        const uint64_t nb = (uint64_t)sg.nmain + sg.nover;
        for (uint64_t b = 0; b < nb; ++b) {
            const uint32_t *w = base[b].w;
            for (int i = 0; i < WK_DATA_SLOTS; ++i)
                if (w[i] != WK_EMPTY_KEY) f(w[i] >> 1, w[i] & 1u, w[WK_OFF_WORD + i], w[WK_DEG_WORD + i]);
        }
        const uint32_t *rp = rowptr + sg.rp_off;
        for (uint32_t dir = 0; dir < 2; ++dir) {
            for (uint32_t x = 0; x < sg.dn[dir]; ++x)
                if (rp[x + 1] > rp[x]) f(sg.dvmin[dir] + x, dir, rp[x], rp[x + 1] - rp[x]);
            rp += sg.rp_entries((int)dir);
        }
    }
};

struct Stats;   // planner statistics (wk_planner.cpp)
Stats *build_stats(const HostStore &hs);
void free_stats(Stats *s);

// The store image from ID-form triples, built on the host (wk_store.cpp);
// wk_build.cu builds the same image on the device.
int build_host_store(const int32_t *s, const int32_t *p, const int32_t *o, int64_t n,
                     int32_t num_ids, HostStore **out);

// Device view of one predicate segment (passed to kernels by value).
struct PredView {
    const Bucket *buckets = nullptr;        // nmain + nover buckets
    const int32_t *edges = nullptr;
    uint32_t nmain = 0;
    uint32_t nover = 0;                     // bound on overflow hops (corruption guard)
    const uint32_t *rp[2] = {nullptr, nullptr};   // dense offsets per direction, or null
    uint32_t vmin[2] = {0u, 0u}, dn[2] = {0u, 0u};
    uint32_t func[2] = {0u, 0u};  // 1: every vertex of the direction has at most one neighbour
    const int32_t *nb[2] = {nullptr, nullptr};    // dense functional: the neighbour per id, or -1
    const uint32_t *bm[2] = {nullptr, nullptr};   // hashed: presence bitmap over [bvmin, bvmin + bn)
    uint32_t bvmin[2] = {0u, 0u}, bn[2] = {0u, 0u};
};

// The device view of segment sg whose buckets, offsets arrays and edges start
// at the given device addresses (offsets arrays in the rowptr image order).
inline PredView make_view(const PredSeg &sg, const Bucket *bk, const uint32_t *rp, const int32_t *edges) {
    PredView v;
    v.buckets = bk;
    v.edges = edges;
    v.nmain = sg.nmain;
    v.nover = sg.nover;
    const uint32_t *nb = rp + sg.rp_entries(0) + sg.rp_entries(1);
    const uint32_t *bm = nb + sg.nb_entries(0) + sg.nb_entries(1);
    for (int d = 0; d < 2; ++d) {
        v.func[d] = sg.maxdeg[d] <= 1u ? 1u : 0u;
        if (sg.dn[d]) {
            v.rp[d] = rp;
            v.vmin[d] = sg.dvmin[d];
            v.dn[d] = sg.dn[d];
        }
        if (sg.nb_entries(d)) v.nb[d] = reinterpret_cast<const int32_t *>(nb);
        if (sg.bn[d]) {
            v.bm[d] = bm;
            v.bvmin[d] = sg.bvmin[d];
            v.bn[d] = sg.bn[d];
        }
        rp += sg.rp_entries(d);
        nb += sg.nb_entries(d);
        bm += sg.bm_words(d);
    }
    return v;
}

}  // namespace wk
