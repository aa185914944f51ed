// Internal declarations shared by the host runtime (.cpp) and the kernels (.cu).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstddef>
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
#define WK_BUCKET_WORDS 16
#define WK_BUCKET_BYTES 64
#define WK_DATA_SLOTS 5
#define WK_LINK_WORD 5
#define WK_OFF_WORD 6
#define WK_DEG_WORD 11
#define WK_EMPTY_KEY 0xffffffffu
#define WK_NO_LINK 0xffffffffu

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
    uint64_t nkeys = 0;
    // statistics (GStore::generate_statistic, core/gstore.hpp:1010-1127)
    int64_t triples = 0, subjects = 0, objects = 0;
    uint64_t bucket_bytes() const { return (uint64_t)(nmain + nover) * WK_BUCKET_BYTES; }
    uint64_t edge_bytes() const { return nedges * 4; }
};

struct HostStore {
    int32_t num_ids = 0;
    std::vector<PredSeg> segs;     // indexed by id, size num_ids + 1
    Bucket *buckets = nullptr;     // all segments' buckets, segment after segment
    int32_t *edges = nullptr;
    uint64_t total_buckets = 0, total_edges = 0, total_keys = 0, total_over = 0;
    bool pinned = false;
    ~HostStore();
    // host lookup in the image; returns degree (0 if absent) and the edge pointer
    uint64_t lookup(uint64_t vid, uint32_t pid, uint32_t dir, const int32_t **edges_out) const;
};

struct Stats;   // planner statistics (wk_planner.cpp)
Stats *build_stats(const HostStore &hs);
void free_stats(Stats *s);

int build_host_store(const int32_t *s, const int32_t *p, const int32_t *o, int64_t n,
                     int32_t num_ids, HostStore **out);

// Device view of one predicate segment (passed to kernels by value).
struct PredView {
    const Bucket *buckets;     // nmain + nover buckets
    const int32_t *edges;
    uint32_t nmain;
    uint32_t nover;            // bound on overflow hops (corruption guard)
};

}  // namespace wk
