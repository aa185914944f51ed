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
#define WK_SLOTS_PER_BUCKET 8      // 8 x 16 B slots = one 128 B bucket
#define WK_DATA_SLOTS 7            // slot 7 of every bucket is the overflow link
#define WK_LINK_TAG 0x80000000u    // set in the high key word of a used link slot

namespace wk {

int set_error(int status, const char *fmt, ...);

// Packed key: bits [0] dir, [1..17] pid, [18..63] vid.  Same bit layout as the
// reference's ikey_t bitfields (core/gstore.hpp:117-149); 0 is the empty key.
static inline uint64_t make_key(uint64_t vid, uint64_t pid, uint64_t dir) {
    return (vid << 18) | (pid << 1) | dir;
}

// Bucket hash: the 64-bit finalizer of MurmurHash3 (fmix64).  Any good mixer
// works here; content, not placement, is what must match the reference.
static inline uint64_t key_mix(uint64_t k) {
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdull;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ull;
    k ^= k >> 33;
    return k;
}

// bucket index in [0, n) by multiply-high ("fastrange"), no division
static inline uint32_t bucket_of(uint64_t h, uint32_t n) {
    return (uint32_t)(((unsigned __int128)h * n) >> 64);
}

// One predicate/type id's segment in the host image.  Buckets hold 16 B
// slots {key lo, key hi, off, deg}; off is relative to the segment's edges.
struct PredSeg {
    uint64_t bucket_off = 0;   // first slot (16 B units) in the host bucket image
    uint32_t nmain = 0;        // main buckets (hash space)
    uint32_t nover = 0;        // overflow buckets appended after the main ones
    uint64_t edge_off = 0;     // first int32 in the host edge image
    uint64_t nedges = 0;       // int32 entries in this id's edge segment
    uint64_t nkeys = 0;
    // statistics (GStore::generate_statistic, core/gstore.hpp:1010-1127)
    int64_t triples = 0, subjects = 0, objects = 0;
    uint64_t bucket_bytes() const { return (uint64_t)(nmain + nover) * WK_SLOTS_PER_BUCKET * 16; }
    uint64_t edge_bytes() const { return nedges * 4; }
};

struct HostStore {
    int32_t num_ids = 0;
    std::vector<PredSeg> segs;     // indexed by id, size num_ids + 1
    uint32_t *buckets = nullptr;   // (sum of buckets) * 8 slots * 4 words
    int32_t *edges = nullptr;
    uint64_t total_slots = 0, total_edges = 0, total_keys = 0, total_over = 0;
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
    const uint4 *buckets;      // nmain + nover buckets of 8 slots
    const int32_t *edges;
    uint32_t nmain;
    uint32_t nover;            // bound on overflow hops (corruption guard)
};

}  // namespace wk
