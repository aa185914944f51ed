// Device-side segment probe, shared by the single-query and batched kernels.
//
// One lane looks up one key.  In a dense direction that is two 4 B reads of
// the offsets array; in a hashed one a 64 B bucket is fetched as two
// independent 32 B loads, so a lane has the whole bucket after one memory
// round trip and resolves the slot in registers: no cross-lane traffic on the
// hit path.
// The reference's lookup is GStore::get_edges_global / get_edges_local
// (core/gstore.hpp:389-409): a key that is absent yields an empty list.
#pragma once

#include "wk_internal.h"

namespace wk {
namespace dev {

#ifndef WK_FULL_MASK
#define WK_FULL_MASK 0xffffffffu
#endif

// 32 B load through the non-coherent path without L1 allocation: bucket reads
// are random and have no reuse inside an SM.  p must be 32 B aligned (buckets
// are 64 B aligned in every image: cudaMalloc and the segment pool give 256 B).
__device__ __forceinline__ void ld_bucket_half(const uint32_t *p, uint32_t (&v)[8]) {
    asm("ld.global.nc.L1::no_allocate.v8.u32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
        : "l"(p));
}

// Look up `key` in a segment of nmain main and nover overflow buckets.
// Returns the degree (0 when the key is absent) and the edge offset in *off.
// Overflow hops are bounded by nover; a longer chain, or a link outside the
// segment, sets bit 0 of *err and reports the key absent.
__device__ __forceinline__ uint32_t probe_seg(const Bucket *bk, uint32_t nmain, uint32_t nover, uint32_t key,
                                              uint32_t *off, int *err) {
    *off = 0u;
    if (nmain == 0u) return 0u;
    uint32_t b = seg_bucket(key, nmain);
    for (uint32_t hop = 0;; ++hop) {
        uint32_t a[8], c[8];
        ld_bucket_half(bk[b].w, a);       // keys 0-4, link, off 0-1
        ld_bucket_half(bk[b].w + 8, c);   // off 2-4, deg 0-4
        if (a[0] == key) { *off = a[6]; return c[3]; }
        if (a[1] == key) { *off = a[7]; return c[4]; }
        if (a[2] == key) { *off = c[0]; return c[5]; }
        if (a[3] == key) { *off = c[1]; return c[6]; }
        if (a[4] == key) { *off = c[2]; return c[7]; }
        const uint32_t link = a[5];
        if (link == WK_NO_LINK) return 0u;
        if (hop >= nover || link >= nmain + nover) {
            atomicOr(err, 1);
            return 0u;
        }
        b = link;
    }
}

// Look up vertex or index key (vid, dir) of a segment: through the
// direction's offsets array when it is dense (two 4 B reads, normally one
// sector), else through the hash table.  Returns the degree, the edge offset
// in *off.
__device__ __forceinline__ uint32_t probe_view(const PredView &pv, uint32_t vid, uint32_t dir, uint32_t *off,
                                               int *err) {
    const uint32_t *rp = dir ? pv.rp[1] : pv.rp[0];
    if (rp != nullptr && vid != 0u) {
        const uint32_t x = vid - (dir ? pv.vmin[1] : pv.vmin[0]);   // wraps above n below vmin
        if (x >= (dir ? pv.dn[1] : pv.dn[0])) {
            *off = 0u;
            return 0u;
        }
        const uint32_t a = __ldg(rp + x), b = __ldg(rp + x + 1);
        *off = a;
        return b - a;
    }
    const uint32_t *bm = dir ? pv.bm[1] : pv.bm[0];
    if (bm != nullptr && vid != 0u) {
        const uint32_t x = vid - (dir ? pv.bvmin[1] : pv.bvmin[0]);   // wraps above bn below bvmin
        if (x >= (dir ? pv.bn[1] : pv.bn[0]) || !((__ldg(bm + (x >> 5)) >> (x & 31u)) & 1u)) {
            *off = 0u;
            return 0u;
        }
    }
    return probe_seg(pv.buckets, pv.nmain, pv.nover, seg_key(vid, dir), off, err);
}

// Probe the 32 keys (vid, dir) of a warp in one segment.  A run of equal keys
// on consecutive lanes (the same start vertex on consecutive rows, as an
// expansion leaves them) is looked up once, by the run's first lane; the
// others read its result.  This keeps a column that repeats one vertex
// millions of times from sending every lane to the same bucket.  vid < 0 is
// not a vertex and is reported absent.
__device__ __forceinline__ void probe_warp(const PredView &pv, int32_t vid, uint32_t dir, uint32_t &r_off,
                                           uint32_t &r_deg, int *err) {
    const int lane = threadIdx.x & 31;
    const bool ok = vid >= 0;
    const uint32_t key = seg_key((uint32_t)vid, dir);
    // a lane without a key carries WK_EMPTY_KEY, which is never stored
    const uint32_t kk = ok ? key : WK_EMPTY_KEY;
    const uint32_t prev = __shfl_up_sync(WK_FULL_MASK, kk, 1);
    const unsigned heads = __ballot_sync(WK_FULL_MASK, lane == 0 || prev != kk);
    const int lead = 31 - __clz(heads & (0xffffffffu >> (31 - lane)));   // run head at or below this lane
    uint32_t o = 0u, d = 0u;
    if (ok && lead == lane) d = probe_view(pv, (uint32_t)vid, dir, &o, err);
    r_off = __shfl_sync(WK_FULL_MASK, o, lead);
    r_deg = __shfl_sync(WK_FULL_MASK, d, lead);
}

// As probe_warp, with a segment per lane (rows of different queries).  Equal
// (segment, key) pairs are probed once.
__device__ __forceinline__ void probe_warp_multi(const PredView &pv, uint32_t seg, bool valid, int32_t vid,
                                                 uint32_t dir, uint32_t &r_off, uint32_t &r_deg, int *err) {
    const int lane = threadIdx.x & 31;
    const bool ok = valid && vid >= 0;
    const uint32_t key = seg_key((uint32_t)vid, dir);
    const unsigned same = __match_any_sync(WK_FULL_MASK, ok ? (((uint64_t)seg << 32) | key) : ~0ull);
    const int lead = __ffs(same) - 1;
    uint32_t o = 0u, d = 0u;
    if (ok && lead == lane) d = probe_view(pv, (uint32_t)vid, dir, &o, err);
    r_off = __shfl_sync(WK_FULL_MASK, o, lead);
    r_deg = __shfl_sync(WK_FULL_MASK, d, lead);
}

}  // namespace dev
}  // namespace wk
