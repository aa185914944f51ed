// The store image built on the device (wk_store_build_device), byte for byte
// the image the host builder makes from the same triples (wk_store.cpp).
//
// Content follows the reference loader and store (core/dgraph.hpp:268-330,
// core/gstore.hpp:296-343, :460-524, :665-870): per predicate, out-lists by
// subject and in-lists by object, ascending and deduplicated; index lists of
// subjects ([0|p|IN]) and objects ([0|p|OUT]); class member lists ([0|c|IN]).
//
// Pipeline, every per-triple and per-key step on the device:
//   1. the triples are checked (ranges, as the host builder does) and sorted
//      by (predicate, s, o) and by (predicate, o, s) (wk_sort.cu);
//   2. per order, flags of distinct pairs and of list heads (a new
//      (predicate, vertex)), and their exclusive scans: an entry's place in
//      the deduplicated edges and a list's key index;
//   3. per id, the ranges of its pairs and keys, its vertex range and longest
//      list -- a few numbers per id, which the host turns into the layout
//      (dense directions, bitmaps, sizes and offsets: the same decisions as
//      split_dense in wk_store.cpp);
//   4. the edge image (out-lists, in-lists, index lists, class members), the
//      offsets and neighbour arrays of dense directions (a binary search in
//      the direction's keys per id of the range), presence bitmaps, and the
//      hashed keys in the host builder's insertion order;
//   5. bucket insertion as the host's cluster chaining leaves it: keys sorted
//      stably by (id, bucket) give each key its rank in its main bucket; rank
//      r goes to slot r mod 5 of chain bucket r / 5; an overflow bucket is
//      numbered by the order, in insertion order, of the keys that open it
//      (rank 5, 10, ...), which is the order the host allocates them in;
//   6. the image is copied into the pinned host image the runtime keeps.
#include "wk_runtime.h"

#include <algorithm>
#include <climits>
#include <cstring>
#include <vector>

namespace wk {

int scan_u32_device(uint32_t *x, int64_t m, DevBuf &scratch, cudaStream_t st, int64_t *launches);
int sort_pairs_device(uint64_t *key, uint32_t *id, uint64_t *key_tmp, uint32_t *id_tmp, int64_t n,
                      const std::vector<int> &key_shifts, int id_bits, cudaStream_t st, int64_t *launches);
void pack_triples_device(const int32_t *s, const int32_t *p, const int32_t *o, int64_t n, int order, uint64_t *key,
                         uint32_t *pid, cudaStream_t st);
int radix_bits(uint64_t v);

namespace bld {

constexpr int kT = 256;

inline unsigned int grid_for(int64_t n) {
    const int64_t b = (n + kT - 1) / kT;
    return (unsigned int)std::max<int64_t>(1, std::min<int64_t>(b, 152 * 32));
}

#define GRID_STRIDE(i, n) \
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += (int64_t)gridDim.x * blockDim.x)

// ---------------------------------------------------------------- checks
// first_bad[k]: the smallest triple index failing check k, in the host
// builder's order of checks: 0 predicate, 1 subject, 2 class of a type
// triple, 3 object; max_vid: the largest of max(s, o) (as the host computes
// it, a signed maximum cast to unsigned).
struct Check {
    unsigned long long first_bad[4];
    unsigned int max_vid;
};

__global__ void validate_kernel(const int32_t *__restrict__ s, const int32_t *__restrict__ p,
                                const int32_t *__restrict__ o, int64_t n, int32_t num_ids, Check *ck) {
    unsigned int mx = 0;
    GRID_STRIDE(i, n) {
        const int32_t si = s[i], pi = p[i], oi = o[i];
        mx = max(mx, (unsigned int)max(si, oi));
        if (pi < 1 || pi > num_ids) atomicMin(&ck->first_bad[0], (unsigned long long)i);
        else if (si < WK_VID_BASE || si == INT32_MAX) atomicMin(&ck->first_bad[1], (unsigned long long)i);
        else if (pi == WK_TYPE_ID) {
            if (oi < 2 || oi > num_ids) atomicMin(&ck->first_bad[2], (unsigned long long)i);
        } else if (oi < WK_VID_BASE || oi == INT32_MAX) {
            atomicMin(&ck->first_bad[3], (unsigned long long)i);
        }
    }
#pragma unroll
    for (int sh = 16; sh > 0; sh >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, sh));
    if ((threadIdx.x & 31) == 0) atomicMax(&ck->max_vid, mx);
}

// ------------------------------------------------------- flags and keys
__device__ __forceinline__ bool new_pid(const uint32_t *P, int64_t i) { return i == 0 || P[i] != P[i - 1]; }
// a distinct (predicate, hi, lo): its lo is an edge entry
__device__ __forceinline__ bool is_uniq(const uint64_t *K, const uint32_t *P, int64_t i) {
    return new_pid(P, i) || K[i] != K[i - 1];
}
// a new (predicate, hi): the head of a list, a vertex key
__device__ __forceinline__ bool is_head(const uint64_t *K, const uint32_t *P, int64_t i) {
    return new_pid(P, i) || (K[i] >> 32) != (K[i - 1] >> 32);
}

// uq[i] / hd[i] = the flags of pair i, 0 at i = n (so the scans end with the totals)
__global__ void flags_kernel(const uint64_t *__restrict__ K, const uint32_t *__restrict__ P, int64_t n,
                             uint32_t *__restrict__ uq, uint32_t *__restrict__ hd) {
    GRID_STRIDE(i, n + 1) {
        uq[i] = i < n && is_uniq(K, P, i) ? 1u : 0u;
        hd[i] = i < n && is_head(K, P, i) ? 1u : 0u;
    }
}

// pstart[q] = the first pair of predicate >= q, q = 0 .. num_ids + 1
__global__ void bounds_kernel(const uint32_t *__restrict__ P, int64_t n, int32_t num_ids, int64_t *__restrict__ pstart) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q > num_ids + 1) return;
    int64_t lo = 0, hi = n;
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (P[mid] < (uint32_t)q) lo = mid + 1;
        else hi = mid;
    }
    pstart[q] = lo;
}

// key k = hscan[i] of every list head i: its vertex, its first edge index
// (uscan[i], in this order's deduplicated edges) and its first neighbour
__global__ void keys_kernel(const uint64_t *__restrict__ K, const uint32_t *__restrict__ P, int64_t n,
                            const uint32_t *__restrict__ uscan, const uint32_t *__restrict__ hscan,
                            uint32_t *__restrict__ kvid, uint32_t *__restrict__ kest, int32_t *__restrict__ kfirst) {
    GRID_STRIDE(i, n) {
        if (!is_head(K, P, i)) continue;
        const uint32_t k = hscan[i];
        kvid[k] = (uint32_t)(K[i] >> 32);
        kest[k] = uscan[i];
        kfirst[k] = (int32_t)(uint32_t)K[i];
    }
}

__global__ void degs_kernel(const uint32_t *__restrict__ kest, int64_t nk, uint32_t utot, uint32_t *__restrict__ kdeg) {
    GRID_STRIDE(k, nk) kdeg[k] = (k + 1 < nk ? kest[k + 1] : utot) - kest[k];
}

// Per id q (0 .. num_ids): its pairs [pstart[q], pstart[q + 1]) hold the keys
// [ks, ke) and the edges [us, ue); vmin / vmax = its first and last key's
// vertex; maxdeg = its longest list (atomics per chunk of keys).
struct PidSum {
    uint32_t ks, ke, us, ue, vmin, vmax, maxdeg, pad;
};

__global__ void pidsum_kernel(const int64_t *__restrict__ pstart, int32_t num_ids, const uint32_t *__restrict__ uscan,
                              const uint32_t *__restrict__ hscan, const uint32_t *__restrict__ kvid,
                              PidSum *__restrict__ out) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q > num_ids) return;
    PidSum x;
    x.ks = hscan[pstart[q]];
    x.ke = hscan[pstart[q + 1]];
    x.us = uscan[pstart[q]];
    x.ue = uscan[pstart[q + 1]];
    x.vmin = x.ke > x.ks ? kvid[x.ks] : 0u;
    x.vmax = x.ke > x.ks ? kvid[x.ke - 1] : 0u;
    x.maxdeg = 0u;
    x.pad = 0u;
    out[q] = x;
}

// the id of key k: the last q with ks[q] <= k (ks ascending; q in [0, nq))
__device__ __forceinline__ int pid_of_key(const PidSum *__restrict__ ps, int nq, uint32_t k) {
    int lo = 0, hi = nq - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (ps[mid].ks <= k) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

constexpr int kMaxChunk = 64;   // keys per thread of the longest-list reduction

__global__ void maxdeg_kernel(const uint32_t *__restrict__ kdeg, int64_t nk, PidSum *__restrict__ ps, int nq) {
    GRID_STRIDE(c, (nk + kMaxChunk - 1) / kMaxChunk) {
        const int64_t k0 = c * kMaxChunk, k1 = min(nk, k0 + kMaxChunk);
        int q = pid_of_key(ps, nq, (uint32_t)k0);
        uint32_t m = 0;
        for (int64_t k = k0; k < k1; ++k) {
            while ((uint32_t)k >= ps[q].ke) {   // the next id's keys
                if (m) atomicMax(&ps[q].maxdeg, m);
                m = 0;
                ++q;
            }
            m = max(m, kdeg[k]);
        }
        if (m) atomicMax(&ps[q].maxdeg, m);
    }
}

// ------------------------------------------------------------ the layout
// Per id, where its parts go (filled on the host from the sums):
//   A out-lists, B in-lists, C subjects index, D objects index, E class
//   members, at image offsets a_off .. e_off; per direction d (0 IN, 1 OUT):
//   whether it is dense / has a bitmap, its hashed keys' first index in the
//   hashed-key list (hk[d]), its offsets / neighbour / bitmap arrays' offsets
//   in the rowptr image.
struct Lay {
    unsigned long long a_off, b_off, c_off, d_off, e_off;
    uint32_t us[2];          // first edge index of the id in order 0 (by subject) / order 1 (by object)
    uint32_t ks[2];          // first key index of the id in order 0 / order 1
    uint32_t a_len;          // A: out-lists' entries (the in-lists' offsets start after them)
    uint32_t cls_est;        // E: first edge index (order 1) of the class's member group
    int32_t dense[2], bitmap[2], func[2];
    uint32_t vmin[2], dn[2], bvmin[2], bn[2];
    unsigned long long rp[2], nb[2], bm[2];   // rowptr image offsets
    unsigned long long hk[2];                 // hashed-key list index of the direction's first key
    uint32_t end[2];         // the end of the direction's lists (segment-local)
    uint32_t pad;
};

// the edge image from one order's distinct pairs.  Order 0: the out-lists
// (A) of every id.  Order 1: the in-lists (B) of every id but rdf:type, whose
// (class, subject) pairs are the class member lists (E of the class).
__global__ void edges_kernel(const uint64_t *__restrict__ K, const uint32_t *__restrict__ P, int64_t n,
                             const uint32_t *__restrict__ uscan, int order, const Lay *__restrict__ lay,
                             int32_t *__restrict__ img) {
    GRID_STRIDE(i, n) {
        if (!is_uniq(K, P, i)) continue;
        const uint32_t q = P[i];
        const uint32_t e = uscan[i];
        const int32_t lo = (int32_t)(uint32_t)K[i];
        if (order == 0) {
            img[lay[q].a_off + (e - lay[q].us[0])] = lo;
        } else if (q != (uint32_t)WK_TYPE_ID) {
            img[lay[q].b_off + (e - lay[q].us[1])] = lo;
        } else {
            const uint32_t c = (uint32_t)(K[i] >> 32);
            img[lay[c].e_off + (e - lay[c].cls_est)] = lo;
        }
    }
}

// the index lists: order 0's keys are the subjects of each id (C), order 1's
// the objects (D); rdf:type has neither (its order-1 keys are the classes)
__global__ void index_lists_kernel(const uint32_t *__restrict__ kvid, int64_t nk, int order,
                                   const PidSum *__restrict__ ps, int nq, const Lay *__restrict__ lay,
                                   int32_t *__restrict__ img) {
    GRID_STRIDE(k, nk) {
        const int q = pid_of_key(ps, nq, (uint32_t)k);
        if (q == WK_TYPE_ID) continue;
        const unsigned long long at = (order == 0 ? lay[q].c_off : lay[q].d_off) + ((uint32_t)k - ps[q].ks);
        img[at] = (int32_t)kvid[k];
    }
}

// Vertex keys of one order (order 0: direction OUT, order 1: IN): in a hashed
// direction each key goes to the hashed-key list at its insertion place and
// sets its bit in the presence bitmap, if the direction has one (dense
// directions are written by dense_kernel).
__global__ void vertex_keys_kernel(const uint32_t *__restrict__ kvid, const uint32_t *__restrict__ kest,
                                   const uint32_t *__restrict__ kdeg, int64_t nk, int order,
                                   const PidSum *__restrict__ ps, int nq, const Lay *__restrict__ lay,
                                   uint32_t *__restrict__ hkey, uint32_t *__restrict__ hoff,
                                   uint32_t *__restrict__ hdeg, uint32_t *__restrict__ rowptr) {
    const int dir = order == 0 ? WK_DIR_OUT : WK_DIR_IN;
    GRID_STRIDE(k, nk) {
        const int q = pid_of_key(ps, nq, (uint32_t)k);
        if (order == 1 && q == WK_TYPE_ID) continue;   // the classes of rdf:type, not vertex keys
        const Lay &L = lay[q];
        if (L.dense[dir]) continue;
        const uint32_t vid = kvid[k];
        const unsigned long long h = L.hk[dir] + ((uint32_t)k - ps[q].ks);
        hkey[h] = seg_key(vid, (uint32_t)dir);
        hoff[h] = (order == 0 ? 0u : L.a_len) + (kest[k] - L.us[order]);
        hdeg[h] = kdeg[k];
        if (L.bitmap[dir]) {
            const uint32_t x = vid - L.bvmin[dir];
            atomicOr(rowptr + L.bm[dir] + (x >> 5), 1u << (x & 31u));
        }
    }
}

// One dense direction of one id: for x in [0, dn], rp[x] = the offset of the
// first list of a vertex >= vmin + x, or the direction's end; for a
// functional direction nb[x] = the neighbour of vmin + x, or -1.  keys: the
// direction's keys [k0, k1) of this order, ascending by vertex.
__global__ void dense_kernel(const uint32_t *__restrict__ kvid, const uint32_t *__restrict__ kest,
                             const int32_t *__restrict__ kfirst, uint32_t k0, uint32_t k1, uint32_t vmin, uint32_t dn,
                             uint32_t off0, uint32_t us, uint32_t end, uint32_t *__restrict__ rp,
                             int32_t *__restrict__ nb) {
    GRID_STRIDE(x, (int64_t)dn + 1) {
        const uint32_t v = vmin + (uint32_t)x;
        uint32_t lo = k0, hi = k1;
        while (lo < hi) {
            const uint32_t mid = lo + ((hi - lo) >> 1);
            if (kvid[mid] < v) lo = mid + 1;
            else hi = mid;
        }
        rp[x] = (x < dn && lo < k1) ? off0 + (kest[lo] - us) : end;
        if (nb && x < dn) nb[x] = (lo < k1 && kvid[lo] == v) ? kfirst[lo] : -1;
    }
}

// a few keys written from the host: the index keys of each id
__global__ void extra_keys_kernel(const unsigned long long *__restrict__ at, const uint32_t *__restrict__ key,
                                  const uint32_t *__restrict__ off, const uint32_t *__restrict__ deg, int m,
                                  uint32_t *__restrict__ hkey, uint32_t *__restrict__ hoff, uint32_t *__restrict__ hdeg) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    hkey[at[i]] = key[i];
    hoff[at[i]] = off[i];
    hdeg[at[i]] = deg[i];
}

// --------------------------------------------------------- insertion
// Per id q: its hashed keys are [hb[q], hb[q + 1]) of the hashed-key list,
// its main buckets nmain[q]; mbase[q] = the main buckets of the ids before.
struct Seg {
    unsigned long long hb, mbase, bucket_off;   // bucket_off: in the final image (after nover is known)
    uint32_t nmain, pad;
};

__device__ __forceinline__ int seg_of(const Seg *__restrict__ sg, int nq, unsigned long long g) {
    int lo = 0, hi = nq - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (sg[mid].hb <= g) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// each hashed key's main bucket; sort key = bucket << 32 | key index (the
// index keeps equal buckets in insertion order), sort id = its id; counts of
// keys per main bucket
__global__ void bucket_kernel(const uint32_t *__restrict__ hkey, int64_t nh, const Seg *__restrict__ sg, int nq,
                              uint64_t *__restrict__ skey, uint32_t *__restrict__ sid, uint32_t *__restrict__ bcnt) {
    GRID_STRIDE(g, nh) {
        const int q = seg_of(sg, nq, (unsigned long long)g);
        const uint32_t b = seg_bucket(hkey[g], sg[q].nmain);
        skey[g] = ((uint64_t)b << 32) | (uint64_t)g;
        sid[g] = (uint32_t)q;
        atomicAdd(bcnt + sg[q].mbase + b, 1u);
    }
}

// trig[g] = 1 when key g opens an overflow bucket -- its rank in its main
// bucket (its position in the sorted order minus the bucket's first
// position) is 5, 10, ... -- else 0; 0 at g = nh
__global__ void rank_kernel(const uint64_t *__restrict__ skey, const uint32_t *__restrict__ sid, int64_t nh,
                            const Seg *__restrict__ sg, const uint32_t *__restrict__ bstart,
                            uint32_t *__restrict__ trig) {
    GRID_STRIDE(i, nh + 1) {
        if (i == nh) { trig[nh] = 0u; continue; }
        const uint32_t g = (uint32_t)skey[i], b = (uint32_t)(skey[i] >> 32);
        const uint32_t r = (uint32_t)i - bstart[sg[sid[i]].mbase + b];
        trig[g] = (r % WK_DATA_SLOTS == 0u && r > 0u) ? 1u : 0u;
    }
}

// empty buckets: every key WK_EMPTY_KEY, no link, offsets and degrees 0
__global__ void empty_buckets_kernel(uint32_t *__restrict__ w, int64_t nb) {
    GRID_STRIDE(i, nb * WK_BUCKET_WORDS) {
        const int j = (int)(i % WK_BUCKET_WORDS);
        w[i] = j < WK_DATA_SLOTS ? WK_EMPTY_KEY : (j == WK_LINK_WORD ? WK_NO_LINK : 0u);
    }
}

// Every key into its slot: rank r, chain bucket r / 5 (the main bucket, or
// the overflow bucket opened by the key at rank 5 (r / 5)), slot r mod 5; the
// key that opens a chain bucket also links it from the one before.
// ovf[g] = the exclusive scan of trig: an overflow bucket's number in its id
// is ovf[opener] - ovf[hb].
__global__ void place_kernel(const uint64_t *__restrict__ skey, const uint32_t *__restrict__ sid, int64_t nh,
                             const Seg *__restrict__ sg, const uint32_t *__restrict__ bstart,
                             const uint32_t *__restrict__ hkey, const uint32_t *__restrict__ hoff,
                             const uint32_t *__restrict__ hdeg, const uint32_t *__restrict__ ovf,
                             uint32_t *__restrict__ w) {
    GRID_STRIDE(i, nh) {
        const uint32_t g = (uint32_t)skey[i], b = (uint32_t)(skey[i] >> 32);
        const Seg &S = sg[sid[i]];
        const uint32_t bs = bstart[S.mbase + b];
        const uint32_t r = (uint32_t)i - bs, slot = r % WK_DATA_SLOTS;
        const uint32_t obase = ovf[S.hb];
        auto chain_bucket = [&](int64_t at, uint32_t rr) -> uint32_t {
            if (rr < (uint32_t)WK_DATA_SLOTS) return b;
            return S.nmain + (ovf[(uint32_t)skey[at]] - obase);   // skey[at]: the chain's opener
        };
        const uint32_t cb = chain_bucket(i - slot, r - slot);
        uint32_t *bw = w + (S.bucket_off + cb) * WK_BUCKET_WORDS;
        bw[slot] = hkey[g];
        bw[WK_OFF_WORD + slot] = hoff[g];
        bw[WK_DEG_WORD + slot] = hdeg[g];
        if (slot == 0u && r > 0u) {
            // the previous chain bucket links to this one
            const uint32_t pb = chain_bucket(i - WK_DATA_SLOTS, r - WK_DATA_SLOTS);
            w[(S.bucket_off + pb) * WK_BUCKET_WORDS + WK_LINK_WORD] = cb;
        }
    }
}

}  // namespace bld

// ================================================================= driver
namespace {

struct OrderData {
    DevBuf K, P;                 // sorted pairs
    DevBuf uscan;                // exclusive scan of the distinct-pair flags (n + 1)
    DevBuf kvid, kest, kfirst, kdeg;
    DevBuf ps;                   // PidSum per id
    std::vector<bld::PidSum> hps;
    uint32_t utot = 0, ktot = 0;
};

int fail(cudaError_t e, const char *what) { return cuda_fail(e, what); }

}  // namespace

int build_store_device(wk_ctx *ctx, const int32_t *s, const int32_t *p, const int32_t *o, int64_t n, int32_t num_ids,
                       HostStore **out) {
    using namespace bld;
    cudaStream_t st = ctx->stream;
    int64_t &launches = ctx->launches;
    int rc;
    cudaError_t e;
    const int nq = num_ids + 1;   // ids 0 .. num_ids (0 holds nothing)

    // ---- 1. upload and check the triples
    DevBuf tri, ckb;
    if ((rc = tri.reserve((size_t)n * 12)) || (rc = ckb.reserve(sizeof(Check)))) return rc;
    int32_t *ds = tri.as<int32_t>(), *dp = ds + n, *dobj = dp + n;
    Check hc;
    for (auto &x : hc.first_bad) x = ~0ull;
    hc.max_vid = 0u;
    if ((e = cudaMemcpyAsync(ds, s, (size_t)n * 4, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (e = cudaMemcpyAsync(dp, p, (size_t)n * 4, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (e = cudaMemcpyAsync(dobj, o, (size_t)n * 4, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (e = cudaMemcpyAsync(ckb.ptr, &hc, sizeof(Check), cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return fail(e, "store build: upload");
    validate_kernel<<<grid_for(n), kT, 0, st>>>(ds, dp, dobj, n, num_ids, ckb.as<Check>());
    ++launches;
    if ((e = cudaMemcpyAsync(&hc, ckb.ptr, sizeof(Check), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (e = cudaStreamSynchronize(st)) != cudaSuccess)
        return fail(e, "store build: checks");
    {
        int kind = -1;
        unsigned long long at = ~0ull;
        for (int k = 0; k < 4; ++k)
            if (hc.first_bad[k] < at) { at = hc.first_bad[k]; kind = k; }
        if (kind >= 0) {
            const long long i = (long long)at;
            switch (kind) {
                case 0: return set_error(WK_EINVAL, "store build: triple %lld has predicate %d outside [1,%d]", i, p[i], num_ids);
                case 1: return set_error(WK_EINVAL, "store build: triple %lld has subject %d outside [2^17, 2^31-1)", i, s[i]);
                case 2: return set_error(WK_EINVAL, "store build: type triple %lld has class %d outside [2,%d]", i, o[i], num_ids);
                default: return set_error(WK_EINVAL, "store build: triple %lld has object %d outside [2^17, 2^31-1)", i, o[i]);
            }
        }
    }

    // ---- 2. both orders sorted, on the device
    OrderData od[2];
    {
        DevBuf kt, pt;
        if ((rc = kt.reserve((size_t)n * 8)) || (rc = pt.reserve((size_t)n * 4))) return rc;
        std::vector<int> shifts;
        const int vb = radix_bits(hc.max_vid);
        for (int sh = 0; sh < vb; sh += 8) shifts.push_back(sh);
        for (int sh = 0; sh < vb; sh += 8) shifts.push_back(32 + sh);
        for (int ord = 0; ord < 2; ++ord) {
            if ((rc = od[ord].K.reserve((size_t)n * 8)) || (rc = od[ord].P.reserve((size_t)n * 4))) return rc;
            pack_triples_device(ds, dp, dobj, n, ord, od[ord].K.as<uint64_t>(), od[ord].P.as<uint32_t>(), st);
            ++launches;
            if ((rc = sort_pairs_device(od[ord].K.as<uint64_t>(), od[ord].P.as<uint32_t>(), kt.as<uint64_t>(),
                                        pt.as<uint32_t>(), n, shifts, radix_bits((uint64_t)num_ids), st, &launches)))
                return rc;
        }
    }
    tri.release();

    // ---- 3. per order: flags, scans, keys, per-id sums
    DevBuf pstart, scr;
    if ((rc = pstart.reserve((size_t)(nq + 1) * 8))) return rc;
    for (int ord = 0; ord < 2; ++ord) {
        OrderData &D = od[ord];
        DevBuf hscan;
        if ((rc = D.uscan.reserve((size_t)(n + 1) * 4)) || (rc = hscan.reserve((size_t)(n + 1) * 4))) return rc;
        flags_kernel<<<grid_for(n + 1), kT, 0, st>>>(D.K.as<uint64_t>(), D.P.as<uint32_t>(), n, D.uscan.as<uint32_t>(),
                                                     hscan.as<uint32_t>());
        ++launches;
        if ((rc = scan_u32_device(D.uscan.as<uint32_t>(), n + 1, scr, st, &launches)) ||
            (rc = scan_u32_device(hscan.as<uint32_t>(), n + 1, scr, st, &launches)))
            return rc;
        bounds_kernel<<<(nq + 1 + kT - 1) / kT, kT, 0, st>>>(D.P.as<uint32_t>(), n, num_ids, pstart.as<int64_t>());
        ++launches;
        if ((e = cudaMemcpyAsync(&D.utot, D.uscan.as<uint32_t>() + n, 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
            (e = cudaMemcpyAsync(&D.ktot, hscan.as<uint32_t>() + n, 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
            (e = cudaStreamSynchronize(st)) != cudaSuccess)
            return fail(e, "store build: totals");
        const size_t nk = D.ktot ? D.ktot : 1;
        if ((rc = D.kvid.reserve(nk * 4)) || (rc = D.kest.reserve(nk * 4)) || (rc = D.kfirst.reserve(nk * 4)) ||
            (rc = D.kdeg.reserve(nk * 4)) || (rc = D.ps.reserve((size_t)nq * sizeof(PidSum))))
            return rc;
        keys_kernel<<<grid_for(n), kT, 0, st>>>(D.K.as<uint64_t>(), D.P.as<uint32_t>(), n, D.uscan.as<uint32_t>(),
                                                hscan.as<uint32_t>(), D.kvid.as<uint32_t>(), D.kest.as<uint32_t>(),
                                                D.kfirst.as<int32_t>());
        degs_kernel<<<grid_for(D.ktot), kT, 0, st>>>(D.kest.as<uint32_t>(), D.ktot, D.utot, D.kdeg.as<uint32_t>());
        pidsum_kernel<<<(nq + kT - 1) / kT, kT, 0, st>>>(pstart.as<int64_t>(), num_ids, D.uscan.as<uint32_t>(),
                                                         hscan.as<uint32_t>(), D.kvid.as<uint32_t>(), D.ps.as<PidSum>());
        maxdeg_kernel<<<grid_for((D.ktot + kMaxChunk - 1) / kMaxChunk), kT, 0, st>>>(D.kdeg.as<uint32_t>(), D.ktot,
                                                                                     D.ps.as<PidSum>(), nq);
        launches += 4;
        D.hps.resize((size_t)nq);
        if ((e = cudaMemcpyAsync(D.hps.data(), D.ps.ptr, (size_t)nq * sizeof(PidSum), cudaMemcpyDeviceToHost, st)) !=
                cudaSuccess ||
            (e = cudaStreamSynchronize(st)) != cudaSuccess)
            return fail(e, "store build: per-id sums");
    }

    // the classes: rdf:type's order-1 keys (vertex = class, first edge, members)
    std::vector<uint32_t> cls_vid, cls_est, cls_deg;
    {
        const PidSum &t1 = od[1].hps[(size_t)std::min<int>(WK_TYPE_ID, num_ids)];
        const size_t m = num_ids >= WK_TYPE_ID ? t1.ke - t1.ks : 0;
        cls_vid.resize(m); cls_est.resize(m); cls_deg.resize(m);
        if (m && ((e = cudaMemcpyAsync(cls_vid.data(), od[1].kvid.as<uint32_t>() + t1.ks, m * 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
                  (e = cudaMemcpyAsync(cls_est.data(), od[1].kest.as<uint32_t>() + t1.ks, m * 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
                  (e = cudaMemcpyAsync(cls_deg.data(), od[1].kdeg.as<uint32_t>() + t1.ks, m * 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
                  (e = cudaStreamSynchronize(st)) != cudaSuccess))
            return fail(e, "store build: classes");
    }
    std::vector<uint32_t> M((size_t)nq, 0u), Mest((size_t)nq, 0u);
    for (size_t i = 0; i < cls_vid.size(); ++i) {
        if (cls_vid[i] < (uint32_t)nq) {
            M[cls_vid[i]] = cls_deg[i];
            Mest[cls_vid[i]] = cls_est[i];
        }
    }

    // ---- 4. the layout, per id (the host builder's decisions, from the sums)
    auto *hs = new HostStore();
    std::unique_ptr<HostStore> hs_guard(hs);
    hs->num_ids = num_ids;
    hs->segs.resize((size_t)nq);
    std::vector<Lay> lay((size_t)nq);
    std::vector<uint64_t> nk_of((size_t)nq, 0), nmain_of((size_t)nq, 0);
    // the index keys of each id, in insertion order after its vertex keys
    std::vector<unsigned long long> x_at;
    std::vector<uint32_t> x_key, x_off, x_deg;
    uint64_t edge_at = 0, rp_at = 0, hb_at = 0, nh = 0, mtot = 0;
    std::vector<uint64_t> hb((size_t)nq + 1, 0), mbase((size_t)nq + 1, 0);
    for (int q = 0; q < nq; ++q) {
        Lay &L = lay[(size_t)q];
        std::memset(&L, 0, sizeof(L));
        PredSeg &sg = hs->segs[(size_t)q];
        const PidSum &a = od[0].hps[(size_t)q], &b = od[1].hps[(size_t)q];
        hb[(size_t)q] = hb_at;
        mbase[(size_t)q] = mtot;
        if (q == 0) continue;
        const uint32_t U = a.ue - a.us;                         // distinct pairs of predicate q
        const bool pred = U > 0 && q != WK_TYPE_ID;
        const uint32_t nS = a.ke - a.ks;                        // out keys (subjects)
        const uint32_t nO = pred ? b.ke - b.ks : 0u;            // in keys (objects)
        const uint64_t A = U, B = pred ? (uint64_t)(b.ue - b.us) : 0, C = pred ? nS : 0, Dn = pred ? nO : 0;
        const uint64_t E = M[(size_t)q];
        L.us[0] = a.us;
        L.us[1] = b.us;
        L.ks[0] = a.ks;
        L.ks[1] = b.ks;
        L.a_len = (uint32_t)A;
        L.cls_est = Mest[(size_t)q];
        L.a_off = edge_at;
        L.b_off = edge_at + A;
        L.c_off = L.b_off + B;
        L.d_off = L.c_off + C;
        L.e_off = L.d_off + Dn;
        sg.nedges = A + B + C + Dn + E;
        if (sg.nedges > 0xffffffffull)
            return set_error(WK_EINVAL, "store build: id %d has more than 2^32 edge entries", q);
        sg.edge_off = edge_at;
        edge_at += sg.nedges;
        // statistics, as the host builder counts them
        sg.triples = (int64_t)U;
        sg.subjects = (int64_t)nS;
        sg.objects = (int64_t)nO;
        if (E) {
            sg.subjects += (int64_t)E;
            sg.triples += (int64_t)E;
        }
        // vertex keys per direction: OUT from order 0, IN from order 1
        const uint32_t cnt[2] = {nO, nS};
        const uint32_t vmn[2] = {pred ? b.vmin : 0u, a.vmin}, vmx[2] = {pred ? b.vmax : 0u, a.vmax};
        const uint32_t mdg[2] = {pred ? b.maxdeg : 0u, nS ? a.maxdeg : 0u};
        bool dense[2] = {false, false}, bmap[2] = {false, false};
        for (int d = 0; d < 2; ++d) {
            sg.maxdeg[d] = mdg[d];
            if (!cnt[d]) continue;
            const uint64_t range = (uint64_t)vmx[d] - vmn[d] + 1;
            if ((uint64_t)cnt[d] * WK_DENSE_RATIO >= range) {
                dense[d] = true;
                sg.dvmin[d] = vmn[d];
                sg.dn[d] = (uint32_t)range;
            } else if (!(range / 8 > (uint64_t)cnt[d] * 64)) {
                bmap[d] = true;
                sg.bvmin[d] = vmn[d];
                sg.bn[d] = (uint32_t)range;
            }
        }
        sg.rp_off = rp_at;
        rp_at += sg.rp_entries(0) + sg.rp_entries(1) + sg.nb_entries(0) + sg.nb_entries(1) + sg.bm_words(0) +
                 sg.bm_words(1);
        // keys: out keys, in keys, [0|q|IN] subjects, [0|q|OUT] objects, [0|q|IN] class members
        const uint64_t nidx = (pred && nS ? 1 : 0) + (pred && nO ? 1 : 0) + (E ? 1 : 0);
        sg.nkeys = (uint64_t)nS + nO + nidx;
        const uint64_t hout = dense[1] ? 0 : nS, hin = dense[0] ? 0 : nO;
        const uint64_t nk = hout + hin + nidx;
        nk_of[(size_t)q] = nk;
        const uint64_t nm = nk ? (nk * 2 + WK_DATA_SLOTS - 1) / WK_DATA_SLOTS : 0;
        if (nm + nk / WK_DATA_SLOTS + 1 >= 0xffffffffull)
            return set_error(WK_EINVAL, "store build: id %d has too many keys", q);
        sg.nmain = (uint32_t)nm;
        nmain_of[(size_t)q] = nm;
        for (int d = 0; d < 2; ++d) {
            L.dense[d] = dense[d] ? 1 : 0;
            L.bitmap[d] = bmap[d] ? 1 : 0;
            L.func[d] = (dense[d] && mdg[d] <= 1u) ? 1 : 0;
            L.vmin[d] = sg.dvmin[d];
            L.dn[d] = sg.dn[d];
            L.bvmin[d] = sg.bvmin[d];
            L.bn[d] = sg.bn[d];
        }
        L.rp[0] = sg.rp_off;
        L.rp[1] = L.rp[0] + sg.rp_entries(0);
        L.nb[0] = L.rp[1] + sg.rp_entries(1);
        L.nb[1] = L.nb[0] + sg.nb_entries(0);
        L.bm[0] = L.nb[1] + sg.nb_entries(1);
        L.bm[1] = L.bm[0] + sg.bm_words(0);
        L.hk[1] = hb_at;           // OUT keys first
        L.hk[0] = hb_at + hout;    // then IN keys
        L.end[1] = (uint32_t)A;
        L.end[0] = (uint32_t)(A + B);
        uint64_t xi = hb_at + hout + hin;
        if (pred && nS) {
            x_at.push_back(xi++); x_key.push_back(seg_key(0u, WK_DIR_IN)); x_off.push_back((uint32_t)(A + B));
            x_deg.push_back(nS);
        }
        if (pred && nO) {
            x_at.push_back(xi++); x_key.push_back(seg_key(0u, WK_DIR_OUT)); x_off.push_back((uint32_t)(A + B + C));
            x_deg.push_back(nO);
        }
        if (E) {
            x_at.push_back(xi++); x_key.push_back(seg_key(0u, WK_DIR_IN)); x_off.push_back((uint32_t)(A + B + C + Dn));
            x_deg.push_back((uint32_t)E);
        }
        hb_at += nk;
        mtot += nm;
    }
    hb[(size_t)nq] = hb_at;
    mbase[(size_t)nq] = mtot;
    nh = hb_at;
    if (nh >= 0xffffffffull) return set_error(WK_EINVAL, "store build: 2^32 or more hashed keys");

    // ---- 5. edges, index lists, dense arrays, bitmaps, hashed keys
    DevBuf dimg, drp, dlay, hkey, hoff, hdeg;
    if ((rc = dimg.reserve((edge_at ? edge_at : 1) * 4)) || (rc = drp.reserve((rp_at ? rp_at : 1) * 4)) ||
        (rc = dlay.reserve((size_t)nq * sizeof(Lay))) || (rc = hkey.reserve((nh ? nh : 1) * 4)) ||
        (rc = hoff.reserve((nh ? nh : 1) * 4)) || (rc = hdeg.reserve((nh ? nh : 1) * 4)))
        return rc;
    if ((e = cudaMemcpyAsync(dlay.ptr, lay.data(), (size_t)nq * sizeof(Lay), cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (e = cudaMemsetAsync(drp.ptr, 0, (rp_at ? rp_at : 1) * 4, st)) != cudaSuccess)
        return fail(e, "store build: layout upload");
    const Lay *L_d = dlay.as<Lay>();
    int32_t *img = dimg.as<int32_t>();
    uint32_t *rowptr = drp.as<uint32_t>();
    for (int ord = 0; ord < 2; ++ord) {
        OrderData &D = od[ord];
        edges_kernel<<<grid_for(n), kT, 0, st>>>(D.K.as<uint64_t>(), D.P.as<uint32_t>(), n, D.uscan.as<uint32_t>(), ord,
                                                 L_d, img);
        index_lists_kernel<<<grid_for(D.ktot), kT, 0, st>>>(D.kvid.as<uint32_t>(), D.ktot, ord, D.ps.as<PidSum>(), nq,
                                                            L_d, img);
        vertex_keys_kernel<<<grid_for(D.ktot), kT, 0, st>>>(D.kvid.as<uint32_t>(), D.kest.as<uint32_t>(),
                                                            D.kdeg.as<uint32_t>(), D.ktot, ord, D.ps.as<PidSum>(), nq,
                                                            L_d, hkey.as<uint32_t>(), hoff.as<uint32_t>(),
                                                            hdeg.as<uint32_t>(), rowptr);
        launches += 3;
    }
    for (int q = 1; q < nq; ++q) {
        const Lay &L = lay[(size_t)q];
        for (int d = 0; d < 2; ++d) {
            if (!L.dense[d]) continue;
            const int ord = d == WK_DIR_OUT ? 0 : 1;
            const PidSum &ps = od[ord].hps[(size_t)q];
            dense_kernel<<<grid_for((int64_t)L.dn[d] + 1), kT, 0, st>>>(
                od[ord].kvid.as<uint32_t>(), od[ord].kest.as<uint32_t>(), od[ord].kfirst.as<int32_t>(), ps.ks, ps.ke,
                L.vmin[d], L.dn[d], d == WK_DIR_OUT ? 0u : L.a_len, ps.us, L.end[d], rowptr + L.rp[d],
                L.func[d] ? reinterpret_cast<int32_t *>(rowptr + L.nb[d]) : nullptr);
            ++launches;
        }
    }
    if (!x_at.empty()) {
        DevBuf xa, xk, xo, xd;
        const size_t m = x_at.size();
        if ((rc = xa.reserve(m * 8)) || (rc = xk.reserve(m * 4)) || (rc = xo.reserve(m * 4)) || (rc = xd.reserve(m * 4)))
            return rc;
        if ((e = cudaMemcpyAsync(xa.ptr, x_at.data(), m * 8, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
            (e = cudaMemcpyAsync(xk.ptr, x_key.data(), m * 4, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
            (e = cudaMemcpyAsync(xo.ptr, x_off.data(), m * 4, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
            (e = cudaMemcpyAsync(xd.ptr, x_deg.data(), m * 4, cudaMemcpyHostToDevice, st)) != cudaSuccess)
            return fail(e, "store build: index keys");
        extra_keys_kernel<<<(unsigned int)((m + kT - 1) / kT), kT, 0, st>>>(
            xa.as<unsigned long long>(), xk.as<uint32_t>(), xo.as<uint32_t>(), xd.as<uint32_t>(), (int)m,
            hkey.as<uint32_t>(), hoff.as<uint32_t>(), hdeg.as<uint32_t>());
        ++launches;
        if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return fail(e, "store build: index keys");
    }
    for (int ord = 0; ord < 2; ++ord) {   // the sorted pairs and keys are done with
        od[ord].K.release(); od[ord].P.release(); od[ord].uscan.release();
        od[ord].kvid.release(); od[ord].kest.release(); od[ord].kfirst.release(); od[ord].kdeg.release();
    }

    // ---- 6. bucket insertion
    std::vector<Seg> segv((size_t)nq);
    for (int q = 0; q < nq; ++q) {
        segv[(size_t)q].hb = hb[(size_t)q];
        segv[(size_t)q].mbase = mbase[(size_t)q];
        segv[(size_t)q].nmain = (uint32_t)nmain_of[(size_t)q];
        segv[(size_t)q].bucket_off = 0;
        segv[(size_t)q].pad = 0;
    }
    std::vector<uint32_t> ovf_at((size_t)nq + 1, 0u);   // the scan of openers at each id's first key
    DevBuf dseg, skey, sid, kt2, pt2, bcnt, trig;
    if ((rc = dseg.reserve((size_t)nq * sizeof(Seg)))) return rc;
    if (nh) {
        if ((rc = skey.reserve(nh * 8)) || (rc = sid.reserve(nh * 4)) || (rc = kt2.reserve(nh * 8)) ||
            (rc = pt2.reserve(nh * 4)) || (rc = bcnt.reserve((mtot + 1) * 4)) || (rc = trig.reserve((nh + 1) * 4)))
            return rc;
        if ((e = cudaMemcpyAsync(dseg.ptr, segv.data(), (size_t)nq * sizeof(Seg), cudaMemcpyHostToDevice, st)) !=
                cudaSuccess ||
            (e = cudaMemsetAsync(bcnt.ptr, 0, (mtot + 1) * 4, st)) != cudaSuccess)
            return fail(e, "store build: insertion setup");
        bucket_kernel<<<grid_for((int64_t)nh), kT, 0, st>>>(hkey.as<uint32_t>(), (int64_t)nh, dseg.as<Seg>(), nq,
                                                           skey.as<uint64_t>(), sid.as<uint32_t>(), bcnt.as<uint32_t>());
        ++launches;
        uint64_t maxm = 0;
        for (uint64_t x : nmain_of) maxm = std::max(maxm, x);
        std::vector<int> shifts;
        for (int sh = 0; sh < radix_bits(nh); sh += 8) shifts.push_back(sh);
        for (int sh = 0; sh < radix_bits(maxm); sh += 8) shifts.push_back(32 + sh);
        if ((rc = sort_pairs_device(skey.as<uint64_t>(), sid.as<uint32_t>(), kt2.as<uint64_t>(), pt2.as<uint32_t>(),
                                    (int64_t)nh, shifts, radix_bits((uint64_t)num_ids), st, &launches)) ||
            (rc = scan_u32_device(bcnt.as<uint32_t>(), (int64_t)mtot + 1, scr, st, &launches)))
            return rc;
        kt2.release();
        pt2.release();
        rank_kernel<<<grid_for((int64_t)nh + 1), kT, 0, st>>>(skey.as<uint64_t>(), sid.as<uint32_t>(), (int64_t)nh,
                                                             dseg.as<Seg>(), bcnt.as<uint32_t>(), trig.as<uint32_t>());
        ++launches;
        if ((rc = scan_u32_device(trig.as<uint32_t>(), (int64_t)nh + 1, scr, st, &launches))) return rc;
        for (int q = 0; q <= nq; ++q)
            if ((e = cudaMemcpyAsync(&ovf_at[(size_t)q], trig.as<uint32_t>() + hb[(size_t)q], 4, cudaMemcpyDeviceToHost,
                                     st)) != cudaSuccess)
                return fail(e, "store build: overflow counts");
        if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return fail(e, "store build: overflow counts");
    }
    uint64_t total_buckets = 0;
    for (int q = 0; q < nq; ++q) {
        PredSeg &sg = hs->segs[(size_t)q];
        sg.nover = nh ? ovf_at[(size_t)q + 1] - ovf_at[(size_t)q] : 0u;
        sg.bucket_off = total_buckets;
        segv[(size_t)q].bucket_off = total_buckets;
        total_buckets += (uint64_t)sg.nmain + sg.nover;
    }
    DevBuf dbk;
    if ((rc = dbk.reserve((total_buckets ? total_buckets : 1) * sizeof(Bucket)))) return rc;
    if (total_buckets) {
        if ((e = cudaMemcpyAsync(dseg.ptr, segv.data(), (size_t)nq * sizeof(Seg), cudaMemcpyHostToDevice, st)) !=
            cudaSuccess)
            return fail(e, "store build: bucket offsets");
        empty_buckets_kernel<<<grid_for((int64_t)total_buckets * WK_BUCKET_WORDS), kT, 0, st>>>(
            dbk.as<uint32_t>(), (int64_t)total_buckets);
        place_kernel<<<grid_for((int64_t)nh), kT, 0, st>>>(skey.as<uint64_t>(), sid.as<uint32_t>(), (int64_t)nh,
                                                          dseg.as<Seg>(), bcnt.as<uint32_t>(), hkey.as<uint32_t>(),
                                                          hoff.as<uint32_t>(), hdeg.as<uint32_t>(),
                                                          trig.as<uint32_t>(), dbk.as<uint32_t>());
        launches += 2;
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return fail(e, "store build: kernels");

    // ---- 7. the image into pinned host memory
    const uint64_t bbytes = (total_buckets ? total_buckets : 1) * sizeof(Bucket);
    const uint64_t ebytes = (edge_at ? edge_at : 1) * 4, rbytes = (rp_at ? rp_at : 1) * 4;
    void *bp = nullptr, *ep = nullptr, *rpp = nullptr;
    bool pinned = cudaHostAlloc(&bp, bbytes, cudaHostAllocPortable) == cudaSuccess &&
                  cudaHostAlloc(&ep, ebytes, cudaHostAllocPortable) == cudaSuccess &&
                  cudaHostAlloc(&rpp, rbytes, cudaHostAllocPortable) == cudaSuccess;
    if (!pinned) {
        cudaGetLastError();
        if (bp) cudaFreeHost(bp);
        if (ep) cudaFreeHost(ep);
        if (rpp) cudaFreeHost(rpp);
        bp = aligned_alloc(WK_BUCKET_BYTES, bbytes);
        ep = malloc(ebytes);
        rpp = malloc(rbytes);
        if (!bp || !ep || !rpp) {
            free(bp); free(ep); free(rpp);
            return set_error(WK_ENOMEM, "store build: out of host memory");
        }
    }
    hs->pinned = pinned;
    hs->buckets = static_cast<Bucket *>(bp);
    hs->edges = static_cast<int32_t *>(ep);
    hs->rowptr = static_cast<uint32_t *>(rpp);
    if ((total_buckets && (e = cudaMemcpyAsync(bp, dbk.ptr, total_buckets * sizeof(Bucket), cudaMemcpyDeviceToHost, st)) != cudaSuccess) ||
        (edge_at && (e = cudaMemcpyAsync(ep, dimg.ptr, edge_at * 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess) ||
        (rp_at && (e = cudaMemcpyAsync(rpp, drp.ptr, rp_at * 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess) ||
        (e = cudaStreamSynchronize(st)) != cudaSuccess)
        return fail(e, "store build: image download");
    hs->total_buckets = total_buckets;
    hs->total_edges = edge_at;
    hs->total_rowptr = rp_at;
    for (int q = 1; q < nq; ++q) {
        hs->total_keys += hs->segs[(size_t)q].nkeys;
        hs->total_over += hs->segs[(size_t)q].nover;
    }
    *out = hs_guard.release();
    return WK_OK;
}

}  // namespace wk
