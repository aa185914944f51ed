// Host-side build of the store image from ID-form triples.
//
// Content follows the reference loader and store:
//  - triples are grouped per predicate, sorted by (s,o) for out-edges and by
//    (o,s) for in-edges and deduplicated (core/dgraph.hpp:268-330, sort orders
//    edge_sort_by_spo / edge_sort_by_ops at core/gstore.hpp:56-99), so every
//    adjacency list is ascending by neighbour id;
//  - key [s|p|OUT] -> objects, key [o|p|IN] -> subjects for p != rdf:type;
//    key [s|1|OUT] -> the vertex's classes; no IN key for type triples
//    (core/gstore.hpp:665-790);
//  - index keys: [0|c|IN] -> members of class c (type index), [0|p|IN] ->
//    subjects of p, [0|p|OUT] -> objects of p (record_index_info,
//    core/gstore.hpp:835-870, insert_type_index_map / insert_index_map
//    :460-524).
// The layout is this library's own: per id, a hash table of 64 B buckets
// (5 slots of 32-bit segment-local keys + 1 overflow link) sized for a load of
// at most 1/2, followed by overflow buckets, an offsets array for each
// direction whose vertices are dense in their id range (those vertices then
// leave the hash table), and one contiguous int32 edge segment holding the
// id's out-lists, in-lists and index lists.
#include "wk_internal.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstdlib>
#include <atomic>
#include <cstring>
#include <functional>
#include <thread>

namespace wk {

HostStore::~HostStore() {
    if (pinned) {
        if (buckets) cudaFreeHost(buckets);
        if (edges) cudaFreeHost(edges);
        if (rowptr) cudaFreeHost(rowptr);
    } else {
        free(buckets);
        free(edges);
        free(rowptr);
    }
}

uint64_t HostStore::lookup(uint64_t vid, uint32_t pid, uint32_t dir, const int32_t **edges_out) const {
    *edges_out = nullptr;
    if (pid < 1 || (int32_t)pid > num_ids || vid >= 0x7fffffffull || dir > 1u) return 0;
    const PredSeg &sg = segs[pid];
    if (vid != 0 && sg.dn[dir]) {
        const uint64_t x = vid - sg.dvmin[dir];
        if (vid < sg.dvmin[dir] || x >= sg.dn[dir]) return 0;
        const uint32_t *rp = rowptr + sg.rp_off + (dir ? sg.rp_entries(0) : 0);
        if (rp[x + 1] == rp[x]) return 0;
        *edges_out = edges + sg.edge_off + rp[x];
        return rp[x + 1] - rp[x];
    }
    if (sg.nmain == 0) return 0;
    const uint32_t key = seg_key((uint32_t)vid, dir);
    uint32_t b = seg_bucket(key, sg.nmain);
    const Bucket *base = buckets + sg.bucket_off;
    for (uint32_t hop = 0; hop <= sg.nover; ++hop) {
        const uint32_t *w = base[b].w;
        for (int i = 0; i < WK_DATA_SLOTS; ++i) {
            if (w[i] == key) {
                *edges_out = edges + sg.edge_off + w[WK_OFF_WORD + i];
                return w[WK_DEG_WORD + i];
            }
        }
        if (w[WK_LINK_WORD] == WK_NO_LINK || w[WK_LINK_WORD] >= sg.nmain + sg.nover) return 0;
        b = w[WK_LINK_WORD];
    }
    return 0;
}

// FNV-1a over the image (segment metadata, buckets, edges, offsets arrays):
// two builds of the same triples give the same digest exactly when their
// images are byte-identical.
uint64_t HostStore::digest() const {
    uint64_t h = 1469598103934665603ull;
    auto mix = [&](const void *p, size_t n) {
        const unsigned char *c = static_cast<const unsigned char *>(p);
        for (size_t i = 0; i < n; ++i) h = (h ^ c[i]) * 1099511628211ull;
    };
    for (size_t id = 1; id < segs.size(); ++id) {
        const PredSeg &g = segs[id];
        const uint64_t meta[] = {g.bucket_off, g.nmain, g.nover, g.edge_off, g.nedges, g.nkeys, g.rp_off,
                                 g.dvmin[0], g.dvmin[1], g.dn[0], g.dn[1], g.maxdeg[0], g.maxdeg[1],
                                 g.bvmin[0], g.bvmin[1], g.bn[0], g.bn[1]};
        mix(meta, sizeof(meta));
    }
    mix(buckets, total_buckets * sizeof(Bucket));
    mix(edges, total_edges * 4);
    mix(rowptr, total_rowptr * 4);
    return h;
}

namespace {

struct KeyRec {       // one key of a segment before insertion
    uint32_t key;     // seg_key(vid, dir)
    uint32_t off;     // offset in the segment's edge list
    uint32_t deg;
};

struct SegBuild {
    std::vector<KeyRec> keys;      // after split_dense: the hashed keys only
    std::vector<int32_t> edges;
    std::vector<uint32_t> rp;      // offsets arrays of the dense directions (IN, then OUT)
    uint64_t nkeys = 0;            // every key
    uint32_t dvmin[2] = {0u, 0u}, dn[2] = {0u, 0u};
    uint32_t maxdeg[2] = {0u, 0u};
    uint32_t bvmin[2] = {0u, 0u}, bn[2] = {0u, 0u};
    int64_t triples = 0, subjects = 0, objects = 0;
};

constexpr uint64_t kBitmapBytesPerKey = 64;   // a presence bitmap may cost at most this per hashed key

// Move the vertex keys of each direction that is dense enough into an offsets
// array.  A direction's vertex keys were emitted in ascending vertex order
// with their lists back to back, which the check below confirms.
void split_dense(SegBuild &sb) {
    sb.nkeys = sb.keys.size();
    for (const KeyRec &kr : sb.keys)
        if ((kr.key >> 1) != 0) sb.maxdeg[kr.key & 1u] = std::max(sb.maxdeg[kr.key & 1u], kr.deg);
    bool dense[2] = {false, false};
    for (uint32_t dir = 0; dir < 2; ++dir) {
        uint64_t count = 0;
        uint32_t vmin = 0, vmax = 0, prev_end = 0;
        bool ordered = true;
        for (const KeyRec &kr : sb.keys) {
            const uint32_t vid = kr.key >> 1;
            if ((kr.key & 1u) != dir || vid == 0) continue;
            if (count == 0) {
                vmin = vid;
            } else if (vid <= vmax || kr.off != prev_end) {
                ordered = false;
            }
            vmax = vid;
            prev_end = kr.off + kr.deg;
            ++count;
        }
        if (count == 0 || !ordered) continue;
        const uint64_t range = (uint64_t)vmax - vmin + 1;
        if (count * WK_DENSE_RATIO < range) continue;
        dense[dir] = true;
        sb.dvmin[dir] = vmin;
        sb.dn[dir] = (uint32_t)range;
    }
    // presence bitmaps of hashed directions, appended after any offsets and neighbour arrays
    auto add_bitmaps = [&]() {
        for (uint32_t dir = 0; dir < 2; ++dir) {
            if (dense[dir]) continue;
            uint64_t count = 0;
            uint32_t vmin = 0xffffffffu, vmax = 0;
            for (const KeyRec &kr : sb.keys) {
                const uint32_t vid = kr.key >> 1;
                if ((kr.key & 1u) != dir || vid == 0) continue;
                vmin = std::min(vmin, vid);
                vmax = std::max(vmax, vid);
                ++count;
            }
            if (count == 0) continue;
            const uint64_t range = (uint64_t)vmax - vmin + 1;
            if (range / 8 > count * kBitmapBytesPerKey) continue;
            sb.bvmin[dir] = vmin;
            sb.bn[dir] = (uint32_t)range;
            const size_t base = sb.rp.size();
            sb.rp.resize(base + (size_t)((range + 31) / 32), 0u);
            uint32_t *bm = sb.rp.data() + base;
            for (const KeyRec &kr : sb.keys) {
                const uint32_t vid = kr.key >> 1;
                if ((kr.key & 1u) != dir || vid == 0) continue;
                const uint32_t x = vid - vmin;
                bm[x >> 5] |= 1u << (x & 31u);
            }
        }
    };
    if (!dense[0] && !dense[1]) {
        add_bitmaps();
        return;
    }
    std::vector<KeyRec> hashed;
    for (uint32_t dir = 0; dir < 2; ++dir) {
        if (!dense[dir]) continue;
        const size_t base = sb.rp.size();
        sb.rp.resize(base + (size_t)sb.dn[dir] + 1);
        uint32_t *rp = sb.rp.data() + base;
        uint64_t pos = 0;
        uint32_t end = 0;
        for (const KeyRec &kr : sb.keys) {
            const uint32_t vid = kr.key >> 1;
            if ((kr.key & 1u) != dir || vid == 0) continue;
            const uint64_t x = vid - sb.dvmin[dir];
            while (pos <= x) rp[pos++] = kr.off;   // absent ids before v: empty lists ending at v's
            end = kr.off + kr.deg;
        }
        while (pos <= sb.dn[dir]) rp[pos++] = end;
    }
    // neighbour arrays of dense functional directions, after both offsets arrays
    for (uint32_t dir = 0; dir < 2; ++dir) {
        if (!dense[dir] || sb.maxdeg[dir] > 1u) continue;
        const size_t base = sb.rp.size();
        sb.rp.resize(base + (size_t)sb.dn[dir], 0xffffffffu);   // -1: no neighbour
        uint32_t *nb = sb.rp.data() + base;
        for (const KeyRec &kr : sb.keys) {
            const uint32_t vid = kr.key >> 1;
            if ((kr.key & 1u) != dir || vid == 0 || kr.deg == 0) continue;
            nb[vid - sb.dvmin[dir]] = (uint32_t)sb.edges[kr.off];
        }
    }
    add_bitmaps();
    for (const KeyRec &kr : sb.keys) {
        const uint32_t vid = kr.key >> 1, dir = kr.key & 1u;
        if (vid == 0 || !dense[dir]) hashed.push_back(kr);
    }
    sb.keys.swap(hashed);
}

// From (hi,lo) pairs packed as hi<<32|lo, sorted, duplicates allowed: one key
// per hi group with the group's distinct lo values as the adjacency list.
// Returns the number of distinct pairs.
size_t emit_sorted(const uint64_t *a, size_t n, uint32_t dir, SegBuild &sb, std::vector<int32_t> *distinct_hi) {
    size_t i = 0, uniq = 0;
    while (i < n) {
        const uint32_t hi = (uint32_t)(a[i] >> 32);
        KeyRec kr;
        kr.key = seg_key(hi, dir);
        kr.off = (uint32_t)sb.edges.size();
        size_t j = i;
        uint64_t prev = ~0ull;
        while (j < n && (uint32_t)(a[j] >> 32) == hi) {
            if (a[j] != prev) {
                sb.edges.push_back((int32_t)(uint32_t)a[j]);
                prev = a[j];
                ++uniq;
            }
            ++j;
        }
        kr.deg = (uint32_t)(sb.edges.size() - kr.off);
        sb.keys.push_back(kr);
        if (distinct_hi) distinct_hi->push_back((int32_t)hi);
        i = j;
    }
    return uniq;
}

// Sort (hi,lo) pairs, dedup, and emit them as emit_sorted does.
void emit_groups(std::vector<uint64_t> &pairs, uint32_t dir, SegBuild &sb,
                 std::vector<int32_t> *distinct_hi) {
    std::sort(pairs.begin(), pairs.end());
    pairs.erase(std::unique(pairs.begin(), pairs.end()), pairs.end());
    emit_sorted(pairs.data(), pairs.size(), dir, sb, distinct_hi);
}

void add_index(uint32_t dir, const std::vector<int32_t> &list, SegBuild &sb) {
    if (list.empty()) return;
    KeyRec kr;
    kr.key = seg_key(0, dir);
    kr.off = (uint32_t)sb.edges.size();
    kr.deg = (uint32_t)list.size();
    sb.edges.insert(sb.edges.end(), list.begin(), list.end());
    sb.keys.push_back(kr);
}

template <class F>
void parallel_for(size_t n, F f) {
    int nt = (int)std::max(1u, std::min<unsigned>(std::thread::hardware_concurrency(), 64));
    std::atomic<size_t> next{0};
    auto w = [&]() {
        for (;;) {
            size_t i = next.fetch_add(1);
            if (i >= n) break;
            f(i);
        }
    };
    std::vector<std::thread> th;
    for (int i = 1; i < nt; ++i) th.emplace_back(w);
    w();
    for (auto &t : th) t.join();
}

}  // namespace

int build_host_store(const int32_t *s, const int32_t *p, const int32_t *o, int64_t n,
                     int32_t num_ids, HostStore **out) {
    if (n < 0 || (n > 0 && (!s || !p || !o)) || num_ids < 1 || num_ids >= WK_VID_BASE)
        return set_error(WK_EINVAL, "store build: bad arguments (n=%lld, num_ids=%d)", (long long)n, num_ids);
    // validate and bucket triples by predicate (counting sort)
    std::vector<int64_t> cnt((size_t)num_ids + 2, 0);
    for (int64_t i = 0; i < n; ++i) {
        int32_t pi = p[i];
        if (pi < 1 || pi > num_ids)
            return set_error(WK_EINVAL, "store build: triple %lld has predicate %d outside [1,%d]",
                             (long long)i, pi, num_ids);
        if (s[i] < WK_VID_BASE || s[i] == INT32_MAX)
            return set_error(WK_EINVAL, "store build: triple %lld has subject %d outside [2^17, 2^31-1)",
                             (long long)i, s[i]);
        if (pi == WK_TYPE_ID) {
            if (o[i] < 2 || o[i] > num_ids)
                return set_error(WK_EINVAL, "store build: type triple %lld has class %d outside [2,%d]",
                                 (long long)i, o[i], num_ids);
        } else if (o[i] < WK_VID_BASE || o[i] == INT32_MAX) {
            return set_error(WK_EINVAL, "store build: triple %lld has object %d outside [2^17, 2^31-1)",
                             (long long)i, o[i]);
        }
        cnt[(size_t)pi]++;
    }
    std::vector<int64_t> start((size_t)num_ids + 2, 0);
    for (int32_t i = 1; i <= num_ids + 1; ++i) start[(size_t)i] = start[(size_t)i - 1] + cnt[(size_t)i - 1];
    // a counting sort by p, whose runs emit_groups sorts per id
    std::vector<uint64_t> so((size_t)n);   // packed s<<32|o, grouped by p
    {
        std::vector<int64_t> at(start);
        for (int64_t i = 0; i < n; ++i)
            so[(size_t)at[(size_t)p[i]]++] = ((uint64_t)(uint32_t)s[i] << 32) | (uint32_t)o[i];
    }

    std::vector<SegBuild> sb((size_t)num_ids + 1);
    // type triples first: they feed both the type lists and the class indexes
    std::vector<std::vector<int32_t>> class_members((size_t)num_ids + 1);
    {
        const int64_t a = start[WK_TYPE_ID], b = start[WK_TYPE_ID + 1];
        std::vector<uint64_t> cs;
        std::vector<uint64_t> out_pairs(so.begin() + a, so.begin() + b);
        emit_groups(out_pairs, WK_DIR_OUT, sb[WK_TYPE_ID], nullptr);
        sb[WK_TYPE_ID].triples = (int64_t)out_pairs.size();
        cs.reserve(out_pairs.size());
        for (uint64_t x : out_pairs) cs.push_back(((x & 0xffffffffull) << 32) | (x >> 32));
        std::sort(cs.begin(), cs.end());
        sb[WK_TYPE_ID].subjects = (int64_t)sb[WK_TYPE_ID].keys.size();
        for (uint64_t x : cs) class_members[(size_t)(x >> 32)].push_back((int32_t)(uint32_t)x);
    }
    // normal predicates in parallel
    parallel_for((size_t)num_ids + 1, [&](size_t id) {
        if (id == 0) return;
        SegBuild &b = sb[id];
        if (id != WK_TYPE_ID && cnt[id] > 0) {
            std::vector<int32_t> subjects, objects;
            std::vector<uint64_t> pairs(so.begin() + start[id], so.begin() + start[id + 1]);
            emit_groups(pairs, WK_DIR_OUT, b, &subjects);
            b.triples = (int64_t)pairs.size();
            for (auto &x : pairs) x = ((x & 0xffffffffull) << 32) | (x >> 32);
            emit_groups(pairs, WK_DIR_IN, b, &objects);
            add_index(WK_DIR_IN, subjects, b);    // [0|p|IN]  subjects of p
            add_index(WK_DIR_OUT, objects, b);    // [0|p|OUT] objects of p
            b.subjects = (int64_t)subjects.size();
            b.objects = (int64_t)objects.size();
        }
        if (!class_members[id].empty()) {                    // [0|c|IN] members of c
            add_index(WK_DIR_IN, class_members[id], b);
            b.subjects += (int64_t)class_members[id].size();
            b.triples += (int64_t)class_members[id].size();
        }
    });
    std::vector<uint64_t>().swap(so);
    parallel_for((size_t)num_ids + 1, [&](size_t id) {
        if (id) split_dense(sb[id]);
    });

    // sizes and image allocation
    HostStore *hs = new HostStore();
    hs->num_ids = num_ids;
    hs->segs.resize((size_t)num_ids + 1);
    uint64_t bucket_at = 0, edge_at = 0, rp_at = 0;
    std::vector<uint64_t> nhash((size_t)num_ids + 1, 0);   // keys in the hash table
    for (size_t id = 1; id <= (size_t)num_ids; ++id) {
        PredSeg &sg = hs->segs[id];
        SegBuild &b = sb[id];
        sg.nkeys = b.nkeys;
        nhash[id] = b.keys.size();
        for (int d = 0; d < 2; ++d) {
            sg.dvmin[d] = b.dvmin[d];
            sg.dn[d] = b.dn[d];
            sg.maxdeg[d] = b.maxdeg[d];
            sg.bvmin[d] = b.bvmin[d];
            sg.bn[d] = b.bn[d];
        }
        sg.rp_off = rp_at;
        rp_at += b.rp.size();
        sg.nedges = b.edges.size();
        sg.triples = b.triples; sg.subjects = b.subjects; sg.objects = b.objects;
        if (sg.nedges > 0xffffffffull) {
            delete hs;
            return set_error(WK_EINVAL, "store build: id %zu has more than 2^32 edge entries", id);
        }
        // main buckets: keys / (5 * 0.5), at least one bucket when there are keys;
        // overflow room: worst case one bucket per 5 keys beyond the first
        const uint64_t nk = nhash[id];
        const uint64_t nm = nk ? (nk * 2 + WK_DATA_SLOTS - 1) / WK_DATA_SLOTS : 0;
        if (nm + nk / WK_DATA_SLOTS + 1 >= 0xffffffffull) {
            delete hs;
            return set_error(WK_EINVAL, "store build: id %zu has too many keys", id);
        }
        sg.nmain = (uint32_t)nm;
        sg.bucket_off = bucket_at;
        sg.edge_off = edge_at;
        if (nk) bucket_at += nm + nk / WK_DATA_SLOTS + 1;
        edge_at += sg.nedges;
    }
    // reserve the upper bound, compact after insertion
    const uint64_t bucket_cap = bucket_at ? bucket_at : 1;
    const uint64_t edge_cap = edge_at ? edge_at : 1;
    Bucket *bk_tmp = static_cast<Bucket *>(malloc(bucket_cap * sizeof(Bucket)));
    if (!bk_tmp) { delete hs; return set_error(WK_ENOMEM, "store build: out of host memory"); }

    // insertion per id in parallel: cluster chaining with a per-id overflow area
    std::vector<uint32_t> nover((size_t)num_ids + 1, 0);
    parallel_for((size_t)num_ids + 1, [&](size_t id) {
        if (id == 0) return;
        PredSeg &sg = hs->segs[id];
        if (!nhash[id]) return;
        Bucket *base = bk_tmp + sg.bucket_off;
        const uint64_t cap = (uint64_t)sg.nmain + nhash[id] / WK_DATA_SLOTS + 1;
        for (uint64_t i = 0; i < cap; ++i) {
            uint32_t *w = base[i].w;
            for (int j = 0; j < WK_DATA_SLOTS; ++j) {
                w[j] = WK_EMPTY_KEY;
                w[WK_OFF_WORD + j] = 0u;
                w[WK_DEG_WORD + j] = 0u;
            }
            w[WK_LINK_WORD] = WK_NO_LINK;
        }
        uint32_t used_over = 0;
        for (const KeyRec &kr : sb[id].keys) {
            uint32_t b = seg_bucket(kr.key, sg.nmain);
            for (;;) {
                uint32_t *w = base[b].w;
                int free_slot = -1;
                for (int i = 0; i < WK_DATA_SLOTS; ++i)
                    if (w[i] == WK_EMPTY_KEY) { free_slot = i; break; }
                if (free_slot >= 0) {
                    w[free_slot] = kr.key;
                    w[WK_OFF_WORD + free_slot] = kr.off;
                    w[WK_DEG_WORD + free_slot] = kr.deg;
                    break;
                }
                if (w[WK_LINK_WORD] != WK_NO_LINK) { b = w[WK_LINK_WORD]; continue; }
                const uint32_t nb = sg.nmain + used_over++;
                w[WK_LINK_WORD] = nb;
                b = nb;
            }
        }
        nover[id] = used_over;
    });

    // compact: final bucket offsets and copy into the (pinned if possible) image
    uint64_t total_buckets = 0;
    for (size_t id = 1; id <= (size_t)num_ids; ++id) {
        PredSeg &sg = hs->segs[id];
        sg.nover = nover[id];
        total_buckets += (uint64_t)sg.nmain + sg.nover;
    }
    const uint64_t bbytes = (total_buckets ? total_buckets : 1) * sizeof(Bucket);
    const uint64_t rbytes = (rp_at ? rp_at : 1) * 4;
    void *bp = nullptr, *ep = nullptr, *rpp = nullptr;
    bool pinned = cudaHostAlloc(&bp, bbytes, cudaHostAllocPortable) == cudaSuccess &&
                  cudaHostAlloc(&ep, edge_cap * 4, cudaHostAllocPortable) == cudaSuccess &&
                  cudaHostAlloc(&rpp, rbytes, cudaHostAllocPortable) == cudaSuccess;
    if (!pinned) {
        cudaGetLastError();
        if (bp) cudaFreeHost(bp);
        if (ep) cudaFreeHost(ep);
        if (rpp) cudaFreeHost(rpp);
        bp = aligned_alloc(WK_BUCKET_BYTES, bbytes);
        ep = malloc(edge_cap * 4);
        rpp = malloc(rbytes);
        if (!bp || !ep || !rpp) { free(bp); free(ep); free(rpp); free(bk_tmp); delete hs;
                                  return set_error(WK_ENOMEM, "store build: out of host memory"); }
    }
    hs->pinned = pinned;
    hs->buckets = static_cast<Bucket *>(bp);
    hs->edges = (int32_t *)ep;
    hs->rowptr = static_cast<uint32_t *>(rpp);
    hs->total_rowptr = rp_at;
    std::vector<uint64_t> new_off((size_t)num_ids + 1, 0);
    uint64_t at = 0;
    for (size_t id = 1; id <= (size_t)num_ids; ++id) {
        new_off[id] = at;
        at += (uint64_t)hs->segs[id].nmain + hs->segs[id].nover;
    }
    parallel_for((size_t)num_ids + 1, [&](size_t id) {
        if (id == 0) return;
        PredSeg &sg = hs->segs[id];
        const uint64_t nb = (uint64_t)sg.nmain + sg.nover;
        if (nb) std::memcpy(hs->buckets + new_off[id], bk_tmp + sg.bucket_off, nb * sizeof(Bucket));
        sg.bucket_off = new_off[id];
        if (sg.nedges) std::memcpy(hs->edges + sg.edge_off, sb[id].edges.data(), sg.nedges * 4);
        if (!sb[id].rp.empty()) std::memcpy(hs->rowptr + sg.rp_off, sb[id].rp.data(), sb[id].rp.size() * 4);
        std::vector<KeyRec>().swap(sb[id].keys);
        std::vector<int32_t>().swap(sb[id].edges);
        std::vector<uint32_t>().swap(sb[id].rp);
    });
    free(bk_tmp);
    hs->total_buckets = total_buckets;
    hs->total_edges = edge_at;
    for (size_t id = 1; id <= (size_t)num_ids; ++id) {
        hs->total_keys += hs->segs[id].nkeys;
        hs->total_over += hs->segs[id].nover;
    }
    *out = hs;
    return WK_OK;
}

}  // namespace wk
