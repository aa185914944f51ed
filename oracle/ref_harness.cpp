// Reference harness -- TEST INFRASTRUCTURE ONLY.
//
// Besides the store, the harness exposes the reference's statistics and
// planner: GStore::generate_statistic fills a data_statistic, the one-server
// part of data_statistic::gather_data (core/data_statistic.hpp:66-157:
// global maps = local maps, then the two type fix-ups) is restated, and
// Planner::generate_plan runs on it unchanged.
//
// Compiles the reference's own store, core/gstore.hpp, from the reference
// sources in place (see the `ref` target of oracle/Makefile: the reference
// headers are reached through symlinks, the missing network/RDMA headers and
// the TBB/boost container names through oracle/ref_shim/).  The store is
// filled exactly as the reference loader does it for one server:
//   - triples are split over nthread_parallel_load (11) loader threads by
//     s % 11 (out-edges) and o % 11 (in-edges), each part sorted with the
//     reference's edge_sort_by_spo / edge_sort_by_ops and deduplicated
//     (DGraph::aggregate_data, core/dgraph.hpp:288-325);
//   - GStore::init sizes the per-predicate main headers (core/gstore.hpp:600);
//   - the 11 threads run GStore::insert_normal concurrently with its
//     per-predicate barrier (core/dgraph.hpp:444-463, core/gstore.hpp:665);
//   - GStore::finish_pred_metas (core/gstore.hpp:957).
// Lookups go through GStore::get_edges_global with one server.  The CPU
// engine's step loops (core/engine.hpp:96-255) are restated below over those
// lookups; they are a few lines each and carry no state of their own.
#include <fcntl.h>
#include <pthread.h>
#include <unistd.h>

#include <algorithm>
#include <cstdlib>
#include <new>
#include <cstdint>
#include <thread>
#include <vector>

#include "gstore.hpp"   // the reference store, compiled from its own sources
#include "planner.hpp"  // the reference statistics planner

namespace {

struct RefStore {
    Mem *mem;
    GStore *g;
    int32_t num_ids;
};

void dedup(std::vector<triple_t> &v) {
    if (v.size() <= 1) return;
    size_t n = 1;
    for (size_t i = 1; i < v.size(); ++i) {
        if (v[i].s == v[n - 1].s && v[i].p == v[n - 1].p && v[i].o == v[n - 1].o) continue;
        v[n++] = v[i];
    }
    v.resize(n);
}

int64_t lookup(RefStore *r, int64_t vid, int64_t pid, int64_t dir, edge_t **out) {
    int sz = 0;
    *out = r->g->get_edges_global(0, vid, dir, pid, &sz);
    return sz;
}

}  // namespace

extern "C" {

void *ref_build(const int32_t *s, const int32_t *p, const int32_t *o, int64_t n, int32_t num_ids,
                int32_t keys_million, int32_t memstore_mb) {
    global_num_servers = 1;
    global_num_engines = 4;
    global_num_keys_million = keys_million;
    global_memstore_size_gb = (memstore_mb + 1023) / 1024;
    RefStore *r = new RefStore();
    r->num_ids = num_ids;
    r->mem = new Mem((uint64_t)memstore_mb << 20);
    // GStore's constructor leaves some counters uninitialised (last_ext among
    // them, core/gstore.hpp:560-597), so the object is built in zero-filled
    // storage, the state a fresh process gives it.
    void *raw = calloc(1, sizeof(GStore));
    r->g = new (raw) GStore(0, r->mem, num_ids);
    std::vector<std::vector<triple_t>> spo(nthread_parallel_load), ops(nthread_parallel_load);
    for (int64_t i = 0; i < n; ++i) {
        triple_t t((uint64_t)s[i], (uint64_t)p[i], (uint64_t)o[i]);
        spo[t.s % nthread_parallel_load].push_back(t);
        ops[t.o % nthread_parallel_load].push_back(t);
    }
    for (int t = 0; t < nthread_parallel_load; ++t) {
        std::sort(spo[t].begin(), spo[t].end(), edge_sort_by_spo());
        dedup(spo[t]);
        std::sort(ops[t].begin(), ops[t].end(), edge_sort_by_ops());
        dedup(ops[t]);
    }
    // the reference loader reports progress on stdout; keep it out of the caller's output
    fflush(stdout);
    const int saved = dup(1), devnull = open("/dev/null", O_WRONLY);
    if (saved >= 0 && devnull >= 0) dup2(devnull, 1);
    r->g->init(spo, ops);
    std::vector<std::thread> th;
    for (int t = 0; t < nthread_parallel_load; ++t)
        th.emplace_back([r, t, &spo, &ops]() { r->g->insert_normal(t, spo[t], ops[t]); });
    for (auto &x : th) x.join();
    r->g->finish_pred_metas();
    fflush(stdout);
    if (saved >= 0) { dup2(saved, 1); close(saved); }
    if (devnull >= 0) close(devnull);
    return r;
}

void ref_free(void *h) {
    RefStore *r = (RefStore *)h;
    if (!r) return;
    r->g->~GStore();
    free(r->g);
    delete r->mem;
    delete r;
}

// degree of [vid|pid|dir]; copies up to cap neighbours into out
int64_t ref_get_edges(void *h, int64_t vid, int32_t pid, int32_t dir, int32_t *out, int64_t cap) {
    edge_t *e = nullptr;
    int64_t sz = lookup((RefStore *)h, vid, pid, dir, &e);
    for (int64_t k = 0; k < sz && k < cap; ++k) out[k] = (int32_t)e[k].val;
    return sz;
}

// Enumerate stored keys: slot cursor in, next data slot out (-1 at the end).
int64_t ref_next_key(void *h, int64_t cursor, int64_t *vid, int32_t *pid, int32_t *dir, int64_t *deg) {
    RefStore *r = (RefStore *)h;
    vertex_t *v = r->g->get_vertices_ptr();
    const uint64_t ns = r->g->get_num_slots();
    for (uint64_t i = (uint64_t)cursor; i < ns; ++i) {
        if (i % 8 == 7) continue;            // link slot of the bucket
        if (v[i].key.is_empty()) continue;
        *vid = (int64_t)v[i].key.vid;
        *pid = (int32_t)v[i].key.pid;
        *dir = (int32_t)v[i].key.dir;
        *deg = (int64_t)v[i].ptr.size;
        return (int64_t)i;
    }
    return -1;
}

// Whole query: the CPU engine's steps with execute_one_step's dispatch
// (core/gpu_engine.hpp:395-467; index lists taken whole, i.e.
// global_mt_threshold = 1).  Returns 0, or -1 on an unsupported shape.
// *out is malloc'ed (free with ref_free_table).
int ref_execute(void *h, const int64_t *cmd, int32_t npat, int32_t **out, int64_t *rows, int32_t *cols,
                int64_t *step_rows) {
    RefStore *r = (RefStore *)h;
    std::vector<int> table, next;
    int col = 0;
    for (int32_t i = 0; i < npat; ++i) {
        const int64_t start = cmd[i * 4], pid = cmd[i * 4 + 1], d = cmd[i * 4 + 2], end = cmd[i * 4 + 3];
        next.clear();
        edge_t *e;
        auto vt = [&](int64_t v) { return v >= 0 ? 2 : ((-v > col) ? 1 : 0); };
        if (i == 0 && is_tpid((int)start)) {
            int sz = 0;
            e = r->g->get_index_edges_local(0, start, d, &sz);
            for (int k = 0; k < sz; ++k) next.push_back((int)e[k].val);
            col = 1;
        } else if (vt(start) == 2 && vt(end) == 1) {
            int64_t sz = lookup(r, start, pid, d, &e);
            for (int64_t k = 0; k < sz; ++k) next.push_back((int)e[k].val);
            col = 1;
        } else if (vt(start) == 0 && vt(end) == 1) {
            const int64_t sc = -start - 1;
            const size_t nr = col ? table.size() / col : 0;
            for (size_t rr = 0; rr < nr; ++rr) {
                int64_t sz = lookup(r, (int64_t)(uint32_t)table[rr * col + sc], pid, d, &e);
                for (int64_t k = 0; k < sz; ++k) {
                    next.insert(next.end(), table.begin() + rr * col, table.begin() + (rr + 1) * col);
                    next.push_back((int)e[k].val);
                }
            }
            col += 1;
        } else if (vt(start) == 0 && (vt(end) == 0 || vt(end) == 2)) {
            const int64_t sc = -start - 1;
            const size_t nr = col ? table.size() / col : 0;
            for (size_t rr = 0; rr < nr; ++rr) {
                int64_t sz = lookup(r, (int64_t)(uint32_t)table[rr * col + sc], pid, d, &e);
                const int target = vt(end) == 0 ? table[rr * col + (-end - 1)] : (int)end;
                for (int64_t k = 0; k < sz; ++k) {
                    if ((int)e[k].val == target) {
                        next.insert(next.end(), table.begin() + rr * col, table.begin() + (rr + 1) * col);
                        break;
                    }
                }
            }
        } else {
            return -1;
        }
        table.swap(next);
        if (step_rows) step_rows[i] = col ? (int64_t)(table.size() / col) : 0;
    }
    *rows = col ? (int64_t)(table.size() / col) : 0;
    *cols = col;
    *out = (int32_t *)malloc((table.size() + 1) * sizeof(int32_t));
    if (!table.empty()) std::copy(table.begin(), table.end(), *out);
    return 0;
}

void ref_free_table(int32_t *p) { free(p); }

// Order-independent content digest, same definition as orc_digest in wk_oracle.c.
static inline uint64_t dmix(uint64_t x) {
    x ^= x >> 31; x *= 0x7fb5d329728ea185ull; x ^= x >> 27; x *= 0x81dadef4bc2dd44dull; x ^= x >> 33;
    return x;
}
uint64_t ref_digest(void *h, int64_t *nkeys, int64_t *nedges) {
    RefStore *r = (RefStore *)h;
    vertex_t *v = r->g->get_vertices_ptr();
    edge_t *e = r->g->get_edges_ptr();
    const uint64_t ns = r->g->get_num_slots();
    uint64_t d = 0;
    int64_t k = 0, ne = 0;
    for (uint64_t i = 0; i < ns; ++i) {
        if (i % 8 == 7 || v[i].key.is_empty()) continue;
        const uint64_t key = ((uint64_t)v[i].key.vid << 18) | ((uint64_t)v[i].key.pid << 1) | (uint64_t)v[i].key.dir;
        const uint64_t sz = v[i].ptr.size, off = v[i].ptr.off;
        uint64_t a = 0;
        for (uint64_t j = 0; j < sz; ++j) a += dmix((uint64_t)e[off + j].val);
        d += dmix(key ^ dmix(sz) ^ dmix(a + 0x9e37));
        ++k;
        ne += (int64_t)sz;
    }
    *nkeys = k;
    *nedges = ne;
    return d;
}


}  // extern "C"

namespace {
struct RefStats {
    data_statistic st;
    boost::mpi::communicator world;
};
}  // namespace

extern "C" {

void *ref_stats(void *h) {
    RefStore *r = (RefStore *)h;
    RefStats *rs = new RefStats();
    rs->st.world = &rs->world;
    rs->st.tcp_adaptor = nullptr;
    fflush(stdout);
    const int saved = dup(1), devnull = open("/dev/null", O_WRONLY);
    if (saved >= 0 && devnull >= 0) dup2(devnull, 1);
    r->g->generate_statistic(rs->st);
    fflush(stdout);
    if (saved >= 0) { dup2(saved, 1); close(saved); }
    if (devnull >= 0) close(devnull);
    data_statistic &d = rs->st;
    // one server: the gathered maps are the local ones (core/data_statistic.hpp:83-142)
    d.global_ptcount = d.predicate_to_triple;
    d.global_pscount = d.predicate_to_subject;
    d.global_pocount = d.predicate_to_object;
    d.global_ppcount = d.correlation;
    d.global_tyscount = d.type_to_subject;
    // type predicate fix-ups (core/data_statistic.hpp:150-156)
    d.global_pocount[1] = d.global_tyscount.size();
    int triple = 0;
    for (auto &kv : d.global_tyscount) triple += kv.second;
    d.global_ptcount[1] = triple;
    return rs;
}

void ref_stats_free(void *p) { delete (RefStats *)p; }

// which: 0 triples, 1 subjects, 2 objects, 3 type members, 4 correlation pair
int ref_stat_get(void *p, int which, int a, int b, int64_t *out4) {
    data_statistic &d = ((RefStats *)p)->st;
    out4[0] = out4[1] = out4[2] = out4[3] = 0;
    auto get = [](unordered_map<int, int> &m, int k) -> int64_t { auto it = m.find(k); return it == m.end() ? 0 : it->second; };
    switch (which) {
        case 0: out4[0] = get(d.global_ptcount, a); break;
        case 1: out4[0] = get(d.global_pscount, a); break;
        case 2: out4[0] = get(d.global_pocount, a); break;
        case 3: out4[0] = get(d.global_tyscount, a); break;
        case 4: {
            auto it = d.global_ppcount.find(make_pair(a, b));
            if (it != d.global_ppcount.end()) {
                out4[0] = it->second.out_out; out4[1] = it->second.out_in;
                out4[2] = it->second.in_in; out4[3] = it->second.in_out;
            }
            break;
        }
        default: return -1;
    }
    return 0;
}

// Planner::generate_plan on the reference statistics.  Returns 0 with a plan,
// 1 when the planner reports an empty result.  *n_out in: room (patterns).
int ref_plan(void *p, const int64_t *cmd, int32_t n, int64_t *out, int32_t *n_out) {
    RefStats *rs = (RefStats *)p;
    request_or_reply req;
    req.cmd_chains.assign(cmd, cmd + (size_t)n * 4);
    Planner planner;
    fflush(stdout);
    const int saved = dup(1), devnull = open("/dev/null", O_WRONLY);
    if (saved >= 0 && devnull >= 0) dup2(devnull, 1);
    const bool ok = planner.generate_plan(req, &rs->st);
    fflush(stdout);
    if (saved >= 0) { dup2(saved, 1); close(saved); }
    if (devnull >= 0) close(devnull);
    if (!ok) { *n_out = 0; return 1; }
    const int32_t m = (int32_t)(req.cmd_chains.size() / 4);
    if (m > *n_out) return -1;
    for (size_t i = 0; i < req.cmd_chains.size(); ++i) out[i] = req.cmd_chains[i];
    *n_out = m;
    return 0;
}

}  // extern "C"
