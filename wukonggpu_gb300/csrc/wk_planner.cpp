// Statistics and the statistics-based query planner.
//
// Statistics: GStore::generate_statistic (core/gstore.hpp:1010-1127) followed
// by the one-server gather of data_statistic::gather_data
// (core/data_statistic.hpp:66-157).  Every stored key is counted, index keys
// included, exactly as the reference iterates every slot of its store:
//   IN key  [v|p|IN]  : triples[p] += deg, objects[p] += 1, (IN, p) joins v's list
//   OUT key [v|p|OUT] : subjects[p] += 1, (OUT, p) joins v's list; for p = type,
//                       every class c of v: type_subjects[c] += 1,
//                       subjects[c] += 1, (OUT, c) joins v's list
//   correlation[(p1,p2)] counts, over every vertex, each pair of its list by
//                       direction (out_out, out_in, in_in, in_out) with p1 < p2
//   gather (one server): objects[type] = number of classes seen,
//                       triples[type] = sum of type_subjects
//
// Planner: Planner::generate_plan (core/planner.hpp:927-1028) -- the constant
// pattern moved first, the depth-first search com_traverse (:123-323) with
// the correlation pruning com_prune (:537-589), the per-variable selectivity
// stacks (Minimum_maintenance :40-102, new_add_selectivity / unadd_selectivity
// :591-664) and the small-query cut-off (COST_THRESHOLD 350), then variables
// renumbered in plan order.  Ties and floating-point order follow the
// reference so that the same statistics give the same plan.
#include "wk_runtime.h"
#include "wk_stats.h"

#include <algorithm>
#include <mutex>
#include <atomic>
#include <cstring>
#include <limits>
#include <memory>
#include <thread>
#include <unordered_map>
#include <vector>

namespace wk {

namespace {

struct DirP {
    uint32_t vid;
    uint32_t pd;   // predicate or class id << 1 | direction
    uint32_t p() const { return pd >> 1; }
    uint32_t dir() const { return pd & 1u; }
};

}  // namespace

namespace {

template <class F>
void par_for(size_t n, F f) {
    const int nt = (int)std::max(1u, std::min<unsigned>(std::thread::hardware_concurrency(), 64));
    std::atomic<size_t> next{0};
    auto w = [&]() {
        for (;;) {
            const size_t i = next.fetch_add(1);
            if (i >= n) break;
            f(i);
        }
    };
    std::vector<std::thread> th;
    for (int i = 1; i < nt; ++i) th.emplace_back(w);
    w();
    for (auto &t : th) t.join();
}

// every pair of one vertex's list, by direction, into pp (p1 < p2 order)
void count_pairs(const DirP *l, size_t k, std::vector<FourNum> &pp, size_t W) {
    for (size_t x = 0; x < k; ++x) {
        for (size_t y = x + 1; y < k; ++y) {
            int p1, d1, p2, d2;
            if (l[x].p() < l[y].p()) {
                p1 = (int)l[x].p(); d1 = (int)l[x].dir(); p2 = (int)l[y].p(); d2 = (int)l[y].dir();
            } else {
                p1 = (int)l[y].p(); d1 = (int)l[y].dir(); p2 = (int)l[x].p(); d2 = (int)l[x].dir();
            }
            FourNum &f = pp[(size_t)p1 * W + (size_t)p2];
            if (d1 == WK_DIR_OUT && d2 == WK_DIR_OUT) f.out_out++;
            if (d1 == WK_DIR_OUT && d2 == WK_DIR_IN) f.out_in++;
            if (d1 == WK_DIR_IN && d2 == WK_DIR_IN) f.in_in++;
            if (d1 == WK_DIR_IN && d2 == WK_DIR_OUT) f.in_out++;
        }
    }
}

}  // namespace

// Build the statistics from the host image, in parallel: per segment, the
// counts and each key's (vertex, predicate/class, direction) entry; then the
// entries are partitioned by vertex range, each range sorted by vertex, and
// the pairs of every vertex's list counted.  The maps get an entry exactly
// when the reference's iteration would create one (po[type] counts the
// classes seen).  Pairs of one predicate with itself depend on the order of a
// vertex's entries, but the planner never reads them (com_prune returns early
// when pre_p == p).
Stats *build_stats(const HostStore &hs) {
    Stats *st = new Stats();
    const int N = hs.num_ids;
    st->num_ids = N;
    const size_t W = (size_t)(N + 1);
    st->pp.assign(W * W, FourNum());

    // 1. entries per segment (a key, plus one per class of a typed vertex)
    std::vector<uint64_t> cnt((size_t)N + 2, 0);
    struct SegCounts {
        int64_t pt = 0, ps = 0, po = 0;
        bool has_in = false, has_out = false;
    };
    std::vector<SegCounts> sc((size_t)N + 1);
    std::vector<int64_t> class_members(W, 0);   // from the type segment
    par_for((size_t)N, [&](size_t k) {
        const int id = (int)k + 1;
        uint64_t c = 0;
        SegCounts &x = sc[(size_t)id];
        hs.for_each_key(id, [&](uint32_t, uint32_t dir, uint32_t, uint32_t deg) {
            ++c;
            if (dir == WK_DIR_IN) {
                x.has_in = true;
                x.pt += deg;
                x.po += 1;
            } else {
                x.has_out = true;
                x.ps += 1;
                if (id == WK_TYPE_ID) c += deg;
            }
        });
        cnt[(size_t)id] = c;
    });
    std::vector<uint64_t> at((size_t)N + 2, 0);
    for (int id = 1; id <= N; ++id) at[(size_t)id + 1] = at[(size_t)id] + cnt[(size_t)id];
    const size_t n = at[(size_t)N + 1];
    std::vector<DirP> lists(n);
    uint32_t max_vid = 0;
    std::mutex mu;
    par_for((size_t)N, [&](size_t k) {
        const int id = (int)k + 1;
        const PredSeg &sg = hs.segs[(size_t)id];
        const uint32_t pid = (uint32_t)id;
        DirP *o = lists.data() + at[(size_t)id];
        uint32_t mv = 0;
        std::vector<int64_t> local_classes;
        if (id == WK_TYPE_ID) local_classes.assign(W, 0);
        hs.for_each_key(id, [&](uint32_t vid, uint32_t dir, uint32_t off, uint32_t deg) {
            mv = std::max(mv, vid);
            *o++ = DirP{vid, (pid << 1) | dir};
            if (dir == WK_DIR_OUT && id == WK_TYPE_ID) {
                const int32_t *e = hs.edges + sg.edge_off + off;
                for (uint32_t q = 0; q < deg; ++q) {
                    local_classes[(size_t)e[q]] += 1;
                    *o++ = DirP{vid, ((uint32_t)e[q] << 1) | (uint32_t)WK_DIR_OUT};
                }
            }
        });
        std::lock_guard<std::mutex> lk(mu);
        max_vid = std::max(max_vid, mv);
        if (id == WK_TYPE_ID) class_members.swap(local_classes);
    });

    // 2. partition by vertex range, then per range: sort by vertex, count pairs
    const size_t kBuckets = 4096;
    const uint64_t span = (uint64_t)max_vid + 1;
    auto bucket_of_vid = [&](uint32_t v) { return (size_t)(((uint64_t)v * kBuckets) / span); };
    const size_t nchunk = 64;
    std::vector<std::vector<uint64_t>> hist(nchunk, std::vector<uint64_t>(kBuckets, 0));
    par_for(nchunk, [&](size_t c) {
        const size_t a = n * c / nchunk, b = n * (c + 1) / nchunk;
        for (size_t i = a; i < b; ++i) hist[c][bucket_of_vid(lists[i].vid)]++;
    });
    std::vector<uint64_t> bstart(kBuckets + 1, 0);
    std::vector<std::vector<uint64_t>> cur(nchunk, std::vector<uint64_t>(kBuckets, 0));
    {
        uint64_t acc = 0;
        for (size_t k = 0; k < kBuckets; ++k) {
            bstart[k] = acc;
            for (size_t c = 0; c < nchunk; ++c) {
                cur[c][k] = acc;
                acc += hist[c][k];
            }
        }
        bstart[kBuckets] = acc;
    }
    std::vector<DirP> part(n);
    par_for(nchunk, [&](size_t c) {
        const size_t a = n * c / nchunk, b = n * (c + 1) / nchunk;
        for (size_t i = a; i < b; ++i) part[cur[c][bucket_of_vid(lists[i].vid)]++] = lists[i];
    });
    std::vector<DirP>().swap(lists);
    const int nt = (int)std::max(1u, std::min<unsigned>(std::thread::hardware_concurrency(), 64));
    std::vector<std::vector<FourNum>> acc_pp((size_t)nt);
    std::atomic<size_t> next{0};
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t) {
        th.emplace_back([&, t]() {
            std::vector<FourNum> &pp = acc_pp[(size_t)t];
            pp.assign(W * W, FourNum());
            for (;;) {
                const size_t k = next.fetch_add(1);
                if (k >= kBuckets) break;
                DirP *l = part.data() + bstart[k];
                const size_t m = bstart[k + 1] - bstart[k];
                std::stable_sort(l, l + m, [](const DirP &x, const DirP &y) { return x.vid < y.vid; });
                size_t i = 0;
                while (i < m) {
                    size_t j = i;
                    while (j < m && l[j].vid == l[i].vid) ++j;
                    count_pairs(l + i, j - i, pp, W);
                    i = j;
                }
            }
        });
    }
    for (auto &x : th) x.join();
    for (auto &pp : acc_pp)
        for (size_t i = 0; i < pp.size(); ++i) {
            st->pp[i].out_out += pp[i].out_out;
            st->pp[i].out_in += pp[i].out_in;
            st->pp[i].in_in += pp[i].in_in;
            st->pp[i].in_out += pp[i].in_out;
        }

    // 3. per-predicate counts, then the one-server gather (core/data_statistic.hpp:150-156)
    for (int id = 1; id <= N; ++id) {
        const SegCounts &x = sc[(size_t)id];
        if (x.has_in) {
            st->pt[id] += x.pt;
            st->po[id] += x.po;
        }
        if (x.has_out) st->ps[id] += x.ps;
    }
    for (size_t c = 0; c < W; ++c)
        if (class_members[c] > 0) {
            st->tys[(int)c] += class_members[c];
            st->ps[(int)c] += class_members[c];
        }
    st->po[WK_TYPE_ID] = (int64_t)st->tys.size();
    int64_t tri = 0;
    for (auto &kv : st->tys) tri += kv.second;
    st->pt[WK_TYPE_ID] = tri;
    return st;
}

namespace {

constexpr double kCostThreshold = 350.0;   // COST_THRESHOLD, core/planner.hpp:18

struct SelectRecord {
    int p, d;
    double v;
};

// Minimum_maintenance (core/planner.hpp:40-102): a stack whose top() is the
// element that first reached the current minimum of v.
struct MinStack {
    std::vector<SelectRecord> s0, s1;
    std::vector<int> order;
    void push(const SelectRecord &r) {
        if (s0.empty() || s0.back().v > r.v) { s0.push_back(r); order.push_back(0); }
        else { s1.push_back(r); order.push_back(1); }
    }
    void pop() {
        if (order.empty()) return;
        if (order.back() == 0) s0.pop_back();
        else s1.pop_back();
        order.pop_back();
    }
    bool top(SelectRecord &r) const {
        if (order.empty()) return false;
        r = s0.back();
        return true;
    }
    bool empty() const { return s0.empty(); }
};

class Planner {
  public:
    explicit Planner(Stats &s) : st_(s) {}

    // returns 0 with a plan, 1 when the query is proved empty, -1 when no order exists
    int generate(std::vector<int64_t> &cmd, double *cost_out) {
        min_path_.clear();
        path_.clear();
        is_empty_ = false;
        min_cost_ = std::numeric_limits<double>::max();
        // the first pattern holding a constant goes first (core/planner.hpp:942-962)
        for (size_t i = 0; i + 3 < cmd.size(); i += 4) {
            if (cmd[i] >= WK_VID_BASE || cmd[i + 3] >= WK_VID_BASE) {
                if (i == 0) break;
                for (int k = 0; k < 4; ++k) std::swap(cmd[i + (size_t)k], cmd[(size_t)k]);
                break;
            }
        }
        triples_ = cmd;
        n_ = (int)(cmd.size() / 4);
        sel_.clear();
        undo_.clear();
        traverse(0u, 0.0, 0.0);
        if (is_empty_) return 1;
        if (min_path_.empty()) return -1;
        // renumber variables in plan order (core/planner.hpp:991-1003)
        std::unordered_map<int64_t, int64_t> conv;
        for (auto &x : min_path_) {
            if (x < 0) {
                auto it = conv.find(x);
                if (it == conv.end()) {
                    const int64_t v = -1 - (int64_t)conv.size();
                    conv.emplace(x, v);
                    x = v;
                } else {
                    x = it->second;
                }
            }
        }
        cmd = min_path_;
        if (cost_out) *cost_out = min_cost_;
        return 0;
    }

  private:
    Stats &st_;
    std::vector<int64_t> triples_, path_, min_path_;
    double min_cost_ = 0.0;
    bool is_empty_ = false;
    int n_ = 0;
    std::unordered_map<int, std::unique_ptr<MinStack>> sel_;
    std::vector<std::vector<int>> undo_;

    double pt(int p) { return (double)st_.pt[p]; }
    double ps(int p) { return (double)st_.ps[p]; }
    double po(int p) { return (double)st_.po[p]; }

    MinStack &fresh(int var) {
        sel_[var].reset(new MinStack());
        return *sel_[var];
    }
    MinStack &stack_of(int var) {
        auto &u = sel_[var];
        if (!u) u.reset(new MinStack());
        return *u;
    }
    bool has_sel(int var) {
        auto it = sel_.find(var);
        return it != sel_.end() && it->second && !it->second->empty();
    }

    void push4(int64_t a, int64_t b, int64_t c, int64_t d) {
        path_.push_back(a); path_.push_back(b); path_.push_back(c); path_.push_back(d);
    }
    void pop4() { path_.resize(path_.size() - 4); }

    // com_prune (core/planner.hpp:537-589)
    double prune(double pre_results, int pre_p, int pre_d, int p, int d) {
        if (pre_p == p) return pre_results;
        double x = 0.0, y = 0.0;
        auto four = [&](int a, int b) -> const FourNum & {
            static const FourNum zero;
            const FourNum *f = st_.pair_c(a, b);
            return f ? *f : zero;
        };
        if (pre_d == WK_DIR_OUT && d == WK_DIR_OUT) {
            x = (double)(pre_p < p ? four(pre_p, p).out_out : four(p, pre_p).out_out);
            y = ps(pre_p);
        }
        if (pre_d == WK_DIR_IN && d == WK_DIR_OUT) {
            x = (double)(pre_p < p ? four(pre_p, p).in_out : four(p, pre_p).out_in);
            y = po(pre_p);
        }
        if (pre_d == WK_DIR_IN && d == WK_DIR_IN) {
            x = (double)(pre_p < p ? four(pre_p, p).in_in : four(p, pre_p).in_in);
            y = po(pre_p);
        }
        if (pre_d == WK_DIR_OUT && d == WK_DIR_IN) {
            x = (double)(pre_p < p ? four(pre_p, p).out_in : four(p, pre_p).in_out);
            y = ps(pre_p);
        }
        const double r = pre_results * (x / y);
        if (x == 0.0) is_empty_ = true;
        return r;
    }

    // new_add_selectivity (core/planner.hpp:591-648)
    void add_sel(int o1, int p, int o2) {
        std::vector<int> touched;
        if (o1 < 0 && o2 > 0) {
            double v;
            int pp = p;
            if (p == WK_TYPE_ID) { v = ps(o2); pp = o2; }
            else v = ps(p) / po(p);
            stack_of(o1).push(SelectRecord{pp, WK_DIR_OUT, v});
            touched.push_back(o1);
        } else if (o2 < 0 && o1 > 0) {
            stack_of(o2).push(SelectRecord{p, WK_DIR_IN, po(p) / ps(p)});
            touched.push_back(o2);
        } else if (o1 < 0 && o2 < 0) {
            stack_of(o1).push(SelectRecord{p, WK_DIR_OUT, ps(p)});
            stack_of(o2).push(SelectRecord{p, WK_DIR_IN, po(p)});
            touched.push_back(o1);
            touched.push_back(o2);
        }
        undo_.push_back(touched);
    }
    void unadd_sel() {
        if (undo_.empty()) return;
        for (int v : undo_.back()) sel_[v]->pop();
        undo_.pop_back();
    }

    // com_traverse (core/planner.hpp:123-323)
    bool traverse(unsigned bits, double cost, double pre_results) {
        if (bits == (1u << n_) - 1u) {
            bool ctn = true;
            if (min_cost_ == std::numeric_limits<double>::max() && cost < kCostThreshold && path_[0] >= WK_VID_BASE)
                ctn = false;   // small query: take the first complete order
            if (cost < min_cost_) {
                min_cost_ = cost;
                min_path_ = path_;
            }
            return ctn;
        }
        for (int pick = 0; pick < n_; ++pick) {
            if (bits & (1u << pick)) continue;
            const int i = 4 * pick;
            double add_cost = 0.0;
            const int o1 = (int)triples_[(size_t)i], p = (int)triples_[(size_t)i + 1],
                      d = (int)triples_[(size_t)i + 2], o2 = (int)triples_[(size_t)i + 3];
            if (path_.empty()) {
                if (o1 < 0 && o2 < 0) {
                    // start from the predicate index: subjects ...
                    push4(p, 0, WK_DIR_IN, o1);
                    add_cost = ps(p);
                    double nc = cost + add_cost;
                    if (nc > min_cost_) { pop4(); continue; }
                    fresh(o1).push(SelectRecord{p, d, ps(p)});
                    bool ctn = traverse(bits, nc, add_cost);
                    sel_[o1]->pop();
                    if (!ctn) return ctn;
                    pop4();
                    // ... or objects
                    push4(p, 0, WK_DIR_OUT, o2);
                    add_cost = po(p);
                    nc = cost + add_cost;
                    if (nc > min_cost_) { pop4(); continue; }
                    fresh(o2).push(SelectRecord{p, WK_DIR_IN, po(p)});
                    ctn = traverse(bits, nc, add_cost);
                    sel_[o2]->pop();
                    if (!ctn) return ctn;
                    pop4();
                }
                if (o1 > 0) {
                    push4(o1, p, d, o2);
                    add_cost = pt(p) / ps(p);
                    const double nc = cost + add_cost;
                    if (nc > min_cost_) { pop4(); continue; }
                    add_sel(o1, p, o2);
                    bool ctn = traverse(bits | (1u << pick), nc, add_cost);
                    unadd_sel();
                    if (!ctn) return ctn;
                    pop4();
                } else if (o2 > 0) {
                    push4(o2, p, WK_DIR_IN, o1);
                    if (p == WK_TYPE_ID) add_cost = ps(o2);
                    else add_cost = pt(p) / po(p);
                    const double nc = cost + add_cost;
                    if (nc > min_cost_) { pop4(); continue; }
                    add_sel(o1, p, o2);
                    bool ctn = traverse(bits | (1u << pick), nc, add_cost);
                    unadd_sel();
                    if (!ctn) return ctn;
                    pop4();
                }
            } else {
                if (has_sel(o1)) {
                    push4(o1, p, d, o2);
                    SelectRecord sr{};
                    sel_[o1]->top(sr);
                    double pr;
                    if (p == WK_TYPE_ID && o2 > 0) {
                        pr = prune(pre_results, sr.p, sr.d, o2, WK_DIR_OUT);
                        add_cost = pr;
                    } else if (o2 >= 0) {
                        pr = prune(pre_results, sr.p, sr.d, p, WK_DIR_OUT);
                        pr = pr / po(p);
                        add_cost = pr * (pt(p) / ps(p));
                    } else {
                        pr = prune(pre_results, sr.p, sr.d, p, WK_DIR_OUT);
                        add_cost = pr * (pt(p) / ps(p));
                    }
                    const double nc = cost + add_cost;
                    if (nc > min_cost_) { pop4(); continue; }
                    add_sel(o1, p, o2);
                    bool ctn = traverse(bits | (1u << pick), nc, add_cost);
                    unadd_sel();
                    if (!ctn) return ctn;
                    pop4();
                }
                if (has_sel(o2)) {
                    push4(o2, p, WK_DIR_IN, o1);
                    SelectRecord sr{};
                    sel_[o2]->top(sr);
                    double pr = prune(pre_results, sr.p, sr.d, p, WK_DIR_IN);
                    if (o1 >= 0) pr = pr / ps(p);
                    add_cost = pr * (pt(p) / po(p));
                    const double nc = cost + add_cost;
                    if (nc > min_cost_) { pop4(); continue; }
                    add_sel(o1, p, o2);
                    bool ctn = traverse(bits | (1u << pick), nc, add_cost);
                    unadd_sel();
                    if (!ctn) return ctn;
                    pop4();
                }
            }
        }
        return true;
    }
};

}  // namespace

int plan_query(Stats &st, std::vector<int64_t> &cmd, double *cost) {
    Planner p(st);
    return p.generate(cmd, cost);
}

void free_stats(Stats *s) { delete s; }

}  // namespace wk

using namespace wk;

Stats &wk::stats_of(wk_ctx *ctx) {
    if (!ctx->store->stats) ctx->store->stats.reset(build_stats(*ctx->store->hs), free_stats);
    return *ctx->store->stats;
}

extern "C" int wk_plan(wk_ctx *ctx, const int64_t *cmd_in, int32_t n, int64_t *cmd_out, int32_t *n_out,
                       double *est_cost, int32_t *proved_empty) {
    if (!ctx || !cmd_in || !cmd_out || !n_out || n <= 0 || n > 10)
        return set_error(WK_EINVAL, "wk_plan: bad arguments (1..10 patterns)");
    if (!ctx->store) return set_error(WK_ENOSTORE, "wk_plan: no store built");
    if (proved_empty) *proved_empty = 0;
    if (!triple_form(cmd_in, n)) {   // already executable (IN steps, an index start): run as written
        *n_out = 0;
        if (est_cost) *est_cost = std::numeric_limits<double>::infinity();
        return WK_OK;
    }
    if (!ctx->store->stats) ctx->store->stats.reset(build_stats(*ctx->store->hs), free_stats);
    std::vector<int64_t> cmd(cmd_in, cmd_in + (size_t)n * 4);
    double cost = 0.0;
    const int r = plan_query(*ctx->store->stats, cmd, &cost);
    if (r == 1) {
        if (proved_empty) *proved_empty = 1;
        *n_out = 0;
        if (est_cost) *est_cost = 0.0;
        return WK_OK;
    }
    if (r < 0 || cmd.empty()) {
        // no complete order: the reference returns an empty plan here (for
        // example when every pattern starts from the same constant, since a
        // constant never carries a selectivity record)
        *n_out = 0;
        if (est_cost) *est_cost = std::numeric_limits<double>::infinity();
        return WK_OK;
    }
    const int32_t m = (int32_t)(cmd.size() / 4);
    if (m > *n_out) return set_error(WK_EOVERFLOW, "wk_plan: plan has %d patterns, room for %d", m, *n_out);
    std::memcpy(cmd_out, cmd.data(), cmd.size() * sizeof(int64_t));
    *n_out = m;
    if (est_cost) *est_cost = cost;
    return WK_OK;
}

extern "C" int wk_stat_get(wk_ctx *ctx, int32_t which, int32_t a, int32_t b, int64_t *out4) {
    if (!ctx || !out4) return set_error(WK_EINVAL, "wk_stat_get: null");
    if (!ctx->store) return set_error(WK_ENOSTORE, "wk_stat_get: no store built");
    if (!ctx->store->stats) ctx->store->stats.reset(build_stats(*ctx->store->hs), free_stats);
    Stats &s = *ctx->store->stats;
    out4[0] = out4[1] = out4[2] = out4[3] = 0;
    switch (which) {
        case 0: out4[0] = s.pt.count(a) ? s.pt[a] : 0; break;
        case 1: out4[0] = s.ps.count(a) ? s.ps[a] : 0; break;
        case 2: out4[0] = s.po.count(a) ? s.po[a] : 0; break;
        case 3: out4[0] = s.tys.count(a) ? s.tys[a] : 0; break;
        case 4: {
            const FourNum *f = s.pair_c(a, b);
            if (f) { out4[0] = f->out_out; out4[1] = f->out_in; out4[2] = f->in_in; out4[3] = f->in_out; }
            break;
        }
        default: return set_error(WK_EINVAL, "wk_stat_get: which %d", which);
    }
    return WK_OK;
}
