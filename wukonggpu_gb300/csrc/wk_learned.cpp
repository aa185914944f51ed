// Features of a plan step, the statistics estimate of its cardinality, and the
// learned planner.
//
// A plan step applies one pattern to the current table.  Its 48 features:
//   0-4   kind one-hot (index start, constant start, k2u, k2k, k2c)
//   5-6   direction one-hot (IN, OUT)
//   7-9   log1p of triples, subjects, objects of the predicate (or class)
//   10-11 log1p of the average degree in the traversal direction / against it
//   12    log1p of the rows of the table before the step
//   13-14 step index / 6, bound columns / 8
//   15-17 end is a constant / a bound variable / a new variable
//   18    log1p of the class's members for a type check against a constant
//   19-22 log1p of the correlation counts {out_out, out_in, in_in, in_out}
//         between the predicate that bound the start variable and this one
//   23    log1p of the statistics estimate of the rows after the step, given
//         the rows before it (the reference planner's cost model, below)
//   24    log1p of the exact list length for an index or constant start
//   25    the start variable was bound walking against an edge (IN)
//   26-47 zero
// The model sees the embedding of the step's predicate (the class for a type
// index) beside these features.
//
// Statistics estimate of one step (the per-step add_cost of
// Planner::com_traverse, core/planner.hpp:123-323, with com_prune):
//   index start:   subjects (IN) or objects (OUT) of p; type index: members
//   constant start: triples / subjects (OUT) or triples / objects (IN)
//   later steps:   rows * (x / y) * avg degree, x / y the correlation ratio of
//                  the binding predicate and p; for a constant end the product
//                  is further divided by the objects of p, as the reference
//                  does
//
// Learned planner: beam search over join orders.  A partial plan is extended
// by every executable pattern -- oriented from a bound end, or for the first
// step from a constant, a type index or a predicate index -- and the model
// predicts the rows after each extension (a first step's rows are exact: the
// length of one stored list).  A plan's cost is the sum of the
// predicted rows of every table it builds; each level keeps the cheapest few
// partial plans (ties: lower pattern index, then OUT before IN).  The result
// has the statistics planner's output format: executable order, variables
// renumbered in binding order, an inserted index pattern when the first
// pattern joins two variables.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <unordered_map>
#include <vector>

#include "wk_runtime.h"
#include "wk_stats.h"

extern "C" {
struct wk_mlp;
int wk_mlp_predict(wk_mlp *m, const float *feats, const int32_t *pids, int64_t n, float *out);
int wk_mlp_is_trusted(wk_mlp *m);
}

namespace wk {
namespace {

constexpr int kF = 48;
enum { K_I2U = 0, K_C2U = 1, K_K2U = 2, K_K2K = 3, K_K2C = 4 };

struct VarInfo {
    int col = -1;
    int pred = 0;    // predicate (or class) whose step bound it
    int dir = 1;     // direction of that step
};

struct Step {            // one oriented step
    int kind;
    int64_t start, pid, dir, end;   // executable form; for an index start: start = index id
    int feat_pid;        // embedding id
};

double l1p(double x) { return std::log1p(std::max(0.0, x)); }

double avg_deg(Stats &st, int p, int dir) {
    const double den = dir == WK_DIR_OUT ? st.get(st.ps, p) : st.get(st.po, p);
    return den > 0 ? st.get(st.pt, p) / den : 0.0;
}

// com_prune's ratio x / y (core/planner.hpp:537-589)
double corr_ratio(Stats &st, int pre_p, int pre_d, int p, int d) {
    if (pre_p == p) return 1.0;
    const FourNum *f = pre_p < p ? st.pair_c(pre_p, p) : st.pair_c(p, pre_p);
    if (!f) return 0.0;
    double x = 0.0, y = 0.0;
    if (pre_d == WK_DIR_OUT && d == WK_DIR_OUT) { x = (double)f->out_out; y = st.get(st.ps, pre_p); }
    if (pre_d == WK_DIR_IN && d == WK_DIR_OUT) { x = (double)(pre_p < p ? f->in_out : f->out_in); y = st.get(st.po, pre_p); }
    if (pre_d == WK_DIR_IN && d == WK_DIR_IN) { x = (double)f->in_in; y = st.get(st.po, pre_p); }
    if (pre_d == WK_DIR_OUT && d == WK_DIR_IN) { x = (double)(pre_p < p ? f->out_in : f->in_out); y = st.get(st.ps, pre_p); }
    return y > 0 ? x / y : 0.0;
}

int64_t list_len(wk_ctx *ctx, uint64_t vid, int pid, int dir) {
    const int32_t *e = nullptr;
    return (int64_t)ctx->store->hs->lookup(vid, (uint32_t)pid, (uint32_t)dir, &e);
}

// statistics estimate of the rows after `s` given `rows` before it
double stats_step(wk_ctx *ctx, Stats &st, const Step &s, double rows, const VarInfo *bind) {
    switch (s.kind) {
        case K_I2U:
            if (s.pid == WK_TYPE_ID) return st.get(st.ps, (int)s.start);   // type index: class members
            return s.dir == WK_DIR_IN ? st.get(st.ps, (int)s.start) : st.get(st.po, (int)s.start);
        case K_C2U: return avg_deg(st, (int)s.pid, (int)s.dir);
        default: {
            const double ratio = bind ? corr_ratio(st, bind->pred, bind->dir, (int)s.pid, (int)s.dir) : 1.0;
            double est = rows * ratio * avg_deg(st, (int)s.pid, (int)s.dir);
            if (s.kind == K_K2C) {
                if (s.pid == WK_TYPE_ID) est = rows * ratio;
                else {
                    const double po = st.get(st.po, (int)s.pid);
                    est = po > 0 ? est / po : 0.0;
                }
            }
            (void)ctx;
            return est;
        }
    }
}

void features(wk_ctx *ctx, Stats &st, const Step &s, double rows, int step_idx, int cols, const VarInfo *bind,
              float *f) {
    std::memset(f, 0, sizeof(float) * kF);
    f[s.kind] = 1.f;
    f[5 + (s.dir == WK_DIR_OUT ? 1 : 0)] = 1.f;
    const int p = s.kind == K_I2U ? (int)s.start : (int)s.pid;
    f[7] = (float)l1p(st.get(st.pt, p));
    f[8] = (float)l1p(st.get(st.ps, p));
    f[9] = (float)l1p(st.get(st.po, p));
    f[10] = (float)l1p(avg_deg(st, p, (int)s.dir));
    f[11] = (float)l1p(avg_deg(st, p, 1 - (int)s.dir));
    f[12] = (float)l1p(rows);
    f[13] = (float)step_idx / 6.f;
    f[14] = (float)cols / 8.f;
    if (s.kind == K_K2C) f[15] = 1.f;
    else if (s.kind == K_K2K) f[16] = 1.f;
    else f[17] = 1.f;
    if (s.kind == K_K2C && s.pid == WK_TYPE_ID) f[18] = (float)l1p(st.get(st.tys, (int)s.end));
    if (bind && bind->pred > 0) {
        const int a = std::min(bind->pred, p), b = std::max(bind->pred, p);
        const FourNum *fn = st.pair_c(a, b);
        if (fn) {
            f[19] = (float)l1p((double)fn->out_out);
            f[20] = (float)l1p((double)fn->out_in);
            f[21] = (float)l1p((double)fn->in_in);
            f[22] = (float)l1p((double)fn->in_out);
        }
        f[25] = bind->dir == WK_DIR_IN ? 1.f : 0.f;
    }
    f[23] = (float)l1p(stats_step(ctx, st, s, rows, bind));
    if (s.kind == K_I2U) f[24] = (float)l1p((double)list_len(ctx, 0, (int)s.start, (int)s.dir));
    if (s.kind == K_C2U) f[24] = (float)l1p((double)list_len(ctx, (uint64_t)s.start, (int)s.pid, (int)s.dir));
}

// Walk an executable plan (cmd_chains as the engine runs it), calling
// `fn(step_index, Step, bind_info_or_null, cols_before)`.
template <class F>
int walk_plan(const int64_t *cmd, int n, F fn) {
    std::unordered_map<int64_t, VarInfo> vars;
    int cols = 0;
    for (int i = 0; i < n; ++i) {
        const int64_t st = cmd[4 * i], p = cmd[4 * i + 1], d = cmd[4 * i + 2], en = cmd[4 * i + 3];
        Step s{};
        const VarInfo *bind = nullptr;
        if (i == 0 && st > 1 && st < WK_VID_BASE) {
            s = Step{K_I2U, st, p, d, en, (int)st};
        } else if (st >= 0) {
            s = Step{K_C2U, st, p, d, en, (int)p};
        } else {
            auto it = vars.find(st);
            if (it == vars.end()) return -1;
            bind = &it->second;
            if (en < 0) s = Step{vars.count(en) ? K_K2K : K_K2U, st, p, d, en, (int)p};
            else s = Step{K_K2C, st, p, d, en, (int)p};
        }
        fn(i, s, bind, cols);
        if (s.kind == K_I2U || s.kind == K_C2U || s.kind == K_K2U) {
            VarInfo v;
            v.col = cols++;
            v.pred = s.kind == K_I2U ? (int)s.start : (int)s.pid;
            v.dir = (int)s.dir;
            vars[en] = v;
        }
    }
    return 0;
}

}  // namespace
}  // namespace wk

using namespace wk;

// Features of every step of an executable plan.  true_rows (may be null)
// holds the rows after each step: step i then sees the true rows before it
// (as in training).  Without them the statistics estimates are chained.
// stats_est (may be null) receives the chained statistics estimate of the
// rows after each step (no true counts used).
extern "C" int wk_featurize(wk_ctx *ctx, const int64_t *cmd, int32_t n, const int64_t *true_rows, float *feats,
                            int32_t *pids, double *stats_est) {
    if (!ctx || !cmd || n < 1 || !feats || !pids) return set_error(WK_EINVAL, "wk_featurize: bad arguments");
    if (!ctx->store) return set_error(WK_ENOSTORE, "wk_featurize: no store");
    Stats &st = stats_of(ctx);
    double chained = 1.0;
    int rc = walk_plan(cmd, n, [&](int i, const Step &s, const VarInfo *bind, int cols) {
        const double before = i == 0 ? 1.0 : (true_rows ? (double)true_rows[i - 1] : chained);
        features(ctx, st, s, i == 0 ? 0.0 : before, i, cols, bind, feats + (size_t)i * kF);
        pids[i] = s.feat_pid;
        chained = stats_step(ctx, st, s, i == 0 ? 1.0 : chained, bind);
        if (stats_est) stats_est[i] = chained;
    });
    if (rc) return set_error(WK_EINVAL, "wk_featurize: the plan is not executable left to right");
    return WK_OK;
}

namespace wk {
namespace {

struct Cand {
    Step s;
    int pat;
    bool consumes;   // false for a predicate-index start, which leaves its pattern to run
};

// A partial plan: the patterns used so far, the variables they bound, the
// executable steps, the predicted rows of the current table and the plan's
// cost so far (the sum of the predicted rows of every table it builds).
struct PState {
    std::vector<int> used;
    std::unordered_map<int64_t, VarInfo> vars;
    std::vector<int64_t> plan;
    double rows = 0.0, cost = 0.0;
    int cols = 0, step = 0;
    bool complete = false;
};

struct QPlan {
    const int64_t *cmd = nullptr;
    int n = 0;
    std::vector<PState> beam;
    bool failed = false;
};

// Executable oriented steps from state S: at the first step a constant, a type
// index or a predicate index; later, every unused pattern from a bound end.
// Returns false when every pattern is used.
bool candidates(const QPlan &Q, const PState &S, std::vector<Cand> &out) {
    out.clear();
    const int n = Q.n;
    if (S.step == 0) {
        for (int i = 0; i < n; ++i) {
            const int64_t a = Q.cmd[4 * i], p = Q.cmd[4 * i + 1], b = Q.cmd[4 * i + 3];
            if (a >= WK_VID_BASE) out.push_back(Cand{Step{K_C2U, a, p, WK_DIR_OUT, b, (int)p}, i, true});
            if (b >= WK_VID_BASE) out.push_back(Cand{Step{K_C2U, b, p, WK_DIR_IN, a, (int)p}, i, true});
            if (p == WK_TYPE_ID && a < 0 && b > 1 && b < WK_VID_BASE)
                out.push_back(Cand{Step{K_I2U, b, WK_TYPE_ID, WK_DIR_IN, a, (int)b}, i, true});
            if (a < 0 && b < 0 && p != WK_TYPE_ID) {
                out.push_back(Cand{Step{K_I2U, p, WK_PREDICATE_ID, WK_DIR_IN, a, (int)p}, i, false});
                out.push_back(Cand{Step{K_I2U, p, WK_PREDICATE_ID, WK_DIR_OUT, b, (int)p}, i, false});
            }
        }
        return true;
    }
    bool any = false;
    for (int i = 0; i < n; ++i) {
        if (S.used[(size_t)i]) continue;
        any = true;
        const int64_t a = Q.cmd[4 * i], p = Q.cmd[4 * i + 1], b = Q.cmd[4 * i + 3];
        const bool ka = a < 0 && S.vars.count(a), kb = b < 0 && S.vars.count(b);
        auto kind_for = [&](int64_t other) {
            if (other >= 0) return (int)K_K2C;
            return S.vars.count(other) ? (int)K_K2K : (int)K_K2U;
        };
        if (ka) out.push_back(Cand{Step{kind_for(b), a, p, WK_DIR_OUT, b, (int)p}, i, true});
        if (kb) out.push_back(Cand{Step{kind_for(a), b, p, WK_DIR_IN, a, (int)p}, i, true});
    }
    return any;
}

PState apply(const PState &S, const Cand &c, double rows_after) {
    PState t = S;
    const Step &s = c.s;
    t.plan.insert(t.plan.end(), {s.start, s.pid, s.dir, s.end});
    if (c.consumes) t.used[(size_t)c.pat] = 1;
    if (s.kind == K_I2U || s.kind == K_C2U || s.kind == K_K2U) {
        VarInfo v;
        v.col = t.cols++;
        v.pred = s.kind == K_I2U ? (int)s.start : (int)s.pid;
        v.dir = (int)s.dir;
        t.vars[s.end] = v;
    }
    t.rows = rows_after;
    t.cost += rows_after;
    t.step++;
    return t;
}

// Beam search over join orders for every query at once.  Each level expands
// every partial plan in every query's beam by each executable step; one model
// call predicts the rows after all of them; each query keeps its `beam`
// cheapest partial plans (cost = the sum of predicted rows of the tables
// built so far -- the quantity the statistics planner's search minimises).
// A beam of 1 is the greedy planner.  On return qs[q].beam[0] is the cheapest
// complete plan, or qs[q].failed is set (no executable order).
int plan_beam(wk_ctx *ctx, wk_mlp *mlp, std::vector<QPlan> &qs, int beam) {
    Stats &st = stats_of(ctx);
    for (auto &Q : qs) {
        PState s0;
        s0.used.assign((size_t)Q.n, 0);
        Q.beam.assign(1, s0);
    }
    struct Kid {
        int q, parent;
        Cand c;
        double exact;   // the rows of an index or constant start (one list's length), else < 0
    };
    std::vector<float> fb, pred;
    std::vector<int32_t> pb;
    std::vector<Kid> kids;
    std::vector<Cand> cands;
    for (int level = 0; level < 12; ++level) {
        fb.clear();
        pb.clear();
        kids.clear();
        for (int q = 0; q < (int)qs.size(); ++q) {
            QPlan &Q = qs[(size_t)q];
            if (Q.failed) continue;
            for (int si = 0; si < (int)Q.beam.size(); ++si) {
                PState &S = Q.beam[(size_t)si];
                if (S.complete) continue;
                if (!candidates(Q, S, cands)) {
                    S.complete = true;
                    continue;
                }
                for (const Cand &c : cands) {
                    const Step &s = c.s;
                    const VarInfo *bind = nullptr;
                    if (s.kind != K_I2U && s.kind != K_C2U) bind = &S.vars.at(s.start);
                    fb.resize(fb.size() + kF);
                    features(ctx, st, s, S.step == 0 ? 0.0 : S.rows, S.step, S.cols, bind,
                             fb.data() + fb.size() - kF);
                    pb.push_back(s.feat_pid);
                    double exact = -1.0;
                    if (s.kind == K_I2U) exact = (double)list_len(ctx, 0, (int)s.start, (int)s.dir);
                    else if (s.kind == K_C2U) exact = (double)list_len(ctx, (uint64_t)s.start, (int)s.pid, (int)s.dir);
                    kids.push_back(Kid{q, si, c, exact});
                }
            }
        }
        if (kids.empty()) break;
        pred.assign(pb.size(), 0.f);
        int rc = wk_mlp_predict(mlp, fb.data(), pb.data(), (int64_t)pb.size(), pred.data());
        if (rc) return rc;
        // next beams: complete plans carried over, plus every child; cheapest first
        size_t k = 0;
        for (int q = 0; q < (int)qs.size(); ++q) {
            QPlan &Q = qs[(size_t)q];
            if (Q.failed) continue;
            std::vector<PState> next;
            for (const PState &S : Q.beam)
                if (S.complete) next.push_back(S);
            bool expanded = false;
            while (k < kids.size() && kids[k].q == q) {
                const Kid &kd = kids[k];
                const double rows = kd.exact >= 0.0 ? kd.exact : std::expm1((double)std::max(0.f, pred[k]));
                next.push_back(apply(Q.beam[(size_t)kd.parent], kd.c, rows));
                expanded = true;
                ++k;
            }
            if (!expanded && next.empty()) {
                Q.failed = true;   // partial plans with no executable step left
                continue;
            }
            // a partial plan that could not be extended (no step from a bound end) is dropped
            std::stable_sort(next.begin(), next.end(),
                             [](const PState &a, const PState &b) { return a.cost < b.cost; });
            if ((int)next.size() > beam) next.resize((size_t)beam);
            Q.beam.swap(next);
        }
    }
    for (auto &Q : qs) {
        if (Q.failed) continue;
        while (!Q.beam.empty() && !Q.beam.front().complete) Q.beam.erase(Q.beam.begin());
        if (Q.beam.empty()) Q.failed = true;
    }
    return WK_OK;
}

// renumber variables in binding order (core/planner.hpp:991-1003)
void renumber(std::vector<int64_t> &plan) {
    std::unordered_map<int64_t, int64_t> conv;
    for (auto &x : plan)
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

constexpr int kBeam = 4;

}  // namespace
}  // namespace wk

// Learned plan of a BGP (SPARQL triple form, any variable numbering): beam
// search over join orders scored by the model.  *est_log_rows receives
// log1p of the plan's predicted cost (the sum of its tables' rows).
extern "C" int wk_plan_learned(wk_ctx *ctx, wk_mlp *mlp, const int64_t *cmd_in, int32_t n, int64_t *cmd_out,
                               int32_t *n_out, double *est_log_rows) {
    if (!ctx || !mlp || !cmd_in || !cmd_out || !n_out || n < 1 || n > 10)
        return set_error(WK_EINVAL, "wk_plan_learned: bad arguments");
    if (!ctx->store) return set_error(WK_ENOSTORE, "wk_plan_learned: no store");
    if (!triple_form(cmd_in, n)) {   // already executable: no plan, run as written
        *n_out = 0;
        if (est_log_rows) *est_log_rows = INFINITY;
        return WK_OK;
    }
    if (!wk_mlp_is_trusted(mlp)) {   // statistics fallback
        int32_t room = *n_out, empty = 0;
        double cost = 0.0;
        int rc = wk_plan(ctx, cmd_in, n, cmd_out, &room, &cost, &empty);
        if (rc) return rc;
        if (room > 0) {
            *n_out = room;
            if (est_log_rows) *est_log_rows = std::log1p(cost);
            return WK_OK;
        }
        // no statistics plan (proved empty, or no order found): the search below
    }
    std::vector<QPlan> qs(1);
    qs[0].cmd = cmd_in;
    qs[0].n = n;
    int rc = plan_beam(ctx, mlp, qs, kBeam);
    if (rc) return rc;
    if (qs[0].failed) {
        *n_out = 0;   // no executable order
        if (est_log_rows) *est_log_rows = INFINITY;
        return WK_OK;
    }
    std::vector<int64_t> plan = qs[0].beam[0].plan;
    renumber(plan);
    const int32_t m = (int32_t)(plan.size() / 4);
    if (m > *n_out) return set_error(WK_EOVERFLOW, "wk_plan_learned: plan has %d patterns, room for %d", m, *n_out);
    std::memcpy(cmd_out, plan.data(), plan.size() * sizeof(int64_t));
    *n_out = m;
    if (est_log_rows) *est_log_rows = std::log1p(qs[0].beam[0].cost);
    return WK_OK;
}

// Learned plans of many BGPs at once: every level of every query's beam
// search is one model call.  cmd_in packs the queries back to back (n_in[q]
// patterns each); cmd_out must hold sum(n_in[q] + 1) patterns; n_out[q]
// receives each plan's length (0: no executable order).
extern "C" int wk_plan_learned_batch(wk_ctx *ctx, wk_mlp *mlp, const int64_t *cmd_in, const int32_t *n_in, int32_t nq,
                                     int64_t *cmd_out, int32_t *n_out) {
    if (!ctx || !mlp || !cmd_in || !n_in || nq < 1 || !cmd_out || !n_out)
        return set_error(WK_EINVAL, "wk_plan_learned_batch: bad arguments");
    if (!ctx->store) return set_error(WK_ENOSTORE, "wk_plan_learned_batch: no store");
    std::vector<QPlan> qs((size_t)nq);
    int64_t at = 0;
    for (int q = 0; q < nq; ++q) {
        if (n_in[q] < 1 || n_in[q] > 10)
            return set_error(WK_EINVAL, "wk_plan_learned_batch: query %d has %d patterns", q, n_in[q]);
        qs[(size_t)q].cmd = cmd_in + at;
        qs[(size_t)q].n = n_in[q];
        if (!triple_form(qs[(size_t)q].cmd, n_in[q])) qs[(size_t)q].failed = true;   // no plan: run as written
        at += 4 * (int64_t)n_in[q];
    }
    // statistics fallback for an untrusted model: queries with a statistics
    // plan take it and skip the search
    std::vector<std::vector<int64_t>> stats_plan((size_t)nq);
    if (!wk_mlp_is_trusted(mlp)) {
        std::vector<int64_t> buf;
        for (int q = 0; q < nq; ++q) {
            int32_t room = qs[(size_t)q].n + 1, empty = 0;
            buf.assign((size_t)room * 4, 0);
            double cost = 0.0;
            int rc = wk_plan(ctx, qs[(size_t)q].cmd, qs[(size_t)q].n, buf.data(), &room, &cost, &empty);
            if (rc) return rc;
            if (room > 0) {
                stats_plan[(size_t)q].assign(buf.begin(), buf.begin() + (ptrdiff_t)room * 4);
                qs[(size_t)q].failed = true;   // excluded from the search
            }
        }
    }
    int rc = plan_beam(ctx, mlp, qs, kBeam);
    if (rc) return rc;
    int64_t out_at = 0;
    for (int q = 0; q < nq; ++q) {
        QPlan &Q = qs[(size_t)q];
        if (!stats_plan[(size_t)q].empty()) {
            const std::vector<int64_t> &sp = stats_plan[(size_t)q];
            std::memcpy(cmd_out + out_at, sp.data(), sp.size() * sizeof(int64_t));
            n_out[q] = (int32_t)(sp.size() / 4);
            out_at += (int64_t)sp.size();
            continue;
        }
        if (Q.failed) {
            n_out[q] = 0;
            continue;
        }
        std::vector<int64_t> plan = Q.beam[0].plan;
        renumber(plan);
        std::memcpy(cmd_out + out_at, plan.data(), plan.size() * sizeof(int64_t));
        n_out[q] = (int32_t)(plan.size() / 4);
        out_at += (int64_t)plan.size();
    }
    return WK_OK;
}
