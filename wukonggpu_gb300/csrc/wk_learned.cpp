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
// Learned planner: greedy.  At every step each executable pattern -- oriented
// from a bound end, or for the first step from a constant, a type index or a
// predicate index -- is scored by the model's predicted log rows after it,
// and the smallest is taken (ties: lower pattern index, then OUT before IN).
// The result has the statistics planner's output format: executable order,
// variables renumbered in binding order, an inserted index pattern when the
// first pattern joins two variables.
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

// Greedy learned plan of a BGP (SPARQL triple form, any variable numbering).
extern "C" int wk_plan_learned(wk_ctx *ctx, wk_mlp *mlp, const int64_t *cmd_in, int32_t n, int64_t *cmd_out,
                               int32_t *n_out, double *est_log_rows) {
    if (!ctx || !mlp || !cmd_in || !cmd_out || !n_out || n < 1 || n > 10)
        return set_error(WK_EINVAL, "wk_plan_learned: bad arguments");
    if (!ctx->store) return set_error(WK_ENOSTORE, "wk_plan_learned: no store");
    Stats &st = stats_of(ctx);
    std::vector<int> used((size_t)n, 0);
    std::unordered_map<int64_t, VarInfo> vars;
    std::vector<int64_t> plan;
    double rows = 0.0, total_est = 0.0;
    int cols = 0;
    std::vector<float> fb;
    std::vector<int32_t> pb;
    std::vector<float> pred;
    struct Cand { Step s; int pat; bool consumes; };
    for (int step = 0; step < n + 1; ++step) {
        std::vector<Cand> cands;
        if (step == 0) {
            for (int i = 0; i < n; ++i) {
                const int64_t a = cmd_in[4 * i], p = cmd_in[4 * i + 1], b = cmd_in[4 * i + 3];
                if (a >= WK_VID_BASE) cands.push_back(Cand{Step{K_C2U, a, p, WK_DIR_OUT, b, (int)p}, i, true});
                if (b >= WK_VID_BASE) cands.push_back(Cand{Step{K_C2U, b, p, WK_DIR_IN, a, (int)p}, i, true});
                if (p == WK_TYPE_ID && a < 0 && b > 1 && b < WK_VID_BASE)
                    cands.push_back(Cand{Step{K_I2U, b, WK_TYPE_ID, WK_DIR_IN, a, (int)b}, i, true});
                if (a < 0 && b < 0 && p != WK_TYPE_ID) {
                    cands.push_back(Cand{Step{K_I2U, p, WK_PREDICATE_ID, WK_DIR_IN, a, (int)p}, i, false});
                    cands.push_back(Cand{Step{K_I2U, p, WK_PREDICATE_ID, WK_DIR_OUT, b, (int)p}, i, false});
                }
            }
        } else {
            bool all = true;
            for (int i = 0; i < n; ++i) {
                if (used[(size_t)i]) continue;
                all = false;
                const int64_t a = cmd_in[4 * i], p = cmd_in[4 * i + 1], b = cmd_in[4 * i + 3];
                const bool ka = a < 0 && vars.count(a), kb = b < 0 && vars.count(b);
                auto kind_for = [&](int64_t other) {
                    if (other >= 0) return (int)K_K2C;
                    return vars.count(other) ? (int)K_K2K : (int)K_K2U;
                };
                if (ka) cands.push_back(Cand{Step{kind_for(b), a, p, WK_DIR_OUT, b, (int)p}, i, true});
                if (kb) cands.push_back(Cand{Step{kind_for(a), b, p, WK_DIR_IN, a, (int)p}, i, true});
            }
            if (all) break;
        }
        if (cands.empty()) {
            *n_out = 0;   // no executable order
            if (est_log_rows) *est_log_rows = INFINITY;
            return WK_OK;
        }
        fb.assign(cands.size() * kF, 0.f);
        pb.assign(cands.size(), 0);
        for (size_t c = 0; c < cands.size(); ++c) {
            const Step &s = cands[c].s;
            const VarInfo *bind = nullptr;
            if (s.kind != K_I2U && s.kind != K_C2U) bind = &vars[s.start];
            features(ctx, st, s, step == 0 ? 0.0 : rows, step, cols, bind, fb.data() + c * kF);
            pb[c] = s.feat_pid;
        }
        pred.assign(cands.size(), 0.f);
        int rc = wk_mlp_predict(mlp, fb.data(), pb.data(), (int64_t)cands.size(), pred.data());
        if (rc) return rc;
        size_t best = 0;
        for (size_t c = 1; c < cands.size(); ++c)
            if (pred[c] < pred[best]) best = c;
        const Cand &ch = cands[best];
        const Step &s = ch.s;
        if (s.kind == K_I2U) plan.insert(plan.end(), {s.start, s.pid, s.dir, s.end});
        else plan.insert(plan.end(), {s.start, s.pid, s.dir, s.end});
        if (ch.consumes) used[(size_t)ch.pat] = 1;
        if (s.kind == K_I2U || s.kind == K_C2U || s.kind == K_K2U) {
            VarInfo v;
            v.col = cols++;
            v.pred = s.kind == K_I2U ? (int)s.start : (int)s.pid;
            v.dir = (int)s.dir;
            vars[s.end] = v;
        }
        rows = std::expm1((double)std::max(0.f, pred[best]));
        total_est += rows;
    }
    // renumber variables in binding order
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
    const int32_t m = (int32_t)(plan.size() / 4);
    if (m > *n_out) return set_error(WK_EOVERFLOW, "wk_plan_learned: plan has %d patterns, room for %d", m, *n_out);
    std::memcpy(cmd_out, plan.data(), plan.size() * sizeof(int64_t));
    *n_out = m;
    if (est_log_rows) *est_log_rows = std::log1p(total_est);
    return WK_OK;
}

// Learned plans of many BGPs at once: the greedy steps of all queries run in
// lockstep, so each step is one model call over every query's candidates.
// cmd_in packs the queries back to back (n_in[q] patterns each); cmd_out must
// hold sum(n_in[q] + 1) patterns; n_out[q] receives each plan's length (0:
// no executable order).
extern "C" int wk_plan_learned_batch(wk_ctx *ctx, wk_mlp *mlp, const int64_t *cmd_in, const int32_t *n_in, int32_t nq,
                                     int64_t *cmd_out, int32_t *n_out) {
    if (!ctx || !mlp || !cmd_in || !n_in || nq < 1 || !cmd_out || !n_out)
        return set_error(WK_EINVAL, "wk_plan_learned_batch: bad arguments");
    if (!ctx->store) return set_error(WK_ENOSTORE, "wk_plan_learned_batch: no store");
    Stats &st = stats_of(ctx);
    struct Cand { Step s; int pat; bool consumes; };
    struct QState {
        const int64_t *cmd;
        int n;
        std::vector<int> used;
        std::unordered_map<int64_t, VarInfo> vars;
        std::vector<int64_t> plan;
        double rows = 0.0;
        int cols = 0, step = 0;
        bool done = false, failed = false;
        std::vector<Cand> cands;
    };
    std::vector<QState> qs((size_t)nq);
    int64_t at = 0;
    for (int q = 0; q < nq; ++q) {
        if (n_in[q] < 1 || n_in[q] > 10) return set_error(WK_EINVAL, "wk_plan_learned_batch: query %d has %d patterns", q, n_in[q]);
        qs[(size_t)q].cmd = cmd_in + at;
        qs[(size_t)q].n = n_in[q];
        qs[(size_t)q].used.assign((size_t)n_in[q], 0);
        at += 4 * (int64_t)n_in[q];
    }
    std::vector<float> fb, pred;
    std::vector<int32_t> pb;
    for (int round = 0; round < 11; ++round) {
        fb.clear();
        pb.clear();
        for (auto &Q : qs) {
            Q.cands.clear();
            if (Q.done) continue;
            const int n = Q.n;
            if (Q.step == 0) {
                for (int i = 0; i < n; ++i) {
                    const int64_t a = Q.cmd[4 * i], p = Q.cmd[4 * i + 1], b = Q.cmd[4 * i + 3];
                    if (a >= WK_VID_BASE) Q.cands.push_back(Cand{Step{K_C2U, a, p, WK_DIR_OUT, b, (int)p}, i, true});
                    if (b >= WK_VID_BASE) Q.cands.push_back(Cand{Step{K_C2U, b, p, WK_DIR_IN, a, (int)p}, i, true});
                    if (p == WK_TYPE_ID && a < 0 && b > 1 && b < WK_VID_BASE)
                        Q.cands.push_back(Cand{Step{K_I2U, b, WK_TYPE_ID, WK_DIR_IN, a, (int)b}, i, true});
                    if (a < 0 && b < 0 && p != WK_TYPE_ID) {
                        Q.cands.push_back(Cand{Step{K_I2U, p, WK_PREDICATE_ID, WK_DIR_IN, a, (int)p}, i, false});
                        Q.cands.push_back(Cand{Step{K_I2U, p, WK_PREDICATE_ID, WK_DIR_OUT, b, (int)p}, i, false});
                    }
                }
            } else {
                bool all = true;
                for (int i = 0; i < n; ++i) {
                    if (Q.used[(size_t)i]) continue;
                    all = false;
                    const int64_t a = Q.cmd[4 * i], p = Q.cmd[4 * i + 1], b = Q.cmd[4 * i + 3];
                    const bool ka = a < 0 && Q.vars.count(a), kb = b < 0 && Q.vars.count(b);
                    auto kind_for = [&](int64_t other) {
                        if (other >= 0) return (int)K_K2C;
                        return Q.vars.count(other) ? (int)K_K2K : (int)K_K2U;
                    };
                    if (ka) Q.cands.push_back(Cand{Step{kind_for(b), a, p, WK_DIR_OUT, b, (int)p}, i, true});
                    if (kb) Q.cands.push_back(Cand{Step{kind_for(a), b, p, WK_DIR_IN, a, (int)p}, i, true});
                }
                if (all) { Q.done = true; continue; }
            }
            if (Q.cands.empty()) { Q.done = true; Q.failed = true; continue; }
            for (const Cand &c : Q.cands) {
                const Step &s = c.s;
                const VarInfo *bind = (s.kind != K_I2U && s.kind != K_C2U) ? &Q.vars[s.start] : nullptr;
                fb.resize(fb.size() + kF);
                features(ctx, st, s, Q.step == 0 ? 0.0 : Q.rows, Q.step, Q.cols, bind, fb.data() + fb.size() - kF);
                pb.push_back(s.feat_pid);
            }
        }
        if (pb.empty()) break;
        pred.assign(pb.size(), 0.f);
        int rc = wk_mlp_predict(mlp, fb.data(), pb.data(), (int64_t)pb.size(), pred.data());
        if (rc) return rc;
        size_t k = 0;
        for (auto &Q : qs) {
            if (Q.cands.empty()) continue;
            size_t best = 0;
            for (size_t c = 1; c < Q.cands.size(); ++c)
                if (pred[k + c] < pred[k + best]) best = c;
            const Cand &ch = Q.cands[best];
            const Step &s = ch.s;
            Q.plan.insert(Q.plan.end(), {s.start, s.pid, s.dir, s.end});
            if (ch.consumes) Q.used[(size_t)ch.pat] = 1;
            if (s.kind == K_I2U || s.kind == K_C2U || s.kind == K_K2U) {
                VarInfo v;
                v.col = Q.cols++;
                v.pred = s.kind == K_I2U ? (int)s.start : (int)s.pid;
                v.dir = (int)s.dir;
                Q.vars[s.end] = v;
            }
            Q.rows = std::expm1((double)std::max(0.f, pred[k + best]));
            Q.step++;
            k += Q.cands.size();
        }
    }
    int64_t out_at = 0;
    for (int q = 0; q < nq; ++q) {
        QState &Q = qs[(size_t)q];
        if (Q.failed) { n_out[q] = 0; continue; }
        std::unordered_map<int64_t, int64_t> conv;
        for (auto &x : Q.plan)
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
        std::memcpy(cmd_out + out_at, Q.plan.data(), Q.plan.size() * sizeof(int64_t));
        n_out[q] = (int32_t)(Q.plan.size() / 4);
        out_at += (int64_t)Q.plan.size();
    }
    return WK_OK;
}
