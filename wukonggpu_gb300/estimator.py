"""Training data, training and evaluation of the learned cardinality estimator.

The engine records the true rows after every step of the queries it executes
(wk_execute's step_rows); each step becomes one sample: its features (with
the true rows before the step), the embedding id of its predicate, and the
target log(1 + true rows after the step).  The statistics planner's own
estimate of the same step, chained from its own earlier estimates, is kept
beside it as the baseline whose q-error the model is compared with.
"""
from __future__ import annotations

import numpy as np

from . import Estimator, RCache, featurize


def qerror(est_rows: np.ndarray, true_rows: np.ndarray) -> np.ndarray:
    """max(est/true, true/est) on (rows + 1)."""
    e = np.asarray(est_rows, np.float64) + 1.0
    t = np.asarray(true_rows, np.float64) + 1.0
    return np.maximum(e / t, t / e)


def build_dataset(rc: RCache, bgps, plan_with: str = "stats", max_rows: int = 1 << 26):
    """Execute every BGP (statistics plan) and return the step samples.

    Returns dict with feats [n x 48], pids [n], target [n] (log1p true rows),
    true_rows [n], stats_est [n], query [n] (index of the BGP), step [n]."""
    F, P, T, R, S, Q, K = [], [], [], [], [], [], []
    for qi, q in enumerate(bgps):
        plan, _ = rc.plan(q) if plan_with == "stats" else (q, 0.0)
        if not plan:
            continue
        try:
            req, rows = rc.execute(plan, download=False)
        except Exception:
            continue
        f, p, est = featurize(rc, plan, rows)
        F.append(f)
        P.append(p)
        T.append(np.log1p(rows.astype(np.float64)).astype(np.float32))
        R.append(rows)
        S.append(est)
        Q.append(np.full(len(rows), qi))
        K.append(np.arange(len(rows)))
    cat = lambda xs, dt: np.concatenate(xs).astype(dt) if xs else np.zeros(0, dt)
    return {
        "feats": np.concatenate(F).astype(np.float32) if F else np.zeros((0, 48), np.float32),
        "pids": cat(P, np.int32), "target": cat(T, np.float32), "true_rows": cat(R, np.int64),
        "stats_est": cat(S, np.float64), "query": cat(Q, np.int64), "step": cat(K, np.int64),
    }


def split(ds: dict, frac_train: float = 0.9, seed: int = 0):
    """Split by query (every step of a query on the same side)."""
    qs = np.unique(ds["query"])
    rng = np.random.default_rng(seed)
    train_q = set(rng.permutation(qs)[: int(len(qs) * frac_train)].tolist())
    m = np.array([q in train_q for q in ds["query"]])
    sub = lambda mask: {k: v[mask] for k, v in ds.items()}
    return sub(m), sub(~m)


def evaluate(est: Estimator, ds: dict) -> dict:
    """Median / p95 q-error of the model and of the statistics estimate."""
    pred = np.expm1(np.maximum(est.predict(ds["feats"], ds["pids"]), 0.0))
    ql = qerror(pred, ds["true_rows"])
    qs = qerror(ds["stats_est"], ds["true_rows"])
    return {"learned_median": float(np.median(ql)), "learned_p95": float(np.percentile(ql, 95)),
            "stats_median": float(np.median(qs)), "stats_p95": float(np.percentile(qs, 95)),
            "samples": int(len(ql))}
