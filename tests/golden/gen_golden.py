"""Generate the golden fixtures from the reference's own store.

Run where the reference sources are present (they are compiled in place by
``make -C oracle ref``):

    python tests/golden/gen_golden.py

For each seeded graph it records the graph checksum, the reference store's
content digest, and for every query of the parity set the reference result
(row count per step, digest of the rows in canonical order, and, for queries
that do not start from an index, the digest of the rows in the reference's
own order).  Index lists are filled by racing loader threads in the
reference, so index-start results are compared in canonical order only.
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
import wukonggpu_gb300 as W  # noqa: E402
from wukonggpu_gb300 import workloads  # noqa: E402

OUT = Path(__file__).resolve().parent


def table_digest(t: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(t, np.int32).tobytes()).hexdigest()


def graph_digest(s, p, o) -> str:
    h = hashlib.sha256()
    for a in (s, p, o):
        h.update(np.ascontiguousarray(a, np.int32).tobytes())
    return h.hexdigest()


def is_index_start(cmd) -> bool:
    return 1 < cmd[0] < W.VID_BASE


def main() -> None:
    oracle.build(with_ref=True)
    spec = W.spec_small()
    g = W.Graph(spec)
    s, p, o = g.arrays()
    ref = oracle.RefStore(s, p, o, g.num_ids, keys_million=16, memstore_mb=1024)
    dig, nkeys, nedges = ref.digest()
    out = {
        "config": "small: 200k entities, rdf:type with 10 classes, 15 Zipf(1.2, cap 64) predicates",
        "spec_seed": int(spec.seed),
        "num_triples": int(g.n),
        "num_ids": int(g.num_ids),
        "graph_sha256": graph_digest(s, p, o),
        "store": {"digest": str(dig), "keys": nkeys, "edges": nedges},
        "queries": [],
    }
    for name, cmd in workloads.small_queries(s, p, o):
        t, step_rows = ref.execute(cmd)
        entry = {
            "name": name,
            "cmd_chains": [int(x) for x in cmd],
            "rows": int(t.shape[0]),
            "cols": int(t.shape[1]) if t.ndim == 2 else 0,
            "step_rows": [int(x) for x in step_rows],
            "canonical_sha256": table_digest(oracle.canonical(t)),
        }
        if not is_index_start(cmd):
            entry["ordered_sha256"] = table_digest(t)
        out["queries"].append(entry)
        print(f"{name:22s} rows={t.shape[0]:8d} steps={list(step_rows)}")
    # the reference planner on seeded random BGPs (core/planner.hpp generate_plan)
    out["plans"] = []
    for q in workloads.random_bgps(s, p, o, 120, seed=77, first_class=g.first_class, n_classes=10):
        plan = ref.plan(q)
        out["plans"].append({"bgp": [int(x) for x in q], "plan": plan})
    (OUT / "small.json").write_text(json.dumps(out, indent=1) + "\n")
    print(f"wrote {OUT / 'small.json'}")


if __name__ == "__main__":
    main()
