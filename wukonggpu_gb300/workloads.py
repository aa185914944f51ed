"""Synthetic workloads: graph specs and seeded query sets of the benchmark configurations.

Queries are ``cmd_chains`` lists (4 ints per pattern: start, predicate,
direction, end; core/query.hpp:68) in the reference's variable encoding
(negative = variable -v-1, >= 0 = constant).  Index-start patterns put a
class id (type index) or a predicate id (predicate index) first with
predicate TYPE_ID / PREDICATE_ID, as the reference planner emits them
(core/query.hpp:177-195).

Constants are chosen deterministically from the graph so that each query's
result is non-empty; the choice uses sparse matrix products over the triples
(no engine involved).
"""
from __future__ import annotations

import numpy as np

from . import IN, OUT, PREDICATE_ID, TYPE_ID, VID_BASE, graph_spec

# --------------------------------------------------------------- layouts
# spec_small: pid 1 = type, 2..16 one-to-many Zipf(1.2, 64), classes 17..26
SMALL_PREDS = list(range(2, 17))
SMALL_FIRST_CLASS = 17


def _adj(s, p, o, pid, n_ent):
    """Sparse 0/1 adjacency (entity index space) of predicate pid, subject -> object."""
    from scipy.sparse import csr_matrix
    m = p == pid
    r = s[m].astype(np.int64) - VID_BASE
    c = o[m].astype(np.int64) - VID_BASE
    return csr_matrix((np.ones(len(r), np.float64), (r, c)), shape=(n_ent, n_ent))


def _pick(cands: np.ndarray, ok: np.ndarray, seed: int) -> int:
    """First candidate (in a seeded order) whose flag is set."""
    rng = np.random.default_rng(seed)
    order = rng.permutation(len(cands))
    for i in order:
        if ok[i]:
            return int(cands[i])
    return int(cands[order[0]])


def small_queries(s, p, o, n_ent: int = 200_000, seed: int = 7):
    """Parity query set on the small graph: every pattern kind, both directions.

    Returns a list of (name, cmd_chains)."""
    A = {pid: _adj(s, p, o, pid, n_ent) for pid in (2, 3, 4, 5, 6, 7, 8, 9)}
    ones = np.ones(n_ent)
    # headline: <c> p2 ?y . ?y p5 ?z . ?z p7 ?w with c among p2 subjects
    v = A[5] @ (A[7] @ ones)
    cnt = A[2] @ v
    subj2 = np.unique(s[p == 2]).astype(np.int64)
    c = _pick(subj2, cnt[subj2 - VID_BASE] > 0, seed)
    # const start, IN direction: <o> p4^-1 ?x . ?x p3 ?y
    obj4 = np.unique(o[p == 4]).astype(np.int64)
    in_cnt = A[4].T @ (A[3] @ ones)
    c_in = _pick(obj4, in_cnt[obj4 - VID_BASE] > 0, seed + 1)
    # a popular object of p2 for known_to_const
    vals, counts = np.unique(o[p == 2], return_counts=True)
    pop = int(vals[np.argmax(counts)])
    C0, C1, C2 = SMALL_FIRST_CLASS, SMALL_FIRST_CLASS + 1, SMALL_FIRST_CLASS + 2
    return [
        ("chain3_const", [c, 2, OUT, -1, -1, 5, OUT, -2, -2, 7, OUT, -3]),
        ("const_in", [c_in, 4, IN, -1, -1, 3, OUT, -2]),
        ("type_chain", [C0, TYPE_ID, IN, -1, -1, 2, OUT, -2, -2, 5, OUT, -3]),
        ("type_star", [C1, TYPE_ID, IN, -1, -1, 3, OUT, -2, -1, 4, OUT, -3, -1, 6, IN, -4]),
        ("type_in_chain", [C2, TYPE_ID, IN, -1, -1, 6, IN, -2, -2, 8, OUT, -3]),
        ("pindex_out", [9, PREDICATE_ID, OUT, -1, -1, 9, IN, -2]),
        ("pindex_in_k2k_back", [2, PREDICATE_ID, IN, -1, -1, 2, OUT, -2, -2, 2, IN, -1]),
        ("k2k_cycle", [3, PREDICATE_ID, IN, -1, -1, 3, OUT, -2, -2, 5, OUT, -3, -1, 4, OUT, -3]),
        ("k2k_wide", [C0, TYPE_ID, IN, -1, -1, 2, OUT, -2, -1, 3, OUT, -3, -2, 3, IN, -4, -4, 2, OUT, -2]),
        ("k2c_type", [4, PREDICATE_ID, IN, -1, -1, 4, OUT, -2, -1, TYPE_ID, OUT, C1]),
        ("k2c_obj", [2, PREDICATE_ID, IN, -1, -1, 2, OUT, pop]),
        ("k2k_same_type", [2, PREDICATE_ID, IN, -1, -1, 2, OUT, -2, -2, TYPE_ID, OUT, -3, -1, TYPE_ID, OUT, -3]),
        ("type_of", [c, 2, OUT, -1, -1, TYPE_ID, OUT, -2]),
        ("empty_const", [VID_BASE + n_ent + 5, 2, OUT, -1, -1, 5, OUT, -2]),
        ("empty_mid", [c, 2, OUT, -1, -1, 2, OUT, -2, -2, 2, OUT, -3, -3, 2, OUT, -4, -4, 2, OUT, -5,
                       -5, 2, OUT, -6, -6, 2, OUT, -7]),
    ]


# --------------------------------------------------------- predicate layouts
class Layout:
    """Predicate ids of a generated graph, by degree mix (generator order)."""

    def __init__(self, n_func: int, n_zipf: int, n_m2o: int, n_classes: int, n_entities: int):
        self.func = list(range(2, 2 + n_func))
        self.zipf = list(range(2 + n_func, 2 + n_func + n_zipf))
        self.m2o = list(range(2 + n_func + n_zipf, 2 + n_func + n_zipf + n_m2o))
        self.first_class = 2 + n_func + n_zipf + n_m2o
        self.n_classes = n_classes
        self.n_entities = n_entities

    @property
    def preds(self):
        return self.func + self.zipf + self.m2o


# spec_single_query (100M triples): 2..9 functional, 10..25 Zipf(1.1, 4096), 26..33 many-to-one, classes 34..48
SQ = Layout(8, 16, 8, 15, 2_000_000)
# spec_serving (1.0e9 triples): 2..17 functional, 18..49 Zipf, 50..65 many-to-one, classes 66..80
SV = Layout(16, 32, 16, 15, 20_000_000)

SQ_FUNC = SQ.func
SQ_ZIPF = SQ.zipf
SQ_M2O = SQ.m2o
SQ_FIRST_CLASS = SQ.first_class


def scale_queries(per_shape: int = 5):
    """Six-pattern star+chain BGPs from a type index (the single-query-scale workload).

    Three query shapes, each instantiated on ``per_shape`` different classes
    (15 classes in all).  With 2M entities a class holds ~1.3e5 members; hub
    fan-in makes the history reach 1e7..1e8 rows over up to 6 columns."""
    C = SQ_FIRST_CLASS
    f, z, m = SQ_FUNC, SQ_ZIPF, SQ_M2O
    out = []
    for k in range(per_shape):
        # ?x type C . ?x m1 ?h . ?h m2^-1 ?y . ?y f1 ?a . ?y m3 ?g . ?x f2 ?b
        out.append((f"star_chain_hub/{k}", [C + k, TYPE_ID, IN, -1, -1, m[0], OUT, -2, -2, m[1], IN, -3,
                                            -3, f[0], OUT, -4, -3, m[2], OUT, -5, -1, f[1], OUT, -6]))
        # ?x type C . ?x z1^-1 ?y . ?y m1 ?h . ?h m2^-1 ?w . ?w f1 ?a . ?w z2 ?c
        out.append((f"chain_zipf_hub/{k}", [C + 5 + k, TYPE_ID, IN, -1, -1, z[0], IN, -2, -2, m[3], OUT, -3,
                                            -3, m[4], IN, -4, -4, f[2], OUT, -5, -4, z[1], OUT, -6]))
        # ?x type C . ?x f1 ?a . ?a m1 ?h . ?h m1^-1 ?y . ?y f1 ?b . ?x z3 ?c
        out.append((f"star_fan_in/{k}", [C + 10 + k, TYPE_ID, IN, -1, -1, f[3], OUT, -2, -2, m[5], OUT, -3,
                                         -3, m[5], IN, -4, -4, f[4], OUT, -5, -1, z[2], OUT, -6]))
    return out


def scale_filter_queries():
    """The single-query-scale shapes closed by checks: cycles back to a bound
    column (known_to_known) and constant objects (known_to_const), each keeping
    a fraction of its rows (1e4..1e7 input rows per check on the 100M graph)."""
    C = SQ_FIRST_CLASS
    f, z, m = SQ_FUNC, SQ_ZIPF, SQ_M2O
    return [
        # ?x type C . ?x m1 ?h . ?h m1^-1 ?y . ?y m2 ?h (k2k: the co-member's other hub is ?h)
        ("k2k_hub_cycle", [C, TYPE_ID, IN, -1, -1, m[0], OUT, -2, -2, m[0], IN, -3, -3, m[1], OUT, -2]),
        # ?x type C . ?x z1^-1 ?y . ?y m3 ?h . ?x m3 ?h (k2k: a star closed on a shared hub)
        ("k2k_shared_hub", [C + 1, TYPE_ID, IN, -1, -1, z[0], IN, -2, -2, m[2], OUT, -3, -1, m[2], OUT, -3]),
        # ?x type C . ?x m1 ?h . ?h m1^-1 ?y . ?y f1 ?a . ?x f1 ?a (k2k on a functional predicate)
        ("k2k_functional", [C, TYPE_ID, IN, -1, -1, m[0], OUT, -2, -2, m[0], IN, -3, -3, f[0], OUT, -4,
                            -1, f[0], OUT, -4]),
        # ?x type C . ?x z2 ?y . ?y type C' (k2c on another class)
        ("k2c_other_class", [C + 3, TYPE_ID, IN, -1, -1, z[1], OUT, -2, -2, TYPE_ID, OUT, C + 4]),
        # ?x type C . ?x m1 ?h . ?h m1^-1 ?y . ?y type C (k2c: co-members of the same class)
        ("k2c_same_class", [C + 5, TYPE_ID, IN, -1, -1, m[3], OUT, -2, -2, m[3], IN, -3, -3, TYPE_ID, OUT, C + 5]),
    ]


# ---------------------------------------------------------- random BGPs
def random_bgps(s, p, o, n: int, seed: int, min_pat: int = 2, max_pat: int = 6, first_class: int | None = None,
                n_classes: int = 0, const_frac: float = 0.4):
    """Seeded random connected BGPs in SPARQL triple form (start, pid, OUT, end),
    as a parser emits them (variables -1, -2, ... in order of appearance).

    Shapes: chains, stars and single cycles (a chain closed by one edge back to
    its first variable).  A query is anchored either on a type constraint
    (``?x rdf:type C``) or on a constant vertex drawn from the subjects of its
    first predicate.  Predicates are drawn among those present in the graph."""
    preds = [int(x) for x in np.unique(p) if x != TYPE_ID]
    return _random_bgps(preds, lambda pid: np.unique(s[p == pid]), n, seed, min_pat, max_pat, first_class,
                        n_classes, const_frac)


def random_bgps_store(rc, layout: Layout, n: int, seed: int, min_pat: int = 2, max_pat: int = 6,
                      const_frac: float = 0.4):
    """random_bgps for graphs too large to scan in numpy: the subjects of a
    predicate come from the store's predicate index [0|p|IN] (ascending, the
    same list np.unique gives), the predicates from the layout."""
    return _random_bgps(layout.preds, lambda pid: rc.get_edges(0, pid, IN), n, seed, min_pat, max_pat,
                        layout.first_class, layout.n_classes, const_frac)


def _random_bgps(preds, subjects_of, n, seed, min_pat, max_pat, first_class, n_classes, const_frac):
    rng = np.random.default_rng(seed)
    subj_by_pred = {}
    out = []
    for q in range(n):
        k = int(rng.integers(min_pat, max_pat + 1))
        shape = ("chain", "star", "cycle")[int(rng.integers(0, 3))]
        pats = []
        nv = 1
        anchor_type = first_class is not None and n_classes > 0 and rng.random() >= const_frac
        body = k - (1 if anchor_type else 0)
        if shape == "cycle" and body < 3:
            shape = "chain"
        cur = -1
        for i in range(body):
            pid = preds[int(rng.integers(0, len(preds)))]
            if shape == "star":
                nv += 1
                pats.append([-1, pid, OUT, -nv])
            elif shape == "cycle" and i == body - 1:
                pats.append([cur, pid, OUT, -1])
            else:
                nv += 1
                pats.append([cur, pid, OUT, -nv])
                cur = -nv
        if anchor_type:
            c = first_class + int(rng.integers(0, n_classes))
            pats.insert(int(rng.integers(0, len(pats) + 1)), [-1, TYPE_ID, OUT, c])
        else:
            pid0 = pats[0][1]
            if pid0 not in subj_by_pred:
                subj_by_pred[pid0] = subjects_of(pid0)
            cands = subj_by_pred[pid0]
            c = int(cands[int(rng.integers(0, len(cands)))])
            # replace variable -1 by the constant everywhere
            pats = [[c if x == -1 else x for x in pat[:1]] + pat[1:3] + [c if pat[3] == -1 else pat[3]]
                    for pat in pats]
            # renumber variables in order of appearance
            conv = {}
            for pat in pats:
                for j in (0, 3):
                    if pat[j] < 0:
                        conv.setdefault(pat[j], -1 - len(conv))
                        pat[j] = conv[pat[j]]
        out.append([x for pat in pats for x in pat])
    return out


# ------------------------------------------------ light constant-start queries
def light_queries(s, p, o, n: int, seed: int, max_pat: int = 4, filters: bool = True):
    """Seeded light queries for batching: a constant start vertex drawn uniformly
    among subjects, then 1..max_pat patterns, each predicate drawn among those
    present on the vertex the walk reached (so results are non-empty and their
    sizes heavy-tailed).  With ``filters`` some later steps are known_to_known /
    known_to_const checks.  Executable as written (start bound, end new)."""
    rng = np.random.default_rng(seed)
    order = np.argsort(s, kind="stable")
    ss, pp, oo = s[order], p[order], o[order]
    starts = np.searchsorted(ss, np.arange(VID_BASE, VID_BASE + int(s.max()) - VID_BASE + 2))

    def out_edges(v):
        i = v - VID_BASE
        if i < 0 or i + 1 >= len(starts):
            return pp[:0], oo[:0]
        a, b = starts[i], starts[i + 1]
        m = pp[a:b] != TYPE_ID
        return pp[a:b][m], oo[a:b][m]

    subj = np.unique(s[p != TYPE_ID])
    out = []
    while len(out) < n:
        c = int(subj[int(rng.integers(0, len(subj)))])
        k = int(rng.integers(1, max_pat + 1))
        q = []
        cur_v, col = c, 0
        ok = True
        for step in range(k):
            ps_, os_ = out_edges(cur_v)
            if len(ps_) == 0:
                ok = step > 0
                break
            j = int(rng.integers(0, len(ps_)))
            pid, nxt = int(ps_[j]), int(os_[j])
            if step == 0:
                q += [c, pid, OUT, -1]
                col = 1
            elif filters and step >= 2 and rng.random() < 0.25:
                # a check on an existing binding: ?x p <const> or ?x p ?y
                if rng.random() < 0.5:
                    q += [-col, pid, OUT, nxt]
                else:
                    q += [-col, pid, OUT, -max(1, col - 1)]
                continue
            else:
                q += [-col, pid, OUT, -(col + 1)]
                col += 1
            cur_v = nxt
        if ok and q:
            out.append(q)
    return out


def light_queries_store(rc, n_entities: int, preds, n: int, seed: int, max_pat: int = 4, max_tries: int = 8):
    """Light constant-start queries by random walks over the store (both
    directions), for graphs too large to index in numpy: start at a uniform
    entity, then 1..max_pat steps, each a (predicate, direction) drawn among
    those present on the vertex reached (rejection over random draws)."""
    rng = np.random.default_rng(seed)
    out = []
    while len(out) < n:
        c = VID_BASE + int(rng.integers(0, n_entities))
        k = int(rng.integers(1, max_pat + 1))
        q, cur, col = [], c, 0
        for step in range(k):
            nxt = None
            for _ in range(max_tries):
                pid = int(preds[int(rng.integers(0, len(preds)))])
                d = OUT if rng.random() < 0.6 else IN
                e = rc.get_edges(cur, pid, d)
                if len(e):
                    nxt = (pid, d, int(e[int(rng.integers(0, len(e)))]))
                    break
            if nxt is None:
                break
            pid, d, v = nxt
            if step == 0:
                q += [c, pid, d, -1]
                col = 1
            else:
                q += [-col, pid, d, -(col + 1)]
                col += 1
            cur = v
        if q:
            out.append(q)
    return out


def serving_heavy_queries(layout: Layout = SQ):
    """Heavy requests of the serving mix, in SPARQL triple form: 4..6 patterns
    around the members of one class (?x rdf:type C), widening through
    one-to-one and many-to-one predicates (one class's members: ~1.3e5 rows
    on the 100M graph, ~1.3e6 on the 1B graph).  A planner starts them from
    the type index; executable_heavy_queries gives that order directly."""
    out = []
    for ex in executable_heavy_queries(layout):
        c = ex[0]
        out.append([-1, TYPE_ID, OUT, c] + ex[4:])
    return out


def executable_heavy_queries(layout: Layout = SQ):
    """The heavy shapes in executable form: type index [C, type, IN, ?x] first."""
    C = layout.first_class
    f, m = layout.func, layout.m2o
    out = []
    for k in range(layout.n_classes):
        c = C + k
        base = [c, TYPE_ID, IN, -1, -1, f[k % 8], OUT, -2, -1, m[k % 8], OUT, -3, -2, f[(k + 1) % 8], OUT, -4]
        if k % 3 == 1:
            base += [-3, f[(k + 2) % 8], OUT, -5]
        if k % 3 == 2:
            base += [-3, f[(k + 2) % 8], OUT, -5, -4, m[(k + 3) % 8], OUT, -6]
        out.append(base)
    return out
