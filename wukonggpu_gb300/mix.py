"""Weighted query mixes in the reference batch driver's format.

A mix file follows the reference's ``scripts/batch/mix_config``: a first line
``<ntypes> <nheavy>``, then one line per query type, ``<query file>
<weight>``.  The first ``ntypes - nheavy`` types are light *templates*,
instantiated with random constants of a class for every request; the last
``nheavy`` are heavy queries, run as written (core/proxy.hpp:287-330).  Each
request draws its type by the integer weights with the rule of
``mymath::get_distribution`` (utils/mymath.hpp:28-41: a random value modulo
the weights' sum, then the first type whose cumulative weight exceeds it)
and fills every random constant of a template from one random seed:
candidate ``seed % n`` of the constant's class (request_template::instantiate,
core/query.hpp:198-205), the candidates being the class's members, as the
proxy collects them with a type query (Proxy::fill_template,
core/proxy.hpp:75-116).

Query files hold the engine's form, one pattern per line: ``start predicate
direction end``.  The reference's templates are SPARQL text; the parser is out
of scope here, so a token names a layout symbol instead:

* ``F<k>``, ``Z<k>``, ``M<k>``: the k-th (1-based) functional, Zipf and
  many-to-one predicate of the graph's layout; ``TYPE`` is rdf:type;
* ``C<k>``: the k-th class (0-based); ``%C<k>``: a random member of it (the
  reference's ``%Type`` placeholder);
* ``IN`` / ``OUT``; negative integers are variables, other integers ids.

A heavy query starts from a type index (``C<k> TYPE IN -1``) and continues
with OUT steps; its SPARQL triple form, which the planners take, moves the
class to the object of the first pattern (``-1 TYPE OUT C<k>``).
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

from . import IN, OUT, TYPE_ID

MIX_DIR = Path(__file__).resolve().parent / "mixes"


def get_distribution(r: int, weights) -> int:
    """Type index for the random value r: utils/mymath.hpp:28-41."""
    total = int(sum(weights))
    if total <= 0:
        raise ValueError("mix weights must have a positive sum")
    r %= total
    for i, w in enumerate(weights):
        if r < w:
            return i
        r -= w
    raise AssertionError("unreachable")


class QueryType:
    def __init__(self, name: str, weight: int, heavy: bool, patterns):
        self.name, self.weight, self.heavy, self.patterns = name, weight, heavy, patterns

    @property
    def placeholders(self):
        """(pattern, field, class index) of every random constant."""
        return [(i, j, int(tok[2:])) for i, pat in enumerate(self.patterns) for j, tok in enumerate(pat)
                if isinstance(tok, str) and tok.startswith("%C")]


def _parse_query(path: Path):
    pats = []
    for line in path.read_text().splitlines():
        line = line.split("#", 1)[0].strip()
        if not line:
            continue
        toks = line.split()
        if len(toks) != 4:
            raise ValueError(f"{path.name}: a pattern needs 4 tokens: {line!r}")
        pats.append(toks)
    if not pats:
        raise ValueError(f"{path.name}: no patterns")
    return pats


def parse_mix(path) -> list[QueryType]:
    """The query types of a mix file (query files are relative to it)."""
    path = Path(path)
    lines = [x.split("#", 1)[0].split() for x in path.read_text().splitlines()]
    lines = [x for x in lines if x]
    ntypes, nheavy = int(lines[0][0]), int(lines[0][1])
    if ntypes <= 0 or not 0 <= nheavy <= ntypes or len(lines) != ntypes + 1:
        raise ValueError(f"{path.name}: header says {ntypes} types ({nheavy} heavy), found {len(lines) - 1}")
    out = []
    for i, (fname, w) in enumerate(lines[1:]):
        if int(w) <= 0:
            raise ValueError(f"{path.name}: weight of {fname} must be positive")
        heavy = i >= ntypes - nheavy
        qt = QueryType(Path(fname).stem, int(w), heavy, _parse_query(path.parent / fname))
        if heavy and qt.placeholders:
            raise ValueError(f"{path.name}: heavy query {fname} has random constants")
        out.append(qt)
    return out


class Mix:
    """A parsed mix bound to a graph layout (workloads.Layout)."""

    def __init__(self, path, layout):
        self.path = Path(path)
        self.types = parse_mix(self.path)
        self.layout = layout
        self._cands = {}

    @property
    def weights(self):
        return [t.weight for t in self.types]

    @property
    def n_light(self) -> int:
        return sum(1 for t in self.types if not t.heavy)

    def _tok(self, tok: str) -> int:
        L = self.layout
        if tok == "IN":
            return IN
        if tok == "OUT":
            return OUT
        if tok == "TYPE":
            return TYPE_ID
        for pre, ids in (("F", L.func), ("Z", L.zipf), ("M", L.m2o)):
            if tok.startswith(pre) and tok[1:].isdigit():
                k = int(tok[1:])
                if not 1 <= k <= len(ids):
                    raise ValueError(f"{tok}: the layout has {len(ids)} such predicates")
                return ids[k - 1]
        if tok.startswith("C") and tok[1:].isdigit():
            k = int(tok[1:])
            if not 0 <= k < L.n_classes:
                raise ValueError(f"{tok}: the layout has {L.n_classes} classes")
            return L.first_class + k
        return int(tok)

    def fill_candidates(self, rc):
        """The members of every class a template draws constants from (the
        type index [0|c|IN] of the store, ascending)."""
        for t in self.types:
            for _, _, k in t.placeholders:
                if k not in self._cands:
                    c = rc.get_edges(0, self.layout.first_class + k, IN)
                    if len(c) == 0:
                        raise ValueError(f"class C{k} has no members")
                    self._cands[k] = np.asarray(c, np.int64)

    def instantiate(self, t: QueryType, seed: int):
        """Executable cmd_chains of type t with its random constants from `seed`."""
        out = []
        for pat in t.patterns:
            for tok in pat:
                if tok.startswith("%C"):
                    c = self._cands[int(tok[2:])]
                    out.append(int(c[seed % len(c)]))
                else:
                    out.append(self._tok(tok))
        return out

    @staticmethod
    def triple_form(cmd):
        """The SPARQL triple form of an executable heavy query (type index
        first, then OUT steps) as the planners take it; None for other shapes."""
        if len(cmd) < 4 or cmd[1] != TYPE_ID or cmd[2] != IN or cmd[3] != -1:
            return None
        if any(cmd[4 * i + 2] != OUT for i in range(1, len(cmd) // 4)):
            return None
        return [-1, TYPE_ID, OUT, cmd[0]] + list(cmd[4:])

    def draw(self, n: int, seed: int):
        """n requests: (type index, executable cmd_chains), seeded."""
        rng = np.random.default_rng(seed)
        w = self.weights
        out = []
        for _ in range(n):
            k = get_distribution(int(rng.integers(0, 1 << 31)), w)
            out.append((k, self.instantiate(self.types[k], int(rng.integers(0, 1 << 31)))))
        return out
