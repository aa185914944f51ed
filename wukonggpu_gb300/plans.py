"""Relating a plan to the BGP it came from.

Planners (statistics or learned) reorder patterns, orient them and renumber
variables in binding order.  ``match_plan`` recovers, for every variable of
the original BGP, the planned variable that carries it, so that the result
tables of different plans of one BGP can be compared binding for binding.
``plan_columns`` turns that into the column order of the original
variables.
"""
from __future__ import annotations

from . import IN, OUT, PREDICATE_ID, TYPE_ID, VID_BASE



def match_plan(q, plan):
    """Original variable -> planned variable, by matching every planned pattern
    to a distinct original pattern (backtracking; an inserted index pattern
    binds the subjects (IN) or objects (OUT) of a pattern with that predicate)."""
    orig = [q[i:i + 4] for i in range(0, len(q), 4)]
    pl = [plan[i:i + 4] for i in range(0, len(plan), 4)]
    index = None
    if pl and pl[0][1] in (PREDICATE_ID, TYPE_ID) and 1 < pl[0][0] < VID_BASE and pl[0][1] == PREDICATE_ID:
        index = pl.pop(0)

    def bind(vmap, x, y):
        if x >= 0 or y >= 0:
            return vmap if x == y else None
        if vmap.get(x, y) != y or (y in vmap.values() and vmap.get(x) != y):
            return None
        v = dict(vmap)
        v[x] = y
        return v

    def rec(k, used, vmap):
        if k == len(pl):
            return vmap if all(used) else None
        st, pid, d, en = pl[k]
        for j, (a, pp, dd, b) in enumerate(orig):
            if used[j] or pp != pid:
                continue
            ca, cb = (a, b) if d == OUT else (b, a)
            v = bind(vmap, ca, st)
            v = bind(v, cb, en) if v is not None else None
            if v is None:
                continue
            u = list(used)
            u[j] = True
            r = rec(k + 1, u, v)
            if r is not None:
                if index is not None:
                    ip, _, idir, ivar = index
                    ok = any(pp == ip and ((idir == IN and r.get(a) == ivar) or (idir == OUT and r.get(b) == ivar))
                             for (a, pp, dd, b) in orig)
                    if not ok:
                        continue
                return r
        return None

    return rec(0, [False] * len(orig), {})




def plan_columns(q, plan):
    """Columns of the plan's table holding the BGP's variables -1, -2, ... (None if unmatched)."""
    m = match_plan(q, plan)
    if m is None:
        return None
    nv = max(-x for x in q if x < 0)
    return [-m[-(k + 1)] - 1 for k in range(nv)]
