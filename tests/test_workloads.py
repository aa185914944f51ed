"""Workload generators (CPU): the store-backed random BGP generator, used for
graphs too large to scan in numpy, gives exactly the queries of the numpy one."""
import wukonggpu_gb300 as W
from wukonggpu_gb300 import workloads


def test_store_backed_bgps_equal_numpy_bgps(lib_built, small_graph):
    g, s, p, o = small_graph
    rc = W.RCache(device=-1)
    rc.build_store(s, p, o, g.num_ids)
    layout = workloads.Layout(0, 15, 0, 10, 200_000)   # spec_small: Zipf predicates 2..16, classes 17..26
    assert layout.first_class == g.first_class
    a = workloads.random_bgps(s, p, o, 400, seed=99, first_class=g.first_class, n_classes=10)
    b = workloads.random_bgps_store(rc, layout, 400, seed=99)
    assert a == b


def test_layouts_match_generator_ids():
    assert workloads.SQ.first_class == 34 and workloads.SQ.preds == list(range(2, 34))
    assert workloads.SV.first_class == 66 and len(workloads.SV.preds) == 64
