"""Dense marker layouts against the CPU restatement: the spread plan's slow
paths.

A sphere sampled far more densely than the usual marker spacing gives grid
nodes hundreds of contributors.  That drives every fallback of the plan fill:
row sub-groups split into single nodes, nodes with more contributors than the
shared-memory list holds (scanned and sorted in place), and warps whose entries
overflow their staging (written straight into the plan).  The forcing and the
post-guess fields must still equal the restatement's bit for bit.
"""
import numpy as np
import pytest

import cases
from ibmdem import scenario

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n_markers", [1500, 4000])
def test_dense_spread_matches_restatement(gpu_lib, oracle_mod, n_markers):
    p, parts, bodies, field = scenario.resolved_case(20, 20, 20, 2, 8.0, seed=12, n_modes=6, n_markers=n_markers)
    g = gpu_lib.Case(p, parts, bodies, field, device=0)
    r = oracle_mod.OracleCase(p, parts, bodies, field)
    for c in (g, r):
        c.InitializationDEM()
        c.MultiDirectForcing()
    cnt = g.counters()
    nodes = cnt["nodes_u"] + cnt["nodes_v"] + cnt["nodes_w"]
    assert cnt["contributions"] > 40 * nodes, "the layout must be dense enough for the fallbacks"
    for a, b in zip(g.get_fluid(), r.get_fluid()):
        assert np.array_equal(a, b)
    gp, nl = g.get_parcels()
    rp, _ = r.get_parcels()
    cases.compare_parcels(gp, rp, nl)
    for c in (g, r):
        c.step(2)
    for a, b in zip(g.get_fluid(), r.get_fluid()):
        assert np.array_equal(a, b)
    gb, rb = g.get_bodies(), r.get_bodies()
    for f in ("x", "v", "omega"):
        assert cases.rel_close(gb[f], rb[f], 1e-9), f
    g.close()
