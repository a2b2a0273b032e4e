"""CompressDEM with parcels to drop among the locals: a sphere that overlaps a
solid wall leaves some of its markers below the wall face, outside the
interior cells, and the reference's compaction drops them.  Every kept parcel
behind a dropped one moves to a lower slot (the in-place compaction's moving
path), so the parcel records, cell lists, contact lists and body state after
the rebuilds must equal the CPU restatement's, bit for bit (bodies to 1e-9)."""
import numpy as np
import pytest

import cases
from ibmdem import scenario

pytestmark = pytest.mark.gpu


def overlapping_case():
    p, parts, bodies, field = scenario.walled_case(24, 24, 24, 4, 8.0, seed=5, walls="z", n_modes=8, touching=0)
    x = bodies["x"].copy()
    # the first body's lowest markers (radius 4 - 0.3) 0.8 below the low z face
    x[0, 2] = 3.7 - 0.8
    parts, bodies2 = scenario.sphere_bodies(x, 8.0, 1.0, 1.14e3, bodies["v"])
    for a in (0, 1):
        parts["x"][:, a] = np.mod(parts["x"][:, a], 24.0)
    return p, parts, bodies2, field


def test_locals_dropped_and_compacted(gpu_lib, oracle_mod):
    p, parts, bodies, field = overlapping_case()
    assert (parts["x"][:, 2] < 0.0).any(), "some markers must start below the wall face"
    g = gpu_lib.Case(p, parts, bodies, field, device=0)
    r = oracle_mod.OracleCase(p, parts, bodies, field)
    for c in (g, r):
        c.InitializationDEM()
    gp, gnl = g.get_parcels()
    rp, rnl = r.get_parcels()
    assert gnl == rnl and gnl < len(parts), "the markers below the face are dropped"
    cases.compare_parcels(gp, rp, gnl)
    for c in (g, r):
        c.step(2)
    for a, b in zip(g.get_cell_lists(), r.get_cell_lists()):
        assert np.array_equal(a, b)
    gs, gi = g.get_collision_lists()
    rs, ri = r.get_collision_lists()
    assert np.array_equal(gs, rs) and np.array_equal(gi, ri)
    gp, gnl = g.get_parcels()
    rp, rnl = r.get_parcels()
    assert gnl == rnl
    cases.compare_parcels(gp, rp, gnl)
    for a, b in zip(g.get_fluid(), r.get_fluid()):
        assert np.array_equal(a, b)
    gb, rb = g.get_bodies(), r.get_bodies()
    for f in ("x", "v", "omega"):
        assert cases.rel_close(gb[f], rb[f], 1e-9), f
    g.close()
