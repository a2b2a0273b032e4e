"""Solid walls on the GPU against the CPU restatement, through the C ABI.

Cases with walls on z (x, y periodic) and on all three axes.  Bit-exact: cell
lists, contact lists (wall images never partners), images with their pType,
the wall spring-dashpot added to fcol, the probe sums, and the post-guess
field with the negated mirrors and the zero wall-normal velocity.  Within
1e-9 relative: body state over several steps (CUDA's cos/sin vs glibc's).
"""
import numpy as np
import pytest

import cases
from ibmdem import scenario
from ibmdem.records import WALL_PROBE

pytestmark = pytest.mark.gpu


def walled(walls="z", seed=2, n=24, nb=4):
    return scenario.walled_case(n, n, n, nb, 8.0, seed=seed, walls=walls, n_modes=8, touching=2)


def probes_for(p, walls):
    n = int(p["nx"])
    pr = np.zeros(3, WALL_PROBE)
    d = "xyz".index(walls[0])  # the touching bodies rest on this axis' low wall
    pr["face"] = 2 * d + 1
    e0, e1 = [e for e in range(3) if e != d]
    # three quadrilaterals on the low wall: two halves and an overlapping middle strip
    for q, (a0, a1) in enumerate([(0.0, 0.5), (0.5, 1.0), (0.25, 0.75)]):
        lo, hi = a0 * n, a1 * n
        quad = np.array([[lo, 0.0], [hi, 0.0], [hi, n], [lo, n]])
        pts = np.zeros((4, 3))
        pts[:, e0], pts[:, e1] = quad[:, 0], quad[:, 1]
        pr[q]["points"] = pts
    return pr


def pair(gpu_lib, oracle_mod, case, walls):
    p, parts, bodies, field = case
    g = gpu_lib.Case(p, parts, bodies, field, device=0)
    r = oracle_mod.OracleCase(p, parts, bodies, field)
    pr = probes_for(p, walls)
    g.set_wall_probes(pr)
    r.set_wall_probes(pr)
    return g, r


def cmp_lists(g, r):
    for a, b in zip(g.get_cell_lists(), r.get_cell_lists()):
        assert np.array_equal(a, b)
    gs, gi = g.get_collision_lists()
    rs, ri = r.get_collision_lists()
    assert np.array_equal(gs, rs) and np.array_equal(gi, ri)
    return len(gi)


def cmp_parcels(g, r):
    gp, gnl = g.get_parcels()
    rp, rnl = r.get_parcels()
    assert gnl == rnl
    cases.compare_parcels(gp, rp, gnl)
    assert np.array_equal(gp["pType"], rp["pType"])
    return gp, gnl


@pytest.mark.parametrize("walls", ["z", "xyz"])
def test_wall_images_and_lists(gpu_lib, oracle_mod, walls):
    g, r = pair(gpu_lib, oracle_mod, walled(walls), walls)
    g.InitializationDEM()
    r.InitializationDEM()
    cmp_lists(g, r)
    gp, nl = cmp_parcels(g, r)
    assert np.any(gp["pType"][nl:] == 1), "parcels next to a wall must have mirror images"


@pytest.mark.parametrize("walls", ["z", "xyz"])
def test_wall_force_probes_and_field(gpu_lib, oracle_mod, walls):
    g, r = pair(gpu_lib, oracle_mod, walled(walls, seed=5), walls)
    for c in (g, r):
        c.InitializationDEM()
        c.MultiDirectForcing()
    for a, b in zip(g.get_fluid(), r.get_fluid()):
        assert np.array_equal(a, b)
    for c in (g, r):
        c.CalculateCollisionForce()
        c.CalculateSolidBoundaryCollisionForce()
    gp, nl = cmp_parcels(g, r)
    gpr, rpr = g.get_wall_probes(), r.get_wall_probes()
    assert np.array_equal(gpr["force"], rpr["force"])
    assert np.any(gpr["force"] != 0), "the touching bodies press on the probed wall"
    # the wall pushes away from itself: positive normal force on the low wall's neighbours
    d = "xyz".index(walls[0])
    assert np.any(gp["fcol"][:nl, d] > 0)


@pytest.mark.parametrize("walls", ["z", "xyz"])
def test_wall_trajectory(gpu_lib, oracle_mod, walls):
    g, r = pair(gpu_lib, oracle_mod, walled(walls, seed=8), walls)
    for c in (g, r):
        c.InitializationDEM()
    g.step(1)
    r.step(1)
    cmp_lists(g, r)
    cmp_parcels(g, r)
    for a, b in zip(g.get_fluid(), r.get_fluid()):
        assert np.array_equal(a, b)
    for s in range(4):
        g.step(1)
        r.step(1)
        gb, rb = g.get_bodies(), r.get_bodies()
        for f in ("x", "v", "omega", "fcol"):
            assert cases.rel_close(gb[f], rb[f], 1e-9), (s, f)
    gp, nl = g.get_parcels()
    rp, _ = r.get_parcels()
    assert cases.rel_close(gp["x"][:nl], rp["x"][:nl], 1e-12)
    assert cases.rel_close(g.get_wall_probes()["force"], r.get_wall_probes()["force"], 1e-9)
