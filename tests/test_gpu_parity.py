"""GPU parity against the CPU restatement, through the C ABI.

Bit-exact: cell lists (cell -> ordered part indices), contact lists (in order),
parcel positions/velocities/forces, delta-weight interpolation, direct forcing,
spread forcing and the post-guess velocity field.  Within 1e-9 relative: body
state after the Rodrigues rotation (CUDA's cos/sin vs glibc's).
"""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu


def _pair(gpu_lib, oracle_mod, case):
    p, parts, bodies, field = case
    g = gpu_lib.Case(p, parts, bodies, field, device=0)
    r = oracle_mod.OracleCase(p, parts, bodies, field)
    return g, r


def _cmp_lists(g, r):
    gs, gi = g.get_cell_lists()
    rs, ri = r.get_cell_lists()
    assert np.array_equal(gs, rs), "cell starts differ"
    assert np.array_equal(gi, ri), "cell items differ"
    gs, gi = g.get_collision_lists()
    rs, ri = r.get_collision_lists()
    assert np.array_equal(gs, rs), "collision list starts differ"
    assert np.array_equal(gi, ri), "collision lists differ"
    return len(gi)


def _cmp_state(g, r, exact_bodies=False):
    gp, gnl = g.get_parcels()
    rp, rnl = r.get_parcels()
    assert gnl == rnl
    cases.compare_parcels(gp, rp, gnl)
    for a, b in zip(g.get_fluid(), r.get_fluid()):
        assert np.array_equal(a, b)
    gb, rb = g.get_bodies(), r.get_bodies()
    for f in ("x", "v", "omega", "AngMom", "fdrag", "fcol", "fmom", "fmomCol", "fhydro", "fmomHydro",
              "rotMatGlo"):
        if exact_bodies:
            assert np.array_equal(gb[f], rb[f]), f
        else:
            assert cases.rel_close(gb[f], rb[f], 1e-9), f


def test_init_lists_and_images(gpu_lib, oracle_mod):
    g, r = _pair(gpu_lib, oracle_mod, cases.contact_case())
    g.InitializationDEM()
    r.InitializationDEM()
    npairs = _cmp_lists(g, r)
    assert npairs > 0
    gp, gnl = g.get_parcels()
    rp, rnl = r.get_parcels()
    assert len(gp) > gnl, "the straddling body must produce periodic images"
    cases.compare_parcels(gp, rp, gnl)


def test_subroutines_one_by_one(gpu_lib, oracle_mod):
    """The fluid step's particle side, subroutine by subroutine."""
    g, r = _pair(gpu_lib, oracle_mod, cases.contact_case(seed=5))
    for c in (g, r):
        c.InitializationDEM()
        c.MultiDirectForcing()
    _cmp_state(g, r, exact_bodies=True)
    for c in (g, r):
        c.CalculateCollisionForce()
        c.AssembleLocalForceMS()
    _cmp_state(g, r, exact_bodies=True)
    for c in (g, r):
        c.EvolutionMS()
        c.ResetVelocityAndPositionLagrangianPoints()
        c.AdjustParcelPosition()
        c.UpdateParcelInfoInGhostRegion()
        c.RebuildAllListOrNot()
    _cmp_lists(g, r)
    _cmp_state(g, r)


def test_one_step(gpu_lib, oracle_mod):
    g, r = _pair(gpu_lib, oracle_mod, cases.contact_case(seed=7))
    for c in (g, r):
        c.InitializationDEM()
        c.step(1)
    _cmp_lists(g, r)
    _cmp_state(g, r)


@pytest.mark.parametrize("couple", [1, 3, 10])
def test_trajectory(gpu_lib, oracle_mod, couple):
    g, r = _pair(gpu_lib, oracle_mod, cases.contact_case(seed=11, coupleInterval=couple))
    for c in (g, r):
        c.InitializationDEM()
    for s in range(6):
        g.step(1)
        r.step(1)
        gb, rb = g.get_bodies(), r.get_bodies()
        for f in ("x", "v", "omega"):
            assert cases.rel_close(gb[f], rb[f], 1e-9), (s, f)
        # the body sums after the step are the last AssembleLocalForceMS's (the
        # library forms only the sums each call's readers need; with several
        # sub-steps the markers have moved since the first call, so fmom would
        # differ by about 1e-5 if the first call's were kept)
        for f in ("fdrag", "fmom"):
            assert cases.rel_close(gb[f], rb[f], 1e-8), (s, f)
    gp, nl = g.get_parcels()
    rp, _ = r.get_parcels()
    assert len(gp) == len(rp)
    assert cases.rel_close(gp["x"][:nl], rp["x"][:nl], 1e-12)


def test_async_fluid_readout_matches_sync(gpu_lib):
    """ibmdem_get_fluid_async overlapping CloudEvolutionMS returns the fields that
    ibmdem_get_fluid returns right after MultiDirectForcing, and the next step,
    which writes the fields, waits for the copies."""
    import ctypes

    import torch

    p, parts, bodies, field = cases.contact_case(seed=6)
    case = gpu_lib.Case(p, parts, bodies, field, device=0)
    case.InitializationDEM()
    case.MultiDirectForcing()
    ref = case.get_fluid()
    case.close()
    case = gpu_lib.Case(p, parts, bodies, field, device=0)
    case.InitializationDEM()
    case.MultiDirectForcing()
    out = [torch.empty(f.shape, dtype=torch.float64, pin_memory=True).numpy() for f in ref]
    s = torch.cuda.Stream()
    rc = case.lib.ibmdem_get_fluid_async(case.h, *[o.ctypes.data for o in out], ctypes.c_void_p(s.cuda_stream))
    assert rc == 0
    case.CloudEvolutionMS()
    case.step(1)  # writes the fields: ordered after the copies
    s.synchronize()
    for a, b in zip(out, ref):
        assert np.array_equal(a, b)
    case.close()


def test_step_graph_matches_kernel_by_kernel(gpu_lib):
    """ibmdem_step as replays of its captured graph (the default) and kernel by
    kernel on the context's stream give the same parcels, bodies and fields; a
    change of the parcels between steps makes the graph be captured again."""
    out = []
    for graphs in (True, False):
        p, parts, bodies, field = cases.contact_case(seed=9, coupleInterval=2)
        c = gpu_lib.Case(p, parts, bodies, field, device=0)
        c.set_step_graphs(graphs)
        c.InitializationDEM()
        c.step(3)
        # new parcels (the same ones again) in the middle of the run
        gp, nl = c.get_parcels()
        c.set_parcels(gp[:nl].copy())
        c.InitializationDEM()
        c.step(2)
        out.append((c.get_parcels(), c.get_bodies(), c.get_fluid(), c.launches))
        c.close()
    (pa, nla), ba, fa, la = out[0]
    (pb, nlb), bb, fb, lb = out[1]
    assert nla == nlb and len(pa) == len(pb)
    for f in ("x", "v", "fcol", "fdrag", "vgap", "globalIdx", "MSIdx", "cellIdx"):
        assert np.array_equal(pa[f], pb[f]), f
    for f in ("x", "v", "omega", "AngMom", "rotMatGlo", "fcol", "fdrag", "fmom", "fmomCol"):
        assert np.array_equal(ba[f], bb[f]), f
    for x, y in zip(fa, fb):
        assert np.array_equal(x, y)
    assert la == lb  # the graph counts the kernels it replays
