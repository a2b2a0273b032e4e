"""Tangential friction of the marker contacts on the GPU against the CPU restatement.

ibmdem_set_friction adds a tangential spring, damping and a Coulomb limit to the
reference's normal contact law, with the tangential displacement of every
touching pair kept across calls by the persistent ids of both parcels (their
index in the array given to set_parcels; the markers' globalIdx is numbered per
body in these cases, so it could not serve as the key).  A periodic
case whose first two bodies press into each other (one straddling a periodic
face, so that some contacts are with images): three contact-force calls on the
same positions, with the lists rebuilt between them, must give bit-identical
forces and tangential history; over six steps of 3 DEM sub-steps each the
lists stay identical and forces, history and bodies agree within 1e-9 relative
(the body rotation uses CUDA's cos/sin).  With friction off the forces are
those of the normal law (the other parity tests run that way).
"""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu

KT_RATIO, MU = 2.0 / 7.0, 0.3


def _pair(gpu_lib, oracle_mod):
    p, parts, bodies, field = cases.contact_case(seed=11, gap=-0.3, coupleInterval=3, vel_std=0.05)
    g = gpu_lib.Case(p, parts, bodies, field, device=0)
    r = oracle_mod.OracleCase(p, parts, bodies, field)
    for c in (g, r):
        c.set_friction(KT_RATIO, MU)
        c.InitializationDEM()
    return g, r


def _history(c):
    start, gid, xi = c.get_friction_history()
    return start, gid, xi


def test_friction_matches_restatement(gpu_lib, oracle_mod):
    g, r = _pair(gpu_lib, oracle_mod)
    # identical input: three contact-force calls on the same positions, the
    # lists rebuilt between them; forces and history bit-identical
    for k in range(3):
        if k:
            for c in (g, r):
                c.RebuildAllListOrNot()
        for c in (g, r):
            c.CalculateCollisionForce()
        gs, gi = g.get_collision_lists()
        rs, ri = r.get_collision_lists()
        assert np.array_equal(gs, rs) and np.array_equal(gi, ri), k
        gp, nl = g.get_parcels()
        rp, _ = r.get_parcels()
        d = np.abs(gp["fcol"][:nl] - rp["fcol"][:nl]).max()
        assert np.array_equal(gp["fcol"][:nl], rp["fcol"][:nl]), (k, d)
        (a0, a1, a2), (b0, b1, b2) = _history(g), _history(r)
        assert np.array_equal(a0, b0) and np.array_equal(a1, b1), k
        assert np.array_equal(a2, b2), (k, np.abs(a2 - b2).max())
    touching = int((a1 >= 0).sum())
    assert touching > 10, "the case must keep contacts with history"
    assert np.abs(a2).max() > 0
    g.close()
    r.close()
    # trajectories: 3 sub-steps per step, history carried through the steps
    g, r = _pair(gpu_lib, oracle_mod)
    for s in range(6):
        for c in (g, r):
            c.step(1)
        gs, gi = g.get_collision_lists()
        rs, ri = r.get_collision_lists()
        assert np.array_equal(gs, rs) and np.array_equal(gi, ri), s
        gp, nl = g.get_parcels()
        rp, _ = r.get_parcels()
        assert cases.rel_close(gp["fcol"][:nl], rp["fcol"][:nl], 1e-9), s
        (a0, a1, a2), (b0, b1, b2) = _history(g), _history(r)
        assert np.array_equal(a0, b0) and np.array_equal(a1, b1), s
        assert cases.rel_close(a2, b2, 1e-9), s
        gb, rb = g.get_bodies(), r.get_bodies()
        for f in ("x", "v", "omega", "fmomCol"):
            assert cases.rel_close(gb[f], rb[f], 1e-9), (s, f)
    g.close()
    r.close()


def test_friction_changes_the_torque_and_switches_off(gpu_lib, oracle_mod):
    p, parts, bodies, field = cases.contact_case(seed=11, gap=-0.3, coupleInterval=3, vel_std=0.05)
    out = []
    for kt in (KT_RATIO, 0.0):
        g = gpu_lib.Case(p, parts, bodies, field, device=0)
        g.set_friction(KT_RATIO, MU)
        g.set_friction(kt, MU)
        g.InitializationDEM()
        g.step(2)
        out.append((g.get_bodies(), g.get_friction_history()))
        g.close()
    ref = gpu_lib.Case(p, parts, bodies, field, device=0)
    ref.InitializationDEM()
    ref.step(2)
    rb = ref.get_bodies()
    ref.close()
    (bf, hf), (b0, h0) = out
    assert not np.array_equal(bf["fmomCol"], b0["fmomCol"]), "friction must act"
    for f in ("x", "v", "omega", "fmomCol", "fcol"):
        assert np.array_equal(b0[f], rb[f]), f
    assert h0[1].size == 0
