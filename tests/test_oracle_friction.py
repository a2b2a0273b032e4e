"""Pins of the tangential friction of the marker contacts in the CPU restatement.

The reference's marker contact law is normal only (ZJS_COLLISION_DEM.F90:53-57);
the library adds, behind ibmdem_set_friction (off by default), a tangential
spring with damping and a Coulomb limit whose displacement is kept per pair
across calls.  These checks pin the restatement against a numpy restatement of
that law on two touching markers of different bodies: a sliding contact sits on
the Coulomb limit, a sticking one accumulates its displacement call after call
(also across a list rebuild), action and reaction are exactly opposite, and
with friction off the force is the reference's normal law.
"""
import math

import numpy as np

from ibmdem.records import MULTISPHERE, PARCEL, make_params

E = 0.9
KT_RATIO, MU = 2.0 / 7.0, 0.3
DT = 1e-3


def eta():
    pi2 = np.float32(np.float32(3.1415926536) * np.float32(3.1415926536))
    return -2 * math.log(E) / math.sqrt(float(pi2) + math.log(E))


def case(d, vrel):
    n = 16
    p = make_params(n, n, n, knCoeff=1e4, ResistCoeff=E, dt=DT)
    parts = np.zeros(2, PARCEL)
    parts["x"] = [[8.0, 8.0, 8.0], [8.0 + d[0], 8.0 + d[1], 8.0 + d[2]]]
    parts["v"] = [[0, 0, 0], vrel]
    parts["radeff"] = 0.75
    parts["vol"] = 0.9
    parts["m"] = [900.0, 1300.0]
    parts["MSIdx"] = [1, 2]
    parts["globalIdx"] = [1, 2]
    bodies = np.zeros(2, MULTISPHERE)
    bodies["x"] = parts["x"]
    bodies["m"] = 1.0
    z = np.zeros((n + 4,) * 3)
    return p, parts, bodies, (z, z, z)


def law(d, vrel, h_old):
    """numpy restatement for marker 1 (at rest) against marker 2: (f, h)."""
    r = -np.asarray(d, float)
    dist = math.sqrt(r @ r)
    n = r / dist
    m1, m2 = 900.0, 1300.0
    meff = 2 * m1 * m2 / (m1 + m2)
    kn = 1e4 / (0.1 * 1.0) * meff
    et = eta()
    etan = et * math.sqrt(meff * kn)
    u = np.zeros(3) - np.asarray(vrel, float)
    vn = n @ u
    fn = kn * (1.5 - dist) - etan * vn
    vt = u - vn * n
    h = h_old - (n @ h_old) * n + DT * vt
    kt = KT_RATIO * kn
    etat = et * math.sqrt(meff * kt)
    ft = -kt * h - etat * vt
    lim = MU * abs(fn)
    if np.linalg.norm(ft) > lim:
        ft = ft * (lim / np.linalg.norm(ft))
        h = -(ft + etat * vt) / kt
    return n * fn + ft, h, fn, ft


def run(oracle_mod, d, vrel, calls, rebuild=False):
    p, parts, bodies, field = case(d, vrel)
    r = oracle_mod.OracleCase(p, parts, bodies, field)
    r.set_friction(KT_RATIO, MU)
    r.InitializationDEM()
    out = []
    for k in range(calls):
        if rebuild and k:
            r.RebuildAllListOrNot()
        r.CalculateCollisionForce()
        pp, nl = r.get_parcels()
        out.append((pp["fcol"][:nl].copy(), r.get_friction_history()))
    r.close()
    return out


def test_sliding_contact_sits_on_the_coulomb_limit(oracle_mod):
    d = np.array([1.49, 0.05, 0.0])  # a light overlap
    vrel = np.array([0.0, 300.0, -200.0])  # fast tangential motion: slides at once
    (f, (start, gid, xi)), = run(oracle_mod, d, vrel, 1)
    ref, h, fn, ft = law(d, vrel, np.zeros(3))
    assert np.allclose(f[0], ref, rtol=1e-13, atol=0)
    assert abs(np.linalg.norm(ft) - MU * abs(fn)) <= 1e-12 * abs(fn)
    assert list(start) == [0, 1, 2] and list(gid) == [1, 0]  # partners' parcel ids
    assert np.allclose(xi[0], h, rtol=1e-12, atol=1e-18)
    assert np.array_equal(f[0], -f[1])
    assert np.array_equal(xi[0], -xi[1])


def test_sticking_contact_accumulates_its_displacement(oracle_mod):
    d = np.array([1.3, 0.2, 0.1])
    vrel = np.array([1e-4, 2e-6, -1e-6])  # slow tangential motion: sticks
    res = run(oracle_mod, d, vrel, 3, rebuild=True)
    h = np.zeros(3)
    for k, (f, (start, gid, xi)) in enumerate(res):
        ref, h, fn, ft = law(d, vrel, h)
        assert np.linalg.norm(ft) < MU * abs(fn), "the contact must stick"
        assert np.allclose(f[0], ref, rtol=1e-13, atol=0), k
        assert np.allclose(xi[0], h, rtol=1e-12, atol=0), k
        assert np.array_equal(f[0], -f[1])
    n = -d / np.linalg.norm(d)
    vt = -vrel - (n @ -vrel) * n
    assert np.allclose(h, 3 * DT * vt, rtol=1e-12, atol=0)


def test_friction_off_is_the_reference_law(oracle_mod):
    d = np.array([1.3, 0.2, 0.1])
    vrel = np.array([0.0, 3.0, -2.0])
    p, parts, bodies, field = case(d, vrel)
    a = oracle_mod.OracleCase(p, parts, bodies, field)
    b = oracle_mod.OracleCase(p, parts, bodies, field)
    b.set_friction(KT_RATIO, MU)
    b.set_friction(0.0, 0.0)
    for r in (a, b):
        r.InitializationDEM()
        r.CalculateCollisionForce()
    fa = a.get_parcels()[0]["fcol"]
    fb = b.get_parcels()[0]["fcol"]
    assert np.array_equal(fa, fb)
    _, fn_only, fn, _ = law(d, vrel, np.zeros(3))
    r_ = -d / np.linalg.norm(d)
    assert np.allclose(fa[0], r_ * fn, rtol=1e-14, atol=0)
    assert b.get_friction_history()[1].size == 0
    a.close()
    b.close()


def test_separated_pair_keeps_no_history(oracle_mod):
    d = np.array([1.55, 0.0, 0.0])  # listed (within the 1.1 buffer) but not touching
    (f, (start, gid, xi)), = run(oracle_mod, d, np.array([0.0, 1.0, 0.0]), 1)
    assert np.array_equal(f, np.zeros_like(f))
    assert list(gid) == [-1, -1] and np.array_equal(xi, np.zeros_like(xi))
