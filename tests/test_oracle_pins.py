"""Pins of the CPU restatement that do not depend on the GPU library.

The reference has no tests or golden vectors for this path and cannot be
built here, so the restatement is pinned by identities the reference's
algorithm satisfies and by independent numpy restatements of its formulas:
partition of unity and linear exactness of the 3-point kernel, the
interpolation/spreading adjoint and momentum balance, pair symmetry, a
two-marker spring-dashpot contact, rigid-body rotation, periodic migration of
a marker and the single-precision literals of eta and the drag law.
"""
import math

import numpy as np
import pytest

import cases
from ibmdem import scenario
from ibmdem.records import MULTISPHERE, PARCEL, make_params


def phi(r):
    """3-point kernel of interpolation.F90:10-30 for |r| (numpy restatement)."""
    r = np.abs(r)
    out = np.zeros_like(r)
    a = r <= 0.5
    b = (r > 0.5) & (r <= 1.5)
    out[a] = (1 + np.sqrt(1 - 3 * r[a] * r[a])) / 3
    out[b] = (5 - 3 * r[b] - np.sqrt(1 - 3 * (1 - r[b]) ** 2)) / 6
    return out


def test_kernel_partition_of_unity_and_first_moment():
    x = np.random.default_rng(0).random(10000) * 7 + 3
    for shift in (0.0, 0.5):
        nodes = np.floor(x)[:, None] + np.arange(-3, 5)[None, :] + 0.5 - shift
        w = phi(x[:, None] - nodes)
        assert np.abs(w.sum(1) - 1).max() < 1e-14
        assert np.abs((w * (x[:, None] - nodes)).sum(1)).max() < 1e-13


def small_case(**kw):
    return cases.contact_case(**kw)


def test_weights_sum_to_one(oracle_mod):
    p, parts, bodies, field = small_case()
    r = oracle_mod.OracleCase(p, parts, bodies, field)
    r.InitializationDEM()
    pp, nl = r.get_parcels()
    w, cells = r.get_weights(len(pp))
    s = w[:nl].sum(axis=1)  # locals; images near the halo edge have truncated stencils
    assert np.abs(s - 1).max() < 1e-13


def test_linear_field_is_interpolated_exactly(oracle_mod):
    n = 24
    p = make_params(n, n, n)
    rng = np.random.default_rng(1)
    X = np.array([[12.3, 11.7, 12.1]])
    parts, bodies = scenario.sphere_bodies(X, 8.0, 1.0, 1.14e3, np.zeros((1, 3)))
    shape = (n + 4, n + 4, n + 4)
    idx = np.arange(-1, n + 3, dtype=float)
    # u on faces x=(i-1), v on y=(j-1), w on z=(k-1); cell centres elsewhere
    K, J, I = np.meshgrid(idx, idx, idx, indexing="ij")
    a = rng.standard_normal(4)
    u = a[0] + a[1] * (I - 1) + a[2] * (J - 0.5) + a[3] * (K - 0.5)
    v = a[0] + a[1] * (I - 0.5) + a[2] * (J - 1) + a[3] * (K - 0.5)
    w = a[0] + a[1] * (I - 0.5) + a[2] * (J - 0.5) + a[3] * (K - 1)
    r = oracle_mod.OracleCase(p, parts, bodies, (u, v, w))
    r.InitializationDEM()
    r.UpdateFluidVelocityOnLagrangianPoints()
    pp, nl = r.get_parcels()
    ulp = pp["vgap"][:nl] + pp["v"][:nl]
    x = pp["x"][:nl]
    exact = a[0] + a[1] * x[:, 0] + a[2] * x[:, 1] + a[3] * x[:, 2]
    for c in range(3):
        assert np.abs(ulp[:, c] - exact).max() < 1e-12


def test_spreading_adjoint_and_momentum_balance(oracle_mod):
    p, parts, bodies, field = small_case(seed=9)
    p["Ns"] = 1
    r = oracle_mod.OracleCase(p, parts, bodies, field)
    r.InitializationDEM()
    r.MultiDirectForcing()
    pp, nl = r.get_parcels()
    _, _, _, fx, fy, fz = r.get_fluid()
    sl = (slice(2, -2),) * 3
    fv = pp["fdrag"][:nl] * pp["vol"][:nl, None]
    ulp = pp["vgap"][:nl] + pp["v"][:nl]
    for c, f in enumerate((fx, fy, fz)):
        fi = f[sl]
        # momentum: every local's weights over the periodic interior sum to 1
        assert abs(fi.sum() + fv[:, c].sum()) <= 1e-11 * np.abs(fv[:, c]).sum()
        # adjoint: <f, u0> = -<fdrag vol, I u0>
        lhs = (fi * field[c][sl]).sum()
        rhs = -(fv[:, c] * ulp[:, c]).sum()
        assert abs(lhs - rhs) <= 1e-11 * np.abs(fv[:, c] * ulp[:, c]).sum()


def test_pair_lists_are_symmetric(oracle_mod):
    p, parts, bodies, field = small_case(seed=4)
    r = oracle_mod.OracleCase(p, parts, bodies, field)
    r.InitializationDEM()
    pp, nl = r.get_parcels()
    st, idx = r.get_collision_lists()
    assert len(idx) > 0
    pairs = set()
    for i in range(nl):
        for j in idx[st[i]:st[i + 1]] - 1:
            assert pp["MSIdx"][i] != pp["MSIdx"][j]
            d = pp["x"][i] - pp["x"][j]
            assert d @ d < (1.5 * 1.1) ** 2
            pairs.add((i, j))
    for i, j in pairs:
        if j < nl:
            assert (j, i) in pairs


def two_marker_case(dist, vrel):
    n = 16
    p = make_params(n, n, n, knCoeff=1e4, ResistCoeff=0.9)
    parts = np.zeros(2, PARCEL)
    parts["x"] = [[8.0, 8.0, 8.0], [8.0 + dist[0], 8.0 + dist[1], 8.0 + dist[2]]]
    parts["v"] = [[0, 0, 0], vrel]
    parts["radeff"] = 0.75
    parts["vol"] = 0.9
    parts["m"] = [900.0, 1300.0]
    parts["MSIdx"] = [1, 2]
    parts["globalIdx"] = 1
    bodies = np.zeros(2, MULTISPHERE)
    bodies["x"] = parts["x"]
    bodies["m"] = 1.0
    z = np.zeros((n + 4,) * 3)
    return p, parts, bodies, (z, z, z)


def test_two_marker_contact_force(oracle_mod):
    d = np.array([0.7, 0.5, -0.6])
    vrel = np.array([0.3, -0.1, 0.2])
    p, parts, bodies, field = two_marker_case(d, vrel)
    r = oracle_mod.OracleCase(p, parts, bodies, field)
    r.InitializationDEM()
    r.CalculateCollisionForce()
    pp, nl = r.get_parcels()
    assert nl == 2
    # numpy restatement of ZJS_COLLISION_DEM.F90:30-57 for marker 1 against marker 2
    e = 0.9
    pi2 = np.float32(np.float32(3.1415926536) * np.float32(3.1415926536))
    eta = -2 * math.log(e) / math.sqrt(float(pi2) + math.log(e))
    rvec = -d
    dist = math.sqrt(rvec @ rvec)
    nvec = rvec / dist
    m1, m2 = 900.0, 1300.0
    meff = 2 * m1 * m2 / (m1 + m2)
    kn = 1e4 / (0.1 * 1.0) * meff
    etan = eta * math.sqrt(meff * kn)
    vn = nvec @ (np.zeros(3) - vrel)
    f = nvec * (kn * (1.5 - dist) - etan * vn)
    assert np.allclose(pp["fcol"][0], f, rtol=1e-14, atol=0)
    assert np.array_equal(pp["fcol"][0], -pp["fcol"][1])
    assert oracle_mod.eta(e) == eta


def test_rigid_rotation(oracle_mod):
    n = 32
    p = make_params(n, n, n, gravity=(0.0, 0.0, 0.0))
    X = np.array([[16.2, 15.9, 16.4]])
    V = np.array([[0.01, -0.02, 0.005]])
    parts, bodies = scenario.sphere_bodies(X, 10.0, 1.0, 1.14e3, V)
    omega = np.array([0.3, -0.2, 0.5])
    bodies["omega"] = omega
    bodies["AngMom"] = bodies["I"][0] * omega
    z = np.zeros((n + 4,) * 3)
    r = oracle_mod.OracleCase(p, parts, bodies, (z, z, z))
    r.InitializationDEM()
    x0 = r.get_parcels()[0]["x"].copy()
    r.EvolutionMS()
    r.ResetVelocityAndPositionLagrangianPoints()
    pp, nl = r.get_parcels()
    b = r.get_bodies()[0]
    th = omega * 1e-3
    ang = np.linalg.norm(th)
    k = th / ang
    Kx = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
    R = np.eye(3) + math.sin(ang) * Kx + (1 - math.cos(ang)) * Kx @ Kx
    Xn = X[0] + V[0] * 1e-3
    assert np.allclose(b["x"], Xn, atol=1e-15)
    expect = (x0 + V[0] * 1e-3 - Xn) @ R.T + Xn
    assert np.abs(pp["x"][:nl] - expect).max() < 1e-12
    vexp = np.cross(b["omega"], pp["x"][:nl] - Xn) + b["v"]
    assert np.abs(pp["v"][:nl] - vexp).max() < 1e-14


def test_periodic_migration_moves_marker_behind_the_locals(oracle_mod):
    n = 16
    p = make_params(n, n, n, gravity=(0.0, 0.0, 0.0))
    parts = np.zeros(3, PARCEL)
    parts["x"] = [[15.9995, 8.0, 8.0], [5.0, 5.0, 5.0], [9.0, 3.0, 12.0]]
    parts["radeff"] = 0.75
    parts["vol"] = 1.0
    parts["m"] = 1.0
    parts["MSIdx"] = [1, 2, 3]
    parts["globalIdx"] = [1, 2, 3]
    bodies = np.zeros(3, MULTISPHERE)
    bodies["x"] = parts["x"]
    bodies["v"] = [[1.0, 0, 0], [0, 0, 0], [0, 0, 0]]
    bodies["m"] = 1.0
    bodies["rho"] = 1e3
    bodies["InertiaTensor"] = np.eye(3).reshape(9)
    bodies["rotMatGlo"] = np.eye(3).reshape(9)
    z = np.zeros((n + 4,) * 3)
    r = oracle_mod.OracleCase(p, parts, bodies, (z, z, z))
    r.InitializationDEM()
    r.EvolutionMS()
    r.ResetVelocityAndPositionLagrangianPoints()
    r.AdjustParcelPosition()
    r.UpdateParcelInfoInGhostRegion()
    r.RebuildAllListOrNot()
    pp, nl = r.get_parcels()
    assert nl == 3
    assert list(pp["globalIdx"][:3]) == [2, 3, 1]
    assert pp["x"][2][0] == (15.9995 + 1.0 * 1e-3) + (-16.0)


def test_drag_law_restatement(oracle_mod):
    rng = np.random.default_rng(3)
    f32 = lambda v: float(np.float32(v))  # noqa: E731
    for _ in range(50):
        rho, rad = 2500.0, rng.random() * 1e-3 + 1e-4
        vp = rng.standard_normal(3) * 0.1
        velf = rng.standard_normal(3) * 0.1
        alpha = rng.random() * 0.6 + 0.35
        beta = oracle_mod.drag_beta(rho, rad, vp, 1000.0, alpha, velf)
        for j in range(3):
            Ur = abs(velf[j] - vp[j])
            Re = max(1.0, Ur * 2 * rad / 1e-5)
            zeta = f32(3.7) - f32(0.65) * math.exp(-0.5 * (1.5 - math.log10(Re)) ** 2)
            fb = 1 + 1.0 / 6.0 * Re ** f32(0.687) if Re < 1000 else f32(0.0183) * Re
            f = f32(8.33) * (1 - alpha) / alpha + f32(0.0972) * Re if alpha < f32(0.8) else fb * alpha ** (-zeta)
            b = 0.75 * (24.0 / Re * f * Ur) / (2 * rad * rho / 1000.0)
            assert beta[j] == pytest.approx(b, rel=1e-12)
