"""Pins of the CPU restatement of the unresolved CFD-DEM path.

The reference holds only the drag law of this path, so the restatement is
pinned by independent numpy restatements and identities of the definition in
include/ibmdem.h: volume conservation of the Gaussian volume fraction, the
normal contact law shared with the resolved path, exact action-reaction of
the contact force, the Coulomb limit of the tangential force and its torque,
the tangential history carried across steps, and one step of a single
particle falling through the fluid.
"""
import math

import numpy as np
import pytest

from ibmdem import scenario
from ibmdem.records import PARTICLE, make_uparams, ufield_shape


def two_particles(d_vec, v_rel, w_i=(0, 0, 0), mu=0.3, n=8, h=1e-3):
    p = make_uparams(n, n, n, h, 0.9e-3, dt=1e-5, gravity=(0.0, 0.0, 0.0), mu=mu, alphaMin=0.0)
    parts = np.zeros(2, PARTICLE)
    c = np.array([4.1, 3.9, 4.05]) * h
    parts["x"] = [c, c + np.asarray(d_vec)]
    parts["v"] = [[0, 0, 0], v_rel]
    parts["omega"][0] = w_i
    parts["rad"] = [0.15e-3, 0.12e-3]
    parts["rho"] = 2500.0
    parts["vol"] = np.pi / 6 * (2 * parts["rad"]) ** 3
    parts["m"] = parts["rho"] * parts["vol"]
    parts["I"] = 0.4 * parts["m"] * parts["rad"] ** 2
    parts["globalIdx"] = [1, 2]
    z = np.zeros(ufield_shape(p))
    return p, parts, (z, z, z)


def eta(e):
    pi2 = float(np.float32(np.float32(3.1415926536) * np.float32(3.1415926536)))
    return -2 * math.log(e) / math.sqrt(pi2 + math.log(e))


def normal_force(p, parts, d_vec):
    r = -np.asarray(d_vec, dtype=float)
    dist = math.sqrt(r @ r)
    n = r / dist
    m1, m2 = parts["m"]
    meff = 2 * m1 * m2 / (m1 + m2)
    kn = float(p["knCoeff"]) / (0.1 * float(p["dx"])) * meff
    etan = eta(float(p["ResistCoeff"])) * math.sqrt(meff * kn)
    vn = n @ (parts["v"][0] - parts["v"][1])
    fn = kn * (parts["rad"].sum() - dist) - etan * vn
    return n, fn, kn, meff


def test_volume_fraction_conserves_particle_volume(oracle_mod):
    p, parts, field = scenario.unresolved_case(16, 3000, seed=4, n_modes=4, alphaMin=0.0)
    r = oracle_mod.OracleUnresolved(p, parts, field)
    r.step(1)
    a = r.get_volume_fraction()
    vcell = float(p["dx"]) ** 3
    assert abs((1.0 - a).sum() * vcell - parts["vol"].sum()) <= 1e-12 * parts["vol"].sum()
    r.close()


def test_head_on_contact_matches_the_normal_law(oracle_mod):
    d_vec = np.array([0.25e-3, 0.0, 0.0])
    p, parts, field = two_particles(d_vec, [-0.01, 0.0, 0.0])
    r = oracle_mod.OracleUnresolved(p, parts, field)
    r.step(1)
    q = r.get_particles()
    n, fn, _, _ = normal_force(p, parts, d_vec)
    assert np.allclose(q["fcol"][0], fn * n, rtol=1e-13, atol=0)
    assert np.array_equal(q["fcol"][0], -q["fcol"][1])
    assert np.all(q["tcol"] == 0)
    st, partner, xi = r.get_contacts()
    assert list(st) == [0, 1, 2] and list(partner) == [1, 0]
    r.close()


def test_sliding_contact_is_coulomb_limited(oracle_mod):
    d_vec = np.array([0.0, 0.0, 0.26e-3])
    vt = np.array([0.5, 0.0, 0.0])  # fast tangential slip: the spring saturates at once
    p, parts, field = two_particles(d_vec, vt)
    r = oracle_mod.OracleUnresolved(p, parts, field)
    r.step(1)
    q = r.get_particles()
    n, fn, _, _ = normal_force(p, parts, d_vec)
    ft = q["fcol"][0] - fn * n
    assert abs(np.linalg.norm(ft) - 0.3 * abs(fn)) <= 1e-12 * abs(fn)
    # friction on particle 0 opposes its slip relative to particle 1 (it moves at -vt relative)
    assert ft @ vt > 0
    torque = -parts["rad"][0] * np.cross(n, ft)
    assert np.allclose(q["tcol"][0], torque, rtol=1e-12, atol=1e-30)
    assert np.array_equal(q["fcol"][0], -q["fcol"][1])
    r.close()


def test_tangential_history_accumulates_while_sticking(oracle_mod):
    d_vec = np.array([0.0, 0.265e-3, 0.0])
    vt = np.array([0.0, 0.0, 1e-6])  # slow: the spring sticks
    p, parts, field = two_particles(d_vec, vt)
    r = oracle_mod.OracleUnresolved(p, parts, field)
    r.step(1)
    _, _, xi1 = r.get_contacts()
    dt = float(p["dt"])
    # particle 0 sees particle 1 slide by +vt: relative tangential velocity -vt
    assert np.allclose(xi1[0], -vt * dt, rtol=1e-12, atol=1e-30)
    assert np.array_equal(xi1[0], -xi1[1])
    r.step(1)
    _, _, xi2 = r.get_contacts()
    assert xi2[0][2] < xi1[0][2] < 0
    r.close()


def test_single_particle_step(oracle_mod):
    n, h = 8, 1e-3
    p = make_uparams(n, n, n, h, 0.5e-3, dt=1e-5, alphaMin=0.0)
    parts = np.zeros(1, PARTICLE)
    parts["x"] = [[3.3e-3, 4.6e-3, 2.2e-3]]
    parts["v"] = [[0.01, -0.02, 0.05]]
    parts["rad"] = 0.125e-3
    parts["rho"] = 2500.0
    parts["vol"] = np.pi / 6 * (0.25e-3) ** 3
    parts["m"] = 2500.0 * parts["vol"]
    parts["I"] = 0.4 * parts["m"] * parts["rad"] ** 2
    shape = ufield_shape(p)
    vel = np.array([0.1, -0.05, 0.3])
    field = [np.full(shape, c) for c in vel]
    r = oracle_mod.OracleUnresolved(p, parts, field)
    r.step(1)
    q = r.get_particles()
    af = q["alphaf"][0]
    # uniform fluid: trilinear returns the uniform value; one particle's fraction
    assert 0.99 < af < 1.0
    beta = oracle_mod.drag_beta(2500.0, 0.125e-3, parts["v"][0], 1.2, af, vel)
    m = parts["m"][0]
    g = np.array([0.0, 0.0, -9.81])
    fd = (m * beta) * (vel - parts["v"][0])
    assert np.allclose(q["fdrag"][0], fd, rtol=1e-14)
    v_new = parts["v"][0] + 1e-5 * ((fd + 0.0) / m + (1 - 1.2 / 2500.0) * g)
    assert np.allclose(q["v"][0], v_new, rtol=1e-14)
    assert np.allclose(q["x"][0], parts["x"][0] + 1e-5 * v_new, rtol=1e-14)
    r.close()


def test_rejects_particles_outside_the_box(oracle_mod):
    p, parts, field = two_particles([0.25e-3, 0, 0], [0, 0, 0])
    parts["x"][1][0] = 9e-3
    with pytest.raises(RuntimeError):
        oracle_mod.OracleUnresolved(p, parts, field)
