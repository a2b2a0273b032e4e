"""Solid walls in the CPU restatement, pinned without the GPU library.

Walls (bType 1) change four things in the reference: the ghost region mirrors
the parcels near a wall about it (ZJS_MPI_DEM.F90:173-269), those mirror images
are never contact partners (ZJS_UPDATE_LIST_DEM.F90:272), parcels next to a
wall feel a parcel-plane spring-dashpot with probe sums
(ZJS_COLLISION_DEM.F90:76-179), and the fluid halo beyond a wall holds the
negated mirror with a zero wall-normal component (boundary.F90:211-245,
fluid.F90:240-249).  Each is checked here against an independent numpy
restatement or the formula.
"""
import math

import numpy as np
import pytest

from ibmdem import scenario
from ibmdem.records import MULTISPHERE, PARCEL, WALL_PROBE, field_shape, make_params


def eta_of(e):
    pi2 = np.float32(np.float32(3.1415926536) * np.float32(3.1415926536))
    return -2 * math.log(e) / math.sqrt(float(pi2) + math.log(e))


def one_marker_case(x, v, walls="z", n=12):
    p = make_params(n, n, n, walls=walls, knCoeff=1e4, ResistCoeff=0.9)
    parts = np.zeros(1, PARCEL)
    parts["x"] = [x]
    parts["v"] = [v]
    parts["radeff"] = 0.75
    parts["vol"] = 0.9
    parts["m"] = 900.0
    parts["MSIdx"] = 1
    parts["globalIdx"] = 1
    bodies = np.zeros(1, MULTISPHERE)
    bodies["x"] = parts["x"]
    bodies["m"] = 1.0
    z = np.zeros(field_shape(p))
    return p, parts, bodies, (z, z.copy(), z.copy())


def test_wall_contact_force_and_probe(oracle_mod):
    x = [6.2, 5.3, 0.4]  # 0.4 above the low z wall, radeff 0.75
    v = [0.01, 0.0, -0.05]
    p, parts, bodies, field = one_marker_case(x, v)
    r = oracle_mod.OracleCase(p, parts, bodies, field)
    probes = np.zeros(2, WALL_PROBE)
    probes["face"] = 5
    probes[0]["points"] = [[5, 5, 0], [7, 5, 0], [7, 6, 0], [5, 6, 0]]  # contains (6.2, 5.3)
    probes[1]["points"] = [[0, 0, 0], [2, 0, 0], [2, 2, 0], [0, 2, 0]]  # does not
    r.set_wall_probes(probes)
    r.InitializationDEM()
    r.CalculateCollisionForce()
    r.CalculateSolidBoundaryCollisionForce()
    pp, nl = r.get_parcels()
    m = 900.0
    kn = 1e4 / (0.1 * 1.0) * m
    etan = eta_of(0.9) * math.sqrt(m * kn)
    delta = 0.75 - 0.4
    f = np.array([0.0, 0.0, 1.0]) * (kn * delta - etan * (-0.05))
    assert np.allclose(pp["fcol"][0], f, rtol=1e-14, atol=0)
    got = r.get_wall_probes()
    assert np.allclose(got[0]["force"], [0.0, 0.0, kn * delta], rtol=1e-14, atol=0)
    assert np.array_equal(got[1]["force"], np.zeros(3))


def test_no_wall_force_away_from_the_wall(oracle_mod):
    p, parts, bodies, field = one_marker_case([6.2, 5.3, 0.8], [0, 0, -0.1])
    r = oracle_mod.OracleCase(p, parts, bodies, field)
    r.InitializationDEM()
    r.CalculateCollisionForce()
    r.CalculateSolidBoundaryCollisionForce()
    assert np.array_equal(r.get_parcels()[0]["fcol"][0], np.zeros(3))


def test_wall_images_are_mirrors_and_never_partners(oracle_mod):
    p, parts, bodies, field = scenario.walled_case(20, 20, 20, 3, 8.0, seed=4, walls="z", n_modes=0)
    r = oracle_mod.OracleCase(p, parts, bodies, field)
    r.InitializationDEM()
    pp, nl = r.get_parcels()
    loc = pp[:nl]
    img = pp[nl:]
    kz = np.floor(loc["x"][:, 2]).astype(int) + 1
    near_lo = (kz >= 1) & (kz <= 2)
    near_hi = (kz >= 19) & (kz <= 20)
    walled = img[img["pType"] == 1]
    # every parcel in the two cell layers next to a wall has exactly one pure z mirror
    pure = walled[(walled["x"][:, 0] >= 0) & (walled["x"][:, 0] < 20) & (walled["x"][:, 1] >= 0) &
                  (walled["x"][:, 1] < 20)]
    assert len(pure) == near_lo.sum() + near_hi.sum()
    lo_src = loc[near_lo]
    lo_img = pure[pure["x"][:, 2] < 0]
    # the face loop makes the images beyond the high wall first (iteration of face 5)
    assert np.array_equal(lo_img["globalIdx"], lo_src["globalIdx"])
    assert np.array_equal(lo_img["x"][:, 2], 0.0 - lo_src["x"][:, 2])
    assert np.array_equal(lo_img["v"][:, 2], -lo_src["v"][:, 2])
    assert np.array_equal(lo_img["v"][:, :2], lo_src["v"][:, :2])
    hi_img = pure[pure["x"][:, 2] >= 20]
    assert np.array_equal(hi_img["x"][:, 2], 2 * 20.0 - loc[near_hi]["x"][:, 2])
    # no image across a wall is anyone's contact partner; periodic images may be
    start, idx = r.get_collision_lists()
    assert np.all(pp["pType"][idx - 1] == -1)
    assert nl > 0 and len(walled) > 0


def test_halo_refill_matches_numpy_restatement(oracle_mod):
    # random interior field; VelocityPostGuess with fx = fxOld = 0 leaves the
    # interior as it is and refills the halo: compare with scenario.fill_halo
    for walls in ("z", "xy", "xyz", ""):
        n = 8
        p = make_params(n, n + 2, n + 1, walls=walls)
        rng = np.random.default_rng(len(walls))
        shape = field_shape(p)
        f = [rng.standard_normal(shape) for _ in range(3)]
        parts = np.zeros(1, PARCEL)
        parts["x"] = [[4.1, 4.2, 4.3]]
        parts["radeff"], parts["vol"], parts["m"], parts["MSIdx"] = 0.75, 0.9, 900.0, 1
        bodies = np.zeros(1, MULTISPHERE)
        bodies["m"] = 1.0
        r = oracle_mod.OracleCase(p, parts, bodies, [a.copy() for a in f])
        r.VelocityPostGuess()
        u, v, w = r.get_fluid()[:3]
        want = scenario.fill_halo(p, [a.copy() for a in f])
        for got, exp in zip((u, v, w), want):
            assert np.array_equal(got, exp), walls
        if "z" in walls:
            assert np.all(w[:3] == 0) and np.all(w[-2:] == 0)
            assert np.array_equal(u[1], -u[2]) and np.array_equal(u[0], -u[3])


def test_unsupported_face_mix_is_refused(oracle_mod):
    p = make_params(8, 8, 8)
    p["bType"] = [1, 0, 0, 0, 0, 0]
    z = np.zeros(field_shape(p))
    with pytest.raises(Exception):
        oracle_mod.OracleCase(p, np.zeros(0, PARCEL), np.zeros(0, MULTISPHERE), (z, z, z))
