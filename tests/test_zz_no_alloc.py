"""ibmdem_interpolate_velocity_noalloc against ibmdem_UpdateFluidVelocityOnLagrangianPoints.

The allocation-free entry point serves callers that cannot allocate device
memory inside their time loop (a fluid solver that has committed the device's
memory to its own arrays, or one whose other streams a cudaMalloc would stall);
it keeps its per-point weights in a static device array.  With every parcel at
rest (v = 0) the existing entry point stores the interpolated velocity itself
in vgap (ulp - 0 is ulp exactly), and both kernels issue the same operations in
the same order, so the two must agree bit for bit:

* at the parcels' positions, on two calls in a row (all locals in order, then
  in reverse order: a stale weight or window left by the first call would show
  in the second), for the sphere contact fixture (dx = 1) and the cylinder
  fixture (dx = 3.75e-5);
* at points within 1.5 cells of every face of the box, whose stencils read the
  halo layers, in a periodic box and in one with solid walls on z;
* right after an asynchronous fluid upload (the call waits for it).

The calls must leave the device's free memory unchanged, and sizes beyond the
array, or points outside the box, must be rejected with IBMDEM_ERANGE.
"""
import ctypes

import numpy as np
import pytest

import golden_util
from ibmdem import scenario

pytestmark = pytest.mark.gpu

MAX_POINTS = 16384  # IBMDEM_PROBE_MAX_POINTS in include/ibmdem.h
ERANGE = -4


def _case(gpu_lib, name):
    _, (p, parts, bodies, field) = golden_util.load(name)
    parts = parts.copy()
    parts["v"] = 0.0
    case = gpu_lib.Case(p, parts, bodies, field, device=0)
    case.InitializationDEM()
    return case


def _probe_dev(case, xd, out):
    return case.lib.ibmdem_interpolate_velocity_noalloc(case.h, xd.shape[0], ctypes.c_void_p(xd.data_ptr()),
                                                        ctypes.c_void_p(out.data_ptr()))


def _probe(case, x):
    import torch
    xd = torch.from_numpy(np.ascontiguousarray(x)).to("cuda:0")
    out = torch.full(x.shape, float("nan"), dtype=torch.float64, device="cuda:0")
    torch.cuda.synchronize()
    rc = _probe_dev(case, xd, out)
    return rc, out.cpu().numpy()


def _reference(case):
    """vgap of the existing entry point with every parcel at rest."""
    case.UpdateFluidVelocityOnLagrangianPoints()
    pp, nl = case.get_parcels()
    assert np.all(pp["v"][:nl] == 0.0)
    return pp["x"][:nl].copy(), pp["vgap"][:nl].copy()


@pytest.mark.parametrize("name", golden_util.NAMES)
def test_noalloc_matches_existing_interpolation(gpu_lib, name):
    case = _case(gpu_lib, name)
    x, ref = _reference(case)
    nl = len(x)
    assert 0 < nl <= MAX_POINTS
    for order in (np.arange(nl), np.arange(nl)[::-1]):
        rc, got = _probe(case, x[order])
        assert rc == 0, case.lib.ibmdem_last_error(case.h).decode()
        assert np.array_equal(got, ref[order])
    case.close()


def _face_points(p, rng):
    """Points within 1.5 cells of each of the six faces (and on the low face)."""
    L = np.array([float(p["nx"]) * float(p["dx"]), float(p["ny"]) * float(p["dy"]), float(p["nz"]) * float(p["dz"])])
    h = float(p["dx"])
    out = []
    for d in range(3):
        for off in (0.0, 0.02, 0.5, 0.97, 1.25, 1.49):
            for face in (0, 1):
                q = rng.uniform(0.0, 1.0, (4, 3)) * L
                q[:, d] = off * h if face == 0 else L[d] - (off + 0.01) * h
                out.append(q)
    # the corners and edges, where images of images exist
    c = rng.uniform(0.0, 1.4, (64, 3)) * h
    flip = rng.random((64, 3)) < 0.5
    c = np.where(flip, L - 0.01 * h - c, c)
    out.append(c)
    return np.concatenate(out)


@pytest.mark.parametrize("walls", ["", "z"])
def test_noalloc_at_points_next_to_every_face(gpu_lib, walls):
    if walls:
        p, parts, bodies, field = scenario.walled_case(24, 20, 28, 2, 8.0, seed=4, walls=walls, n_modes=6,
                                                       touching=0)
    else:
        p, parts, bodies, field = scenario.resolved_case(24, 20, 28, 2, 8.0, seed=4, n_modes=6)
    x = _face_points(p, np.random.default_rng(9))
    # parcels of body 1 at the probe points, at rest
    pts = np.repeat(parts[:1], len(x))
    pts["x"] = x
    pts["v"] = 0.0
    pts["globalIdx"] = np.arange(1, len(x) + 1)
    pts["MSIdx"] = 1
    case = gpu_lib.Case(p, pts, bodies, field, device=0)
    case.InitializationDEM()
    xs, ref = _reference(case)
    assert np.array_equal(xs, x)
    for order in (np.arange(len(x)), np.arange(len(x))[::-1]):
        rc, got = _probe(case, x[order])
        assert rc == 0, case.lib.ibmdem_last_error(case.h).decode()
        assert np.array_equal(got, ref[order])
    case.close()


def test_noalloc_waits_for_async_upload(gpu_lib):
    import torch

    case = _case(gpu_lib, "sphere_contact")
    x, _ = _reference(case)
    u, v, w = case.get_fluid()[:3]
    # new fields: the old ones scaled, in pinned host memory
    new = []
    for f, s in zip((u, v, w), (3.0, -2.0, 5.0)):
        t = torch.empty(f.shape, dtype=torch.float64, pin_memory=True).numpy()
        t[...] = f * s
        new.append(t)
    case.set_fluid(*new)
    rc, want = _probe(case, x)
    assert rc == 0
    case.set_fluid(u, v, w)
    xd = torch.from_numpy(x).to("cuda:0")
    out = torch.full(x.shape, float("nan"), dtype=torch.float64, device="cuda:0")
    torch.cuda.synchronize()
    for _ in range(3):
        rc = case.lib.ibmdem_set_fluid_async(case.h, *[a.ctypes.data for a in new])
        assert rc == 0
        rc = _probe_dev(case, xd, out)  # at once: the call must wait for the upload
        assert rc == 0, case.lib.ibmdem_last_error(case.h).decode()
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy(), want)
        case.set_fluid(u, v, w)
    case.close()


def test_noalloc_allocates_nothing(gpu_lib):
    import torch

    case = _case(gpu_lib, "sphere_contact")
    x, ref = _reference(case)
    xd = torch.from_numpy(x).to("cuda:0")
    out = torch.full(x.shape, float("nan"), dtype=torch.float64, device="cuda:0")
    torch.cuda.synchronize()
    assert _probe_dev(case, xd, out) == 0  # the first call looks the array up
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info(0)
    for _ in range(5):
        assert _probe_dev(case, xd, out) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info(0)
    assert free1 == free0, (free0, free1)
    assert np.array_equal(out.cpu().numpy(), ref)
    case.close()


def test_noalloc_rejects_oversize_and_outside_points(gpu_lib):
    case = _case(gpu_lib, "sphere_contact")
    pp, nl = case.get_parcels()
    x = np.repeat(pp["x"][:1], MAX_POINTS + 1, axis=0)
    rc, _ = _probe(case, x)
    assert rc == ERANGE
    assert "static array" in case.lib.ibmdem_last_error(case.h).decode()
    x = pp["x"][:8].copy()
    x[5, 1] = -0.25
    rc, got = _probe(case, x)
    assert rc == ERANGE
    msg = case.lib.ibmdem_last_error(case.h).decode()
    assert "point 5" in msg and "outside the box" in msg
    assert np.isnan(got[5]).all() and np.isfinite(got[:5]).all()
    case.close()
