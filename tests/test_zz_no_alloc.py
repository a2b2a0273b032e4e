"""ibmdem_interpolate_velocity_noalloc against ibmdem_UpdateFluidVelocityOnLagrangianPoints.

The allocation-free entry point keeps its weights in a static device array.
With every parcel at rest (v = 0) the existing entry point stores the
interpolated velocity itself in vgap (ulp - 0), so both must agree at the
parcels' positions to the suite's per-value tolerance (1e-12 relative), on two
calls in a row: all locals in order, then in reverse order (a stale weight or
window left by the first call would show in the second).  Cases: the sphere
contact fixture (dx = 1) and the cylinder fixture (dx = 3.75e-5).
"""
import ctypes

import numpy as np
import pytest

import cases
import golden_util

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


def _probe(case, x):
    import torch
    xd = torch.from_numpy(np.ascontiguousarray(x)).to("cuda:0")
    out = torch.full(x.shape, float("nan"), dtype=torch.float64, device="cuda:0")
    torch.cuda.synchronize()
    rc = case.lib.ibmdem_interpolate_velocity_noalloc(case.h, len(x), ctypes.c_void_p(xd.data_ptr()),
                                                      ctypes.c_void_p(out.data_ptr()))
    return rc, out.cpu().numpy()


@pytest.mark.parametrize("name", golden_util.NAMES)
def test_noalloc_matches_existing_interpolation(gpu_lib, name):
    case = _case(gpu_lib, name)
    case.UpdateFluidVelocityOnLagrangianPoints()
    pp, nl = case.get_parcels()
    assert np.all(pp["v"][:nl] == 0.0)
    ref = pp["vgap"][:nl].copy()
    x = pp["x"][:nl].copy()
    assert 0 < nl <= MAX_POINTS
    for order in (np.arange(nl), np.arange(nl)[::-1]):
        rc, got = _probe(case, x[order])
        assert rc == 0, case.lib.ibmdem_last_error(case.h).decode()
        assert cases.rel_close(got, ref[order], 1e-12)
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
    assert "point 5" in case.lib.ibmdem_last_error(case.h).decode()
    assert np.isnan(got[5]).all() and np.isfinite(got[:5]).all()
    case.close()
