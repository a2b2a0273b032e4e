"""The CUDA unresolved CFD-DEM path against the CPU restatement.

A 32^3 case whose packed bed starts in contact (bed spacing 0.95 of the
largest diameter), so the contact lists, friction and history are exercised.
After one step: contact lists (partners) bit for bit, contact forces and
torques bit for bit (no library math on that path), tangential displacements,
the volume-fraction field, drag and the new state within 1e-12 relative (exp,
pow and log10 come from different math libraries); after five steps the
trajectories within 1e-9 relative.
"""
import numpy as np
import pytest

import cases
from ibmdem import api, scenario

pytestmark = pytest.mark.gpu


def make(seed=2):
    return scenario.unresolved_case(32, 20000, seed=seed, n_modes=8, bed_spacing=0.95)


def test_unresolved_step_matches_oracle(gpu_lib, oracle_mod):
    p, parts, field = make()
    g = api.Unresolved(p, parts, field)
    r = oracle_mod.OracleUnresolved(p, parts, field)
    g.step(1)
    r.step(1)
    gs, gp, gx = g.get_contacts()
    rs, rp, rx = r.get_contacts()
    assert len(rp) > 1000
    assert np.array_equal(gs, rs) and np.array_equal(gp, rp)
    assert cases.rel_close(gx, rx, 1e-12)
    a, b = g.get_particles(), r.get_particles()
    for f in ("fcol", "tcol"):
        assert np.array_equal(a[f], b[f]), f
    assert cases.rel_close(g.get_volume_fraction(), r.get_volume_fraction(), 1e-12)
    for f in ("fdrag", "alphaf", "x", "v", "omega"):
        assert cases.rel_close(a[f], b[f], 1e-12), f
    g.step(4)
    r.step(4)
    a, b = g.get_particles(), r.get_particles()
    for f in ("x", "v", "omega", "fcol", "fdrag"):
        assert cases.rel_close(a[f], b[f], 1e-9), f
    g.close()
    r.close()


def test_drag_law_batch_matches_oracle(gpu_lib, oracle_mod):
    import ctypes

    import torch

    rng = np.random.default_rng(5)
    n = 4096
    rho = np.full(n, 2500.0)
    rad = rng.uniform(0.1e-3, 0.2e-3, n)
    v = rng.standard_normal((n, 3)) * 0.1
    velf = rng.standard_normal((n, 3)) * 0.5
    alpha = rng.uniform(0.35, 1.0, n)
    dev = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in (rho, rad, v, alpha, velf)]
    beta = torch.zeros((n, 3), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rc = gpu_lib.load().ibmdem_CalculateDragForce(n, *[ctypes.c_void_p(t.data_ptr()) for t in dev[:3]], 1.2,
                                                  ctypes.c_void_p(dev[3].data_ptr()),
                                                  ctypes.c_void_p(dev[4].data_ptr()),
                                                  ctypes.c_void_p(beta.data_ptr()), None)
    assert rc == 0
    torch.cuda.synchronize()
    got = beta.cpu().numpy()
    ref = np.stack([oracle_mod.drag_beta(2500.0, rad[i], v[i], 1.2, alpha[i], velf[i]) for i in range(n)])
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
