"""GPU parity against the CPU restatement at the benchmark configurations' sizes.

The other parity tests use small cases; these run the workloads the library is
measured on, so that the code paths only large cases reach are compared too:

* 128^3, 64 spheres of d = 16h (51,456 markers), 100 frozen-fluid steps.
  Every step is checked twice:
  - lockstep: a restatement case is loaded with the GPU's parcels and bodies
    before the step (InitializationDEM rebuilds its lists), so both sides step
    from identical input.  The lists the restatement rebuilds must equal the
    GPU's bit for bit, and after the step the spread forcing, the post-guess
    velocity field, fdrag and vgap must be bit-identical; the body state within
    1e-9 relative (CUDA's cos/sin replace glibc's in the Rodrigues rotation).
  - free-running: a second restatement case advances on its own from the same
    start.  Bodies and parcels must stay within 1e-9 relative over all 100
    steps; a contact or cell list may differ only by pairs whose distance sits
    within that tolerance of the cut-off (|dist^2 - cut^2| is reported).
* 256x256x512, 2,048 spheres of d = 12h (925,696 markers), 2 steps, the same
  two checks (the benchmark's own case).
* 1,048,576 unresolved particles on 128^3, 2 steps: contact lists and contact
  forces bit for bit after the first step, volume fraction, drag and state
  within 1e-12; after the second step lists exact (or flips at the cut-off)
  and state within 1e-9.
* 16 cases of the 256-case batched mix (grids up to 128^3, up to 512 bodies):
  each member of a batch bit-identical to the case run alone, with each
  member's own forcing launches and with shared ones, and each case's first
  step against the restatement as above.
* 128^3 between solid walls in z, 64 spheres of d = 16h with 4 against the low
  wall, 20 steps, the same two checks.
"""
import numpy as np
import pytest

import cases
from ibmdem import api, scenario

pytestmark = pytest.mark.gpu

LIST_TOL = 1e-9  # the trajectory tolerance; a list flip must sit this close to the cut-off


def _cut2(p):
    cd = float(p["collisionDist"]) * (1.0 + float(p["collisionBuffer"]))
    return cd * cd


def _pairs(starts, idx):
    n = len(starts) - 1
    owner = np.repeat(np.arange(n), np.diff(starts))
    return set(zip(owner.tolist(), (idx - 1).tolist()))


def _list_margin(g_parts, p, gs, gi, rs, ri):
    """Largest relative |dist^2 - cut^2| over pairs present in only one of two
    contact lists (0 when the lists are equal), from the GPU's positions."""
    if np.array_equal(gs, rs) and np.array_equal(gi, ri):
        return 0.0
    cut2 = _cut2(p)
    worst = 0.0
    for i, j in _pairs(gs, gi) ^ _pairs(rs, ri):
        d = g_parts["x"][i] - g_parts["x"][j]
        worst = max(worst, abs(float(d @ d) - cut2) / cut2)
    return worst


def _lists(c):
    return c.get_cell_lists(), c.get_collision_lists()


def _assert_lists_equal(a, b, what):
    (acs, aci), (aps, api_) = a
    (bcs, bci), (bps, bpi) = b
    assert np.array_equal(acs, bcs), f"{what}: cell starts differ"
    assert np.array_equal(aci, bci), f"{what}: cell items differ"
    assert np.array_equal(aps, bps), f"{what}: contact list starts differ"
    assert np.array_equal(api_, bpi), f"{what}: contact lists differ"


def _lock_from(gpu, lock):
    """Load the GPU's current locals and bodies into the restatement case."""
    gp, nl = gpu.get_parcels()
    lock.set_parcels(gp[:nl].copy())
    lock.set_bodies(gpu.get_bodies())
    lock.InitializationDEM()


def _step_pair(gpu, lock, free, p, s, stats):
    """One step of the GPU case, the lockstep restatement and the free-running
    one, with the checks described in the module docstring."""
    if s > 0:
        _lock_from(gpu, lock)
        _assert_lists_equal(_lists(gpu), _lists(lock), f"step {s}: rebuilt lists")
    gpu.step(1)
    lock.step(1)
    free.step(1)
    # identical input through the forcing loop: bit-identical
    for a, b in zip(gpu.get_fluid(), lock.get_fluid()):
        assert np.array_equal(a, b), f"step {s}: forcing or post-guess field differs"
    gp, gnl = gpu.get_parcels()
    lp, lnl = lock.get_parcels()
    gb, lb = gpu.get_bodies(), lock.get_bodies()
    exact = all(np.array_equal(gb[f], lb[f]) for f in ("x", "v", "omega", "rotMatGlo", "AngMom"))
    stats["exact_steps"] += int(exact)
    for f in ("fdrag", "fcol", "fmom", "fmomCol", "fhydro", "fmomHydro"):
        assert np.array_equal(gb[f], lb[f]), f"step {s}: body sum {f} differs"
    for f in ("x", "v", "omega", "AngMom", "rotMatGlo"):
        assert cases.rel_close(gb[f], lb[f], 1e-9), f"step {s}: body {f}"
    assert gnl == lnl
    if exact:
        # the same bodies move the same markers: everything downstream is exact
        cases.compare_parcels(gp, lp, gnl)
        _assert_lists_equal(_lists(gpu), _lists(lock), f"step {s}: lists after the step")
    else:
        for f in ("fdrag", "vgap"):
            assert np.array_equal(gp[f][:gnl], lp[f][:gnl]), f"step {s}: {f}"
        cases.compare_parcels(gp, lp, gnl, exact=False, fields_img=("x", "v"))
    # free-running trajectory
    fb = free.get_bodies()
    for f in ("x", "v", "omega"):
        assert cases.rel_close(gb[f], fb[f], 1e-9), f"step {s}: free-running body {f}"
    (gs, gi), (fs, fi) = gpu.get_collision_lists(), free.get_collision_lists()
    m = _list_margin(gp, p, gs, gi, fs, fi)
    stats["max_flip_margin"] = max(stats["max_flip_margin"], m)
    stats["flip_steps"] += int(m > 0)
    assert m <= LIST_TOL, f"step {s}: a contact pair differs {m:.3e} (relative) away from the cut-off"


def _run_resolved(gpu_lib, oracle_mod, case, steps):
    p, parts, bodies, field = case
    gpu = gpu_lib.Case(p, parts, bodies, field, device=0)
    lock = oracle_mod.OracleCase(p, parts, bodies, field)
    free = oracle_mod.OracleCase(p, parts, bodies, field)
    for c in (gpu, lock, free):
        c.InitializationDEM()
    _assert_lists_equal(_lists(gpu), _lists(lock), "initial lists")
    gp, gnl = gpu.get_parcels()
    lp, _ = lock.get_parcels()
    assert len(gp) > gnl, "periodic images expected"
    cases.compare_parcels(gp, lp, gnl, fields_local=("x", "v", "vol", "m", "radeff"))
    stats = {"exact_steps": 0, "flip_steps": 0, "max_flip_margin": 0.0, "pairs": 0}
    for s in range(steps):
        _step_pair(gpu, lock, free, p, s, stats)
        stats["pairs"] = max(stats["pairs"], len(gpu.get_collision_lists()[1]))
    gpu.close()
    lock.close()
    free.close()
    print(stats)
    return stats


def test_config_128cube_64_spheres_100_steps(gpu_lib, oracle_mod):
    case = scenario.resolved_case(128, 128, 128, 64, 16.0, seed=0, n_modes=32, amp=0.05, vel_std=0.01,
                                  field_device="cuda")
    assert len(case[1]) == 51456
    stats = _run_resolved(gpu_lib, oracle_mod, case, 100)
    assert stats["pairs"] > 0, "the case must make contacts"


def test_config_256x256x512_2048_spheres(gpu_lib, oracle_mod):
    case = scenario.resolved_case(256, 256, 512, 2048, 12.0, seed=0, n_modes=64, amp=0.05, vel_std=0.01,
                                  field_device="cuda")
    assert len(case[1]) == 925696
    stats = _run_resolved(gpu_lib, oracle_mod, case, 2)
    assert stats["pairs"] > 0


def test_config_unresolved_1048576_particles(gpu_lib, oracle_mod):
    p, parts, field = scenario.unresolved_case(128, 1_048_576, seed=0, n_modes=32, field_device="cuda",
                                               bed_spacing=0.9)
    g = api.Unresolved(p, parts, field)
    r = oracle_mod.OracleUnresolved(p, parts, field)
    g.step(1)
    r.step(1)
    gs, gp, gx = g.get_contacts()
    rs, rp, rx = r.get_contacts()
    assert len(rp) > 100000
    assert np.array_equal(gs, rs) and np.array_equal(gp, rp)
    assert cases.rel_close(gx, rx, 1e-12)
    a, b = g.get_particles(), r.get_particles()
    for f in ("fcol", "tcol"):
        assert np.array_equal(a[f], b[f]), f
    assert cases.rel_close(g.get_volume_fraction(), r.get_volume_fraction(), 1e-12)
    for f in ("fdrag", "alphaf", "x", "v", "omega"):
        assert cases.rel_close(a[f], b[f], 1e-12), f
    g.step(1)
    r.step(1)
    a, b = g.get_particles(), r.get_particles()
    for f in ("x", "v", "omega", "fdrag"):
        assert cases.rel_close(a[f], b[f], 1e-9), f
    gs, gp, _ = g.get_contacts()
    rs, rp, _ = r.get_contacts()
    if not (np.array_equal(gs, rs) and np.array_equal(gp, rp)):
        # a pair may only flip where its distance sits at the contact distance
        L = float(p["nx"]) * float(p["dx"])
        worst = 0.0
        for i, j in _pairs(gs, gp + 1) ^ _pairs(rs, rp + 1):
            dv = a["x"][i] - a["x"][j]
            dv -= L * np.round(dv / L)
            rr = a["rad"][i] + a["rad"][j]
            worst = max(worst, abs(float(np.sqrt(dv @ dv)) - rr) / rr)
        assert worst <= LIST_TOL, worst
    g.close()
    r.close()


def test_config_batched_mix_16_cases(gpu_lib, oracle_mod):
    mix = scenario.batched_mix(16, seed=0, n_modes=32, field_device="cuda")
    assert max(int(c[0]["nx"]) for c in mix) == 128
    members, ref = [], []
    for p, parts, bodies, field in mix:
        alone = api.Case(p, parts, bodies, field, device=0)
        lock = oracle_mod.OracleCase(p, parts, bodies, field)
        for c in (alone, lock):
            c.InitializationDEM()
            c.step(1)
        for a, b in zip(alone.get_fluid(), lock.get_fluid()):
            assert np.array_equal(a, b)
        gb, lb = alone.get_bodies(), lock.get_bodies()
        for f in ("x", "v", "omega"):
            assert cases.rel_close(gb[f], lb[f], 1e-9), f
        gp, nl = alone.get_parcels()
        lp, _ = lock.get_parcels()
        for f in ("fdrag", "vgap"):
            assert np.array_equal(gp[f][:nl], lp[f][:nl]), f
        lock.close()
        alone.step(1)
        ref.append((alone.get_parcels(), alone.get_bodies(), alone.get_fluid()))
        alone.close()
        m = api.Case(p, parts, bodies, field, device=0)
        m.InitializationDEM()
        members.append(m)
    # the batch with each member's own forcing launches, then with shared ones
    for fused in (False, True):
        if fused:
            members = []
            for p, parts, bodies, field in mix:
                m = api.Case(p, parts, bodies, field, device=0)
                m.InitializationDEM()
                members.append(m)
        b = api.Batch(members)
        b.set_fused(fused)
        b.step(2)
        b.synchronize()
        for m, ((rp, rnl), rb, rf) in zip(members, ref):
            gp, gnl = m.get_parcels()
            assert gnl == rnl and len(gp) == len(rp)
            for f in ("x", "v", "fcol", "fdrag", "vgap", "globalIdx", "MSIdx", "cellIdx"):
                assert np.array_equal(gp[f], rp[f]), (fused, f)
            gb = m.get_bodies()
            for f in ("x", "v", "omega", "AngMom", "rotMatGlo", "fcol", "fdrag", "fmom", "fmomCol"):
                assert np.array_equal(gb[f], rb[f]), (fused, f)
            for x, y in zip(m.get_fluid(), rf):
                assert np.array_equal(x, y)
        b.close()
        for m in members:
            m.close()


def test_config_128cube_walled_64_spheres_20_steps(gpu_lib, oracle_mod):
    """The 128^3 case between solid walls in z (x and y periodic), 4 of the 64
    spheres resting against the low wall: wall contacts, mirror images across
    the wall and the wall halo rules at the benchmark's grid size, lockstep and
    free-running as above."""
    case = scenario.walled_case(128, 128, 128, 64, 16.0, seed=1, walls="z", n_modes=32, touching=4)
    stats = _run_resolved(gpu_lib, oracle_mod, case, 20)
    assert stats["pairs"] > 0
