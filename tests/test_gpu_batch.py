"""Many cases on one device: batch (one graph launch per step) and request server.

Each case must give the same parcels, bodies and fields in a batch, or through
the server while other requests overlap it, as when it runs alone.  The
kernels of a case are the same in all three paths and none of them sums across
cases, so the comparison is exact.
"""
import numpy as np
import pytest

import cases
from ibmdem import api, scenario

pytestmark = pytest.mark.gpu

PARCEL_FIELDS = ("x", "v", "fcol", "fdrag", "vgap", "globalIdx", "MSIdx", "cellIdx")
BODY_FIELDS = ("x", "v", "omega", "AngMom", "rotMatGlo", "fcol", "fdrag", "fmom", "fmomCol")


def mixed_cases():
    out = [cases.contact_case(seed=3)]
    out.append(scenario.resolved_case(32, 32, 32, 6, 8.0, seed=5, n_modes=8))
    out.append(scenario.resolved_case(40, 32, 24, 3, 10.0, seed=6, n_modes=8))
    p, parts, bodies, _ = scenario.resolved_case(28, 28, 28, 4, 8.0, seed=7, n_modes=0)
    out.append((p, parts, bodies, None))  # a fluid at rest
    return out


def make_case(c):
    p, parts, bodies, field = c
    if field is None:
        shape = api.field_shape(np.array(p, dtype=api.PARAMS))
        field = [np.zeros(shape) for _ in range(3)]
    case = api.Case(p, parts, bodies, field, device=0)
    case.InitializationDEM()
    return case


def snapshot(case):
    parts, nl = case.get_parcels()
    bodies = case.get_bodies()
    u, v, w, fx, fy, fz = case.get_fluid()
    return parts, nl, bodies, (u, v, w, fx, fy, fz)


def assert_same(a, b, fields=True):
    pa, nla, ba, fa = a
    pb, nlb, bb, fb = b
    assert nla == nlb and len(pa) == len(pb)
    for f in PARCEL_FIELDS:
        assert np.array_equal(pa[f], pb[f]), f
    for f in BODY_FIELDS:
        assert np.array_equal(ba[f], bb[f]), f
    if fields:
        for x, y in zip(fa, fb):
            assert np.array_equal(x, y)


def alone(c, steps):
    case = make_case(c)
    case.step(steps)
    out = snapshot(case)
    case.close()
    return out


@pytest.mark.parametrize("lanes", [0, 1, 2])
def test_batch_matches_each_case_alone(gpu_lib, lanes):
    cs = mixed_cases()
    steps = 3
    ref = [alone(c, steps) for c in cs]
    members = [make_case(c) for c in cs]
    b = api.Batch(members, lanes=lanes)
    b.step(1)
    b.step(steps - 1)
    b.synchronize()
    for case, r in zip(members, ref):
        assert_same(snapshot(case), r)
    b.close()
    for case in members:
        case.close()


@pytest.mark.parametrize("lanes,interp_block", [(0, 256), (2, 128), (1, 256)])
def test_batch_shared_forcing_launches_match_alone(gpu_lib, lanes, interp_block):
    """The forcing loops of all members in shared launches (one interpolation and
    one spread per iteration for the whole batch): each member exactly as alone,
    periodic and walled members mixed."""
    cs = mixed_cases()
    cs.append(scenario.walled_case(24, 20, 28, 2, 8.0, seed=4, walls="z", n_modes=6, touching=0))
    assert len({int(c[0]["Ns"]) for c in cs}) == 1
    steps = 3
    ref = [alone(c, steps) for c in cs]
    members = [make_case(c) for c in cs]
    b = api.Batch(members, lanes=lanes)
    b.set_fused(True, interp_block)
    assert b.config()[1:] == (1, interp_block)
    b.step(1)
    b.step(steps - 1)
    b.synchronize()
    for case, r in zip(members, ref):
        assert_same(snapshot(case), r)
    # back to each member's own launches: still the same as alone
    b.set_fused(False)
    b.step(1)
    b.synchronize()
    for case, c in zip(members, cs):
        assert_same(snapshot(case), alone(c, steps + 1))
    b.close()
    for case in members:
        case.close()


def test_batch_shared_launches_nonunit_spacing_and_substeps(gpu_lib):
    """Shared forcing launches over members with physical units (the cylinder
    fixture, dx = 3.75e-5 m), three DEM sub-steps and periodic spheres: each
    member exactly as alone."""
    import golden_util

    _, cyl = golden_util.load("cylinders")
    cs = [cyl, cases.contact_case(seed=11, coupleInterval=3), mixed_cases()[1]]
    assert len({int(np.asarray(c[0])["Ns"]) for c in cs}) == 1
    steps = 2
    ref = [alone(c, steps) for c in cs]
    members = [make_case(c) for c in cs]
    b = api.Batch(members, lanes=2)
    b.set_fused(True, 128)
    b.step(steps)
    b.synchronize()
    for case, r in zip(members, ref):
        assert_same(snapshot(case), r)
    b.close()
    for case in members:
        case.close()


@pytest.mark.parametrize("fused", [False, True])
def test_batch_with_an_empty_member(gpu_lib, fused):
    """A member without parcels or bodies steps in a batch (with each member's
    own forcing launches and with shared ones) and leaves its fluid as it was;
    the other members are exactly as alone."""
    from ibmdem.records import MULTISPHERE, PARCEL, make_params

    p = make_params(16, 16, 16)
    z = [np.zeros((20, 20, 20)) for _ in range(3)]
    empty = (p, np.zeros(0, PARCEL), np.zeros(0, MULTISPHERE), z)
    cs = [mixed_cases()[1], empty, mixed_cases()[2]]
    steps = 2
    ref = [alone(c, steps) for c in cs]
    members = [make_case(c) for c in cs]
    b = api.Batch(members)
    b.set_fused(fused)
    b.step(steps)
    b.synchronize()
    for case, r in zip(members, ref):
        assert_same(snapshot(case), r)
    parts, nl = members[1].get_parcels()
    assert len(parts) == 0 and nl == 0
    b.close()
    for case in members:
        case.close()


def test_batch_shared_launches_fall_back_for_unequal_iterations(gpu_lib):
    """Members with different forcing iteration counts cannot share the
    launches: the batch keeps each member's own and the results stay exact."""
    cs = mixed_cases()[:2]
    p, parts, bodies, field = scenario.resolved_case(32, 32, 32, 5, 8.0, seed=9, n_modes=8, Ns=3)
    cs.append((p, parts, bodies, field))
    steps = 2
    ref = [alone(c, steps) for c in cs]
    members = [make_case(c) for c in cs]
    b = api.Batch(members)
    b.set_fused(True)
    b.step(steps)
    b.synchronize()
    for case, r in zip(members, ref):
        assert_same(snapshot(case), r)
    b.close()
    for case in members:
        case.close()


def test_batch_autotune_and_recapture(gpu_lib):
    cs = mixed_cases()[:3]
    members = [make_case(c) for c in cs]
    b = api.Batch(members)
    lanes = b.autotune(trial_steps=1)
    assert 1 <= lanes <= len(cs)
    assert b.config()[0] == lanes and b.config()[2] in (128, 256)
    # each trial: one warm-up + one trial step; every lane count with the
    # members' own launches, then the two best with shared launches and both
    # interpolation block sizes
    n_lanes = len({len(cs), 2, 1})
    n_auto = 2 * (n_lanes + 2 * min(2, n_lanes))
    b.step(2)
    b.synchronize()
    # a member changed outside the batch is re-captured: reload case 0 and rebuild it
    p, parts, bodies, field = cs[0]
    members[0].set_parcels(parts)
    members[0].set_bodies(bodies)
    members[0].set_fluid(*field)
    members[0].InitializationDEM()
    b.step(2)
    b.synchronize()
    assert_same(snapshot(members[0]), alone(cs[0], 2))
    for i in (1, 2):
        assert_same(snapshot(members[i]), alone(cs[i], n_auto + 4))
    b.close()
    for case in members:
        case.close()


@pytest.mark.parametrize("policy", ["arrival", "least_work"])
def test_server_admission_order(gpu_lib, policy):
    """One case at a time (max_active 1), requests submitted largest first:
    in arrival order they run in that order, under the least-work policy the
    smallest runs first; the results are exactly as alone either way."""
    cs = mixed_cases()
    steps = 2
    ref = [alone(c, steps) for c in cs]
    order = sorted(range(len(cs)), key=lambda i: -len(cs[i][1]))
    srv = api.Server(10 ** 11, max_active=1)
    if policy == "least_work":
        srv.set_policy(api.Server.LEAST_WORK)
    ids = {i: srv.submit(cs[i][0], cs[i][1], cs[i][2], cs[i][3], nsteps=steps, keep_parcels=True) for i in order}
    for _ in range(200000):
        if srv.poll() == 0:
            break
    queued = {i: srv.state(ids[i])[2] for i in order}
    run_order = sorted(order, key=lambda i: queued[i])
    expect = order if policy == "arrival" else sorted(order, key=lambda i: len(cs[i][1]))
    assert run_order == expect
    for i in order:
        parts, nl, bodies = srv.result(ids[i])
        assert_same((parts, nl, bodies, None), ref[i], fields=False)
        srv.release(ids[i])
    srv.close()


def test_server_results_match_alone_under_overlap(gpu_lib):
    cs = mixed_cases()
    steps = 4
    ref = [alone(c, steps) for c in cs]
    sizes = [api.case_bytes(c[0], c[1], len(c[2])) for c in cs]
    # room for the largest case and one more: the rest wait in the queue
    budget = max(sizes) + min(sizes)
    srv = api.Server(budget, max_active=8)
    ids = [srv.submit(c[0], c[1], c[2], c[3], nsteps=steps, keep_parcels=True) for c in cs]
    peak = 0
    for _ in range(200000):
        pending = srv.poll()
        used, _ = srv.memory()
        peak = max(peak, used)
        if pending == 0:
            break
    assert pending == 0
    assert 0 < peak <= budget
    lat = []
    for rid, r in zip(ids, ref):
        st, latency, queued = srv.state(rid)
        assert st == api.Server.DONE, st
        assert latency >= queued >= 0
        lat.append(latency)
        parts, nl, bodies = srv.result(rid)
        assert_same((parts, nl, bodies, None), r, fields=False)
        srv.release(rid)
    with pytest.raises(api.IbmDemError):
        big = scenario.resolved_case(64, 64, 64, 8, 12.0, seed=1, n_modes=0)
        srv.submit(big[0], big[1], big[2], None, nsteps=1)
    srv.close()
