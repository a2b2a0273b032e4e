"""Host-side logic: synthetic case generation and the multi-rank timing
reduction of bench.py (replicas only: ranks never exchange case data)."""
import os
import socket

import numpy as np
import pytest

from ibmdem import scenario
from ibmdem.records import field_shape, make_params


def test_rsa_respects_minimum_image_distance():
    rng = np.random.default_rng(0)
    L = np.array([64.0, 64.0, 128.0])
    c = scenario.rsa_centres(L, 60, 12.0, rng)
    d = c[:, None, :] - c[None, :, :]
    d -= L * np.round(d / L)
    dist = np.sqrt((d ** 2).sum(-1)) + np.eye(len(c)) * 1e9
    assert dist.min() > 12.0


def test_sphere_records():
    parts, bodies = scenario.sphere_bodies(np.array([[10.0, 10.0, 10.0]]), 12.0, 1.0, 1140.0, np.zeros((1, 3)))
    assert len(parts) == round(np.pi * 144)
    r = np.linalg.norm(parts["x"] - 10.0, axis=1)
    assert np.allclose(r, 6.0 - 0.3)
    assert bodies["rad"][0] == pytest.approx(6.0)
    assert np.allclose(bodies["InertiaTensor"][0].reshape(3, 3), np.eye(3) * bodies["I"][0])


def test_fourier_field_halo_is_periodic_and_field_is_solenoidal_in_the_mean():
    p = make_params(16, 16, 24)
    u, v, w = scenario.fourier_field(p, 8, 0.05, seed=1)
    assert u.shape == field_shape(p)
    for f in (u, v, w):
        assert np.array_equal(f[:, :, 0:2], f[:, :, 16:18])
        assert np.array_equal(f[:, 0:2, :], f[:, 16:18, :])
        assert np.array_equal(f[0:2], f[24:26])
    # discrete divergence on the MAC grid is small compared with the gradients
    s = (slice(2, -3),) * 3
    div = (u[2:-3, 2:-3, 3:-2] - u[s]) + (v[2:-3, 3:-2, 2:-3] - v[s]) + (w[3:-2, 2:-3, 2:-3] - w[s])
    assert np.abs(div).max() < 0.1 * np.abs(u).max()


def test_wrap_coord_is_one_add():
    L = np.array([16.0, 16.0, 16.0])
    x = np.array([[-0.3, 16.2, 5.0]])
    y = scenario.wrap_coord(x, L)
    assert y[0, 0] == -0.3 + 16.0 and y[0, 1] == 16.2 + (-16.0) and y[0, 2] == 5.0


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    q.put((rank, bench.max_over_ranks(1.5 + rank)))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_gloo_two_ranks():
    import torch.multiprocessing as mp

    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    out = dict(q.get(timeout=120) for _ in procs)
    for pr in procs:
        pr.join(timeout=60)
        assert pr.exitcode == 0
    assert out == {0: 2.5, 1: 2.5}


def test_case_bytes_estimate():
    """ibmdem_case_bytes is host arithmetic over the same buffer list the
    context allocates: it grows with the grid and the parcels, counts the
    periodic images, and rejects what ibmdem_create rejects."""
    from ibmdem import api
    p, parts, bodies, _ = scenario.resolved_case(32, 32, 32, 4, 8.0, seed=2, n_modes=0)
    b0 = api.case_bytes(p, parts[:0], 0)
    b1 = api.case_bytes(p, parts, len(bodies))
    assert b1 > b0 > 9 * 36 ** 3 * 8
    p2 = make_params(48, 48, 48)
    assert api.case_bytes(p2, parts, len(bodies)) - b1 >= 9 * 8 * (52 ** 3 - 36 ** 3)
    # the same parcels moved next to a face need image capacity
    edge = parts.copy()
    edge["x"][:, 0] = 0.25
    assert api.case_bytes(p, edge, len(bodies)) > b1
    bad = p.copy()
    bad["bType"][0] = 1
    with pytest.raises(api.IbmDemError):
        api.case_bytes(bad, parts, len(bodies))
