"""Fast bodies against the CPU restatement: markers cross cells, half cells and
the periodic faces every step, so the lists, images, spread plan and migration
(a marker whose periodic image becomes the local) change all the time.  The
fields and parcels must equal the restatement's bit for bit, and the bodies
within 1e-9."""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu


def run(gpu_lib, oracle_mod, case, steps):
    p, parts, bodies, field = case
    g = gpu_lib.Case(p, parts, bodies, field, device=0)
    r = oracle_mod.OracleCase(p, parts, bodies, field)
    for c in (g, r):
        c.InitializationDEM()
    for s in range(steps):
        g.step(1)
        r.step(1)
        for a, b in zip(g.get_fluid(), r.get_fluid()):
            assert np.array_equal(a, b), s
        gp, nl = g.get_parcels()
        rp, _ = r.get_parcels()
        cases.compare_parcels(gp, rp, nl)
        gb, rb = g.get_bodies(), r.get_bodies()
        for f in ("x", "v", "omega"):
            assert cases.rel_close(gb[f], rb[f], 1e-9), (s, f)
    g.close()


def test_fast_bodies_and_migration(gpu_lib, oracle_mod):
    p, parts, bodies, field = cases.contact_case(seed=22, vel_std=0.0, n_modes=4, gap=3.0, straddle=True)
    # bodies moving 0.2 cells per step
    rng = np.random.default_rng(5)
    v = rng.standard_normal((len(bodies), 3))
    v *= 200.0 / np.linalg.norm(v, axis=1, keepdims=True)
    bodies["v"] = v
    parts["v"] = v[parts["MSIdx"] - 1]
    run(gpu_lib, oracle_mod, (p, parts, bodies, field), 6)
