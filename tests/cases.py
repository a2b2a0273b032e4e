"""Seeded cases shared by the parity tests and the smoke check."""
import numpy as np

from ibmdem import scenario


def contact_case(n=24, nb=4, d=8.0, seed=3, gap=0.4, n_modes=6, straddle=True, vel_std=0.01, **kw):
    """Periodic spheres where body 2 touches body 1 (centre distance d + gap)
    and, optionally, body 1 straddles the x = 0 face."""
    p, parts, bodies, field = scenario.resolved_case(n, n, n, nb, d, seed=seed, n_modes=n_modes, vel_std=vel_std,
                                                     **kw)
    L = np.array([n, n, n], dtype=float)
    X = bodies["x"].copy()
    if straddle:
        X[0] = np.array([0.7, 0.45 * n, 0.55 * n])
    X[1] = X[0] + np.array([d + gap, 0.3, -0.2])
    X = X % L
    # keep the other bodies clear of the first two
    for b in range(2, nb):
        for _ in range(1000):
            dv = X[:b] - X[b]
            dv -= L * np.round(dv / L)
            if np.min(np.einsum("ij,ij->i", dv, dv)) > (d + 0.5) ** 2:
                break
            X[b] = np.random.default_rng(seed + b).random(3) * L
    parts, bodies2 = scenario.sphere_bodies(X, d, 1.0, 1.14e3, bodies["v"])
    parts["x"] = scenario.wrap_coord(parts["x"], L)
    return p, parts, bodies2, field


def compare_parcels(a, b, nl, exact=True, fields_local=("x", "v", "fcol", "fdrag", "vgap", "vol", "m", "radeff"),
                    fields_img=("x", "v", "fdrag")):
    """Assert two parcel record arrays agree: locals on `fields_local`, images on
    `fields_img` (image vgap/wdrag are unspecified slot contents in the reference)."""
    assert len(a) == len(b), (len(a), len(b))
    for f in ("MSIdx", "globalIdx", "cellIdx"):
        assert np.array_equal(a[f], b[f]), f
    for f in fields_local:
        if exact:
            assert np.array_equal(a[f][:nl], b[f][:nl]), f"local {f}: max diff {np.abs(a[f][:nl] - b[f][:nl]).max()}"
        else:
            assert np.allclose(a[f][:nl], b[f][:nl], rtol=1e-9, atol=1e-13), f
    for f in fields_img:
        if exact:
            assert np.array_equal(a[f][nl:], b[f][nl:]), f"image {f}"
        else:
            assert np.allclose(a[f][nl:], b[f][nl:], rtol=1e-9, atol=1e-13), f


def rel_close(a, b, rtol=1e-9):
    """max |a-b| <= rtol * max(|b|) per field (the trajectory tolerance, 1e-9 by default)."""
    a = np.asarray(a, dtype=float)
    b = np.asarray(b, dtype=float)
    scale = max(np.abs(b).max(), 1e-300)
    return np.abs(a - b).max() <= rtol * scale
