"""A numpy solve of the reference's pressure-correction system, independent
of the GPU code, for the Poisson tests: the rows of the 7-point Laplacian
(periodic, or Neumann behind the walls of `walls`), with the row of interior
node (1,1,1) replaced by p = 0 (poisson.F90:50-131).

Every other row reads (L p)_c = b_c with L singular and its rows summing to
zero, so the pinned row's value is -sum_{c != 0} b_c; the walled axes are
extended evenly to twice their length, the consistent periodic system is
solved with numpy's FFT, and the solution is shifted to p = 0 at the pin."""
import numpy as np


def solve(b, h, walls=""):
    """b: interior right-hand side, numpy axes (z, y, x); h: (dx, dy, dz)."""
    bt = np.array(b, dtype=np.float64, copy=True)
    bt[0, 0, 0] = -(bt.sum() - bt[0, 0, 0])
    lam = 0.0
    for ax, name in enumerate("zyx"):
        if name in walls:
            bt = np.concatenate([bt, np.flip(bt, axis=ax)], axis=ax)
    for ax, name in enumerate("zyx"):
        n = bt.shape[ax]
        dl = h[2 - ax]
        l1 = 4.0 * np.sin(np.pi * np.arange(n) / n) ** 2 / (dl * dl)
        shape = [1, 1, 1]
        shape[ax] = n
        lam = lam + l1.reshape(shape)
    spec = np.fft.fftn(bt)
    with np.errstate(divide="ignore", invalid="ignore"):
        spec = np.where(lam > 0, spec / lam, 0.0)
    q = np.fft.ifftn(spec).real[: b.shape[0], : b.shape[1], : b.shape[2]]
    return q - q[0, 0, 0]
