"""Seeded synthetic cases for the resolved IBM-DEM path.

The reference builds its cases from marker template files (ZJS_INIT_DEM.F90:
350-494 for cylinders; :233-348 for spheres, whose template file is not in the
repository).  These generators produce the same records from formulas:

* spheres: a Fibonacci lattice of n = round(pi d^2) markers per sphere at radius
  radSphere = R - 0.3 dx, with the marker volume, mass and effective radius of
  the sphere initialiser (ZJS_INIT_DEM.F90:250, 311-314) and the body mass and
  moment of inertia of ZJS_INIT_DEM.F90:327-331;
* centres by random sequential addition (minimum-image distance > d);
* a periodic fluid field made of random Fourier modes with amplitude vectors
  perpendicular to their wave vectors, sampled on the MAC faces that the
  interpolation addresses (u at x=(i-1)h, y=(j-1/2)h, z=(k-1/2)h and the
  analogous v, w faces) with a periodic 2-cell halo.

Two choices differ from the reference initialiser because the reference only
starts bodies at rest and in one sub-domain: markers of a body that crosses a
periodic face are stored at their periodic image (x -/+ L), and bodies start
with vold = v and markers with v = V so that the first step sees no spurious
acceleration.  The sphere initialiser never fills InertiaTensor; the generator
sets it to diag(I, I, I), which EvolutionMS needs.
"""
import math

import numpy as np

from .records import MULTISPHERE, PARCEL, field_shape, make_params

PI32 = float(np.float32(3.1415926536))  # default-real literal of ZJS_INIT_DEM.F90:312


def fibonacci_sphere(n):
    i = np.arange(n, dtype=np.float64) + 0.5
    z = 1.0 - 2.0 * i / n
    r = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    phi = i * (math.pi * (3.0 - math.sqrt(5.0)))
    return np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=1)


def rsa_centres(L, nb, d, rng, max_tries=2_000_000):
    """Random sequential addition with minimum-image centre distance > d."""
    L = np.asarray(L, dtype=np.float64)
    out = np.empty((nb, 3))
    placed = 0
    tries = 0
    batch = 256
    while placed < nb:
        cand = rng.random((batch, 3)) * L
        for c in cand:
            tries += 1
            if tries > max_tries:
                raise RuntimeError(f"RSA could not place {nb} spheres of diameter {d}")
            if placed:
                dv = out[:placed] - c
                dv -= L * np.round(dv / L)
                if np.min(np.einsum("ij,ij->i", dv, dv)) <= d * d:
                    continue
            out[placed] = c
            placed += 1
            if placed == nb:
                break
    return out


def wrap_coord(x, L):
    """Periodic image of a coordinate as the reference forms it: one add of +/-L."""
    x = np.array(x, dtype=np.float64)
    for d in range(3):
        lo = x[..., d] < 0.0
        hi = x[..., d] >= L[d]
        x[..., d] = np.where(lo, x[..., d] + L[d], np.where(hi, x[..., d] + (-L[d]), x[..., d]))
    return x


def sphere_bodies(centres, d, h, rho_p, vel, n_markers=None):
    """Parcels and bodies for spheres of diameter d (in length units)."""
    nb = centres.shape[0]
    R = 0.5 * d
    rad_sphere = R - 0.3 * h
    n = int(round(math.pi * (d / h) ** 2)) if n_markers is None else int(n_markers)
    tpl = fibonacci_sphere(n)
    parts = np.zeros(nb * n, PARCEL)
    bodies = np.zeros(nb, MULTISPHERE)
    vol_p = PI32 * h / 3 / n * (12 * rad_sphere * rad_sphere + h * h)
    eye = np.eye(3).reshape(9)
    # body b's markers are parcels b*n .. b*n+n-1
    parts["x"] = ((rad_sphere * tpl)[None, :, :] + centres[:, None, :]).reshape(nb * n, 3)
    parts["v"] = np.repeat(np.asarray(vel, dtype=np.float64).reshape(nb, 3), n, axis=0)
    parts["MSIdx"] = np.repeat(np.arange(1, nb + 1), n)
    parts["globalIdx"] = np.tile(np.arange(1, n + 1), nb)
    parts["radeff"] = h * 0.75
    parts["rad"] = 0.0
    parts["rho"] = rho_p
    parts["vol"] = vol_p
    parts["m"] = rho_p * vol_p
    parts["pType"] = -1
    rad = rad_sphere + 0.3 * h
    vol = 4.0 / 3 * math.pi * (rad * rad * rad)
    m = vol * rho_p
    inertia = 0.4 * m * (rad * rad)
    bodies["globalIdx"] = np.arange(1, nb + 1)
    bodies["x"] = centres
    bodies["v"] = vel
    bodies["vold"] = vel
    bodies["rad"] = rad
    bodies["rho"] = rho_p
    bodies["vol"] = vol
    bodies["m"] = m
    bodies["I"] = inertia
    bodies["InertiaTensor"] = np.diag([inertia] * 3).reshape(9)
    bodies["rotMat"] = eye
    bodies["rotMatGlo"] = eye
    bodies["rotMatGloOld"] = eye
    return parts, bodies


def fourier_field(p, n_modes, amp, seed, kmax=4, device="cpu"):
    """u, v, w on the MAC faces (Fortran layout incl. halo) as float64 numpy arrays."""
    import torch

    rng = np.random.default_rng(seed + 7919)
    nx, ny, nz = int(p["nx"]), int(p["ny"]), int(p["nz"])
    h = float(p["dx"])
    L = np.array([nx * h, ny * h, nz * h])
    ks, amps, phases = [], [], []
    while len(ks) < n_modes:
        kv = rng.integers(-kmax, kmax + 1, size=3)
        if not kv.any() or np.linalg.norm(kv) > kmax:
            continue
        k = 2 * math.pi * kv / L
        a = rng.standard_normal(3)
        a -= k * (a @ k) / (k @ k)
        a /= np.linalg.norm(a)
        ks.append(k)
        amps.append(a)
        phases.append(rng.random() * 2 * math.pi)
    w = rng.random(n_modes) + 0.5
    w *= amp / w.sum()
    shape = field_shape(p)
    dev = torch.device(device)
    # plane waves at cell centres; component c sits half a cell lower along axis c,
    # which is the phase factor exp(-i k_c h/2) on the same wave
    cen = [(torch.arange(1, n + 1, dtype=torch.float64, device=dev) - 0.5) * h for n in (nx, ny, nz)]
    accs = [torch.zeros((nz, ny, nx), dtype=torch.float64, device=dev) for _ in range(3)]
    for m in range(n_modes):
        k = ks[m]
        ex = torch.exp(1j * (k[0] * cen[0]))
        ey = torch.exp(1j * (k[1] * cen[1]))
        ez = torch.exp(1j * (k[2] * cen[2] + phases[m]))
        wave = (ez[:, None] * ey[None, :])[:, :, None] * ex[None, None, :]
        for comp in range(3):
            coef = complex(w[m] * amps[m][comp]) * complex(np.exp(-0.5j * k[comp] * h))
            accs[comp] += (coef * wave).real
        del wave
    out = []
    for comp in range(3):
        full = torch.zeros(shape, dtype=torch.float64, device=dev)
        full[2:-2, 2:-2, 2:-2] = accs[comp]
        # periodic halo, as FillGhostRegionForFluid leaves it
        iz = (torch.arange(shape[0], device=dev) - 2) % nz + 2
        iy = (torch.arange(shape[1], device=dev) - 2) % ny + 2
        ix = (torch.arange(shape[2], device=dev) - 2) % nx + 2
        full = full[iz][:, iy][:, :, ix]
        out.append(np.ascontiguousarray(full.cpu().numpy()))
    return out


def resolved_case(nx, ny, nz, nbodies, d, seed=0, h=1.0, vel_std=0.01, n_modes=32, amp=0.05,
                  rho_p=1.14e3, field_device="cpu", n_markers=None, **param_kw):
    """A triply periodic case of monodisperse spheres in a frozen Fourier field.

    Returns (params, parcels, bodies, (u, v, w))."""
    p = make_params(nx, ny, nz, h=h, **param_kw)
    rng = np.random.default_rng(seed)
    L = np.array([nx * h, ny * h, nz * h])
    centres = rsa_centres(L, nbodies, d * h, rng)
    vel = rng.standard_normal((nbodies, 3)) * vel_std
    parts, bodies = sphere_bodies(centres, d * h, h, rho_p, vel, n_markers=n_markers)
    parts["x"] = wrap_coord(parts["x"], L)
    field = fourier_field(p, n_modes, amp, seed, device=field_device) if n_modes > 0 else \
        [np.zeros(field_shape(p)) for _ in range(3)]
    return p, parts, bodies, field


def kolmogorov_field(p, amp=0.05):
    """Periodic shear u_x = amp*sin(2*pi*z/Lz) on the u faces (z = (k-1/2)h), v = w = 0,
    Fortran layout with the periodic 2-cell halo."""
    nz = int(p["nz"])
    h = float(p["dz"])
    shape = field_shape(p)
    k = (np.arange(shape[0]) - 2) % nz + 1  # interior index of every z layer, halo wrapped
    prof = amp * np.sin(2 * math.pi * ((k - 0.5) * h) / (nz * h))
    u = np.broadcast_to(prof[:, None, None], shape).copy()
    return [u, np.zeros(shape), np.zeros(shape)]


def fill_halo(p, fields):
    """The fluid solver's boundary treatment of u, v, w (in place): the halo refill
    of FillGhostRegionForFluid (boundary.F90:122-147) face by face -- periodic
    copies, or beyond a solid wall the mirrored cells with all components
    negated (DealWithBoundaryFluid, boundary.F90:211-245) -- then Boundary()
    (fluid.F90:240-249), which zeroes the wall-normal velocity on the wall face
    and beyond.  A field handed to the library should already satisfy this."""
    n = [int(p["nx"]), int(p["ny"]), int(p["nz"])]
    bt = [int(b) for b in p["bType"]]

    def ax(d):  # array axis of grid axis d (arrays are (k, j, i))
        return 2 - d

    def sl(d, lo, hi, e_lo):  # index tuple: axis d in [lo, hi] (Fortran), others per e_lo
        idx = [slice(None)] * 3
        for e in range(3):
            if e == d:
                idx[ax(e)] = slice(lo + 1, hi + 2)
            elif e > d:  # not yet filled: interior only
                idx[ax(e)] = slice(2, n[e] + 2)
            else:
                idx[ax(e)] = slice(None)
        return tuple(idx)

    for side in range(6):
        recv = side ^ 1
        d = recv // 2
        wall = bt[recv] == 1
        src_side = recv if wall else side
        s_lo = 1 if src_side % 2 == 0 else n[d] - 1
        src = sl(d, s_lo, s_lo + 1, None)
        if not wall:
            r_lo = -1 if recv % 2 == 0 else n[d] + 1
            dst = sl(d, r_lo, r_lo + 1, None)
            for f in fields:
                f[dst] = f[src]
        else:
            # filled outward from the wall: source cell t -> halo cell t beyond
            for f in fields:
                block = -np.flip(f[src], axis=ax(d)) if recv % 2 == 0 else -f[src]
                if recv % 2 == 0:
                    f[sl(d, -1, 0, None)] = block          # halo(0) = -f(1), halo(-1) = -f(2)
                else:
                    f[sl(d, n[d] + 1, n[d] + 2, None)] = np.flip(block, axis=ax(d))
    for side in range(6):
        if bt[side] != 1:
            continue
        d = side // 2
        idx = [slice(None)] * 3
        idx[ax(d)] = slice(0, 3) if side % 2 == 0 else slice(n[d] + 2, n[d] + 4)
        fields[d][tuple(idx)] = 0.0
    return fields


def walled_case(nx, ny, nz, nbodies, d, seed=0, h=1.0, walls="z", vel_std=0.01, n_modes=16, amp=0.05,
                rho_p=1.14e3, n_markers=None, touching=2, **param_kw):
    """Spheres between solid walls on the axes in `walls` (the others periodic):
    `touching` bodies rest against the low wall of the first walled axis (their
    nearest markers within the contact distance of the wall, moving towards it),
    the rest are placed at random clear of the walls.  The Fourier field is
    given the wall conditions by fill_halo.  Returns (params, parcels, bodies,
    (u, v, w))."""
    p = make_params(nx, ny, nz, h=h, walls=walls, **param_kw)
    rng = np.random.default_rng(seed)
    L = np.array([nx * h, ny * h, nz * h])
    R = 0.5 * d * h
    wa = ["xyz".index(a) for a in walls]
    centres = []
    for b in range(touching):
        # clear of the other walls and of each other
        for _ in range(100_000):
            c = rng.uniform(0, 1, 3) * L
            for a in wa[1:]:
                c[a] = rng.uniform(R + 1.5 * h, L[a] - R - 1.5 * h)
            # lowest markers at radius R - 0.3h sit 0.4h from the wall (< radeff = 0.75h)
            c[wa[0]] = (R - 0.3 * h) + 0.4 * h
            dd = [c - q for q in centres]
            for v in dd:
                for e in range(3):
                    if e not in wa:
                        v[e] -= L[e] * round(v[e] / L[e])
            if all(float(v @ v) > (2 * R + 0.5 * h) ** 2 for v in dd):
                break
        centres.append(c)
    tries = 0
    while len(centres) < nbodies:
        tries += 1
        if tries > 1_000_000:
            raise RuntimeError("could not place the bodies")
        c = rng.uniform(0, 1, 3) * L
        if any(c[a] < R + 1.5 * h or c[a] > L[a] - R - 1.5 * h for a in wa):
            continue
        ok = True
        for q in centres:
            dd = c - q
            for e in range(3):
                if e not in wa:
                    dd[e] -= L[e] * round(dd[e] / L[e])
            if float(dd @ dd) <= (2 * R + 0.5 * h) ** 2:
                ok = False
                break
        if ok:
            centres.append(c)
    centres = np.array(centres)
    vel = rng.standard_normal((nbodies, 3)) * vel_std
    vel[:touching, wa[0]] = -abs(vel[:touching, wa[0]]) - 0.01
    parts, bodies = sphere_bodies(centres, d * h, h, rho_p, vel, n_markers=n_markers)
    per = np.array([0 if e in wa else 1 for e in range(3)], bool)
    x = parts["x"].copy()
    xw = wrap_coord(x, L)
    x[:, per] = xw[:, per]
    parts["x"] = x
    field = fourier_field(p, n_modes, amp, seed) if n_modes > 0 else [np.zeros(field_shape(p)) for _ in range(3)]
    field = [np.array(f, dtype=np.float64, copy=True) for f in field]
    fill_halo(p, field)
    return p, parts, bodies, field


def _capped_bodies(n_cells, d, nb, max_fraction):
    cap = int(max_fraction * n_cells / (math.pi / 6.0 * d ** 3))
    return max(1, min(nb, cap))


def batched_mix(n_cases=256, seed=0, max_fraction=0.25, n_modes=32, field_device="cpu"):
    """Independent resolved cases of uneven size: case i draws (seed + i) a cubic
    grid from {32, 64, 96, 128}^3, a diameter from {8, 12, 16}h and a body count
    log-uniform in 8..512, capped so that the spheres fill at most max_fraction
    of the box; positions, velocities and the Fourier field as resolved_case."""
    out = []
    for i in range(n_cases):
        r = np.random.default_rng(seed + i)
        n = int(r.choice([32, 64, 96, 128]))
        d = float(r.choice([8.0, 12.0, 16.0]))
        nb = int(round(math.exp(r.uniform(math.log(8), math.log(512)))))
        nb = _capped_bodies(n ** 3, d, nb, max_fraction)
        out.append(resolved_case(n, n, n, nb, d, seed=seed + i, n_modes=n_modes, field_device=field_device))
    return out


def serve_requests(n_requests=32, seed=0, rate=200.0, d=12.0, max_fraction=0.2, grids=(64, 96, 128, 192, 256)):
    """A Poisson request stream (mean `rate` per second): request i has an
    arrival time, a body count log-uniform in 16..2048 on the smallest cubic grid
    of `grids` that keeps the solid fraction at most max_fraction (the largest
    grid caps the count), and is a settling case (fluid at rest, gravity) or a
    shear case (Kolmogorov field of amplitude 0.05), alternating at random.
    Returns a list of dicts with arrival, kind and the case (params, parcels,
    bodies, field or None)."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(n_requests):
        t += rng.exponential(1.0 / rate)
        nb = int(round(math.exp(rng.uniform(math.log(16), math.log(2048)))))
        vol = math.pi / 6.0 * d ** 3
        n = next((g for g in grids if nb * vol <= max_fraction * g ** 3), grids[-1])
        nb = _capped_bodies(n ** 3, d, nb, max_fraction)
        kind = "shear" if rng.random() < 0.5 else "settling"
        p, parts, bodies, _ = resolved_case(n, n, n, nb, d, seed=seed * 100003 + i, n_modes=0)
        field = kolmogorov_field(p) if kind == "shear" else None
        out.append({"arrival": t, "kind": kind, "case": (p, parts, bodies, field)})
    return out


def unresolved_case(n=128, n_particles=1_048_576, seed=0, h=1e-3, d_mean=0.25, bed_share=0.75, u_up=0.5,
                    perturb=0.05, n_modes=32, rho_p=2500.0, field_device="cpu", bed_spacing=1.05, **param_kw):
    """Unresolved CFD-DEM case: n^3 periodic fluid cells of size h, polydisperse
    spheres with d uniform in [0.8, 1.2] * d_mean * h.  A packed bed: the first
    bed_share of the particles on a jittered lattice of spacing 1.05 * max d
    filling layers from z = 0 (bed_spacing < 1 packs them into contact); the
    rest on a coarser jittered lattice spread over the gas region above.  Fluid: uniform upward flow u_up
    plus a divergence-free Fourier perturbation of amplitude perturb * u_up.
    Bed particles start at rest, gas particles with N(0, 0.01 u_up) velocities.
    DEM cells of 1.1 * max d.  Returns (params, particles, (u, v, w))."""
    from .records import PARTICLE, make_params, make_uparams

    rng = np.random.default_rng(seed)
    L = n * h
    dmax = 1.2 * d_mean * h
    d = rng.uniform(0.8, 1.2, n_particles) * d_mean * h
    nbed = int(round(bed_share * n_particles))
    a = bed_spacing * dmax
    m = int(L // a)
    per_layer = m * m
    k = np.arange(nbed)
    lay, rem = k // per_layer, k % per_layer
    jit = abs(a - dmax) / 2
    bed = np.stack([(rem % m + 0.5) * a, (rem // m + 0.5) * a, (lay + 0.5) * a], axis=1)
    bed += rng.uniform(-jit, jit, bed.shape)
    top = (lay.max() + 1) * a if nbed else 0.0
    ngas = n_particles - nbed
    gas = np.zeros((0, 3))
    if ngas:
        hgt = L - top - a
        ag = (L * L * hgt / ngas) ** (1.0 / 3.0)
        mx, mz = max(int(L // ag), 1), max(int(hgt // ag), 1)
        while mx * mx * mz < ngas:
            ag *= 0.98
            mx, mz = max(int(L // ag), 1), max(int(hgt // ag), 1)
        pick = rng.permutation(mx * mx * mz)[:ngas]
        gx, gy, gz = pick % mx, (pick // mx) % mx, pick // (mx * mx)
        sx, sz = L / mx, hgt / mz
        gas = np.stack([(gx + 0.5) * sx, (gy + 0.5) * sx, top + a / 2 + (gz + 0.5) * sz], axis=1)
        gj = (min(sx, sz) - dmax) / 2
        gas += rng.uniform(-gj, gj, gas.shape)
    x = np.concatenate([bed, gas]) % L
    parts = np.zeros(n_particles, PARTICLE)
    parts["globalIdx"] = np.arange(1, n_particles + 1)
    parts["x"] = x
    parts["rad"] = d / 2
    parts["rho"] = rho_p
    parts["vol"] = np.pi / 6.0 * d ** 3
    parts["m"] = rho_p * parts["vol"]
    parts["I"] = 0.1 * parts["m"] * d ** 2
    parts["v"][nbed:] = rng.standard_normal((ngas, 3)) * 0.01 * u_up
    p = make_uparams(n, n, n, h, 1.1 * dmax, **param_kw)
    pf = make_params(n, n, n, h=h)
    field = fourier_field(pf, n_modes, perturb * u_up, seed, device=field_device) if n_modes else \
        [np.zeros(field_shape(pf)) for _ in range(3)]
    field[2] = field[2] + u_up
    return p, parts, field
