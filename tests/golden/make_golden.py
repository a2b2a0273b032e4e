"""Generate the golden fixtures of tests/test_golden.py and tests/test_gpu_golden.py.

Two single-rank periodic cases, run through the CPU restatement (oracle/):
  sphere_contact  24^3 grid, h = 1: four spheres (d = 8h), two in contact, one
                  straddling the x = 0 face;
  cylinders       48x24x48 grid with the reference's own units (dx = 3.75e-5 m):
                  three cylinders built exactly as InitCylinderParcelsDEM
                  (ZJS_INIT_DEM.F90:350-494) builds them from the reference's
                  marker template CYLINDER_LP1125.dat -- radius 2.08e-4 (a
                  single-precision literal), height 4x radius, template scaled by
                  (rad-0.3dx)*height/rad and height-0.6dx, rotated by an initial
                  angle about y, rho = 2650, the cylinder inertia tensor.
Inputs (parameters, parcels, bodies, a float32-exact fluid field) and outputs
(cell lists and contact lists after InitializationDEM; parcels, bodies and the
touched fluid/forcing values after two frozen-fluid steps) are stored in
sphere_contact.npz and cylinders.npz.

Run from the repository root (needs the reference checkout for the template):
    python tests/golden/make_golden.py /path/to/reference
"""
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (os.path.join(ROOT, "ibm-dem_gb300"), os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    sys.path.insert(0, p)

import cases  # noqa: E402
import oracle as O  # noqa: E402
from ibmdem import scenario  # noqa: E402
from ibmdem.records import MULTISPHERE, PARCEL, make_params  # noqa: E402


def f32_field(field):
    return [np.asarray(f, dtype=np.float32).astype(np.float64) for f in field]


def rotate_matrix(theta):
    """CalculateRotateMatrix (couplesolverCylinder.F90:76-97)."""
    mag = max(math.sqrt(theta[0] ** 2 + theta[1] ** 2 + theta[2] ** 2), 1e-10)
    ux, uy, uz = theta[0] / mag, theta[1] / mag, theta[2] / mag
    c, s = math.cos(mag), math.sin(mag)
    return np.array([(1 - c) * ux * ux + c, (1 - c) * ux * uy - s * uz, (1 - c) * ux * uz + s * uy,
                     (1 - c) * uy * ux + s * uz, (1 - c) * uy * uy + c, (1 - c) * uy * uz - s * ux,
                     (1 - c) * uz * ux - s * uy, (1 - c) * uz * uy + s * ux, (1 - c) * uz * uz + c])


CYLINDER_CENTRES = [[0.55e-3, 0.45e-3, 0.9e-3], [1.42e-3, 0.46e-3, 0.62e-3], [0.95e-3, 0.44e-3, 1.55e-3]]


def cylinder_geometry(dx):
    """InitCylinderParcelsDEM's shape constants (ZJS_INIT_DEM.F90:370-381): radius
    2.08e-4 (a single-precision literal), height 4x radius, the template scaled by
    (rad-0.3dx)*height/rad and height-0.6dx, rho = 2650."""
    rad = float(np.float32(2.08e-4))
    height = rad * 4
    return {"rad": rad, "height": height, "radratio": (rad - 0.3 * dx) * height / rad,
            "heightratio": height - 0.3 * 2 * dx, "pi": math.acos(-1.0), "rho": 2.65e3}


def cylinder_bodies(centres, rnd, vel, dx):
    """The cylinders' body records as InitCylinderParcelsDEM fills them: mass
    properties, the cylinder inertia tensor and a rotation by pi/2*rnd about y."""
    g = cylinder_geometry(dx)
    rad, height, pi = g["rad"], g["height"], g["pi"]
    centres, vel = np.asarray(centres, dtype=np.float64), np.asarray(vel, dtype=np.float64)
    bodies = np.zeros(len(centres), MULTISPHERE)
    for j in range(len(centres)):
        rot = rotate_matrix([0.0, pi / 2.0 * rnd[j], 0.0])
        B = bodies[j:j + 1]
        B["globalIdx"] = j + 1
        B["x"] = centres[j]
        B["v"] = vel[j]
        B["vold"] = vel[j]
        B["rad"] = rad
        B["rho"] = g["rho"]
        B["vol"] = (pi * rad ** 2) * height
        B["m"] = B["vol"] * B["rho"]
        it = np.zeros(9)
        it[0] = B["m"][0] * (3.0 * rad ** 2 + height ** 2) / 12.0
        it[4] = it[0]
        it[8] = 0.5 * B["m"][0] * rad ** 2
        B["InertiaTensor"] = it
        B["rotMat"] = rot
        B["rotMatGlo"] = rot
        B["rotMatGloOld"] = rot
    return bodies


def cylinder_markers(tpl, bodies, dx, L=None):
    """Every body's template markers, scaled, rotated about the body centre and
    (with a box length L) wrapped into the box, body by body."""
    g = cylinder_geometry(dx)
    nl = len(tpl)
    parts = np.zeros(len(bodies) * nl, PARCEL)
    for j in range(len(bodies)):
        c = bodies["x"][j]
        R = bodies["rotMat"][j].reshape(3, 3)
        x = np.stack([g["radratio"] * tpl[:, 0] + c[0], g["radratio"] * tpl[:, 1] + c[1],
                      g["heightratio"] * tpl[:, 2] + c[2]], axis=1)
        xt = x - c
        x = np.stack([R[0, 0] * xt[:, 0] + R[0, 1] * xt[:, 1] + R[0, 2] * xt[:, 2],
                      R[1, 0] * xt[:, 0] + R[1, 1] * xt[:, 1] + R[1, 2] * xt[:, 2],
                      R[2, 0] * xt[:, 0] + R[2, 1] * xt[:, 1] + R[2, 2] * xt[:, 2]], axis=1) + c
        sl = slice(j * nl, (j + 1) * nl)
        parts["x"][sl] = x if L is None else scenario.wrap_coord(x, L)
        parts["v"][sl] = bodies["v"][j]
        parts["radeff"][sl] = dx * 0.75
        parts["vol"][sl] = g["pi"] * dx / nl * (g["rad"] ** 2 + 2 * g["rad"] * g["height"] + 0.25 * dx ** 2)
        parts["rho"][sl] = g["rho"]
        parts["m"][sl] = parts["rho"][sl] * parts["vol"][sl]
        parts["MSIdx"][sl] = j + 1
        parts["globalIdx"][sl] = np.arange(1, nl + 1)
    return parts


def cylinder_case(template, centres=CYLINDER_CENTRES):
    n = (48, 24, 48)
    dx = 9e-3 / 240  # PartitionInitialization(4,1,4,240,32,240,9d-3,1.2d-3,9d-3)
    p = make_params(*n, h=dx, dt=5e-5, coupleInterval=2, knCoeff=4e4, ResistCoeff=0.9)
    tpl = np.loadtxt(template)
    rnd = [0.2, 0.7, 0.45]
    vel = np.array([[1e-3, 0.0, -5e-4], [-1e-3, 2e-4, 0.0], [0.0, -3e-4, 8e-4]])
    bodies = cylinder_bodies(centres, rnd, vel, dx)
    parts = cylinder_markers(tpl, bodies, dx, np.array(n) * dx)
    field = scenario.fourier_field(p, 6, 0.02, seed=5)
    return p, parts, bodies, f32_field(field)


def sphere_case():
    p, parts, bodies, field = cases.contact_case(seed=3)
    return p, parts, bodies, f32_field(field)


def run(case):
    p, parts, bodies, field = case
    r = O.OracleCase(p, parts, bodies, field)
    r.InitializationDEM()
    out = {}
    out["cell_start"], out["cell_items"] = r.get_cell_lists()
    out["pair_start"], out["pair_idx"] = r.get_collision_lists()
    pi, nli = r.get_parcels()
    out["init_parcels"] = pi
    out["init_nlocal"] = nli
    r.step(2)
    pp, nl = r.get_parcels()
    out["parcels"] = pp
    out["nlocal"] = nl
    out["bodies"] = r.get_bodies()
    u, v, w, fx, fy, fz = r.get_fluid()
    for name, a, a0 in (("u", u, field[0]), ("v", v, field[1]), ("w", w, field[2]),
                        ("fx", fx, None), ("fy", fy, None), ("fz", fz, None)):
        ref = np.zeros_like(a) if a0 is None else a0
        idx = np.flatnonzero(a.ravel() != ref.ravel())
        out[name + "_idx"] = idx.astype(np.int64)
        out[name + "_val"] = a.ravel()[idx]
    out["params"] = np.array(p)
    out["in_parcels"] = parts
    out["in_bodies"] = bodies
    for c, f in zip("uvw", field):
        out["in_" + c] = f.astype(np.float32)
    r.close()
    return out


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: python make_golden.py <directory of the reference sources holding CYLINDER_LP1125.dat>")
    ref = sys.argv[1]
    np.savez_compressed(os.path.join(HERE, "sphere_contact.npz"), **run(sphere_case()))
    np.savez_compressed(os.path.join(HERE, "cylinders.npz"),
                        **run(cylinder_case(os.path.join(ref, "CYLINDER_LP1125.dat"))))


if __name__ == "__main__":
    main()
