"""The C ABI driven by a compiled caller, as the reference's Fortran would drive it.

`tests/c_caller/coupled_step.c` is built with gcc against `include/ibmdem.h`
and `libibmdem.so` and runs the coupled sequence that replaces the particle
side of FirstOrderForwardEuler and the time loop (fluid.F90:252-285,
couplesolverCylinder.F90:189-217) on plain host arrays: ibmdem_set_fluid,
ibmdem_MultiDirectForcing, ibmdem_get_fluid, ibmdem_CloudEvolutionMS, the
returned velocity fed into the next step.  The same sequence through the Python
binding (whose results the other GPU tests compare with the CPU restatement)
must give the same fields, bodies and parcels bit for bit: the boundary carries
nothing but pointers, sizes and the record layouts.
"""
import os
import subprocess

import numpy as np
import pytest

import cases
import golden_util
from ibmdem import api
from ibmdem.records import MULTISPHERE, PARAMS, PARCEL

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
STEPS = 3


def _build(tmp):
    exe = os.path.join(tmp, "coupled_step")
    libdir = os.path.dirname(api.LIB_PATH)
    subprocess.run(["gcc", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"),
                    os.path.join(HERE, "c_caller", "coupled_step.c"), "-o", exe,
                    "-L", libdir, "-libmdem", "-Wl,-rpath," + libdir], check=True)
    return exe


def _python_run(p, parts, bodies, field):
    c = api.Case(p, parts, bodies, field, device=0)
    c.InitializationDEM()
    u, v, w = [np.array(f, dtype=np.float64) for f in field]
    out = None
    for _ in range(STEPS):
        c.set_fluid(u, v, w)
        c.MultiDirectForcing()
        out = c.get_fluid()
        c.CloudEvolutionMS()
        u, v, w = out[0], out[1], out[2]
    bodies_out = c.get_bodies()
    parcels, nl = c.get_parcels()
    c.close()
    return out, bodies_out, parcels[:nl]


@pytest.mark.parametrize("which", ["spheres", "cylinders"])
def test_compiled_caller_matches_the_binding(gpu_lib, tmp_path, which):
    if which == "spheres":
        p, parts, bodies, field = cases.contact_case(seed=8)
    else:
        _, (p, parts, bodies, field) = golden_util.load("cylinders")
    p = np.asarray(p, dtype=PARAMS)
    parts = np.ascontiguousarray(parts, dtype=PARCEL)
    bodies = np.ascontiguousarray(bodies, dtype=MULTISPHERE)
    shape = api.field_shape(p)
    field = [np.ascontiguousarray(np.asarray(f, dtype=np.float64).reshape(shape)) for f in field]
    tmp = str(tmp_path)
    p.reshape(1).tofile(os.path.join(tmp, "params.bin"))
    parts.tofile(os.path.join(tmp, "parcels.bin"))
    bodies.tofile(os.path.join(tmp, "bodies.bin"))
    for name, f in zip("uvw", field):
        f.tofile(os.path.join(tmp, name + ".bin"))
    exe = _build(tmp)
    run = subprocess.run([exe, tmp, str(STEPS)], capture_output=True, text=True)
    assert run.returncode == 0, run.stderr
    fields_c = np.fromfile(os.path.join(tmp, "fields.bin"), dtype=np.float64).reshape((6,) + shape)
    bodies_c = np.fromfile(os.path.join(tmp, "bodies.bin.out"), dtype=MULTISPHERE)
    parcels_c = np.fromfile(os.path.join(tmp, "parcels.bin.out"), dtype=PARCEL)

    fields_py, bodies_py, parcels_py = _python_run(p, parts, bodies, field)
    for a, b in zip(fields_c, fields_py):
        assert np.array_equal(a, b)
    assert len(bodies_c) == len(bodies_py)
    for f in ("x", "v", "omega", "AngMom", "rotMatGlo", "fdrag", "fcol", "fmom", "fmomCol", "fhydro"):
        assert np.array_equal(bodies_c[f], bodies_py[f]), f
    assert len(parcels_c) == len(parcels_py)
    for f in ("x", "v", "fdrag", "fcol", "vgap", "globalIdx", "MSIdx", "cellIdx"):
        assert np.array_equal(parcels_c[f], parcels_py[f]), f
    # the forcing loop did work
    assert np.abs(fields_c[3]).max() > 0.0
