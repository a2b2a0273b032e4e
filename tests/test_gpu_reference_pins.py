"""The CUDA library against the reference's own subroutines, through the C ABI.

The fixtures tests/golden/ref_*.npz hold the state of the reference's Fortran
statements (run by tests/golden/make_reference_golden.py) after
InitializationDEM and after each forcing loop and CloudEvolutionMS of two or
three coupled steps.  The library replays the same stages from the same inputs
and agrees bit for bit at every one of them: cell lists, contact lists, every
parcel field the reference defines (images included), the fields u, v, w with
their halo and fx, fy, fz, the bodies, the wall-probe forces.  (The body
rotation goes through CUDA's cos and sin, the reference's through the host's;
on these cases they agree to the last bit.)
"""
import os
import sys

import numpy as np
import pytest


pytestmark = pytest.mark.gpu

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from test_reference_pins import IMAGE_FIELDS, load, mrg  # noqa: E402

BODY_FIELDS = ("x", "v", "omega", "AngMom", "rotMat", "rotMatGlo", "fdrag", "fcol", "fmom", "fmomCol", "fhydro",
               "fmomHydro", "vold", "AngMomOld")


def same(a, b, what):
    assert np.array_equal(a, b), what


def check(ref, tag, c, fields=False):
    s, i = c.get_cell_lists()
    assert np.array_equal(s, ref[tag + "_cell_start"]) and np.array_equal(i, ref[tag + "_cell_items"]), \
        f"{tag}: cell lists"
    s, i = c.get_collision_lists()
    assert np.array_equal(s, ref[tag + "_pair_start"]) and np.array_equal(i, ref[tag + "_pair_items"]), \
        f"{tag}: contact lists"
    parts, nl = c.get_parcels()
    want = ref[tag + "_parcels"]
    assert nl == int(ref[tag + "_nlocal"]) and len(parts) == len(want), tag
    for f in ("globalIdx", "cellIdx", "MSIdx", "pType"):
        assert np.array_equal(parts[f], want[f]), f"{tag}: parcel {f}"
    for f in ("x", "v", "fdrag", "vol", "m", "radeff"):
        same(parts[f], want[f], f"{tag}: parcel {f}")
    for f in ("fcol", "vgap"):
        same(parts[f][:nl], want[f][:nl], f"{tag}: local parcel {f}")
    assert set(IMAGE_FIELDS) >= {"x", "v", "fdrag"}
    bodies, wb = c.get_bodies(), ref[tag + "_bodies"]
    for f in BODY_FIELDS:
        same(bodies[f], wb[f], f"{tag}: body {f}")
    if len(ref[tag + "_probe_force"]):
        got = np.array([p["force"] for p in c.get_wall_probes()])
        same(got, ref[tag + "_probe_force"], f"{tag}: probe forces")
    if fields:
        for name, a in zip(("u", "v", "w", "fx", "fy", "fz"), c.get_fluid()):
            same(a[2:-2, 2:-2, 2:-2], ref[f"{tag}_{name}"], f"{tag}: {name}")


@pytest.mark.parametrize("name", ["periodic", "walled", "single"])
def test_library_matches_the_reference(gpu_lib, name):
    ref = load(name)
    field = (ref["in_u"], ref["in_v"], ref["in_w"])
    c = gpu_lib.Case(ref["params"], ref["in_parcels"], ref["in_bodies"], field, device=0)
    try:
        if len(ref["in_probes"]):
            c.set_wall_probes(ref["in_probes"])
        c.InitializationDEM()
        check(ref, "init", c)
        for s in range(int(ref["steps"])):
            c.set_fluid(*field)
            c.MultiDirectForcing()
            check(ref, f"mdf{s}", c, fields=True)
            c.CloudEvolutionMS()
            check(ref, f"step{s}", c)
    finally:
        c.close()



@pytest.mark.parametrize("name", ["corner", "edge", "empty", "cylinders"])
def test_compact_cases(gpu_lib, name):
    """Fixtures stored as digests (tests/golden/ref_{corner,edge,empty,cylinders}.npz):
    every stage's parcels, cell lists, contact lists, fields and probe forces
    match the reference's digests, the bodies and the final parcel positions and
    velocities are bit-identical."""
    from test_reference_pins import compact_stage

    ref = load(name)
    field = tuple(ref[f"in_{a}"].astype(np.float64) for a in "uvw")
    c = gpu_lib.Case(ref["params"], ref["in_parcels"], ref["in_bodies"], field, device=0)
    try:
        if len(ref["in_probes"]):
            c.set_wall_probes(ref["in_probes"])
        c.InitializationDEM()
        compact_stage(ref, "init", c, windows=False)
        for s in range(int(ref["steps"])):
            c.set_fluid(*field)
            c.MultiDirectForcing()
            compact_stage(ref, f"mdf{s}", c, fields=True, windows=False)
            c.CloudEvolutionMS()
            compact_stage(ref, f"step{s}", c, windows=False)
        parts, _ = c.get_parcels()
        assert np.array_equal(parts["x"], ref["final_x"]) and np.array_equal(parts["v"], ref["final_v"])
    finally:
        c.close()


def test_hundred_step_trajectory(gpu_lib):
    """One hundred coupled steps of the periodic case (tests/golden/ref_trajectory.npz):
    after every step the bodies, the parcels and the forcing loop's fields are
    bit-identical to the reference's."""
    from ibmdem import records

    ref = load("trajectory")
    field = (ref["in_u"], ref["in_v"], ref["in_w"])
    c = gpu_lib.Case(ref["params"], ref["in_parcels"], ref["in_bodies"], field, device=0)
    try:
        c.InitializationDEM()
        for s in range(int(ref["steps"])):
            c.set_fluid(*field)
            c.MultiDirectForcing()
            same(mrg.field_digest(c.get_fluid()), ref["field_digest"][s], f"step {s}: fields")
            c.CloudEvolutionMS()
            parts, nl = c.get_parcels()
            same(mrg.parcel_digest(parts, nl), ref["parcel_digest"][s], f"step {s}: parcels")
            got = c.get_bodies()
            for f in records.MULTISPHERE.names:
                same(got[f], ref["bodies"][s][f], f"step {s}: body {f}")
    finally:
        c.close()


def test_whole_time_step(gpu_lib):
    """The reference's FirstOrderForwardEuler (fluid.F90:252-327) on the library:
    StoreOldVelocity, the forcing loop, VelocityGuess, ModifyBulkVelocity,
    VelocityDivergence, PressureCorrection with the fixture's supplied Poisson
    solve (tests/fft_poisson.py), VelocityCorrection, each with its halo refill,
    and CloudEvolutionMS (tests/golden/ref_coupled.npz, first step).  The
    library forms ModifyBulkVelocity's sums in an order of its own, so u, v, w
    and P agree to 1e-10 of their largest value; the bodies, which the forcing
    loop before it sets, bit for bit."""
    import cases
    import fft_poisson
    from ibmdem import records

    ref = load("coupled")
    p = ref["params"]
    h = (float(p["dx"]), float(p["dy"]), float(p["dz"]))
    field = tuple(ref[f"in_{a}"].astype(np.float64) for a in "uvw")
    b = ref["bulk"]
    c = gpu_lib.Case(p, ref["in_parcels"], ref["in_bodies"], field, device=0)
    try:
        c.set_fluid_params(float(ref["visc"]))
        c.InitializationDEM()
        c.StoreOldVelocity()
        c.MultiDirectForcing()
        c.VelocityGuess(1.0, 0.0, 1.0)
        c.FillGhostRegionForFluid()
        c.Boundary()
        c.ModifyBulkVelocity(int(b[0]), int(b[1]), int(b[2]), b[3], b[4], b[5])
        c.FillGhostRegionForFluid()
        c.Boundary()
        c.VelocityDivergence(1.0)
        c.FillGhostRegionForFluid()
        c.Boundary()
        pc = c.get_fluid_field("Pcorr")
        pc[2:-2, 2:-2, 2:-2] = fft_poisson.solve(c.get_fluid_field("velDiv")[2:-2, 2:-2, 2:-2], h, str(ref["walls"]))
        c.PressureCorrection(pc)
        c.FillGhostRegionForFluid()
        c.Boundary()
        c.VelocityCorrection(1.0)
        c.FillGhostRegionForFluid()
        c.Boundary()
        c.CloudEvolutionMS()
        for f in ("u", "v", "w", "P"):
            assert cases.rel_close(c.get_fluid_field(f), ref[f"step0_{f}_values"], 1e-10), f
        got = c.get_bodies()
        for f in records.MULTISPHERE.names:
            same(got[f], ref["step0_bodies"][f], f"body {f}")
    finally:
        c.close()


def test_benchmark_configuration(gpu_lib):
    """The benchmark's CPU-runnable configuration (128^3 periodic, 64 spheres of
    d = 16h, 51,456 markers), regenerated from its seed: after
    InitializationDEM and the first forcing loop the parcels, cell lists,
    contact lists and fields equal the reference's; after CloudEvolutionMS every
    body's translation does, and the rotation of each body that does not
    straddle a periodic face (tests/golden/ref_config.npz)."""
    from ibmdem import records

    ref = load("config")
    p, parts, bodies, field = mrg.config_case()
    same(mrg.parcel_digest(parts, len(parts)), ref["in_parcel_digest"], "regenerated parcels")
    same(mrg.digest(*[bodies[f] for f in records.MULTISPHERE.names]), ref["in_body_digest"], "regenerated bodies")
    same(mrg.digest(*field), ref["in_field_digest"], "regenerated field")
    c = gpu_lib.Case(p, parts, bodies, field, device=0)
    try:
        c.InitializationDEM()
        for tag in ("init", "mdf0"):
            if tag == "mdf0":
                c.set_fluid(*field)
                c.MultiDirectForcing()
                same(mrg.field_digest(c.get_fluid()), ref["mdf0_field_digest"], "mdf0: fields")
            got, nl = c.get_parcels()
            same(mrg.parcel_digest(got, nl), ref[tag + "_parcel_digest"], f"{tag}: parcels")
            same(mrg.digest(*c.get_cell_lists()), ref[tag + "_cell_digest"], f"{tag}: cell lists")
            same(mrg.digest(*c.get_collision_lists()), ref[tag + "_pair_digest"], f"{tag}: contact lists")
        c.CloudEvolutionMS()
        got, want, far = c.get_bodies(), ref["step0_bodies"], ref["straddlers"]
        for f in ("x", "v", "vold", "fdrag", "fcol", "fhydro"):
            same(got[f], want[f], f"body {f}")
        for f in ("omega", "AngMom", "rotMat", "rotMatGlo", "fmom", "fmomCol", "fmomHydro"):
            same(got[f][~far], want[f][~far], f"body {f} (bodies inside the box)")
    finally:
        c.close()


def test_runge_kutta_fluid_step(gpu_lib):
    """The reference's ThirdOrderLowStorageRungeKutta (fluid.F90:329-366) between
    walls in z, each stage's Poisson solve replaced by the fixture's correction:
    the velocity and divergence where each solve starts and every field written
    by the end are bit-identical (tests/golden/ref_fluid_rk3_walls_z.npz)."""
    from test_reference_pins import digest

    ref = load("fluid_rk3_walls_z")
    # the fluid stencils work on the fields ibmdem_set_fluid installs
    c = gpu_lib.Case(ref["params"], field=(ref["in_u"], ref["in_v"], ref["in_w"]), device=0)
    try:
        for f in mrg.FLUID_INPUTS:
            c.set_fluid_field(f, ref["in_" + f])
        c.set_fluid_params(float(ref["visc"]))
        aRK = [32.0 / 60.0, 25.0 / 60.0, 45.0 / 60.0]
        bRK = [0.0, -17.0 / 60.0, -25.0 / 60.0]
        for k in range(3):
            cRK = aRK[k] + bRK[k]
            c.VelocityGuess(aRK[k], bRK[k], cRK)
            c.FillGhostRegionForFluid()
            c.Boundary()
            c.VelocityDivergence(cRK)
            c.FillGhostRegionForFluid()
            c.Boundary()
            for f in ("u", "v", "w", "velDiv"):
                assert np.array_equal(digest(c.get_fluid_field(f)), ref[f"rk{k}_{f}"]), f"stage {k}: {f}"
            c.set_fluid_field("Pcorr", ref[f"in_pcorr{k}"])
            c.PressureCorrection()
            c.FillGhostRegionForFluid()
            c.Boundary()
            c.VelocityCorrection(cRK)
            c.FillGhostRegionForFluid()
            c.Boundary()
        for f in mrg.RK3_WRITTEN:
            assert np.array_equal(digest(c.get_fluid_field(f)), ref[f"end_{f}"]), f
    finally:
        c.close()
