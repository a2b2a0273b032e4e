"""The CPU restatement in oracle/ against the reference's own subroutines.

The fixtures tests/golden/ref_*.npz were made by make_reference_golden.py, which
runs the reference's Fortran statements (through fortran_subset.py, on one
rank) on seeded cases.  Here the restatement replays the same stages from the
same inputs and must agree bit for bit at every one of them:

* three coupled cases, three steps of two or three DEM sub-steps each:
  periodic with a body contact; walls in z with wall contact and probes; one
  body, where the reference's own one-rank CloudEvolutionStepMS runs unchanged
  (the other two run its multi-rank branch).  After InitializationDEM, after each forcing
  loop (fluid.F90:258-280) and after each CloudEvolutionMS
  (couplesolverCylinder.F90:189-217) -- every parcel field the reference
  defines (images included), every body field, the per-cell parcel lists, the
  contact lists, the interpolation windows and weights, the fields u, v, w
  (halo included) and fx, fy, fz, the wall-probe forces;
* the fluid step's stencils (fluid.F90:2-250, boundary.F90:122-245) on random
  fields, periodic and between walls;
* the drag law CalculateDragForce (ZJS_DRAGFORCE_DEM.F90:2-35).
"""
import hashlib
import os
import sys

import numpy as np
import pytest

from ibmdem import records

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
if GOLDEN not in sys.path:
    sys.path.insert(0, GOLDEN)
import make_reference_golden as mrg  # noqa: E402

IMAGE_FIELDS = mrg.IMAGE_FIELDS


def load(name):
    with np.load(os.path.join(GOLDEN, f"ref_{name}.npz"), allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


def digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return np.frombuffer(h.digest(), np.uint8)


def check_stage(ref, tag, c):
    """State of the restatement `c` against the reference's at stage `tag`."""
    parts, nl = c.get_parcels()
    want = ref[tag + "_parcels"]
    assert nl == int(ref[tag + "_nlocal"]), tag
    assert len(parts) == len(want), tag
    for f in records.PARCEL.names:
        if f == "pad_":
            continue
        assert np.array_equal(parts[f][:nl], want[f][:nl]), f"{tag}: local parcel {f}"
        if f in IMAGE_FIELDS:
            assert np.array_equal(parts[f][nl:], want[f][nl:]), f"{tag}: image parcel {f}"
    bodies, wb = c.get_bodies(), ref[tag + "_bodies"]
    for f in records.MULTISPHERE.names:
        assert np.array_equal(bodies[f], wb[f]), f"{tag}: body {f}"
    s, i = c.get_cell_lists()
    assert np.array_equal(s, ref[tag + "_cell_start"]) and np.array_equal(i, ref[tag + "_cell_items"]), \
        f"{tag}: cell lists"
    s, i = c.get_collision_lists()
    assert np.array_equal(s, ref[tag + "_pair_start"]) and np.array_equal(i, ref[tag + "_pair_items"]), \
        f"{tag}: contact lists"
    n = len(parts)
    w, cells = c.get_weights(n)
    cnt = ref[tag + "_window_count"]
    used = np.arange(125)[None, :] < cnt[:, None]
    assert np.array_equal(digest(np.where(used, cells, 0).astype(np.int32), np.where(used[..., None], w, 0.0)),
                          ref[tag + "_window_digest"]), f"{tag}: interpolation windows"
    if len(ref[tag + "_probe_force"]):
        got = np.array([p["force"] for p in c.get_wall_probes()])
        assert np.array_equal(got, ref[tag + "_probe_force"]), f"{tag}: probe forces"


def check_fields(ref, tag, c):
    for name, a in zip(("u", "v", "w", "fx", "fy", "fz"), c.get_fluid()):
        assert np.array_equal(a[2:-2, 2:-2, 2:-2], ref[f"{tag}_{name}"]), f"{tag}: {name}"


@pytest.mark.parametrize("name", ["periodic", "walled", "single"])
def test_coupled_steps_match_the_reference(oracle_mod, name):
    ref = load(name)
    field = (ref["in_u"], ref["in_v"], ref["in_w"])
    c = oracle_mod.OracleCase(ref["params"], ref["in_parcels"], ref["in_bodies"], field)
    if len(ref["in_probes"]):
        c.set_wall_probes(ref["in_probes"])
    c.InitializationDEM()
    check_stage(ref, "init", c)
    if len(ref["in_bodies"]) > 1:
        assert len(ref["init_pair_items"]) > 0, "the case has contacts"
    assert len(ref["init_parcels"]) > int(ref["init_nlocal"]), "the case has images"
    for s in range(int(ref["steps"])):
        c.set_fluid(*field)
        c.MultiDirectForcing()
        check_stage(ref, f"mdf{s}", c)
        check_fields(ref, f"mdf{s}", c)
        c.CloudEvolutionMS()
        check_stage(ref, f"step{s}", c)
    c.close()


def compact_stage(ref, tag, c, fields=False, bodies=True, windows=True):
    """A stage of a fixture stored as digests (bodies and probe forces in full);
    `windows` off for a case without get_weights."""
    parts, nl = c.get_parcels()
    assert nl == int(ref[tag + "_nlocal"]) and len(parts) == int(ref[tag + "_np"]), tag
    assert np.array_equal(mrg.parcel_digest(parts, nl), ref[tag + "_parcel_digest"]), f"{tag}: parcels"
    if bodies:
        got, wb = c.get_bodies(), ref[tag + "_bodies"]
        for f in records.MULTISPHERE.names:
            assert np.array_equal(got[f], wb[f]), f"{tag}: body {f}"
    assert np.array_equal(mrg.digest(*c.get_cell_lists()), ref[tag + "_cell_digest"]), f"{tag}: cell lists"
    assert np.array_equal(mrg.digest(*c.get_collision_lists()), ref[tag + "_pair_digest"]), f"{tag}: contact lists"
    if windows:
        w, cells = c.get_weights(len(parts))
        assert np.array_equal(mrg.digest(cells, w), ref[tag + "_window_digest"]), f"{tag}: interpolation windows"
    if fields:
        assert np.array_equal(mrg.field_digest(c.get_fluid()), ref[tag + "_field_digest"]), f"{tag}: fields"
    if tag + "_probe_force" in ref and len(ref[tag + "_probe_force"]):
        got = np.array([p["force"] for p in c.get_wall_probes()])
        assert np.array_equal(got, ref[tag + "_probe_force"]), f"{tag}: probe forces"


COMPACT = {
    "cylinders": "three cylinders from the reference's marker template in its own units (dx = 3.75e-5 m, "
                 "dt = 5e-5 s), two of them in contact",
    "corner": "two spheres between walls in x and z, one in the corner: wall contact on both walls, mirror "
              "images across each wall and across the corner, periodic images in y, a probe on each wall",
    "edge": "markers on cell corners and centres (the delta kernel's branch points) and at the contact "
            "cut-off distance, one ulp either side of it",
    "empty": "bodies without markers",
}


@pytest.mark.parametrize("name", sorted(COMPACT))
def test_compact_cases_match_the_reference(oracle_mod, name):
    """Fixtures stored as SHA-256 digests of every stage (bodies in full)."""
    ref = load(name)
    field = tuple(ref[f"in_{a}"].astype(np.float64) for a in "uvw")
    c = oracle_mod.OracleCase(ref["params"], ref["in_parcels"], ref["in_bodies"], field)
    if len(ref["in_probes"]):
        c.set_wall_probes(ref["in_probes"])
    c.InitializationDEM()
    compact_stage(ref, "init", c)
    for s in range(int(ref["steps"])):
        c.set_fluid(*field)
        c.MultiDirectForcing()
        compact_stage(ref, f"mdf{s}", c, fields=True)
        c.CloudEvolutionMS()
        compact_stage(ref, f"step{s}", c)
    parts, _ = c.get_parcels()
    assert np.array_equal(parts["x"], ref["final_x"]) and np.array_equal(parts["v"], ref["final_v"])
    c.close()


def test_compact_cases_exercise_what_they_claim():
    cyl, corner, edge, empty = (load(n) for n in ("cylinders", "corner", "edge", "empty"))
    assert int(cyl["init_npairs"]) > 0 and float(cyl["params"]["dx"]) == 9e-3 / 240
    assert int(corner["init_np"]) > int(corner["init_nlocal"]), "mirror and periodic images"
    assert (corner["step0_probe_force"][:, 0] > 0).any() or (corner["step0_probe_force"][:, 2] > 0).any()
    assert int(edge["init_npairs"]) >= 4, "the pairs at the cut-off"
    assert int(empty["init_np"]) == 0 and len(empty["init_bodies"]) == 2


def test_benchmark_configuration_matches_the_reference(oracle_mod):
    """The benchmark's CPU-runnable configuration (128^3 periodic, 64 spheres of
    d = 16h, 51,456 markers), regenerated from its seed: after
    InitializationDEM and the first forcing loop every parcel, list, window and
    field is bit-identical to the reference's; after CloudEvolutionMS every
    body's translation is, and the rotation of each body that does not straddle
    a periodic face (a straddling one takes the raw torque arm in the
    reference)."""
    ref = load("config")
    p, parts, bodies, field = mrg.config_case()
    assert int(ref["seed"]) == mrg.CONFIG_SEED
    assert np.array_equal(mrg.parcel_digest(parts, len(parts)), ref["in_parcel_digest"]), "regenerated parcels"
    assert np.array_equal(mrg.digest(*[bodies[f] for f in records.MULTISPHERE.names]), ref["in_body_digest"])
    assert np.array_equal(mrg.digest(*field), ref["in_field_digest"]), "regenerated field"
    c = oracle_mod.OracleCase(p, parts, bodies, field)
    c.InitializationDEM()
    compact_stage(ref, "init", c, bodies=False)
    c.set_fluid(*field)
    c.MultiDirectForcing()
    compact_stage(ref, "mdf0", c, fields=True, bodies=False)
    c.CloudEvolutionMS()
    got, want, far = c.get_bodies(), ref["step0_bodies"], ref["straddlers"]
    for f in ("x", "v", "vold", "fdrag", "fcol", "fhydro"):
        assert np.array_equal(got[f], want[f]), f"body {f}"
    for f in ("omega", "AngMom", "rotMat", "rotMatGlo", "fmom", "fmomCol", "fmomHydro"):
        assert np.array_equal(got[f][~far], want[f][~far]), f"body {f} (bodies inside the box)"
    assert 0 < far.sum() < len(far)
    c.close()


def test_cylinder_generation_matches_the_reference():
    """The reference's own InitCylinderParcelsDEM on the grid of its run (86
    cylinders, 96,750 markers from CYLINDER_LP1125.dat) against the cylinder
    generator of tests/golden/make_golden.py, which built the cylinder cases:
    every body record bit-identical here, the markers by their digests (the
    template is the reference's data, compared when the fixture was made)."""
    import make_golden

    ref = load("generation")
    want = ref["bodies"]
    got = make_golden.cylinder_bodies(want["x"], ref["rnd"], want["v"], float(ref["dx"]))
    for f in records.MULTISPHERE.names:
        assert np.array_equal(got[f], want[f]), f"body {f}"
    assert int(ref["np"]) == 86 * 1125
    assert np.array_equal(ref["generator_marker_digest"], ref["marker_digest"]), "markers"


def test_whole_time_step_matches_the_reference(oracle_mod):
    """The reference's FirstOrderForwardEuler (fluid.F90:252-327) as it stands,
    three steps on 16x12x16 between walls in y with two spheres in contact: the
    forcing loop, VelocityGuess, ModifyBulkVelocity, VelocityDivergence, the
    Poisson solve, PressureCorrection, VelocityCorrection (each with its halo
    refill) and CloudEvolutionMS, the fluid evolving.  The restatement's
    particle and fluid halves, chained in the same order with the same supplied
    Poisson solve (tests/fft_poisson.py), agree bit for bit after every step."""
    import fft_poisson

    ref = load("coupled")
    p = ref["params"]
    h = (float(p["dx"]), float(p["dy"]), float(p["dz"]))
    walls = str(ref["walls"])
    field = [ref[f"in_{a}"].astype(np.float64) for a in "uvw"]
    c = oracle_mod.OracleCase(p, ref["in_parcels"], ref["in_bodies"], field)
    F = oracle_mod.OracleFluid(p)
    F.set_fluid_params(float(ref["visc"]))
    b = ref["bulk"]
    FL = records.FLUID
    c.InitializationDEM()
    for s in range(int(ref["steps"])):
        u0 = field
        c.set_fluid(*u0)
        c.MultiDirectForcing()
        after = c.get_fluid()
        for k, name in enumerate(("u", "v", "w", "fx", "fy", "fz")):
            F.set_field(FL[name], after[k])
        for k, name in enumerate(("uold", "vold", "wold")):
            F.set_field(FL[name], u0[k])
        F.VelocityGuess(1.0, 0.0, 1.0)
        F.FillGhostRegionForFluid()
        F.Boundary()
        F.ModifyBulkVelocity(int(b[0]), int(b[1]), int(b[2]), b[3], b[4], b[5])
        F.FillGhostRegionForFluid()
        F.Boundary()
        F.VelocityDivergence(1.0)
        F.FillGhostRegionForFluid()
        F.Boundary()
        pc = F.get_field(FL["Pcorr"])
        pc[2:-2, 2:-2, 2:-2] = fft_poisson.solve(F.get_field(FL["velDiv"])[2:-2, 2:-2, 2:-2], h, walls)
        F.set_field(FL["Pcorr"], pc)
        F.PressureCorrection()
        F.FillGhostRegionForFluid()
        F.Boundary()
        F.VelocityCorrection(1.0)
        F.FillGhostRegionForFluid()
        F.Boundary()
        c.CloudEvolutionMS()
        parts, nl = c.get_parcels()
        assert nl == int(ref[f"step{s}_nlocal"]), s
        assert np.array_equal(mrg.parcel_digest(parts, nl), ref[f"step{s}_parcel_digest"]), f"step {s}: parcels"
        got, want = c.get_bodies(), ref[f"step{s}_bodies"]
        for f in records.MULTISPHERE.names:
            assert np.array_equal(got[f], want[f]), f"step {s}: body {f}"
        for f in mrg.COUPLED_FIELDS:
            a = F.get_field(FL[f])
            if f in ("fx", "fy", "fz"):
                a = a[2:-2, 2:-2, 2:-2]
            assert np.array_equal(digest(a), ref[f"step{s}_{f}"]), f"step {s}: {f}"
        field = [F.get_field(FL[a]) for a in "uvw"]
    c.close()
    F.close()


def test_output_files_hold_the_reference_values(tmp_path):
    """The library's host writers against the reference's own output routines
    after one coupled step: the marker file of OutputCloudTecplot
    (ZJS_IO_DEM.F90:82-121) and the per-body probe lines of PostProcessing
    (fluid.F90:392-397) hold the same records and, read back from their 17
    significant digits, exactly the values the reference writes (the body
    accelerations fdrag/m*rhof, fmom/I*rhof and fcol/m formed as it forms
    them)."""
    from ibmdem import api

    ref = load("output")
    path = tmp_path / "Particle_1_0.dat"
    api.write_tecplot_markers(path, ref["parcels"])
    lines = path.read_text().splitlines()
    assert [" ".join(x.split()) for x in lines[:2]] == list(ref["marker_header"])
    rows = np.array([[float(t) for t in x.split()] for x in lines[2:]])
    assert np.array_equal(rows, ref["marker_rows"])
    api.write_body_probes(tmp_path, int(ref["step"]), ref["bodies"], float(ref["rhof"]))
    for k, i in enumerate(ref["probe_ids"]):
        line = (tmp_path / f"{i}.probe").read_text().splitlines()
        assert len(line) == 1
        assert np.array_equal(np.array([float(t) for t in line[0].split()]), ref["probe_rows"][k]), i


@pytest.mark.parametrize("name", ["poisson_walls_y", "poisson_periodic"])
def test_pressure_system_matches_the_reference(oracle_mod, name):
    """The pressure-correction matrix the restatement applies (the system the
    library's Poisson solve is checked against) equals, entry for entry, the
    one the reference's SetPressureCorrectionJacobian assembles through
    MatSetValues (poisson.F90:46-105), pinned row included; and the reference's
    SetPressureVector right-hand side is the divergence with the pinned entry
    set to zero."""
    ref = load(name)
    p = ref["params"]
    n = int(p["nx"]) * int(p["ny"]) * int(p["nz"])
    A = np.zeros((n, n))
    A[ref["rows"], ref["cols"]] = ref["vals"]
    F = oracle_mod.OracleFluid(p)
    got = np.zeros((n, n))
    inner = (int(p["nz"]), int(p["ny"]), int(p["nx"]))
    for c in range(n):
        unit = np.zeros(n)
        unit[c] = 1.0
        e = np.zeros(F.shape)
        e[2:-2, 2:-2, 2:-2] = unit.reshape(inner)
        got[:, c] = F.PressureOperator(e)[2:-2, 2:-2, 2:-2].reshape(-1)
    F.close()
    assert np.array_equal(got, A)
    want = ref["velDiv"][2:-2, 2:-2, 2:-2].reshape(-1).copy()
    want[0] = 0.0
    assert np.array_equal(ref["rhs"], want)


def test_hundred_step_trajectory_matches_the_reference(oracle_mod):
    """One hundred coupled steps of the periodic case (three spheres, one
    contact, images on four faces; two DEM sub-steps a step): after every step
    the bodies, the parcels and the forcing loop's fields are bit-identical to
    the reference's."""
    ref = load("trajectory")
    field = (ref["in_u"], ref["in_v"], ref["in_w"])
    c = oracle_mod.OracleCase(ref["params"], ref["in_parcels"], ref["in_bodies"], field)
    c.InitializationDEM()
    for s in range(int(ref["steps"])):
        c.set_fluid(*field)
        c.MultiDirectForcing()
        assert np.array_equal(mrg.field_digest(c.get_fluid()), ref["field_digest"][s]), f"step {s}: fields"
        c.CloudEvolutionMS()
        parts, nl = c.get_parcels()
        assert np.array_equal(mrg.parcel_digest(parts, nl), ref["parcel_digest"][s]), f"step {s}: parcels"
        got = c.get_bodies()
        for f in records.MULTISPHERE.names:
            assert np.array_equal(got[f], ref["bodies"][s][f]), f"step {s}: body {f}"
    assert ref["npairs"].min() > 0
    c.close()


def test_pins_catch_planted_mistakes(oracle_mod):
    """The comparisons are not vacuous: a restatement with ModifyBulkVelocity
    left out fails the whole-time-step pin, and one parcel moved by one ulp
    fails the periodic case at its first stage."""
    import types

    class NoBulk(oracle_mod.OracleFluid):
        def ModifyBulkVelocity(self, *args):
            pass

    with pytest.raises(AssertionError):
        test_whole_time_step_matches_the_reference(types.SimpleNamespace(OracleCase=oracle_mod.OracleCase,
                                                                         OracleFluid=NoBulk))

    class Nudged(oracle_mod.OracleCase):
        def __init__(self, params, parcels=None, bodies=None, field=None):
            parcels = np.array(parcels, copy=True)
            parcels["x"][5, 0] = np.nextafter(parcels["x"][5, 0], np.inf)
            super().__init__(params, parcels, bodies, field)

    with pytest.raises(AssertionError, match="init"):
        test_coupled_steps_match_the_reference(types.SimpleNamespace(OracleCase=Nudged), "periodic")


@pytest.mark.parametrize("name", ["multirank", "multirank_straddle", "multirank_corner"])
def test_one_rank_restatement_matches_the_reference_on_two_ranks(oracle_mod, name):
    """The restatement keeps the reference's multi-rank body semantics on one
    rank.  Against the reference's own multi-rank code on two ranks (threads
    sharing a translated MPI; tests/golden/ref_multirank.npz: a body straddling
    the ranks' seam, one touching it from the other rank, bodies and parcels
    exchanged as ghosts with the periodic shift), two coupled steps agree to
    1e-13 of each quantity's largest value: the ranks sum a node's forcing and
    a body's forces in their own order (measured: 4e-15 at most), while the
    body positions come out bit-identical (on two ranks the rotations and
    contact forces too).  ref_multirank_corner.npz splits x and z over 2x1x2
    ranks, as the reference's own run splits them 4x1x4, with a body on the
    corner where the four ranks meet.
    ref_multirank_straddle.npz has a body straddling the periodic x face: there
    the one-rank reference takes a torque arm a box length long, while on two
    ranks the body reaches its far markers' rank as a ghost shifted by the box
    length, which is the nearest-image arm the restatement uses."""
    import cases

    ref = load(name)
    field = [ref[f"in_{a}"].astype(np.float64) for a in "uvw"]
    c = oracle_mod.OracleCase(ref["params"], ref["in_parcels"], ref["in_bodies"], field)
    c.InitializationDEM()
    key = lambda a: a["MSIdx"].astype(np.int64) * 1000000 + a["globalIdx"]  # noqa: E731
    for s in range(int(ref["steps"])):
        c.set_fluid(*field)
        c.MultiDirectForcing()
        got = c.get_fluid()
        assert cases.rel_close(got[0][2:-2, 2:-2, 2:-2], ref[f"step{s}_u"], 1e-13), f"step {s}: u"
        assert cases.rel_close(got[3][2:-2, 2:-2, 2:-2], ref[f"step{s}_fx"], 1e-13), f"step {s}: fx"
        c.CloudEvolutionMS()
        bodies, want = c.get_bodies(), ref[f"step{s}_bodies"]
        assert np.array_equal(bodies["globalIdx"], want["globalIdx"])
        for f in ("x", "v", "omega", "AngMom", "rotMatGlo", "fdrag", "fcol", "fmom", "fmomCol"):
            assert cases.rel_close(bodies[f], want[f], 1e-13), f"step {s}: body {f}"
        exact = ("x", "omega", "AngMom", "fcol", "fmomCol") if int(np.prod(ref["cpus"])) == 2 else ("x",)
        for f in exact:
            assert np.array_equal(bodies[f], want[f]), f"step {s}: body {f} bit for bit"
        parts, nl = c.get_parcels()
        parts = parts[:nl][np.argsort(key(parts[:nl]))]
        assert np.array_equal(parts["MSIdx"], ref[f"step{s}_parcel_MSIdx"])
        assert np.array_equal(parts["globalIdx"], ref[f"step{s}_parcel_globalIdx"])
        for f in ("x", "v", "fdrag", "fcol"):
            assert cases.rel_close(parts[f], ref[f"step{s}_parcel_{f}"], 1e-13), f"step {s}: parcel {f}"
    assert (ref["step0_ranks"] > 0).all() and len(ref["step0_ranks"]) == int(np.prod(ref["cpus"]))
    c.close()


def test_walled_case_exercises_wall_contact():
    ref = load("walled")
    f = ref["step0_probe_force"]
    assert f[0][2] > 0 and not f[1].any(), "one probe under the body, one beside it"
    assert list(ref["params"]["bType"]) == [0, 0, 0, 0, 1, 1]


@pytest.mark.parametrize("name", ["fluid_walls_y", "fluid_periodic"])
def test_fluid_stencils_match_the_reference(oracle_mod, name):
    ref = load(name)
    F = oracle_mod.OracleFluid(ref["params"])
    for f in mrg.FLUID_INPUTS:
        F.set_field(records.FLUID[f], ref["in_" + f])
    F.set_fluid_params(float(ref["visc"]))
    b = ref["bulk"]
    for stage, calls, written in mrg.FLUID_STAGES:
        for call in calls:
            if call[0] == "ModifyBulkVelocity":
                F.ModifyBulkVelocity(int(b[0]), int(b[1]), int(b[2]), b[3], b[4], b[5])
            else:
                getattr(F, call[0])(*call[1:])
        for f in written:
            assert np.array_equal(digest(F.get_field(records.FLUID[f])), ref[f"{stage}_{f}"]), f"{stage}: {f}"
    F.close()


def test_runge_kutta_fluid_step_matches_the_reference(oracle_mod):
    """The reference's ThirdOrderLowStorageRungeKutta (fluid.F90:329-366), walls
    in z: VelocityGuess with the kept right-hand side (bRK != 0), the divergence
    and the corrections scaled by cRK = aRK + bRK, each stage's Poisson solve
    replaced by a given correction."""
    ref = load("fluid_rk3_walls_z")
    F = oracle_mod.OracleFluid(ref["params"])
    for f in mrg.FLUID_INPUTS:
        F.set_field(records.FLUID[f], ref["in_" + f])
    F.set_fluid_params(float(ref["visc"]))
    aRK = [32.0 / 60.0, 25.0 / 60.0, 45.0 / 60.0]
    bRK = [0.0, -17.0 / 60.0, -25.0 / 60.0]
    for k in range(3):
        cRK = aRK[k] + bRK[k]
        F.VelocityGuess(aRK[k], bRK[k], cRK)
        F.FillGhostRegionForFluid()
        F.Boundary()
        F.VelocityDivergence(cRK)
        F.FillGhostRegionForFluid()
        F.Boundary()
        for f in ("u", "v", "w", "velDiv"):
            assert np.array_equal(digest(F.get_field(records.FLUID[f])), ref[f"rk{k}_{f}"]), f"stage {k}: {f}"
        F.set_field(records.FLUID["Pcorr"], ref[f"in_pcorr{k}"])
        F.PressureCorrection()
        F.FillGhostRegionForFluid()
        F.Boundary()
        F.VelocityCorrection(cRK)
        F.FillGhostRegionForFluid()
        F.Boundary()
    for f in mrg.RK3_WRITTEN:
        assert np.array_equal(digest(F.get_field(records.FLUID[f])), ref[f"end_{f}"]), f
    F.close()


def test_drag_law_matches_the_reference(oracle_mod):
    ref = load("drag")
    for i in range(len(ref["rho"])):
        beta = oracle_mod.drag_beta(ref["rho"][i], ref["rad"][i], ref["v"][i], ref["denf"][i], ref["alphaf"][i],
                                    ref["velf"][i])
        assert np.array_equal(beta, ref["beta"][i]), i


@pytest.mark.skipif(not os.environ.get("IBMDEM_REFERENCE_DIR"), reason="IBMDEM_REFERENCE_DIR (the reference's "
                    "Fortran sources) not set")
def test_fixtures_reproduce_from_the_reference_sources():
    """With the reference's sources at hand, the translator reproduces the stored
    fixtures byte for byte (the edge, empty and drag ones, which take seconds)."""
    sources = mrg.load_sources(os.environ["IBMDEM_REFERENCE_DIR"])
    for name, job in (("edge", lambda: mrg.run_compact(sources, *mrg.edge_case(), 3)),
                      ("empty", lambda: mrg.run_compact(sources, *mrg.empty_case(), 2)),
                      ("drag", lambda: mrg.run_drag(sources, 9))):
        new, old = job(), load(name)
        assert sorted(new) == sorted(old), name
        for k in old:
            assert np.array_equal(np.asarray(new[k]), old[k]), f"{name}: {k}"
