"""Golden fixtures from the reference's own subroutines (tests/golden/ref_*.npz).

The reference's Fortran is read from the source directory given on the command
line and executed through fortran_subset.py on one MPI rank.  Each case is
advanced by the reference's particle-side subroutines, and the state after
every stage is stored: parcels, bodies, the fluid fields, the per-cell parcel
lists and the contact lists.  tests/test_reference_pins.py replays the same
stages on the C restatement in oracle/ (bit for bit) and
tests/test_gpu_reference_pins.py on the CUDA library.

What the harness supplies instead of the reference (each a configuration the
reference hard-codes or a step it takes on several ranks only):
  * the case: grid size, boundary types (SetBoundaryType,
    initialization.F90:317-351, fixes them), dt and rhof (GridInitialization),
    knCoeff, ResistCoeff and coupleInterval (InitParameters), collisionDist,
    the parcels, bodies and wall probes (InitCylinderParcelsDEM and
    SetWallProbe, ZJS_INIT_DEM.F90:369-509), all set in the reference's module
    variables after the routine that would have set them;
  * the multi-rank body exchange: on one rank CloudEvolutionStepMS integrates
    only body 1 (couplesolverCylinder.F90:114-121,130), so for more than one
    body (the single-body case runs that one-rank path unchanged) the harness runs its
    multi-rank branch, with the two steps that ranks exchange for replaced by
    their one-rank result: AssembleForceMS is AssembleLocalForceMS followed by
    its own copy from MSGlo into MS (ZJS_MS_DEM.F90:417-422), and
    UpdateMSInfoInGhostRegion is its own copy from MS into MSGlo
    (ZJS_MS_DEM.F90:165-167);
  * the frozen fluid: each step starts from the case's u, v, w (halo refilled
    by FillGhostRegionForFluid and Boundary), then runs the forcing loop of
    FirstOrderForwardEuler (fluid.F90:256-280) and CloudEvolutionMS.
Bodies never straddle a periodic face in these cases: there the reference's
raw body-relative vector and the nearest-image one of the library agree.

Usage: python tests/golden/make_reference_golden.py <reference source dir> [fixture names] [--check-bounds]
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(HERE)), "ibm-dem_gb300"))

import fortran_subset as fs  # noqa: E402
from ibmdem import scenario  # noqa: E402
from ibmdem.records import MULTISPHERE, PARCEL, WALL_PROBE, field_shape, make_params  # noqa: E402

# the makefile's sources, less the main program, the PETSc Poisson solve and the fluid's file output
SOURCES = ["vars.F90", "ZJS_VARS.F90", "boundary.F90", "initialization.F90", "allocate.F90", "fluid.F90",
           "interpolation.F90", "ZJS_AUXILIARY_DEM.F90", "ZJS_COLLISION_DEM.F90", "ZJS_DRAGFORCE_DEM.F90",
           "ZJS_EVOLUTION_DEM.F90", "ZJS_INIT_DEM.F90", "ZJS_INTERPOLATE_DEM.F90", "ZJS_MPI_DEM.F90",
           "ZJS_UPDATE_LIST_DEM.F90", "ZJS_VOLUMEFRACTION_DEM.F90", "ZJS_MS_DEM.F90",
           "couplesolverCylinder.F90", "ZJS_IO_DEM.F90"]
# maxPartNo sizes neighCellWeight(125, maxPartNo, 3): 100000 would take 300 MB for cases of a few thousand
CAPACITIES = {"maxpartno": 8000}
# --check-bounds on the command line checks every subscript of the reference's statements against its extent
CHECK_BOUNDS = False


def load_sources(ref_dir):
    return [(f, open(os.path.join(ref_dir, f)).read()) for f in SOURCES]


class ReferenceCase:
    """One case held by the reference's translated subroutines."""

    def __init__(self, sources, p, parts, bodies, field, probes=None, one_rank_bodies=False, capacities=None):
        """`one_rank_bodies` keeps the reference's own one-rank body update
        (defined for a single body) instead of its multi-rank branch."""
        self.p = p
        self.T = fs.Translator(sources, capacities or CAPACITIES, CHECK_BOUNDS)
        overrides = {"setboundarytype": self._set_boundary_type}
        if not one_rank_bodies:
            overrides.update({"assembleforcems": self._assemble_force_ms,
                              "cloudevolutionstepms": self._cloud_evolution_step_ms})
        else:
            assert len(bodies) == 1, "the one-rank body update integrates body 1 only"
        self.T.build(overrides=overrides)
        self.G = G = self.T.new_state()
        c = self.call
        n = [int(p["nx"]), int(p["ny"]), int(p["nz"])]
        h = [float(p["dx"]), float(p["dy"]), float(p["dz"])]
        assert float(p["collisionBuffer"]) == 0.1, "collisionBuffer is a parameter of the reference"
        assert list(p["gravity"]) == [0.0, 0.0, -9.81], "the reference's gravity"
        c("PartitionInitialization", 1, 1, 1, n[0], n[1], n[2], n[0] * h[0], n[1] * h[1], n[2] * h[2])
        assert (G.m_dx, G.m_dy, G.m_dz) == tuple(h), "grid spacing"
        c("GridInitialization")
        G.m_dt, G.m_rhof = float(p["dt"]), float(p["rhof"])
        c("SetCellIndexMap")
        c("BuildMPIRecvAndSendIndexForFluid")
        # InitializationDEM (ZJS_INIT_DEM.F90:2-37), the case in place of InitCylinderParcelsDEM
        c("InitParameters")
        G.m_kncoeff, G.m_resistcoeff = float(p["knCoeff"]), float(p["ResistCoeff"])
        G.m_coupleinterval = int(p["coupleInterval"])
        G.m_dtdem = G.m_dt / G.m_coupleinterval
        for name in ("CopyGridInformationDEM", "AllocateDEM", "SetCellType", "SetCellIndexMapDEM",
                     "SetNeighCellIndexForCellsDEM", "SetBoundaryNormsAndPoints", "SetMirrorAndShiftCoords"):
            c(name)
        G.m_collisiondist = float(p["collisionDist"])
        self._load_parcels(parts)
        self._load_bodies(bodies)
        G.m_nppartincell.a[:] = 0
        c("PutParcelsIntoCellsDEM", 1, G.m_np, 0)
        self._load_probes(probes)
        self.set_field(field)
        self.u0 = [G.m_u.a.copy(), G.m_v.a.copy(), G.m_w.a.copy()]
        for name in ("RebuildParcelInCellListDEM", "RebuildParcelCollisionListDEM",
                     "RebuildNeighborCellListForParcelsDEM", "UpdateLocalCellWeightListDEM",
                     "UpdateParcelInfoInGhostRegion", "UpdateGhostCellWeightListDEM"):
            c(name)

    def call(self, name, *args):
        return self.T.call(self.G, name, *args)

    # harness replacements ---------------------------------------------------
    def _set_boundary_type(self, G):
        bt = [int(b) for b in self.p["bType"]]
        G.m_bw, G.m_be, G.m_bb, G.m_bf, G.m_bs, G.m_bn = bt
        G.m_bwg, G.m_beg, G.m_bbg, G.m_bfg, G.m_bsg, G.m_bng = bt
        G.m_btype.a[:] = bt
        return ()

    def _assemble_force_ms(self, G):
        self.call("AssembleLocalForceMS")
        for i in range(G.m_nmslocal):
            g = int(G.m_ms.a["globalidx"][i]) - 1
            for f in ("fcol", "fmom", "fmomcol", "fdrag"):
                G.m_ms.a[f][i] = G.m_msglo.a[f][g]
        return ()

    def _cloud_evolution_step_ms(self, G):
        c = self.call
        c("CalculateCollisionForce")
        c("CalculateSolidBoundaryCollisionForce")
        c("AssembleForceMS")
        c("EvolutionMS")
        for i in range(G.m_nms):
            G.m_msglo.a[int(G.m_ms.a["globalidx"][i]) - 1] = G.m_ms.a[i]
        for name in ("ResetVelocityAndPositionLagrangianPoints", "AdjustParcelPosition",
                     "UpdateParcelInfoInGhostRegion", "RebuildAllListOrNot", "UpdateLocalCellWeightListDEM",
                     "UpdateParcelInfoInGhostRegion", "UpdateGhostCellWeightListDEM"):
            c(name)
        return ()

    # state in and out -------------------------------------------------------
    def _load_parcels(self, parts):
        G = self.G
        n = len(parts)
        for f in PARCEL.names:
            if f != "pad_":
                G.m_part.a[f.lower()][:n] = parts[f]
        G.m_np = G.m_nplocal = n

    def _load_bodies(self, bodies):
        G = self.G
        n = len(bodies)
        for f in MULTISPHERE.names:
            G.m_ms.a[f.lower()][:n] = bodies[f]
            G.m_msglo.a[f.lower()][:n] = bodies[f]
        G.m_nms = G.m_nmslocal = G.m_nmsglo = n

    def _load_probes(self, probes):
        G = self.G
        G.m_numwallprobe.a[:] = 0
        if probes is None:
            return
        for pr in probes:
            face = int(pr["face"])
            G.m_numwallprobe.a[face - 1] += 1
            k = int(G.m_numwallprobe.a[face - 1]) - 1
            G.m_wallprobe.a["points"][k, face - 1] = np.asarray(pr["points"]).T
            G.m_wallprobe.a["force"][k, face - 1] = 0.0

    def set_field(self, field):
        G = self.G
        for arr, f in zip((G.m_u, G.m_v, G.m_w), field):
            arr.a[...] = np.asarray(f, dtype=np.float64).reshape(field_shape(self.p)).T
        self.call("FillGhostRegionForFluid")
        self.call("Boundary")

    def parcels(self):
        G = self.G
        out = np.zeros(G.m_np, PARCEL)
        for f in PARCEL.names:
            if f != "pad_":
                out[f] = G.m_part.a[f.lower()][:G.m_np]
        return out

    def bodies(self):
        G = self.G
        out = np.zeros(G.m_nms, MULTISPHERE)
        for f in MULTISPHERE.names:
            out[f] = G.m_ms.a[f.lower()][:G.m_nms]
        return out

    def fields(self):
        G = self.G
        return [a.a.T.copy() for a in (G.m_u, G.m_v, G.m_w, G.m_fx, G.m_fy, G.m_fz)]

    def cell_lists(self):
        """CSR over the haloed grid's cells in 1D index order; 1-based parcel indices."""
        G = self.G
        cnt = G.m_nppartincell.a.astype(np.int64)
        start = np.zeros(len(cnt) + 1, np.int64)
        np.cumsum(cnt, out=start[1:])
        items = np.concatenate([G.m_partidxincell.a[:c, k] for k, c in enumerate(cnt)]) if cnt.sum() else \
            np.zeros(0, np.int32)
        return start.astype(np.int32), items.astype(np.int32)

    def collision_lists(self):
        G = self.G
        nl = G.m_nplocal
        cnt = G.m_neighpartno.a[:nl].astype(np.int64)
        start = np.zeros(nl + 1, np.int64)
        np.cumsum(cnt, out=start[1:])
        items = np.concatenate([G.m_neighpartidx.a[:c, k] for k, c in enumerate(cnt)]) if cnt.sum() else \
            np.zeros(0, np.int32)
        return start.astype(np.int32), items.astype(np.int32)

    def probe_forces(self):
        G = self.G
        out = []
        for face in range(6):
            for k in range(int(G.m_numwallprobe.a[face])):
                out.append(G.m_wallprobe.a["force"][k, face].copy())
        return np.array(out).reshape(-1, 3)

    # the coupled step on a frozen fluid ----------------------------------------
    def multi_direct_forcing(self):
        """The forcing loop of FirstOrderForwardEuler (fluid.F90:258-280)."""
        G = self.G
        for a, a0 in zip((G.m_u, G.m_v, G.m_w), self.u0):
            a.a[...] = a0
        G.m_part.a["fdrag"][:G.m_nplocal] = 0.0
        G.m_fx.a[...] = 0.0
        G.m_fy.a[...] = 0.0
        G.m_fz.a[...] = 0.0
        for _ in range(int(self.p["Ns"])):
            for name in ("UpdateFluidVelocityOnLagrangianPoints", "UpdateParcelInfoInGhostRegion",
                         "UpdateMomentumSourceTerm", "VelocityPostGuess", "FillGhostRegionForFluid", "Boundary"):
                self.call(name)

    def cloud_evolution(self):
        self.call("CloudEvolutionMS")

    def weights(self):
        """Every parcel's window cells and delta weights, as (np, 125[, 3]),
        zero past its neighCellNo entries."""
        G = self.G
        n = G.m_np
        cnt = G.m_neighcellno.a[:n]
        used = np.arange(125)[None, :] < cnt[:, None]
        cells = np.where(used, G.m_neighcellidx.a[:, :n].T, 0).astype(np.int32)
        w = np.where(used[..., None], G.m_neighcellweight.a[:, :n, :].transpose(1, 0, 2), 0.0)
        return cnt.astype(np.int32), cells, np.ascontiguousarray(w)

    def snapshot(self):
        s = {"parcels": self.parcels(), "nlocal": np.int32(self.G.m_nplocal), "bodies": self.bodies()}
        s["cell_start"], s["cell_items"] = self.cell_lists()
        s["pair_start"], s["pair_items"] = self.collision_lists()
        s["probe_force"] = self.probe_forces()
        cnt, cells, w = self.weights()
        s["window_count"] = cnt
        s["window_digest"] = digest(cells, w)
        return s


class ReferenceFluid:
    """The reference's fluid stencils on one rank (fluid.F90, boundary.F90)."""

    def __init__(self, sources, p, visc, extra=None):
        self.p = p
        self.T = fs.Translator(sources, CAPACITIES, CHECK_BOUNDS)
        overrides = {"setboundarytype": lambda G: ReferenceCase._set_boundary_type(self, G)}
        overrides.update(extra or {})
        self.T.build(overrides=overrides)
        self.G = G = self.T.new_state()
        n = [int(p["nx"]), int(p["ny"]), int(p["nz"])]
        h = [float(p["dx"]), float(p["dy"]), float(p["dz"])]
        self.call("PartitionInitialization", 1, 1, 1, n[0], n[1], n[2], n[0] * h[0], n[1] * h[1], n[2] * h[2])
        self.call("GridInitialization")
        G.m_dt, G.m_rhof, G.m_visc = float(p["dt"]), float(p["rhof"]), float(visc)
        self.call("SetCellIndexMap")
        self.call("BuildMPIRecvAndSendIndexForFluid")

    def call(self, name, *args):
        return self.T.call(self.G, name, *args)

    def set(self, name, a):
        getattr(self.G, "m_" + name.lower()).a[...] = np.asarray(a, dtype=np.float64).reshape(
            field_shape(self.p)).T

    def get(self, name):
        return getattr(self.G, "m_" + name.lower()).a.T.copy()


# the fluid step of FirstOrderForwardEuler after the forcing loop (fluid.F90:256,281-324), the Poisson
# solve (SetPressureVector, PoissonSolver) replaced by a given pressure correction; each stage with the
# fields it writes
FLUID_STAGES = [
    ("guess", [("StoreOldVelocity",), ("VelocityGuess", 1.0, 0.0, 1.0), ("FillGhostRegionForFluid",),
               ("Boundary",)], ["u", "v", "w", "uold", "vold", "wold", "RHSul", "RHSvl", "RHSwl", "Px", "Py", "Pz"]),
    ("bulk", [("ModifyBulkVelocity",), ("FillGhostRegionForFluid",), ("Boundary",)], ["u", "v", "w"]),
    ("divergence", [("VelocityDivergence", 1.0), ("FillGhostRegionForFluid",), ("Boundary",)], ["velDiv"]),
    ("pressure", [("PressureCorrection",), ("FillGhostRegionForFluid",), ("Boundary",)], ["P", "Pcorr"]),
    ("correction", [("VelocityCorrection", 1.0), ("FillGhostRegionForFluid",), ("Boundary",)],
     ["u", "v", "w", "omegaX", "omegaY", "omegaZ"]),
]
FLUID_INPUTS = ["u", "v", "w", "fx", "fy", "fz", "P", "Pcorr", "RHSul", "RHSvl", "RHSwl"]


def run_fluid(sources, name, p, visc, seed):
    """Random fields through FLUID_STAGES; the digest of every written field after every stage."""
    import hashlib
    rng = np.random.default_rng(seed)
    R = ReferenceFluid(sources, p, visc)
    out = {"params": np.asarray(p), "visc": np.float64(visc)}
    for f in FLUID_INPUTS:
        a = rng.standard_normal(field_shape(p)) * (1e3 if f in ("P", "Pcorr") else 0.1)
        out["in_" + f] = a
        R.set(f, a)
    # the bulk-velocity switches and targets GridInitialization sets (initialization.F90:262-264)
    G = R.G
    out["bulk"] = np.array([G.m_defavebulkuswitch, G.m_defavebulkvswitch, G.m_defavebulkwswitch,
                            G.m_bulku, G.m_bulkv, G.m_bulkw], dtype=np.float64)
    for stage, calls, written in FLUID_STAGES:
        for c in calls:
            if c[0] == "StoreOldVelocity":
                for a in "uvw":
                    getattr(G, f"m_{a}old").a[...] = getattr(G, f"m_{a}").a
                continue
            R.call(*c)
        for f in written:
            out[f"{stage}_{f}"] = np.frombuffer(hashlib.sha256(R.get(f).tobytes()).digest(), np.uint8)
    print(f"{name}: fluid stages done", flush=True)
    return out


def digest(*arrays):
    """SHA-256 of the arrays' bytes, in order."""
    import hashlib
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return np.frombuffer(h.digest(), np.uint8)


# image slots hold only what MyMPIUpdateVelocityAndPosition sends (ZJS_MPI_DEM.F90:102-170)
IMAGE_FIELDS = ("globalIdx", "cellIdx", "pType", "MSIdx", "radeff", "rad", "rho", "vol", "m", "x", "v", "fdrag")


def parcel_digest(parts, nl):
    """Every parcel field the reference defines: all of a local's, an image's IMAGE_FIELDS."""
    cols = [parts[f][:nl] for f in PARCEL.names if f != "pad_"] + [parts[f][nl:] for f in IMAGE_FIELDS]
    return digest(*cols)


def field_digest(fields):
    """u, v, w with their halo; fx, fy, fz on the interior (the reference discards their halo)."""
    return digest(*fields[:3], *[f[2:-2, 2:-2, 2:-2] for f in fields[3:]])


def run_drag(sources, seed, n=400):
    """CalculateDragForce (ZJS_DRAGFORCE_DEM.F90:2-35) on random parcels and
    fluid states covering both Reynolds-number branches, the Rep >= 1 clamp and
    both voidage branches."""
    rng = np.random.default_rng(seed)
    T = fs.Translator(sources, CAPACITIES, CHECK_BOUNDS)
    T.build()
    G = T.new_state()
    rho = rng.uniform(500.0, 3000.0, n)
    rad = 10.0 ** rng.uniform(-5.0, -2.0, n)
    vp = rng.standard_normal((n, 3)) * 10.0 ** rng.uniform(-4.0, 0.5, (n, 1))
    denf = rng.uniform(800.0, 1200.0, n)
    alphaf = rng.uniform(0.3, 1.0, n)
    alphaf[:20] = np.float32(0.8)  # at the single-precision literal of the voidage branch
    velf = vp + rng.standard_normal((n, 3)) * 10.0 ** rng.uniform(-6.0, 0.5, (n, 1))
    beta = np.zeros((n, 3))
    for i in range(n):
        G.m_part.a["rho"][0], G.m_part.a["rad"][0] = rho[i], rad[i]
        G.m_part.a["v"][0] = vp[i]
        b = np.zeros(3)
        T.call(G, "CalculateDragForce", 1, float(denf[i]), float(alphaf[i]), velf[i].copy(), b)
        beta[i] = b
    return {"rho": rho, "rad": rad, "v": vp, "denf": denf, "alphaf": alphaf, "velf": velf, "beta": beta}


RK3_WRITTEN = ["u", "v", "w", "RHSul", "RHSvl", "RHSwl", "Px", "Py", "Pz", "velDiv", "P", "Pcorr", "omegaX",
               "omegaY", "omegaZ"]


def run_fluid_rk3(sources, name, p, visc, seed):
    """The reference's ThirdOrderLowStorageRungeKutta (fluid.F90:329-366) as it
    stands, its Poisson solve (SetPressureVector, PoissonSolver) replaced by a
    given pressure correction per stage; digests of the velocity and the
    divergence where each stage's solve would start, and of every written
    field at the end."""
    rng = np.random.default_rng(seed)
    pcorr = [rng.standard_normal(field_shape(p)) * 1e3 for _ in range(3)]
    out = {"params": np.asarray(p), "visc": np.float64(visc)}
    hook = {"stage": 0}
    R = None

    def poisson(G):
        k = hook["stage"]
        for f in ("u", "v", "w", "velDiv"):
            out[f"rk{k}_{f}"] = digest(R.get(f))
        R.set("Pcorr", pcorr[k])
        hook["stage"] += 1
        return ()

    R = ReferenceFluid(sources, p, visc, extra={"setpressurevector": lambda G: (), "poissonsolver": poisson})
    for f in FLUID_INPUTS:
        a = rng.standard_normal(field_shape(p)) * (1e3 if f in ("P", "Pcorr") else 0.1)
        out["in_" + f] = a
        R.set(f, a)
    for k in range(3):
        out[f"in_pcorr{k}"] = pcorr[k]
    R.call("ThirdOrderLowStorageRungeKutta")
    assert hook["stage"] == 3
    for f in RK3_WRITTEN:
        out[f"end_{f}"] = digest(R.get(f))
    print(f"{name}: three Runge-Kutta stages done", flush=True)
    return out


# ----------------------------------------------------------------------------
# the cases


def _interior(p, a):
    return np.asarray(a)[2:-2, 2:-2, 2:-2]


def periodic_case():
    """Three spheres of 6 cells on 16^3, periodic: bodies 1 and 2 in contact,
    markers within the two-cell image band of four faces, no body straddling
    a face."""
    n, d = 16, 6.0
    p, parts, bodies, field = scenario.resolved_case(n, n, n, 1, d, seed=11, n_modes=6, vel_std=0.02,
                                                    coupleInterval=2, knCoeff=1e4, ResistCoeff=0.9)
    X = np.array([[4.4, 5.0, 6.5], [4.4 + d + 0.35, 5.4, 6.2], [8.2, 11.6, 12.1]])
    V = np.array([[0.02, -0.01, 0.005], [-0.02, 0.01, 0.0], [0.0, 0.015, -0.01]])
    parts, bodies = scenario.sphere_bodies(X, d, 1.0, 1.14e3, V)
    return "periodic", p, parts, bodies, field, None


def walled_case():
    """Two spheres of 6 cells on 14x14x16 with solid walls in z: body 1 a
    quarter cell from the low wall (wall contact, one probe covering its
    footprint and one beside it), body 2 touching body 1."""
    n, d = 14, 6.0
    p, parts, bodies, field = scenario.resolved_case(n, n, 16, 1, d, seed=5, n_modes=6, vel_std=0.02,
                                                    coupleInterval=2, knCoeff=1e4, ResistCoeff=0.9, walls="z")
    scenario.fill_halo(p, field)
    X = np.array([[6.6, 7.1, 3.2], [6.6 + d + 0.3, 7.3, 3.5]])
    V = np.array([[0.0, 0.01, -0.03], [-0.01, 0.0, 0.0]])
    parts, bodies = scenario.sphere_bodies(X, d, 1.0, 1.14e3, V)
    probes = np.zeros(2, WALL_PROBE)
    probes["face"] = 5
    probes[0]["points"] = [[4, 5, 0], [9, 5, 0], [9, 9, 0], [4, 9, 0]]
    probes[1]["points"] = [[10, 1, 0], [13, 1, 0], [13, 4, 0], [10, 4, 0]]
    return "walled", p, parts, bodies, field, probes


def single_case():
    """One sphere of 8 cells on 16x14x18, periodic, markers in the image band of
    three faces: the reference's own one-rank CloudEvolutionStepMS
    (couplesolverCylinder.F90:99-187, ncputot == 1) runs unchanged."""
    d = 8.0
    p, parts, bodies, field = scenario.resolved_case(16, 14, 18, 1, d, seed=17, n_modes=6, vel_std=0.02,
                                                    coupleInterval=3, knCoeff=1e4, ResistCoeff=0.9)
    X = np.array([[5.2, 6.9, 13.4]])
    V = np.array([[0.01, -0.02, 0.015]])
    parts, bodies = scenario.sphere_bodies(X, d, 1.0, 1.14e3, V)
    return "single", p, parts, bodies, field, None


def run_case(sources, name, p, parts, bodies, field, probes, steps):
    t0 = time.time()
    R = ReferenceCase(sources, p, parts, bodies, field, probes, one_rank_bodies=(name == "single"))
    # the fields as the reference holds them: halo refilled by FillGhostRegionForFluid and Boundary
    u0 = [a.T.copy() for a in R.u0]
    out = {"params": np.asarray(p), "in_parcels": parts, "in_bodies": bodies,
           "in_u": u0[0], "in_v": u0[1], "in_w": u0[2],
           "in_probes": probes if probes is not None else np.zeros(0, WALL_PROBE), "steps": np.int32(steps)}
    for k, v in R.snapshot().items():
        out["init_" + k] = v
    for s in range(steps):
        R.multi_direct_forcing()
        for k, v in R.snapshot().items():
            out[f"mdf{s}_" + k] = v
        for k, v in zip(("u", "v", "w", "fx", "fy", "fz"), R.fields()):
            out[f"mdf{s}_" + k] = _interior(p, v)
        R.cloud_evolution()
        for k, v in R.snapshot().items():
            out[f"step{s}_" + k] = v
        print(f"{name}: step {s + 1}/{steps} after {time.time() - t0:.0f} s", flush=True)
    return out


def cylinder_case(ref_dir):
    """Three cylinders from the reference's marker template CYLINDER_LP1125.dat in
    its own units (dx = 3.75e-5 m, dt = 5e-5 s), built as InitCylinderParcelsDEM
    builds them (tests/golden/make_golden.py), on 48x24x48, periodic, two in contact,
    none straddling a face."""
    import make_golden
    centres = [[0.52e-3, 0.45e-3, 0.6e-3], [1.16e-3, 0.46e-3, 0.63e-3], [0.9e-3, 0.44e-3, 1.25e-3]]
    p, parts, bodies, field = make_golden.cylinder_case(os.path.join(ref_dir, "CYLINDER_LP1125.dat"), centres)
    return "cylinders", p, parts, bodies, field, None


def _f32(field):
    """A field rounded to single precision, so that a fixture can store it as float32."""
    return [np.asarray(f, dtype=np.float32).astype(np.float64) for f in field]


def corner_case():
    """Two spheres (d = 4h) on 12x10x12 between walls in x and in z, periodic in
    y: body 1 in the corner of the low x and low z walls (wall contact on both,
    mirror images across each wall and across the corner, periodic images across
    the low y face), body 2 touching it; a probe on each of the two walls."""
    p = make_params(12, 10, 12, walls="xz", knCoeff=1e4, ResistCoeff=0.9, coupleInterval=2)
    field = _f32(scenario.fourier_field(p, 4, 0.02, seed=21))
    scenario.fill_halo(p, field)
    X = np.array([[2.3, 2.6, 2.4], [2.3 + 4.0 + 0.3, 2.8, 2.6]])
    V = np.array([[-0.02, 0.01, -0.02], [-0.01, 0.0, 0.0]])
    parts, bodies = scenario.sphere_bodies(X, 4.0, 1.0, 1.14e3, V)
    probes = np.zeros(2, WALL_PROBE)
    probes[0]["face"], probes[1]["face"] = 1, 5
    probes[0]["points"] = [[0, 1, 1], [0, 4, 1], [0, 4, 4], [0, 1, 4]]
    probes[1]["points"] = [[1, 1, 0], [4, 1, 0], [4, 4, 0], [1, 4, 0]]
    return "corner", p, parts, bodies, field, probes


def edge_case():
    """Markers placed by hand on exact boundaries, 12^3 periodic: body 1's on
    cell corners and cell centres (so window offsets of exactly 0.5 and 1.5
    cells meet the delta kernel's branch points), body 2's at the contact
    cut-off distance collisionDist*(1+collisionBuffer) from them, one ulp either
    side of it and exactly as the sum rounds, plus one overlapping pair."""
    p = make_params(12, 12, 12, knCoeff=1e4, ResistCoeff=0.9, coupleInterval=2)
    field = _f32(scenario.fourier_field(p, 4, 0.02, seed=23))
    cut = float(p["collisionDist"]) * (1.0 + float(p["collisionBuffer"]))
    up, down = np.inf, -np.inf
    a = [(4.0, 4.0, 4.0), (4.5, 4.5, 4.5), (7.0, 5.0, 4.0), (4.0, 7.5, 6.5), (8.0, 8.0, 8.0)]
    b = [(4.0 + cut, 4.0, 4.0), (4.5, np.nextafter(4.5 + cut, down), 4.5), (7.0, 5.0, np.nextafter(4.0 - cut, up)),
         (np.nextafter(4.0 - cut, down), 7.5, 6.5), (8.0 + 1.2, 8.0, 8.0)]
    n = len(a) + len(b)
    parts = np.zeros(n, PARCEL)
    parts["x"] = np.array(a + b)
    parts["MSIdx"] = [1] * len(a) + [2] * len(b)
    parts["globalIdx"] = list(range(1, len(a) + 1)) + list(range(1, len(b) + 1))
    parts["radeff"], parts["rho"], parts["vol"], parts["pType"] = 0.75, 1.14e3, 0.5, -1
    parts["m"] = parts["rho"] * parts["vol"]
    parts["v"] = [[0.01, 0.0, 0.0]] * len(a) + [[-0.01, 0.005, 0.0]] * len(b)
    bodies = np.zeros(2, MULTISPHERE)
    for k, pts in enumerate((a, b)):
        B = bodies[k:k + 1]
        B["globalIdx"] = k + 1
        B["x"] = np.mean(pts, axis=0)
        B["v"] = B["vold"] = parts["v"][0 if k == 0 else len(a)]
        B["rad"], B["rho"], B["vol"] = 2.0, 1.14e3, 5.0
        B["m"] = B["rho"] * B["vol"]
        B["I"] = 0.4 * B["m"] * 4.0
        B["InertiaTensor"] = np.diag([B["I"][0]] * 3).reshape(9)
        B["rotMat"] = B["rotMatGlo"] = B["rotMatGloOld"] = np.eye(3).reshape(9)
    return "edge", p, parts, bodies, field, None


def empty_case():
    """Two bodies and no markers, 10^3 periodic: the lists are empty, the
    forcing loop leaves the fluid as it was and the bodies fall under gravity."""
    p = make_params(10, 10, 10, coupleInterval=2)
    field = _f32(scenario.fourier_field(p, 4, 0.02, seed=25))
    _, bodies = scenario.sphere_bodies(np.array([[3.0, 4.0, 5.0], [7.0, 6.0, 5.0]]), 4.0, 1.0, 1.14e3,
                                       np.array([[0.01, 0.0, 0.0], [0.0, -0.01, 0.02]]))
    return "empty", p, np.zeros(0, PARCEL), bodies, field, None


def run_compact(sources, name, p, parts, bodies, field, probes, steps):
    """As run_case, but stages stored as digests, with the bodies in full and the
    final parcel positions and velocities."""
    t0 = time.time()
    R = ReferenceCase(sources, p, parts, bodies, field, probes)
    # the case's field is single-precision exact: stored as float32
    u0 = [a.T.astype(np.float32) for a in R.u0]
    assert all(np.array_equal(a.astype(np.float64), b.T) for a, b in zip(u0, R.u0))
    out = {"params": np.asarray(p), "in_parcels": parts, "in_bodies": bodies,
           "in_u": u0[0], "in_v": u0[1], "in_w": u0[2], "steps": np.int32(steps),
           "in_probes": probes if probes is not None else np.zeros(0, WALL_PROBE)}

    def stage(tag, fields=False):
        parts_now, nl = R.parcels(), R.G.m_nplocal
        out[tag + "_nlocal"] = np.int32(nl)
        out[tag + "_np"] = np.int32(len(parts_now))
        out[tag + "_parcel_digest"] = parcel_digest(parts_now, nl)
        out[tag + "_bodies"] = R.bodies()
        out[tag + "_cell_digest"] = digest(*R.cell_lists())
        out[tag + "_pair_digest"] = digest(*R.collision_lists())
        out[tag + "_npairs"] = np.int32(len(R.collision_lists()[1]))
        cnt, cells, w = R.weights()
        out[tag + "_window_digest"] = digest(cells, w)
        if fields:
            out[tag + "_field_digest"] = field_digest(R.fields())
        out[tag + "_probe_force"] = R.probe_forces()

    stage("init")
    for s in range(steps):
        R.multi_direct_forcing()
        stage(f"mdf{s}", fields=True)
        R.cloud_evolution()
        stage(f"step{s}")
        print(f"{name}: step {s + 1}/{steps} after {time.time() - t0:.0f} s", flush=True)
    final = R.parcels()
    out["final_x"], out["final_v"] = final["x"], final["v"]
    return out


CONFIG_SEED = 1


def config_case():
    """The plain resolved configuration the benchmark's CPU-runnable case names:
    128^3 periodic, 64 spheres of d = 16h (about 800 markers each), seeded
    random sequential addition, velocities N(0, 0.01).  The fluid is seeded
    integers times 2^-25 (|u| < 0.032) instead of Fourier modes, so that any
    host regenerates it bit for bit; the tests regenerate the whole case from
    the seed (the fixture holds digests of the inputs)."""
    p, parts, bodies, _ = scenario.resolved_case(128, 128, 128, 64, 16.0, seed=CONFIG_SEED, n_modes=0,
                                                vel_std=0.01)
    rng = np.random.default_rng(CONFIG_SEED + 100)
    shape = field_shape(p)
    field = []
    for _ in range(3):
        a = np.zeros(shape)
        a[2:-2, 2:-2, 2:-2] = rng.integers(-2 ** 20, 2 ** 20, size=(128, 128, 128)) * 2.0 ** -25
        field.append(a)
    scenario.fill_halo(p, field)
    return p, parts, bodies, field


def straddlers(p, parts, bodies):
    """Bodies with a marker more than half a box length from the centre along an
    axis: the ones whose torque arms the reference takes across the box."""
    L = np.array([int(p["nx"]) * float(p["dx"]), int(p["ny"]) * float(p["dy"]), int(p["nz"]) * float(p["dz"])])
    d = np.abs(parts["x"] - bodies["x"][parts["MSIdx"] - 1])
    far = (d > 0.5 * L[None, :]).any(1)
    mask = np.zeros(len(bodies), bool)
    mask[parts["MSIdx"][far] - 1] = True
    return mask


def run_config(sources):
    """config_case through InitializationDEM, one forcing loop and one
    CloudEvolutionMS: digests of the init and forcing stages, the bodies after
    the step in full.  Bodies that straddle a face take the raw torque arm in
    the reference (the library's deviation 2), so only their translation is
    comparable after the step."""
    t0 = time.time()
    p, parts, bodies, field = config_case()
    R = ReferenceCase(sources, p, parts, bodies, field, None, capacities={"maxpartno": 2 * len(parts)})
    print(f"config: initialised after {time.time() - t0:.0f} s", flush=True)
    u0 = [a.T.copy() for a in R.u0]
    out = {"params": np.asarray(p), "seed": np.int32(CONFIG_SEED), "in_parcel_digest": parcel_digest(parts, len(parts)),
           "in_body_digest": digest(*[bodies[f] for f in MULTISPHERE.names]), "in_field_digest": digest(*u0),
           "straddlers": straddlers(p, parts, bodies)}

    def stage(tag, fields=False):
        parts_now, nl = R.parcels(), R.G.m_nplocal
        out[tag + "_nlocal"] = np.int32(nl)
        out[tag + "_np"] = np.int32(len(parts_now))
        out[tag + "_parcel_digest"] = parcel_digest(parts_now, nl)
        out[tag + "_cell_digest"] = digest(*R.cell_lists())
        out[tag + "_pair_digest"] = digest(*R.collision_lists())
        out[tag + "_npairs"] = np.int32(len(R.collision_lists()[1]))
        cnt, cells, w = R.weights()
        out[tag + "_window_digest"] = digest(cells, w)
        if fields:
            out[tag + "_field_digest"] = field_digest(R.fields())

    stage("init")
    R.multi_direct_forcing()
    stage("mdf0", fields=True)
    print(f"config: forcing loop after {time.time() - t0:.0f} s", flush=True)
    R.cloud_evolution()
    out["step0_bodies"] = R.bodies()
    print(f"config: step after {time.time() - t0:.0f} s", flush=True)
    return out


COUPLED_FIELDS = ["u", "v", "w", "fx", "fy", "fz", "P", "Pcorr", "velDiv", "omegaX", "omegaY", "omegaZ"]


def coupled_case():
    """Two spheres (d = 6h) in contact on 16x12x16 between walls in y (the
    reference's own boundary set-up, initialization.F90:317-351), a Fourier
    field, 2 DEM sub-steps per fluid step."""
    p = make_params(16, 12, 16, walls="y", knCoeff=1e4, ResistCoeff=0.9, coupleInterval=2)
    field = _f32(scenario.fourier_field(p, 4, 0.02, seed=29))
    scenario.fill_halo(p, field)
    X = np.array([[5.1, 5.8, 7.9], [5.1 + 6.0 + 0.3, 6.1, 8.2]])
    V = np.array([[0.02, -0.01, 0.0], [-0.02, 0.01, 0.005]])
    parts, bodies = scenario.sphere_bodies(X, 6.0, 1.0, 1.14e3, V)
    return "coupled", p, parts, bodies, field, None


def pressure_solve(G, walls):
    """SetPressureVector + PoissonSolver (poisson.F90:107-158) supplied: the pinned
    pressure-correction system solved by the numpy FFT of tests/fft_poisson.py,
    the interior of Pcorr written as GetLocalArray writes it."""
    import fft_poisson

    b = G.m_veldiv.a[2:-2, 2:-2, 2:-2].T
    G.m_pcorr.a[2:-2, 2:-2, 2:-2] = fft_poisson.solve(b, (G.m_dx, G.m_dy, G.m_dz), walls).T
    return ()


def run_coupled(sources, steps):
    """The reference's whole time step, FirstOrderForwardEuler (fluid.F90:252-327)
    as it stands: uold, the forcing loop, VelocityGuess, ModifyBulkVelocity,
    VelocityDivergence, the Poisson solve (supplied), PressureCorrection,
    VelocityCorrection, each with its halo refill, then CloudEvolutionMS; the
    fluid is not frozen.  Digests of the fields, the parcels and the bodies
    (in full) after every step."""
    t0 = time.time()
    name, p, parts, bodies, field, probes = coupled_case()
    walls = "".join(a for a, f in zip("xyz", range(0, 6, 2)) if int(p["bType"][f]) == 1)
    R = ReferenceCase(sources, p, parts, bodies, field, probes)
    R.T.ns["f_setpressurevector"] = lambda G: ()
    R.T.ns["f_poissonsolver"] = lambda G: pressure_solve(G, walls)
    G = R.G
    G.m_visc = 1e-3
    u0 = [a.T.astype(np.float32) for a in R.u0]
    assert all(np.array_equal(a.astype(np.float64), b.T) for a, b in zip(u0, R.u0))
    out = {"params": np.asarray(p), "in_parcels": parts, "in_bodies": bodies, "in_u": u0[0], "in_v": u0[1],
           "in_w": u0[2], "steps": np.int32(steps), "visc": np.float64(G.m_visc),
           "bulk": np.array([G.m_defavebulkuswitch, G.m_defavebulkvswitch, G.m_defavebulkwswitch, G.m_bulku,
                             G.m_bulkv, G.m_bulkw], dtype=np.float64), "walls": np.array(walls)}
    for s in range(steps):
        R.call("FirstOrderForwardEuler")
        parts_now, nl = R.parcels(), G.m_nplocal
        out[f"step{s}_nlocal"] = np.int32(nl)
        out[f"step{s}_parcel_digest"] = parcel_digest(parts_now, nl)
        out[f"step{s}_bodies"] = R.bodies()
        for f in COUPLED_FIELDS:
            a = getattr(G, "m_" + f.lower()).a.T.copy()
            # the reference accumulates fx, fy, fz into halo cells it then ignores
            out[f"step{s}_{f}"] = digest(a[2:-2, 2:-2, 2:-2] if f in ("fx", "fy", "fz") else a)
            if s == 0 and f in ("u", "v", "w", "P"):
                out[f"step0_{f}_values"] = a
        print(f"coupled: step {s + 1}/{steps} after {time.time() - t0:.0f} s", flush=True)
    return out


def run_output(sources):
    """The reference's output routines after one coupled step of the periodic
    case: OutputCloudTecplot (ZJS_IO_DEM.F90:82-121, the marker file) and
    PostProcessing (fluid.F90:368-404, one probe line per body), their records'
    values as the translator keeps them, beside the parcels and bodies they were
    written from."""
    name, p, parts, bodies, field, probes = periodic_case()
    R = ReferenceCase(sources, p, parts, bodies, field, probes)
    R.multi_direct_forcing()
    R.cloud_evolution()
    G = R.G
    G.m_step = 7
    R.call("OutputCloudTecplot", "1")
    R.call("PostProcessing")
    out = {"params": np.asarray(p), "parcels": R.parcels()[:G.m_nplocal], "bodies": R.bodies(),
           "step": np.int32(G.m_step), "rhof": np.float64(G.m_rhof)}
    recs = G.io_written["Results/Particle_1_0.dat"]
    out["marker_header"] = np.array([" ".join(str(x) for x in recs[0]), " ".join(str(x) for x in recs[1])])
    out["marker_rows"] = np.array(recs[2:], dtype=np.float64)
    ids = sorted(int(k.split("/")[-1].split(".")[0]) for k in G.io_written if k.endswith(".probe"))
    out["probe_ids"] = np.array(ids, np.int32)
    out["probe_rows"] = np.array([G.io_written[f"./DEM/{i}.probe"][0] for i in ids], dtype=np.float64)
    print(f"output: {len(recs) - 2} marker records, {len(ids)} probe lines", flush=True)
    return out


PETSC_CALLS = ("MatCreate", "MatSetSizes", "MatSetType", "MatMPIAIJSetPreallocation", "MatSetFromOptions",
               "MatSetup", "VecCreateMPI", "VecSetFromOptions", "ISCreateGeneral", "VecScatterCreate",
               "MatAssemblyBegin", "MatAssemblyEnd", "VecAssemblyBegin", "VecAssemblyEnd")


def run_poisson(ref_dir, name, p, seed):
    """The reference's pressure-correction system as poisson.F90 assembles it
    (InitPressureCorrectionMatrix, SetPressureCorrectionJacobian and
    SetPressureVector, poisson.F90:2-131): the translator runs them with
    PETSc's MatSetValues and VecSetValues supplied as recorders (ADD_VALUES
    accumulating, INSERT_VALUES replacing) and the rest of PETSc's calls as
    nothing; the matrix in coordinate form and the right-hand side of a random
    divergence are stored."""
    sources = load_sources(ref_dir) + [("poisson.F90", open(os.path.join(ref_dir, "poisson.F90")).read())]
    entries, rhs = {}, {}

    def mat_set_values(G, mat, m, idxm, n, idxn, v, mode, ierr):
        assert m == 1 and n == 1
        key = (int(idxm), int(idxn))
        entries[key] = (entries.get(key, 0.0) + v) if mode == fs.MPI_CONSTANTS["add_values"] else v
        return (mat, m, idxm, n, idxn, v, mode, 0)

    def vec_set_values(G, vec, n, idx, v, mode, ierr):
        assert n == 1
        rhs[int(idx)] = v
        return (vec, n, idx, v, mode, 0)

    noop = lambda G, *a: a  # noqa: E731
    extra = {c.lower(): noop for c in PETSC_CALLS}
    extra.update({"matsetvalues": mat_set_values, "vecsetvalues": vec_set_values})
    R = ReferenceFluid(sources, p, 1e-3, extra=extra)
    R.call("InitPressureCorrectionMatrix")
    R.call("SetPressureCorrectionJacobian")
    div = np.random.default_rng(seed).standard_normal(field_shape(p))
    R.set("velDiv", div)
    R.call("SetPressureVector")
    keys = sorted(entries)
    n = int(p["nx"]) * int(p["ny"]) * int(p["nz"])
    assert sorted(rhs) == list(range(n))
    print(f"{name}: {len(keys)} matrix entries on {n} rows", flush=True)
    return {"params": np.asarray(p), "rows": np.array([k[0] for k in keys], np.int32),
            "cols": np.array([k[1] for k in keys], np.int32), "vals": np.array([entries[k] for k in keys]),
            "velDiv": div, "rhs": np.array([rhs[i] for i in range(n)])}


def run_trajectory(sources, steps):
    """The periodic case over `steps` coupled steps (each the forcing loop on the
    frozen fluid, then CloudEvolutionMS with its 2 sub-steps): after every step
    the bodies in full and digests of the parcels and of the fields the forcing
    loop left."""
    t0 = time.time()
    name, p, parts, bodies, field, probes = periodic_case()
    R = ReferenceCase(sources, p, parts, bodies, field, probes)
    u0 = [a.T.copy() for a in R.u0]
    out = {"params": np.asarray(p), "in_parcels": parts, "in_bodies": bodies, "in_u": u0[0], "in_v": u0[1],
           "in_w": u0[2], "steps": np.int32(steps), "bodies": [], "parcel_digest": [], "field_digest": [],
           "npairs": []}
    for s in range(steps):
        R.multi_direct_forcing()
        out["field_digest"].append(field_digest(R.fields()))
        R.cloud_evolution()
        out["bodies"].append(R.bodies())
        out["parcel_digest"].append(parcel_digest(R.parcels(), R.G.m_nplocal))
        out["npairs"].append(len(R.collision_lists()[1]))
        if (s + 1) % 10 == 0:
            print(f"trajectory: step {s + 1}/{steps} after {time.time() - t0:.0f} s", flush=True)
    for k in ("bodies", "parcel_digest", "field_digest", "npairs"):
        out[k] = np.array(out[k])
    return out


def multirank_case():
    """Three spheres (d = 6h) on 24x16x16, periodic in x, walls in y and z, for
    two ranks along x: body 1 straddles the ranks' seam at x = 12, body 2
    touches it from the other rank, body 3 lies in the image band of the
    periodic x face."""
    p = make_params(24, 16, 16, walls="yz", knCoeff=1e4, ResistCoeff=0.9, coupleInterval=2)
    field = _f32(scenario.fourier_field(p, 4, 0.02, seed=41))
    scenario.fill_halo(p, field)
    X = np.array([[11.2, 7.9, 8.1], [11.2 + 6.0 + 0.3, 8.2, 7.8], [3.6, 8.0, 8.3]])
    V = np.array([[0.02, -0.01, 0.0], [-0.02, 0.01, 0.005], [0.0, 0.01, -0.01]])
    parts, bodies = scenario.sphere_bodies(X, 6.0, 1.0, 1.14e3, V)
    return p, parts, bodies, field


def multirank_straddle_case():
    """multirank_case with body 1 straddling the periodic x face (centre 0.8
    cells from it, its far markers local to the other rank), body 2 touching
    it, body 3 in the middle of the second rank's box."""
    p = make_params(24, 16, 16, walls="yz", knCoeff=1e4, ResistCoeff=0.9, coupleInterval=2)
    field = _f32(scenario.fourier_field(p, 4, 0.02, seed=43))
    scenario.fill_halo(p, field)
    X = np.array([[0.8, 7.9, 8.1], [0.8 + 6.0 + 0.3, 8.2, 7.8], [15.5, 8.0, 8.3]])
    V = np.array([[0.02, -0.01, 0.0], [-0.02, 0.01, 0.005], [0.0, 0.01, -0.01]])
    parts, bodies = scenario.sphere_bodies(X, 6.0, 1.0, 1.14e3, V)
    parts["x"] = scenario.wrap_coord(parts["x"], np.array([24.0, 16.0, 16.0]))
    return p, parts, bodies, field


def multirank_corner_case():
    """Three spheres (d = 6h) on 24x16x24, periodic in x and z, walls in y, for
    2x1x2 ranks (the reference's own run splits x and z, 4x1x4): body 1 on the
    corner where the four ranks meet, body 2 touching it across the z seam,
    body 3 in the image band of the periodic x and z faces."""
    p = make_params(24, 16, 24, walls="y", knCoeff=1e4, ResistCoeff=0.9, coupleInterval=2)
    field = _f32(scenario.fourier_field(p, 4, 0.02, seed=47))
    scenario.fill_halo(p, field)
    X = np.array([[12.3, 7.9, 11.6], [12.1, 8.2, 11.6 + 6.0 + 0.3], [3.4, 8.0, 3.6]])
    V = np.array([[0.02, -0.01, 0.0], [-0.02, 0.01, 0.005], [0.0, 0.01, -0.01]])
    parts, bodies = scenario.sphere_bodies(X, 6.0, 1.0, 1.14e3, V)
    return p, parts, bodies, field


def run_multirank(sources, steps, cpus=(2, 1, 1), make_case=None):
    """The reference as it runs in production, on several MPI ranks (threads of
    this process sharing a fortran_subset.World), its multi-rank code unchanged:
    the bodies and parcels split by rank, their ghosts exchanged with the
    periodic shift, AssembleForceMS, UpdateMSInfoInGhostRegion and RebuildListMS
    as written.  The harness supplies SetBoundaryType with the case's global
    types and each rank's share of the case (InitCylinderParcelsDEM's role: the
    bodies centred in the rank's box, then RebuildListMS, then the markers of
    the bodies it holds inside its box).  Stored after every coupled step: the
    fields assembled from the ranks' slabs, the bodies and the parcels."""
    import threading

    p, parts, bodies, field = (make_case or multirank_case)()
    nr = cpus[0] * cpus[1] * cpus[2]
    bt_glo = [int(b) for b in p["bType"]]

    def set_boundary_type(G):
        G.m_bwg, G.m_beg, G.m_bbg, G.m_bfg, G.m_bsg, G.m_bng = bt_glo
        b = [-1] * 6
        for ax, (idx, ncpu) in enumerate(((G.m_cpuidxx, G.m_cpunx), (G.m_cpuidxy, G.m_cpuny),
                                          (G.m_cpuidxz, G.m_cpunz))):
            if idx == 0:
                b[2 * ax] = bt_glo[2 * ax]
            if idx == ncpu - 1:
                b[2 * ax + 1] = bt_glo[2 * ax + 1]
        G.m_bw, G.m_be, G.m_bb, G.m_bf, G.m_bs, G.m_bn = b
        G.m_btype.a[:] = b
        return ()

    T = fs.Translator(sources, CAPACITIES, CHECK_BOUNDS)
    T.build(overrides={"setboundarytype": set_boundary_type})
    world = fs.World(nr)
    n = [int(p["nx"]), int(p["ny"]), int(p["nz"])]
    results, errors = [None] * nr, []

    def rank(r):
        G = T.new_state()
        G.world, G.rank = world, r
        c = lambda name, *a: T.call(G, name, *a)  # noqa: E731
        try:
            c("PartitionInitialization", *cpus, *n, *[float(k) for k in n])
            c("GridInitialization")
            G.m_dt, G.m_rhof = float(p["dt"]), float(p["rhof"])
            c("SetCellIndexMap")
            c("BuildMPIRecvAndSendIndexForFluid")
            c("InitParameters")
            G.m_kncoeff, G.m_resistcoeff = float(p["knCoeff"]), float(p["ResistCoeff"])
            G.m_coupleinterval = int(p["coupleInterval"])
            G.m_dtdem = G.m_dt / G.m_coupleinterval
            for name in ("CopyGridInformationDEM", "AllocateDEM", "SetCellType", "SetCellIndexMapDEM",
                         "SetNeighCellIndexForCellsDEM", "SetBoundaryNormsAndPoints", "SetMirrorAndShiftCoords"):
                c(name)
            G.m_collisiondist = float(p["collisionDist"])
            lo = np.array([G.m_xstart, G.m_ystart, G.m_zstart])
            hi = np.array([G.m_xend, G.m_yend, G.m_zend])
            G.m_nmsglo = len(bodies)
            inside = [j for j in range(len(bodies)) if np.all(bodies["x"][j] > lo) and np.all(bodies["x"][j] < hi)]
            for k, j in enumerate(inside):
                for f in MULTISPHERE.names:
                    G.m_ms.a[f.lower()][k] = bodies[f][j]
                    G.m_msglo.a[f.lower()][j] = bodies[f][j]
            G.m_nms = G.m_nmslocal = len(inside)
            c("RebuildListMS")
            held = {int(G.m_ms.a["globalidx"][i]) for i in range(G.m_nms)}
            mine = parts[[q for q in range(len(parts)) if int(parts["MSIdx"][q]) in held and
                          np.all(parts["x"][q] > lo) and np.all(parts["x"][q] < hi)]]
            for f in PARCEL.names:
                if f != "pad_":
                    G.m_part.a[f.lower()][:len(mine)] = mine[f]
            G.m_np = G.m_nplocal = len(mine)
            G.m_nmslocal = G.m_nms
            G.m_nppartincell.a[:] = 0
            c("PutParcelsIntoCellsDEM", 1, G.m_np, 0)
            sl = (slice(G.m_sg1 - 1, G.m_eg1), slice(G.m_sg2 - 1, G.m_eg2), slice(G.m_sg3 - 1, G.m_eg3))
            for arr, f in zip((G.m_u, G.m_v, G.m_w), field):
                arr.a[2:-2, 2:-2, 2:-2] = np.asarray(f)[2:-2, 2:-2, 2:-2].T[sl]
            c("FillGhostRegionForFluid")
            c("Boundary")
            u0 = [G.m_u.a.copy(), G.m_v.a.copy(), G.m_w.a.copy()]
            # the rest of InitializationDEM (ZJS_INIT_DEM.F90:24-35)
            for name in ("RebuildListMS", "RebuildParcelInCellListDEM", "RebuildParcelCollisionListDEM",
                         "RebuildNeighborCellListForParcelsDEM", "UpdateLocalCellWeightListDEM",
                         "UpdateParcelInfoInGhostRegion", "UpdateGhostCellWeightListDEM"):
                c(name)
            out = []
            for _ in range(steps):
                for a, a0 in zip((G.m_u, G.m_v, G.m_w), u0):
                    a.a[...] = a0
                G.m_part.a["fdrag"][:G.m_nplocal] = 0.0
                for a in (G.m_fx, G.m_fy, G.m_fz):
                    a.a[...] = 0.0
                for _ in range(int(p["Ns"])):
                    for name in ("UpdateFluidVelocityOnLagrangianPoints", "UpdateParcelInfoInGhostRegion",
                                 "UpdateMomentumSourceTerm", "VelocityPostGuess", "FillGhostRegionForFluid",
                                 "Boundary"):
                        c(name)
                slab = [a.a[2:-2, 2:-2, 2:-2].copy() for a in (G.m_u, G.m_fx)]
                c("CloudEvolutionMS")
                loc = np.zeros(G.m_nplocal, PARCEL)
                for f in PARCEL.names:
                    if f != "pad_":
                        loc[f] = G.m_part.a[f.lower()][:G.m_nplocal]
                bl = np.zeros(G.m_nmslocal, MULTISPHERE)
                for f in MULTISPHERE.names:
                    bl[f] = G.m_ms.a[f.lower()][:G.m_nmslocal]
                out.append((slab, sl, loc, bl))
            results[r] = out
        except BaseException:
            import traceback
            errors.append(traceback.format_exc())
            world.barrier.abort()

    threads = [threading.Thread(target=rank, args=(r,)) for r in range(nr)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    if errors:
        raise RuntimeError(errors[0])
    out = {"params": np.asarray(p), "in_parcels": parts, "in_bodies": bodies, "steps": np.int32(steps),
           "cpus": np.array(cpus, np.int32)}
    for a, f in zip("uvw", field):
        out["in_" + a] = np.asarray(f, dtype=np.float32)
    key = lambda a: a["MSIdx"].astype(np.int64) * 1000000 + a["globalIdx"]  # noqa: E731
    for s in range(steps):
        for k, name in enumerate(("u", "fx")):
            glob = np.zeros(n)
            for r in range(nr):
                slab, sl, _, _ = results[r][s]
                glob[sl] = slab[k]
            out[f"step{s}_{name}"] = np.ascontiguousarray(glob.T)
        b = np.concatenate([results[r][s][3] for r in range(nr)])
        out[f"step{s}_bodies"] = b[np.argsort(b["globalIdx"])]
        q = np.concatenate([results[r][s][2] for r in range(nr)])
        q = q[np.argsort(key(q))]
        for f in ("MSIdx", "globalIdx", "x", "v", "fdrag", "fcol"):
            out[f"step{s}_parcel_{f}"] = q[f]
        out[f"step{s}_ranks"] = np.array([len(results[r][s][2]) for r in range(nr)], np.int32)
    print(f"multirank: {nr} ranks, parcels per rank {out['step0_ranks'].tolist()}", flush=True)
    return out


GENERATION_FIELDS = ("x", "v", "radeff", "rho", "vol", "m", "MSIdx", "globalIdx")


def run_generation(sources, ref_dir, seed):
    """The reference's InitCylinderParcelsDEM (ZJS_INIT_DEM.F90:351-505) as it
    stands, on the grid of its own run (PartitionInitialization(.,.,.,240,32,240,
    9d-3,1.2d-3,9d-3), here one rank holding the whole box): 86 cylinders from
    CYLINDER_LP1125.dat, rotated by pi/2 times a random number each.  The random
    numbers (gfortran's random_number) are supplied, and SetNeighCellIndex (the
    fluid's global neighbour table, which the generation does not read) is
    skipped.  tests/golden/make_golden.py's cylinder generator, given the
    reference's centres and random numbers, must produce the same records: its
    bodies are compared in the tests, its markers here (their digests are
    stored side by side)."""
    import make_golden

    rnd = list(np.random.default_rng(seed).random(86))
    supply = iter(rnd)

    def random_number(G, x):
        return (next(supply),)

    T = fs.Translator(sources, None, CHECK_BOUNDS)
    T.build(overrides={"random_number": random_number, "setneighcellindex": lambda G: ()})
    G = T.new_state(io_dir=ref_dir)
    c = lambda name, *a: T.call(G, name, *a)  # noqa: E731
    c("PartitionInitialization", 1, 1, 1, 240, 32, 240, 9e-3, 1.2e-3, 9e-3)
    c("GridInitialization")
    for name in ("InitParameters", "CopyGridInformationDEM", "AllocateDEM", "SetCellIndexMapDEM",
                 "InitCylinderParcelsDEM"):
        c(name)
    n = G.m_np
    parts = np.zeros(n, PARCEL)
    for f in PARCEL.names:
        if f != "pad_":
            parts[f] = G.m_part.a[f.lower()][:n]
    bodies = np.zeros(G.m_nmsglo, MULTISPHERE)
    for f in MULTISPHERE.names:
        bodies[f] = G.m_msglo.a[f.lower()][:G.m_nmsglo]
    tpl = np.loadtxt(os.path.join(ref_dir, "CYLINDER_LP1125.dat"))
    dx = 9e-3 / 240
    assert G.m_dx == dx
    mine = make_golden.cylinder_markers(tpl, make_golden.cylinder_bodies(bodies["x"], rnd, bodies["v"], dx), dx)
    ref_digest = digest(*[parts[f] for f in GENERATION_FIELDS])
    my_digest = digest(*[mine[f] for f in GENERATION_FIELDS])
    print(f"generation: {n} markers of {len(bodies)} cylinders, generator "
          f"{'identical' if np.array_equal(ref_digest, my_digest) else 'DIFFERENT'}", flush=True)
    return {"rnd": np.array(rnd), "bodies": bodies, "np": np.int32(n), "marker_digest": ref_digest,
            "generator_marker_digest": my_digest, "dx": np.float64(dx)}


def main(ref_dir, only=None):
    sources = load_sources(ref_dir)
    jobs = {
        "drag": lambda: run_drag(sources, 9),
        "fluid_walls_y": lambda: run_fluid(sources, "fluid_walls_y", make_params(10, 8, 12, walls="y"), 1e-3, 3),
        "fluid_periodic": lambda: run_fluid(sources, "fluid_periodic", make_params(8, 10, 6), 1e-3, 4),
        "fluid_rk3_walls_z": lambda: run_fluid_rk3(sources, "fluid_rk3_walls_z", make_params(8, 6, 10, walls="z"),
                                                   2e-3, 6),
        "periodic": lambda: run_case(sources, *periodic_case(), 3),
        "walled": lambda: run_case(sources, *walled_case(), 3),
        "single": lambda: run_case(sources, *single_case(), 3),
        "cylinders": lambda: run_compact(sources, *cylinder_case(ref_dir), 2),
        "config": lambda: run_config(sources),
        "generation": lambda: run_generation(sources, ref_dir, 27),
        "coupled": lambda: run_coupled(sources, 3),
        "output": lambda: run_output(sources),
        "trajectory": lambda: run_trajectory(sources, 100),
        "multirank": lambda: run_multirank(sources, 2),
        "multirank_straddle": lambda: run_multirank(sources, 2, make_case=multirank_straddle_case),
        "multirank_corner": lambda: run_multirank(sources, 2, cpus=(2, 1, 2), make_case=multirank_corner_case),
        "poisson_walls_y": lambda: run_poisson(ref_dir, "poisson_walls_y", make_params(6, 5, 4, walls="y", h=0.5),
                                               31),
        "poisson_periodic": lambda: run_poisson(ref_dir, "poisson_periodic", make_params(5, 4, 6), 32),
        "corner": lambda: run_compact(sources, *corner_case(), 3),
        "edge": lambda: run_compact(sources, *edge_case(), 3),
        "empty": lambda: run_compact(sources, *empty_case(), 2),
    }
    for name, job in jobs.items():
        if only and name not in only:
            continue
        path = os.path.join(HERE, f"ref_{name}.npz")
        np.savez_compressed(path, **job())
        print(f"wrote {path} ({os.path.getsize(path) // 1024} KB)", flush=True)


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if a != "--check-bounds"]
    CHECK_BOUNDS = len(args) < len(sys.argv) - 1
    if not args:
        sys.exit(__doc__)
    main(args[0], args[1:])
