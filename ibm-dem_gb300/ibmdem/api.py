"""Python mirror of the reference's particle-side subroutines over the C ABI.

`Case` owns one device-resident case (an `ibmdem_ctx`).  Its methods carry the
reference's subroutine names (InitializationDEM, RebuildAllListOrNot,
UpdateFluidVelocityOnLagrangianPoints, ...) and call the CUDA library
libibmdem.so; there is no CPU fallback: constructing a Case without the built
library, or without a CUDA device, raises.
"""
import ctypes
import os

import numpy as np

from . import records
from .records import MULTISPHERE, PARAMS, PARCEL, PARTICLE, UPARAMS, field_shape, ufield_shape

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libibmdem.so")

# include/ibmdem.h exports (checked by the symbol test)
EXPORTS = [
    "ibmdem_create", "ibmdem_destroy", "ibmdem_last_error", "ibmdem_abi_version", "ibmdem_set_stream",
    "ibmdem_synchronize", "ibmdem_set_fluid", "ibmdem_get_fluid", "ibmdem_set_parcels", "ibmdem_get_parcels",
    "ibmdem_set_bodies", "ibmdem_get_bodies", "ibmdem_get_cell_lists", "ibmdem_get_collision_lists",
    "ibmdem_RebuildAllListOrNot", "ibmdem_UpdateLocalCellWeightListDEM", "ibmdem_UpdateGhostCellWeightListDEM",
    "ibmdem_UpdateParcelInfoInGhostRegion", "ibmdem_CalculateCollisionForce",
    "ibmdem_CalculateSolidBoundaryCollisionForce", "ibmdem_set_wall_probes", "ibmdem_get_wall_probes",
    "ibmdem_write_tecplot_markers", "ibmdem_write_body_probes", "ibmdem_output_async", "ibmdem_output_wait",
    "ibmdem_update_fluid_async", "ibmdem_update_fluid_wait", "ibmdem_update_fluid_bytes",
    "ibmdem_UpdateFluidVelocityOnLagrangianPoints", "ibmdem_UpdateMomentumSourceTerm", "ibmdem_VelocityPostGuess",
    "ibmdem_AssembleLocalForceMS", "ibmdem_EvolutionMS", "ibmdem_ResetVelocityAndPositionLagrangianPoints",
    "ibmdem_AdjustParcelPosition", "ibmdem_InitializationDEM", "ibmdem_MultiDirectForcing",
    "ibmdem_CloudEvolutionStepMS", "ibmdem_CloudEvolutionMS", "ibmdem_step", "ibmdem_launch_count",
    "ibmdem_get_counters", "ibmdem_timing_enable", "ibmdem_get_timing", "ibmdem_phase_name",
    "ibmdem_measure_fp64_rate", "ibmdem_interpolate_velocity_noalloc", "ibmdem_case_bytes",
    "ibmdem_batch_create", "ibmdem_batch_destroy", "ibmdem_batch_last_error", "ibmdem_batch_add",
    "ibmdem_batch_set_lanes", "ibmdem_batch_step", "ibmdem_batch_synchronize", "ibmdem_batch_autotune",
    "ibmdem_server_create", "ibmdem_server_destroy", "ibmdem_server_last_error", "ibmdem_server_submit",
    "ibmdem_server_poll", "ibmdem_server_status", "ibmdem_server_result", "ibmdem_server_release",
    "ibmdem_server_memory", "ibmdem_server_set_work_limit", "ibmdem_server_set_policy",
    "ibmdem_unresolved_create", "ibmdem_unresolved_destroy", "ibmdem_unresolved_last_error",
    "ibmdem_unresolved_set_stream", "ibmdem_unresolved_set_fluid", "ibmdem_unresolved_set_particles",
    "ibmdem_unresolved_get_particles", "ibmdem_unresolved_get_volume_fraction", "ibmdem_unresolved_get_contacts",
    "ibmdem_unresolved_step", "ibmdem_unresolved_synchronize", "ibmdem_unresolved_launch_count",
    "ibmdem_CalculateDragForce", "ibmdem_unresolved_timing_enable", "ibmdem_unresolved_get_timing",
    "ibmdem_unresolved_phase_name", "ibmdem_get_fluid_async",
    "ibmdem_set_fluid_async", "ibmdem_set_fluid_params", "ibmdem_set_fluid_field", "ibmdem_get_fluid_field", "ibmdem_StoreOldVelocity",
    "ibmdem_VelocityGuess", "ibmdem_FillGhostRegionForFluid", "ibmdem_Boundary", "ibmdem_ModifyBulkVelocity",
    "ibmdem_VelocityDivergence", "ibmdem_PressureCorrection", "ibmdem_VelocityCorrection", "ibmdem_PoissonSolver",
    "ibmdem_set_friction", "ibmdem_get_friction_history", "ibmdem_batch_set_fused", "ibmdem_batch_get_config", "ibmdem_set_step_graphs",
]

SUBROUTINES = [
    "RebuildAllListOrNot", "UpdateLocalCellWeightListDEM", "UpdateGhostCellWeightListDEM",
    "UpdateParcelInfoInGhostRegion", "CalculateCollisionForce", "CalculateSolidBoundaryCollisionForce",
    "UpdateFluidVelocityOnLagrangianPoints",
    "UpdateMomentumSourceTerm", "VelocityPostGuess", "AssembleLocalForceMS", "EvolutionMS",
    "ResetVelocityAndPositionLagrangianPoints", "AdjustParcelPosition", "InitializationDEM", "MultiDirectForcing",
    "CloudEvolutionStepMS", "CloudEvolutionMS",
]

_lib = None


def load(path=LIB_PATH):
    """Load libibmdem.so and declare its prototypes; raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"libibmdem.so not built ({path}); run __graft_entry__.build()")
    lib = ctypes.CDLL(path)
    vp, i32, i64 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64
    P = ctypes.POINTER
    lib.ibmdem_create.argtypes = [vp, i32, P(vp)]
    lib.ibmdem_destroy.argtypes = [vp]
    lib.ibmdem_last_error.restype = ctypes.c_char_p
    lib.ibmdem_last_error.argtypes = [vp]
    lib.ibmdem_set_stream.argtypes = [vp, vp]
    lib.ibmdem_synchronize.argtypes = [vp]
    lib.ibmdem_set_fluid.argtypes = [vp, vp, vp, vp]
    lib.ibmdem_set_fluid_async.argtypes = [vp, vp, vp, vp]
    lib.ibmdem_get_fluid.argtypes = [vp] + [vp] * 6
    lib.ibmdem_get_fluid_async.argtypes = [vp] + [vp] * 6 + [vp]
    lib.ibmdem_set_parcels.argtypes = [vp, i32, vp]
    lib.ibmdem_get_parcels.argtypes = [vp, vp, i32, P(i32), P(i32)]
    lib.ibmdem_set_bodies.argtypes = [vp, i32, vp]
    lib.ibmdem_get_bodies.argtypes = [vp, vp, i32, P(i32)]
    lib.ibmdem_get_cell_lists.argtypes = [vp, vp, vp, P(i64), P(i32)]
    lib.ibmdem_get_collision_lists.argtypes = [vp, vp, vp, P(i32), P(i32)]
    lib.ibmdem_get_counters.argtypes = [vp, vp, i32]
    lib.ibmdem_launch_count.restype = i64
    lib.ibmdem_launch_count.argtypes = [vp]
    lib.ibmdem_step.argtypes = [vp, i32]
    lib.ibmdem_interpolate_velocity_noalloc.argtypes = [vp, i32, vp, vp]
    d = ctypes.c_double
    lib.ibmdem_set_friction.argtypes = [vp, d, d]
    lib.ibmdem_get_friction_history.argtypes = [vp, vp, vp, vp, P(i32), P(i32)]
    lib.ibmdem_set_fluid_params.argtypes = [vp, d, d, d, d]
    lib.ibmdem_set_fluid_field.argtypes = [vp, i32, vp]
    lib.ibmdem_get_fluid_field.argtypes = [vp, i32, vp]
    for name in ("StoreOldVelocity", "FillGhostRegionForFluid", "Boundary"):
        getattr(lib, "ibmdem_" + name).argtypes = [vp]
    lib.ibmdem_VelocityGuess.argtypes = [vp, d, d, d]
    lib.ibmdem_VelocityDivergence.argtypes = [vp, d]
    lib.ibmdem_VelocityCorrection.argtypes = [vp, d]
    lib.ibmdem_PoissonSolver.argtypes = [vp]
    lib.ibmdem_PressureCorrection.argtypes = [vp, vp]
    lib.ibmdem_ModifyBulkVelocity.argtypes = [vp, i32, i32, i32, d, d, d]
    lib.ibmdem_timing_enable.argtypes = [vp, i32]
    lib.ibmdem_get_timing.argtypes = [vp, vp, vp, i32, i32]
    lib.ibmdem_phase_name.restype = ctypes.c_char_p
    lib.ibmdem_phase_name.argtypes = [i32]
    lib.ibmdem_measure_fp64_rate.argtypes = [i32, P(ctypes.c_double)]
    for name in SUBROUTINES:
        getattr(lib, "ibmdem_" + name).argtypes = [vp]
    lib.ibmdem_set_wall_probes.argtypes = [vp, i32, vp]
    lib.ibmdem_write_tecplot_markers.argtypes = [ctypes.c_char_p, i32, vp, vp]
    lib.ibmdem_write_body_probes.argtypes = [ctypes.c_char_p, i64, i32, vp, ctypes.c_double]
    lib.ibmdem_output_async.argtypes = [vp, ctypes.c_char_p, ctypes.c_char_p, i64]
    lib.ibmdem_output_wait.argtypes = [vp]
    lib.ibmdem_update_fluid_async.argtypes = [vp] + [vp] * 6 + [vp]
    lib.ibmdem_update_fluid_wait.argtypes = [vp]
    lib.ibmdem_update_fluid_bytes.argtypes = [vp, P(i64)]
    lib.ibmdem_get_wall_probes.argtypes = [vp, vp, i32, P(i32)]
    dp = P(ctypes.c_double)
    lib.ibmdem_case_bytes.argtypes = [vp, i32, vp, i32, P(i64)]
    lib.ibmdem_batch_create.argtypes = [i32, P(vp)]
    lib.ibmdem_batch_destroy.argtypes = [vp]
    lib.ibmdem_batch_last_error.restype = ctypes.c_char_p
    lib.ibmdem_batch_last_error.argtypes = [vp]
    lib.ibmdem_batch_add.argtypes = [vp, vp]
    lib.ibmdem_batch_set_lanes.argtypes = [vp, i32]
    lib.ibmdem_batch_step.argtypes = [vp, i32]
    lib.ibmdem_batch_synchronize.argtypes = [vp, P(i32)]
    lib.ibmdem_batch_autotune.argtypes = [vp, i32, P(i32)]
    lib.ibmdem_batch_set_fused.argtypes = [vp, i32, i32]
    lib.ibmdem_set_step_graphs.argtypes = [vp, i32]
    lib.ibmdem_batch_get_config.argtypes = [vp, P(i32), P(i32), P(i32)]
    lib.ibmdem_server_create.argtypes = [i32, i64, i32, P(vp)]
    lib.ibmdem_server_destroy.argtypes = [vp]
    lib.ibmdem_server_last_error.restype = ctypes.c_char_p
    lib.ibmdem_server_last_error.argtypes = [vp]
    lib.ibmdem_server_submit.argtypes = [vp, vp, i32, vp, i32, vp, vp, vp, vp, i32, i32, P(i64)]
    lib.ibmdem_server_poll.argtypes = [vp, P(i32)]
    lib.ibmdem_server_status.argtypes = [vp, i64, P(i32), dp, dp]
    lib.ibmdem_server_result.argtypes = [vp, i64, vp, i32, P(i32), P(i32), vp, i32, P(i32)]
    lib.ibmdem_server_release.argtypes = [vp, i64]
    lib.ibmdem_server_memory.argtypes = [vp, P(i64), P(i64)]
    lib.ibmdem_server_set_work_limit.argtypes = [vp, i64]
    lib.ibmdem_server_set_policy.argtypes = [vp, i32, ctypes.c_double]
    lib.ibmdem_unresolved_create.argtypes = [vp, i32, P(vp)]
    lib.ibmdem_unresolved_destroy.argtypes = [vp]
    lib.ibmdem_unresolved_last_error.restype = ctypes.c_char_p
    lib.ibmdem_unresolved_last_error.argtypes = [vp]
    lib.ibmdem_unresolved_set_stream.argtypes = [vp, vp]
    lib.ibmdem_unresolved_set_fluid.argtypes = [vp, vp, vp, vp]
    lib.ibmdem_unresolved_set_particles.argtypes = [vp, i32, vp]
    lib.ibmdem_unresolved_get_particles.argtypes = [vp, vp, i32, P(i32)]
    lib.ibmdem_unresolved_get_volume_fraction.argtypes = [vp, vp]
    lib.ibmdem_unresolved_get_contacts.argtypes = [vp, vp, vp, vp, P(i32)]
    lib.ibmdem_unresolved_step.argtypes = [vp, i32]
    lib.ibmdem_unresolved_synchronize.argtypes = [vp]
    lib.ibmdem_unresolved_launch_count.restype = i64
    lib.ibmdem_unresolved_launch_count.argtypes = [vp]
    lib.ibmdem_CalculateDragForce.argtypes = [i32, vp, vp, vp, ctypes.c_double, vp, vp, vp, vp]
    lib.ibmdem_unresolved_timing_enable.argtypes = [vp, i32]
    lib.ibmdem_unresolved_get_timing.argtypes = [vp, vp, vp, i32, i32]
    lib.ibmdem_unresolved_phase_name.restype = ctypes.c_char_p
    lib.ibmdem_unresolved_phase_name.argtypes = [i32]
    _lib = lib
    return lib


def fp64_rate(device=0):
    """Measured FP64 multiply-add rate of the device in G operations/s."""
    lib = load()
    g = ctypes.c_double()
    rc = lib.ibmdem_measure_fp64_rate(int(device), ctypes.byref(g))
    if rc != 0:
        raise RuntimeError(f"ibmdem_measure_fp64_rate failed ({rc})")
    return g.value


class IbmDemError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class Case:
    """One single-rank periodic case resident on a GB300."""

    def __init__(self, params, parcels=None, bodies=None, field=None, device=0, stream=None):
        self.lib = load()
        self.params = np.array(params, dtype=PARAMS, copy=True)
        h = ctypes.c_void_p()
        rc = self.lib.ibmdem_create(self.params.ctypes.data, int(device), ctypes.byref(h))
        if rc != 0:
            raise IbmDemError(rc, "ibmdem_create failed (no CUDA device, or unsupported parameters)")
        self.h = h
        self.shape = field_shape(self.params)
        if stream is not None:
            self.set_stream(stream)
        if field is not None:
            self.set_fluid(*field)
        if bodies is not None:
            self.set_bodies(bodies)
        if parcels is not None:
            self.set_parcels(parcels)

    # -- lifetime --------------------------------------------------------------
    def close(self):
        if getattr(self, "h", None):
            self.lib.ibmdem_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, rc, what):
        if rc != 0:
            raise IbmDemError(rc, f"{what}: {self.lib.ibmdem_last_error(self.h).decode()}")

    def set_stream(self, stream):
        handle = stream if isinstance(stream, int) else int(getattr(stream, "cuda_stream", stream))
        self._chk(self.lib.ibmdem_set_stream(self.h, ctypes.c_void_p(handle)), "set_stream")

    def synchronize(self):
        self._chk(self.lib.ibmdem_synchronize(self.h), "synchronize")

    @property
    def launches(self):
        return int(self.lib.ibmdem_launch_count(self.h))

    # -- state -----------------------------------------------------------------
    def set_fluid(self, u, v, w):
        a = [np.ascontiguousarray(x, dtype=np.float64).reshape(self.shape) for x in (u, v, w)]
        self._chk(self.lib.ibmdem_set_fluid(self.h, a[0].ctypes.data, a[1].ctypes.data, a[2].ctypes.data),
                  "set_fluid")

    def get_fluid(self):
        out = [np.empty(self.shape) for _ in range(6)]
        self._chk(self.lib.ibmdem_get_fluid(self.h, *[o.ctypes.data for o in out]), "get_fluid")
        return out

    def set_parcels(self, parcels):
        a = np.ascontiguousarray(parcels, dtype=PARCEL)
        self._chk(self.lib.ibmdem_set_parcels(self.h, len(a), a.ctypes.data), "set_parcels")

    def get_parcels(self):
        npo, nl = ctypes.c_int32(), ctypes.c_int32()
        self._chk(self.lib.ibmdem_get_parcels(self.h, None, 0, ctypes.byref(npo), ctypes.byref(nl)), "get_parcels")
        out = np.zeros(npo.value, PARCEL)
        self._chk(self.lib.ibmdem_get_parcels(self.h, out.ctypes.data, len(out), ctypes.byref(npo),
                                              ctypes.byref(nl)), "get_parcels")
        return out, nl.value

    def set_bodies(self, bodies):
        a = np.ascontiguousarray(bodies, dtype=MULTISPHERE)
        self._chk(self.lib.ibmdem_set_bodies(self.h, len(a), a.ctypes.data), "set_bodies")

    def get_bodies(self):
        n = ctypes.c_int32()
        self._chk(self.lib.ibmdem_get_bodies(self.h, None, 0, ctypes.byref(n)), "get_bodies")
        out = np.zeros(n.value, MULTISPHERE)
        self._chk(self.lib.ibmdem_get_bodies(self.h, out.ctypes.data, n.value, ctypes.byref(n)), "get_bodies")
        return out

    def get_cell_lists(self):
        nc, ni = ctypes.c_int64(), ctypes.c_int32()
        self._chk(self.lib.ibmdem_get_cell_lists(self.h, None, None, ctypes.byref(nc), ctypes.byref(ni)), "cells")
        start = np.empty(nc.value + 1, np.int32)
        items = np.empty(ni.value, np.int32)
        self._chk(self.lib.ibmdem_get_cell_lists(self.h, start.ctypes.data, items.ctypes.data, ctypes.byref(nc),
                                                 ctypes.byref(ni)), "cells")
        return start, items

    def get_collision_lists(self):
        nl, npairs = ctypes.c_int32(), ctypes.c_int32()
        self._chk(self.lib.ibmdem_get_collision_lists(self.h, None, None, ctypes.byref(nl), ctypes.byref(npairs)),
                  "pairs")
        start = np.empty(nl.value + 1, np.int32)
        idx = np.empty(npairs.value, np.int32)
        self._chk(self.lib.ibmdem_get_collision_lists(self.h, start.ctypes.data, idx.ctypes.data, ctypes.byref(nl),
                                                      ctypes.byref(npairs)), "pairs")
        return start, idx

    def set_friction(self, ktRatio, mu):
        """Tangential friction of the marker contacts (0 = off, the reference's law)."""
        self._chk(self.lib.ibmdem_set_friction(self.h, float(ktRatio), float(mu)), "set_friction")

    def get_friction_history(self):
        """(start, partner globalIdx, displacement) of the last contact-force call."""
        nl, n = ctypes.c_int32(), ctypes.c_int32()
        self._chk(self.lib.ibmdem_get_friction_history(self.h, None, None, None, ctypes.byref(nl), ctypes.byref(n)),
                  "get_friction_history")
        start = np.zeros(nl.value + 1, np.int32)
        gid = np.empty(n.value, np.int32)
        xi = np.empty((n.value, 3))
        self._chk(self.lib.ibmdem_get_friction_history(self.h, start.ctypes.data, gid.ctypes.data, xi.ctypes.data,
                                                       ctypes.byref(nl), ctypes.byref(n)), "get_friction_history")
        return start, gid, xi

    # ---- fluid stencils (ibmdem_VelocityGuess and the others) ----------------
    def set_fluid_params(self, visc, CPx=0.0, CPy=0.0, CPz=0.0):
        self._chk(self.lib.ibmdem_set_fluid_params(self.h, visc, CPx, CPy, CPz), "set_fluid_params")

    def set_fluid_field(self, which, a):
        """One field of records.FLUID_FIELDS (name or IBMDEM_FLUID_* number)."""
        which = records.FLUID[which] if isinstance(which, str) else int(which)
        a = np.ascontiguousarray(a, dtype=np.float64).reshape(self.shape)
        self._chk(self.lib.ibmdem_set_fluid_field(self.h, which, a.ctypes.data), "set_fluid_field")

    def get_fluid_field(self, which):
        which = records.FLUID[which] if isinstance(which, str) else int(which)
        out = np.empty(self.shape)
        self._chk(self.lib.ibmdem_get_fluid_field(self.h, which, out.ctypes.data), "get_fluid_field")
        return out

    def StoreOldVelocity(self):
        self._chk(self.lib.ibmdem_StoreOldVelocity(self.h), "StoreOldVelocity")

    def VelocityGuess(self, aRK, bRK, cRK):
        self._chk(self.lib.ibmdem_VelocityGuess(self.h, aRK, bRK, cRK), "VelocityGuess")

    def FillGhostRegionForFluid(self):
        self._chk(self.lib.ibmdem_FillGhostRegionForFluid(self.h), "FillGhostRegionForFluid")

    def Boundary(self):
        self._chk(self.lib.ibmdem_Boundary(self.h), "Boundary")

    def ModifyBulkVelocity(self, swU, swV, swW, bulkU, bulkV, bulkW):
        self._chk(self.lib.ibmdem_ModifyBulkVelocity(self.h, swU, swV, swW, bulkU, bulkV, bulkW), "ModifyBulkVelocity")

    def VelocityDivergence(self, cRK):
        self._chk(self.lib.ibmdem_VelocityDivergence(self.h, cRK), "VelocityDivergence")

    def PressureCorrection(self, Pcorr=None):
        ptr = None
        if Pcorr is not None:
            Pcorr = np.ascontiguousarray(Pcorr, dtype=np.float64).reshape(self.shape)
            ptr = Pcorr.ctypes.data
        self._chk(self.lib.ibmdem_PressureCorrection(self.h, ptr), "PressureCorrection")

    def VelocityCorrection(self, cRK):
        self._chk(self.lib.ibmdem_VelocityCorrection(self.h, cRK), "VelocityCorrection")

    def PoissonSolver(self):
        """SetPressureVector + PoissonSolver (poisson.F90:110-186): PCORR on the
        interior from VELDIV."""
        self._chk(self.lib.ibmdem_PoissonSolver(self.h), "PoissonSolver")

    def set_wall_probes(self, probes):
        """Wall collision probes (records.WALL_PROBE) on solid-wall faces."""
        probes = np.ascontiguousarray(probes, dtype=records.WALL_PROBE)
        self._chk(self.lib.ibmdem_set_wall_probes(self.h, len(probes), probes.ctypes.data), "set_wall_probes")

    def output_async(self, tecplot_path=None, probe_dir=None, step=0):
        """Snapshot the parcels and bodies and write the Tecplot marker file and the
        body probe lines from a host thread (ibmdem_output_async)."""
        enc = lambda x: None if x is None else os.fsencode(x)  # noqa: E731
        self._chk(self.lib.ibmdem_output_async(self.h, enc(tecplot_path), enc(probe_dir), int(step)), "output_async")

    def output_wait(self):
        self._chk(self.lib.ibmdem_output_wait(self.h), "output_wait")

    def get_wall_probes(self):
        """The probes with the force sums of the last wall-force call."""
        n = ctypes.c_int32()
        self._chk(self.lib.ibmdem_get_wall_probes(self.h, None, 0, ctypes.byref(n)), "get_wall_probes")
        out = np.zeros(n.value, records.WALL_PROBE)
        self._chk(self.lib.ibmdem_get_wall_probes(self.h, out.ctypes.data, n.value, ctypes.byref(n)),
                  "get_wall_probes")
        return out

    def counters(self):
        out = np.zeros(7, np.int64)
        self._chk(self.lib.ibmdem_get_counters(self.h, out.ctypes.data, 7), "counters")
        keys = ["npLocal", "np", "pairs", "nodes_u", "nodes_v", "nodes_w", "contributions"]
        return dict(zip(keys, (int(x) for x in out)))

    def timing(self, on=True):
        self._chk(self.lib.ibmdem_timing_enable(self.h, 1 if on else 0), "timing_enable")

    def phase_times(self, reset=True):
        """{phase: (total ms, spans)} accumulated since the last reset."""
        ms = np.zeros(32)
        cnt = np.zeros(32, np.int64)
        n = self.lib.ibmdem_get_timing(self.h, ms.ctypes.data, cnt.ctypes.data, 32, 1 if reset else 0)
        return {self.lib.ibmdem_phase_name(i).decode(): (float(ms[i]), int(cnt[i])) for i in range(n)}

    # -- the reference subroutines ----------------------------------------------
    def call(self, name):
        self._chk(getattr(self.lib, "ibmdem_" + name)(self.h), name)

    def step(self, n=1):
        self._chk(self.lib.ibmdem_step(self.h, int(n)), "step")

    def set_step_graphs(self, on):
        """ibmdem_step as replays of a captured graph (True, the default) or kernel by kernel."""
        self._chk(self.lib.ibmdem_set_step_graphs(self.h, int(bool(on))), "set_step_graphs")


def _make_method(name):
    def method(self):
        self.call(name)
    method.__name__ = name
    method.__doc__ = f"ibmdem_{name} (the reference subroutine of the same name)."
    return method


for _name in SUBROUTINES:
    setattr(Case, _name, _make_method(_name))


def write_tecplot_markers(path, parcels, centre=(0.0, 0.0, 0.0)):
    """OutputCloudTecplot's marker file from host parcel records (no GPU needed)."""
    lib = load()
    a = np.ascontiguousarray(parcels, dtype=PARCEL)
    c = np.ascontiguousarray(centre, dtype=np.float64)
    rc = lib.ibmdem_write_tecplot_markers(os.fsencode(path), len(a), a.ctypes.data if len(a) else None, c.ctypes.data)
    if rc != 0:
        raise IbmDemError(rc, "ibmdem_write_tecplot_markers")


def write_body_probes(directory, step, bodies, rhof):
    """Append the per-body probe lines of fluid.F90:392-397 (no GPU needed)."""
    lib = load()
    b = np.ascontiguousarray(bodies, dtype=MULTISPHERE)
    rc = lib.ibmdem_write_body_probes(os.fsencode(directory), int(step), len(b), b.ctypes.data if len(b) else None,
                                      float(rhof))
    if rc != 0:
        raise IbmDemError(rc, "ibmdem_write_body_probes")


def case_bytes(params, parcels, n_bodies):
    """Device bytes a case takes once created and initialised (ibmdem_case_bytes)."""
    lib = load()
    p = np.array(params, dtype=PARAMS, copy=True)
    a = np.ascontiguousarray(parcels, dtype=PARCEL)
    out = ctypes.c_int64()
    rc = lib.ibmdem_case_bytes(p.ctypes.data, len(a), a.ctypes.data if len(a) else None, int(n_bodies),
                               ctypes.byref(out))
    if rc != 0:
        raise IbmDemError(rc, "ibmdem_case_bytes")
    return out.value


class Batch:
    """Many cases advanced together, one CUDA graph launch per step (ibmdem_batch_*).

    The member `Case` objects stay owned by the caller and must outlive the batch."""

    def __init__(self, cases=(), device=0, lanes=0):
        self.lib = load()
        h = ctypes.c_void_p()
        rc = self.lib.ibmdem_batch_create(int(device), ctypes.byref(h))
        if rc != 0:
            raise IbmDemError(rc, "ibmdem_batch_create failed")
        self.h = h
        self.cases = []
        for c in cases:
            self.add(c)
        if lanes:
            self.set_lanes(lanes)

    def _chk(self, rc, what):
        if rc != 0:
            raise IbmDemError(rc, f"{what}: {self.lib.ibmdem_batch_last_error(self.h).decode()}")

    def add(self, case):
        self._chk(self.lib.ibmdem_batch_add(self.h, case.h), "batch_add")
        self.cases.append(case)

    def set_lanes(self, lanes):
        self._chk(self.lib.ibmdem_batch_set_lanes(self.h, int(lanes)), "batch_set_lanes")

    def set_fused(self, fused, interp_block=256):
        """All members' forcing loops in shared launches (see ibmdem_batch_set_fused)."""
        self._chk(self.lib.ibmdem_batch_set_fused(self.h, int(bool(fused)), int(interp_block)), "batch_set_fused")

    def config(self):
        """(lanes, fused, interp_block) the next step runs with."""
        v = [ctypes.c_int32() for _ in range(3)]
        self._chk(self.lib.ibmdem_batch_get_config(self.h, *(ctypes.byref(x) for x in v)), "batch_get_config")
        return tuple(x.value for x in v)

    def step(self, n=1):
        self._chk(self.lib.ibmdem_batch_step(self.h, int(n)), "batch_step")

    def synchronize(self):
        failed = ctypes.c_int32(-1)
        self._chk(self.lib.ibmdem_batch_synchronize(self.h, ctypes.byref(failed)), "batch_synchronize")

    def autotune(self, trial_steps=3):
        lanes = ctypes.c_int32()
        self._chk(self.lib.ibmdem_batch_autotune(self.h, int(trial_steps), ctypes.byref(lanes)), "batch_autotune")
        return lanes.value

    def close(self):
        if getattr(self, "h", None):
            self.lib.ibmdem_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """A request server on one device (ibmdem_server_*): admission by device
    memory budget, each admitted case on its own stream, results read back on
    completion.  Input arrays are kept referenced until the request is admitted."""

    QUEUED, RUNNING, DONE = 0, 1, 2
    ARRIVAL, LEAST_WORK = 0, 1

    def __init__(self, hbm_budget, max_active=64, device=0, work_limit=0):
        self.lib = load()
        h = ctypes.c_void_p()
        rc = self.lib.ibmdem_server_create(int(device), int(hbm_budget), int(max_active), ctypes.byref(h))
        if rc != 0:
            raise IbmDemError(rc, "ibmdem_server_create failed")
        self.h = h
        self._inputs = {}
        if work_limit:
            self._chk(self.lib.ibmdem_server_set_work_limit(self.h, int(work_limit)), "server_set_work_limit")

    def _chk(self, rc, what):
        if rc != 0:
            raise IbmDemError(rc, f"{what}: {self.lib.ibmdem_server_last_error(self.h).decode()}")

    def set_policy(self, policy, age_limit_s=0.0):
        """Admission order: Server.ARRIVAL or Server.LEAST_WORK (fewest marker-steps
        first, the oldest first again once one has waited age_limit_s > 0)."""
        self._chk(self.lib.ibmdem_server_set_policy(self.h, int(policy), float(age_limit_s)), "server_set_policy")

    def submit(self, params, parcels, bodies, field=None, nsteps=100, keep_parcels=False):
        p = np.array(params, dtype=PARAMS, copy=True)
        a = np.ascontiguousarray(parcels, dtype=PARCEL)
        b = np.ascontiguousarray(bodies, dtype=MULTISPHERE)
        shape = field_shape(p)
        f = None if field is None else [np.ascontiguousarray(x, dtype=np.float64).reshape(shape) for x in field]
        fp = [None, None, None] if f is None else [x.ctypes.data for x in f]
        rid = ctypes.c_int64()
        self._chk(self.lib.ibmdem_server_submit(self.h, p.ctypes.data, len(a), a.ctypes.data, len(b), b.ctypes.data,
                                                fp[0], fp[1], fp[2], int(nsteps), int(bool(keep_parcels)),
                                                ctypes.byref(rid)), "server_submit")
        self._inputs[rid.value] = (p, a, b, f)
        return rid.value

    def poll(self):
        pending = ctypes.c_int32()
        self._chk(self.lib.ibmdem_server_poll(self.h, ctypes.byref(pending)), "server_poll")
        for rid in [r for r in self._inputs if self.state(r)[0] != self.QUEUED]:
            del self._inputs[rid]
        return pending.value

    def state(self, rid):
        st, lat, q = ctypes.c_int32(), ctypes.c_double(), ctypes.c_double()
        self._chk(self.lib.ibmdem_server_status(self.h, int(rid), ctypes.byref(st), ctypes.byref(lat),
                                                ctypes.byref(q)), "server_status")
        return st.value, lat.value, q.value

    def result(self, rid):
        npo, nl, nb = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        self._chk(self.lib.ibmdem_server_result(self.h, int(rid), None, 0, ctypes.byref(npo), ctypes.byref(nl), None, 0,
                                                ctypes.byref(nb)), "server_result")
        parts = np.zeros(npo.value, PARCEL)
        bodies = np.zeros(nb.value, MULTISPHERE)
        self._chk(self.lib.ibmdem_server_result(self.h, int(rid), parts.ctypes.data, len(parts), ctypes.byref(npo),
                                                ctypes.byref(nl), bodies.ctypes.data, len(bodies),
                                                ctypes.byref(nb)), "server_result")
        return parts, nl.value, bodies

    def release(self, rid):
        self._chk(self.lib.ibmdem_server_release(self.h, int(rid)), "server_release")

    def memory(self):
        used, budget = ctypes.c_int64(), ctypes.c_int64()
        self._chk(self.lib.ibmdem_server_memory(self.h, ctypes.byref(used), ctypes.byref(budget)), "server_memory")
        return used.value, budget.value

    def close(self):
        if getattr(self, "h", None):
            self.lib.ibmdem_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Unresolved:
    """One unresolved CFD-DEM case (point particles) resident on a GB300 (ibmdem_unresolved_*)."""

    def __init__(self, params, particles=None, field=None, device=0, stream=None):
        self.lib = load()
        self.params = np.array(params, dtype=UPARAMS, copy=True)
        h = ctypes.c_void_p()
        rc = self.lib.ibmdem_unresolved_create(self.params.ctypes.data, int(device), ctypes.byref(h))
        if rc != 0:
            raise IbmDemError(rc, "ibmdem_unresolved_create failed (no CUDA device, or unsupported parameters)")
        self.h = h
        self.shape = ufield_shape(self.params)
        self.nint = int(self.params["nx"]) * int(self.params["ny"]) * int(self.params["nz"])
        if stream is not None:
            handle = stream if isinstance(stream, int) else int(getattr(stream, "cuda_stream", stream))
            self._chk(self.lib.ibmdem_unresolved_set_stream(self.h, ctypes.c_void_p(handle)), "set_stream")
        if field is not None:
            self.set_fluid(*field)
        if particles is not None:
            self.set_particles(particles)

    def close(self):
        if getattr(self, "h", None):
            self.lib.ibmdem_unresolved_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, rc, what):
        if rc != 0:
            raise IbmDemError(rc, f"{what}: {self.lib.ibmdem_unresolved_last_error(self.h).decode()}")

    @property
    def launches(self):
        return int(self.lib.ibmdem_unresolved_launch_count(self.h))

    def set_fluid(self, u, v, w):
        a = [np.ascontiguousarray(x, dtype=np.float64).reshape(self.shape) for x in (u, v, w)]
        self._chk(self.lib.ibmdem_unresolved_set_fluid(self.h, *[x.ctypes.data for x in a]), "set_fluid")

    def set_particles(self, parts):
        a = np.ascontiguousarray(parts, dtype=PARTICLE)
        self._chk(self.lib.ibmdem_unresolved_set_particles(self.h, len(a), a.ctypes.data), "set_particles")

    def get_particles(self):
        n = ctypes.c_int32()
        self._chk(self.lib.ibmdem_unresolved_get_particles(self.h, None, 0, ctypes.byref(n)), "get_particles")
        out = np.zeros(n.value, PARTICLE)
        self._chk(self.lib.ibmdem_unresolved_get_particles(self.h, out.ctypes.data, len(out), ctypes.byref(n)),
                  "get_particles")
        return out

    def get_volume_fraction(self):
        out = np.zeros(self.nint)
        self._chk(self.lib.ibmdem_unresolved_get_volume_fraction(self.h, out.ctypes.data), "get_volume_fraction")
        return out

    def get_contacts(self):
        n = ctypes.c_int32()
        self._chk(self.lib.ibmdem_unresolved_get_contacts(self.h, None, None, None, ctypes.byref(n)), "get_contacts")
        nparts = ctypes.c_int32()
        self._chk(self.lib.ibmdem_unresolved_get_particles(self.h, None, 0, ctypes.byref(nparts)), "get_particles")
        start = np.zeros(nparts.value + 1, np.int32)
        partner = np.zeros(max(n.value, 1), np.int32)
        xi = np.zeros((max(n.value, 1), 3))
        self._chk(self.lib.ibmdem_unresolved_get_contacts(self.h, start.ctypes.data, partner.ctypes.data,
                                                          xi.ctypes.data, ctypes.byref(n)), "get_contacts")
        return start, partner[:n.value], xi[:n.value]

    def step(self, n=1):
        self._chk(self.lib.ibmdem_unresolved_step(self.h, int(n)), "step")

    def synchronize(self):
        self._chk(self.lib.ibmdem_unresolved_synchronize(self.h), "synchronize")

    def timing(self, on=True):
        self._chk(self.lib.ibmdem_unresolved_timing_enable(self.h, int(bool(on))), "timing_enable")

    def phase_times(self, reset=False):
        """{phase: (total ms, spans)} accumulated since the last reset (synchronises)."""
        ms = np.zeros(8)
        cnt = np.zeros(8, np.int64)
        n = self.lib.ibmdem_unresolved_get_timing(self.h, ms.ctypes.data, cnt.ctypes.data, 8, int(bool(reset)))
        return {self.lib.ibmdem_unresolved_phase_name(i).decode(): (float(ms[i]), int(cnt[i])) for i in range(n)}
