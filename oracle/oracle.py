"""ctypes binding of the CPU restatement (oracle/libibmdem_oracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU legs of bench.py, never by the product.  Parity pinned to the reference's
own subroutines, run by tests/golden/fortran_subset.py; see ibmdem_oracle.c.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libibmdem_oracle.so")
_lib = None


def build(quiet=True):
    """Compile the oracle with its Makefile (gcc, OpenMP)."""
    r = subprocess.run(["make", "-C", _HERE], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    if not quiet:
        print(r.stdout)
    return _LIB_PATH


def _load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_LIB_PATH):
        build()
    lib = ctypes.CDLL(_LIB_PATH)
    vp, i32, i64 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64
    P = ctypes.POINTER
    lib.orc_create.restype = vp
    lib.orc_create.argtypes = [vp]
    lib.orc_destroy.argtypes = [vp]
    lib.orc_last_error.restype = ctypes.c_char_p
    lib.orc_last_error.argtypes = [vp]
    lib.orc_set_threads.argtypes = [ctypes.c_int]
    lib.orc_get_threads.restype = ctypes.c_int
    lib.orc_set_fluid.argtypes = [vp, vp, vp, vp]
    lib.orc_get_fluid.argtypes = [vp] + [vp] * 6
    lib.orc_set_parcels.argtypes = [vp, i32, vp]
    lib.orc_get_parcels.argtypes = [vp, vp, i32, P(i32), P(i32)]
    lib.orc_set_bodies.argtypes = [vp, i32, vp]
    lib.orc_get_bodies.argtypes = [vp, vp, i32, P(i32)]
    lib.orc_get_cell_lists.argtypes = [vp, vp, vp, P(i64), P(i32)]
    lib.orc_get_collision_lists.argtypes = [vp, vp, vp, P(i32), P(i32)]
    lib.orc_get_weights.argtypes = [vp, i32, vp, vp]
    for name in ("RebuildAllListOrNot", "UpdateLocalCellWeightListDEM", "UpdateGhostCellWeightListDEM",
                 "UpdateParcelInfoInGhostRegion", "CalculateCollisionForce", "CalculateSolidBoundaryCollisionForce",
                 "UpdateFluidVelocityOnLagrangianPoints", "UpdateMomentumSourceTerm", "VelocityPostGuess",
                 "AssembleLocalForceMS", "EvolutionMS", "ResetVelocityAndPositionLagrangianPoints",
                 "AdjustParcelPosition", "InitializationDEM", "MultiDirectForcing", "CloudEvolutionStepMS",
                 "CloudEvolutionMS"):
        getattr(lib, "orc_" + name).argtypes = [vp]
        getattr(lib, "orc_" + name).restype = ctypes.c_int
    lib.orc_step.argtypes = [vp, i32]
    lib.orc_set_friction.argtypes = [vp, ctypes.c_double, ctypes.c_double]
    lib.orc_get_friction_history.argtypes = [vp, vp, vp, vp, P(i32), P(i32)]
    lib.orc_set_wall_probes.argtypes = [vp, i32, vp]
    lib.orc_get_wall_probes.argtypes = [vp, vp, i32, P(i32)]
    lib.orc_eta.restype = ctypes.c_double
    lib.orc_eta.argtypes = [ctypes.c_double]
    lib.orc_CalculateDragForce.argtypes = [ctypes.c_double, ctypes.c_double, vp, ctypes.c_double,
                                           ctypes.c_double, vp, vp]
    lib.orc_u_create.restype = vp
    lib.orc_u_create.argtypes = [vp]
    lib.orc_u_destroy.argtypes = [vp]
    lib.orc_u_last_error.restype = ctypes.c_char_p
    lib.orc_u_last_error.argtypes = [vp]
    lib.orc_u_set_fluid.argtypes = [vp, vp, vp, vp]
    lib.orc_u_set_particles.argtypes = [vp, i32, vp]
    lib.orc_u_get_particles.argtypes = [vp, vp, i32, P(i32)]
    lib.orc_u_get_volume_fraction.argtypes = [vp, vp]
    lib.orc_u_get_contacts.argtypes = [vp, vp, vp, vp, P(i32)]
    lib.orc_u_step.argtypes = [vp, i32]
    d = ctypes.c_double
    lib.orc_fluid_create.restype = vp
    lib.orc_fluid_create.argtypes = [vp]
    lib.orc_fluid_destroy.argtypes = [vp]
    lib.orc_fluid_set_params.argtypes = [vp, d, d, d, d]
    lib.orc_fluid_set_field.argtypes = [vp, ctypes.c_int, vp]
    lib.orc_fluid_get_field.argtypes = [vp, ctypes.c_int, vp]
    for name in ("StoreOldVelocity", "FillGhostRegionForFluid", "Boundary", "PressureCorrection"):
        getattr(lib, "orc_fluid_" + name).argtypes = [vp]
    lib.orc_fluid_VelocityGuess.argtypes = [vp, d, d, d]
    lib.orc_fluid_VelocityDivergence.argtypes = [vp, d]
    lib.orc_fluid_VelocityCorrection.argtypes = [vp, d]
    lib.orc_fluid_PressureOperator.argtypes = [vp, vp, vp]
    lib.orc_fluid_ModifyBulkVelocity.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, d, d, d]
    _lib = lib
    return lib


def set_threads(n):
    _load().orc_set_threads(int(n))


def eta(e):
    return _load().orc_eta(float(e))


def drag_beta(rho_p, rad_p, v_p, denf, alphaf, velf):
    beta = np.zeros(3)
    v_p = np.ascontiguousarray(v_p, dtype=np.float64)
    velf = np.ascontiguousarray(velf, dtype=np.float64)
    _load().orc_CalculateDragForce(rho_p, rad_p, v_p.ctypes.data, denf, alphaf, velf.ctypes.data, beta.ctypes.data)
    return beta


class OracleCase:
    """One single-rank periodic case held by the CPU restatement."""

    def __init__(self, params, parcels=None, bodies=None, field=None):
        self.lib = _load()
        self.params = np.array(params, copy=True)
        self.h = self.lib.orc_create(self.params.ctypes.data)
        if not self.h:
            raise ValueError("orc_create rejected the parameters")
        n = self.params
        self.shape = (int(n["nz"]) + 4, int(n["ny"]) + 4, int(n["nx"]) + 4)
        if field is not None:
            self.set_fluid(*field)
        if parcels is not None:
            self.set_parcels(parcels)
        if bodies is not None:
            self.set_bodies(bodies)

    def close(self):
        if self.h:
            self.lib.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, rc, what):
        if rc != 0:
            raise RuntimeError(f"oracle {what} failed ({rc}): {self.lib.orc_last_error(self.h).decode()}")

    def set_fluid(self, u, v, w):
        a = [np.ascontiguousarray(x, dtype=np.float64).reshape(self.shape) for x in (u, v, w)]
        self._chk(self.lib.orc_set_fluid(self.h, a[0].ctypes.data, a[1].ctypes.data, a[2].ctypes.data), "set_fluid")

    def get_fluid(self):
        out = [np.empty(self.shape) for _ in range(6)]
        self._chk(self.lib.orc_get_fluid(self.h, *[o.ctypes.data for o in out]), "get_fluid")
        return out

    def set_parcels(self, parcels):
        from ibmdem.records import PARCEL
        a = np.ascontiguousarray(parcels, dtype=PARCEL)
        self._chk(self.lib.orc_set_parcels(self.h, len(a), a.ctypes.data), "set_parcels")

    def get_parcels(self):
        from ibmdem.records import PARCEL
        npo, nl = ctypes.c_int32(), ctypes.c_int32()
        self.lib.orc_get_parcels(self.h, None, 0, ctypes.byref(npo), ctypes.byref(nl))
        out = np.zeros(npo.value, PARCEL)
        self._chk(self.lib.orc_get_parcels(self.h, out.ctypes.data, len(out), ctypes.byref(npo), ctypes.byref(nl)),
                  "get_parcels")
        return out, nl.value

    def set_bodies(self, bodies):
        from ibmdem.records import MULTISPHERE
        a = np.ascontiguousarray(bodies, dtype=MULTISPHERE)
        self._chk(self.lib.orc_set_bodies(self.h, len(a), a.ctypes.data), "set_bodies")

    def get_bodies(self):
        from ibmdem.records import MULTISPHERE
        n = ctypes.c_int32()
        self.lib.orc_get_bodies(self.h, None, 0, ctypes.byref(n))
        out = np.zeros(n.value, MULTISPHERE)
        self._chk(self.lib.orc_get_bodies(self.h, out.ctypes.data, n.value, ctypes.byref(n)), "get_bodies")
        return out

    def get_cell_lists(self):
        nc, ni = ctypes.c_int64(), ctypes.c_int32()
        self._chk(self.lib.orc_get_cell_lists(self.h, None, None, ctypes.byref(nc), ctypes.byref(ni)), "cells")
        start = np.empty(nc.value + 1, np.int32)
        items = np.empty(ni.value, np.int32)
        self._chk(self.lib.orc_get_cell_lists(self.h, start.ctypes.data, items.ctypes.data, ctypes.byref(nc),
                                              ctypes.byref(ni)), "cells")
        return start, items

    def get_collision_lists(self):
        nl, npairs = ctypes.c_int32(), ctypes.c_int32()
        self._chk(self.lib.orc_get_collision_lists(self.h, None, None, ctypes.byref(nl), ctypes.byref(npairs)),
                  "pairs")
        start = np.empty(nl.value + 1, np.int32)
        idx = np.empty(npairs.value, np.int32)
        self._chk(self.lib.orc_get_collision_lists(self.h, start.ctypes.data, idx.ctypes.data, ctypes.byref(nl),
                                                   ctypes.byref(npairs)), "pairs")
        return start, idx

    def get_weights(self, n):
        w = np.empty((n, 125, 3))
        cells = np.empty((n, 125), np.int32)
        self._chk(self.lib.orc_get_weights(self.h, n, w.ctypes.data, cells.ctypes.data), "weights")
        return w, cells

    def call(self, name):
        self._chk(getattr(self.lib, "orc_" + name)(self.h), name)

    def step(self, n=1):
        self._chk(self.lib.orc_step(self.h, int(n)), "step")

    def set_friction(self, ktRatio, mu):
        self._chk(self.lib.orc_set_friction(self.h, float(ktRatio), float(mu)), "set_friction")

    def get_friction_history(self):
        nl, n = ctypes.c_int32(), ctypes.c_int32()
        self.lib.orc_get_friction_history(self.h, None, None, None, ctypes.byref(nl), ctypes.byref(n))
        start = np.zeros(nl.value + 1, np.int32)
        gid = np.empty(n.value, np.int32)
        xi = np.empty((n.value, 3))
        self.lib.orc_get_friction_history(self.h, start.ctypes.data, gid.ctypes.data, xi.ctypes.data,
                                          ctypes.byref(nl), ctypes.byref(n))
        return start, gid, xi

    def set_wall_probes(self, probes):
        from ibmdem import records
        probes = np.ascontiguousarray(probes, dtype=records.WALL_PROBE)
        self._chk(self.lib.orc_set_wall_probes(self.h, len(probes), probes.ctypes.data), "set_wall_probes")

    def get_wall_probes(self):
        from ibmdem import records
        n = ctypes.c_int32()
        self._chk(self.lib.orc_get_wall_probes(self.h, None, 0, ctypes.byref(n)), "get_wall_probes")
        out = np.zeros(n.value, records.WALL_PROBE)
        self._chk(self.lib.orc_get_wall_probes(self.h, out.ctypes.data, n.value, ctypes.byref(n)), "get_wall_probes")
        return out


_SUBROUTINES = ("RebuildAllListOrNot", "UpdateLocalCellWeightListDEM", "UpdateGhostCellWeightListDEM",
                "UpdateParcelInfoInGhostRegion", "CalculateCollisionForce", "CalculateSolidBoundaryCollisionForce",
                "UpdateFluidVelocityOnLagrangianPoints",
                "UpdateMomentumSourceTerm", "VelocityPostGuess", "AssembleLocalForceMS", "EvolutionMS",
                "ResetVelocityAndPositionLagrangianPoints", "AdjustParcelPosition", "InitializationDEM",
                "MultiDirectForcing", "CloudEvolutionStepMS", "CloudEvolutionMS")


def _make(name):
    def method(self):
        self.call(name)
    method.__name__ = name
    return method


for _n in _SUBROUTINES:
    setattr(OracleCase, _n, _make(_n))


class OracleUnresolved:
    """One unresolved CFD-DEM case held by the CPU restatement (unresolved_oracle.c)."""

    def __init__(self, params, particles=None, field=None):
        import sys
        sys.path.insert(0, os.path.join(os.path.dirname(_HERE), "ibm-dem_gb300"))
        from ibmdem.records import PARTICLE, UPARAMS, ufield_shape

        self._PARTICLE = PARTICLE
        self.lib = _load()
        self.params = np.array(params, dtype=UPARAMS, copy=True)
        self.h = self.lib.orc_u_create(self.params.ctypes.data)
        if not self.h:
            raise RuntimeError("orc_u_create rejected the parameters")
        self.shape = ufield_shape(self.params)
        n = self.params
        self.nint = int(n["nx"]) * int(n["ny"]) * int(n["nz"])
        if field is not None:
            self.set_fluid(*field)
        if particles is not None:
            self.set_particles(particles)

    def close(self):
        if getattr(self, "h", None):
            self.lib.orc_u_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, rc, what):
        if rc != 0:
            raise RuntimeError(f"{what} [{rc}]: {self.lib.orc_u_last_error(self.h).decode()}")

    def set_fluid(self, u, v, w):
        a = [np.ascontiguousarray(x, dtype=np.float64).reshape(self.shape) for x in (u, v, w)]
        self._chk(self.lib.orc_u_set_fluid(self.h, *[x.ctypes.data for x in a]), "set_fluid")

    def set_particles(self, parts):
        a = np.ascontiguousarray(parts, dtype=self._PARTICLE)
        self._chk(self.lib.orc_u_set_particles(self.h, len(a), a.ctypes.data), "set_particles")

    def get_particles(self):
        n = ctypes.c_int32()
        self._chk(self.lib.orc_u_get_particles(self.h, None, 0, ctypes.byref(n)), "get_particles")
        out = np.zeros(n.value, self._PARTICLE)
        self._chk(self.lib.orc_u_get_particles(self.h, out.ctypes.data, len(out), ctypes.byref(n)), "get_particles")
        return out

    def get_volume_fraction(self):
        out = np.zeros(self.nint)
        self._chk(self.lib.orc_u_get_volume_fraction(self.h, out.ctypes.data), "get_volume_fraction")
        return out

    def get_contacts(self):
        n = ctypes.c_int32()
        self._chk(self.lib.orc_u_get_contacts(self.h, None, None, None, ctypes.byref(n)), "get_contacts")
        np_ = len(self.get_particles())
        start = np.zeros(np_ + 1, np.int32)
        partner = np.zeros(max(n.value, 1), np.int32)
        xi = np.zeros((max(n.value, 1), 3))
        self._chk(self.lib.orc_u_get_contacts(self.h, start.ctypes.data, partner.ctypes.data, xi.ctypes.data,
                                              ctypes.byref(n)), "get_contacts")
        return start, partner[:n.value], xi[:n.value]

    def step(self, n=1):
        self._chk(self.lib.orc_u_step(self.h, int(n)), "step")


class OracleFluid:
    """The fluid stencils of FirstOrderForwardEuler held by the CPU restatement
    (fluid_oracle.c): fields indexed by the IBMDEM_FLUID_* numbers of
    include/ibmdem.h (ibmdem.records.FLUID_FIELDS), in the layout of
    ibmdem_set_fluid."""

    def __init__(self, params):
        import sys
        sys.path.insert(0, os.path.join(os.path.dirname(_HERE), "ibm-dem_gb300"))
        from ibmdem.records import PARAMS, field_shape

        self.lib = _load()
        self.params = np.array(params, dtype=PARAMS, copy=True)
        self.h = self.lib.orc_fluid_create(self.params.ctypes.data)
        if not self.h:
            raise RuntimeError("orc_fluid_create failed")
        self.shape = field_shape(self.params)

    def close(self):
        if getattr(self, "h", None):
            self.lib.orc_fluid_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_fluid_params(self, visc, CPx=0.0, CPy=0.0, CPz=0.0):
        self.lib.orc_fluid_set_params(self.h, visc, CPx, CPy, CPz)

    def set_field(self, which, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        assert a.size == int(np.prod(self.shape))
        if self.lib.orc_fluid_set_field(self.h, int(which), a.ctypes.data):
            raise RuntimeError("orc_fluid_set_field failed")

    def get_field(self, which):
        out = np.empty(self.shape, np.float64)
        if self.lib.orc_fluid_get_field(self.h, int(which), out.ctypes.data):
            raise RuntimeError("orc_fluid_get_field failed")
        return out

    def StoreOldVelocity(self):
        self.lib.orc_fluid_StoreOldVelocity(self.h)

    def VelocityGuess(self, aRK, bRK, cRK):
        self.lib.orc_fluid_VelocityGuess(self.h, aRK, bRK, cRK)

    def FillGhostRegionForFluid(self):
        self.lib.orc_fluid_FillGhostRegionForFluid(self.h)

    def Boundary(self):
        self.lib.orc_fluid_Boundary(self.h)

    def ModifyBulkVelocity(self, swU, swV, swW, bulkU, bulkV, bulkW):
        self.lib.orc_fluid_ModifyBulkVelocity(self.h, swU, swV, swW, bulkU, bulkV, bulkW)

    def VelocityDivergence(self, cRK):
        self.lib.orc_fluid_VelocityDivergence(self.h, cRK)

    def PressureCorrection(self):
        self.lib.orc_fluid_PressureCorrection(self.h)

    def VelocityCorrection(self, cRK):
        self.lib.orc_fluid_VelocityCorrection(self.h, cRK)

    def PressureOperator(self, p):
        """The reference's pressure-correction matrix (with the pinned row)
        applied to the field p: the interior of the result, halo zero."""
        p = np.ascontiguousarray(p, dtype=np.float64)
        assert p.shape == tuple(self.shape)
        out = np.zeros(self.shape, np.float64)
        self.lib.orc_fluid_PressureOperator(self.h, p.ctypes.data, out.ctypes.data)
        return out
