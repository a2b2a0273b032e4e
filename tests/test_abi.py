"""The C-ABI library loads and exports every entry point include/ibmdem.h
declares, and the Python record dtypes match the C struct layouts (checked by
compiling a probe against the header).  No GPU is needed: nothing is called
that touches a device."""
import ctypes
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "ibmdem.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(ibmdem_\w+)\s*\(", src)))


def test_header_declares_the_reference_subroutines():
    names = declared_functions()
    for sub in ("RebuildAllListOrNot", "UpdateLocalCellWeightListDEM", "UpdateGhostCellWeightListDEM",
                "UpdateParcelInfoInGhostRegion", "CalculateCollisionForce",
                "UpdateFluidVelocityOnLagrangianPoints", "UpdateMomentumSourceTerm", "VelocityPostGuess",
                "AssembleLocalForceMS", "EvolutionMS", "ResetVelocityAndPositionLagrangianPoints",
                "AdjustParcelPosition", "InitializationDEM", "CloudEvolutionStepMS", "CloudEvolutionMS"):
        assert "ibmdem_" + sub in names, sub


def test_library_exports_every_declared_symbol(gpu_lib):
    lib = ctypes.CDLL(gpu_lib.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    assert set(gpu_lib.EXPORTS) <= set(declared_functions())
    assert lib.ibmdem_abi_version() == 1


def test_record_layouts_match_the_header():
    from ibmdem.records import MULTISPHERE, PARAMS, PARCEL

    probe = r"""
#include <stdio.h>
#include <stddef.h>
#include "ibmdem.h"
#define F(T, f) printf("%s %s %zu\n", #T, #f, offsetof(T, f));
int main(void) {
  printf("sizes %zu %zu %zu\n", sizeof(ibmdem_parcel), sizeof(ibmdem_multisphere), sizeof(ibmdem_params));
  F(ibmdem_parcel, MSIdx) F(ibmdem_parcel, radeff) F(ibmdem_parcel, x) F(ibmdem_parcel, fdrag)
  F(ibmdem_parcel, wsum)
  F(ibmdem_multisphere, rotMat) F(ibmdem_multisphere, InertiaTensor) F(ibmdem_multisphere, x)
  F(ibmdem_multisphere, fmomCol) F(ibmdem_multisphere, I) F(ibmdem_multisphere, m)
  F(ibmdem_params, bType) F(ibmdem_params, dx) F(ibmdem_params, collisionBuffer) F(ibmdem_params, gravity)
  return 0;
}
"""
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "probe.c")
        exe = os.path.join(d, "probe")
        open(c, "w").write(probe)
        subprocess.run(["gcc", "-I", os.path.dirname(HEADER), c, "-o", exe], check=True)
        out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split("\n")
    sizes = out[0].split()[1:]
    assert [int(x) for x in sizes] == [PARCEL.itemsize, MULTISPHERE.itemsize, PARAMS.itemsize]
    dt = {"ibmdem_parcel": PARCEL, "ibmdem_multisphere": MULTISPHERE, "ibmdem_params": PARAMS}
    for line in out[1:]:
        if not line:
            continue
        T, f, off = line.split()
        assert dt[T].fields[f][1] == int(off), (T, f)


def test_oracle_library_builds_and_loads(oracle_mod):
    lib = oracle_mod._load()
    for n in ("orc_create", "orc_step", "orc_InitializationDEM", "orc_CalculateDragForce"):
        assert hasattr(lib, n)


def test_create_rejects_unsupported_parameters(oracle_mod):
    from ibmdem.records import make_params

    p = make_params(16, 16, 16)
    p["bType"][2] = 1  # a wall on one face of an axis whose other face is periodic
    with pytest.raises(ValueError):
        oracle_mod.OracleCase(p)
    p = make_params(2, 16, 16)
    with pytest.raises(ValueError):
        oracle_mod.OracleCase(p)


def test_null_handles_are_rejected(gpu_lib):
    """No CUDA call is made for a null handle, so this runs without a GPU."""
    import ctypes
    lib = ctypes.CDLL(gpu_lib.LIB_PATH)
    for name in ("ibmdem_synchronize", "ibmdem_step", "ibmdem_MultiDirectForcing", "ibmdem_batch_step",
                 "ibmdem_server_poll", "ibmdem_unresolved_step", "ibmdem_destroy", "ibmdem_batch_destroy",
                 "ibmdem_server_destroy", "ibmdem_unresolved_destroy"):
        f = getattr(lib, name)
        rc = f(None, 1) if name.endswith("_step") else f(None, None) if name == "ibmdem_server_poll" else f(None)
        assert rc == -1, name
    lib.ibmdem_last_error.restype = ctypes.c_char_p
    assert lib.ibmdem_last_error(None) == b"null context"


def test_compiled_caller_builds_against_the_header():
    """The compiled coupled caller (run on the GPU by test_gpu_c_caller.py)
    compiles against the header without warnings."""
    src = os.path.join(os.path.dirname(os.path.abspath(__file__)), "c_caller", "coupled_step.c")
    with tempfile.TemporaryDirectory() as d:
        subprocess.run(["gcc", "-Wall", "-Wextra", "-Werror", "-I", os.path.dirname(HEADER), "-c", src, "-o",
                        os.path.join(d, "coupled_step.o")], check=True)
