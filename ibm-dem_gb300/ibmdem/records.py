"""Record layouts of the C ABI (include/ibmdem.h) as numpy dtypes.

`PARCEL` mirrors `type Parcel` (ZJS_VARS.F90:6-12) and `MULTISPHERE` mirrors
`type MultiSphere` (ZJS_VARS.F90:97-102); `PARAMS` carries the constants the
reference hard-codes in source.  Sizes are checked against the C structs when
the library loads.
"""
import numpy as np

PARCEL = np.dtype([
    ("globalIdx", "<i4"), ("localIdx", "<i4"), ("cellIdx", "<i4"), ("pType", "<i4"),
    ("MSIdx", "<i4"), ("pad_", "<i4"),
    ("radeff", "<f8"), ("rad", "<f8"), ("rho", "<f8"), ("vol", "<f8"), ("m", "<f8"),
    ("x", "<f8", 3), ("v", "<f8", 3), ("fcol", "<f8", 3), ("fdrag", "<f8", 3), ("vgap", "<f8", 3),
    ("wdrag", "<f8"), ("wsum", "<f8"),
])
assert PARCEL.itemsize == 200

MULTISPHERE = np.dtype([
    ("globalIdx", "<i4"), ("cpuIdx", "<i4"),
    ("rotMat", "<f8", 9), ("rotMatGlo", "<f8", 9), ("rotMatGloOld", "<f8", 9), ("InertiaTensor", "<f8", 9),
    ("x", "<f8", 3), ("xold", "<f8", 3), ("v", "<f8", 3), ("vold", "<f8", 3), ("omega", "<f8", 3),
    ("omegaold", "<f8", 3), ("fcol", "<f8", 3), ("fmom", "<f8", 3), ("fdrag", "<f8", 3),
    ("AngMom", "<f8", 3), ("AngMomOld", "<f8", 3), ("fhydro", "<f8", 3), ("fmomHydro", "<f8", 3),
    ("fmomCol", "<f8", 3),
    ("I", "<f8"), ("rad", "<f8"), ("rho", "<f8"), ("vol", "<f8"), ("m", "<f8"),
])
assert MULTISPHERE.itemsize == 672

PARAMS = np.dtype([
    ("nx", "<i4"), ("ny", "<i4"), ("nz", "<i4"), ("coupleInterval", "<i4"), ("Ns", "<i4"),
    ("bType", "<i4", 6), ("pad_", "<i4"),
    ("dx", "<f8"), ("dy", "<f8"), ("dz", "<f8"), ("dt", "<f8"), ("rhof", "<f8"),
    ("knCoeff", "<f8"), ("ResistCoeff", "<f8"), ("collisionDist", "<f8"), ("collisionBuffer", "<f8"),
    ("gravity", "<f8", 3),
])
assert PARAMS.itemsize == 144

# type WallColProbe (ZJS_VARS.F90:92-94): a quadrilateral on a wall face (1..6)
WALL_PROBE = np.dtype([("face", "<i4"), ("pad_", "<i4"), ("points", "<f8", (4, 3)), ("force", "<f8", 3)])
assert WALL_PROBE.itemsize == 128
MAX_WALL_PROBES = 60


def make_params(nx, ny, nz, h=1.0, dt=1e-3, coupleInterval=1, Ns=5, rhof=1e3, knCoeff=1e4,
                ResistCoeff=0.9, collisionBuffer=0.1, gravity=(0.0, 0.0, -9.81), collisionDist=None,
                walls=""):
    """Case parameters; collisionDist defaults to dx*0.75*2 (ZJS_INIT_DEM.F90:413).

    `walls` names the axes bounded by two solid walls (bType 1), e.g. "z";
    the others are periodic (bType 0)."""
    p = np.zeros((), PARAMS)
    p["nx"], p["ny"], p["nz"] = nx, ny, nz
    p["coupleInterval"], p["Ns"] = coupleInterval, Ns
    p["bType"] = [1 if "xxyyzz"[f] in walls else 0 for f in range(6)]
    p["dx"] = p["dy"] = p["dz"] = h
    p["dt"], p["rhof"], p["knCoeff"], p["ResistCoeff"] = dt, rhof, knCoeff, ResistCoeff
    p["collisionDist"] = h * 0.75 * 2 if collisionDist is None else collisionDist
    p["collisionBuffer"] = collisionBuffer
    p["gravity"] = gravity
    return p


# fields of the fluid stencils (IBMDEM_FLUID_* of include/ibmdem.h)
FLUID_FIELDS = ["u", "v", "w", "fx", "fy", "fz", "uold", "vold", "wold", "P", "Pcorr", "velDiv",
                "Px", "Py", "Pz", "RHSul", "RHSvl", "RHSwl", "omegaX", "omegaY", "omegaZ"]
FLUID = {name: i for i, name in enumerate(FLUID_FIELDS)}


def field_shape(p):
    """(nk, nj, ni) C-order view of a Fortran (lg1:ug1, lg2:ug2, lg3:ug3) array."""
    return (int(p["nz"]) + 4, int(p["ny"]) + 4, int(p["nx"]) + 4)


# unresolved CFD-DEM path (point particles); no counterpart record in the reference
PARTICLE = np.dtype([
    ("globalIdx", "<i4"), ("pad_", "<i4"),
    ("rad", "<f8"), ("rho", "<f8"), ("vol", "<f8"), ("m", "<f8"), ("I", "<f8"),
    ("x", "<f8", 3), ("v", "<f8", 3), ("omega", "<f8", 3),
    ("fcol", "<f8", 3), ("tcol", "<f8", 3), ("fdrag", "<f8", 3), ("alphaf", "<f8"),
])
assert PARTICLE.itemsize == 200

UPARAMS = np.dtype([
    ("nx", "<i4"), ("ny", "<i4"), ("nz", "<i4"), ("maxContacts", "<i4"),
    ("dx", "<f8"), ("dcell", "<f8"), ("dt", "<f8"), ("rhof", "<f8"), ("viscf", "<f8"),
    ("knCoeff", "<f8"), ("ResistCoeff", "<f8"), ("ktRatio", "<f8"), ("mu", "<f8"),
    ("bandwidth", "<f8"), ("alphaMin", "<f8"), ("gravity", "<f8", 3),
])
assert UPARAMS.itemsize == 128


def make_uparams(nx, ny, nz, dx, dcell, dt=1e-5, rhof=1.2, viscf=1e-5, knCoeff=1e4, ResistCoeff=0.9,
                 ktRatio=2.0 / 7.0, mu=0.3, bandwidth=3.0, alphaMin=0.2, maxContacts=16,
                 gravity=(0.0, 0.0, -9.81)):
    """Unresolved-path parameters (viscf defaults to the reference's 1e-5, ZJS_VARS.F90:77)."""
    p = np.zeros((), UPARAMS)
    p["nx"], p["ny"], p["nz"], p["maxContacts"] = nx, ny, nz, maxContacts
    p["dx"], p["dcell"], p["dt"], p["rhof"], p["viscf"] = dx, dcell, dt, rhof, viscf
    p["knCoeff"], p["ResistCoeff"], p["ktRatio"], p["mu"] = knCoeff, ResistCoeff, ktRatio, mu
    p["bandwidth"], p["alphaMin"], p["gravity"] = bandwidth, alphaMin, gravity
    return p


def ufield_shape(p):
    """Fluid array shape of an unresolved case (same layout as field_shape)."""
    return (int(p["nz"]) + 4, int(p["ny"]) + 4, int(p["nx"]) + 4)
