"""ibmdem_update_fluid_async: the sparse read-out leaves the caller's arrays
equal, bit for bit, to a full ibmdem_get_fluid after each MultiDirectForcing,
over several coupled steps (the arrays are fed back through ibmdem_set_fluid),
periodic and between walls, while CloudEvolutionMS runs beside the copies."""
import ctypes

import numpy as np
import pytest

import cases
from ibmdem import scenario

pytestmark = pytest.mark.gpu


def pinned_copy(a):
    import torch
    t = torch.empty(a.shape, dtype=torch.float64, pin_memory=True).numpy()
    t[...] = a
    return t


@pytest.mark.parametrize("kind", ["periodic", "walls"])
def test_sparse_readout_equals_full(gpu_lib, kind):
    import torch
    if kind == "periodic":
        p, parts, bodies, field = cases.contact_case(seed=9)
    else:
        p, parts, bodies, field = scenario.walled_case(24, 24, 24, 4, 8.0, seed=3, walls="z", n_modes=8)
    case = gpu_lib.Case(p, parts, bodies, field, device=0)
    case.InitializationDEM()
    u = [pinned_copy(f) for f in field]
    fo = [pinned_copy(np.zeros_like(field[0])) for _ in range(3)]
    s = torch.cuda.Stream()
    ptr = lambda a: ctypes.c_void_p(a.ctypes.data)  # noqa: E731
    for step in range(4):
        case._chk(case.lib.ibmdem_set_fluid(case.h, *[ptr(a) for a in u]), "set_fluid")
        case.MultiDirectForcing()
        full = case.get_fluid()
        case._chk(case.lib.ibmdem_update_fluid_async(case.h, *[ptr(a) for a in u + fo],
                                                      ctypes.c_void_p(s.cuda_stream)), "update_fluid_async")
        case.CloudEvolutionMS()
        case._chk(case.lib.ibmdem_update_fluid_wait(case.h), "update_fluid_wait")
        for a, b in zip(u + fo, full):
            assert np.array_equal(a, b), step
        nb = ctypes.c_int64()
        case.lib.ibmdem_update_fluid_bytes(case.h, ctypes.byref(nb))
        # a count and 20 bytes per touched node, far below the six fields
        assert nb.value > 4 and (nb.value - 4) % 20 == 0
        assert nb.value < 6 * full[0].nbytes // 4
    case.close()


def test_async_upload_equals_sync(gpu_lib):
    """ibmdem_set_fluid_async (each component's forcing loop starts when that
    component has arrived) and ibmdem_get_fluid_async (each component leaves
    when done) give the fields of the synchronous calls bit for bit, over
    coupled steps that feed the fields back."""
    import torch
    p, parts, bodies, field = cases.contact_case(seed=11)
    a = gpu_lib.Case(p, parts, bodies, field, device=0)
    b = gpu_lib.Case(p, parts, bodies, field, device=0)
    for c in (a, b):
        c.InitializationDEM()
    ua = [pinned_copy(f) for f in field]
    ub = [pinned_copy(f) for f in field]
    outb = [pinned_copy(np.zeros_like(field[0])) for _ in range(6)]
    s = torch.cuda.Stream()
    ptr = lambda x: ctypes.c_void_p(x.ctypes.data)  # noqa: E731
    for step in range(3):
        a._chk(a.lib.ibmdem_set_fluid(a.h, *[ptr(x) for x in ua]), "set_fluid")
        a.MultiDirectForcing()
        fa = a.get_fluid()
        a.CloudEvolutionMS()
        b._chk(b.lib.ibmdem_set_fluid_async(b.h, *[ptr(x) for x in ub]), "set_fluid_async")
        b.MultiDirectForcing()
        b._chk(b.lib.ibmdem_get_fluid_async(b.h, *[ptr(x) for x in outb], ctypes.c_void_p(s.cuda_stream)),
               "get_fluid_async")
        b.CloudEvolutionMS()
        gb = b.get_bodies()
        s.synchronize()
        for x, y in zip(fa, outb):
            assert np.array_equal(x, y), step
        assert np.array_equal(a.get_bodies()["x"], gb["x"])
        for x, y, z in zip(ua, ub, fa[:3]):
            x[...] = z
            y[...] = z
    a.close()
    b.close()
