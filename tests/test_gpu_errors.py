"""Error paths and edge cases through the C ABI: every failure comes back as a
status code with a message, and the context stays usable.  Nothing here makes
a GPU fault: bad inputs are rejected on the host or flagged by the kernels'
own bounds checks."""
import numpy as np
import pytest

import cases
from ibmdem import api, scenario
from ibmdem.records import MULTISPHERE, PARCEL, make_params

pytestmark = pytest.mark.gpu

ERANGE, ECAPACITY, ESTATE = -4, -5, -7


def test_parcels_outside_the_region_or_nan_are_rejected(gpu_lib):
    p, parts, bodies, field = cases.contact_case(seed=2)
    case = api.Case(p, None, bodies, field)
    for bad in (np.nan, np.inf, -5.0, 1e9):
        q = parts.copy()
        q["x"][7, 1] = bad
        with pytest.raises(api.IbmDemError) as e:
            case.set_parcels(q)
        assert e.value.code == ERANGE
    case.set_parcels(parts)  # still usable
    case.InitializationDEM()
    case.step(1)
    case.close()


def test_calls_out_of_order_report_state(gpu_lib):
    p, parts, bodies, field = cases.contact_case(seed=2)
    case = api.Case(p, parts, bodies, field)
    with pytest.raises(api.IbmDemError) as e:
        case.MultiDirectForcing()
    assert e.value.code == ESTATE
    with pytest.raises(api.IbmDemError) as e:
        case.CalculateCollisionForce()
    assert e.value.code == ESTATE
    case.InitializationDEM()
    case.MultiDirectForcing()
    case.close()


def test_empty_case_steps(gpu_lib, oracle_mod):
    p = make_params(16, 16, 16)
    z = [np.zeros((20, 20, 20)) for _ in range(3)]
    case = api.Case(p, np.zeros(0, PARCEL), np.zeros(0, MULTISPHERE), z)
    case.InitializationDEM()
    case.step(2)
    parts, nl = case.get_parcels()
    assert len(parts) == 0 and nl == 0
    u, v, w, fx, fy, fz = case.get_fluid()
    assert not fx.any() and np.array_equal(u, z[0])
    case.close()


def test_body_at_a_box_corner_matches_oracle(gpu_lib, oracle_mod):
    """A sphere centred near (0, 0, 0) has markers in all 8 octants of the
    periodic box: images of every one of the 7 shift classes."""
    n = 24
    p = make_params(n, n, n)
    X = np.array([[0.4, 23.7, 0.9], [12.0, 11.5, 12.3]])
    V = np.array([[0.01, -0.02, 0.015], [0.0, 0.01, -0.01]])
    parts, bodies = scenario.sphere_bodies(X, 8.0, 1.0, 1.14e3, V)
    parts["x"] = scenario.wrap_coord(parts["x"], np.array([n, n, n], float))
    field = scenario.fourier_field(p, 6, 0.02, seed=4)
    g = api.Case(p, parts, bodies, field)
    r = oracle_mod.OracleCase(p, parts, bodies, field)
    for c in (g, r):
        c.InitializationDEM()
        c.step(2)
    gp, gnl = g.get_parcels()
    rp, rnl = r.get_parcels()
    assert gnl == rnl and len(gp) == len(rp) and len(gp) > gnl
    assert np.array_equal(g.get_cell_lists()[1], r.get_cell_lists()[1])
    assert cases.rel_close(gp["x"], rp["x"], 1e-12)
    gf, rf = g.get_fluid(), r.get_fluid()
    for a, b in zip(gf, rf):
        assert cases.rel_close(a, b, 1e-9)
    g.close()
    r.close()


def test_unresolved_contact_capacity_and_range(gpu_lib):
    p, parts, field = scenario.unresolved_case(16, 4000, seed=3, n_modes=0, bed_spacing=0.9, maxContacts=1)
    u = api.Unresolved(p, parts, field)
    u.step(1)
    with pytest.raises(api.IbmDemError) as e:
        u.synchronize()
    assert e.value.code == ECAPACITY
    q = parts.copy()
    q["x"][3, 2] = np.nan
    with pytest.raises(api.IbmDemError) as e:
        u.set_particles(q)
    assert e.value.code == ERANGE
    u.close()
