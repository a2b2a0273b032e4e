"""The CPU restatement of the fluid stencils (oracle/fluid_oracle.c) on cases
with known answers: a uniform stream and a linear pressure (VelocityGuess),
a shear flow (exactly divergence-free on the staggered grid), the halo fill
against numpy's wrap-around and wall mirrors, the Boundary zeroing, and the
bulk-velocity shift reaching its target."""
import numpy as np
import pytest

from ibmdem import records

F = records.FLUID


@pytest.fixture
def fluid(oracle_mod):
    made = []

    def make(nx=8, ny=6, nz=5, walls="", dt=1e-3, rhof=1e3, h=1.0):
        p = records.make_params(nx, ny, nz, h=h, dt=dt, rhof=rhof, walls=walls)
        f = oracle_mod.OracleFluid(p)
        made.append(f)
        return f

    yield make
    for f in made:
        f.close()


def interior(a):
    return a[2:-2, 2:-2, 2:-2]


def test_uniform_stream_and_linear_pressure(fluid):
    f = fluid()
    shape = f.shape
    U0 = 0.3
    f.set_field(F["u"], np.full(shape, U0))
    f.set_field(F["uold"], np.full(shape, U0))
    # P = 0.5 * i along x (Fortran order: the last numpy axis is x)
    P = np.broadcast_to(0.5 * np.arange(shape[2], dtype=np.float64), shape).copy()
    f.set_field(F["P"], P)
    f.set_fluid_params(visc=1e-3, CPx=0.02)
    f.VelocityGuess(1.0, 0.0, 1.0)
    px = 0.5 / 1.0 / 1e3
    assert np.all(interior(f.get_field(F["Px"])) == px)
    # no convection or diffusion of a uniform stream: u = uold + dt*(CPx - Px)
    want = U0 + 1e-3 * (1.0 * (0.0 + 0.0 + 0.02 + 0.0) + 0.0 * 0.0 - 1.0 * px)
    assert np.all(interior(f.get_field(F["u"])) == want)
    assert np.all(interior(f.get_field(F["RHSul"])) == 0.02)
    assert np.all(interior(f.get_field(F["v"])) == 0.0)


def test_shear_flow_is_divergence_free(fluid):
    f = fluid()
    shape = f.shape
    y = np.arange(shape[1], dtype=np.float64)
    u = np.broadcast_to(np.sin(0.7 * y)[None, :, None], shape).copy()
    f.set_field(F["u"], u)
    f.VelocityDivergence(1.0)
    assert np.all(interior(f.get_field(F["velDiv"])) == 0.0)
    f.VelocityCorrection(1.0)
    # omegaZ = (v(i+1)-v)/dx - (u(j+1)-u)/dy
    oz = interior(f.get_field(F["omegaZ"]))
    want = -(np.sin(0.7 * (y[3:-1])) - np.sin(0.7 * y[2:-2]))
    assert np.array_equal(oz, np.broadcast_to(want[None, :, None], oz.shape))


@pytest.mark.parametrize("walls", ["", "z", "xyz"])
def test_halo_fill(fluid, walls):
    f = fluid(walls=walls)
    shape = f.shape
    rng = np.random.default_rng(3)
    fields = {}
    for name in ("u", "v", "w", "P", "omegaZ", "Pcorr"):
        a = np.zeros(shape)
        a[2:-2, 2:-2, 2:-2] = rng.standard_normal((shape[0] - 4, shape[1] - 4, shape[2] - 4))
        fields[name] = a
        f.set_field(F[name], a)
    f.FillGhostRegionForFluid()
    for name, a in fields.items():
        got = f.get_field(F[name])
        want = a[2:-2, 2:-2, 2:-2]
        # numpy axes (z, y, x); a periodic axis wraps, a walled one mirrors about
        # the face with u,v,w negated
        for ax, name_ax in enumerate("zyx"):
            if name_ax in walls:
                sign = -1.0 if name in ("u", "v", "w") else 1.0
                lo = np.flip(np.take(want, [0, 1], axis=ax), axis=ax) * sign
                hi = np.flip(np.take(want, [-2, -1], axis=ax), axis=ax) * sign
                want = np.concatenate([lo, want, hi], axis=ax)
            else:
                want = np.concatenate([np.take(want, [-2, -1], axis=ax), want, np.take(want, [0, 1], axis=ax)],
                                      axis=ax)
        assert np.array_equal(got, want), name


def test_boundary_zeroes_wall_normal_velocity(fluid):
    f = fluid(walls="z")
    shape = f.shape
    f.set_field(F["w"], np.ones(shape))
    f.set_field(F["u"], np.ones(shape))
    f.Boundary()
    w = f.get_field(F["w"])
    # w(:,:,lg3:sg3) = 0 and w(:,:,eg3+1:ug3) = 0: numpy z rows 0..2 and nz+3..nz+4
    assert np.all(w[:3] == 0.0) and np.all(w[-2:] == 0.0) and np.all(w[3:-2] == 1.0)
    assert np.all(f.get_field(F["u"]) == 1.0)


def test_bulk_velocity_reaches_target(fluid):
    f = fluid()
    rng = np.random.default_rng(5)
    f.set_field(F["u"], rng.standard_normal(f.shape))
    f.ModifyBulkVelocity(1, 0, 0, 0.1, 0.0, 0.0)
    assert abs(interior(f.get_field(F["u"])).mean() - 0.1) < 1e-12


def test_pressure_operator_known_answers(fluid):
    """The restated matrix: a constant lies in the Laplacian's null space (every
    row but the pinned identity row gives 0), and a Fourier mode of a periodic
    box is an eigenvector away from the pinned node and its neighbours."""
    for walls in ("", "z", "xyz"):
        f = fluid(walls=walls, h=0.5)
        shape = f.shape
        out = interior(f.PressureOperator(np.full(shape, 3.0)))
        want = np.zeros_like(out)
        want[0, 0, 0] = 3.0
        assert np.allclose(out, want, atol=1e-12), walls
    f = fluid(nx=8, ny=6, nz=5)
    # cos(2 pi x / 8) along x (the period of the interior), x the 0-based
    # interior index; the halo holds the periodic continuation
    x = np.arange(f.shape[2], dtype=np.float64) - 2.0
    p = np.broadcast_to(np.cos(2 * np.pi * x / 8.0), f.shape).copy()
    out = interior(f.PressureOperator(p))
    lam = 2.0 - 2.0 * np.cos(2 * np.pi / 8.0)
    want = lam * interior(p)
    want[0, 0, 0] = interior(p)[0, 0, 0]
    assert np.allclose(out, want, rtol=0, atol=1e-13)


@pytest.mark.parametrize("walls,h", [("", 1.0), ("z", 1.0), ("xyz", 0.7), ("y", 0.5)])
def test_fft_solution_satisfies_the_reference_system(fluid, walls, h):
    """The numpy FFT solve used by the GPU Poisson test solves the restated
    system far below the reference's KSP tolerance (1e-10, run.sh)."""
    import fft_poisson

    f = fluid(nx=8, ny=6, nz=5, walls=walls, h=h)
    rng = np.random.default_rng(11)
    b = rng.standard_normal(tuple(n - 4 for n in f.shape))
    p = fft_poisson.solve(b, (h, h, h), walls)
    full = np.zeros(f.shape)
    full[2:-2, 2:-2, 2:-2] = p
    rhs = b.copy()
    rhs[0, 0, 0] = 0.0
    res = interior(f.PressureOperator(full)) - rhs
    assert np.linalg.norm(res) <= 1e-12 * np.linalg.norm(rhs)
    assert p[0, 0, 0] == 0.0
