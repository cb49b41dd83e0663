"""The field-parallel small-grid kernels (gf_set_field_parallel): one thread group per field,
FFT radix 2, 4 or 8, against the classic row and column kernels and the FP64 oracle.

Same products, stage epilogue and PV inversion per element as the classic kernels; the
transforms differ in their radix, so states agree to rounding: FP32 1e-5, FP64 and df64
1e-13 relative L2 after calls that mix unobserved steps (pruned columns) and observed ones.
Covered: every radix and column count, TwoDNavierStokes, SingleLayerQG (beta, stochastic
forcing, finite deformation radius, topography with U, PV-gradient products), SurfaceQG and
BarotropicQGQL (three product fields), square and rectangular grids of 32 ... 512, a batch,
the steppers' stage epilogues, calcN!, the adjoint's forward recompute, and the default
selection rule."""
import numpy as np
import pytest

import gf_oracle as O

pytestmark = pytest.mark.gpu

gfcuda = pytest.importorskip("gfcuda")
from gfcuda import BarotropicQGQL as QL, MultiLayerQG as ML, SingleLayerQG as SL  # noqa: E402
from gfcuda import SurfaceQG as SQ, TwoDNavierStokes as TD  # noqa: E402
from gfcuda import Forcing, adjoint, stepforward  # noqa: E402

CLASSIC = (8, 1, 8, 1)


def tol(T):
    return 1e-5 if T == np.float32 else 1e-13


def zeta0(nx, ny, seed, B=None):
    g = O.Grid(nx, 2 * np.pi, ny, 2 * np.pi)
    z = [O.peakedisotropicspectrum(g, 5, 0.5, seed=seed + i) for i in range(B or 1)]
    return np.stack(z) if B else z[0]


CASES = {
    "twodns": lambda nx, ny, T, prec, B, st: (
        lambda: TD.Problem("GPU", nx=nx, ny=ny, dt=0.002, nu=1e-4, nnu=1, stepper=st or "FilteredRK4", T=T,
                           precision=prec, batch=B or 1),
        lambda p: TD.set_zeta(p, zeta0(nx, ny, 3, B))),
    "slqg_forced": lambda nx, ny, T, prec, B, st: (
        lambda: SL.Problem("GPU", nx=nx, ny=ny, beta=10.0, mu=0.01, dt=0.01, stepper=st or "ETDRK4", T=T,
                           precision=prec, batch=B or 1,
                           forcing=Forcing("stochastic", spectrum=O.ring_forcing_spectrum(
                               O.Grid(nx, 2 * np.pi, ny, 2 * np.pi), 6.0, 1.5, 1e-3), seed=9)),
        lambda p: SL.set_q(p, 0.1 * zeta0(nx, ny, 4, B))),
    "slqg_topo": lambda nx, ny, T, prec, B, st: (
        lambda: SL.Problem("GPU", nx=nx, ny=ny, deformation_radius=0.35, U=0.2, beta=1.0, dt=0.01,
                           eta=0.1 * np.cos(np.linspace(0, 2 * np.pi, nx, endpoint=False))[None, :] * np.ones((ny, 1)),
                           stepper=st or "ETDRK4", T=T, precision=prec, batch=B or 1),
        lambda p: SL.set_q(p, zeta0(nx, ny, 5, B))),
    "sqg": lambda nx, ny, T, prec, B, st: (
        lambda: SQ.Problem("GPU", nx=nx, ny=ny, dt=0.002, nu=1e-4, nnu=1, stepper=st or "RK4", T=T, precision=prec,
                           batch=B or 1),
        lambda p: SQ.set_b(p, zeta0(nx, ny, 6, B))),
    "qgql": lambda nx, ny, T, prec, B, st: (
        lambda: QL.Problem("GPU", nx=nx, ny=ny, beta=2.0, nu=1e-3, nnu=1, mu=0.05, dt=0.005,
                           stepper=st or "FilteredRK4", T=T, precision=prec, batch=B or 1),
        lambda p: QL.set_zeta(p, zeta0(nx, ny, 7, B))),
}


def run(make, setup, fp, nsteps=(5, 1, 6)):
    """fp = (row radix, column radix, columns), or None for the classic kernels"""
    p = make()
    if fp is None:
        p.launch_shape = CLASSIC
        assert p.field_parallel == (0, 0, 0)
    else:
        p.field_parallel = fp
        assert p.field_parallel == fp
    setup(p)
    for n in nsteps:
        stepforward(p, n)
    sol = p.sol
    p.close()
    return sol


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("T,prec", [(np.float32, None), (np.float64, None), (np.float64, "DF64")])
def test_field_parallel_equals_classic(case, T, prec):
    n = 128
    make, setup = CASES[case](n, n, T, prec, None, None)
    ref = run(make, setup, None)
    for fp in ((2, 2, 1), (4, 4, 1), (8, 8, 1), (4, 2, 2), (2, 8, 2)):
        got = run(make, setup, fp)
        assert O.rel_l2(got, ref) <= tol(T), (case, fp, O.rel_l2(got, ref))


@pytest.mark.parametrize("nx,ny", [(32, 32), (64, 128), (256, 64), (256, 256), (512, 512)])
@pytest.mark.parametrize("T,prec", [(np.float32, None), (np.float64, "DF64")])
def test_field_parallel_sizes(nx, ny, T, prec):
    make, setup = CASES["slqg_forced"](nx, ny, T, prec, None, None)
    ref = run(make, setup, None, nsteps=(4, 1))
    for fp in ((2, 2, 1), (4, 4, 2), (8, 8, 4), (4, 8, 1)):
        try:
            got = run(make, setup, fp, nsteps=(4, 1))
        except ValueError:  # block too large: rejected
            assert 3 * (nx // fp[0]) > 384 or 3 * fp[2] * (ny // fp[1]) > 384
            continue
        assert O.rel_l2(got, ref) <= tol(T), (nx, ny, fp)


@pytest.mark.parametrize("stepper", ["ForwardEuler", "RK4", "AB3", "FilteredETDRK4", "FilteredAB3"])
def test_field_parallel_steppers(stepper):
    make, setup = CASES["twodns"](64, 64, np.float64, None, None, stepper)
    ref = run(make, setup, None)
    assert O.rel_l2(run(make, setup, (4, 4, 1)), ref) <= 1e-13


def test_field_parallel_batch_of_instances():
    make, setup = CASES["slqg_forced"](64, 64, np.float64, None, 3, None)
    ref = run(make, setup, None)
    assert O.rel_l2(run(make, setup, (2, 4, 2)), ref) <= 1e-13


@pytest.mark.parametrize("prec", [None, "DF64"])
def test_field_parallel_against_oracle(prec):
    """the benchmark's small case: TwoDNavierStokes 128^2 FilteredRK4 from the peaked
    isotropic state, with the default (field-parallel) kernels, against the FP64 oracle"""
    n, dt = 128, 0.005
    r = O.TwoDNavierStokes(nx=n, dt=dt, stepper="FilteredRK4")
    z0 = O.peakedisotropicspectrum(r.grid, 6, 0.5, mask=r.timestepper.filter, seed=1234)
    r.set_zeta(z0)
    p = TD.Problem("GPU", nx=n, dt=dt, stepper="FilteredRK4", T=np.float64, precision=prec)
    assert p.field_parallel[0] > 0 and p.field_parallel[1] > 0
    TD.set_zeta(p, z0)
    for _ in range(4):
        stepforward(p, 25)
        r.stepforward(25)
        assert O.rel_l2(p.sol, r.sol) <= 1e-12
    assert abs(TD.energy(p) - r.energy()) <= 1e-12 * abs(r.energy())
    p.close()


def test_calcN_field_parallel():
    n = 64
    rng = np.random.default_rng(3)
    sol = np.fft.rfft2(rng.standard_normal((n, n)))
    out = []
    for fp in (None, (2, 4, 1)):
        p = SL.Problem("GPU", nx=n, beta=3.0, deformation_radius=0.5, T=np.float64)
        if fp is None:
            p.launch_shape = CLASSIC
        else:
            p.field_parallel = fp
        out.append(p.calcN(sol, 0.0)[0])
        p.close()
    assert O.rel_l2(out[1], out[0]) <= 1e-13


def test_adjoint_with_field_parallel_forward():
    """the gradient through the field-parallel forward recompute equals the classic one"""
    n, ns = 64, 8
    z0 = zeta0(n, n, 11)
    res = []
    for fp in (None, (4, 4, 1)):
        p = TD.Problem("GPU", nx=n, dt=0.01, nu=1e-3, nnu=1, stepper="ETDRK4", T=np.float64)
        if fp is None:
            p.launch_shape = CLASSIC
        else:
            p.field_parallel = fp
        TD.set_zeta(p, z0)
        res.append(adjoint.grad(p, ns, checkpoint_every=3))
        p.close()
    (l0, g0, _), (l1, g1, _) = res
    assert abs(l1 - l0) <= 1e-13 * abs(l0) and O.rel_l2(g1, g0) <= 1e-12


def test_default_selection_and_rejection():
    p = TD.Problem("GPU", nx=128, T=np.float64)   # 64 row pairs: field-parallel
    assert p.field_parallel == (4, 2, 1)
    r = TD.Problem("GPU", nx=256, T=np.float64)
    assert r.field_parallel == (4, 4, 1)
    r.close()
    p.launch_shape = CLASSIC                        # an explicit launch shape: classic kernels
    assert p.field_parallel == (0, 0, 0)
    p.field_parallel = (2, 8, 2)
    p.tma_columns = 1                               # the TMA column stage: classic column kernel
    assert p.field_parallel == (2, 0, 0)
    with pytest.raises(ValueError):
        p.field_parallel = (3, 4, 1)                # radix
    with pytest.raises(ValueError):
        p.field_parallel = (4, 2, 4)                # 3 x 4 x 64 threads > 384
    p.close()
    q = TD.Problem("GPU", nx=64, T=np.float32, batch=8)   # 256 row pairs: classic
    assert q.field_parallel == (0, 0, 0)
    q.close()
    big = TD.Problem("GPU", nx=512, T=np.float32)   # 256 row pairs: classic by default
    assert big.field_parallel == (0, 0, 0)
    with pytest.raises(ValueError):
        big.field_parallel = (2, 4, 1)              # radix 2 at 512: 3 x 256 threads > 384
    big.field_parallel = (4, 8, 1)
    big.close()
    huge = TD.Problem("GPU", nx=1024, T=np.float32)
    with pytest.raises(gfcuda.GFError):
        huge.field_parallel = (4, 4, 1)             # lengths above 512
    huge.close()
    m = ML.Problem(2, "GPU", nx=64, H=[0.3, 0.7], b=[-1.0, -1.4], T=np.float64)
    assert m.field_parallel == (0, 0, 0)
    with pytest.raises(gfcuda.GFError):
        m.field_parallel = (4, 4, 1)                # several layers
    m.close()


def test_observed_and_unobserved_steps_field_parallel():
    """a call of 12 steps equals 12 single-step calls bit for bit with the field-parallel
    kernels too (unobserved steps skip the aliased modes only)"""
    make, setup = CASES["slqg_forced"](128, 128, np.float64, None, None, None)
    a = run(make, setup, (4, 4, 1), nsteps=(12,))
    b = run(make, setup, (4, 4, 1), nsteps=(1,) * 12)
    assert np.array_equal(a, b)
