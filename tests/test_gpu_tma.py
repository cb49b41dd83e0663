"""The TMA column stage (gf_set_tma_columns) against the per-thread-copy column kernel.

Both run the same FFT passes (same radix, twiddles and butterfly order) and the same stage
epilogue; the two kernels are compiled separately, so the compiler may fuse multiply-adds
differently and the states agree to rounding (FP32 1e-6, FP64 and df64 1e-13 relative L2
after 12 steps), not bit for bit.  The test compares them after calls that mix unobserved
steps (pruned columns) and observed ones, for every
column count the context offers, in FP32, FP64 and df64, for TwoDNavierStokes, SingleLayerQG
(beta, stochastic forcing, finite deformation radius, topography with U) and SurfaceQG, on
square and rectangular grids and for a batch of instances.  One case also checks the TMA
path against the FP64 oracle directly."""
import numpy as np
import pytest

import gf_oracle as O

pytestmark = pytest.mark.gpu

gfcuda = pytest.importorskip("gfcuda")
from gfcuda import SingleLayerQG as SL, SurfaceQG as SQ, TwoDNavierStokes as TD  # noqa: E402
from gfcuda import Forcing, stepforward  # noqa: E402


def cands(T, prec):
    return (2, 4) if (T == np.float32) else (1, 2)


def close(a, b, T):
    return O.rel_l2(a, b) <= (1e-6 if T == np.float32 else 1e-13)


def zeta0(nx, ny, seed, B=None):
    g = O.Grid(nx, 2 * np.pi, ny, 2 * np.pi)
    z = [O.peakedisotropicspectrum(g, 5, 0.5, seed=seed + i) for i in range(B or 1)]
    return np.stack(z) if B else z[0]


def run(make, setup, C, R, nsteps=(5, 1, 6)):
    p = make()
    shape = list(p.launch_shape)
    shape[2] = R
    p.launch_shape = shape
    p.tma_columns = C
    assert p.tma_columns == C
    setup(p)
    for n in nsteps:
        stepforward(p, n)
    sol = p.sol
    p.close()
    return sol


CASES = {
    "twodns": lambda nx, ny, T, prec, B: (
        lambda: TD.Problem("GPU", nx=nx, ny=ny, dt=0.002, nu=1e-4, nnu=1, stepper="FilteredRK4", T=T,
                           precision=prec, batch=B or 1),
        lambda p: TD.set_zeta(p, zeta0(nx, ny, 3, B))),
    "slqg_forced": lambda nx, ny, T, prec, B: (
        lambda: SL.Problem("GPU", nx=nx, ny=ny, beta=10.0, mu=0.01, dt=0.01, stepper="ETDRK4", T=T, precision=prec,
                           batch=B or 1, forcing=Forcing("stochastic",
                                                    spectrum=O.ring_forcing_spectrum(O.Grid(nx, 2 * np.pi, ny, 2 * np.pi),
                                                                                     10.0, 1.5, 1e-3), seed=9)),
        lambda p: SL.set_q(p, 0.1 * zeta0(nx, ny, 4, B))),
    "slqg_topo": lambda nx, ny, T, prec, B: (
        lambda: SL.Problem("GPU", nx=nx, ny=ny, deformation_radius=0.35, U=0.2, beta=1.0, dt=0.01,
                           eta=0.1 * np.cos(np.linspace(0, 2 * np.pi, nx, endpoint=False))[None, :] * np.ones((ny, 1)),
                           stepper="ETDRK4", T=T, precision=prec, batch=B or 1),
        lambda p: SL.set_q(p, zeta0(nx, ny, 5, B))),
    "sqg": lambda nx, ny, T, prec, B: (
        lambda: SQ.Problem("GPU", nx=nx, ny=ny, dt=0.002, nu=1e-4, nnu=1, stepper="RK4", T=T, precision=prec,
                           batch=B or 1),
        lambda p: SQ.set_b(p, zeta0(nx, ny, 6, B))),
}


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("T,prec,R", [(np.float32, None, 16), (np.float32, None, 8), (np.float64, "DF64", 8),
                                      (np.float64, None, 8)])
def test_tma_column_stage_equals_copy_kernel(case, T, prec, R):
    nx, ny = 256, 256
    make, setup = CASES[case](nx, ny, T, prec, None)
    ref = run(make, setup, 0, R)
    for C in cands(T, prec):
        got = run(make, setup, C, R)
        assert close(got, ref, T), (case, C, O.rel_l2(got, ref))


@pytest.mark.parametrize("nx,ny", [(512, 128), (128, 512), (2048, 2048)])
@pytest.mark.parametrize("T,prec,R", [(np.float32, None, 16), (np.float64, "DF64", 8)])
def test_tma_rectangular_and_large(nx, ny, T, prec, R):
    make, setup = CASES["twodns"](nx, ny, T, prec, None)
    ref = run(make, setup, 0, R, nsteps=(3, 1))
    for C in cands(T, prec):
        assert close(run(make, setup, C, R, nsteps=(3, 1)), ref, T), C


@pytest.mark.parametrize("T,prec", [(np.float32, None), (np.float64, None)])
def test_tma_batch_of_instances(T, prec):
    make, setup = CASES["slqg_forced"](128, 128, T, prec, 3)
    ref = run(make, setup, 0, 8)
    for C in cands(T, prec):
        assert close(run(make, setup, C, 8), ref, T), C


def test_tma_fp64_against_oracle():
    n, dt = 128, 0.005
    r = O.TwoDNavierStokes(nx=n, dt=dt, nu=1e-4, nnu=1, stepper="FilteredRK4")
    z0 = zeta0(n, n, 7)
    r.set_zeta(z0)
    p = TD.Problem("GPU", nx=n, dt=dt, nu=1e-4, nnu=1, stepper="FilteredRK4", T=np.float64)
    p.tma_columns = 2
    TD.set_zeta(p, z0)
    for _ in range(4):
        stepforward(p, 5)
        r.stepforward(5)
        assert O.rel_l2(p.sol, r.sol) <= 1e-12
    p.synchronize()
    p.close()


def test_tma_columns_rejected_where_not_supported():
    from gfcuda import MultiLayerQG as ML
    p = ML.Problem(2, "GPU", nx=64, ny=64, H=[0.2, 0.8], b=[-1.0, -1.2], T=np.float32)
    with pytest.raises(gfcuda.GFError):
        p.tma_columns = 2
    p.close()
    q = TD.Problem("GPU", nx=64, T=np.float32)
    with pytest.raises(gfcuda.GFError):
        q.tma_columns = 3
    q.close()
