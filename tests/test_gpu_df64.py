"""GPU parity of the FP64-plain mode computed in double-float arithmetic (precision="DF64"):
the same oracle comparisons as the FP64 path, at the task's FP64 bar of 1e-12 relative L2 per
step, and the reference's known-answer tests at 1e-12 (df64 carries a 48-bit significand)."""
import math

import numpy as np
import pytest

import gf_oracle as O

pytestmark = pytest.mark.gpu

gfcuda = pytest.importorskip("gfcuda")
from gfcuda import MultiLayerQG as ML, SingleLayerQG as SL, SurfaceQG as SQ, TwoDNavierStokes as TD  # noqa: E402
from gfcuda import Forcing, stepforward  # noqa: E402

TOL = 1e-12


def rel(a, b):
    return O.rel_l2(a, b)


def ic(n, filt):
    return O.peakedisotropicspectrum(O.Grid(n), 6, 0.5, mask=filt, seed=1234)


@pytest.mark.parametrize("n", [128, 512])
def test_df64_fft_matches_numpy(n):
    rng = np.random.default_rng(3)
    p = TD.Problem("GPU", nx=n, ny=n // 2, precision="DF64")
    f = rng.standard_normal((n // 2, n))
    assert rel(p.fwdtransform(f), np.fft.rfft2(f)) <= 1e-13
    assert rel(p.invtransform(np.fft.rfft2(f)), f) <= 1e-13


@pytest.mark.parametrize("module", ["TwoDNavierStokes", "SurfaceQG", "SingleLayerQG"])
def test_df64_calcN_matches_oracle(module):
    rng = np.random.default_rng(4)
    n = 128
    if module == "TwoDNavierStokes":
        p, r = TD.Problem("GPU", nx=n, precision="DF64"), O.TwoDNavierStokes(nx=n)
    elif module == "SurfaceQG":
        p, r = SQ.Problem("GPU", nx=n, H=1.3, precision="DF64"), O.SurfaceQG(nx=n, H=1.3)
    else:
        x, y = O.Grid(n).gridpoints()
        eta = 0.3 * np.cos(3 * x) * np.sin(2 * y)
        kw = dict(nx=n, beta=2.0, U=0.4, eta=eta, deformation_radius=1.5)
        p, r = SL.Problem("GPU", precision="DF64", **kw), O.SingleLayerQG(**kw)
    sol = np.fft.rfft2(rng.standard_normal((n, n)))
    N_gpu, _ = p.calcN(sol, 0.0)
    N_ref = np.zeros_like(sol)
    r.calcN(N_ref, sol.copy(), 0.0)
    assert rel(N_gpu, N_ref) <= TOL


@pytest.mark.parametrize("n", [128, 512])
def test_df64_filteredrk4_single_step_parity(n):
    dt = 0.005 * 128 / n
    r = O.TwoDNavierStokes(nx=n, dt=dt, stepper="FilteredRK4")
    r.set_zeta(ic(n, r.timestepper.filter))
    r.stepforward(10)
    p = TD.Problem("GPU", nx=n, dt=dt, stepper="FilteredRK4", precision="DF64")
    for _ in range(3):
        p.sol = r.sol
        p.set_clock(r.clock.t, r.clock.step)
        stepforward(p, 1)
        r.stepforward(1)
        assert rel(p.sol, r.sol) <= TOL


def test_df64_decaying_128_100_steps():
    n, dt = 128, 0.005
    r = O.TwoDNavierStokes(nx=n, dt=dt, stepper="FilteredRK4")
    z0 = ic(n, r.timestepper.filter)
    r.set_zeta(z0)
    p = TD.Problem("GPU", nx=n, dt=dt, stepper="FilteredRK4", precision="DF64")
    TD.set_zeta(p, z0)
    r.stepforward(100)
    stepforward(p, 100)
    assert rel(p.sol, r.sol) <= 100 * TOL
    assert abs(TD.energy(p) - r.energy()) <= 1e-11 * r.energy()
    assert abs(TD.enstrophy(p) - r.enstrophy()) <= 1e-11 * r.enstrophy()


def test_df64_known_answers_and_manufactured_solution():
    """test/test_twodnavierstokes.jl:221-317 on the df64 path (bar 1e-12)"""
    nx, Lx, ny, Ly = 128, 2 * np.pi, 128, 3 * np.pi
    p = TD.Problem("GPU", nx=nx, Lx=Lx, ny=ny, Ly=Ly, stepper="ForwardEuler", precision="DF64")
    x, y = p.grid.gridpoints()
    k0, l0 = 2 * np.pi / Lx, 2 * np.pi / Ly
    z0 = (-((2 * k0) ** 2 + (2 * l0) ** 2) * np.sin(2 * k0 * x) * np.cos(2 * l0 * y)
          - (k0 ** 2 + (3 * l0) ** 2) * 2 * np.sin(k0 * x) * np.cos(3 * l0 * y))
    TD.set_zeta(p, z0)
    assert abs(TD.energy(p) - 29 / 9) <= TOL * 29 / 9
    assert abs(TD.enstrophy(p) - 2701 / 162) <= TOL * 2701 / 162
    n, nu, dt = 128, 1e-2, 0.0005
    x, y = O.Grid(n).gridpoints()
    zf = -8 * np.sin(2 * x) * np.cos(2 * y) - 20 * np.sin(x) * np.cos(3 * y)
    Ff = -(nu * (64 * np.sin(2 * x) * np.cos(2 * y) + 200 * np.sin(x) * np.cos(3 * y))
           + 8 * (np.cos(x) * np.cos(3 * y) * np.sin(2 * x) * np.sin(2 * y)
                  - 3 * np.cos(2 * x) * np.cos(2 * y) * np.sin(x) * np.sin(3 * y)))
    p = TD.Problem("GPU", nx=n, nu=nu, dt=dt, stepper="ForwardEuler", forcing=Forcing("static", Fh=O.rfft2(Ff)),
                   precision="DF64")
    TD.set_zeta(p, zf)
    stepforward(p, round(1.0 / dt))
    TD.updatevars(p)
    assert rel(p.vars.zeta, zf) <= TOL


@pytest.mark.parametrize("stepper", ["ETDRK4", "FilteredETDRK4", "RK4", "AB3"])
def test_df64_slqg_steppers_and_stochastic_forcing(stepper):
    n, dt = 128, 0.02
    g = O.Grid(n)
    spec = O.ring_forcing_spectrum(g, 14.0, 1.5, 1e-3)
    f = Forcing("stochastic", spectrum=spec, seed=9)
    kw = dict(nx=n, beta=10.0, mu=0.01, nu=1e-6, nnu=2, dt=dt, stepper=stepper)
    p = SL.Problem("GPU", forcing=f, precision="DF64", **kw)
    r = O.SingleLayerQG(forcing=O.Forcing("stochastic", spectrum=spec, seed=9), **kw)
    stepforward(p, 10)
    r.stepforward(10)
    assert rel(p.sol, r.sol) <= 10 * TOL
    assert abs(SL.energy(p) - r.energy()) <= 1e-11 * r.energy()


def test_df64_mlqg_etdrk4_parity():
    n, nl = 128, 3
    rng = np.random.default_rng(6)
    kw = dict(nx=n, f0=1.0, beta=5.0, H=[0.2, 0.3, 0.5], b=[-1.0, -1.2, -1.290909], U=[1.0, 0.5, 0.0], mu=0.05,
              dt=2.5e-3, stepper="ETDRK4")
    p, r = ML.Problem(nl, "GPU", precision="DF64", **kw), O.MultiLayerQG(nl, **kw)
    q0 = 1e-2 * rng.standard_normal((nl, n, n))
    ML.set_q(p, q0)
    r.set_q(q0)
    stepforward(p, 10)
    r.stepforward(10)
    assert rel(p.sol, r.sol) <= 10 * TOL


def test_df64_sqg_known_answer():
    """test/test_surfaceqg.jl:72-106 (H = 1) on the df64 path"""
    H, nx, Lx, ny, Ly = 1.0, 128, 2 * np.pi, 128, 3 * np.pi
    p = SQ.Problem("GPU", nx=nx, Lx=Lx, ny=ny, Ly=Ly, H=H, stepper="ForwardEuler", precision="DF64")
    x, y = p.grid.gridpoints()
    k0, l0 = 2 * np.pi / Lx, 2 * np.pi / Ly
    K1, K2 = math.sqrt((2 * k0) ** 2 + (2 * l0) ** 2), math.sqrt(k0 ** 2 + (3 * l0) ** 2)
    t1, t2 = math.tanh(K1 * H), math.tanh(K2 * H)
    b0 = -K1 * t1 * np.sin(2 * k0 * x) * np.cos(2 * l0 * y) - K2 * t2 * 2 * np.sin(k0 * x) * np.cos(3 * l0 * y)
    SQ.set_b(p, b0)
    ke = (K1 ** 2 + 4 * K2 ** 2) / 8
    assert abs(SQ.kinetic_energy(p) - ke) <= TOL * ke
