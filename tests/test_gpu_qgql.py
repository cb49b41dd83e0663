"""BarotropicQGQL on the GPU through the C ABI: calcN!, steps and updatevars! against the
oracle, and the reference's own tests (test/test_barotropicqgql.jl) run on the device."""
import numpy as np
import pytest

import gf_oracle as O
from test_oracle_qgql import qgql_advection_case
from test_oracle_reference import isapprox

pytestmark = pytest.mark.gpu

gfcuda = pytest.importorskip("gfcuda")
from gfcuda import BarotropicQGQL as QL  # noqa: E402
from gfcuda import Diagnostic, Forcing, stepforward  # noqa: E402


def rel(a, b):
    return O.rel_l2(a, b)


@pytest.mark.parametrize("T,prec,tol", [(np.float64, None, 1e-12), (np.float64, "DF64", 1e-12),
                                        (np.float32, None, 3e-6)])
def test_qgql_calcN_and_updatevars_match_oracle(T, prec, tol):
    n = 128
    rng = np.random.default_rng(4)
    kw = dict(nx=n, beta=2.0, nu=1e-3, nnu=1, mu=0.05)
    p, r = QL.Problem("GPU", T=T, precision=prec, **kw), O.BarotropicQGQL(**kw)
    sol = np.fft.rfft2(rng.standard_normal((n, n)))
    N_gpu, _ = p.calcN(sol, 0.0)
    N_ref = np.zeros_like(sol)
    r.calcN(N_ref, sol.copy(), 0.0)
    assert rel(N_gpu, N_ref) <= tol
    z = rng.standard_normal((n, n))
    QL.set_zeta(p, z)
    r.set_zeta(z)
    for name in ("zeta", "Zeta", "psi", "Psi", "u", "v", "U"):
        assert rel(getattr(p.vars, name), getattr(r, name)) <= max(tol, 1e-13), name


@pytest.mark.parametrize("stepper,dt,nsteps", [
    ("ETDRK4", 1e-2, 20), ("FilteredETDRK4", 1e-2, 20), ("RK4", 1e-2, 20), ("FilteredRK4", 1e-2, 20),
    ("AB3", 1e-3, 200), ("FilteredAB3", 1e-3, 200), ("ForwardEuler", 1e-4, 2000), ("FilteredForwardEuler", 1e-4, 2000)])
def test_qgql_rossbywave_gpu(stepper, dt, nsteps):
    """test/test_barotropicqgql.jl:1-44"""
    nx, beta = 64, 2.0
    p = QL.Problem("GPU", nx=nx, beta=beta, stepper=stepper, dt=dt)
    x, y = p.grid.gridpoints()
    ampl, kw, lw = 1e-2, 3.0, 2.0
    w = -beta * kw / (kw ** 2 + lw ** 2)
    QL.set_zeta(p, ampl * np.cos(kw * x) * np.cos(lw * y))
    stepforward(p, nsteps)
    QL.updatevars(p)
    zt = ampl * np.cos(kw * (x - w / kw * p.clock.t)) * np.cos(lw * y)
    assert isapprox(zt, p.vars.zeta, nx * nx * nsteps * 1e-12)


def test_qgql_advection_manufactured_gpu():
    """test/test_barotropicqgql.jl:144-190 on the device (rtol 1e-13)"""
    n, dt = 128, 0.0005
    qf, Fh, nu = qgql_advection_case(n)
    p = QL.Problem("GPU", nx=n, nu=nu, nnu=1, dt=dt, stepper="ForwardEuler", forcing=Forcing("static", Fh=Fh))
    QL.set_zeta(p, qf)
    stepforward(p, round(1.0 / dt))
    QL.updatevars(p)
    assert isapprox(p.vars.zeta + p.vars.Zeta, qf, 1e-13)


def test_qgql_energy_enstrophy_gpu():
    """test/test_barotropicqgql.jl:192-222 at 64 x 64, Ly = 3 pi"""
    nx, Lx, ny, Ly = 64, 2 * np.pi, 64, 3 * np.pi
    k0, l0 = 2 * np.pi / Lx, 2 * np.pi / Ly
    p = QL.Problem("GPU", nx=nx, Lx=Lx, ny=ny, Ly=Ly, stepper="ForwardEuler",
                   eta=np.zeros((ny, nx)))
    x, y = p.grid.gridpoints()
    z0 = (-((2 * k0) ** 2 + (2 * l0) ** 2) * np.sin(2 * k0 * x) * np.cos(2 * l0 * y)
          - (k0 ** 2 + (3 * l0) ** 2) * 2 * np.sin(k0 * x) * np.cos(3 * l0 * y))
    QL.set_zeta(p, z0)
    assert abs(QL.energy(p) - 29 / 9) <= 1e-13 * 29 / 9
    assert abs(QL.enstrophy(p) - 2701 / 162) <= 1e-13 * 2701 / 162


@pytest.mark.parametrize("kind", ["deterministic", "stochastic"])
def test_qgql_budgets_gpu(kind):
    """test/test_barotropicqgql.jl:46-142 on the device, diagnostics streamed per step"""
    n, L, nu, nnu, mu = 256, 2 * np.pi, 1e-7, 2, 1e-1
    dt = 0.005
    nt = round(0.1 / mu / dt)
    g = O.Grid(n, L)
    if kind == "stochastic":
        Kr = np.broadcast_to(g.kr, g.Krsq.shape)
        spec = np.exp(-(np.sqrt(g.Krsq) - 12.0) ** 2 / (2 * 2.0 ** 2))
        spec[g.Krsq < 4] = 0
        spec[g.Krsq > 400] = 0
        spec[Kr < 2 * np.pi / L] = 0
        spec = 0.1 / (O.parsevalsum(spec * g.invKrsq / 2, g) / (g.Lx * g.Ly)) * spec
        forcing = Forcing("stochastic_phase", spectrum=spec, seed=1234)
    else:
        x, y = g.gridpoints()
        forcing = Forcing("harmonic", Fh=O.rfft2(0.01 * np.cos(4 * x) * np.cos(5 * y)), omega=2.0)
    p = QL.Problem("GPU", nx=n, Lx=L, nu=nu, nnu=nnu, mu=mu, dt=dt, stepper="RK4", forcing=forcing)
    QL.set_zeta(p, np.zeros((n, n)))
    E, D, R, W = (Diagnostic(f, p) for f in (QL.energy, QL.dissipation, QL.drag, QL.work))
    stepforward(p, [E, D, R, W], nt)
    E, D, R, W = (np.asarray(d.data) for d in (E, D, R, W))
    if kind == "stochastic":
        assert isapprox((E[1:] - E[:-1]) / dt, W[1:] - D[:-1] - R[:-1], 1e-3)
    else:
        assert isapprox((E[2:] - E[:-2]) / (2 * dt), W[1:-1] - D[1:-1] - R[1:-1], atol=1e-10)


@pytest.mark.parametrize("stepper", ["FilteredRK4", "ETDRK4", "AB3"])
def test_qgql_steps_match_oracle(stepper):
    n, dt = 128, 0.005
    spec = O.ring_forcing_spectrum(O.Grid(n), 10.0, 1.5, 1e-3)
    kw = dict(nx=n, beta=3.0, nu=1e-3, nnu=1, mu=0.02, dt=dt, stepper=stepper)
    p = QL.Problem("GPU", forcing=Forcing("stochastic", spectrum=spec, seed=8), **kw)
    r = O.BarotropicQGQL(forcing=O.Forcing("stochastic", spectrum=spec, seed=8), **kw)
    z0 = O.peakedisotropicspectrum(O.Grid(n), 6, 0.5, seed=2)
    QL.set_zeta(p, z0)
    r.set_zeta(z0)
    stepforward(p, 15)
    r.stepforward(15)
    assert rel(p.sol, r.sol) <= 15e-12
    assert abs(QL.energy(p) - r.energy()) <= 1e-11 * r.energy()
