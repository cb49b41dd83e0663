"""The oracle's BarotropicQGQL through the reference's own tests
(test/test_barotropicqgql.jl, called at test/runtests.jl:90-107), at the reference's sizes
and tolerances."""
import numpy as np
import pytest

import gf_oracle as O
from test_oracle_reference import isapprox


def qgql_rossbywave(stepper, dt, nsteps):
    """test/test_barotropicqgql.jl:1-44"""
    nx, beta = 64, 2.0
    p = O.BarotropicQGQL(nx=nx, Lx=2 * np.pi, beta=beta, stepper=stepper, dt=dt)
    g = p.grid
    x, y = g.gridpoints()
    ampl, kw, lw = 1e-2, 3 * 2 * np.pi / g.Lx, 2 * 2 * np.pi / g.Ly
    w = -beta * kw / (kw ** 2 + lw ** 2)
    p.set_zeta(ampl * np.cos(kw * x) * np.cos(lw * y))
    p.stepforward(nsteps)
    O.dealias(p.sol, g)
    p.updatevars()
    zt = ampl * np.cos(kw * (x - w / kw * p.clock.t)) * np.cos(lw * y)
    return isapprox(zt, p.zeta, g.nx * g.ny * nsteps * 1e-12)


@pytest.mark.parametrize("stepper,dt,nsteps", [
    ("ETDRK4", 1e-2, 20), ("FilteredETDRK4", 1e-2, 20), ("RK4", 1e-2, 20), ("FilteredRK4", 1e-2, 20),
    ("AB3", 1e-3, 200), ("FilteredAB3", 1e-3, 200), ("ForwardEuler", 1e-4, 2000), ("FilteredForwardEuler", 1e-4, 2000)])
def test_qgql_rossbywave(stepper, dt, nsteps):
    assert qgql_rossbywave(stepper, dt, nsteps)


def qgql_budget(kind, n=256):
    """test/test_barotropicqgql.jl:46-142 (energy budget with stochastic / deterministic forcing)"""
    L, nu, nnu, mu = 2 * np.pi, 1e-7, 2, 1e-1
    dt, tf = 0.005, 0.1 / mu
    nt = round(tf / dt)
    g = O.Grid(n, L)
    if kind == "stochastic":
        kf, dkf, eps = 12.0, 2.0, 0.1
        Kr = np.broadcast_to(g.kr, g.Krsq.shape)
        spec = np.exp(-(np.sqrt(g.Krsq) - kf) ** 2 / (2 * dkf ** 2))
        spec[g.Krsq < 4] = 0
        spec[g.Krsq > 400] = 0
        spec[Kr < 2 * np.pi / L] = 0
        spec = eps / (O.parsevalsum(spec * g.invKrsq / 2, g) / (g.Lx * g.Ly)) * spec
        forcing = O.Forcing("stochastic_phase", spectrum=spec, seed=1234)
    else:
        x, y = g.gridpoints()
        forcing = O.Forcing("harmonic", Fh=O.rfft2(0.01 * np.cos(4 * x) * np.cos(5 * y)), omega=2.0)
    p = O.BarotropicQGQL(nx=n, Lx=L, nu=nu, nnu=nnu, mu=mu, dt=dt, stepper="RK4", forcing=forcing)
    p.set_zeta(np.zeros((n, n)))
    E, D, R, W = [p.energy()], [p.dissipation()], [p.drag()], [p.work()]
    for _ in range(nt):
        p.stepforward()
        E.append(p.energy()); D.append(p.dissipation()); R.append(p.drag()); W.append(p.work())
    E, D, R, W = map(np.array, (E, D, R, W))
    if kind == "stochastic":
        return isapprox((E[1:] - E[:-1]) / dt, W[1:] - D[:-1] - R[:-1], 1e-3)
    return isapprox((E[2:] - E[:-2]) / (2 * dt), W[1:-1] - D[1:-1] - R[1:-1], atol=1e-10)


@pytest.mark.parametrize("kind", ["deterministic", "stochastic"])
def test_qgql_budgets(kind):
    assert qgql_budget(kind)


def qgql_advection_case(n=128):
    x, y = O.Grid(n).gridpoints()
    nu = 1e-2
    qf = -9 * np.cos(3 * y) - 8 * np.sin(2 * x) * np.cos(2 * y) - 20 * np.sin(x) * np.cos(3 * y)
    Ff = (nu * (81 * np.cos(3 * y) + 200 * np.cos(3 * y) * np.sin(x) + 64 * np.cos(2 * y) * np.sin(2 * x))
          - 3 * np.sin(3 * y) * (-16 * np.cos(2 * x) * np.cos(2 * y) - 20 * np.cos(x) * np.cos(3 * y))
          - 27 * np.sin(3 * y) * (2 * np.cos(2 * x) * np.cos(2 * y) + 2 * np.cos(x) * np.cos(3 * y)))
    return qf, -O.rfft2(Ff), nu


def test_qgql_advection_manufactured():
    """test/test_barotropicqgql.jl:144-190 (ForwardEuler dt = 5e-4 to t = 1, rtol 1e-13)"""
    n, dt = 128, 0.0005
    qf, Fh, nu = qgql_advection_case(n)
    p = O.BarotropicQGQL(nx=n, nu=nu, nnu=1, dt=dt, stepper="ForwardEuler", forcing=O.Forcing("static", Fh=Fh))
    p.set_zeta(qf)
    p.stepforward(round(1.0 / dt))
    p.updatevars()
    assert isapprox(p.zeta + p.Zeta, qf, 1e-13)


def test_qgql_energy_enstrophy():
    """test/test_barotropicqgql.jl:192-222"""
    nx, Lx, ny, Ly = 64, 2 * np.pi, 64, 3 * np.pi
    g = O.Grid(nx, Lx, ny, Ly)
    k0, l0 = 2 * np.pi / Lx, 2 * np.pi / Ly
    x, y = g.gridpoints()
    eta = np.cos(10 * k0 * x) * np.cos(10 * l0 * y)
    z0 = (-((2 * k0) ** 2 + (2 * l0) ** 2) * np.sin(2 * k0 * x) * np.cos(2 * l0 * y)
          - (k0 ** 2 + (3 * l0) ** 2) * 2 * np.sin(k0 * x) * np.cos(3 * l0 * y))
    p = O.BarotropicQGQL(nx=nx, Lx=Lx, ny=ny, Ly=Ly, eta=eta, stepper="ForwardEuler")
    p.set_zeta(z0)
    assert abs(p.energy() - 29 / 9) <= 1e-13 * 29 / 9
    assert abs(p.enstrophy() - 2701 / 162) <= 1e-13 * 2701 / 162
