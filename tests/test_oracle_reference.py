"""Pins the FP64 oracle against the reference's own known-answer tests.

Each test restates one test of GeophysicalFlows.jl v0.16.5 (file:line cited) with the
reference's tolerance; the Julia RNG draws of the budget tests are replaced by Philox draws
(the budget closure holds for any draw).
"""
import math

import numpy as np
import pytest

import gf_oracle as O

RTOL = 1e-13  # test/runtests.jl:21-25


def isapprox(a, b, rtol=0.0, atol=0.0):
    a, b = np.asarray(a, dtype=np.complex128), np.asarray(b, dtype=np.complex128)
    return np.linalg.norm((a - b).ravel()) <= max(atol, rtol * max(np.linalg.norm(a.ravel()), np.linalg.norm(b.ravel())))


# --------------------------------------------------------------------- grid semantics
def test_grid_and_dealias_ranges():
    g = O.Grid(128)
    assert g.x[0] == -math.pi and abs(g.x[-1] - (math.pi - g.dx)) < 1e-15
    assert list(g.kralias[[0, -1]]) == [42, 64]
    assert list(g.lalias[[0, -1]]) == [42, 85]
    f = O.makefilter(g)
    assert f[0, 0] == 1.0 and f[0, -1] < 1e-14


def test_parsevalsum_matches_physical_sum():
    rng = np.random.default_rng(0)
    for nx, ny in ((16, 12), (15, 10), (32, 32)):
        g = O.Grid(nx, 2.0, ny, 3.0)
        f = rng.standard_normal((ny, nx))
        fh = O.rfft2(f)
        assert abs(O.parsevalsum2(fh, g) - np.sum(f ** 2) * g.dx * g.dy) < 1e-12 * np.sum(f ** 2)


# --------------------------------------------------------------------- TwoDNavierStokes
def test_twodns_energy_enstrophy_palinstrophy():
    """test/test_twodnavierstokes.jl:259-317"""
    nx, Lx, ny, Ly = 128, 2 * np.pi, 126, 3 * np.pi
    p = O.TwoDNavierStokes(nx=nx, Lx=Lx, ny=ny, Ly=Ly, stepper="ForwardEuler")
    x, y = p.grid.gridpoints()
    k0, l0 = 2 * np.pi / Lx, 2 * np.pi / Ly
    z0 = (-((2 * k0) ** 2 + (2 * l0) ** 2) * np.sin(2 * k0 * x) * np.cos(2 * l0 * y)
          - (k0 ** 2 + (3 * l0) ** 2) * 2 * np.sin(k0 * x) * np.cos(3 * l0 * y))
    p.set_zeta(z0)
    assert isapprox(p.energy(), 29 / 9, RTOL)
    assert isapprox(p.enstrophy(), 2701 / 162, RTOL)
    assert isapprox(p.palinstrophy(), 126277 / 1458, RTOL)


def test_twodns_lambdipole():
    """test/test_twodnavierstokes.jl:1-23 (n = 256, dt = 1e-3, runtests.jl:44): a Lamb dipole of
    speed Ue = 1 and radius L/20 (src/utils.jl:8-20), FilteredRK4, nu = 0; the |zeta|-weighted
    centroid moves at Ue within rtol_lambdipole = 1e-2 over three intervals of round(0.01 L /
    Ue / dt) steps, the speed taken as the centroid shift over (nt - 1) dt as in the reference."""
    L, n, dt, Ue = 2 * math.pi, 256, 1e-3, 1.0
    nt, nm = round(L / Ue * 0.01 / dt), 3
    r = O.TwoDNavierStokes(nx=n, Lx=L, nu=0.0, nnu=1, dt=dt, stepper="FilteredRK4")
    r.set_zeta(O.lambdipole(Ue, L / 20, r.grid))
    x, _ = r.grid.gridpoints()
    xz, um = np.zeros(nm), np.zeros(nm)
    for i in range(nm):
        r.stepforward(nt)
        r.updatevars()
        a = np.abs(r.zeta)
        xz[i] = np.mean(a * x) / np.mean(a)
        if i > 0:
            um[i] = (xz[i] - xz[i - 1]) / ((nt - 1) * dt)
    assert isapprox(Ue, np.mean(um[1:]), rtol=1e-2)


def test_twodns_advection_manufactured():
    """test/test_twodnavierstokes.jl:221-257 (ForwardEuler dt=5e-4, 2000 steps, rtol 1e-13)"""
    n, L, nu, nnu, dt = 128, 2 * np.pi, 1e-2, 1, 0.0005
    g = O.Grid(n, L)
    x, y = g.gridpoints()
    zf = -8 * np.sin(2 * x) * np.cos(2 * y) - 20 * np.sin(x) * np.cos(3 * y)
    Ff = -(nu * (64 * np.sin(2 * x) * np.cos(2 * y) + 200 * np.sin(x) * np.cos(3 * y))
           + 8 * (np.cos(x) * np.cos(3 * y) * np.sin(2 * x) * np.sin(2 * y)
                  - 3 * np.cos(2 * x) * np.cos(2 * y) * np.sin(x) * np.sin(3 * y)))
    p = O.TwoDNavierStokes(nx=n, Lx=L, nu=nu, nnu=nnu, dt=dt, stepper="ForwardEuler",
                           forcing=O.Forcing("static", Fh=O.rfft2(Ff)))
    p.set_zeta(zf)
    p.stepforward(round(1.0 / dt))
    p.updatevars()
    assert isapprox(p.zeta, zf, RTOL)


def _twodns_budget(kind, which):
    """test/test_twodnavierstokes.jl:25-208 (energy/enstrophy budgets, RK4)"""
    n, L, nu, nnu, mu, nmu = 256, 2 * np.pi, 1e-7, 2, 1e-1, 0
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
        e0 = O.parsevalsum(spec * (g.invKrsq / 2 if which == "energy" else 0.5), g) / (g.Lx * g.Ly)
        spec = eps / e0 * spec
        forcing = O.Forcing("stochastic_phase", spectrum=spec, seed=1234)
    else:
        x, y = g.gridpoints()
        forcing = O.Forcing("harmonic", Fh=O.rfft2(0.01 * np.cos(4 * x) * np.cos(5 * y)), omega=2.0)
    p = O.TwoDNavierStokes(nx=n, Lx=L, nu=nu, nnu=nnu, mu=mu, nmu=nmu, dt=dt, stepper="RK4",
                           forcing=forcing)
    p.set_zeta(np.zeros((n, n)))
    f = {"energy": (p.energy, p.energy_dissipation_hyperviscosity, p.energy_dissipation_hypoviscosity, p.energy_work),
         "enstrophy": (p.enstrophy, p.enstrophy_dissipation_hyperviscosity, p.enstrophy_dissipation_hypoviscosity, p.enstrophy_work)}[which]
    E, D, R, W = [f[0]()], [f[1]()], [f[2]()], [f[3]()]
    for _ in range(nt):
        p.stepforward()
        E.append(f[0]()); D.append(f[1]()); R.append(f[2]()); W.append(f[3]())
    E, D, R, W = map(np.array, (E, D, R, W))
    if kind == "stochastic":
        num = (E[1:] - E[:-1]) / dt
        comp = W[1:] + D[:-1] + R[:-1]
        return isapprox(num, comp, 1e-3)
    num = (E[2:] - E[:-2]) / (2 * dt)
    comp = W[1:-1] + D[1:-1] + R[1:-1]
    return isapprox(num, comp, 1e-4)


@pytest.mark.parametrize("kind", ["deterministic", "stochastic"])
@pytest.mark.parametrize("which", ["energy", "enstrophy"])
def test_twodns_budgets(kind, which):
    assert _twodns_budget(kind, which)


# --------------------------------------------------------------------- SingleLayerQG
def rossbywave(stepper, dt, nsteps, nx=64, ell=np.inf, U=0.0, U_array=False):
    """test/test_singlelayerqg.jl:8-46 with parameters test/runtests.jl:57-65"""
    Lx, beta = 2 * np.pi, 2.0
    Uarg = np.full(nx, U) if U_array else U
    p = O.SingleLayerQG(nx=nx, Lx=Lx, deformation_radius=ell, beta=beta, U=Uarg, stepper=stepper, dt=dt)
    g = p.grid
    x, y = g.gridpoints()
    ampl, kw, lw = 1e-2, 3 * 2 * np.pi / g.Lx, 2 * 2 * np.pi / g.Ly
    w = -beta * kw / (kw ** 2 + lw ** 2 + (0 if np.isinf(ell) else 1 / ell ** 2))
    p.set_q(ampl * np.cos(kw * x) * np.cos(lw * y))
    p.stepforward(nsteps)
    O.dealias(p.sol, g)
    p.updatevars()
    qt = ampl * np.cos(kw * (x - (U + w / kw) * p.clock.t)) * np.cos(lw * y)
    return isapprox(qt, p.q, g.nx * g.ny * nsteps * 1e-12)


ROSSBY = list(zip(O.STEPPERS[::1], ()))


@pytest.mark.parametrize("stepper,dt,nsteps", [
    ("ETDRK4", 1e-2, 20), ("FilteredETDRK4", 1e-2, 20), ("RK4", 1e-2, 20), ("FilteredRK4", 1e-2, 20),
    ("AB3", 1e-3, 200), ("FilteredAB3", 1e-3, 200), ("ForwardEuler", 1e-4, 2000), ("FilteredForwardEuler", 1e-4, 2000)])
@pytest.mark.parametrize("ell,U", [(np.inf, 0.0), (np.inf, 0.3), (1.23, 0.0), (1.23, 0.3)])
def test_slqg_rossbywave(stepper, dt, nsteps, ell, U):
    assert rossbywave(stepper, dt, nsteps, ell=ell, U=U)
    if stepper in ("ETDRK4", "RK4", "AB3"):
        assert rossbywave(stepper, dt, nsteps, ell=ell, U=U, U_array=True)


def slqg_nonlinear(add_topography=False, add_background_flow=False, vary_in_y=True, ell=None):
    """test/test_singlelayerqg.jl:276-399"""
    n, L, nu, nnu, dt = 128, 2 * np.pi, 1e-2, 1, 0.0005
    nt = round(1.0 / dt)
    g = O.Grid(n, L)
    x, y = g.gridpoints()
    s, c = np.sin, np.cos
    if ell is None:
        e0 = 0.4 if add_topography else 0.0
        eta = e0 * c(10 * x) * c(10 * y)
        qf = -8 * s(2 * x) * c(2 * y) - 20 * s(x) * c(3 * y)
        Ff = (-nu * (64 * s(2 * x) * c(2 * y) + 200 * s(x) * c(3 * y))
              - 8 * (c(x) * c(3 * y) * s(2 * x) * s(2 * y) - 3 * c(2 * x) * c(2 * y) * s(x) * s(3 * y))
              - 20 * e0 * (s(10 * x) * c(10 * y) * (s(2 * x) * s(2 * y) + 3 * s(x) * s(3 * y))
                           + c(10 * x) * s(10 * y) * (c(2 * x) * c(2 * y) + c(x) * c(3 * y))))
        U, Uyy, U0 = 0.0, 0.0, 0.0
        if add_background_flow and not vary_in_y:
            U = U0 = 0.2
        elif add_background_flow:
            U = 0.2 / np.cosh(2 * y) ** 2
            Uyy = O.irfft2(-g.l ** 2 * O.rfft2(U), g)
            U0 = U[:, 0]
        Ff = Ff + (-U * (16 * c(2 * x) * c(2 * y) + 20 * c(x) * c(3 * y))
                   - Uyy * (2 * c(2 * x) * c(2 * y) + 2 * c(x) * c(3 * y))
                   - e0 * U * 10 * s(10 * x) * c(10 * y))
        p = O.SingleLayerQG(nx=n, Lx=L, U=U0, eta=eta, nu=nu, nnu=nnu, dt=dt, stepper="ForwardEuler",
                            forcing=O.Forcing("static", Fh=O.rfft2(Ff)))
    else:
        e0 = 0.4
        eta = e0 * c(10 * x) * c(10 * y)
        psif = s(2 * x) * c(2 * y) + 2 * s(x) * c(3 * y)
        qf = -8 * s(2 * x) * c(2 * y) - 10 * 2 * s(x) * c(3 * y) - psif / ell ** 2
        Ff = (-nu * (64 * s(2 * x) * c(2 * y) + 200 * s(x) * c(3 * y)
                     + (8 * s(2 * x) * c(2 * y) + 20 * s(x) * c(3 * y)) / ell ** 2)
              - 8 * (c(x) * c(3 * y) * s(2 * x) * s(2 * y) - 3 * c(2 * x) * c(2 * y) * s(x) * s(3 * y))
              - 20 * e0 * (c(10 * y) * s(10 * x) * (s(2 * x) * s(2 * y) + 3 * s(x) * s(3 * y))
                           + c(10 * x) * s(10 * y) * (c(2 * x) * c(2 * y) + c(x) * c(3 * y))))
        p = O.SingleLayerQG(nx=n, Lx=L, eta=eta, nu=nu, nnu=nnu, dt=dt, deformation_radius=ell,
                            stepper="ForwardEuler", forcing=O.Forcing("static", Fh=O.rfft2(Ff)))
    p.set_q(qf)
    p.stepforward(nt)
    p.updatevars()
    return isapprox(p.q, qf, RTOL)


@pytest.mark.parametrize("kw", [dict(), dict(add_topography=True), dict(add_background_flow=True, vary_in_y=False),
                                dict(add_background_flow=True, vary_in_y=False, add_topography=True),
                                dict(add_background_flow=True, vary_in_y=True), dict(ell=1.23)])
def test_slqg_nonlinear_advection(kw):
    assert slqg_nonlinear(**kw)


def test_slqg_energies():
    """test/test_singlelayerqg.jl:406-474"""
    nx, Lx, ny, Ly = 64, 2 * np.pi, 64, 3 * np.pi
    k0, l0 = 2 * np.pi / Lx, 2 * np.pi / Ly
    g = O.Grid(nx, Lx, ny, Ly)
    x, y = g.gridpoints()
    eta = np.cos(10 * k0 * x) * np.cos(10 * l0 * y)
    psi0 = np.sin(2 * k0 * x) * np.cos(2 * l0 * y) + 2 * np.sin(k0 * x) * np.cos(3 * l0 * y)
    q0 = (-((2 * k0) ** 2 + (2 * l0) ** 2) * np.sin(2 * k0 * x) * np.cos(2 * l0 * y)
          - (k0 ** 2 + (3 * l0) ** 2) * 2 * np.sin(k0 * x) * np.cos(3 * l0 * y))
    p = O.SingleLayerQG(nx=nx, Lx=Lx, ny=ny, Ly=Ly, eta=eta, stepper="ForwardEuler")
    p.set_q(q0)
    assert isapprox(p.energy(), 29 / 9, RTOL)
    assert isapprox(p.enstrophy(), 10885 / 648, RTOL)
    assert p.potential_energy() == 0
    ell = 1.23
    p = O.SingleLayerQG(nx=nx, Lx=Lx, ny=ny, Ly=Ly, eta=eta, deformation_radius=ell, stepper="ForwardEuler")
    p.set_q(q0 - psi0 / ell ** 2)
    assert isapprox(p.kinetic_energy(), 29 / 9, RTOL)
    assert isapprox(p.potential_energy(), 5 / (8 * ell ** 2), RTOL)
    with pytest.raises(NotImplementedError):
        p.energy_dissipation()


# --------------------------------------------------------------------- SurfaceQG
@pytest.mark.parametrize("H", [np.inf, 1.0])
def test_sqg_energy_buoyancy_variance(H):
    """test/test_surfaceqg.jl:72-106"""
    nx, Lx, ny, Ly = 128, 2 * np.pi, 128, 3 * np.pi
    g = O.Grid(nx, Lx, ny, Ly)
    x, y = g.gridpoints()
    k0, l0 = 2 * np.pi / Lx, 2 * np.pi / Ly
    K1, K2 = math.sqrt((2 * k0) ** 2 + (2 * l0) ** 2), math.sqrt(k0 ** 2 + (3 * l0) ** 2)
    t1, t2 = math.tanh(K1 * H), math.tanh(K2 * H)
    b0 = -K1 * t1 * np.sin(2 * k0 * x) * np.cos(2 * l0 * y) - K2 * t2 * 2 * np.sin(k0 * x) * np.cos(3 * l0 * y)
    p = O.SurfaceQG(nx=nx, Lx=Lx, ny=ny, Ly=Ly, H=H, stepper="ForwardEuler")
    p.set_b(b0)
    assert isapprox(p.kinetic_energy(), (K1 ** 2 + 4 * K2 ** 2) / 8, RTOL)
    assert isapprox(p.buoyancy_variance(), (K1 ** 2 * t1 ** 2 + 4 * K2 ** 2 * t2 ** 2) / 4, RTOL)
    assert isapprox(p.total_3D_energy(), (K1 * t1 + 4 * K2 * t2) / 8, RTOL)


@pytest.mark.parametrize("H", [np.inf, 1.0])
def test_sqg_advection_manufactured(H):
    """test/test_surfaceqg.jl:35-70 (ForwardEuler dt=5e-4 to t=0.5)"""
    n, L, nu, nnu, dt = 128, 2 * np.pi, 1e-2, 1, 0.0005
    g = O.Grid(n, L)
    x, y = g.gridpoints()
    s, c, r8, r10 = np.sin, np.cos, math.sqrt(8), math.sqrt(10)
    t8, t10 = math.tanh(r8 * H), math.tanh(r10 * H)
    bf = -r8 * t8 * s(2 * x) * c(2 * y) - r10 * t10 * 2 * s(x) * c(3 * y)
    Ff = (-nu * (8 * r8 * t8 * s(2 * x) * c(2 * y) + 10 * r10 * t10 * 2 * s(x) * c(3 * y))
          - 4 * (r10 * t10 - r8 * t8) * (c(x) * c(3 * y) * s(2 * x) * s(2 * y) - 3 * c(2 * x) * c(2 * y) * s(x) * s(3 * y)))
    p = O.SurfaceQG(nx=n, Lx=L, nu=nu, nnu=nnu, H=H, dt=dt, stepper="ForwardEuler",
                    forcing=O.Forcing("static", Fh=O.rfft2(Ff)))
    p.set_b(bf)
    p.stepforward(round(0.5 / dt))
    p.updatevars()
    assert isapprox(p.b, bf, RTOL)


# --------------------------------------------------------------------- MultiLayerQG
def fields_3layer(g):
    """test/test_multilayerqg.jl:61-116"""
    x, y = g.gridpoints()
    k0, l0 = 2 * np.pi / g.Lx, 2 * np.pi / g.Ly
    c, s = np.cos, np.sin
    p1 = 1e-3 * (1 / 4 * c(2 * k0 * x) * c(5 * l0 * y) + 1 / 3 * c(3 * k0 * x) * c(3 * l0 * y))
    p2 = 1e-3 * (c(3 * k0 * x) * c(4 * l0 * y) + 1 / 2 * c(4 * k0 * x) * c(2 * l0 * y))
    p3 = 1e-3 * (c(1 * k0 * x) * c(3 * l0 * y) + 1 / 2 * c(2 * k0 * x) * c(2 * l0 * y))
    d1 = 1e-3 * (-1 / 4 * ((2 * k0) ** 2 + (5 * l0) ** 2) * c(2 * k0 * x) * c(5 * l0 * y)
                 - 1 / 3 * ((3 * k0) ** 2 + (3 * l0) ** 2) * c(3 * k0 * x) * c(3 * l0 * y))
    d2 = 1e-3 * (-((3 * k0) ** 2 + (4 * l0) ** 2) * c(3 * k0 * x) * c(4 * l0 * y)
                 - 1 / 2 * ((4 * k0) ** 2 + (2 * l0) ** 2) * c(4 * k0 * x) * c(2 * l0 * y))
    d3 = 1e-3 * (-((1 * k0) ** 2 + (3 * l0) ** 2) * c(1 * k0 * x) * c(3 * l0 * y)
                 - 1 / 2 * ((2 * k0) ** 2 + (2 * l0) ** 2) * c(2 * k0 * x) * c(2 * l0 * y))
    q1 = d1 + 20 * p2 - 20 * p1
    q2 = d2 + 20 * p1 - 44 * p2 + 24 * p3
    q3 = d3 + 12 * p2 - 12 * p3
    return np.stack([p1, p2, p3]), np.stack([q1, q2, q3])


def test_mlqg_pv_inversion_3layer():
    """test/test_multilayerqg.jl:166-212"""
    p = O.MultiLayerQG(3, nx=128, Lx=2 * np.pi, f0=1, H=[0.25, 0.25, 0.5], b=[-1.0, -1.2, -1.2 - 1 / 6])
    psi, q = fields_3layer(p.grid)
    qq = O.irfft2(p.pvfromstreamfunction(O.rfft2(psi)), p.grid)
    pp = O.irfft2(p.streamfunctionfrompv(O.rfft2(q)), p.grid)
    assert isapprox(qq, q, RTOL) and isapprox(pp, psi, RTOL)


def test_mlqg_energies():
    """test/test_multilayerqg.jl:502-536"""
    nx, ny = 64, 66
    p = O.MultiLayerQG(2, nx=nx, ny=ny, f0=1, H=[2.5, 7.5], b=[-1.0, -1.5])
    g = p.grid
    x, y = g.gridpoints()
    k0, l0 = 2 * np.pi / g.Lx, 2 * np.pi / g.Ly
    base = np.cos(2 * k0 * x) * np.cos(2 * l0 * y)
    p.set_psi(np.stack([base, 0.5 * base]))
    KE, PE = p.energies()
    assert isapprox(KE[0], 1 / 4, RTOL) and isapprox(KE[1], 3 / 4 / 4, RTOL) and isapprox(PE[0], 1 / 16 / 10, RTOL)


@pytest.mark.parametrize("nlayers", [2, 3])
def test_mlqg_fluxes(nlayers):
    """test/test_multilayerqg.jl:567-623"""
    nx, ny = 128, 126
    if nlayers == 2:
        H, b = [0.2, 0.8], [-1.0, -1.2]
    else:
        H, b = [0.2, 0.35, 0.45], [-1.0, -1.2, -1.2 + 1e-9]
    g = O.Grid(nx, 2 * np.pi, ny, 2 * np.pi)
    U = np.zeros((ny, nlayers))
    U[:, 0] = 1 / np.cosh(g.y / 0.2) ** 2
    p = O.MultiLayerQG(nlayers, nx=nx, ny=ny, f0=1, H=H, b=b, U=U)
    x, y = g.gridpoints()
    k0, l0 = 2 * np.pi / g.Lx, 2 * np.pi / g.Ly
    p1 = np.cos(k0 * x) * np.cos(l0 * y) + np.sin(k0 * x)
    p2 = np.cos(k0 * x + np.pi / 10) * np.cos(l0 * y)
    psi = np.stack([p1, p2] + ([p2] if nlayers == 3 else []))
    p.set_psi(psi)
    lat, ver = p.fluxes()
    assert isapprox(lat[0], 0.00626267, 1e-6) and abs(lat[1]) < 1e-12 and isapprox(ver[0], -0.196539, 1e-6)
    if nlayers == 3:
        assert abs(lat[2]) < 1e-12 and abs(ver[1]) < 1e-12


def test_mlqg_topographic_pv_largescale_gradient():
    """test/test_multilayerqg.jl:709-753: with bumps h0 cos(k0 x) cos(l0 y) and a large-scale
    topographic PV gradient f0/H2 (0.01, 0.1), the bottom layer's Qx and Qy equal the analytic
    fields (32 x 34 grid, no dealiasing)"""
    nx, ny, L = 32, 34, 2 * math.pi
    g = O.Grid(nx, L, ny, L)
    x, y = g.gridpoints()
    k0, l0 = 2 * math.pi / L, 2 * math.pi / L
    f0, H, b, U = 1.0, [0.2, 0.8], [-1.0, -1.2], [1.0, 0.0]
    h0, sx, sy = 0.1, 1e-2, 1e-1
    eta = f0 * h0 * np.cos(k0 * x) * np.cos(l0 * y) / H[1]
    p = O.MultiLayerQG(2, nx=nx, ny=ny, Lx=L, Ly=L, f0=f0, H=H, b=b, U=U, beta=0.0, eta=eta,
                       topographic_pv_gradient=(f0 / H[1] * sx, f0 / H[1] * sy), dt=0.001,
                       stepper="ForwardEuler", aliased_fraction=0)
    gp = b[0] - b[1]
    F1 = f0 ** 2 / (H[1] * gp)
    Q2x = f0 * (sx - h0 * k0 * np.sin(k0 * x) * np.cos(l0 * y)) / H[1]
    Q2y = f0 * (sy - h0 * l0 * np.cos(k0 * x) * np.sin(l0 * y)) / H[1] + F1 * (-U[0] + U[1])
    assert isapprox(p.Qx[1], Q2x, rtol=RTOL)
    assert isapprox(p.Qy[1], Q2y, rtol=RTOL)


def test_mlqg_energy_single_layer():
    """test/test_multilayerqg.jl:538-559: one layer, 64 x 64 on [0, 2 pi) x [0, 3 pi), energies
    of the known streamfunction = 29/9"""
    nx, Lx, ny, Ly = 64, 2 * math.pi, 64, 3 * math.pi
    g = O.Grid(nx, Lx, ny, Ly)
    x, y = g.gridpoints()
    k0, l0 = 2 * math.pi / Lx, 2 * math.pi / Ly
    q0 = (-((2 * k0) ** 2 + (2 * l0) ** 2) * np.sin(2 * k0 * x) * np.cos(2 * l0 * y)
          - (k0 ** 2 + (3 * l0) ** 2) * 2 * np.sin(k0 * x) * np.cos(3 * l0 * y))
    p = O.MultiLayerQG(1, nx=nx, ny=ny, Lx=Lx, Ly=Ly, U=np.zeros(ny), stepper="ForwardEuler", dt=0.001)
    p.set_q(q0[None])
    assert isapprox(p.energies(), 29 / 9, rtol=RTOL)


def test_mlqg_fluxes_single_layer():
    """test/test_multilayerqg.jl:630-655"""
    nx, ny = 128, 126
    g = O.Grid(nx, 2 * np.pi, ny, 2 * np.pi)
    p = O.MultiLayerQG(1, nx=nx, ny=ny, U=1 / np.cosh(g.y / 0.2) ** 2)
    x, y = g.gridpoints()
    k0, l0 = 2 * np.pi / g.Lx, 2 * np.pi / g.Ly
    p.set_psi(np.cos(k0 * x) * np.cos(l0 * y) + np.sin(k0 * x))
    assert abs(p.fluxes() - 0.0313134) < 1e-7


def mlqg_nonlinear(nlayers, linear=False):
    """test/test_multilayerqg.jl:225-494 (ForwardEuler dt=5e-3, 200 steps / to t=0.5)"""
    dt = 0.005
    nx, ny = 64, 66
    Lx, Ly = 2 * np.pi, (2 * np.pi if nlayers == 2 else 5 * np.pi)
    g = O.Grid(nx, Lx, ny, Ly)
    x, y = g.gridpoints()
    l0 = 2 * np.pi / g.Ly
    beta = 0.35
    if nlayers == 2:
        H, b = [0.2, 0.8], [-1.0, -1.2]
        Uc = [0.1, 0.05] if linear else [0.02, 0.025]
        amp1 = 0.5 if linear else 0.05
        uu = [amp1 / np.cosh(g.y / (Ly / 15)) ** 2, 0.02 * np.cos(3 * l0 * g.y)]
    else:
        H, b = [0.25, 0.25, 0.5], [-1.0, -1.2, -1.2 - 1 / 6]
        Uc = [0.02, 0.025, 0.01]
        uu = [0.05 / np.cosh(g.y / (Ly / 15)) ** 2, 0.02 * np.cos(3 * l0 * g.y), 0.01 * np.cos(3 * l0 * g.y)]
    ly = g.l[:, 0]
    uyy = [np.real(np.fft.ifft(-ly ** 2 * np.fft.fft(u))) for u in uu]
    U = np.stack([uu[j] + Uc[j] for j in range(nlayers)], axis=1)
    mu, nu = 0.1, 0.05
    sx, sy = Lx / 25, Ly / 20
    eta = np.exp(-(x + Lx / 8) ** 2 / (2 * sx ** 2) - (y - Ly / 8) ** 2 / (2 * sy ** 2))
    etax = -(x + Lx / 8) / sx ** 2 * eta
    if nlayers == 2:
        from test_oracle_reference import fields_2layer
        psi, q = fields_2layer(g)
        coup = [lambda U_: -25 * (U_[1] - U_[0]), lambda U_: -25 / 4 * (U_[0] - U_[1])]
    else:
        psi, q = fields_3layer(g)
        coup = [lambda U_: -20 * (U_[1] - U_[0]),
                lambda U_: -20 * (U_[0] - U_[1]) - 24 * (U_[2] - U_[1]),
                lambda U_: -12 * (U_[1] - U_[2])]
    Ufull = [U[:, j][:, None] for j in range(nlayers)]
    lap = lambda f: O.irfft2(-g.Krsq * O.rfft2(f), g)
    Ff = []
    for j in range(nlayers):
        px = O.irfft2(1j * g.kr * O.rfft2(psi[j]), g)
        qx = O.irfft2(1j * g.kr * O.rfft2(q[j]), g)
        f = (beta - uyy[j][:, None] + coup[j](Ufull)) * px + Ufull[j] * qx - nu * lap(q[j])
        if not linear:
            f = f + O.jacobian(psi[j], q[j], g)
        Ff.append(f)
    Ff[-1] = Ff[-1] + O.jacobian(psi[-1], eta, g) + Ufull[-1] * etax + mu * lap(psi[-1])
    Ffh = O.rfft2(np.stack(Ff))
    p = O.MultiLayerQG(nlayers, nx=nx, ny=ny, Lx=Lx, Ly=Ly, f0=1, H=H, b=b, U=U, eta=eta, beta=beta,
                       mu=mu, nu=nu, nnu=1, dt=dt, stepper="ForwardEuler", linear=linear,
                       forcing=O.Forcing("static", Fh=Ffh))
    p.set_q(q)
    p.stepforward(round(0.5 / dt) if linear else 200)
    p.updatevars()
    return isapprox(p.q, q, RTOL) and isapprox(p.psi, psi, RTOL)


def fields_2layer(g):
    """test/test_multilayerqg.jl:8-55"""
    x, y = g.gridpoints()
    k0, l0 = 2 * np.pi / g.Lx, 2 * np.pi / g.Ly
    c = np.cos
    p1 = 1e-3 * (1 / 4 * c(2 * k0 * x) * c(5 * l0 * y) + 1 / 3 * c(3 * k0 * x) * c(3 * l0 * y))
    p2 = 1e-3 * (c(3 * k0 * x) * c(4 * l0 * y) + 1 / 2 * c(4 * k0 * x) * c(2 * l0 * y))
    d1 = 1e-3 * (-1 / 4 * ((2 * k0) ** 2 + (5 * l0) ** 2) * c(2 * k0 * x) * c(5 * l0 * y)
                 - 1 / 3 * ((3 * k0) ** 2 + (3 * l0) ** 2) * c(3 * k0 * x) * c(3 * l0 * y))
    d2 = 1e-3 * (-((3 * k0) ** 2 + (4 * l0) ** 2) * c(3 * k0 * x) * c(4 * l0 * y)
                 - 1 / 2 * ((4 * k0) ** 2 + (2 * l0) ** 2) * c(4 * k0 * x) * c(2 * l0 * y))
    return np.stack([p1, p2]), np.stack([d1 + 25 * p2 - 25 * p1, d2 + 25 / 4 * p1 - 25 / 4 * p2])


@pytest.mark.parametrize("nlayers,linear", [(2, False), (3, False), (2, True)])
def test_mlqg_advection_manufactured(nlayers, linear):
    assert mlqg_nonlinear(nlayers, linear)


def test_mlqg_rossbywave_one_layer():
    """test/test_multilayerqg.jl:809-838 (1-layer RK4)"""
    nx, beta = 64, 2.0
    p = O.MultiLayerQG(1, nx=nx, beta=beta, stepper="RK4", dt=1e-2)
    g = p.grid
    x, y = g.gridpoints()
    ampl, kw, lw = 1e-2, 3 * 2 * np.pi / g.Lx, 2 * 2 * np.pi / g.Ly
    w = -beta * kw / (kw ** 2 + lw ** 2)
    p.set_q(ampl * np.cos(kw * x) * np.cos(lw * y))
    p.stepforward(20)
    O.dealias(p.sol, g)
    p.updatevars()
    qt = ampl * np.cos(kw * x - w * p.clock.t) * np.cos(lw * y)
    assert isapprox(qt, p.q[0], g.nx * g.ny * 20 * 1e-12)


# --------------------------------------------------------------------- utils
def test_peakedisotropicspectrum_slope():
    """test/test_utils.jl:4-15: radial spectrum of allones IC falls as k^-2 for 15<k<=17.5"""
    g = O.Grid(128, 2 * np.pi)
    qi = O.peakedisotropicspectrum(g, 6, 0.5, allones=True)
    qh = O.rfft2(qi) * g.invKrsq
    # angular integral over annuli of width 1 (FourierFlows.radialspectrum integrates over
    # the angle on a polar regrid; |psi_hat| ~ k^-3 there, so the integral falls as k^-2)
    K = np.sqrt(g.Krsq)
    ks = np.arange(15, 19)
    vals = np.array([np.mean(np.abs(qh[(K >= k - 0.5) & (K < k + 0.5) & (g.kr > 0)])) * k for k in ks])
    assert isapprox(vals / vals[0], (ks / ks[0]) ** -2.0, 3e-2)
    with pytest.raises(ValueError):
        O.peakedisotropicspectrum(O.Grid(32, 2 * np.pi, 34, 3 * np.pi), 6, 0.5, allones=True)


def test_philox_known_answer():
    """Random123 Philox4x32-10 known-answer vectors (kat_vectors: ctr=0,key=0 and ctr=key=all ones)."""
    r = O.philox4x32_10(0, 0, 0, 0, 0, 0)
    assert [int(v) for v in r] == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    m = 0xFFFFFFFF
    r = O.philox4x32_10(m, m, m, m, m, m)
    assert [int(v) for v in r] == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    r = O.philox4x32_10(0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344, 0xA4093822, 0x299F31D0)
    assert [int(v) for v in r] == [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]
