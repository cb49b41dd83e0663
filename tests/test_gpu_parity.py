"""GPU parity: libgfcuda (through its C ABI) against the FP64 oracle and the reference's own
known-answer tests.  Tolerances: FP64 path <= 1e-12 relative L2 per step (the parity bar of
the task), known-answer tests at the reference's rtol 1e-13, FP32 path <= 1e-5 relative L2
against the FP64 oracle."""
import math

import numpy as np
import pytest

import gf_oracle as O

pytestmark = pytest.mark.gpu

gfcuda = pytest.importorskip("gfcuda")
from gfcuda import MultiLayerQG as ML, SingleLayerQG as SL, SurfaceQG as SQ, TwoDNavierStokes as TD  # noqa: E402
from gfcuda import Forcing, stepforward  # noqa: E402

RTOL_REF = 1e-13
TOL64 = 1e-12
TOL32 = 1e-5


class _Stop(Exception):
    """Stops a restated reference test once its problem set-up has been captured."""


def rel(a, b):
    return O.rel_l2(a, b)


def isapprox(a, b, rtol):
    a, b = np.asarray(a, dtype=np.complex128), np.asarray(b, dtype=np.complex128)
    return np.linalg.norm((a - b).ravel()) <= rtol * max(np.linalg.norm(a.ravel()), np.linalg.norm(b.ravel()))


def to_oracle_forcing(f):
    if f is None:
        return None
    return O.Forcing(f.kind, Fh=f.Fh, spectrum=f.spectrum, omega=f.omega, phase=f.phase, seed=f.seed)


# ------------------------------------------------------------------------------ transforms
@pytest.mark.parametrize("T,tol", [(np.float64, 1e-13), (np.float32, 2e-6)])
@pytest.mark.parametrize("nx,ny", [(128, 64), (32, 256), (2048, 32), (64, 2048)])
def test_fft_matches_numpy(T, tol, nx, ny):
    rng = np.random.default_rng(1)
    p = TD.Problem("GPU", nx=nx, ny=ny, Ly=3.0, T=T)
    f = rng.standard_normal((ny, nx))
    fh = p.fwdtransform(f)
    assert rel(fh, np.fft.rfft2(f)) <= tol
    back = p.invtransform(np.fft.rfft2(f))
    assert rel(back, f) <= tol


# ------------------------------------------------------------------------------ calcN!
@pytest.mark.parametrize("module", ["TwoDNavierStokes", "SurfaceQG", "SingleLayerQG"])
def test_calcN_matches_oracle(module):
    rng = np.random.default_rng(2)
    n = 128
    if module == "TwoDNavierStokes":
        p, r = TD.Problem("GPU", nx=n), O.TwoDNavierStokes(nx=n)
    elif module == "SurfaceQG":
        p, r = SQ.Problem("GPU", nx=n, H=1.3), O.SurfaceQG(nx=n, H=1.3)
    else:
        g = O.Grid(n)
        x, y = g.gridpoints()
        eta = 0.3 * np.cos(3 * x) * np.sin(2 * y)
        p = SL.Problem("GPU", nx=n, beta=2.0, U=0.4, eta=eta, deformation_radius=1.5)
        r = O.SingleLayerQG(nx=n, beta=2.0, U=0.4, eta=eta, deformation_radius=1.5)
    sol = np.fft.rfft2(rng.standard_normal((n, n)))
    N_gpu, sol_gpu = p.calcN(sol, 0.0)
    N_ref = np.zeros_like(sol)
    s_ref = sol.copy()
    r.calcN(N_ref, s_ref, 0.0)
    assert rel(N_gpu, N_ref) <= TOL64
    assert rel(sol_gpu, s_ref) <= 1e-15


# ---------------------------------------------------------------- 2DNS decaying 128^2 workload
def _peaked_ic(n, filt):
    g = O.Grid(n)
    return O.peakedisotropicspectrum(g, 6, 0.5, mask=filt, seed=1234)


def test_twodns_filteredrk4_single_step_parity():
    n, dt = 128, 0.005
    r = O.TwoDNavierStokes(nx=n, dt=dt, stepper="FilteredRK4")
    r.set_zeta(_peaked_ic(n, r.timestepper.filter))
    r.stepforward(20)  # a developed state
    p = TD.Problem("GPU", nx=n, dt=dt, stepper="FilteredRK4")
    for _ in range(3):
        p.sol = r.sol
        p.set_clock(r.clock.t, r.clock.step)
        stepforward(p, 1)
        r.stepforward(1)
        assert rel(p.sol, r.sol) <= TOL64


def test_twodns_decaying_128_parity_100_steps():
    """The decaying 128^2 workload: FP64 FilteredRK4 dt=0.005 nu=0, peaked isotropic IC (k0=6, E=0.5)"""
    n, dt = 128, 0.005
    r = O.TwoDNavierStokes(nx=n, dt=dt, stepper="FilteredRK4")
    z0 = _peaked_ic(n, r.timestepper.filter)
    r.set_zeta(z0)
    p = TD.Problem("GPU", nx=n, dt=dt, stepper="FilteredRK4")
    TD.set_zeta(p, z0)
    assert rel(p.sol, r.sol) <= 1e-14
    for _ in range(2):
        r.stepforward(50)
        stepforward(p, 50)
        err = rel(p.sol, r.sol)
        assert err <= 100 * TOL64, err
        assert abs(TD.energy(p) - r.energy()) <= 1e-11 * r.energy()
        assert abs(TD.enstrophy(p) - r.enstrophy()) <= 1e-11 * r.enstrophy()
    TD.updatevars(p)
    r.updatevars()
    assert rel(p.vars.zeta, r.zeta) <= 100 * TOL64
    assert rel(p.vars.u, r.u) <= 100 * TOL64


# ------------------------------------------------------------------------------ reference known answers via GPU
def test_twodns_energy_enstrophy_palinstrophy_gpu():
    """test/test_twodnavierstokes.jl:259-317 on a square 128 grid (the reference's 128 x 126 grid runs
    in test_gpu_generic_sizes.py)"""
    nx, Lx, ny, Ly = 128, 2 * np.pi, 128, 3 * np.pi
    p = TD.Problem("GPU", nx=nx, Lx=Lx, ny=ny, Ly=Ly, stepper="ForwardEuler")
    x, y = p.grid.gridpoints()
    k0, l0 = 2 * np.pi / Lx, 2 * np.pi / Ly
    z0 = (-((2 * k0) ** 2 + (2 * l0) ** 2) * np.sin(2 * k0 * x) * np.cos(2 * l0 * y)
          - (k0 ** 2 + (3 * l0) ** 2) * 2 * np.sin(k0 * x) * np.cos(3 * l0 * y))
    TD.set_zeta(p, z0)
    assert isapprox(TD.energy(p), 29 / 9, RTOL_REF)
    assert isapprox(TD.enstrophy(p), 2701 / 162, RTOL_REF)
    assert isapprox(TD.palinstrophy(p), 126277 / 1458, RTOL_REF)


_LAMB = {}


def _lamb_oracle(L, n, dt, Ue, nt, nm):
    """the oracle's Lamb-dipole run: the |zeta| centroids after each interval and the final zeta"""
    key = (L, n, dt, Ue, nt, nm)
    if key not in _LAMB:
        r = O.TwoDNavierStokes(nx=n, Lx=L, nu=0.0, nnu=1, dt=dt, stepper="FilteredRK4")
        r.set_zeta(O.lambdipole(Ue, L / 20, r.grid))
        x, _ = r.grid.gridpoints()
        xs = []
        for _ in range(nm):
            r.stepforward(nt)
            r.updatevars()
            a = np.abs(r.zeta)
            xs.append(np.mean(a * x) / np.mean(a))
        _LAMB[key] = (np.array(xs), r.zeta.copy())
    return _LAMB[key]


@pytest.mark.parametrize("T,precision,tol", [(np.float64, None, 1e-11), (np.float64, "DF64", 1e-11),
                                             (np.float32, None, 1e-5)])
def test_twodns_lambdipole_gpu(T, precision, tol):
    """test/test_twodnavierstokes.jl:1-23 (runtests.jl:44: n = 256, dt = 1e-3) on the GPU: the
    dipole from gfcuda.lambdipole (src/utils.jl:8-20) moves at Ue within rtol 1e-2, and the field
    after the three intervals equals the oracle's run"""
    L, n, dt, Ue = 2 * math.pi, 256, 1e-3, 1.0
    nt, nm = round(L / Ue * 0.01 / dt), 3
    p = TD.Problem("GPU", nx=n, Lx=L, nu=0.0, nnu=1, dt=dt, stepper="FilteredRK4", T=T, precision=precision)
    TD.set_zeta(p, gfcuda.lambdipole(Ue, L / 20, p.grid))
    x, _ = O.Grid(n).gridpoints()
    xz, um = np.zeros(nm), np.zeros(nm)
    for i in range(nm):
        stepforward(p, nt)
        TD.updatevars(p)
        a = np.abs(np.asarray(p.vars.zeta, dtype=np.float64))
        xz[i] = np.mean(a * x) / np.mean(a)
        if i > 0:
            um[i] = (xz[i] - xz[i - 1]) / ((nt - 1) * dt)
    assert isapprox(Ue, np.mean(um[1:]), 1e-2)
    xs_ref, z_ref = _lamb_oracle(L, n, dt, Ue, nt, nm)
    assert np.max(np.abs(xz - xs_ref)) <= 100 * tol
    assert rel(p.vars.zeta, z_ref) <= tol
    p.close()


def test_twodns_advection_manufactured_gpu():
    """test/test_twodnavierstokes.jl:221-257"""
    n, L, nu, dt = 128, 2 * np.pi, 1e-2, 0.0005
    g = O.Grid(n, L)
    x, y = g.gridpoints()
    zf = -8 * np.sin(2 * x) * np.cos(2 * y) - 20 * np.sin(x) * np.cos(3 * y)
    Ff = -(nu * (64 * np.sin(2 * x) * np.cos(2 * y) + 200 * np.sin(x) * np.cos(3 * y))
           + 8 * (np.cos(x) * np.cos(3 * y) * np.sin(2 * x) * np.sin(2 * y)
                  - 3 * np.cos(2 * x) * np.cos(2 * y) * np.sin(x) * np.sin(3 * y)))
    p = TD.Problem("GPU", nx=n, Lx=L, nu=nu, nnu=1, dt=dt, stepper="ForwardEuler",
                   forcing=Forcing("static", Fh=O.rfft2(Ff)))
    TD.set_zeta(p, zf)
    stepforward(p, round(1.0 / dt))
    TD.updatevars(p)
    assert isapprox(p.vars.zeta, zf, RTOL_REF)


@pytest.mark.parametrize("stepper,dt,nsteps", [
    ("ETDRK4", 1e-2, 20), ("FilteredETDRK4", 1e-2, 20), ("RK4", 1e-2, 20), ("FilteredRK4", 1e-2, 20),
    ("AB3", 1e-3, 200), ("FilteredAB3", 1e-3, 200), ("ForwardEuler", 1e-4, 2000), ("FilteredForwardEuler", 1e-4, 2000)])
@pytest.mark.parametrize("ell,U,U_array", [(np.inf, 0.0, False), (np.inf, 0.3, False), (1.23, 0.0, False),
                                           (1.23, 0.3, False), (np.inf, 0.3, True), (1.23, 0.3, True)])
def test_slqg_rossbywave_gpu(stepper, dt, nsteps, ell, U, U_array):
    """test/test_singlelayerqg.jl:8-46 with test/runtests.jl:57-65, checked against the
    analytic wave and against the oracle."""
    nx, beta = 64, 2.0
    Uarg = np.full(nx, U) if U_array else U
    p = SL.Problem("GPU", nx=nx, deformation_radius=ell, beta=beta, U=Uarg, stepper=stepper, dt=dt)
    r = O.SingleLayerQG(nx=nx, deformation_radius=ell, beta=beta, U=Uarg, stepper=stepper, dt=dt)
    x, y = r.grid.gridpoints()
    ampl, kw, lw = 1e-2, 3.0, 2.0
    w = -beta * kw / (kw ** 2 + lw ** 2 + (0 if np.isinf(ell) else 1 / ell ** 2))
    q0 = ampl * np.cos(kw * x) * np.cos(lw * y)
    SL.set_q(p, q0)
    r.set_q(q0)
    stepforward(p, nsteps)
    r.stepforward(nsteps)
    SL.updatevars(p)
    qt = ampl * np.cos(kw * (x - (U + w / kw) * p.clock.t)) * np.cos(lw * y)
    assert isapprox(qt, p.vars.q, nx * nx * nsteps * 1e-12)
    assert rel(p.sol, r.sol) <= TOL64 * 10


@pytest.mark.parametrize("kw", [dict(), dict(add_topography=True), dict(add_background_flow=True, vary_in_y=False),
                                dict(add_background_flow=True, vary_in_y=False, add_topography=True),
                                dict(add_background_flow=True, vary_in_y=True), dict(ell=1.23)])
def test_slqg_nonlinear_advection_gpu(kw):
    """test/test_singlelayerqg.jl:276-399 through the GPU path"""
    import test_oracle_reference as T
    captured = {}

    class Capture(O.SingleLayerQG):
        def __init__(self, **a):
            captured.update(a)
            super().__init__(**a)

        def set_q(self, q):
            captured["q0"] = q

        def stepforward(self, nsteps=1):
            captured["nsteps"] = nsteps
            raise _Stop

    orig = O.SingleLayerQG
    O.SingleLayerQG = Capture
    try:
        T.slqg_nonlinear(**kw)
    except _Stop:
        pass
    finally:
        O.SingleLayerQG = orig
    a = dict(captured)
    fo = a.pop("forcing")
    nsteps, q0 = a.pop("nsteps"), a.pop("q0")
    p = SL.Problem("GPU", forcing=Forcing("static", Fh=fo.Fh0), **a)
    SL.set_q(p, q0)
    stepforward(p, nsteps)
    SL.updatevars(p)
    assert isapprox(p.vars.q, q0, RTOL_REF)


@pytest.mark.parametrize("H", [np.inf, 1.0])
def test_sqg_known_answers_gpu(H):
    """test/test_surfaceqg.jl:35-106"""
    nx, Lx, ny, Ly = 128, 2 * np.pi, 128, 3 * np.pi
    p = SQ.Problem("GPU", nx=nx, Lx=Lx, ny=ny, Ly=Ly, H=H, stepper="ForwardEuler")
    x, y = p.grid.gridpoints()
    k0, l0 = 2 * np.pi / Lx, 2 * np.pi / Ly
    K1, K2 = math.sqrt((2 * k0) ** 2 + (2 * l0) ** 2), math.sqrt(k0 ** 2 + (3 * l0) ** 2)
    t1, t2 = math.tanh(K1 * H), math.tanh(K2 * H)
    b0 = -K1 * t1 * np.sin(2 * k0 * x) * np.cos(2 * l0 * y) - K2 * t2 * 2 * np.sin(k0 * x) * np.cos(3 * l0 * y)
    SQ.set_b(p, b0)
    assert isapprox(SQ.kinetic_energy(p), (K1 ** 2 + 4 * K2 ** 2) / 8, RTOL_REF)
    assert isapprox(SQ.buoyancy_variance(p), (K1 ** 2 * t1 ** 2 + 4 * K2 ** 2 * t2 ** 2) / 4, RTOL_REF)
    assert isapprox(SQ.total_3D_energy(p), (K1 * t1 + 4 * K2 * t2) / 8, RTOL_REF)
    # manufactured steady solution
    n, nu, dt = 128, 1e-2, 0.0005
    g = O.Grid(n)
    x, y = g.gridpoints()
    s, c, r8, r10 = np.sin, np.cos, math.sqrt(8), math.sqrt(10)
    t8, t10 = math.tanh(r8 * H), math.tanh(r10 * H)
    bf = -r8 * t8 * s(2 * x) * c(2 * y) - r10 * t10 * 2 * s(x) * c(3 * y)
    Ff = (-nu * (8 * r8 * t8 * s(2 * x) * c(2 * y) + 10 * r10 * t10 * 2 * s(x) * c(3 * y))
          - 4 * (r10 * t10 - r8 * t8) * (c(x) * c(3 * y) * s(2 * x) * s(2 * y) - 3 * c(2 * x) * c(2 * y) * s(x) * s(3 * y)))
    p = SQ.Problem("GPU", nx=n, nu=nu, nnu=1, H=H, dt=dt, stepper="ForwardEuler",
                   forcing=Forcing("static", Fh=O.rfft2(Ff)))
    SQ.set_b(p, bf)
    stepforward(p, round(0.5 / dt))
    SQ.updatevars(p)
    assert isapprox(p.vars.b, bf, RTOL_REF)


def test_slqg_energies_gpu():
    """test/test_singlelayerqg.jl:406-474"""
    nx, Lx, ny, Ly = 64, 2 * np.pi, 64, 3 * np.pi
    k0, l0 = 2 * np.pi / Lx, 2 * np.pi / Ly
    g = O.Grid(nx, Lx, ny, Ly)
    x, y = g.gridpoints()
    eta = np.cos(10 * k0 * x) * np.cos(10 * l0 * y)
    psi0 = np.sin(2 * k0 * x) * np.cos(2 * l0 * y) + 2 * np.sin(k0 * x) * np.cos(3 * l0 * y)
    q0 = (-((2 * k0) ** 2 + (2 * l0) ** 2) * np.sin(2 * k0 * x) * np.cos(2 * l0 * y)
          - (k0 ** 2 + (3 * l0) ** 2) * 2 * np.sin(k0 * x) * np.cos(3 * l0 * y))
    p = SL.Problem("GPU", nx=nx, Lx=Lx, ny=ny, Ly=Ly, eta=eta, stepper="ForwardEuler")
    SL.set_q(p, q0)
    assert isapprox(SL.energy(p), 29 / 9, RTOL_REF)
    assert isapprox(SL.enstrophy(p), 10885 / 648, RTOL_REF)
    assert SL.potential_energy(p) == 0
    ell = 1.23
    p = SL.Problem("GPU", nx=nx, Lx=Lx, ny=ny, Ly=Ly, eta=eta, deformation_radius=ell, stepper="ForwardEuler")
    SL.set_q(p, q0 - psi0 / ell ** 2)
    assert isapprox(SL.kinetic_energy(p), 29 / 9, RTOL_REF)
    assert isapprox(SL.potential_energy(p), 5 / (8 * ell ** 2), RTOL_REF)
    with pytest.raises(NotImplementedError):
        SL.energy_dissipation(p)


# ------------------------------------------------------------------------------ MultiLayerQG
def test_mlqg_pv_inversion_and_energies_gpu():
    """test/test_multilayerqg.jl:166-212 and :502-536 on square grids (the reference's 64 x 66 grid
    runs in test_gpu_generic_sizes.py)"""
    import test_oracle_reference as T
    p = ML.Problem(3, "GPU", nx=128, f0=1, H=[0.25, 0.25, 0.5], b=[-1.0, -1.2, -1.2 - 1 / 6])
    psi, q = T.fields_3layer(O.Grid(128))
    ML.set_psi(p, psi)
    assert isapprox(p.vars.q, q, RTOL_REF)
    assert isapprox(p.vars.psi, psi, RTOL_REF)
    ML.set_q(p, q)
    assert isapprox(p.vars.psi, psi, RTOL_REF)
    p = ML.Problem(2, "GPU", nx=64, ny=64, f0=1, H=[2.5, 7.5], b=[-1.0, -1.5])
    x, y = p.grid.gridpoints()
    base = np.cos(2 * x) * np.cos(2 * y)
    ML.set_psi(p, np.stack([base, 0.5 * base]))
    KE, PE = ML.energies(p)
    assert isapprox(KE[0], 1 / 4, RTOL_REF) and isapprox(KE[1], 3 / 4 / 4, RTOL_REF)
    assert isapprox(PE[0], 1 / 16 / 10, RTOL_REF)


@pytest.mark.parametrize("nlayers,linear", [(2, False), (3, False), (2, True)])
def test_mlqg_advection_manufactured_gpu(nlayers, linear):
    """test/test_multilayerqg.jl:225-494 through the GPU path on a 64 x 64 grid (the reference's
    64 x 66 grid runs in test_gpu_generic_sizes.py)"""
    import test_oracle_reference as T
    captured = {}
    orig = O.MultiLayerQG

    class Capture(orig):
        def __init__(self, nl, **a):
            captured.update(a, nlayers=nl)
            super().__init__(nl, **a)

        def set_q(self, q):
            captured["q0"] = q

        def stepforward(self, nsteps=1):
            captured["nsteps"] = nsteps
            raise _Stop

    orig_grid = O.Grid

    def grid64(nx, Lx=2 * np.pi, ny=None, Ly=None, aliased_fraction=1 / 3):
        return orig_grid(nx, Lx, 64 if ny == 66 else ny, Ly, aliased_fraction)

    O.MultiLayerQG, O.Grid = Capture, grid64
    try:
        T.mlqg_nonlinear(nlayers, linear)
    except _Stop:
        pass
    finally:
        O.MultiLayerQG, O.Grid = orig, orig_grid
    a = dict(captured)
    n = a.pop("nlayers")
    fo = a.pop("forcing")
    nsteps, q0 = a.pop("nsteps"), a.pop("q0")
    a["ny"] = 64
    p = ML.Problem(n, "GPU", forcing=Forcing("static", Fh=fo.Fh0), **a)
    ML.set_q(p, q0)
    stepforward(p, nsteps)
    ML.updatevars(p)
    assert isapprox(p.vars.q, q0, RTOL_REF)


def test_mlqg_etdrk4_parity():
    n, nl = 128, 3
    rng = np.random.default_rng(5)
    kw = dict(nx=n, f0=1.0, beta=5.0, H=[0.2, 0.3, 0.5], b=[-1.0, -1.2, -1.290909], U=[1.0, 0.5, 0.0], mu=0.05,
              dt=2.5e-3, stepper="ETDRK4")
    p, r = ML.Problem(nl, "GPU", **kw), O.MultiLayerQG(nl, **kw)
    q0 = 1e-2 * rng.standard_normal((nl, n, n))
    ML.set_q(p, q0)
    r.set_q(q0)
    stepforward(p, 20)
    r.stepforward(20)
    assert rel(p.sol, r.sol) <= 10 * TOL64
    KE, PE = ML.energies(p)
    KEr, PEr = r.energies()
    assert rel(KE, KEr) <= 1e-11 and rel(PE, PEr) <= 1e-11


# ------------------------------------------------------------------------------ forcing
@pytest.mark.parametrize("kind", ["stochastic", "stochastic_phase"])
def test_stochastic_forcing_matches_oracle(kind):
    n, dt = 128, 0.01
    g = O.Grid(n)
    spec = O.ring_forcing_spectrum(g, 8.0, 1.5, 1e-3)
    f = Forcing(kind, spectrum=spec, seed=42)
    p = TD.Problem("GPU", nx=n, dt=dt, nu=1e-4, nnu=1, stepper="FilteredRK4", forcing=f)
    r = O.TwoDNavierStokes(nx=n, dt=dt, nu=1e-4, nnu=1, stepper="FilteredRK4", forcing=to_oracle_forcing(f))
    stepforward(p, 10)
    r.stepforward(10)
    assert rel(p.sol, r.sol) <= TOL64
    assert abs(TD.energy_work(p) - r.energy_work()) <= 1e-11 * abs(r.energy_work())


def test_twodns_stochastic_energy_budget_gpu():
    """test/test_twodnavierstokes.jl:25-66 on the GPU (Philox draws)"""
    n, L, nu, nnu, mu, nmu, dt = 256, 2 * np.pi, 1e-7, 2, 1e-1, 0, 0.005
    nt = round(0.1 / mu / dt)
    g = O.Grid(n, L)
    kf, dkf, eps = 12.0, 2.0, 0.1
    Kr = np.broadcast_to(g.kr, g.Krsq.shape)
    spec = np.exp(-(np.sqrt(g.Krsq) - kf) ** 2 / (2 * dkf ** 2))
    spec[g.Krsq < 4] = 0
    spec[g.Krsq > 400] = 0
    spec[Kr < 2 * np.pi / L] = 0
    spec = eps / (O.parsevalsum(spec * g.invKrsq / 2, g) / (g.Lx * g.Ly)) * spec
    p = TD.Problem("GPU", nx=n, Lx=L, nu=nu, nnu=nnu, mu=mu, nmu=nmu, dt=dt, stepper="RK4",
                   forcing=Forcing("stochastic_phase", spectrum=spec, seed=1234))
    TD.set_zeta(p, np.zeros((n, n)))
    ids = [0, 3, 4, 7]
    vals = [p.diagnostics(ids)]
    for _ in range(nt):
        stepforward(p, 1)
        vals.append(p.diagnostics(ids))
    E, D, R, W = np.array(vals).T
    num = (E[1:] - E[:-1]) / dt
    comp = W[1:] + D[:-1] + R[:-1]
    assert isapprox(num, comp, 1e-3)


# ------------------------------------------------------------------------------ FP32
def test_fp32_slqg_beta_forced_against_fp64_oracle():
    """The beta-plane forced SingleLayerQG physics (beta=10, mu=0.01, ETDRK4 dt=0.05,
    stochastic ring forcing at kf=14)
    at 256^2 for 100 steps: FP32 bulk vs the FP64 oracle."""
    n, dt = 256, 0.05
    g = O.Grid(n)
    spec = O.ring_forcing_spectrum(g, 14.0, 1.5, 1e-3)
    f = Forcing("stochastic", spectrum=spec, seed=7)
    p = SL.Problem("GPU", nx=n, beta=10.0, mu=0.01, dt=dt, stepper="ETDRK4", forcing=f, T=np.float32)
    r = O.SingleLayerQG(nx=n, beta=10.0, mu=0.01, dt=dt, stepper="ETDRK4", forcing=to_oracle_forcing(f))
    stepforward(p, 100)
    r.stepforward(100)
    assert rel(p.sol, r.sol) <= TOL32
    assert abs(SL.energy(p) - r.energy()) <= 1e-5 * r.energy()


def test_fp32_twodns_against_fp64_oracle():
    n, dt = 256, 0.005
    r = O.TwoDNavierStokes(nx=n, dt=dt, stepper="FilteredRK4")
    z0 = _peaked_ic(n, r.timestepper.filter)
    r.set_zeta(z0)
    p = TD.Problem("GPU", nx=n, dt=dt, stepper="FilteredRK4", T=np.float32)
    TD.set_zeta(p, z0)
    stepforward(p, 100)
    r.stepforward(100)
    assert rel(p.sol, r.sol) <= TOL32


@pytest.mark.parametrize("nlayers", [1, 2, 3])
@pytest.mark.parametrize("prec", [None, "DF64"])
def test_mlqg_fluxes_gpu(nlayers, prec):
    """MultiLayerQG.fluxes on the device: the known answers of test/test_multilayerqg.jl:567-655
    (at 128 x 128) and the oracle on a random state, to 1e-12"""
    from gfcuda import MultiLayerQG as MLg
    nx = ny = 128
    H, b = {1: (None, None), 2: ([0.2, 0.8], [-1.0, -1.2]),
            3: ([0.2, 0.35, 0.45], [-1.0, -1.2, -1.2 + 1e-9])}[nlayers]
    g = O.Grid(nx, 2 * np.pi, ny, 2 * np.pi)
    U = np.zeros((ny, nlayers))
    U[:, 0] = 1 / np.cosh(g.y / 0.2) ** 2
    kw = dict(nx=nx, ny=ny, f0=1, H=H, b=b, U=U if nlayers > 1 else U[:, 0])
    p = MLg.Problem(nlayers, "GPU", precision=prec, **kw)
    r = O.MultiLayerQG(nlayers, **kw)
    x, y = g.gridpoints()
    k0, l0 = 2 * np.pi / g.Lx, 2 * np.pi / g.Ly
    p1 = np.cos(k0 * x) * np.cos(l0 * y) + np.sin(k0 * x)
    p2 = np.cos(k0 * x + np.pi / 10) * np.cos(l0 * y)
    psi = np.stack([p1, p2, p2][:nlayers])
    MLg.set_psi(p, psi if nlayers > 1 else p1)
    if nlayers == 1:
        assert abs(MLg.fluxes(p) - 0.0313134) < 1e-7
    else:
        lat, ver = MLg.fluxes(p)
        assert abs(lat[0] - 0.00626267) < 1e-8 and abs(ver[0] + 0.196539) < 2e-7
        assert np.all(np.abs(lat[1:]) < 1e-12) and np.all(np.abs(ver[1:]) < 1e-12)
    if nlayers == 3:
        # the known-answer configuration has g'_{5/2} = 1e-9 (PV inversion conditioned ~1e9):
        # compare a random state on a well-conditioned stratification instead
        kw["b"] = [-1.0, -1.2, -1.3]
        p = MLg.Problem(nlayers, "GPU", precision=prec, **kw)
        r = O.MultiLayerQG(nlayers, **kw)
    rng = np.random.default_rng(5)
    q = 0.1 * rng.standard_normal((nlayers, ny, nx))
    MLg.set_q(p, q if nlayers > 1 else q[0])
    r.set_q(q if nlayers > 1 else q[0])
    got, ref = MLg.fluxes(p), r.fluxes()
    if nlayers == 1:
        assert abs(got - ref) <= 1e-12 * abs(ref)
    else:
        for a, c in zip(got, ref):
            assert np.allclose(a, c, rtol=1e-12, atol=1e-14 * np.max(np.abs(c)))


@pytest.mark.parametrize("ell", [np.inf, 1.23])
@pytest.mark.parametrize("T,precision,tol", [(np.float64, None, 1e-12), (np.float64, "DF64", 1e-12),
                                             (np.float32, None, 1e-6)])
def test_slqg_streamfunctionfrompv_gpu(ell, T, precision, tol):
    """test/test_singlelayerqg.jl:490-510 on the GPU: set_q! with the PV of a known streamfunction,
    barotropic and equivalent-barotropic (deformation radius 1.23); the device's psi is that
    streamfunction"""
    nx = 64
    p = SL.Problem("GPU", nx=nx, deformation_radius=ell, T=T, precision=precision)
    x, y = O.Grid(nx).gridpoints()
    k0 = l0 = 1.0
    psi = np.sin(2 * k0 * x) * np.cos(3 * l0 * y)
    extra = 0.0 if np.isinf(ell) else 1 / ell ** 2
    SL.set_q(p, -((2 * k0) ** 2 + (3 * l0) ** 2 + extra) * psi)
    SL.updatevars(p)
    assert rel(p.vars.psi, psi) <= tol
    p.close()
