"""Grid sizes other than the powers of two 32 ... 2048: the generic-length path.

FourierFlows' TwoDGrid takes any nx, ny, and the reference's own tests use 128 x 126
(test/test_twodnavierstokes.jl:261, test/test_multilayerqg.jl:571,635), 64 x 66
(test/test_multilayerqg.jl:232-504), 32 x 34 (:664-763) and nx = 16
(test/test_singlelayerqg.jl:513-543).  Here those tests run on the GPU at their own sizes,
the transforms are checked against numpy's FFT, and the step of every module against the
FP64 oracle (<= 1e-12 relative L2 in FP64 and df64, <= 1e-5 in FP32) on grids whose
lengths mix the radices 2, 3, 5, 7, 11, 13, 17 and one length from each of the compiled-in
and generic families."""
import numpy as np
import pytest

import gf_oracle as O

pytestmark = pytest.mark.gpu

gfcuda = pytest.importorskip("gfcuda")
from gfcuda import BarotropicQGQL as QL, MultiLayerQG as ML, SingleLayerQG as SL, SurfaceQG as SQ  # noqa: E402
from gfcuda import TwoDNavierStokes as TD, Forcing, stepforward  # noqa: E402

RTOL_REF = 1e-13
TOL64 = 1e-12


def rel(a, b):
    return O.rel_l2(a, b)


def isapprox(a, b, rtol):
    a, b = np.asarray(a, dtype=np.complex128), np.asarray(b, dtype=np.complex128)
    return np.linalg.norm((a - b).ravel()) <= rtol * max(np.linalg.norm(a.ravel()), np.linalg.norm(b.ravel()))


SIZES = [(128, 126), (64, 66), (32, 34), (16, 16), (96, 60), (98, 50), (22, 26), (2 * 17, 128), (100, 2048),
         (4096, 12)]


@pytest.mark.parametrize("nx,ny", SIZES)
@pytest.mark.parametrize("T,prec,tol", [(np.float64, None, 1e-13), (np.float64, "DF64", 1e-13),
                                        (np.float32, None, 2e-6)])
def test_fft_matches_numpy_generic_sizes(nx, ny, T, prec, tol):
    if prec == "DF64" and 4096 in (nx, ny):
        pytest.skip("generic lengths are limited to 2048 in FP64 and df64")
    if T == np.float64 and prec is None and 4096 in (nx, ny):
        pytest.skip("generic lengths are limited to 2048 in FP64 and df64")
    rng = np.random.default_rng(nx * 1000 + ny)
    p = TD.Problem("GPU", nx=nx, ny=ny, Ly=3.0, T=T, precision=prec)
    f = rng.standard_normal((ny, nx))
    assert rel(p.fwdtransform(f), np.fft.rfft2(f)) <= tol
    assert rel(p.invtransform(np.fft.rfft2(f)), f) <= tol
    p.close()


def test_unsupported_sizes_are_rejected():
    for nx, ny in ((63, 64), (64, 2 * 67), (2, 64)):
        with pytest.raises(gfcuda.GFError):
            TD.Problem("GPU", nx=nx, ny=ny)
    with pytest.raises(gfcuda.GFError):
        TD.Problem("GPU", nx=4096, ny=64, T=np.float64)


# ------------------------------------------------------------------ the reference's tests at their sizes
def test_twodns_energy_enstrophy_palinstrophy_128x126():
    """test/test_twodnavierstokes.jl:259-317 at its own 128 x 126 grid"""
    nx, Lx, ny, Ly = 128, 2 * np.pi, 126, 3 * np.pi
    p = TD.Problem("GPU", nx=nx, Lx=Lx, ny=ny, Ly=Ly, stepper="ForwardEuler")
    x, y = p.grid.gridpoints()
    k0, l0 = 2 * np.pi / Lx, 2 * np.pi / Ly
    z0 = (-((2 * k0) ** 2 + (2 * l0) ** 2) * np.sin(2 * k0 * x) * np.cos(2 * l0 * y)
          - (k0 ** 2 + (3 * l0) ** 2) * 2 * np.sin(k0 * x) * np.cos(3 * l0 * y))
    TD.set_zeta(p, z0)
    assert isapprox(TD.energy(p), 29 / 9, RTOL_REF)
    assert isapprox(TD.enstrophy(p), 2701 / 162, RTOL_REF)
    assert isapprox(TD.palinstrophy(p), 126277 / 1458, RTOL_REF)
    p.close()


def test_mlqg_energies_64x66():
    """test/test_multilayerqg.jl:502-536 at its own 64 x 66 grid"""
    p = ML.Problem(2, "GPU", nx=64, ny=66, f0=1, H=[2.5, 7.5], b=[-1.0, -1.5])
    x, y = p.grid.gridpoints()
    base = np.cos(2 * x) * np.cos(2 * y)
    ML.set_psi(p, np.stack([base, 0.5 * base]))
    KE, PE = ML.energies(p)
    assert isapprox(KE[0], 1 / 4, RTOL_REF) and isapprox(KE[1], 3 / 4 / 4, RTOL_REF)
    assert isapprox(PE[0], 1 / 16 / 10, RTOL_REF)
    p.close()


@pytest.mark.parametrize("nlayers,linear", [(2, False), (3, False), (2, True)])
def test_mlqg_advection_manufactured_64x66(nlayers, linear):
    """test/test_multilayerqg.jl:225-494 through the GPU path at the reference's 64 x 66"""
    import test_oracle_reference as T

    class _Stop(Exception):
        pass

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

    O.MultiLayerQG = Capture
    try:
        T.mlqg_nonlinear(nlayers, linear)
    except _Stop:
        pass
    finally:
        O.MultiLayerQG = orig
    a = dict(captured)
    n = a.pop("nlayers")
    fo = a.pop("forcing")
    nsteps, q0 = a.pop("nsteps"), a.pop("q0")
    assert a["ny"] == 66
    p = ML.Problem(n, "GPU", forcing=Forcing("static", Fh=fo.Fh0), **a)
    ML.set_q(p, q0)
    stepforward(p, nsteps)
    ML.updatevars(p)
    assert isapprox(p.vars.q, q0, RTOL_REF)
    p.close()


@pytest.mark.parametrize("nlayers", [1, 2])
def test_mlqg_fluxes_128x126(nlayers):
    """test/test_multilayerqg.jl:567-655 at its own 128 x 126 grid"""
    nx, ny = 128, 126
    H, b = {1: (None, None), 2: ([0.2, 0.8], [-1.0, -1.2])}[nlayers]
    g = O.Grid(nx, 2 * np.pi, ny, 2 * np.pi)
    U = np.zeros((ny, nlayers))
    U[:, 0] = 1 / np.cosh(g.y / 0.2) ** 2
    p = ML.Problem(nlayers, "GPU", nx=nx, ny=ny, f0=1, H=H, b=b, U=U if nlayers > 1 else U[:, 0])
    x, y = g.gridpoints()
    k0, l0 = 2 * np.pi / g.Lx, 2 * np.pi / g.Ly
    p1 = np.cos(k0 * x) * np.cos(l0 * y) + np.sin(k0 * x)
    p2 = np.cos(k0 * x + np.pi / 10) * np.cos(l0 * y)
    ML.set_psi(p, np.stack([p1, p2]) if nlayers > 1 else p1)
    if nlayers == 1:
        assert abs(ML.fluxes(p) - 0.0313134) < 1e-7
    else:
        lat, ver = ML.fluxes(p)
        assert abs(lat[0] - 0.00626267) < 1e-8 and abs(ver[0] + 0.196539) < 2e-7
    p.close()


def test_mlqg_set_q_set_psi_32x34():
    """test/test_multilayerqg.jl:663-707 (set_q!, set_psi!) at its own 32 x 34 grid, against the
    oracle"""
    kw = dict(nx=32, ny=34, f0=1, H=[0.3, 0.7], b=[-1.0, -1.4])
    p, r = ML.Problem(2, "GPU", **kw), O.MultiLayerQG(2, **kw)
    rng = np.random.default_rng(3)
    q = rng.standard_normal((2, 34, 32))
    ML.set_q(p, q)
    r.set_q(q)
    assert rel(p.sol, r.sol) <= TOL64
    ML.set_psi(p, q)
    r.set_psi(q)
    assert rel(p.sol, r.sol) <= TOL64
    p.close()


@pytest.mark.parametrize("what", [0, 1, 2])
def test_slqg_budget_diagnostics_nx16_finite_radius_raise(what):
    """test/test_singlelayerqg.jl:512-545: budgets are not defined for a finite deformation
    radius, at the reference's nx = 16"""
    p = SL.Problem("GPU", nx=16, deformation_radius=2.23)
    f = [SL.energy_dissipation, SL.enstrophy_dissipation, SL.energy_drag][what]
    with pytest.raises((ValueError, gfcuda.GFError, NotImplementedError)):
        f(p)
    p.close()


# ------------------------------------------------------------------ steps against the oracle
def _zeta0(nx, ny, seed):
    g = O.Grid(nx, 2 * np.pi, ny, 2 * np.pi)
    return O.peakedisotropicspectrum(g, 4, 0.5, seed=seed)


CASES = {
    "twodns": dict(mod=TD, ora=O.TwoDNavierStokes, kw=dict(dt=0.004, nu=1e-4, nnu=1, stepper="FilteredRK4"),
                   init="zeta"),
    "slqg": dict(mod=SL, ora=O.SingleLayerQG, kw=dict(dt=0.01, beta=3.0, deformation_radius=0.8, U=0.2,
                                                      stepper="ETDRK4"), init="q", eta=True),
    "sqg": dict(mod=SQ, ora=O.SurfaceQG, kw=dict(dt=0.004, nu=1e-4, nnu=1, stepper="RK4"), init="b"),
    "qgql": dict(mod=QL, ora=O.BarotropicQGQL, kw=dict(dt=0.004, beta=2.0, nu=1e-4, nnu=1, stepper="RK4"),
                 init="zeta"),
}


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("nx,ny", [(96, 126), (66, 64), (64, 70)])
@pytest.mark.parametrize("T,prec,tol", [(np.float64, None, TOL64), (np.float64, "DF64", TOL64),
                                        (np.float32, None, 1e-5)])
def test_steps_match_oracle_generic_sizes(case, nx, ny, T, prec, tol):
    c = CASES[case]
    kw = dict(c["kw"], nx=nx, ny=ny)
    if c.get("eta"):
        x = np.linspace(0, 2 * np.pi, nx, endpoint=False)[None, :]
        y = np.linspace(-np.pi, np.pi, ny, endpoint=False)[:, None]
        kw["eta"] = 0.1 * np.cos(2 * x) * np.sin(y)
    p = c["mod"].Problem("GPU", T=T, precision=prec, **kw)
    r = c["ora"](**kw)
    z0 = _zeta0(nx, ny, 11)
    getattr(c["mod"], "set_" + c["init"])(p, z0)
    getattr(r, "set_" + c["init"])(z0)
    for n in (3, 1, 6):
        stepforward(p, n)
        r.stepforward(n)
        assert rel(p.sol, r.sol) <= tol, (case, n, rel(p.sol, r.sol))
    p.close()


@pytest.mark.parametrize("T,prec,tol", [(np.float64, None, 10 * TOL64), (np.float32, None, 1e-5)])
def test_mlqg_etdrk4_matches_oracle_64x66(T, prec, tol):
    kw = dict(nx=64, ny=66, f0=1.0, beta=5.0, H=[0.2, 0.3, 0.5], b=[-1.0, -1.2, -1.290909], U=[1.0, 0.5, 0.0],
              mu=0.05, dt=2.5e-3, stepper="ETDRK4")
    p, r = ML.Problem(3, "GPU", T=T, precision=prec, **kw), O.MultiLayerQG(3, **kw)
    q0 = 1e-2 * np.random.default_rng(5).standard_normal((3, 66, 64))
    ML.set_q(p, q0)
    r.set_q(q0)
    stepforward(p, 20)
    r.stepforward(20)
    assert rel(p.sol, r.sol) <= tol
    p.close()


def test_batched_generic_size_equals_single_runs():
    n1, n2, B = 60, 84, 3
    spec = O.ring_forcing_spectrum(O.Grid(n1, 2 * np.pi, n2, 2 * np.pi), 6.0, 1.5, 1e-3)
    kw = dict(nx=n1, ny=n2, dt=0.01, nu=1e-4, nnu=1, stepper="FilteredRK4")
    pb = TD.Problem("GPU", batch=B, forcing=Forcing("stochastic", spectrum=spec, seed=40), **kw)
    stepforward(pb, 8)
    sb = pb.sol
    for i in range(B):
        p = TD.Problem("GPU", forcing=Forcing("stochastic", spectrum=spec, seed=40 + i), **kw)
        stepforward(p, 8)
        assert rel(sb[i], p.sol) <= 1e-14
        r = O.TwoDNavierStokes(**kw, forcing=O.Forcing("stochastic", spectrum=spec, seed=40 + i))
        r.stepforward(8)
        assert rel(sb[i], r.sol) <= TOL64
        p.close()
    pb.close()


@pytest.mark.parametrize("T,precision,tol", [(np.float64, None, 1e-12), (np.float64, "DF64", 1e-12),
                                             (np.float32, None, 1e-5)])
def test_mlqg_topographic_pv_largescale_gradient_gpu(T, precision, tol):
    """test/test_multilayerqg.jl:709-753 set-up on the GPU (32 x 34, two layers, bumps plus a
    large-scale topographic PV gradient, no dealiasing): the library's Qx, Qy enter calcN!, which
    matches the oracle's (whose Qx, Qy equal the analytic fields, test_oracle_reference.py), and
    so do 20 ForwardEuler steps"""
    nx, ny, L = 32, 34, 2 * np.pi
    g = O.Grid(nx, L, ny, L)
    x, y = g.gridpoints()
    f0, H, b, U = 1.0, [0.2, 0.8], [-1.0, -1.2], [1.0, 0.0]
    eta = f0 * 0.1 * np.cos(x) * np.cos(y) / H[1]
    kw = dict(nx=nx, ny=ny, Lx=L, Ly=L, f0=f0, H=H, b=b, U=U, beta=0.0, eta=eta,
              topographic_pv_gradient=(f0 / H[1] * 1e-2, f0 / H[1] * 1e-1), dt=0.001, stepper="ForwardEuler",
              aliased_fraction=0)
    p = ML.Problem(2, "GPU", T=T, precision=precision, **kw)
    r = O.MultiLayerQG(2, **kw)
    rng = np.random.default_rng(3)
    q0 = 0.1 * rng.standard_normal((2, ny, nx))
    sol = np.stack([np.fft.rfft2(q) for q in q0])
    N_gpu, _ = p.calcN(sol, 0.0)
    N_ref = np.zeros_like(sol)
    r.calcN(N_ref, sol.copy(), 0.0)
    assert rel(N_gpu, N_ref) <= tol
    ML.set_q(p, q0)
    r.set_q(q0)
    stepforward(p, 20)
    r.stepforward(20)
    assert rel(p.sol, r.sol) <= tol
    p.close()


@pytest.mark.parametrize("precision", [None, "DF64"])
def test_mlqg_energy_single_layer_gpu(precision):
    """test/test_multilayerqg.jl:538-559 on the GPU: one layer, 64 x 64 on [0, 2 pi) x [0, 3 pi),
    energies = 29/9 at rtol 1e-13"""
    nx, Lx, ny, Ly = 64, 2 * np.pi, 64, 3 * np.pi
    p = ML.Problem(1, "GPU", nx=nx, ny=ny, Lx=Lx, Ly=Ly, U=np.zeros(ny), stepper="ForwardEuler", dt=0.001,
                   precision=precision)
    x, y = O.Grid(nx, Lx, ny, Ly).gridpoints()
    k0, l0 = 2 * np.pi / Lx, 2 * np.pi / Ly
    q0 = (-((2 * k0) ** 2 + (2 * l0) ** 2) * np.sin(2 * k0 * x) * np.cos(2 * l0 * y)
          - (k0 ** 2 + (3 * l0) ** 2) * 2 * np.sin(k0 * x) * np.cos(3 * l0 * y))
    ML.set_q(p, q0)
    assert isapprox(ML.energies(p), 29 / 9, 1e-13)
    p.close()
