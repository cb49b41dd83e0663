"""GPU adjoint of the ETDRK4 and RK4 steps of TwoDNavierStokes, SingleLayerQG (constant U and
U(y)) and MultiLayerQG (gf_adjoint_* / gf_grad) against the oracle's discrete
adjoint (oracle/gf_adjoint.py, itself pinned by finite differences and the tangent-linear
dot-product identity), against central finite differences of the GPU forward model, and for
checkpoint-interval invariance."""
import numpy as np
import pytest

import gf_adjoint as AD
import gf_oracle as O

pytestmark = pytest.mark.gpu

gfcuda = pytest.importorskip("gfcuda")
from gfcuda import MultiLayerQG as ML, SingleLayerQG as SL, TwoDNavierStokes as TD, adjoint  # noqa: E402
from gfcuda import stepforward  # noqa: E402


def rel(a, b):
    return O.rel_l2(a, b)


def slqg_case(n, stepper="ETDRK4", U=0.2, beta=1.0, ell=0.35, dt=0.01):
    g = O.Grid(n)
    eta = AD.random_topography(g, 8, 0.1, 7)
    q0 = O.peakedisotropicspectrum(g, 6, 0.5, seed=1234)
    kw = dict(nx=n, deformation_radius=ell, eta=eta, dt=dt, stepper=stepper, U=U, beta=beta)
    return kw, q0, eta


def gpu_grad(kw, q0, nsteps, every, T=np.float64, precision=None):
    p = SL.Problem("GPU", T=T, precision=precision, **kw)
    SL.set_q(p, q0)
    loss, dq0, deta = adjoint.grad(p, nsteps, checkpoint_every=every)
    return p, loss, dq0, deta


@pytest.mark.parametrize("stepper,U,beta,ell", [("ETDRK4", 0.2, 1.0, 0.35), ("FilteredETDRK4", 0.0, 0.0, 0.35),
                                                ("ETDRK4", 0.3, 2.0, np.inf), ("RK4", 0.2, 1.0, 0.35),
                                                ("FilteredRK4", 0.0, 2.0, np.inf)])
def test_gradient_matches_oracle_adjoint(stepper, U, beta, ell):
    n, ns = 64, 12
    kw, q0, eta = slqg_case(n, stepper, U, beta, ell)
    p, loss, dq0, deta = gpu_grad(kw, q0, ns, 5)
    A = AD.SLQGAdjoint(O.SingleLayerQG(**kw))
    L, gq, ge = A.gradient(q0, eta, ns)
    assert abs(loss - L) <= 1e-13 * L
    assert rel(dq0, gq) <= 1e-11
    assert rel(deta, ge) <= 1e-11


@pytest.mark.parametrize("stepper", ["ETDRK4", "FilteredRK4"])
@pytest.mark.parametrize("prec,T,tol", [("DF64", np.float64, 1e-10), (None, np.float32, 2e-4)])
def test_gradient_other_precisions(prec, T, tol, stepper):
    n, ns = 64, 12
    kw, q0, eta = slqg_case(n, stepper)
    p, loss, dq0, deta = gpu_grad(kw, q0, ns, 4, T=T, precision=prec)
    L, gq, ge = AD.SLQGAdjoint(O.SingleLayerQG(**kw)).gradient(q0, eta, ns)
    assert abs(loss - L) <= max(tol, 1e-12) * L
    assert rel(dq0, gq) <= tol
    assert rel(deta, ge) <= tol


def test_twodns_gradient_and_state_restored():
    n, ns = 64, 10
    g = O.Grid(n)
    z0 = O.peakedisotropicspectrum(g, 6, 0.5, seed=5)
    kw = dict(nx=n, dt=0.01, nu=1e-3, nnu=1, stepper="ETDRK4")
    p = TD.Problem("GPU", **kw)
    TD.set_zeta(p, z0)
    loss, dq0, deta = adjoint.grad(p, ns, checkpoint_every=3)
    assert deta is None
    # TwoDNavierStokes is SingleLayerQG with eta = 0, l = inf, beta = 0 and the same L
    r = O.SingleLayerQG(nx=n, dt=0.01, nu=1e-3, nnu=1, stepper="ETDRK4")
    L, gq, _ = AD.SLQGAdjoint(r).gradient(z0, np.zeros((n, n)), ns)
    assert abs(loss - L) <= 1e-13 * L and rel(dq0, gq) <= 1e-11
    # the context holds the forward result again, clock included
    q = TD.Problem("GPU", **kw)
    TD.set_zeta(q, z0)
    stepforward(q, ns)
    assert np.array_equal(p.sol, q.sol)
    assert p.clock.step == ns and p.clock.t == q.clock.t
    with pytest.raises(ValueError):
        adjoint.grad(p, ns, topography=True)


def test_checkpoint_interval_does_not_change_the_gradient():
    kw, q0, eta = slqg_case(64)
    ref = None
    for every in (1, 4, 12, 100):
        _, loss, dq0, deta = gpu_grad(kw, q0, 12, every)
        if ref is None:
            ref = (loss, dq0, deta)
        else:
            assert loss == ref[0] and np.array_equal(dq0, ref[1]) and np.array_equal(deta, ref[2])


def test_pullback_matches_oracle_step_adjoint():
    kw, q0, eta = slqg_case(64)
    ns = 6
    p = SL.Problem("GPU", **kw)
    SL.set_q(p, q0)
    pull = adjoint.stepforward_with_pullback(p, ns, checkpoint_every=4)
    rng = np.random.default_rng(11)
    sol_bar = np.fft.rfft2(rng.standard_normal((64, 64)))
    s0, eb = pull(sol_bar)
    A = AD.SLQGAdjoint(O.SingleLayerQG(**kw))
    us = [A.initial_state(q0)]
    for _ in range(ns):
        us.append(A.step(us[-1], eta)[0])
    ub, etab = sol_bar, np.zeros_like(eta)
    for k in range(ns - 1, -1, -1):
        ub, e = A.step_adj(us[k], eta, ub)
        etab += e
    assert rel(s0, ub) <= 1e-11 and rel(eb, etab) <= 1e-11
    assert rel(p.sol, us[-1]) <= 1e-12


def _fd_check(n, ns, every, ndir, seed, richardson=False, stepper="ETDRK4"):
    kw, q0, eta = slqg_case(n, stepper, U=0.0, beta=0.0, ell=0.35)
    _, loss, dq0, deta = gpu_grad(kw, q0, ns, every)
    rng = np.random.default_rng(seed)

    def L(q, e):
        k2 = dict(kw)
        k2["eta"] = e
        p = SL.Problem("GPU", **k2)
        SL.set_q(p, q)
        stepforward(p, ns)
        return SL.kinetic_energy(p)

    def D(eps, dq, de):
        return (L(q0 + eps * dq, eta + eps * de) - L(q0 - eps * dq, eta - eps * de)) / (2 * eps)

    eps = 1e-6
    g = O.Grid(n)
    for i in range(ndir):
        if richardson:   # band-limited directions: random Fourier modes |k| <= 8
            dq = AD.random_topography(g, 8, 1.0, seed + 2 * i)
            de = AD.random_topography(g, 8, 0.1, seed + 2 * i + 1)
        else:
            dq, de = rng.standard_normal(q0.shape), 0.1 * rng.standard_normal(eta.shape)
        ad = float(np.sum(dq0 * dq) + np.sum(deta * de))
        d1 = D(eps, dq, de)
        if richardson:
            # over 500 steps the flow is nonlinear enough that the O(eps^2) truncation of a
            # plain central difference reaches ~1e-6 relative (up to 5e-5 along grid-scale
            # white-noise directions; the FP64 oracle's exact adjoint shows the same); the
            # eps^2 term is removed with a second difference at 2 eps
            assert abs(d1 - ad) <= 5e-5 * abs(ad), (d1, ad)
            fd = (4 * d1 - D(2 * eps, dq, de)) / 3
        else:
            fd = d1
        assert abs(fd - ad) <= 1e-6 * abs(ad), (fd, ad)


def test_central_differences_small():
    _fd_check(64, 20, 5, 4, 1)


def test_central_differences_small_filtered_rk4():
    _fd_check(64, 20, 5, 4, 2, stepper="FilteredRK4")


@pytest.mark.parametrize("stepper", ["ETDRK4", "RK4"])
def test_classic_and_field_parallel_adjoint_kernels_agree(stepper):
    """the classic adjoint kernels (an explicit launch shape) and the field-parallel ones
    (the default at 64^2) give the same gradient to rounding, and both match the oracle"""
    n, ns = 64, 10
    kw, q0, eta = slqg_case(n, stepper)
    res = []
    for classic in (True, False):
        p = SL.Problem("GPU", **kw)
        if classic:
            p.launch_shape = (8, 1, 8, 1)
        SL.set_q(p, q0)
        res.append(adjoint.grad(p, ns, checkpoint_every=4))
        p.close()
    (l0, g0, e0), (l1, g1, e1) = res
    assert abs(l1 - l0) <= 1e-13 * l0 and rel(g1, g0) <= 1e-12 and rel(e1, e0) <= 1e-12
    L, gq, ge = AD.SLQGAdjoint(O.SingleLayerQG(**kw)).gradient(q0, eta, ns)
    assert rel(g0, gq) <= 1e-11 and rel(e0, ge) <= 1e-11


@pytest.mark.parametrize("stepper", ["ETDRK4", "FilteredRK4"])
@pytest.mark.parametrize("classic", [False, True])
def test_varying_U_gradient_matches_oracle(stepper, classic):
    """SingleLayerQG with a zonal jet U(y) (the third product (U + u) Qx + v Qy and the
    topography entering through Qx, Qy): gradients of the final kinetic energy with respect
    to q0 and the topography against the oracle's discrete adjoint, with the field-parallel
    (default at 64^2) and the classic adjoint kernels"""
    n, ns = 64, 12
    g = O.Grid(n)
    Uy = 0.3 * np.cos(2 * g.y) + 0.1 * np.sin(g.y)
    kw, q0, eta = slqg_case(n, stepper, U=Uy, beta=1.0, ell=0.35)
    p = SL.Problem("GPU", T=np.float64, **kw)
    if classic:
        p.launch_shape = (8, 1, 8, 1)
    SL.set_q(p, q0)
    loss, dq0, deta = adjoint.grad(p, ns, checkpoint_every=5)
    p.close()
    L, gq, ge = AD.SLQGAdjoint(O.SingleLayerQG(**kw)).gradient(q0, eta, ns)
    assert abs(loss - L) <= 1e-13 * L
    assert rel(dq0, gq) <= 1e-11
    assert rel(deta, ge) <= 1e-11


def test_twodns_filtered_rk4_gradient():
    """TwoDNavierStokes with FilteredRK4 (the decaying run's stepper) and viscosity: the
    gradient of the final kinetic energy against the oracle's discrete adjoint"""
    n, ns = 64, 12
    g = O.Grid(n)
    z0 = O.peakedisotropicspectrum(g, 6, 0.5, seed=5)
    kw = dict(nx=n, dt=0.005, nu=1e-3, nnu=1, stepper="FilteredRK4")
    p = TD.Problem("GPU", T=np.float64, **kw)
    TD.set_zeta(p, z0)
    loss, dq0, deta = adjoint.grad(p, ns, checkpoint_every=5)
    assert deta is None
    r = O.SingleLayerQG(nx=n, dt=0.005, nu=1e-3, nnu=1, stepper="FilteredRK4")
    L, gq, _ = AD.SLQGAdjoint(r).gradient(z0, np.zeros((n, n)), ns)
    assert abs(loss - L) <= 1e-13 * L and rel(dq0, gq) <= 1e-11


def test_adjoint_slqg256_central_differences_8_directions():
    """SingleLayerQG 256^2, deformation radius 0.35, topography |k| <= 8 amplitude 0.1,
    ETDRK4 dt = 0.01, 500 steps, checkpoint every 25, loss = final kinetic energy: central
    differences (eps = 1e-6, Richardson-extrapolated with 2 eps) along 8 seeded band-limited
    directions within 1e-6 (FP64)."""
    _fd_check(256, 500, 25, 8, 2024, richardson=True)


def test_adjoint_slqg256_central_differences_100_steps():
    """the same case over 100 steps, where the plain eps = 1e-6 central difference is
    already within 1e-6"""
    _fd_check(256, 100, 25, 8, 7)


def _schedule_cost(n, s):
    """C(n, s) of the binomial schedule, restated independently of the library"""
    from functools import lru_cache

    @lru_cache(maxsize=None)
    def C(n, s):
        if n == 1:
            return 0
        if s == 0:
            return n * (n - 1) // 2
        return min(m + C(n - m, s - 1) + C(m, s) for m in range(1, n))
    return C(n, s)


def test_binomial_checkpointing_same_gradient_fewer_snapshots():
    """fewer snapshot slots: the same gradient (bit for bit) with the unit advances of the
    optimal binomial schedule"""
    kw, q0, eta = slqg_case(64)
    ns, every = 24, 2
    ref = None
    for snaps in (None, 1, 2, 3, 5):
        p = SL.Problem("GPU", **kw)
        SL.set_q(p, q0)
        adjoint.setup(p, ns, every, snapshots=snaps)
        loss, dq0, deta = adjoint.grad(p)
        units, slots, adv = adjoint.info(p)
        assert units == 12 and slots == (12 if snaps is None else snaps)
        # the forward pass takes the schedule's first snapshots; the rest is recomputation
        assert adv <= _schedule_cost(units, slots - 1)
        if snaps is None:
            assert adv == 0
        if snaps == 1:
            assert adv == units * (units - 1) // 2
        if ref is None:
            ref = (loss, dq0, deta)
        else:
            assert loss == ref[0] and np.array_equal(dq0, ref[1]) and np.array_equal(deta, ref[2])


def mlqg_case(n, nl, stepper):
    g = O.Grid(n)
    kw = dict(nx=n, f0=1.0, beta=5.0, H=[0.2, 0.3, 0.5], b=[-1.0, -1.2, -1.2 - 0.5 / 5.5], U=[1.0, 0.5, 0.0],
              mu=0.05, dt=2.5e-3, stepper=stepper, eta=AD.random_topography(g, 6, 0.3, 9))
    if nl == 2:
        kw.update(H=[0.4, 0.6], b=[-1.0, -1.2], U=[0.5, 0.0])
    q0 = 1e-2 * np.random.default_rng(1234).standard_normal((nl, n, n))
    return kw, q0


@pytest.mark.parametrize("nl,stepper", [(3, "ETDRK4"), (2, "FilteredRK4"), (3, "RK4")])
def test_mlqg_gradient_matches_oracle_adjoint(nl, stepper):
    """MultiLayerQG (PV inversion across layers, bottom drag, topographic and planetary PV
    gradients, a mean flow per layer): the gradient of the total kinetic energy with respect
    to the initial PV of every layer against the oracle's discrete adjoint"""
    n, ns = 64, 10
    kw, q0 = mlqg_case(n, nl, stepper)
    p = ML.Problem(nl, "GPU", T=np.float64, **kw)
    ML.set_q(p, q0)
    loss, dq0, deta = adjoint.grad(p, ns, checkpoint_every=4)
    assert dq0.shape == (nl, n, n) and deta.shape == (n, n)
    KE = ML.energies(p)[0]
    p.close()
    A = AD.MLQGAdjoint(O.MultiLayerQG(nl, **kw))
    L, gq, ge = A.gradient(q0, kw["eta"], ns)
    assert abs(loss - L) <= 1e-13 * L and abs(float(np.sum(KE)) - L) <= 1e-12 * L
    assert rel(dq0, gq) <= 1e-11 and rel(deta, ge) <= 1e-11


def test_mlqg_gradient_df64_and_checkpoint_invariance():
    n, ns, nl = 64, 8, 3
    kw, q0 = mlqg_case(n, nl, "ETDRK4")
    A = AD.MLQGAdjoint(O.MultiLayerQG(nl, **kw))
    L, gq, _ = A.gradient(q0, kw["eta"], ns)
    ref = None
    for every in (1, 3, 8):
        p = ML.Problem(nl, "GPU", T=np.float64, **kw)
        ML.set_q(p, q0)
        loss, dq0, _ = adjoint.grad(p, ns, checkpoint_every=every)
        p.close()
        if ref is None:
            ref = (loss, dq0)
        else:
            assert loss == ref[0] and np.array_equal(dq0, ref[1])
    p = ML.Problem(nl, "GPU", T=np.float64, precision="DF64", **kw)
    ML.set_q(p, q0)
    loss, dq0, _ = adjoint.grad(p, ns, checkpoint_every=4)
    p.close()
    assert abs(loss - L) <= 1e-12 * L and rel(dq0, gq) <= 1e-10


@pytest.mark.parametrize("stepper,H", [("FilteredETDRK4", np.inf), ("RK4", 1.0)])
def test_sqg_gradient_matches_oracle_adjoint(stepper, H):
    from gfcuda import SurfaceQG as SQ
    n, ns = 64, 10
    g = O.Grid(n)
    kw = dict(nx=n, H=H, nu=1e-4, nnu=1, dt=0.005, stepper=stepper)
    b0 = O.peakedisotropicspectrum(g, 5, 0.5, seed=3)
    p = SQ.Problem("GPU", T=np.float64, **kw)
    SQ.set_b(p, b0)
    loss, db0, deta = adjoint.grad(p, ns, checkpoint_every=4)
    p.close()
    assert deta is None
    L, gb, _ = AD.SQGAdjoint(O.SurfaceQG(**kw)).gradient(b0, np.zeros((n, n)), ns)
    assert abs(loss - L) <= 1e-13 * L and rel(db0, gb) <= 1e-11
