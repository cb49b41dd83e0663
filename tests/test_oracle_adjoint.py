"""The oracle's tangent-linear and adjoint SingleLayerQG ETDRK4 and RK4 steps (oracle/gf_adjoint.py):
its forward pass is the oracle's stepforward!, its gradients of the final kinetic energy with
respect to q0 and the topography match central finite differences (eps = 1e-6) along seeded
directions, and adjoint and tangent-linear satisfy the dot-product identity."""
import numpy as np
import pytest

import gf_adjoint as AD
import gf_oracle as O


def setup(n, stepper, ell=0.35, U=0.0, beta=0.0, nsteps=12):
    g = O.Grid(n)
    eta = AD.random_topography(g, 8, 0.1, 7)
    if U == "y":   # a zonal jet U(y)
        U = 0.3 * np.cos(2 * g.y) + 0.1 * np.sin(g.y)
    kw = dict(nx=n, deformation_radius=ell, eta=eta, dt=0.01, stepper=stepper, U=U, beta=beta)
    p = O.SingleLayerQG(**kw)
    q0 = O.peakedisotropicspectrum(g, 6, 0.5, seed=1234)
    return p, AD.SLQGAdjoint(p), q0, eta, kw


CASES = [("ETDRK4", 0.35, 0.0, 0.0), ("ETDRK4", np.inf, 0.3, 2.0), ("FilteredETDRK4", 0.35, 0.1, 1.0),
         ("RK4", 0.35, 0.2, 1.0), ("FilteredRK4", np.inf, 0.0, 2.0), ("ETDRK4", 0.35, "y", 1.0),
         ("FilteredRK4", np.inf, "y", 0.0)]


@pytest.mark.parametrize("stepper,ell,U,beta", CASES)
def test_adjoint_forward_is_stepforward(stepper, ell, U, beta):
    p, A, q0, eta, kw = setup(32, stepper, ell, U, beta)
    p.set_q(q0)
    p.stepforward(12)
    assert A.loss(q0, eta, 12) == pytest.approx(p.kinetic_energy(), rel=1e-14)


@pytest.mark.parametrize("stepper,ell,U,beta", CASES)
def test_gradient_matches_central_differences(stepper, ell, U, beta):
    """the SingleLayerQG 256^2 adjoint check in miniature: 8 seeded directions, eps = 1e-6, 1e-6 relative"""
    p, A, q0, eta, kw = setup(32, stepper, ell, U, beta)
    ns = 12
    _, gq, ge = A.gradient(q0, eta, ns)
    rng = np.random.default_rng(8)
    for _ in range(8):
        dq, de = rng.standard_normal(q0.shape), 0.1 * rng.standard_normal(eta.shape)
        eps = 1e-6
        fd = (A.loss(q0 + eps * dq, eta + eps * de, ns) - A.loss(q0 - eps * dq, eta - eps * de, ns)) / (2 * eps)
        ad = np.sum(gq * dq) + np.sum(ge * de)
        assert abs(fd - ad) <= 1e-6 * abs(ad)


@pytest.mark.parametrize("stepper,U", [("ETDRK4", 0.2), ("FilteredRK4", 0.2), ("ETDRK4", "y")])
def test_dot_product_identity(stepper, U):
    p, A, q0, eta, kw = setup(32, stepper, 0.35, U, 1.0)
    ns = 6
    rng = np.random.default_rng(3)
    u = A.initial_state(q0)
    for _ in range(ns):
        u = A.step(u, eta)[0]
    du = A.initial_state(rng.standard_normal(q0.shape))
    de = rng.standard_normal(eta.shape)
    ubar = np.fft.rfft2(rng.standard_normal(q0.shape))
    lhs = np.sum(np.real(np.conj(ubar) * A.step_tlm(u, eta, du, de)))
    xb, eb = A.step_adj(u, eta, ubar)
    rhs = np.sum(np.real(np.conj(xb) * du)) + np.sum(eb * de)
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)
    # the transforms' transposes
    x = rng.standard_normal((16, 16))
    X = np.fft.rfft2(rng.standard_normal((16, 16))) + 0.3j * rng.standard_normal((16, 9))
    g = O.Grid(16)
    assert np.sum(np.real(np.conj(X) * O.rfft2(x))) == pytest.approx(np.sum(x * AD.rfft2_T(X, g)), rel=1e-12)
    assert np.sum(np.real(np.conj(X) * AD.irfft2_T(x, g))) == pytest.approx(np.sum(x * O.irfft2(X, g)), rel=1e-12)


def ml_setup(stepper, n=32, nl=3):
    g = O.Grid(n)
    kw = dict(nx=n, f0=1.0, beta=5.0, H=[0.2, 0.3, 0.5], b=[-1.0, -1.2, -1.2 - 0.5 / 5.5][:nl], U=[1.0, 0.5, 0.0][:nl],
              mu=0.05, dt=2.5e-3, stepper=stepper)
    if nl == 2:
        kw["H"] = [0.4, 0.6]
    kw["eta"] = AD.random_topography(g, 6, 0.3, 9)
    q0 = 1e-2 * np.random.default_rng(1234).standard_normal((nl, n, n))
    p = O.MultiLayerQG(nl, **kw)
    return p, AD.MLQGAdjoint(p), q0, kw


@pytest.mark.parametrize("stepper,nl", [("ETDRK4", 3), ("FilteredRK4", 2), ("RK4", 3)])
def test_mlqg_adjoint_forward_and_central_differences(stepper, nl):
    p, A, q0, kw = ml_setup(stepper, nl=nl)
    ns = 10
    p.set_q(q0)
    p.stepforward(ns)
    KE = p.energies()[0]
    assert A.loss(q0, kw["eta"], ns) == pytest.approx(float(np.sum(KE)), rel=1e-12)
    eta = kw["eta"]
    _, gq, ge = A.gradient(q0, eta, ns)
    rng = np.random.default_rng(5)
    g = O.Grid(32)
    for i in range(4):
        dq = rng.standard_normal(q0.shape)
        de = AD.random_topography(g, 6, 0.3, 40 + i)
        eps = 1e-6
        fd = (A.loss(q0 + eps * dq, eta + eps * de, ns) - A.loss(q0 - eps * dq, eta - eps * de, ns)) / (2 * eps)
        ad = float(np.sum(gq * dq)) + float(np.sum(ge * de))
        assert abs(fd - ad) <= 1e-6 * abs(ad)


def test_mlqg_dot_product_identity():
    p, A, q0, kw = ml_setup("ETDRK4")
    rng = np.random.default_rng(2)
    eta = kw["eta"]
    u = A.initial_state(q0)
    for _ in range(3):
        u = A.step(u, eta)[0]
    du = A.initial_state(rng.standard_normal(q0.shape))
    de = rng.standard_normal(eta.shape)
    ubar = np.fft.rfft2(rng.standard_normal(q0.shape))
    lhs = np.sum(np.real(np.conj(ubar) * A.step_tlm(u, eta, du, de)))
    xb, eb = A.step_adj(u, eta, ubar)
    rhs = np.sum(np.real(np.conj(xb) * du)) + np.sum(eb * de)
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)


@pytest.mark.parametrize("stepper,H", [("FilteredETDRK4", np.inf), ("RK4", 1.0)])
def test_sqg_adjoint_forward_and_central_differences(stepper, H):
    n, ns = 32, 10
    g = O.Grid(n)
    kw = dict(nx=n, H=H, nu=1e-4, nnu=1, dt=0.005, stepper=stepper)
    p = O.SurfaceQG(**kw)
    A = AD.SQGAdjoint(p)
    b0 = O.peakedisotropicspectrum(g, 5, 0.5, seed=3)
    p.set_b(b0)
    p.stepforward(ns)
    zero = np.zeros((n, n))
    assert A.loss(b0, zero, ns) == pytest.approx(p.kinetic_energy(), rel=1e-12)
    _, gb, _ = A.gradient(b0, zero, ns)
    rng = np.random.default_rng(6)
    for _ in range(4):
        db = rng.standard_normal(b0.shape)
        eps = 1e-6
        fd = (A.loss(b0 + eps * db, zero, ns) - A.loss(b0 - eps * db, zero, ns)) / (2 * eps)
        ad = float(np.sum(gb * db))
        assert abs(fd - ad) <= 1e-6 * abs(ad)
