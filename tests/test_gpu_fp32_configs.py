"""FP32 bulk arithmetic against the FP64 oracle at the full sizes of the benchmark workloads.

The FP32 form of the step must stay within 1e-5 relative L2 of the FP64 oracle after 100
steps on each workload it is timed on (the oracle follows the reference's Float64 CPU path):

* TwoDNavierStokes 2048^2 FilteredRK4 dt = 5e-4, nu = 0, peaked isotropic initial vorticity
  (k0 = 6, E = 0.5) -- the headline workload;
* SingleLayerQG 512^2 beta-plane, beta = 10, mu = 0.01, ETDRK4 dt = 0.05, stochastic ring
  forcing at kf = 14 (width 1.5, injection 1e-3), q0 = 0;
* MultiLayerQG 3 x 1024^2 ETDRK4 dt = 2.5e-3, H = [.2, .3, .5], b from rho = [4, 5, 5.5]
  (g = 1), f0 = 1, beta = 5, U = [1, .5, 0], bottom drag 0.05, q0 white noise 1e-2;
* the 1536-run TwoDNavierStokes ensemble (1024 x 64^2, 384 x 128^2, 128 x 256^2,
  FilteredRK4 dt = 0.01, nu = 1e-4, per-instance stochastic ring forcing kf = 8), 200 steps,
  instances sampled from every size class;
* the FP32 adjoint of SingleLayerQG 256^2 (deformation radius 0.35, topography |k| <= 8
  amplitude 0.1, ETDRK4 dt = 0.01): gradient of the final kinetic energy against the
  oracle's discrete adjoint over one checkpoint interval (25 steps, <= 1e-5), and against
  the FP64 GPU gradient over the full 500 steps (<= 2e-2: chaotic growth of rounding).

The oracle runs its FFTs on every host core (scipy.fft workers) so that the 2048^2 and
3 x 1024^2 references finish in about a minute each."""
import os

import numpy as np
import pytest

import gf_adjoint as AD
import gf_oracle as O

pytestmark = pytest.mark.gpu

gfcuda = pytest.importorskip("gfcuda")
from gfcuda import MultiLayerQG as ML, SingleLayerQG as SL, TwoDNavierStokes as TD, adjoint  # noqa: E402
from gfcuda import Forcing, ensemble_step, stepforward  # noqa: E402

TOL32 = 1e-5


@pytest.fixture(autouse=True)
def _threaded_oracle():
    O.set_fft_workers(os.cpu_count())
    yield
    O.set_fft_workers(None)


def rel(a, b):
    return O.rel_l2(a, b)


def test_fp32_twodns_2048_against_fp64_oracle():
    n, dt, ns = 2048, 5e-4, 100
    r = O.TwoDNavierStokes(nx=n, dt=dt, stepper="FilteredRK4")
    z0 = O.peakedisotropicspectrum(r.grid, 6, 0.5, mask=r.timestepper.filter, seed=1234)
    r.set_zeta(z0)
    p = TD.Problem("GPU", nx=n, dt=dt, stepper="FilteredRK4", T=np.float32)
    TD.set_zeta(p, z0)
    stepforward(p, ns)
    r.stepforward(ns)
    err = rel(p.sol, r.sol)
    print(f"2048^2 FilteredRK4 FP32 vs oracle after {ns} steps: {err:.3e}")
    assert err <= TOL32
    assert abs(TD.energy(p) - r.energy()) <= TOL32 * r.energy()
    p.close()


def test_fp32_slqg_512_beta_forced_against_fp64_oracle():
    n, dt, ns = 512, 0.05, 100
    spec = O.ring_forcing_spectrum(O.Grid(n), 14.0, 1.5, 1e-3)
    f = Forcing("stochastic", spectrum=spec, seed=1234)
    p = SL.Problem("GPU", nx=n, beta=10.0, mu=0.01, dt=dt, stepper="ETDRK4", forcing=f, T=np.float32)
    r = O.SingleLayerQG(nx=n, beta=10.0, mu=0.01, dt=dt, stepper="ETDRK4",
                        forcing=O.Forcing("stochastic", spectrum=spec, seed=1234))
    SL.set_q(p, np.zeros((n, n)))
    stepforward(p, ns)
    r.stepforward(ns)
    err = rel(p.sol, r.sol)
    print(f"SLQG 512^2 ETDRK4 FP32 vs oracle after {ns} steps: {err:.3e}")
    assert err <= TOL32
    assert abs(SL.energy(p) - r.energy()) <= TOL32 * r.energy()
    p.close()


MLQG = dict(nx=1024, ny=1024, f0=1.0, beta=5.0, H=[0.2, 0.3, 0.5], b=[-1.0, -1.2, -1.2 - 0.5 / 5.5],
            U=[1.0, 0.5, 0.0], mu=0.05, dt=2.5e-3, stepper="ETDRK4")


def test_fp32_mlqg_3x1024_against_fp64_oracle():
    ns = 100
    q0 = 1e-2 * np.random.default_rng(1234).standard_normal((3, 1024, 1024))
    p = ML.Problem(3, "GPU", T=np.float32, **MLQG)
    r = O.MultiLayerQG(3, **MLQG)
    ML.set_q(p, q0)
    r.set_q(q0)
    stepforward(p, ns)
    r.stepforward(ns)
    err = rel(p.sol, r.sol)
    per_layer = [rel(p.sol[a], r.sol[a]) for a in range(3)]
    print(f"MLQG 3x1024^2 ETDRK4 FP32 vs oracle after {ns} steps: {err:.3e} (layers {per_layer})")
    assert err <= TOL32
    p.close()


def test_fp32_ensemble_1536_sampled_instances_against_fp64_oracle():
    dt, ns = 0.01, 200
    classes = ((64, 1024, (0, 517, 1023)), (128, 384, (0, 383)), (256, 128, (0, 127)))
    probs, specs = [], []
    for n, B, _ in classes:
        spec = O.ring_forcing_spectrum(O.Grid(n), 8.0, 1.5, 1e-3)
        specs.append(spec)
        probs.append(TD.Problem("GPU", nx=n, dt=dt, nu=1e-4, nnu=1, stepper="FilteredRK4", T=np.float32, batch=B,
                                forcing=Forcing("stochastic", spectrum=spec, seed=1000 * n)))
    for p in probs:
        p.set_graph_steps(10)
    ensemble_step(probs, ns)
    for p, spec, (n, B, sample) in zip(probs, specs, classes):
        sol = p.sol
        for i in sample:
            r = O.TwoDNavierStokes(nx=n, dt=dt, nu=1e-4, nnu=1, stepper="FilteredRK4",
                                   forcing=O.Forcing("stochastic", spectrum=spec, seed=1000 * n + i))
            r.stepforward(ns)
            err = rel(sol[i], r.sol)
            print(f"ensemble {n}^2 instance {i} FP32 vs oracle after {ns} steps: {err:.3e}")
            assert err <= TOL32, (n, i)
        p.close()


ADJ = dict(nx=256, deformation_radius=0.35, dt=0.01, stepper="ETDRK4")


def _adj_case():
    g = O.Grid(256)
    eta = AD.random_topography(g, 8, 0.1, 7)
    q0 = O.peakedisotropicspectrum(g, 6, 0.5, seed=1234)
    return dict(ADJ, eta=eta), q0, eta


def _gpu_grad(kw, q0, ns, every, T):
    p = SL.Problem("GPU", T=T, **kw)
    SL.set_q(p, q0)
    loss, dq0, deta = adjoint.grad(p, ns, checkpoint_every=every)
    p.close()
    return loss, dq0, deta


def test_fp32_adjoint_256_one_interval_against_oracle_adjoint():
    kw, q0, eta = _adj_case()
    ns = 25
    loss, dq0, deta = _gpu_grad(kw, q0, ns, 25, np.float32)
    L, gq, ge = AD.SLQGAdjoint(O.SingleLayerQG(**kw)).gradient(q0, eta, ns)
    eq, ee = rel(dq0, gq), rel(deta, ge)
    print(f"adjoint 256^2 FP32 vs oracle adjoint, {ns} steps: loss {abs(loss - L) / L:.2e} dq0 {eq:.2e} deta {ee:.2e}")
    assert abs(loss - L) <= TOL32 * L
    assert eq <= TOL32 and ee <= TOL32


def test_fp32_adjoint_256_500_steps_against_fp64_gradient():
    """Over 500 nonlinear steps the FP32 and FP64 trajectories separate by chaotic growth of
    rounding: the losses agree to ~1e-6, the gradients (which weigh the fastest-growing
    perturbations) to ~5e-3 on GB300; 2e-2 is the bound checked."""
    kw, q0, _ = _adj_case()
    l32, q32, e32 = _gpu_grad(kw, q0, 500, 25, np.float32)
    l64, q64, e64 = _gpu_grad(kw, q0, 500, 25, np.float64)
    eq, ee = rel(q32, q64), rel(e32, e64)
    print(f"adjoint 256^2 FP32 vs FP64 GPU gradient, 500 steps: loss {abs(l32 - l64) / l64:.2e} dq0 {eq:.2e} "
          f"deta {ee:.2e}")
    assert abs(l32 - l64) <= TOL32 * l64
    assert eq <= 2e-2 and ee <= 2e-2
