"""The persistent ensemble launch (gf_ensemble_step with the persistent kernels): every stage
of every size class in one row launch and one column launch whose blocks walk the work list
of all classes' tiles.

It must step each instance as an independent run does: against the per-class execution (one
batched context per stream) to rounding (its radices and tiles differ: FP32 1e-6, FP64 1e-13
relative L2), and sampled instances of every class against the FP64 oracle (FP64 and df64
1e-12, FP32 1e-5), for FilteredRK4 with per-instance stochastic forcing (the benchmark's
ensemble physics) and ETDRK4 SingleLayerQG with beta, over calls that mix pruned and
observed steps.  Members it cannot fuse (AB3, several layers) fall back to per-class
execution with the same results."""
import numpy as np
import pytest

import gf_oracle as O

pytestmark = pytest.mark.gpu

gfcuda = pytest.importorskip("gfcuda")
from gfcuda import MultiLayerQG as ML, SingleLayerQG as SL, TwoDNavierStokes as TD  # noqa: E402
from gfcuda import Forcing, ensemble_step  # noqa: E402

CLASSES = ((64, 6), (128, 3), (256, 2), (32, 5))


def make_twodns(T, prec, stepper="FilteredRK4"):
    probs, specs = [], []
    for n, B in CLASSES:
        spec = O.ring_forcing_spectrum(O.Grid(n), 8.0, 1.5, 1e-3)
        specs.append(spec)
        probs.append(TD.Problem("GPU", nx=n, dt=0.01, nu=1e-4, nnu=1, stepper=stepper, T=T, precision=prec, batch=B,
                                forcing=Forcing("stochastic", spectrum=spec, seed=1000 * n)))
    return probs, specs


def run(probs, calls, persistent, graph_steps=4):
    for p in probs:
        p.set_graph_steps(graph_steps)
    for n in calls:
        ensemble_step(probs, n, persistent=persistent)
    return [p.sol for p in probs]


@pytest.mark.parametrize("T,prec,tol", [(np.float32, None, 1e-6), (np.float64, None, 1e-13),
                                        (np.float64, "DF64", 1e-13)])
def test_persistent_equals_per_class_execution(T, prec, tol):
    calls = (9, 4, 3)
    a = run(make_twodns(T, prec)[0], calls, True)
    b = run(make_twodns(T, prec)[0], calls, False)
    for x, y in zip(a, b):
        assert O.rel_l2(x, y) <= tol


@pytest.mark.parametrize("T,prec,tol", [(np.float32, None, 1e-5), (np.float64, None, 1e-12),
                                        (np.float64, "DF64", 1e-12)])
def test_persistent_instances_match_oracle(T, prec, tol):
    probs, specs = make_twodns(T, prec)
    ns = 16
    sols = run(probs, (ns,), True)
    for (n, B), spec, sol in zip(CLASSES, specs, sols):
        for i in (0, B - 1):
            r = O.TwoDNavierStokes(nx=n, dt=0.01, nu=1e-4, nnu=1, stepper="FilteredRK4",
                                   forcing=O.Forcing("stochastic", spectrum=spec, seed=1000 * n + i))
            r.stepforward(ns)
            assert O.rel_l2(sol[i], r.sol) <= tol, (n, i)


def test_persistent_slqg_etdrk4_beta():
    rng = np.random.default_rng(4)
    sizes = ((64, 3), (128, 2))
    kw = dict(beta=10.0, mu=0.01, dt=0.02, stepper="ETDRK4", T=np.float64)
    probs = [SL.Problem("GPU", nx=n, batch=B, **kw) for n, B in sizes]
    q0 = [0.1 * rng.standard_normal((B, n, n)) for n, B in sizes]
    for p, q in zip(probs, q0):
        SL.set_q(p, q)
    sols = run(probs, (6, 2), True)
    for (n, B), q, sol in zip(sizes, q0, sols):
        for i in range(B):
            r = O.SingleLayerQG(nx=n, beta=10.0, mu=0.01, dt=0.02, stepper="ETDRK4")
            r.set_q(q[i])
            r.stepforward(8)
            assert O.rel_l2(sol[i], r.sol) <= 1e-12


def test_members_that_cannot_fuse_fall_back():
    """an AB3 member or a two-layer member: the call runs the per-class execution"""
    def mk():
        a = TD.Problem("GPU", nx=64, dt=0.005, nu=1e-3, nnu=1, stepper="AB3", T=np.float64, batch=2)
        b = ML.Problem(2, "GPU", nx=64, H=[0.3, 0.7], b=[-1.0, -1.4], dt=0.005, stepper="RK4", T=np.float64)
        TD.set_zeta(a, 0.1 * np.random.default_rng(1).standard_normal((2, 64, 64)))
        ML.set_q(b, 0.1 * np.random.default_rng(2).standard_normal((2, 64, 64)))
        return [a, b]
    x = run(mk(), (7,), True, graph_steps=3)
    y = run(mk(), (7,), False, graph_steps=3)
    for u, v in zip(x, y):
        assert np.array_equal(u, v)
