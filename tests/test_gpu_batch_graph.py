"""Ensembles (batched contexts), graph replay of captured steps and gf_ensemble_step.

A batched context must give, instance by instance, what independent single-instance runs
give (instance i draws its stochastic forcing with key seed + i), and replaying captured
graphs must give what kernel-by-kernel launches give."""
import numpy as np
import pytest

import gf_oracle as O

pytestmark = pytest.mark.gpu

gfcuda = pytest.importorskip("gfcuda")
from gfcuda import SingleLayerQG as SL, TwoDNavierStokes as TD  # noqa: E402
from gfcuda import Forcing, ensemble_step, stepforward  # noqa: E402


def rel(a, b):
    return O.rel_l2(a, b)


def zeta0(n, seed):
    return O.peakedisotropicspectrum(O.Grid(n), 4, 0.5, mask=O.makefilter(O.Grid(n)), seed=seed)


@pytest.mark.parametrize("T", [np.float32, np.float64])
def test_batch_matches_independent_runs(T):
    n, B, dt = 64, 3, 0.01
    spec = O.ring_forcing_spectrum(O.Grid(n), 8.0, 1.5, 1e-3)
    kw = dict(nx=n, dt=dt, nu=1e-4, nnu=1, stepper="FilteredRK4", T=T)
    pb = TD.Problem("GPU", batch=B, forcing=Forcing("stochastic", spectrum=spec, seed=100), **kw)
    TD.set_zeta(pb, np.stack([zeta0(n, s) for s in range(B)]))
    stepforward(pb, 7)
    sol_b = pb.sol
    E_b = pb.diagnostics([0, 1])
    assert sol_b.shape == (B, n, n // 2 + 1) and E_b.shape == (B, 2)
    for i in range(B):
        p = TD.Problem("GPU", forcing=Forcing("stochastic", spectrum=spec, seed=100 + i), **kw)
        TD.set_zeta(p, zeta0(n, i))
        stepforward(p, 7)
        assert rel(sol_b[i], p.sol) <= (1e-6 if T == np.float32 else 1e-14)
        assert np.allclose(E_b[i], p.diagnostics([0, 1]), rtol=1e-6 if T == np.float32 else 1e-13)


@pytest.mark.parametrize("stepper", ["FilteredRK4", "ETDRK4", "AB3", "ForwardEuler"])
@pytest.mark.parametrize("forcing", ["harmonic", "stochastic"])
def test_graph_replay_matches_direct_launches(stepper, forcing):
    n, dt = 128, 0.005
    g = O.Grid(n)
    x, y = g.gridpoints()
    if forcing == "harmonic":
        f = lambda: Forcing("harmonic", Fh=O.rfft2(0.1 * np.cos(4 * x) * np.cos(5 * y)), omega=2.0, phase=0.3)
    else:
        spec = O.ring_forcing_spectrum(g, 10.0, 1.5, 1e-2)
        f = lambda: Forcing("stochastic", spectrum=spec, seed=5)
    sols = []
    for graph_steps in (0, 4, 1):
        p = TD.Problem("GPU", nx=n, dt=dt, nu=1e-3, nnu=1, mu=0.05, nmu=0, stepper=stepper, forcing=f())
        p.set_graph_steps(graph_steps)
        TD.set_zeta(p, zeta0(n, 3))
        stepforward(p, 5)
        p.set_clock(p.clock.t, p.clock.step)   # a clock reset in between must be honoured
        stepforward(p, 9)
        sols.append((p.sol, p.clock.t, p.clock.step, TD.energy(p)))
    for s in sols[1:]:
        assert rel(s[0], sols[0][0]) <= 1e-15
        assert s[1] == sols[0][1] and s[2] == sols[0][2] == 14
        assert s[3] == sols[0][3]


def test_graph_matches_oracle_with_harmonic_forcing():
    """graph replay with the device clock against the FP64 oracle"""
    n, dt = 64, 0.01
    g = O.Grid(n)
    x, y = g.gridpoints()
    Fh = O.rfft2(0.1 * np.cos(4 * x) * np.cos(5 * y))
    p = TD.Problem("GPU", nx=n, dt=dt, nu=1e-3, nnu=1, stepper="RK4",
                   forcing=Forcing("harmonic", Fh=Fh, omega=2.0, phase=0.3))
    r = O.TwoDNavierStokes(nx=n, dt=dt, nu=1e-3, nnu=1, stepper="RK4",
                           forcing=O.Forcing("harmonic", Fh=Fh, omega=2.0, phase=0.3))
    z = zeta0(n, 1)
    TD.set_zeta(p, z)
    r.set_zeta(z)
    stepforward(p, 12)
    r.stepforward(12)
    assert rel(p.sol, r.sol) <= 1e-12
    assert abs(TD.energy_work(p) - r.energy_work()) <= 1e-11 * abs(r.energy_work())


def test_ensemble_step_three_size_classes():
    """the 1536-run ensemble in miniature: three batched size classes stepped by one call"""
    probs, refs = [], []
    for n, B in ((64, 4), (128, 2), (256, 1)):
        spec = O.ring_forcing_spectrum(O.Grid(n), 8.0, 1.5, 1e-3)
        kw = dict(nx=n, dt=0.01, nu=1e-4, nnu=1, stepper="FilteredRK4", T=np.float32)
        probs.append(TD.Problem("GPU", batch=B, forcing=Forcing("stochastic", spectrum=spec, seed=n), **kw))
        refs.append(TD.Problem("GPU", batch=B, forcing=Forcing("stochastic", spectrum=spec, seed=n), **kw))
    ensemble_step(probs, 6)
    for p, q in zip(probs, refs):
        stepforward(q, 6)
        assert rel(p.sol, q.sol) <= 1e-7
        assert p.clock.step == 6


def test_batched_slqg_etdrk4_parity():
    n, B = 64, 2
    spec = O.ring_forcing_spectrum(O.Grid(n), 10.0, 1.5, 1e-3)
    kw = dict(nx=n, beta=10.0, mu=0.01, dt=0.05, stepper="ETDRK4")
    p = SL.Problem("GPU", batch=B, forcing=Forcing("stochastic", spectrum=spec, seed=21), **kw)
    stepforward(p, 6)
    for i in range(B):
        r = O.SingleLayerQG(forcing=O.Forcing("stochastic", spectrum=spec, seed=21 + i), **kw)
        r.stepforward(6)
        assert rel(p.sol[i], r.sol) <= 1e-12


@pytest.mark.parametrize("T", [np.float32, np.float64])
@pytest.mark.parametrize("stepper", ["FilteredRK4", "AB3"])
def test_autotune_keeps_state_and_results(T, stepper):
    """the autotuner restores state, clock and AB3 history, and every launch shape gives the
    same step up to rounding (FP32: radices 4, 8, 16 reorder the butterflies)"""
    n = 128
    spec = O.ring_forcing_spectrum(O.Grid(n), 8.0, 1.5, 1e-3)
    kw = dict(nx=n, dt=0.01, nu=1e-4, nnu=1, stepper=stepper, T=T)
    mk = lambda: TD.Problem("GPU", forcing=Forcing("stochastic", spectrum=spec, seed=3), **kw)
    p, q = mk(), mk()
    for r in (p, q):
        TD.set_zeta(r, zeta0(n, 2))
        stepforward(r, 5)
    sol0 = p.sol
    shape = p.autotune(reps=2)
    assert np.array_equal(p.sol, sol0) and p.clock.step == 5
    assert shape["col_radix"] in ((4, 8, 16) if T == np.float32 else (8,))
    assert p.launch_shape == tuple(shape[k] for k in ("row_radix", "row_pairs", "col_radix", "col_columns"))
    assert p.tma_columns == shape["tma_columns"]
    stepforward(p, 6)
    stepforward(q, 6)
    assert rel(p.sol, q.sol) <= (1e-5 if T == np.float32 else 1e-13)
    for sh in ((16, 1, 16, 1), (4, 2, 4, 4), (8, 4, 8, 2)) if T == np.float32 else ((8, 2, 8, 4),):
        r = mk()
        r.launch_shape = sh
        TD.set_zeta(r, zeta0(n, 2))
        stepforward(r, 11)
        assert rel(r.sol, q.sol) <= (1e-5 if T == np.float32 else 1e-13)
    with pytest.raises(ValueError):
        p.launch_shape = (3, 1, 8, 1)


def test_ensemble_graph_ordering_remainders_and_fallback():
    """one ensemble graph over several contexts: results equal per-context stepping for step
    counts that are not multiples of the graph length, calls on any member after it see its
    result, and contexts that cannot share a graph (AB3) step on their own streams"""
    def make(n, B, stepper, seed):
        spec = O.ring_forcing_spectrum(O.Grid(n), 8.0, 1.5, 1e-3)
        return TD.Problem("GPU", nx=n, dt=0.01, nu=1e-4, nnu=1, stepper=stepper, T=np.float32, batch=B,
                          forcing=Forcing("stochastic", spectrum=spec, seed=seed))
    for steppers in (("FilteredRK4", "FilteredRK4", "ETDRK4"), ("FilteredRK4", "AB3", "ETDRK4")):
        probs = [make(n, B, st, 10 * n) for (n, B), st in zip(((64, 3), (128, 2), (32, 5)), steppers)]
        refs = [make(n, B, st, 10 * n) for (n, B), st in zip(((64, 3), (128, 2), (32, 5)), steppers)]
        for p, q in zip(probs, refs):
            z = np.stack([zeta0(p.grid.nx, i) for i in range(p.batch)])
            TD.set_zeta(p, z)
            TD.set_zeta(q, z)
        ensemble_step(probs, 11)           # 2 graph replays + 3 single steps
        for p in probs[1:]:
            TD.set_zeta(p, p.invtransform(p.sol))   # work issued on a member's stream after it
        ensemble_step(probs, 5)
        for k, q in enumerate(refs):
            stepforward(q, 11)
            if k > 0:
                TD.set_zeta(q, q.invtransform(q.sol))
            stepforward(q, 5)
        for p, q in zip(probs, refs):
            assert rel(p.sol, q.sol) <= 1e-6 and p.clock.step == q.clock.step == 16
