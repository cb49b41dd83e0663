"""Unobserved steps: inside a stepforward!(prob, n) call only the last step (AB3: the last
three) computes the aliased modes of the state; the others form the products only for
kr < kcut and update only the kept modes.  Every calcN! starts with dealias!(sol)
(FourierFlows src/timesteppers.jl stage loops; GeophysicalFlows calcN! of each module), so
what a call leaves behind -- every mode of sol, the clock, the diagnostics -- must equal,
bit for bit, n calls of one step each (every step observed)."""
import numpy as np
import pytest

import gf_oracle as O

pytestmark = pytest.mark.gpu

gfcuda = pytest.importorskip("gfcuda")
from gfcuda import BarotropicQGQL as QL  # noqa: E402
from gfcuda import MultiLayerQG as ML  # noqa: E402
from gfcuda import SingleLayerQG as SL  # noqa: E402
from gfcuda import SurfaceQG as SQ  # noqa: E402
from gfcuda import TwoDNavierStokes as TD  # noqa: E402
from gfcuda import Forcing, ensemble_step, stepforward  # noqa: E402

N_STEPS = 9


def zeta0(n, seed, batch=None):
    z = lambda s: O.peakedisotropicspectrum(O.Grid(n), 4, 0.5, mask=O.makefilter(O.Grid(n)), seed=s)
    return z(seed) if batch is None else np.stack([z(seed + i) for i in range(batch)])


def pair(make, init, graph_steps=0):
    """two identical problems: p stepped by one call of N_STEPS steps, q by N_STEPS calls"""
    p, q = make(), make()
    for r in (p, q):
        r.set_graph_steps(graph_steps)
        init(r)
    stepforward(p, N_STEPS)
    for _ in range(N_STEPS):
        stepforward(q, 1)
    return p, q


def same(p, q):
    assert np.array_equal(p.sol, q.sol)
    assert p.clock.step == q.clock.step and p.clock.t == q.clock.t


@pytest.mark.parametrize("stepper", ["FilteredRK4", "RK4", "ETDRK4", "FilteredETDRK4", "AB3", "FilteredAB3",
                                     "ForwardEuler"])
@pytest.mark.parametrize("T,prec", [(np.float32, None), (np.float64, None), (np.float64, "DF64")])
def test_twodns_one_call_equals_single_steps(stepper, T, prec):
    n = 128
    spec = O.ring_forcing_spectrum(O.Grid(n), 8.0, 1.5, 1e-3)
    make = lambda: TD.Problem("GPU", nx=n, dt=0.005, nu=1e-4, nnu=1, mu=0.05, nmu=0, stepper=stepper, T=T,
                              precision=prec, forcing=Forcing("stochastic", spectrum=spec, seed=11))
    p, q = pair(make, lambda r: TD.set_zeta(r, zeta0(n, 2)))
    same(p, q)
    # the step's own forcing and previous state (the work diagnostic) and the energy
    assert TD.energy_work(p) == TD.energy_work(q)
    assert TD.energy(p) == TD.energy(q) and TD.enstrophy(p) == TD.enstrophy(q)
    # the aliased modes of the result are there (nonzero) after the call
    aliased = O.Grid(n).dealias_mask() == 0
    assert np.count_nonzero(p.sol[aliased]) > 0.5 * np.count_nonzero(aliased)


@pytest.mark.parametrize("nx,ny,Lx,Ly", [(128, 64, 2 * np.pi, np.pi), (64, 256, 3.0, 7.0)])
def test_rectangular_grids(nx, ny, Lx, Ly):
    """kcut and the aliased l band of a rectangular grid (the launch grid of unobserved steps
    covers the kept columns only)"""
    make = lambda: TD.Problem("GPU", nx=nx, ny=ny, Lx=Lx, Ly=Ly, dt=0.002, nu=1e-4, nnu=1,
                              stepper="FilteredRK4", T=np.float64)
    rng = np.random.default_rng(3)
    z0 = rng.standard_normal((ny, nx))
    p, q = pair(make, lambda r: TD.set_zeta(r, z0))
    same(p, q)
    r = O.TwoDNavierStokes(nx=nx, ny=ny, Lx=Lx, Ly=Ly, dt=0.002, nu=1e-4, nnu=1, stepper="FilteredRK4")
    r.set_zeta(z0)
    r.stepforward(N_STEPS)
    assert O.rel_l2(p.sol, r.sol) <= 1e-12


@pytest.mark.parametrize("graph_steps", [0, 4])
def test_slqg_topography_stochastic_etdrk4(graph_steps):
    n = 128
    g = O.Grid(n)
    x, y = g.gridpoints()
    eta = 0.2 * np.cos(3 * x) * np.sin(2 * y)
    spec = O.ring_forcing_spectrum(g, 10.0, 1.5, 1e-3)
    make = lambda: SL.Problem("GPU", nx=n, beta=10.0, mu=0.01, U=0.3, eta=eta, deformation_radius=1.2, dt=0.02,
                              stepper="ETDRK4", forcing=Forcing("stochastic", spectrum=spec, seed=4))
    rng = np.random.default_rng(1)
    q0 = 0.1 * rng.standard_normal((n, n))
    p, q = pair(make, lambda r: SL.set_q(r, q0), graph_steps)
    same(p, q)


@pytest.mark.parametrize("prec", [None, "DF64"])
def test_mlqg_three_layers_drag(prec):
    n, nl = 128, 3
    kw = dict(nx=n, f0=1.0, beta=5.0, H=[0.2, 0.3, 0.5], b=[-1.0, -1.2, -1.290909], U=[1.0, 0.5, 0.0], mu=0.05,
              dt=2.5e-3, stepper="ETDRK4")
    rng = np.random.default_rng(5)
    q0 = 1e-2 * rng.standard_normal((nl, n, n))
    p, q = pair(lambda: ML.Problem(nl, "GPU", precision=prec, **kw), lambda r: ML.set_q(r, q0))
    same(p, q)
    for a, b in zip(ML.energies(p), ML.energies(q)):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("nl", [4, 5])
def test_mlqg_more_than_three_layers(nl):
    """beyond three layers the inverse column launch reads the layers' X from global memory
    (no staging into its three work buffers): oracle parity and one call = single steps"""
    n = 64
    H = list(np.linspace(0.1, 0.3, nl))
    b = list(-1.0 - 0.15 * np.arange(nl))
    U = list(np.linspace(1.0, 0.0, nl))
    kw = dict(nx=n, f0=1.0, beta=5.0, H=H, b=b, U=U, mu=0.05, dt=2.5e-3, stepper="ETDRK4")
    rng = np.random.default_rng(nl)
    q0 = 1e-2 * rng.standard_normal((nl, n, n))
    p, q = pair(lambda: ML.Problem(nl, "GPU", **kw), lambda r: ML.set_q(r, q0))
    same(p, q)
    r = O.MultiLayerQG(nl, **kw)
    r.set_q(q0)
    r.stepforward(N_STEPS)
    assert O.rel_l2(p.sol, r.sol) <= 1e-11


def test_mlqg_batched_layer_split():
    """a batched three-layer context (instance = blockIdx.y, layer = blockIdx.z of the split
    column launches) equals independent runs bit for bit"""
    n, nl, B = 64, 3, 2
    kw = dict(nx=n, f0=1.0, beta=5.0, H=[0.2, 0.3, 0.5], b=[-1.0, -1.2, -1.290909], U=[1.0, 0.5, 0.0], mu=0.05,
              dt=2.5e-3, stepper="ETDRK4")
    rng = np.random.default_rng(8)
    q0 = 1e-2 * rng.standard_normal((B, nl, n, n))
    pb = ML.Problem(nl, "GPU", batch=B, **kw)
    ML.set_q(pb, q0)
    stepforward(pb, N_STEPS)
    for i in range(B):
        p = ML.Problem(nl, "GPU", **kw)
        ML.set_q(p, q0[i])
        stepforward(p, N_STEPS)
        assert np.array_equal(pb.sol[i], p.sol)


def test_surfaceqg_and_qgql():
    n = 128
    rng = np.random.default_rng(9)
    b0 = 0.1 * rng.standard_normal((n, n))
    p, q = pair(lambda: SQ.Problem("GPU", nx=n, nu=1e-4, nnu=1, H=1.3, dt=0.005, stepper="FilteredRK4"),
                lambda r: SQ.set_b(r, b0))
    same(p, q)
    p, q = pair(lambda: QL.Problem("GPU", nx=n, beta=2.0, nu=1e-3, nnu=1, mu=0.05, dt=0.005, stepper="RK4"),
                lambda r: QL.set_zeta(r, b0))
    same(p, q)


@pytest.mark.parametrize("stepper", ["FilteredRK4", "ETDRK4", "AB3"])
@pytest.mark.parametrize("nsteps", [8, 12, 13])
def test_graph_replays_of_a_long_call(stepper, nsteps):
    """calls longer than the graph: replays followed by more steps of the same call capture
    every step unobserved, the replay that ends the call its last step (AB3: three)
    observed; the result equals single-step calls bit for bit"""
    n = 128
    spec = O.ring_forcing_spectrum(O.Grid(n), 8.0, 1.5, 1e-3)
    make = lambda: TD.Problem("GPU", nx=n, dt=0.005, nu=1e-4, nnu=1, stepper=stepper, T=np.float32,
                              forcing=Forcing("stochastic", spectrum=spec, seed=7))
    p, q = make(), make()
    for r in (p, q):
        TD.set_zeta(r, zeta0(n, 4))
    p.set_graph_steps(4)
    q.set_graph_steps(0)
    stepforward(p, nsteps)
    stepforward(p, nsteps)        # the captured graphs replayed again
    for _ in range(2 * nsteps):
        stepforward(q, 1)
    same(p, q)
    assert TD.energy_work(p) == TD.energy_work(q)


@pytest.mark.parametrize("shape", [(8, 1, 8, 5), (8, 1, 16, 5)])
def test_wide_column_blocks(shape):
    """FP32 columns of 1024 with five columns per block (640 threads: the wide instantiation,
    two shared-memory buffers) in the unobserved steps; the observed steps run 512-thread
    blocks, whose FFT code differs (lockstep grouping, the compiler's FMA contraction), so
    one call equals single observed steps to FP32 rounding, and matches the FP64 path."""
    n = 1024
    make = lambda: TD.Problem("GPU", nx=n, dt=0.001, nu=1e-4, nnu=1, stepper="FilteredRK4", T=np.float32)
    z = zeta0(n, 3)

    def init(r):
        r.launch_shape = shape
        TD.set_zeta(r, z)
    p, q = pair(make, init)
    assert p.clock.step == q.clock.step == N_STEPS
    assert O.rel_l2(p.sol, q.sol) <= 1e-6
    r = TD.Problem("GPU", nx=n, dt=0.001, nu=1e-4, nnu=1, stepper="FilteredRK4", T=np.float64)
    TD.set_zeta(r, z)
    stepforward(r, N_STEPS)
    assert O.rel_l2(p.sol, r.sol) <= 1e-5


@pytest.mark.parametrize("prec", [None, "DF64"])
def test_narrow_column_blocks(prec):
    """FP64 and df64 columns of 1024, one column per block (df64: the narrow 256-thread
    instantiation with three blocks per SM and two shared-memory buffers) in observed and
    unobserved steps: one call equals single steps bit for bit, and the FP64 oracle"""
    n = 1024
    make = lambda: TD.Problem("GPU", nx=n, dt=0.001, nu=1e-4, nnu=1, stepper="FilteredRK4", T=np.float64,
                              precision=prec)
    rng = np.random.default_rng(6)
    z = 0.5 * np.fft.irfft2(np.fft.rfft2(rng.standard_normal((n, n))) * O.Grid(n).dealias_mask(), s=(n, n))

    def init(r):
        r.launch_shape = (8, 1, 8, 1)
        TD.set_zeta(r, z)
    p, q = pair(make, init)
    same(p, q)
    r = O.TwoDNavierStokes(nx=n, dt=0.001, nu=1e-4, nnu=1, stepper="FilteredRK4")
    r.set_zeta(z)
    r.stepforward(N_STEPS)
    assert O.rel_l2(p.sol, r.sol) <= 1e-12


def test_df64_two_buffer_rows_with_topography():
    """df64 rows of 1024 with topography: the two-buffer row instantiation forms q + eta once
    and keeps it for both products; it matches the IEEE FP64 path"""
    n = 1024
    g = O.Grid(n)
    x, y = g.gridpoints()
    eta = 0.2 * np.cos(3 * x) * np.sin(2 * y)
    rng = np.random.default_rng(2)
    q0 = 0.1 * np.fft.irfft2(np.fft.rfft2(rng.standard_normal((n, n))) * g.dealias_mask(), s=(n, n))
    sols = []
    for prec in ("DF64", None):
        p = SL.Problem("GPU", nx=n, beta=10.0, mu=0.01, U=0.3, eta=eta, deformation_radius=1.2, dt=0.002,
                       stepper="ETDRK4", T=np.float64, precision=prec)
        p.launch_shape = (8, 1, 8, 1)
        SL.set_q(p, q0)
        stepforward(p, N_STEPS)
        sols.append(p.sol)
    assert O.rel_l2(sols[0], sols[1]) <= 1e-12


def test_batched_and_ensemble_graph():
    """a batched context and one ensemble graph over two contexts (graph of 4 steps: the
    last step of every replay observed)"""
    def make(n, B):
        spec = O.ring_forcing_spectrum(O.Grid(n), 8.0, 1.5, 1e-3)
        return TD.Problem("GPU", nx=n, dt=0.01, nu=1e-4, nnu=1, stepper="FilteredRK4", T=np.float32, batch=B,
                          forcing=Forcing("stochastic", spectrum=spec, seed=n))
    probs = [make(64, 3), make(128, 2)]
    refs = [make(64, 3), make(128, 2)]
    for r in probs + refs:
        r.set_graph_steps(4)
        TD.set_zeta(r, zeta0(r.grid.nx, 0, r.batch))
    ensemble_step(probs, N_STEPS)
    for r in refs:
        for _ in range(N_STEPS):
            stepforward(r, 1)
    for p, q in zip(probs, refs):
        same(p, q)

