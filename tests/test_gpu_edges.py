"""Edge cases of the GPU path against the oracle: other dealiasing fractions (including none),
rectangular grids in every module, the smallest and largest supported sizes, and the
Filtered steppers' filter parameters."""
import numpy as np
import pytest

import gf_oracle as O

pytestmark = pytest.mark.gpu

gfcuda = pytest.importorskip("gfcuda")
from gfcuda import (BarotropicQGQL as QL, MultiLayerQG as ML, SingleLayerQG as SL,  # noqa: E402
                    SurfaceQG as SQ, TwoDNavierStokes as TD)
from gfcuda import stepforward  # noqa: E402


def rel(a, b):
    return O.rel_l2(a, b)


def pair(module, **kw):
    if module == "TwoDNavierStokes":
        return TD.Problem("GPU", **kw), O.TwoDNavierStokes(**kw)
    if module == "SurfaceQG":
        return SQ.Problem("GPU", H=1.3, **kw), O.SurfaceQG(H=1.3, **kw)
    if module == "SingleLayerQG":
        k2 = dict(kw, beta=2.0, deformation_radius=1.7, U=0.2)
        return SL.Problem("GPU", **k2), O.SingleLayerQG(**k2)
    if module == "BarotropicQGQL":
        k2 = dict(kw, beta=2.0, mu=0.01)
        return QL.Problem("GPU", **k2), O.BarotropicQGQL(**k2)
    k2 = dict(kw, f0=1.0, beta=1.5, H=[0.3, 0.7], b=[-1.0, -1.3], U=[0.4, 0.0], mu=0.05)
    return ML.Problem(2, "GPU", **k2), O.MultiLayerQG(2, **k2)


def random_state(p, seed):
    rng = np.random.default_rng(seed)
    shp = p.phys_shape
    return np.fft.rfft2(rng.standard_normal(shp), axes=(-2, -1))


@pytest.mark.parametrize("af", [0.0, 0.25, 0.5])
@pytest.mark.parametrize("module", ["TwoDNavierStokes", "SingleLayerQG", "MultiLayerQG", "BarotropicQGQL"])
def test_aliased_fractions(module, af):
    """calcN! and 10 RK4 steps with dealiasing fractions other than 1/3 (0: no dealiasing)"""
    p, r = pair(module, nx=64, aliased_fraction=af, dt=0.002, stepper="RK4")
    sol = random_state(p, 3)
    N, _ = p.calcN(sol, 0.0)
    Nr = np.zeros_like(sol)
    r.calcN(Nr, sol.copy(), 0.0)
    assert rel(N, Nr) <= 1e-12
    p.sol = 0.01 * sol
    r.sol[...] = 0.01 * sol
    stepforward(p, 10)
    r.stepforward(10)
    assert rel(p.sol, r.sol) <= 1e-11


@pytest.mark.parametrize("nx,ny", [(128, 32), (32, 256), (256, 64)])
@pytest.mark.parametrize("module", ["TwoDNavierStokes", "SurfaceQG", "SingleLayerQG", "MultiLayerQG", "BarotropicQGQL"])
def test_rectangular_grids(module, nx, ny):
    """calcN! and ETDRK4 steps on nx != ny, Lx != Ly"""
    p, r = pair(module, nx=nx, ny=ny, Lx=2 * np.pi, Ly=2 * np.pi * ny / nx * 1.3, dt=0.002, stepper="ETDRK4")
    sol = random_state(p, 5)
    N, _ = p.calcN(sol, 0.0)
    Nr = np.zeros_like(sol)
    r.calcN(Nr, sol.copy(), 0.0)
    assert rel(N, Nr) <= 1e-12
    p.sol = 0.01 * sol
    r.sol[...] = 0.01 * sol
    stepforward(p, 6)
    r.stepforward(6)
    assert rel(p.sol, r.sol) <= 1e-11


@pytest.mark.parametrize("n", [32, 2048])
def test_smallest_and_largest_sizes(n):
    """one FilteredRK4 step at 32^2 and 2048^2 (FP64) against the oracle"""
    r = O.TwoDNavierStokes(nx=n, dt=1e-3, stepper="FilteredRK4")
    z = O.peakedisotropicspectrum(r.grid, 6 if n > 32 else 3, 0.5, mask=r.timestepper.filter, seed=9)
    r.set_zeta(z)
    p = TD.Problem("GPU", nx=n, dt=1e-3, stepper="FilteredRK4")
    TD.set_zeta(p, z)
    r.stepforward(2)
    stepforward(p, 2)
    assert rel(p.sol, r.sol) <= 1e-12


def test_filter_parameters_are_used():
    """filter_order / innerK / outerK of gf_config reach the Filtered steppers' filter"""
    from gfcuda import _abi as A
    import ctypes as C
    n = 64
    g = O.Grid(n)
    lib = A.load()
    cfg = A.gf_config()
    cfg.module, cfg.precision, cfg.stepper = 0, A.F64, A.STEPPERS["FilteredRK4"]
    cfg.nx = cfg.ny = n
    cfg.nlayers = 1
    cfg.Lx = cfg.Ly = 2 * np.pi
    cfg.dt, cfg.aliased_fraction = 0.01, 1 / 3
    cfg.filter_order, cfg.filter_innerK, cfg.filter_outerK = 6.0, 0.5, 0.9
    ctx = C.c_void_p()
    A.check(lib, None, lib.gf_create(C.byref(cfg), None, C.byref(ctx)))
    try:
        f = np.empty((n, n // 2 + 1))
        A.check(lib, ctx, lib.gf_get_filter(ctx, f.ctypes.data))
        assert np.max(np.abs(f - O.makefilter(g, order=6.0, innerK=0.5, outerK=0.9))) <= 1e-14
    finally:
        lib.gf_destroy(ctx)


@pytest.mark.parametrize("T", [np.float32, np.float64])
@pytest.mark.parametrize("kind", ["TwoDNavierStokes", "SingleLayerQG", "SurfaceQG", "BarotropicQGQL", "MLQG1", "MLQG2"])
def test_problemtype(kind, T):
    """test_*_problemtype (test/test_twodnavierstokes.jl:319-325, test_singlelayerqg.jl,
    test_surfaceqg.jl, test_barotropicqgql.jl, test_multilayerqg.jl:790-801; runtests.jl runs them
    with Float32): the state is complex of the problem's real type, the grid points and the
    physical fields real of it; MultiLayerQG arrays keep a layer axis for one layer as well"""
    CT = np.complex64 if T == np.float32 else np.complex128
    mod = {"TwoDNavierStokes": TD, "SingleLayerQG": SL, "SurfaceQG": SQ}.get(kind)
    if mod is not None:
        p = mod.Problem("GPU", nx=32, T=T)
    elif kind == "BarotropicQGQL":
        p = QL.Problem("GPU", nx=32, T=T)
    else:
        p = ML.Problem(int(kind[-1]), "GPU", nx=32, T=T)
    try:
        assert p.sol.dtype == CT
        assert p.grid.x.dtype == T and p.grid.y.dtype == T
        p.updatevars()
        assert p.vars.u.dtype == T
        nd = 3 if kind.startswith("MLQG") else 2
        assert p.sol.ndim == nd and p.vars.u.ndim == nd
    finally:
        p.close()


def test_mlqg_params_constructor_U_floats_or_vectors():
    """test/test_multilayerqg.jl:760-788: U given per layer as floats or as (ny, nlayers) vectors
    defines the same problem -- the same mean flow and, on the GPU, the same calcN!"""
    nx, ny, L = 32, 34, 2 * np.pi
    kw = dict(nx=nx, ny=ny, Lx=L, f0=1.0, H=[0.2, 0.8], b=[-1.0, -1.2])
    Uvec = np.zeros((ny, 2))
    Uvec[:, 0], Uvec[:, 1] = 0.1, 0.05
    pv = ML.Problem(2, "GPU", U=Uvec, **kw)
    pf = ML.Problem(2, "GPU", U=np.array([0.1, 0.05]), **kw)
    try:
        np.testing.assert_array_equal(pv.Uy, pf.Uy)
        rng = np.random.default_rng(4)
        sol = np.stack([np.fft.rfft2(0.1 * rng.standard_normal((ny, nx))) for _ in range(2)])
        np.testing.assert_array_equal(pv.calcN(sol, 0.0)[0], pf.calcN(sol, 0.0)[0])
    finally:
        pv.close()
        pf.close()


@pytest.mark.parametrize("n", [16, 32])
@pytest.mark.parametrize("precision", [None, "DF64"])
def test_sqg_noforcing(n, precision):
    """test/test_surfaceqg.jl:127-145 (n = 16): calcN! of a zero state is the forcing alone --
    zero without forcing, and the static forcing 2 at every mode (aliased ones included) with
    it; at the reference's 16 points (generic-length kernels) and at 32 (compiled-in)"""
    from gfcuda import Forcing
    pu = SQ.Problem("GPU", nx=n, stepper="ForwardEuler", precision=precision)
    shape = pu.spec_shape
    pf = SQ.Problem("GPU", nx=n, stepper="ForwardEuler", precision=precision,
                    forcing=Forcing("static", Fh=2 * np.ones(shape, dtype=np.complex128)))
    try:
        zero = np.zeros(shape, dtype=np.complex128)
        np.testing.assert_array_equal(pu.calcN(zero, 0.0)[0], np.zeros(shape))
        np.testing.assert_array_equal(pf.calcN(zero, 0.0)[0], 2 * np.ones(shape))
    finally:
        pu.close()
        pf.close()
