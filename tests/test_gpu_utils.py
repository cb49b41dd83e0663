"""peakedisotropicspectrum (src/utils.jl:29-54) on the device against the oracle, and the
Filtered steppers' filter read back through prob.timestepper.filter."""
import numpy as np
import pytest

import gf_oracle as O

pytestmark = pytest.mark.gpu

gfcuda = pytest.importorskip("gfcuda")
from gfcuda import TwoDNavierStokes as TD, peakedisotropicspectrum  # noqa: E402


@pytest.mark.parametrize("T,prec,tol", [(np.float64, None, 1e-13), (np.float64, "DF64", 1e-12),
                                        (np.float32, None, 2e-6)])
def test_peakedisotropicspectrum_matches_oracle(T, prec, tol):
    n = 128
    p = TD.Problem("GPU", nx=n, dt=0.005, stepper="FilteredRK4", T=T, precision=prec)
    g = O.Grid(n)
    filt = O.makefilter(g)
    assert np.max(np.abs(p.timestepper.filter - filt)) <= 1e-14
    z = peakedisotropicspectrum(p.grid, 6, 0.5, mask=p.timestepper.filter, seed=1234)
    zr = O.peakedisotropicspectrum(g, 6, 0.5, mask=filt, seed=1234)
    assert z.shape == (n, n) and z.dtype == T
    assert O.rel_l2(z, zr) <= tol
    # set_zeta! with it gives the requested energy (normalised over the half spectrum, :50)
    zo = peakedisotropicspectrum(p.grid, 3, 2.0, allones=True)
    assert O.rel_l2(zo, O.peakedisotropicspectrum(g, 3, 2.0, allones=True)) <= tol


def test_peakedisotropicspectrum_rectangle_and_batch():
    n, B = 64, 3
    p = TD.Problem("GPU", nx=n, batch=B)
    z = peakedisotropicspectrum(p.grid, 4, 0.5, seed=77)
    assert z.shape == (B, n, n)
    for i in range(B):
        assert O.rel_l2(z[i], O.peakedisotropicspectrum(O.Grid(n), 4, 0.5, seed=77 + i)) <= 1e-13
    q = TD.Problem("GPU", nx=n, ny=2 * n, Ly=4 * np.pi)
    with pytest.raises(ValueError, match="not square"):   # src/utils.jl:30 raises too
        peakedisotropicspectrum(q.grid, 4, 0.5)
    r = TD.Problem("GPU", nx=n, stepper="RK4")
    with pytest.raises(AttributeError):
        r.timestepper.filter


def test_streamed_diagnostics_match_per_step_values():
    """stepforward!(prob, diags, n): the diagnostics reduced on the device after every step
    into a ring buffer equal the values read one step at a time, and follow the oracle."""
    n, ns = 128, 25
    z0 = O.peakedisotropicspectrum(O.Grid(n), 6, 0.5, seed=3)
    kw = dict(nx=n, dt=0.005, nu=1e-3, nnu=1, stepper="FilteredRK4")
    p = TD.Problem("GPU", **kw)
    TD.set_zeta(p, z0)
    E, Z = gfcuda.Diagnostic(TD.energy, p), gfcuda.Diagnostic(TD.enstrophy, p)
    gfcuda.stepforward(p, [E, Z], ns)
    q = TD.Problem("GPU", **kw)
    TD.set_zeta(q, z0)
    r = O.TwoDNavierStokes(nx=n, dt=0.005, nu=1e-3, nnu=1, stepper="FilteredRK4")
    r.set_zeta(z0)
    for k in range(1, ns + 1):
        gfcuda.stepforward(q, 1)
        r.stepforward(1)
        assert E[k] == TD.energy(q) and Z[k] == TD.enstrophy(q)
        assert abs(E[k] - r.energy()) <= 1e-12 * r.energy()
    assert E.steps[-1] == ns and E.t[-1] == q.clock.t == p.clock.t
    assert np.array_equal(p.sol, q.sol)


@pytest.mark.parametrize("stepper", ["RK4", "ETDRK4", "AB3"])
def test_host_calcF_callback_matches_device_harmonic_forcing(stepper):
    """an arbitrary host calcF! called per stage (gf_step_callback) gives the same steps as the
    device's harmonic forcing kind F cos(omega t + phase) evaluated at the stage times"""
    n, dt = 64, 0.01
    g = O.Grid(n)
    x, y = g.gridpoints()
    Fh0 = O.rfft2(0.1 * np.cos(4 * x) * np.cos(5 * y))
    kw = dict(nx=n, dt=dt, nu=1e-3, nnu=1, stepper=stepper)
    times = []

    def calcF(Fh, sol, t, clock, vars, params, grid):
        times.append(t)
        Fh[...] = Fh0 * np.cos(2.0 * t + 0.3)

    p = TD.Problem("GPU", forcing=gfcuda.Forcing("callback", calcF=calcF), **kw)
    q = TD.Problem("GPU", forcing=gfcuda.Forcing("harmonic", Fh=Fh0, omega=2.0, phase=0.3), **kw)
    z = O.peakedisotropicspectrum(g, 4, 0.5, seed=4)
    TD.set_zeta(p, z)
    TD.set_zeta(q, z)
    gfcuda.stepforward(p, 7)
    gfcuda.stepforward(q, 7)
    assert O.rel_l2(p.sol, q.sol) <= 1e-14
    nst = 1 if stepper == "AB3" else 4
    assert len(times) == 7 * nst and abs(times[1 if nst == 4 else 0] - (0.5 * dt if nst == 4 else 0.0)) < 1e-15

    def bad(Fh, *a):
        raise RuntimeError("boom")
    r = TD.Problem("GPU", forcing=gfcuda.Forcing("callback", calcF=bad), **kw)
    with pytest.raises(RuntimeError, match="boom"):
        gfcuda.stepforward(r, 1)


@pytest.mark.parametrize("prec", [None, "DF64"])
def test_output_streaming_matches_stepwise_reads(prec):
    """gf_step_output: fields and diagnostics every `every` steps equal those read after
    stepping by hand; trailing steps are stepped too"""
    n = 64
    z0 = O.peakedisotropicspectrum(O.Grid(n), 6, 0.5, seed=5)
    kw = dict(nx=n, dt=0.005, stepper="FilteredRK4", precision=prec)
    p, q = TD.Problem("GPU", **kw), TD.Problem("GPU", **kw)
    TD.set_zeta(p, z0)
    TD.set_zeta(q, z0)
    d, f = gfcuda.stepforward_output(p, 23, 5, diagnostics=[TD.energy, TD.enstrophy], fields=["zeta", "u"])
    assert d.shape == (4, 2) and f["zeta"].shape == (4, n, n)
    for k in range(4):
        gfcuda.stepforward(q, 5)
        assert d[k, 0] == TD.energy(q) and d[k, 1] == TD.enstrophy(q)   # before updatevars! dealiases
        TD.updatevars(q)
        assert np.array_equal(f["zeta"][k], q.vars.zeta) and np.array_equal(f["u"][k], q.vars.u)
    gfcuda.stepforward(q, 3)
    assert p.clock.step == q.clock.step == 23 and np.array_equal(p.sol, q.sol)
