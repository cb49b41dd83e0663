"""GeophysicalFlows utilities (src/utils.jl) on libgfcuda.

peakedisotropicspectrum runs on the device (gf_peakedisotropicspectrum); ring_forcing_spectrum
is the host-side set-up the reference's forced examples build before they make a Problem
(examples/singlelayerqg_betaforced.jl:61-73, examples/twodnavierstokes_stochasticforcing.jl),
handed to the library through Forcing("stochastic", spectrum=...).
"""
import numpy as np

from . import _abi as A


def _problem_of(grid_or_prob):
    p = getattr(grid_or_prob, "_ctx", None) and grid_or_prob
    if p is None:
        ref = getattr(grid_or_prob, "_prob", None)
        p = ref() if ref is not None else None
    if p is None or not p._ctx:
        raise ValueError("pass the grid of a live Problem (prob.grid) or the Problem itself")
    return p


def peakedisotropicspectrum(grid, kpeak, E0, mask=None, allones=False, seed=1234):
    """peakedisotropicspectrum(grid, kpeak, E0; mask, allones) (src/utils.jl:29-54): a random
    isotropic vorticity field whose streamfunction spectrum peaks at kpeak (in units of
    2 pi / Lx), with energy E0.  Computed on the device; the random coefficients are Philox
    draws from `seed` (instance i of a batched Problem uses seed + i).  Returns the physical
    field, shape (ny, nx) or (batch, ny, nx), in the Problem's real type."""
    p = _problem_of(grid)
    g = p.grid
    m = None
    if mask is not None:
        m = np.ascontiguousarray(np.broadcast_to(mask, (g.ny, g.nkr)), dtype=np.float64)
    out = np.empty(p.phys_shape, dtype=p.T)
    p._c(p._lib.gf_peakedisotropicspectrum(p._ctx, float(kpeak), float(E0), None if m is None else m.ctypes.data,
                                           int(bool(allones)), int(seed) & 0xFFFFFFFFFFFFFFFF, out.ctypes.data,
                                           A.HOST))
    return out


def lambdipole(U, R, grid, center=None):
    """lambdipole(U, R, grid; center) (src/utils.jl:8-20): the vorticity of a Lamb dipole that
    moves along x at speed U, radius R, centred by default at the means of the grid's x and y
    coordinates.  Host-side set-up (SciPy's Bessel functions): J1(k r) (y - yc) / r scaled by
    -2 U k / J0(k R) inside r < R, k R the first zero of J1, zero outside.  Shape (ny, nx)."""
    from scipy.special import j0, j1
    kR = 3.8317059702075123156  # first zero of J1
    k = kR / R
    amp = -2.0 * U * k / j0(kR)
    xs, ys = np.asarray(grid.x, dtype=np.float64), np.asarray(grid.y, dtype=np.float64)
    xc, yc = (xs.mean(), ys.mean()) if center is None else center
    X, Y = np.meshgrid(xs, ys, indexing="xy")
    r = np.hypot(X - xc, Y - yc)
    inside = r < R
    out = np.zeros_like(r)
    out[inside] = amp * j1(k * r[inside]) * (Y[inside] - yc) / r[inside]
    return out


def parsevalsum(fh, grid):
    """FourierFlows.parsevalsum of a real field's half spectrum fh (ny, nkr): the sum over the
    full spectrum (interior kr columns counted twice, kr = 0 and, for even nx, the Nyquist
    column once) times Lx Ly / (nx ny)^2, real part."""
    w = np.full(grid.nkr, 2.0)
    w[0] = 1.0
    if grid.nx % 2 == 0:
        w[-1] = 1.0
    return grid.Lx * grid.Ly / (grid.nx * grid.ny) ** 2 * float(np.real(np.sum(np.asarray(fh) * w)))


def ring_forcing_spectrum(grid, kf, dkf, eps):
    """Isotropic Gaussian ring forcing spectrum exp(-(|k| - kf)^2 / (2 dkf^2)) (zero at k = 0),
    normalised so that white-in-time forcing with this spectrum injects energy at rate eps:
    eps0 = parsevalsum(spectrum / (2 K^2)) / (Lx Ly) (examples/singlelayerqg_betaforced.jl:61-73).
    kf, dkf in the grid's wavenumber units (radians per unit length)."""
    K = np.sqrt(grid.Krsq)
    spec = np.exp(-(K - kf) ** 2 / (2 * dkf ** 2))
    spec[grid.Krsq == 0] = 0.0
    eps0 = parsevalsum(spec * grid.invKrsq / 2, grid) / (grid.Lx * grid.Ly)
    return spec * (eps / eps0)


def random_topography(grid, kmax, amp, seed):
    """A random topographic PV field: Fourier modes 0 < |k| <= kmax (in units of 2 pi / Lx)
    with complex-normal coefficients from numpy's seeded generator, scaled so that the
    field's maximum |eta| is amp; shape (ny, nx)."""
    rng = np.random.default_rng(seed)
    K = np.sqrt(grid.Krsq) * grid.Lx / (2 * np.pi)
    z = rng.standard_normal(grid.Krsq.shape) + 1j * rng.standard_normal(grid.Krsq.shape)
    eh = np.where((K <= kmax) & (grid.Krsq > 0), z, 0)
    eta = np.fft.irfft2(eh, s=(grid.ny, grid.nx))
    return amp * eta / np.max(np.abs(eta))


def radialspectrum(fh, grid, n=None, m=None, refinement=2):
    """Azimuthal integral of a half-spectrum array fh (ny, nx/2+1) in the manner of
    FourierFlows.radialspectrum (called at test/test_utils.jl:9 and in the decaying-turbulence
    example): fh is extended to the full (Hermitian) plane and centred, interpolated
    bilinearly on a polar grid of n radii in [0, min(max|k|, max|l|)] and m angles in
    [-pi, pi), and integrated, F(rho) = rho * sum_theta f(rho, theta) dtheta.  n and m default
    to refinement * max(nx, ny).  Returns (rho, F).  A host-side post-processing helper."""
    fh = np.asarray(fh)
    nx, ny = grid.nx, grid.ny
    n = refinement * max(nx, ny) if n is None else int(n)
    m = refinement * max(nx, ny) if m is None else int(m)
    full = np.zeros((ny, nx), dtype=np.result_type(fh, np.complex128))
    full[:, : grid.nkr] = fh
    jj = (-np.arange(ny)) % ny
    for i in range(1, nx - grid.nkr + 1):      # negative kx from the Hermitian symmetry
        full[:, nx - i] = np.conj(fh[jj, i])
    fs = np.fft.fftshift(full)
    dk, dl = 2 * np.pi / grid.Lx, 2 * np.pi / grid.Ly
    kmax, lmax = dk * (nx // 2 - 1), dl * (ny // 2 - 1)
    rho = np.linspace(0.0, min(kmax, lmax), n)
    theta = -np.pi + 2 * np.pi * np.arange(m) / m
    kx = rho[:, None] * np.cos(theta)[None, :]
    ly = rho[:, None] * np.sin(theta)[None, :]
    # fractional indices into the centred array (index nx//2 is k = 0)
    fx, fy = kx / dk + nx // 2, ly / dl + ny // 2
    x0, y0 = np.floor(fx).astype(int), np.floor(fy).astype(int)
    ax, ay = fx - x0, fy - y0
    x1, y1 = np.minimum(x0 + 1, nx - 1), np.minimum(y0 + 1, ny - 1)
    f = ((1 - ax) * (1 - ay) * fs[y0, x0] + ax * (1 - ay) * fs[y0, x1]
         + (1 - ax) * ay * fs[y1, x0] + ax * ay * fs[y1, x1])
    F = rho * f.sum(axis=1) * (2 * np.pi / m)
    return rho, F
