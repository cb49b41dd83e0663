"""FP64 CPU oracle for the pseudospectral time step -- TEST INFRASTRUCTURE ONLY.

This module restates, in NumPy float64, the algorithm of GeophysicalFlows.jl v0.16.5
(TwoDNavierStokes, SingleLayerQG, MultiLayerQG, SurfaceQG) together with the pieces of
its un-vendored dependency FourierFlows.jl 0.10.5 (``Project.toml:25``) that the step
uses: ``TwoDGrid``, ``dealias!``, ``makefilter``, ``parsevalsum[2]`` and the
ForwardEuler / AB3 / RK4 / ETDRK4 timesteppers and their ``Filtered*`` variants.
FourierFlows' own source is not in the reference tree, so those pieces follow its
published algorithm (Kassam & Trefethen 2005 contour integrals for ETDRK4, the
exponential filter ``exp(-decay (K - innerK)^order)``); the details no reference test is
sensitive to (exact filter shape, exact dealias index boundaries, ETDRK4 contour
count/radius) are fixed here and used identically by the CUDA path.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may
import this file.  The CUDA library never calls it; it is the checker.

Parity pins: ``tests/test_oracle_reference.py`` runs this oracle through the reference's
own known-answer tests (analytic energies/enstrophies, manufactured steady solutions at
rtol 1e-13, Rossby-wave evolution for all 8 steppers, PV inversion, MLQG fluxes) and they
pass, which pins calcN!, the steppers and the diagnostics.

Array layout: NumPy C-order arrays of shape ``(ny, nx)`` (physical) and ``(ny, nkr)``
(spectral), and ``(nlayers, ny, ·)`` for layered fields, which is the same memory order as
the reference's column-major ``(nx, ny[, nlayers])`` Julia arrays.
"""
from __future__ import annotations

import math
import numpy as np

# ---------------------------------------------------------------------------------------
# Philox4x32-10 counter-based RNG (Salmon, Moraes, Dror & Shaw, SC'11).  The reference
# draws with Julia's `randn!` (examples/singlelayerqg_betaforced.jl:86-90) whose stream
# cannot be reproduced without Julia; the oracle and the CUDA kernels share this one.
# ---------------------------------------------------------------------------------------
_M32 = np.uint64(0xFFFFFFFF)
_PM0 = np.uint64(0xD2511F53)
_PM1 = np.uint64(0xCD9E8D57)
_PW0 = np.uint64(0x9E3779B9)
_PW1 = np.uint64(0xBB67AE85)

TAG_FORCING = 0x464F5243   # counter word 3 for forcing draws
TAG_INITIAL = 0x494E4954   # counter word 3 for initial-condition draws


def philox4x32_10(c0, c1, c2, c3, k0, k1):
    """Vectorised Philox4x32 with 10 rounds; all inputs are uint32-valued arrays/ints."""
    c0 = np.asarray(c0, dtype=np.uint64) & _M32
    c1 = np.asarray(c1, dtype=np.uint64) & _M32
    c2 = np.asarray(c2, dtype=np.uint64) & _M32
    c3 = np.asarray(c3, dtype=np.uint64) & _M32
    k0 = np.uint64(int(k0) & 0xFFFFFFFF)
    k1 = np.uint64(int(k1) & 0xFFFFFFFF)
    for r in range(10):
        if r > 0:
            k0 = (k0 + _PW0) & _M32
            k1 = (k1 + _PW1) & _M32
        p0 = _PM0 * c0
        p1 = _PM1 * c2
        hi0, lo0 = p0 >> np.uint64(32), p0 & _M32
        hi1, lo1 = p1 >> np.uint64(32), p1 & _M32
        c0, c1, c2, c3 = (hi1 ^ c1 ^ k0), lo1, (hi0 ^ c3 ^ k1), lo0
    return c0, c1, c2, c3


def _u01(x):
    """uint32 -> float64 uniform in (0, 1): (x + 1/2) / 2^32."""
    return (x.astype(np.float64) + 0.5) * (1.0 / 4294967296.0)


def complex_normal(n, seed, step, tag=TAG_FORCING):
    """n complex normals with E|z|^2 = 1 (real and imaginary parts of variance 1/2).

    Element e uses counter (e, step_lo, step_hi, tag), key (seed_lo, seed_hi) and one
    Box-Muller pair from the first two output words.
    """
    e = np.arange(n, dtype=np.uint64)
    step = int(step)
    x0, x1, _, _ = philox4x32_10(e, step & 0xFFFFFFFF, (step >> 32) & 0xFFFFFFFF, tag,
                                 int(seed) & 0xFFFFFFFF, (int(seed) >> 32) & 0xFFFFFFFF)
    u0, u1 = _u01(x0), _u01(x1)
    r = np.sqrt(-2.0 * np.log(u0))
    th = 2.0 * np.pi * u1
    return (r * np.cos(th) + 1j * r * np.sin(th)) * math.sqrt(0.5)


def random_phase(n, seed, step, tag=TAG_FORCING):
    """n unit-modulus complex numbers exp(2 pi i u), u uniform (reference budget tests'
    `exp.(2π * im * rand(...))`, test/test_twodnavierstokes.jl:42)."""
    e = np.arange(n, dtype=np.uint64)
    step = int(step)
    x0, _, _, _ = philox4x32_10(e, step & 0xFFFFFFFF, (step >> 32) & 0xFFFFFFFF, tag,
                                int(seed) & 0xFFFFFFFF, (int(seed) >> 32) & 0xFFFFFFFF)
    return np.exp(2j * np.pi * _u01(x0))


# ---------------------------------------------------------------------------------------
# FourierFlows TwoDGrid (called at src/twodnavierstokes.jl:91; x in [-Lx/2, Lx/2),
# docs/src/aliasing.md:16-23)
# ---------------------------------------------------------------------------------------
def aliased_indices(nk, nkr, aliased_fraction):
    """0-based index ranges zeroed by FourierFlows' dealias! along one dimension.

    The upper `aliased_fraction` of |k| is removed: with L=(1-f)/2, R=(1+f)/2 the 1-based
    full-spectrum range is floor(L nk)+1 : ceil(R nk) and the half-spectrum range runs from
    the same start to nkr.
    """
    if aliased_fraction <= 0:
        return np.zeros(0, dtype=np.int64), np.zeros(0, dtype=np.int64)
    if aliased_fraction >= 1:
        raise ValueError("`aliased_fraction` must be less than 1")
    L = (1 - aliased_fraction) / 2
    R = (1 + aliased_fraction) / 2
    iL = math.floor(L * nk) + 1
    iR = math.ceil(R * nk)
    return np.arange(iL - 1, iR, dtype=np.int64), np.arange(iL - 1, nkr, dtype=np.int64)


class Grid:
    """Restatement of FourierFlows.TwoDGrid (periodic, Lx x Ly, nx x ny)."""

    def __init__(self, nx, Lx=2 * np.pi, ny=None, Ly=None, aliased_fraction=1 / 3):
        ny = nx if ny is None else ny
        Ly = Lx if Ly is None else Ly
        self.nx, self.ny, self.Lx, self.Ly = int(nx), int(ny), float(Lx), float(Ly)
        self.nkr, self.nl, self.nk = nx // 2 + 1, ny, nx
        self.dx, self.dy = Lx / nx, Ly / ny
        self.x = -Lx / 2 + self.dx * np.arange(nx)
        self.y = -Ly / 2 + self.dy * np.arange(ny)
        self.kr = (2 * np.pi / Lx) * np.arange(self.nkr, dtype=np.float64)[None, :]
        self.l = (2 * np.pi / Ly) * (np.fft.fftfreq(ny) * ny)[:, None]
        self.k = (2 * np.pi / Lx) * (np.fft.fftfreq(nx) * nx)[None, :]
        self.Krsq = self.kr ** 2 + self.l ** 2
        with np.errstate(divide="ignore"):
            self.invKrsq = np.where(self.Krsq == 0, 0.0, 1.0 / np.where(self.Krsq == 0, 1, self.Krsq))
        self.aliased_fraction = aliased_fraction
        _, self.kralias = aliased_indices(self.nk, self.nkr, aliased_fraction)
        self.lalias, _ = aliased_indices(self.nl, self.nl // 2 + 1, aliased_fraction)

    def gridpoints(self):
        """X, Y of shape (ny, nx): X[j, i] = x[i], Y[j, i] = y[j]."""
        return np.meshgrid(self.x, self.y, indexing="xy")

    def dealias_mask(self):
        m = np.ones((self.ny, self.nkr))
        m[:, self.kralias] = 0
        m[self.lalias, :] = 0
        return m


_FFT_WORKERS = None  # None: numpy.fft (single thread); n: scipy.fft with n worker threads


def set_fft_workers(n):
    """Use scipy.fft with n threads (the CPU-baseline timing uses all host cores, like the
    reference's FFTW.set_num_threads, README.md:79-86); None restores numpy.fft."""
    global _FFT_WORKERS
    _FFT_WORKERS = n


def rfft2(f):
    """Unnormalised r2c along x then c2c along y (FFTW `mul!(fh, rfftplan, f)`)."""
    if _FFT_WORKERS:
        import scipy.fft as sf
        return sf.rfft2(f, axes=(-2, -1), workers=_FFT_WORKERS)
    return np.fft.rfft2(f, axes=(-2, -1))


def irfft2(fh, grid):
    """Normalised c2r (FFTW `ldiv!(f, rfftplan, fh)`), y-pass first, then x c2r."""
    if _FFT_WORKERS:
        import scipy.fft as sf
        return sf.irfft2(fh, s=(grid.ny, grid.nx), axes=(-2, -1), workers=_FFT_WORKERS)
    return np.fft.irfft2(fh, s=(grid.ny, grid.nx), axes=(-2, -1))


def dealias(fh, grid):
    """In-place FourierFlows dealias!: zero the aliased kr columns and l rows."""
    fh[..., :, grid.kralias] = 0
    fh[..., grid.lalias, :] = 0


def makefilter(grid, order=4, innerK=0.65, outerK=1.0):
    """FourierFlows exponential spectral filter on the half spectrum.

    K = sqrt((kr dx/pi)^2 + (l dy/pi)^2) (1 at the Nyquist wavenumber);
    filter = exp(-decay (K - innerK)^order) for K >= innerK, 1 below, with
    decay = 15 ln(10) / (outerK - innerK)^order.
    """
    K = np.sqrt((grid.kr * grid.dx / np.pi) ** 2 + (grid.l * grid.dy / np.pi) ** 2)
    decay = 15 * math.log(10) / (outerK - innerK) ** order
    filt = np.exp(-decay * (K - innerK) ** order)
    filt[K < innerK] = 1.0
    return filt


def parsevalsum(uh, grid):
    """FourierFlows parsevalsum on a half-spectrum array (last axis kr).

    Interior kr columns count twice; kr=0 and (even nx) the Nyquist column once.
    Normalisation Lx Ly / (nx ny)^2; the real part is returned.
    """
    w = np.full(grid.nkr, 2.0)
    w[0] = 1.0
    if grid.nx % 2 == 0:
        w[-1] = 1.0
    norm = grid.Lx * grid.Ly / (grid.nx ** 2 * grid.ny ** 2)
    return norm * float(np.real(np.sum(uh * w)))


def parsevalsum2(uh, grid):
    return parsevalsum(np.abs(uh) ** 2, grid)


def jacobian(a, b, grid):
    """FourierFlows.jacobian: a_x b_y - a_y b_x computed spectrally."""
    ah, bh = rfft2(a), rfft2(b)
    ax, ay = irfft2(1j * grid.kr * ah, grid), irfft2(1j * grid.l * ah, grid)
    bx, by = irfft2(1j * grid.kr * bh, grid), irfft2(1j * grid.l * bh, grid)
    return ax * by - ay * bx


# ---------------------------------------------------------------------------------------
# Timesteppers (FourierFlows 0.10.5; names listed at test/runtests.jl:58)
# ---------------------------------------------------------------------------------------
def etdrk4_coefficients(L, dt, ncirc=32, rcirc=1.0):
    """Kassam & Trefethen (2005) contour-integral ETDRK4 coefficients (zeta, alpha, beta,
    Gamma) plus exp(L dt) and exp(L dt / 2).  Real parts are taken when L is real."""
    L = np.asarray(L)
    circ = rcirc * np.exp(2j * np.pi / ncirc * (np.arange(ncirc) + 0.5))
    zc = dt * L[..., None] + circ
    ez, ez2 = np.exp(zc), np.exp(zc / 2)
    zeta = dt * np.mean((ez2 - 1) / zc, axis=-1)
    alpha = dt * np.mean((-4 - zc + ez * (4 - 3 * zc + zc ** 2)) / zc ** 3, axis=-1)
    beta = dt * np.mean((2 + zc + ez * (-2 + zc)) / zc ** 3, axis=-1)
    gamma = dt * np.mean((-4 - 3 * zc - zc ** 2 + ez * (4 - zc)) / zc ** 3, axis=-1)
    if not np.iscomplexobj(L):
        zeta, alpha, beta, gamma = (np.real(a) for a in (zeta, alpha, beta, gamma))
    return zeta, alpha, beta, gamma, np.exp(dt * L), np.exp(dt * L / 2)


STEPPERS = ("ForwardEuler", "FilteredForwardEuler", "RK4", "FilteredRK4",
            "ETDRK4", "FilteredETDRK4", "AB3", "FilteredAB3")


class TimeStepper:
    def __init__(self, name, prob):
        if name not in STEPPERS:
            raise ValueError(f"unknown stepper {name}")
        self.name = name
        self.filtered = name.startswith("Filtered")
        self.kind = name.replace("Filtered", "")
        shape = prob.sol.shape
        self.filter = np.broadcast_to(makefilter(prob.grid), shape).copy() if self.filtered else None
        z = lambda: np.zeros(shape, dtype=np.complex128)
        if self.kind == "ForwardEuler":
            self.N = z()
        elif self.kind == "RK4":
            self.sol1, self.RHS1, self.RHS2, self.RHS3, self.RHS4 = z(), z(), z(), z(), z()
        elif self.kind == "ETDRK4":
            (self.zeta, self.alpha, self.beta, self.gamma,
             self.expLdt, self.expLdt2) = etdrk4_coefficients(prob.L, prob.clock.dt)
            self.sol1, self.sol2, self.N1, self.N2, self.N3, self.N4 = z(), z(), z(), z(), z(), z()
        elif self.kind == "AB3":
            self.RHS, self.RHSm1, self.RHSm2 = z(), z(), z()

    def step(self, prob):
        sol, cl, L, N_ = prob.sol, prob.clock, prob.L, prob.calcN
        t, dt = cl.t, cl.dt
        if self.kind == "ForwardEuler":
            N_(self.N, sol, t)
            new = sol + dt * (self.N + L * sol)
        elif self.kind == "RK4":
            N_(self.RHS1, sol, t); self.RHS1 += L * sol
            self.sol1[...] = sol + dt / 2 * self.RHS1
            N_(self.RHS2, self.sol1, t + dt / 2); self.RHS2 += L * self.sol1
            self.sol1[...] = sol + dt / 2 * self.RHS2
            N_(self.RHS3, self.sol1, t + dt / 2); self.RHS3 += L * self.sol1
            self.sol1[...] = sol + dt * self.RHS3
            N_(self.RHS4, self.sol1, t + dt); self.RHS4 += L * self.sol1
            new = sol + dt * (self.RHS1 / 6 + self.RHS2 / 3 + self.RHS3 / 3 + self.RHS4 / 6)
        elif self.kind == "ETDRK4":
            e2, zt = self.expLdt2, self.zeta
            N_(self.N1, sol, t)
            self.sol1[...] = e2 * sol + zt * self.N1
            N_(self.N2, self.sol1, t + dt / 2)
            self.sol2[...] = e2 * sol + zt * self.N2
            N_(self.N3, self.sol2, t + dt / 2)
            self.sol2[...] = e2 * self.sol1 + zt * (2 * self.N3 - self.N1)
            N_(self.N4, self.sol2, t + dt)
            new = (self.expLdt * sol + self.alpha * self.N1
                   + 2 * self.beta * (self.N2 + self.N3) + self.gamma * self.N4)
        elif self.kind == "AB3":
            N_(self.RHS, sol, t); self.RHS += L * sol
            if cl.step < 3:
                new = sol + dt * self.RHS
            else:
                new = sol + dt * (23 / 12 * self.RHS - 16 / 12 * self.RHSm1 + 5 / 12 * self.RHSm2)
            self.RHSm2[...] = self.RHSm1
            self.RHSm1[...] = self.RHS
        if self.filtered:
            new = self.filter * new
        sol[...] = new
        cl.t += dt
        cl.step += 1


class Clock:
    def __init__(self, dt):
        self.dt, self.t, self.step = float(dt), 0.0, 0


# ---------------------------------------------------------------------------------------
# Forcing (the reference's `calcF!` callbacks, e.g. examples/singlelayerqg_betaforced.jl:86-90)
# ---------------------------------------------------------------------------------------
class Forcing:
    """kind: None | 'static' (Fh fixed) | 'harmonic' (Fh cos(omega t + phase)) |
    'stochastic' (randn * sqrt(spectrum/dt), drawn once per step) |
    'stochastic_phase' (exp(2 pi i u) * sqrt(spectrum/dt), [0,0] = 0)."""

    def __init__(self, kind=None, Fh=None, spectrum=None, omega=0.0, phase=0.0, seed=0):
        self.kind, self.Fh0, self.spectrum = kind, Fh, spectrum
        self.omega, self.phase, self.seed = omega, phase, seed

    @property
    def stochastic(self):
        return self.kind in ("stochastic", "stochastic_phase")

    def calcF(self, Fh, t, clock):
        if self.kind == "static":
            Fh[...] = self.Fh0
        elif self.kind == "harmonic":
            Fh[...] = self.Fh0 * math.cos(self.omega * t + self.phase)
        elif self.kind == "stochastic":
            z = complex_normal(Fh.size, self.seed, clock.step).reshape(Fh.shape)
            Fh[...] = z * np.sqrt(self.spectrum) / math.sqrt(clock.dt)
        elif self.kind == "stochastic_phase":
            z = random_phase(Fh.size, self.seed, clock.step).reshape(Fh.shape)
            z.reshape(-1, Fh.shape[-2] * Fh.shape[-1])[:, 0] = 0
            Fh[...] = z * np.sqrt(self.spectrum) / math.sqrt(clock.dt)


class Problem:
    """Mirror of FourierFlows.Problem: sol, clock, L, calcN!, vars, params, grid."""

    def __init__(self, grid, L, calcN, sol_shape, dt, stepper, forcing):
        self.grid, self.L, self._calcN = grid, L, calcN
        self.sol = np.zeros(sol_shape, dtype=np.complex128)
        self.clock = Clock(dt)
        self.forcing = forcing if forcing is not None else Forcing(None)
        self.Fh = np.zeros(sol_shape, dtype=np.complex128) if self.forcing.kind else None
        self.prevsol = np.zeros(sol_shape, dtype=np.complex128) if self.forcing.stochastic else None
        self.timestepper = TimeStepper(stepper, self)

    def calcN(self, N, sol, t):
        self._calcN(N, sol, t)
        self.addforcing(N, sol, t)

    def addforcing(self, N, sol, t):
        f = self.forcing
        if f.kind is None:
            return
        if f.stochastic:
            if t == self.clock.t:
                self.prevsol[...] = sol
                f.calcF(self.Fh, t, self.clock)
        else:
            f.calcF(self.Fh, t, self.clock)
        N += self.Fh

    def stepforward(self, nsteps=1):
        for _ in range(nsteps):
            self.timestepper.step(self)


def _powK(Krsq, n):
    """Krsq^n with Julia's conventions at Krsq = 0 (0^0 = 1, 0^-n = Inf); callers zero the
    k = 0 entry afterwards as the reference does."""
    with np.errstate(divide="ignore", invalid="ignore"):
        K = np.where(Krsq == 0, 1.0, Krsq) ** n
        return np.where(Krsq == 0, 0.0 if n > 0 else (1.0 if n == 0 else np.inf), K)


# ---------------------------------------------------------------------------------------
# TwoDNavierStokes (src/twodnavierstokes.jl)
# ---------------------------------------------------------------------------------------
class TwoDNavierStokes(Problem):
    """src/twodnavierstokes.jl:71-100 (Problem), :149-154 (Equation), :253-294 (calcN!)."""

    def __init__(self, nx=256, ny=None, Lx=2 * np.pi, Ly=None, nu=0.0, nnu=1, mu=0.0, nmu=0,
                 dt=0.01, stepper="RK4", forcing=None, aliased_fraction=1 / 3):
        g = Grid(nx, Lx, ny, Ly, aliased_fraction)
        self.nu, self.nnu, self.mu, self.nmu = nu, nnu, mu, nmu
        L = -nu * _powK(g.Krsq, nnu) - mu * _powK(g.Krsq, nmu)
        L[0, 0] = 0
        super().__init__(g, L, self._advection, (g.ny, g.nkr), dt, stepper, forcing)
        self.zeta = np.zeros((g.ny, g.nx)); self.u = np.zeros_like(self.zeta); self.v = np.zeros_like(self.zeta)

    def _advection(self, N, sol, t):
        g = self.grid
        dealias(sol, g)
        uh = 1j * g.l * g.invKrsq * sol
        vh = -1j * g.kr * g.invKrsq * sol
        u, v, z = irfft2(uh, g), irfft2(vh, g), irfft2(sol, g)
        N[...] = -1j * g.kr * rfft2(u * z) - 1j * g.l * rfft2(v * z)

    def updatevars(self):
        g, sol = self.grid, self.sol
        dealias(sol, g)
        self.zeta = irfft2(sol, g)
        self.u = irfft2(1j * g.l * g.invKrsq * sol, g)
        self.v = irfft2(-1j * g.kr * g.invKrsq * sol, g)

    def set_zeta(self, zeta):
        self.sol[...] = rfft2(zeta)
        self.sol[0, 0] = 0
        self.updatevars()

    # diagnostics (src/twodnavierstokes.jl:374-535)
    def _ps(self, a):
        g = self.grid
        return parsevalsum(a, g) / (g.Lx * g.Ly)

    def energy(self):
        return self._ps(0.5 * self.grid.invKrsq * np.abs(self.sol) ** 2)

    def enstrophy(self):
        return self._ps(np.abs(self.sol) ** 2) / 2

    def palinstrophy(self):
        return self._ps(0.5 * self.grid.Krsq * np.abs(self.sol) ** 2)

    def energy_dissipation(self, xi, nxi):
        with np.errstate(invalid="ignore"):
            a = -xi * _powK(self.grid.Krsq, nxi - 1) * np.abs(self.sol) ** 2
        a[0, 0] = 0
        return self._ps(a)

    def enstrophy_dissipation(self, xi, nxi):
        a = -xi * _powK(self.grid.Krsq, nxi) * np.abs(self.sol) ** 2
        a[0, 0] = 0
        return self._ps(a)

    def energy_dissipation_hyperviscosity(self):
        return self.energy_dissipation(self.nu, self.nnu)

    def energy_dissipation_hypoviscosity(self):
        return self.energy_dissipation(self.mu, self.nmu)

    def enstrophy_dissipation_hyperviscosity(self):
        return self.enstrophy_dissipation(self.nu, self.nnu)

    def enstrophy_dissipation_hypoviscosity(self):
        return self.enstrophy_dissipation(self.mu, self.nmu)

    def _worksol(self):
        return (self.prevsol + self.sol) / 2 if self.forcing.stochastic else self.sol

    def energy_work(self):
        return self._ps(self.grid.invKrsq * self._worksol() * np.conj(self.Fh))

    def enstrophy_work(self):
        return self._ps(self._worksol() * np.conj(self.Fh))


# ---------------------------------------------------------------------------------------
# SingleLayerQG (src/singlelayerqg.jl)
# ---------------------------------------------------------------------------------------
class BarotropicQGQL(Problem):
    """Quasi-linear barotropic QG: src/barotropicqgql.jl:75-110 (Problem), :168-173
    (Equation), :294-344 (calcN_advection!, calcN!), :380-431 (updatevars!, set_zeta!),
    :433-510 (diagnostics).  The state is split into the zonal mean (the kr = 0 column, Z)
    and the eddies (kr > 0, z): N = NZ + Nz with NZ the kr = 0 part of
    -i kr (u z)^ - i l (v z)^ and Nz the kr > 0 part of -i kr (U z + u Z)^ - i l (v Z)^, where
    u, v are the eddy velocities and U the mean zonal flow.  The topography is carried in
    the parameters but does not enter the advection (as in the reference)."""

    def __init__(self, nx=256, ny=None, Lx=2 * np.pi, Ly=None, beta=0.0, eta=None, nu=0.0, nnu=1, mu=0.0,
                 dt=0.01, stepper="RK4", forcing=None, aliased_fraction=1 / 3):
        g = Grid(nx, Lx, ny, Ly, aliased_fraction)
        self.beta, self.nu, self.nnu, self.mu = beta, nu, nnu, mu
        self.eta = np.zeros((g.ny, g.nx)) if eta is None else np.asarray(eta, dtype=np.float64)
        L = -mu - nu * _powK(g.Krsq, nnu) + 1j * beta * g.kr * g.invKrsq
        L = np.asarray(L, dtype=np.complex128)
        L[0, 0] = 0
        super().__init__(g, L, self._advection, (g.ny, g.nkr), dt, stepper, forcing)

    @staticmethod
    def _split(sol):
        eddy, mean = sol.copy(), sol.copy()
        eddy[..., :, 0] = 0
        mean[..., :, 1:] = 0
        return eddy, mean

    def _advection(self, N, sol, t):
        g = self.grid
        dealias(sol, g)
        zh, Zh = self._split(sol)
        u = irfft2(1j * g.l * g.invKrsq * zh, g)
        v = irfft2(-1j * g.kr * g.invKrsq * zh, g)
        U = irfft2(1j * g.l * g.invKrsq * Zh, g)
        z, Z = irfft2(zh, g), irfft2(Zh, g)
        NZ = -1j * g.kr * rfft2(u * z) - 1j * g.l * rfft2(v * z)
        NZ[:, 1:] = 0
        Nz = -1j * g.kr * rfft2(U * z + u * Z) - 1j * g.l * rfft2(v * Z)
        Nz[:, 0] = 0
        N[...] = NZ + Nz

    def updatevars(self):
        g, sol = self.grid, self.sol
        dealias(sol, g)
        sol[0, 0] = 0
        zh, Zh = self._split(sol)
        psih, Psih = -zh * g.invKrsq, -Zh * g.invKrsq
        self.zeta, self.Zeta = irfft2(zh, g), irfft2(Zh, g)
        self.psi, self.Psi = irfft2(psih, g), irfft2(Psih, g)
        self.u, self.v = irfft2(-1j * g.l * psih, g), irfft2(1j * g.kr * psih, g)
        self.U = irfft2(1j * g.l * Zh * g.invKrsq, g)

    def set_zeta(self, zeta):
        self.sol[...] = rfft2(zeta)
        self.sol[0, 0] = 0
        self.updatevars()

    def _ps(self, a):
        g = self.grid
        return parsevalsum(a, g) / (g.Lx * g.Ly)

    def energy(self):
        g = self.grid
        return 0.5 * (parsevalsum2(g.kr * g.invKrsq * self.sol, g) + parsevalsum2(g.l * g.invKrsq * self.sol, g)) / (g.Lx * g.Ly)

    def enstrophy(self):
        g = self.grid
        a = self.sol.copy()
        a[0, 0] = 0
        return 0.5 * parsevalsum2(a, g) / (g.Lx * g.Ly)

    def dissipation(self):
        with np.errstate(invalid="ignore", divide="ignore"):
            a = _powK(self.grid.Krsq, self.nnu - 1) * np.abs(self.sol) ** 2
        a[0, 0] = 0
        return self.nu * self._ps(a)

    def work(self):
        s = (self.prevsol + self.sol) / 2 if self.forcing.stochastic else self.sol
        return self._ps(self.grid.invKrsq * s * np.conj(self.Fh))

    def drag(self):
        a = self.grid.invKrsq * np.abs(self.sol) ** 2
        a[0, 0] = 0
        return self.mu * self._ps(a)


class SingleLayerQG(Problem):
    """src/singlelayerqg.jl:91-126 (Problem), :174-207 (Params), :230-252 (Equation),
    :356-432 (calcN_advection!), :484-490 (streamfunctionfrompv!)."""

    def __init__(self, nx=256, ny=None, Lx=2 * np.pi, Ly=None, beta=0.0, deformation_radius=np.inf,
                 U=0.0, eta=None, nu=0.0, nnu=1, mu=0.0, dt=0.01, stepper="RK4", forcing=None,
                 aliased_fraction=1 / 3):
        g = Grid(nx, Lx, ny, Ly, aliased_fraction)
        self.beta, self.mu, self.nu, self.nnu = beta, mu, nu, nnu
        self.ell = None if (deformation_radius is None or np.isinf(deformation_radius)) else float(deformation_radius)
        self.eta = np.zeros((g.ny, g.nx)) if eta is None else np.asarray(eta, dtype=np.float64)
        self.etah = rfft2(self.eta)
        self.Qx = irfft2(1j * g.kr * self.etah, g)
        self.Qy = irfft2(1j * g.l * self.etah, g)
        self.U_is_number = np.isscalar(U)
        if self.U_is_number:
            self.U = float(U)
        else:
            Uy = np.asarray(U, dtype=np.float64).reshape(g.ny)
            self.U = np.repeat(Uy[:, None], g.nx, axis=1)
            Uyy = irfft2(-g.l ** 2 * rfft2(self.U), g)
            self.Qy = self.Qy - Uyy
        if self.ell is None:
            L = -mu - nu * _powK(g.Krsq, nnu) + 1j * beta * g.kr * g.invKrsq
        else:
            L = -mu - nu * _powK(g.Krsq, nnu) + 1j * beta * g.kr / (g.Krsq + 1 / self.ell ** 2)
        if self.U_is_number:
            L = L - 1j * self.U * g.kr
        L = np.asarray(L, dtype=np.complex128)
        L[0, 0] = 0
        super().__init__(g, L, self._advection, (g.ny, g.nkr), dt, stepper, forcing)

    def streamfunctionfrompv(self, qh):
        g = self.grid
        if self.ell is None:
            return -g.invKrsq * qh
        return -qh / (g.Krsq + 1 / self.ell ** 2)

    def _advection(self, N, sol, t):
        g = self.grid
        dealias(sol, g)
        qh = sol.copy()
        psih = self.streamfunctionfrompv(qh)
        uh, vh = -1j * g.l * psih, 1j * g.kr * psih
        q, u, v = irfft2(qh, g), irfft2(uh, g), irfft2(vh, g)
        if self.U_is_number:
            qe = q + self.eta
            N[...] = -1j * g.kr * rfft2(u * qe) - 1j * g.l * rfft2(v * qe)
            N -= 1j * g.kr * self.U * self.etah
        else:
            u = u + self.U
            N[...] = -rfft2(u * self.Qx)
            N -= rfft2(v * self.Qy)
            N -= 1j * g.kr * rfft2(u * q) + 1j * g.l * rfft2(v * q)

    def updatevars(self):
        g, sol = self.grid, self.sol
        dealias(sol, g)
        psih = self.streamfunctionfrompv(sol)
        self.q, self.psi = irfft2(sol, g), irfft2(psih, g)
        self.u, self.v = irfft2(-1j * g.l * psih, g), irfft2(1j * g.kr * psih, g)

    def set_q(self, q):
        self.sol[...] = rfft2(q)
        self.updatevars()

    def _ps(self, a):
        g = self.grid
        return parsevalsum(a, g) / (g.Lx * g.Ly)

    def kinetic_energy(self):
        g = self.grid
        psih = self.streamfunctionfrompv(self.sol)
        return parsevalsum2(np.sqrt(g.Krsq) * psih, g) / (2 * g.Lx * g.Ly)

    def potential_energy(self):
        if self.ell is None:
            return 0.0
        g = self.grid
        return parsevalsum2(self.streamfunctionfrompv(self.sol), g) / (2 * g.Lx * g.Ly) / self.ell ** 2

    def energy(self):
        return self.kinetic_energy() + self.potential_energy()

    def enstrophy(self):
        g = self.grid
        return parsevalsum2(self.sol + self.etah, g) / (2 * g.Lx * g.Ly)

    def _barotropic_only(self):
        if self.ell is not None:
            raise NotImplementedError("not implemented for finite deformation radius")

    def energy_dissipation(self):
        self._barotropic_only()
        a = self.nu * _powK(self.grid.Krsq, self.nnu - 1) * np.abs(self.sol) ** 2
        a[0, 0] = 0
        return self._ps(a)

    def enstrophy_dissipation(self):
        self._barotropic_only()
        a = self.nu * _powK(self.grid.Krsq, self.nnu) * np.abs(self.sol) ** 2
        a[0, 0] = 0
        return self._ps(a)

    def _worksol(self):
        return (self.prevsol + self.sol) / 2 if self.forcing.stochastic else self.sol

    def energy_work(self):
        self._barotropic_only()
        return self._ps(self.grid.invKrsq * self._worksol() * np.conj(self.Fh))

    def enstrophy_work(self):
        self._barotropic_only()
        return self._ps(self._worksol() * np.conj(self.Fh))

    def energy_drag(self):
        self._barotropic_only()
        a = self.mu * self.grid.invKrsq * np.abs(self.sol) ** 2
        a[0, 0] = 0
        return self._ps(a)

    def enstrophy_drag(self):
        self._barotropic_only()
        a = self.mu * np.abs(self.sol) ** 2
        a[0, 0] = 0
        return self._ps(a)


# ---------------------------------------------------------------------------------------
# SurfaceQG (src/surfaceqg.jl)
# ---------------------------------------------------------------------------------------
class SurfaceQG(Problem):
    """src/surfaceqg.jl:76-100 (Problem), :127-130 (psihfrombh), :149-154 (Equation),
    :257-297 (calcN!)."""

    def __init__(self, nx=256, ny=None, Lx=2 * np.pi, Ly=None, H=np.inf, nu=0.0, nnu=1, dt=0.01,
                 stepper="RK4", forcing=None, aliased_fraction=1 / 3):
        g = Grid(nx, Lx, ny, Ly, aliased_fraction)
        self.H, self.nu, self.nnu = H, nu, nnu
        K = np.sqrt(g.Krsq)
        with np.errstate(divide="ignore", invalid="ignore"):
            self.psihfrombh = np.where(K == 0, 0.0, 1.0 / np.where(K == 0, 1, K) / np.tanh(H * K))
        L = -nu * _powK(g.Krsq, nnu)
        L[0, 0] = 0
        super().__init__(g, L, self._advection, (g.ny, g.nkr), dt, stepper, forcing)

    def _advection(self, N, sol, t):
        g = self.grid
        dealias(sol, g)
        uh = 1j * g.l * self.psihfrombh * sol
        vh = -1j * g.kr * self.psihfrombh * sol
        u, v, b = irfft2(uh, g), irfft2(vh, g), irfft2(sol, g)
        N[...] = -1j * g.kr * rfft2(u * b) - 1j * g.l * rfft2(v * b)

    def updatevars(self):
        g, sol = self.grid, self.sol
        dealias(sol, g)
        self.b = irfft2(sol, g)
        self.u = irfft2(1j * g.l * self.psihfrombh * sol, g)
        self.v = irfft2(-1j * g.kr * self.psihfrombh * sol, g)

    def set_b(self, b):
        self.sol[...] = rfft2(b)
        self.sol[0, 0] = 0
        self.updatevars()

    def get_streamfunction(self):
        return irfft2(self.psihfrombh * self.sol, self.grid)

    def _ps(self, a):
        g = self.grid
        return parsevalsum(a, g) / (g.Lx * g.Ly)

    def kinetic_energy(self):
        return self._ps(0.5 * self.grid.Krsq * np.abs(self.psihfrombh * self.sol) ** 2)

    def buoyancy_variance(self):
        return self._ps(np.abs(self.sol) ** 2)

    def total_3D_energy(self):
        return self._ps(0.5 * self.psihfrombh * np.abs(self.sol) ** 2)

    def buoyancy_dissipation(self):
        a = 2 * self.nu * _powK(self.grid.Krsq, self.nnu) * np.abs(self.sol) ** 2
        a[0, 0] = 0
        return self._ps(a)

    def buoyancy_work(self):
        if self.forcing.stochastic:
            return self._ps((self.prevsol + self.sol) * np.conj(self.Fh))
        return self._ps(2 * self.sol * np.conj(self.Fh))


# ---------------------------------------------------------------------------------------
# MultiLayerQG (src/multilayerqg.jl)
# ---------------------------------------------------------------------------------------
class MultiLayerQG(Problem):
    """src/multilayerqg.jl:87-135 (Problem), :255-320 (Params), :338-347 (hyperviscosity),
    :603-634 (calcS!, calcS⁻¹!), :651-731 (calcN!), :675-779 (linear variant)."""

    def __init__(self, nlayers, nx=128, ny=None, Lx=2 * np.pi, Ly=None, f0=1.0, beta=0.0, U=None,
                 H=None, b=None, eta=None, topographic_pv_gradient=(0.0, 0.0), mu=0.0, nu=0.0,
                 nnu=1, dt=0.01, stepper="RK4", forcing=None, linear=False,
                 aliased_fraction=1 / 3):
        g = Grid(nx, Lx, ny, Ly, aliased_fraction)
        n = self.nlayers = int(nlayers)
        self.f0, self.beta, self.mu, self.nu, self.nnu, self.linear = f0, beta, mu, nu, nnu, linear
        H = np.full(n, 1 / n) if H is None else np.asarray(H, dtype=np.float64)
        b = -(1 + np.arange(n) / n) if b is None else np.asarray(b, dtype=np.float64)
        self.H, self.b = H, b
        # U -> (nlayers, ny) (convert_U_to_U3D, src/multilayerqg.jl:219-250)
        if U is None:
            Uy = np.zeros((n, g.ny))
        elif np.isscalar(U):
            Uy = np.full((n, g.ny), float(U))
        else:
            Ua = np.asarray(U, dtype=np.float64)
            if Ua.ndim == 1 and Ua.size == n:
                Uy = np.repeat(Ua[:, None], g.ny, axis=1)
            elif Ua.ndim == 1:
                Uy = np.repeat(Ua.reshape(1, g.ny), n, axis=0)
            else:  # (ny, nlayers) as in the reference tests
                Uy = Ua.reshape(g.ny, n).T.copy()
        self.Uy = Uy
        ly = g.l[:, 0]
        Uyy = np.real(np.fft.ifft(-ly ** 2 * np.fft.fft(Uy, axis=1), axis=1))
        eta = np.zeros((g.ny, g.nx)) if eta is None else np.asarray(eta, dtype=np.float64)
        self.eta = eta
        etah = rfft2(eta)
        etax = irfft2(1j * g.kr * etah, g) + topographic_pv_gradient[0]
        etay = irfft2(1j * g.l * etah, g) + topographic_pv_gradient[1]
        self.Qx = np.zeros((n, g.ny, g.nx))
        self.Qx[n - 1] += etax
        Qy = np.repeat((beta - Uyy)[:, :, None], g.nx, axis=2)
        Qy[n - 1] += etay
        if n >= 2:
            gp = b[:-1] - b[1:]
            self.gprime = gp
            self.Fm = f0 ** 2 / (gp * H[1:])
            self.Fp = f0 ** 2 / (gp * H[:-1])
            F = np.zeros((n, n))
            for j in range(n - 1):
                F[j, j + 1] = self.Fp[j]
                F[j + 1, j] = self.Fm[j]
            for j in range(n):
                F[j, j] = -((self.Fp[j] if j < n - 1 else 0) + (self.Fm[j - 1] if j > 0 else 0))
            self.F = F
            K2 = g.Krsq
            self.S = -K2[..., None, None] * np.eye(n) + F          # (ny, nkr, n, n)
            K2i = np.where(K2 == 0, 1.0, K2)
            self.Sinv = np.linalg.inv(-K2i[..., None, None] * np.eye(n) + F)
            self.Sinv[0, 0] = 0
            Ux = np.repeat(Uy[:, :, None], g.nx, axis=2)
            Qy[0] -= self.Fp[0] * (Ux[1] - Ux[0])
            for j in range(1, n - 1):
                Qy[j] -= self.Fp[j] * (Ux[j + 1] - Ux[j]) + self.Fm[j - 1] * (Ux[j - 1] - Ux[j])
            Qy[n - 1] -= self.Fm[n - 2] * (Ux[n - 2] - Ux[n - 1])
        self.Qy = Qy
        L = np.repeat((-nu * _powK(g.Krsq, nnu))[None], n, axis=0)
        L[:, 0, 0] = 0
        calc = self._linear_advection if linear else self._advection
        super().__init__(g, L, calc, (n, g.ny, g.nkr), dt, stepper, forcing)
        self.psih = np.zeros_like(self.sol)

    def streamfunctionfrompv(self, qh):
        if self.nlayers == 1:
            return -self.grid.invKrsq * qh
        return np.einsum("yxij,jyx->iyx", self.Sinv, qh)

    def pvfromstreamfunction(self, psih):
        if self.nlayers == 1:
            return -self.grid.Krsq * psih
        return np.einsum("yxij,jyx->iyx", self.S, psih)

    def _terms(self, sol):
        g = self.grid
        psih = self.streamfunctionfrompv(sol)
        uh, vh = -1j * g.l * psih, 1j * g.kr * psih
        u = irfft2(uh, g) + self.Uy[:, :, None]
        v = irfft2(vh, g)
        q = irfft2(sol, g)
        return psih, u, v, q

    def _advection(self, N, sol, t):
        g = self.grid
        dealias(sol, g)
        psih, u, v, q = self._terms(sol)
        N[...] = -rfft2(u * self.Qx)
        N -= rfft2(v * self.Qy)
        N -= 1j * g.kr * rfft2(u * q) + 1j * g.l * rfft2(v * q)
        N[-1] += self.mu * g.Krsq * psih[-1]
        self.psih = psih

    def _linear_advection(self, N, sol, t):
        g = self.grid
        psih, u, v, q = self._terms(sol)
        N[...] = -rfft2(u * self.Qx)
        N -= rfft2(v * self.Qy)
        N -= 1j * g.kr * rfft2(self.Uy[:, :, None] * q)
        N[-1] += self.mu * g.Krsq * psih[-1]
        self.psih = psih

    def updatevars(self):
        g, sol = self.grid, self.sol
        dealias(sol, g)
        psih = self.streamfunctionfrompv(sol)
        self.q, self.psi = irfft2(sol, g), irfft2(psih, g)
        self.u, self.v = irfft2(-1j * g.l * psih, g), irfft2(1j * g.kr * psih, g)
        self.psih = psih

    def set_q(self, q):
        qh = rfft2(np.asarray(q, dtype=np.float64).reshape(self.sol.shape[0], self.grid.ny, self.grid.nx))
        qh[:, 0, 0] = 0
        self.sol[...] = qh
        self.updatevars()

    def set_psi(self, psi):
        psih = rfft2(np.asarray(psi, dtype=np.float64).reshape(self.sol.shape[0], self.grid.ny, self.grid.nx))
        q = irfft2(self.pvfromstreamfunction(psih), self.grid)
        self.set_q(q)

    def energies(self):
        g = self.grid
        psih = self.streamfunctionfrompv(self.sol)
        a = g.Krsq * np.abs(psih) ** 2
        if self.nlayers == 1:
            return parsevalsum(a[0], g) / (2 * g.Lx * g.Ly)
        V = g.Lx * g.Ly * np.sum(self.H)
        KE = np.array([parsevalsum(a[j], g) / (2 * V) * self.H[j] for j in range(self.nlayers)])
        PE = np.array([parsevalsum2(psih[j] - psih[j + 1], g) / (2 * V) * self.f0 ** 2 / self.gprime[j]
                       for j in range(self.nlayers - 1)])
        return KE, PE

    def fluxes(self):
        g = self.grid
        self.updatevars()
        uh = -1j * g.l * self.psih
        uy = irfft2(1j * g.l * uh, g)
        U = self.Uy[:, :, None]
        if self.nlayers == 1:
            return float(np.sum(U * self.v * uy)) * g.dx * g.dy / (g.Lx * g.Ly)
        V = g.Lx * g.Ly * np.sum(self.H)
        lateral = self.H * np.sum(U * self.v * uy, axis=(1, 2)) * g.dx * g.dy / V
        vertical = np.array([np.sum(self.f0 ** 2 / self.gprime[j] * (U[j] - U[j + 1]) * self.v[j + 1] * self.psi[j])
                             for j in range(self.nlayers - 1)]) * g.dx * g.dy / V
        return lateral, vertical


# ---------------------------------------------------------------------------------------
# Initial-condition helpers (src/utils.jl)
# ---------------------------------------------------------------------------------------
def peakedisotropicspectrum(grid, kpeak, E0, mask=None, allones=False, seed=1234):
    """src/utils.jl:29-54.  Complex-Gaussian coefficients (Philox, tag TAG_INITIAL)
    scaled by |psi_hat| = (K^2 (1 + (K/k0)^4))^(-1/2); energy normalised with a sum over the
    half spectrum only, as the reference does (:50); returns zeta = irfft(-K^2 psi_hat)."""
    if grid.Lx != grid.Ly:
        raise ValueError("the domain is not square")
    k0 = kpeak * 2 * np.pi / grid.Lx
    modk = np.sqrt(grid.Krsq)
    with np.errstate(divide="ignore"):
        modpsi = (modk ** 2 * (1 + (modk / k0) ** 4)) ** -0.5
    modpsi[0, 0] = 0.0
    if allones:
        psih = modpsi.astype(np.complex128)
    else:
        phases = complex_normal(grid.Krsq.size, seed, 0, TAG_INITIAL).reshape(grid.Krsq.shape)
        psih = phases * modpsi
    if mask is not None:
        psih = psih * mask
    e0 = np.sum(grid.Krsq * np.abs(psih) ** 2) / (grid.nx * grid.ny) ** 2
    psih = psih * math.sqrt(E0 / e0)
    return irfft2(-grid.Krsq * psih, grid)


def lambdipole(U, R, grid, center=None):
    """src/utils.jl:8-20: the Lamb dipole of strength U and radius R, centred at the means of
    the grid coordinates (-dx/2, -dy/2 for the grid x = -Lx/2 + i dx): with k = j1 / R (j1 the
    first zero of J1) and q0 = -2 U k / J0(k R), q = q0 J1(k r) (y - yc) / r inside r < R and
    zero outside.  Returns (ny, nx)."""
    from scipy.special import j0, j1
    firstzero = 3.8317059702075123156
    k = firstzero / R
    q0 = -2 * U * k / j0(k * R)
    x, y = grid.gridpoints()
    xc, yc = (np.mean(grid.x), np.mean(grid.y)) if center is None else center
    r = np.sqrt((x - xc) ** 2 + (y - yc) ** 2)
    q = q0 * j1(k * r) * (y - yc) / r
    return np.where(r >= R, 0.0, q)


def ring_forcing_spectrum(grid, kf, dkf, eps):
    """Gaussian ring forcing spectrum normalised to inject energy at rate eps
    (examples/singlelayerqg_betaforced.jl:61-73)."""
    K = np.sqrt(grid.Krsq)
    spec = np.exp(-(K - kf) ** 2 / (2 * dkf ** 2))
    spec[grid.Krsq == 0] = 0
    eps0 = parsevalsum(spec * grid.invKrsq / 2, grid) / (grid.Lx * grid.Ly)
    return spec * (eps / eps0)


def rel_l2(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))
