"""Host-side mirror of FourierFlows.Problem / stepforward! / Diagnostic over libgfcuda.

The reference's user-facing objects (FourierFlows 0.10.5, re-exported at
src/GeophysicalFlows.jl:15) are mirrored with the same names and meaning; the state lives
on the GPU and crosses the boundary only when a field is read:

    prob.sol          spectral state (numpy copy, shape (nlayers?, ny, nkr))
    prob.clock        t, dt, step
    prob.grid         TwoDGrid quantities (x, y, kr, l, Krsq, invKrsq, ...)
    prob.vars         physical fields after updatevars!
    stepforward(prob, nsteps) / stepforward(prob, diags, nsteps)

NumPy arrays are C-ordered with shape (ny, nx) / (ny, nkr), the same memory order as the
reference's column-major (nx, ny) / (nkr, ny) Julia arrays.
"""
import ctypes as C
import math
import weakref

import numpy as np

from . import _abi as A


class Grid:
    """Wavenumber and grid-point arrays of FourierFlows.TwoDGrid (x in [-Lx/2, Lx/2))."""

    def __init__(self, nx, ny, Lx, Ly, aliased_fraction, T):
        self.nx, self.ny, self.Lx, self.Ly = nx, ny, Lx, Ly
        self.nkr, self.nl, self.nk = nx // 2 + 1, ny, nx
        self.dx, self.dy = Lx / nx, Ly / ny
        self.x = (-Lx / 2 + self.dx * np.arange(nx)).astype(T)
        self.y = (-Ly / 2 + self.dy * np.arange(ny)).astype(T)
        self.kr = (2 * np.pi / Lx) * np.arange(self.nkr)[None, :]
        self.l = (2 * np.pi / Ly) * (np.fft.fftfreq(ny) * ny)[:, None]
        self.Krsq = self.kr ** 2 + self.l ** 2
        self.invKrsq = np.where(self.Krsq == 0, 0.0, 1.0 / np.where(self.Krsq == 0, 1.0, self.Krsq))
        self.aliased_fraction = aliased_fraction
        self.T = T
        self._prob = None  # weak reference to the Problem whose context computes on this grid

    def gridpoints(self):
        return np.meshgrid(self.x, self.y, indexing="xy")


class TimeStepper:
    """prob.timestepper: the stepper's name and, for the Filtered steppers, its filter
    ([ny, nx/2+1], FourierFlows makefilter as built by the library)."""

    def __init__(self, prob, name):
        self._prob, self.name = weakref.ref(prob), name

    @property
    def filter(self):
        p = self._prob()
        out = np.empty((p.grid.ny, p.grid.nkr), dtype=np.float64)
        code = p._lib.gf_get_filter(p._ctx, out.ctypes.data)
        if code == A.GF_ERR_STATE:
            raise AttributeError(f"{self.name} has no filter")
        p._c(code)
        return out


class Clock:
    def __init__(self, prob, dt):
        self._prob, self.dt = prob, dt

    @property
    def t(self):
        t = C.c_double()
        A.check(self._prob._lib, self._prob._ctx, self._prob._lib.gf_get_clock(self._prob._ctx, C.byref(t), None))
        return t.value

    @property
    def step(self):
        s = C.c_int64()
        A.check(self._prob._lib, self._prob._ctx, self._prob._lib.gf_get_clock(self._prob._ctx, None, C.byref(s)))
        return s.value


class Forcing:
    """Device-side forms of the reference's calcF! callbacks (see include/gfcuda.h), or
    kind="callback" with calcF(Fh, sol, t, clock, vars, params, grid): an arbitrary host
    calcF! called before every stage with its time (sol is None: the state stays on the
    device); it fills the half-spectrum Fh in place.  The callback path waits for the host at
    every stage (the library's gf_step_callback)."""

    def __init__(self, kind=None, Fh=None, spectrum=None, omega=0.0, phase=0.0, seed=0, calcF=None):
        if kind not in A.FORCING and kind != "callback":
            raise ValueError(f"unknown forcing kind {kind}")
        if kind == "callback" and calcF is None:
            raise ValueError("kind='callback' needs calcF")
        self.kind, self.Fh, self.spectrum, self.omega, self.phase, self.seed = kind, Fh, spectrum, omega, phase, seed
        self.calcF = calcF

    @property
    def stochastic(self):
        return self.kind in ("stochastic", "stochastic_phase")


class Vars:
    """Physical fields of prob.vars, filled by updatevars!."""

    def __init__(self, names):
        self._names = names
        for n in names.values():
            setattr(self, n, None)


class Problem:
    """FourierFlows.Problem backed by a libgfcuda context."""

    module = None
    field_names = {A.FIELD_Q: "q", A.FIELD_PSI: "psi", A.FIELD_U: "u", A.FIELD_V: "v"}

    def __init__(self, cfg_kwargs, nx, ny, Lx, Ly, dt, stepper, T, aliased_fraction, forcing, nlayers=1,
                 stream=None, precision=None, batch=1):
        self._lib = A.load()
        self._ctx = C.c_void_p()
        if stepper not in A.STEPPERS:
            raise ValueError(f"unknown stepper {stepper}")
        T = np.dtype(T).type
        if T not in (np.float32, np.float64):
            raise ValueError("T must be Float32 or Float64")
        self.T, self.CT = T, (np.complex64 if T == np.float32 else np.complex128)
        self.nlayers = nlayers
        self.grid = Grid(nx, ny, Lx, Ly, aliased_fraction, T)
        self.forcing = forcing if forcing is not None else Forcing(None)
        self.stepper = stepper
        cfg = A.gf_config()
        cfg.module = A.MODULES[self.module]
        precision = (precision or ("F32" if T == np.float32 else "F64")).upper()
        if precision not in ("F32", "F64", "DF64") or (precision == "F32") != (T == np.float32):
            raise ValueError("precision must be F32 (T=Float32), F64 or DF64 (T=Float64)")
        self.precision = precision
        cfg.precision = {"F32": A.F32, "F64": A.F64, "DF64": A.DF64}[precision]
        cfg.stepper = A.STEPPERS[stepper]
        cfg.nx, cfg.ny, cfg.nlayers = nx, ny, nlayers
        cfg.Lx, cfg.Ly, cfg.dt, cfg.aliased_fraction = Lx, Ly, dt, aliased_fraction
        cfg.forcing_kind = A.FORCING["static" if self.forcing.kind == "callback" else self.forcing.kind]
        cfg.seed = int(self.forcing.seed)
        self.batch = int(batch)
        cfg.batch = self.batch
        cfg.forcing_omega, cfg.forcing_phase = self.forcing.omega, self.forcing.phase
        self._keep = []  # arrays referenced by cfg during gf_create
        for k, v in cfg_kwargs.items():
            if isinstance(v, np.ndarray):
                a = np.ascontiguousarray(v, dtype=np.float64)
                self._keep.append(a)
                setattr(cfg, k, a.ctypes.data_as(C.POINTER(C.c_double)))
            elif k == "topographic_pv_gradient":
                cfg.topographic_pv_gradient[0], cfg.topographic_pv_gradient[1] = float(v[0]), float(v[1])
            else:
                setattr(cfg, k, v)
        A.check(self._lib, None, self._lib.gf_create(C.byref(cfg), stream, C.byref(self._ctx)))
        self._keep = []
        self.clock = Clock(self, dt)
        self.timestepper = TimeStepper(self, stepper)
        self.grid._prob = weakref.ref(self)
        self.vars = Vars(self.field_names)
        if self.forcing.kind in ("static", "harmonic") and self.forcing.Fh is not None:
            self.set_forcing(self.forcing.Fh)
        elif self.forcing.stochastic and self.forcing.spectrum is not None:
            self.set_forcing(self.forcing.spectrum)

    # -- shapes
    @property
    def spec_shape(self):
        g = self.grid
        shp = (self.nlayers, g.ny, g.nkr) if self.module == "MultiLayerQG" else (g.ny, g.nkr)
        return ((self.batch,) + shp) if self.batch > 1 else shp

    @property
    def phys_shape(self):
        g = self.grid
        shp = (self.nlayers, g.ny, g.nx) if self.module == "MultiLayerQG" else (g.ny, g.nx)
        return ((self.batch,) + shp) if self.batch > 1 else shp

    def _c(self, code):
        A.check(self._lib, self._ctx, code)

    def close(self):
        if getattr(self, "_ctx", None):
            self._lib.gf_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- state
    @property
    def sol(self):
        out = np.empty(self.spec_shape, dtype=self.CT)
        self._c(self._lib.gf_get_state(self._ctx, out.ctypes.data, A.HOST))
        return out

    @sol.setter
    def sol(self, value):
        a = np.ascontiguousarray(np.broadcast_to(value, self.spec_shape), dtype=self.CT)
        self._c(self._lib.gf_set_state(self._ctx, a.ctypes.data, A.HOST))

    def set_clock(self, t, step):
        self._c(self._lib.gf_set_clock(self._ctx, float(t), int(step)))

    def autotune(self, reps=4):
        """Time the step kernels at every candidate launch shape and keep the fastest;
        returns {row_radix, row_pairs, col_radix, col_columns, tma_columns, field_parallel}
        (tma_columns > 0: the column stage runs with TMA tile copies, that many columns per
        block; field_parallel: (row radix, column radix, columns) of the field-parallel
        small-grid kernels, radix 0 where the classic kernel runs)."""
        sh = (C.c_int32 * 4)()
        self._c(self._lib.gf_autotune(self._ctx, int(reps), sh))
        d = dict(zip(("row_radix", "row_pairs", "col_radix", "col_columns"), list(sh)))
        d["tma_columns"] = self.tma_columns
        d["field_parallel"] = self.field_parallel
        return d

    @property
    def field_parallel(self):
        """(row radix, column radix, columns per block) of the field-parallel small-grid
        kernels; radix 0: that half of the stage runs the classic kernel."""
        v = (C.c_int32 * 3)()
        self._c(self._lib.gf_get_field_parallel(self._ctx, v))
        return tuple(v)

    @field_parallel.setter
    def field_parallel(self, rrc):
        r, rc, cols = (tuple(rrc) + (0, 0, 0))[:3]
        self._c(self._lib.gf_set_field_parallel(self._ctx, int(r), int(rc), int(cols)))

    @property
    def tma_columns(self):
        """Columns per block of the TMA column stage (0: per-thread-copy column kernel)."""
        v = C.c_int32()
        self._c(self._lib.gf_get_tma_columns(self._ctx, C.byref(v)))
        return v.value

    @tma_columns.setter
    def tma_columns(self, n):
        self._c(self._lib.gf_set_tma_columns(self._ctx, int(n)))

    @property
    def launch_shape(self):
        sh = (C.c_int32 * 4)()
        self._c(self._lib.gf_get_launch_shape(self._ctx, sh))
        return tuple(sh)

    @launch_shape.setter
    def launch_shape(self, shape):
        sh = (C.c_int32 * 4)(*[int(v) for v in shape])
        self._c(self._lib.gf_set_launch_shape(self._ctx, sh))

    def set_graph_steps(self, n):
        """Steps per captured CUDA graph (0: launch kernel by kernel)."""
        self._c(self._lib.gf_set_graph_steps(self._ctx, int(n)))

    def set_forcing(self, data):
        if self.forcing.stochastic:
            a = np.ascontiguousarray(data, dtype=self.T).reshape(self.grid.ny, self.grid.nkr)
        else:
            a = np.ascontiguousarray(np.broadcast_to(data, self.spec_shape), dtype=self.CT)
        self._c(self._lib.gf_set_forcing(self._ctx, a.ctypes.data, A.HOST))

    def _set_physical(self, which, field):
        a = np.ascontiguousarray(np.asarray(field).reshape(self.phys_shape), dtype=self.T)
        self._c(self._lib.gf_set_physical(self._ctx, which, a.ctypes.data, A.HOST))
        self._pull_vars()

    def updatevars(self):
        self._c(self._lib.gf_updatevars(self._ctx))
        self._pull_vars()

    def _pull_vars(self):
        for which, name in self.field_names.items():
            out = np.empty(self.phys_shape, dtype=self.T)
            self._c(self._lib.gf_get_field(self._ctx, which, out.ctypes.data, A.HOST))
            setattr(self.vars, name, out)

    def calcN(self, sol, t):
        """calcN!(N, sol, t, ...): returns (N, dealiased sol)."""
        s = np.ascontiguousarray(np.broadcast_to(sol, self.spec_shape), dtype=self.CT).copy()
        N = np.empty(self.spec_shape, dtype=self.CT)
        self._c(self._lib.gf_calcN(self._ctx, N.ctypes.data, s.ctypes.data, float(t), A.HOST))
        return N, s

    def fwdtransform(self, field):
        a = np.ascontiguousarray(np.asarray(field).reshape(self.phys_shape), dtype=self.T)
        out = np.empty(self.spec_shape, dtype=self.CT)
        self._c(self._lib.gf_fwdtransform(self._ctx, out.ctypes.data, a.ctypes.data, A.HOST))
        return out

    def invtransform(self, fieldh):
        a = np.ascontiguousarray(np.broadcast_to(fieldh, self.spec_shape), dtype=self.CT)
        out = np.empty(self.phys_shape, dtype=self.T)
        self._c(self._lib.gf_invtransform(self._ctx, out.ctypes.data, a.ctypes.data, A.HOST))
        return out

    def diagnostics(self, ids):
        """Values of the diagnostics `ids`; shape (len(ids),) or (batch, len(ids))."""
        ids = np.ascontiguousarray(ids, dtype=np.int32)
        out = np.empty(len(ids) * self.batch, dtype=np.float64)
        self._c(self._lib.gf_diagnostics(self._ctx, ids.ctypes.data_as(C.POINTER(C.c_int32)), len(ids),
                                         out.ctypes.data_as(C.POINTER(C.c_double))))
        return out.reshape(self.batch, len(ids)) if self.batch > 1 else out

    def synchronize(self):
        self._c(self._lib.gf_synchronize(self._ctx))


class Diagnostic:
    """FourierFlows.Diagnostic: a time series recorded after every step (freq=1)."""

    def __init__(self, calc, prob, nsteps=100):
        self.calc, self.prob = calc, prob
        self.data = [calc(prob)]
        self.t = [prob.clock.t]
        self.steps = [prob.clock.step]

    @property
    def i(self):
        return len(self.data)

    def __getitem__(self, k):
        return np.asarray(self.data)[k]

    def increment(self):
        self.data.append(self.calc(self.prob))
        self.t.append(self.prob.clock.t)
        self.steps.append(self.prob.clock.step)


def stepforward(prob, *args):
    """stepforward!(prob[, nsteps]) or stepforward!(prob, diags, nsteps)."""
    if len(args) == 0:
        diags, n = None, 1
    elif len(args) == 1:
        diags, n = None, int(args[0])
    else:
        diags, n = args[0], int(args[1])
    if prob.forcing.kind == "callback":
        _step_callback(prob, n, diags)
        return
    if not diags:
        prob._c(prob._lib.gf_step(prob._ctx, n))
        return
    diags = diags if isinstance(diags, (list, tuple)) else [diags]
    ids = [getattr(d.calc, "diag_id", None) for d in diags]
    if prob.batch == 1 and all(i is not None for i in ids) and n > 0:
        # library diagnostics: reduced on the device after every step, one host wait per call
        idv = np.ascontiguousarray(ids, dtype=np.int32)
        out = np.empty((n, len(ids)), dtype=np.float64)
        t, step, dt = prob.clock.t, prob.clock.step, prob.clock.dt
        prob._c(prob._lib.gf_step_diags(prob._ctx, n, idv.ctypes.data_as(C.POINTER(C.c_int32)), len(ids),
                                        out.ctypes.data_as(C.POINTER(C.c_double))))
        for k in range(n):
            t += dt
            for j, d in enumerate(diags):
                d.data.append(float(out[k, j]))
                d.t.append(t)
                d.steps.append(step + k + 1)
        return
    for _ in range(n):
        prob._c(prob._lib.gf_step(prob._ctx, 1))
        for d in diags:
            d.increment()


class _StageClock:
    """clock seen by a callback calcF: t of the stage, the step number and dt"""

    def __init__(self, t, step, dt):
        self.t, self.step, self.dt = t, step, dt


def _step_callback(prob, n, diags=None):
    g = prob.grid
    shape = prob.spec_shape
    nel = int(np.prod(shape))
    calcF = prob.forcing.calcF
    err = []

    def fn(t, step, stage, ptr, user):
        try:
            Fh = np.ctypeslib.as_array(C.cast(ptr, C.POINTER(C.c_float if prob.T == np.float32 else C.c_double)),
                                       shape=(2 * nel,)).view(prob.CT).reshape(shape)
            calcF(Fh, None, t, _StageClock(t, step, prob.clock.dt), prob.vars, getattr(prob, "params", None), g)
            return 0
        except Exception as e:  # reported after the library call returns
            err.append(e)
            return 1

    cb = A.FORCING_FN(fn)
    diags = (diags if isinstance(diags, (list, tuple)) else [diags]) if diags else []
    for _ in range(n if diags else 1):
        code = prob._lib.gf_step_callback(prob._ctx, 1 if diags else n, cb, None)
        if err:
            raise err[0]
        prob._c(code)
        for d in diags:
            d.increment()


def stepforward_output(prob, nsteps, every, diagnostics=(), fields=()):
    """Step nsteps and record, after every `every` steps, the library diagnostics (ids or
    module diagnostic functions such as TwoDNavierStokes.energy) and physical fields (names
    in prob.field_names, e.g. "zeta"), without a host wait per output.  Returns
    (diag array [nout, (batch,) nd], {field name: array [nout, (batch,) ...]})."""
    ids = [d if isinstance(d, (int, np.integer)) else d.diag_id for d in diagnostics]
    names = {v: k for k, v in prob.field_names.items()}
    fsel = [names[f] for f in fields]
    nout = int(nsteps) // int(every)
    shp = prob.phys_shape
    idv = np.ascontiguousarray(ids, dtype=np.int32)
    fv = np.ascontiguousarray(fsel, dtype=np.int32)
    dout = np.empty((nout, prob.batch, len(ids)), dtype=np.float64)
    fout = np.empty((nout, len(fsel)) + shp, dtype=prob.T)
    prob._c(prob._lib.gf_step_output(prob._ctx, int(nsteps), int(every), idv.ctypes.data_as(C.POINTER(C.c_int32)),
                                     len(ids), dout.ctypes.data_as(C.POINTER(C.c_double)),
                                     fv.ctypes.data_as(C.POINTER(C.c_int32)), len(fsel), fout.ctypes.data))
    if prob.batch == 1:
        dout = dout[:, 0]
    return dout, {f: fout[:, i] for i, f in enumerate(fields)}


def ensemble_step(probs, nsteps, persistent=False):
    """Step several problems (e.g. batched problems of different grid sizes) together, from
    one CUDA graph when graphs are on.  persistent=False: each problem runs its own launches
    on its own stream, concurrently; persistent=True: where the problems allow it (one layer,
    square 32/64/128/256 grids, one precision, not AB3), every stage of all of them runs in one
    persistent row launch and one persistent column launch over a work list of all tiles."""
    lib = probs[0]._lib
    probs[0]._c(lib.gf_set_ensemble_mode(probs[0]._ctx, 1 if persistent else 0))
    arr = (C.c_void_p * len(probs))(*[p._ctx.value for p in probs])
    code = lib.gf_ensemble_step(arr, len(probs), int(nsteps))
    if code != A.GF_OK:
        raise A.GFError(code, lib.gf_last_error(None).decode(errors="replace"))


def dealias(prob):
    """dealias!(prob.sol, prob.grid) on the device state (updatevars! does it too)."""
    prob._c(prob._lib.gf_updatevars(prob._ctx))


def _check_dev(dev):
    """The reference takes dev = CPU() | GPU(); this library runs on the GPU only."""
    if str(dev).upper().rstrip("()") != "GPU":
        raise ValueError("libgfcuda runs on the GPU only: pass dev='GPU'")
