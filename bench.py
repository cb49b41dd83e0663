"""Benchmark of the pseudospectral time step on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Headline workload: TwoDNavierStokes 2048^2, FilteredRK4, nu = 0, peaked isotropic initial
vorticity (k0 = 6, E = 0.5) -- the configuration the FP32-fused vs FP64-plain target is
quoted on.  A "step" is one FilteredRK4 time step (4 calcN! stages); --steps K and --warmup W
count these model steps.  `value` is FP32-fused grid-point*steps/s with the state resident in
HBM, timed over exactly K steps run as stepforward! calls of 10 steps (an output interval: the
state is looked at after every call, so the last step of each call computes every mode and
the others only the modes a later step reads), each call one replay of the context's captured
10-step CUDA graph; the per-kernel times behind the roofline come from the same calls run
again with the library's per-launch events (no graphs; `ms_per_step_instrumented`);
single-step calls (every step observed) are timed beside it (`value_single_step_calls`).  The FP64-plain arm, its roofline and the
FP32-vs-FP64 error are reported beside it, and so are the other GPU workloads: SingleLayerQG
512^2 ETDRK4 with stochastic forcing, MultiLayerQG 3 x 1024^2 ETDRK4, and the 1536-run
TwoDNavierStokes ensemble (1024 x 64^2 + 384 x 128^2 + 128 x 256^2).  L2 is flushed (256 MiB
write) before every timed call; graph-replayed timings of the same calls are reported too.
`--impl reference` times the FP64 CPU restatement of the reference (oracle/, scipy.fft on all
host cores) on the same workload.  For N > 1 (torchrun) every rank runs an independent
replica (the path does not shard) and rank 0 reports the aggregate over the slowest rank.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(ROOT, "geophysicalflows.jl_gb300"), os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "grid-pt·steps/s FP32-fused vs FP64-plain (≤1e-5 rel L2); adjoint/forward step time"
UNIT = "grid-pt*steps/s"
HEADLINE = dict(module="TwoDNavierStokes", nx=2048, ny=2048, stepper="FilteredRK4", dt=5e-4)
SLQG512 = dict(module="SingleLayerQG", nx=512, ny=512, stepper="ETDRK4", dt=0.05, beta=10.0, mu=0.01,
               forcing="stochastic")
# 3 layers, H = [.2,.3,.5], rho = [4, 5, 5.5] -> b with g' = g (rho_{j+1} - rho_j) / rho_{j+1}, g = 1
MLQG1024X3 = dict(module="MultiLayerQG", nx=1024, ny=1024, nlayers=3, stepper="ETDRK4", dt=2.5e-3, f0=1.0, beta=5.0,
               H=[0.2, 0.3, 0.5], b=[-1.0, -1.2, -1.2 - 0.5 / 5.5], U=[1.0, 0.5, 0.0], mu=0.05)
# the decaying 128^2 run (nu = 0, FilteredRK4 dt = 0.005, from the peaked isotropic state)
DECAY128 = dict(module="TwoDNavierStokes", nx=128, ny=128, stepper="FilteredRK4", dt=0.005)
# gradient of the final kinetic energy: SingleLayerQG 256^2, deformation radius 0.35,
# topography |k| <= 8 amplitude 0.1, ETDRK4 dt = 0.01, 500 steps, checkpoint every 25
ADJOINT256 = dict(module="SingleLayerQG", nx=256, ny=256, stepper="ETDRK4", dt=0.01, ell=0.35, nsteps=500, every=25)
# 1536 independent TwoDNavierStokes runs in three batched size classes (size, instances)
ENSEMBLE = dict(classes=((64, 1024), (128, 384), (256, 128)), stepper="FilteredRK4", dt=0.01, nu=1e-4, nnu=1,
                kf=8.0, dkf=1.5, eps=1e-3)


def dealias_geometry(nx, ny):
    """Kept spectral columns and rows of the 2/3 rule (FourierFlows TwoDGrid with
    aliased_fraction = 1/3): kr < kcut and l outside the aliased band."""
    nkr = nx // 2 + 1
    lo, hi = (1 - 1 / 3) / 2, (1 + 1 / 3) / 2
    kcut = min(int(math.floor(lo * nx)), nkr)
    lA, lB = int(math.floor(lo * ny)), int(math.ceil(hi * ny)) - 1
    return nkr, kcut, ny - (lB - lA + 1)


def launch_bytes(w, cb, observed):
    """Bytes one row-kernel and one column-kernel launch must move -- every element of every
    array the launch reads or writes, once -- averaged over the stages of a step.  `cb` is
    the complex element size.  An observed step forms all nkr columns of the products and
    updates every mode of the state; an unobserved one (every step of a stepforward! call
    but the last) forms the products for kr < kcut and updates the kept modes only.  The
    stage input is read at kept modes only (the dealias of calcN!); the pruned inverse
    fields W hold kr < kcut."""
    nx, ny, nl = w["nx"], w["ny"], w.get("nlayers", 1)
    nkr, kcut, rows = dealias_geometry(nx, ny)
    rb = cb // 2
    kept = kcut * rows * nl                       # kept modes, all layers
    S = nl * nkr * ny if observed else kept       # modes the stage combination runs on
    kout = nkr if observed else kcut              # product columns formed
    m = 3 if w["module"] == "MultiLayerQG" else 2
    Wb = 3 * nl * ny * kcut * cb                  # (q, u, v) after the column pass
    Pb = m * nl * ny * kout * cb                  # products after the row pass
    hasL = w.get("nu", 0) > 0 or (w["module"] == "TwoDNavierStokes" and w.get("mu", 0) > 0)
    tables_cplx = w.get("beta", 0) != 0 and w["module"] == "SingleLayerQG"
    tb = cb if tables_cplx else rb
    St = S // nl                                  # table elements ([j][kr], shared by the layers)
    state = 0.0                                   # bytes of the stage combination, whole step
    if "RK4" in w["stepper"] and "ETD" not in w["stepper"]:
        state += (4 * kept + 7 * S) * cb          # sol at kept modes x4; acc w, (r+w) x2, r; sol w
        if hasL:
            state += (3 * kept + 3 * S) * cb + 4 * St * rb   # X written x3, read x3 (kept); L table
        if w["stepper"].startswith("Filtered"):
            state += St * rb                      # filter, last stage
    else:                                         # ETDRK4: s1, N1, acc; e2, zeta, alpha/beta, e, gamma
        state += (3 * kept + 11 * S) * cb + 11 * St * tb
    if w.get("forcing") == "stochastic":
        state += 5 * S * cb + St * rb             # draw -> F (w), F read x3, previous state (w); spectrum
    if w.get("mu", 0) > 0 and w["module"] == "MultiLayerQG":
        state += 4 * (St * cb + ny * kcut * cb)   # bottom drag term: read (epilogue), write (inverse part)
    if nl > 1:
        state += 4 * (nl * ny * kout + kept) * cb  # next-stage X between the two column launches
    stages = 4
    return Wb + Pb, Pb + Wb + state / stages


def algorithmic_bytes(w, word):
    """Bytes per step of the two-sweep reference model of a pseudospectral step: per calcN!
    stage read the stage input (1 word/pt), write and read k inverse-transformed fields,
    write and read m products, write N (1), read a physical parameter arrays, plus C
    stage-combination sweeps per step (RK4 / FilteredRK4 16, ETDRK4 23); `word` = 4 (FP32)
    or 8 (FP64).  It counts every mode in every step (no pruning, no L2 reuse), so it is an
    upper figure beside launch_bytes."""
    k, m, a = 3, 2, 0
    if w["module"] == "MultiLayerQG":
        m = 3
    if w["module"] == "SingleLayerQG" and w.get("eta"):
        a = 1
    C = 23 if "ETDRK4" in w["stepper"] else 16
    return word * points(w) * (4 * (2 + 2 * k + 2 * m + a) + C)


def model_launch_bytes(w, word):
    """The two-sweep model's bytes (algorithmic_bytes) split between the two kernels of a
    stage: the row kernel reads the k inverse-transformed fields and the a parameter arrays
    and writes the m products (k + m + a words/pt); the column kernel reads the m products
    and the stage input, writes the k inverse fields of the next stage and N, and carries the
    stage combination (m + 1 + k + 1 + C/4 words/pt).  Returns (row, column) bytes per launch."""
    k, m, a = 3, 2, 0
    if w["module"] == "MultiLayerQG":
        m = 3
    if w["module"] == "SingleLayerQG" and w.get("eta"):
        a = 1
    C = 23 if "ETDRK4" in w["stepper"] else 16
    n = word * points(w)
    return n * (k + m + a), n * (m + 1 + k + 1 + C / 4)


def step_roofline(w, ms_per_step, word, peaks):
    """The whole step against HBM with the two-sweep model's bytes (algorithmic_bytes)."""
    b = algorithmic_bytes(w, word)
    ach = b / (ms_per_step * 1e-3) / 1e9
    return {"model": "two-sweep words/pt*step", "bytes_per_step": b, "achieved": ach, "unit": "GB/s",
            "frac": ach / peaks["hbm_gbs"]}


CALL_STEPS = 10  # steps per stepforward! call in the timed region (an output interval)


def call_bytes(w, cb, call_steps=CALL_STEPS):
    """Per-launch bytes averaged over the launches of one stepforward! call of call_steps
    steps (the last one observed)."""
    ro, co = launch_bytes(w, cb, True)
    ru, cu = launch_bytes(w, cb, False)
    f = 1.0 / call_steps
    return f * ro + (1 - f) * ru, f * co + (1 - f) * cu


def is_rank0():
    return int(os.environ.get("RANK", "0")) == 0


def dist_setup(n):
    if n <= 1 and int(os.environ.get("WORLD_SIZE", "1")) <= 1:
        return None
    import torch
    import torch.distributed as dist
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    return dist


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during a timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __enter__(self):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
            time.sleep(1.5)  # let the sampler finish starting up before anything is timed
        except OSError:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            self.p.wait()
        self.f.flush()

    def summary(self, dev=0):
        rows = []
        try:
            for line in open(self.f.name):
                parts = [s.strip() for s in line.split(",")]
                if len(parts) >= 9 and parts[0] == str(dev):
                    rows.append(parts)
        finally:
            os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for n, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": float(rows[0][2]) if rows[0][2].replace(".", "").isdigit() else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))), "measured"
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0}, "fallback"


def ncu_figure(kernel, workload, key):
    """A per-launch figure of `kernel` from the committed ncu summary of `workload`
    (profiles/<kernel>_<workload>.md, line '<key>: value'), else None."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_{workload}.md")
    try:
        for line in open(path):
            if line.startswith(key + ":"):
                return float(line.split(":", 1)[1].split()[0])
    except (OSError, ValueError, IndexError):
        pass
    return None


def ncu_traffic(kernel, workload):
    """DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) from ncu."""
    return ncu_figure(kernel, workload, "traffic_bytes_per_launch")


def fft_flops_per_step(w, call_steps=CALL_STEPS):
    """Flop of the transforms of one step of a one-layer 2-D workload, averaged over a call of
    call_steps steps: 5 n log2(n) per complex length-n transform (the standard radix-2 count),
    per stage five transforms per row pair (length nx) and five per column (length ny) -- the
    kcut kept columns in the call's unobserved steps, all nkr in its last one."""
    nx, ny = w["nx"], w["ny"]
    nkr, kcut, _ = dealias_geometry(nx, ny)
    fx, fy = 5 * nx * math.log2(nx), 5 * ny * math.log2(ny)
    rows = 4 * 5 * (ny // 2) * fx
    cols = (4 * 5 * fy) * ((call_steps - 1) * kcut + nkr) / call_steps
    return rows + cols


def fp64_gemm_peak_tflops(n=4096, reps=5):
    """FP64 peak for the IEEE FP64 arm's compute roofline, measured here (MEASURED_PEAKS.json
    holds no FP64 figure): cuBLAS DGEMM through torch.matmul in float64, n^3, best of `reps`
    after one warm-up, CUDA events."""
    import torch
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = math.inf
    for _ in range(reps):
        (e0, e1), = _events(1)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    del a, b
    return 2.0 * n ** 3 / (best * 1e-3) / 1e12


def fp64_compute_roofline(w, ms_per_step, peak_tflops):
    """IEEE FP64 arm against the FP64 pipe: the transforms' flop per step (fft_flops_per_step)
    over the step time, as a fraction of the measured DGEMM rate."""
    fl = fft_flops_per_step(w)
    ach = fl / (ms_per_step * 1e-3) / 1e12
    return {"bound": "fp64", "flop_per_step": fl, "flop_model": "5 n log2 n per complex transform, "
            "5 row and 5 column transforms per stage, kept columns in unobserved steps",
            "achieved": ach, "peak": peak_tflops, "unit": "TFLOP/s", "frac": ach / peak_tflops,
            "peak_source": "measured in this run: cuBLAS DGEMM 4096^3 (torch.matmul float64), best of 5"}


def compute_roofline(roof, workload):
    """Issue-rate roofline of a kernel whose arithmetic, not memory, bounds it (df64): the
    fraction of the SM's instruction-issue slots and of the FMA pipe's cycles it uses (ncu,
    committed summary), and the HBM fraction it would reach at the full issue rate."""
    issue = ncu_figure(roof["kernel"], workload, "issue_active_frac")
    fma = ncu_figure(roof["kernel"], workload, "fma_pipe_active_frac")
    if issue is None:
        return None
    return {"kernel": roof["kernel"], "bound": "issue", "issue_active": issue, "fma_pipe_active": fma,
            "hbm_frac": roof["frac"], "hbm_frac_at_full_issue": roof["frac"] / issue,
            "source": f"ncu --set full, profiles/{roof['kernel']}_{workload}.md"}


def make_problem(w, T, precision=None):
    import gfcuda
    if w["module"] == "TwoDNavierStokes":
        return gfcuda.TwoDNavierStokes.Problem("GPU", nx=w["nx"], ny=w["ny"], dt=w["dt"], stepper=w["stepper"], T=T,
                                               precision=precision)
    if w["module"] == "MultiLayerQG":
        return gfcuda.MultiLayerQG.Problem(w["nlayers"], "GPU", nx=w["nx"], ny=w["ny"], f0=w["f0"], beta=w["beta"],
                                           H=w["H"], b=w["b"], U=w["U"], mu=w["mu"], dt=w["dt"],
                                           stepper=w["stepper"], T=T, precision=precision)
    from gfcuda.core import Grid
    g = Grid(w["nx"], w["ny"], 2 * np.pi, 2 * np.pi, 1 / 3, np.float64)
    spec = gfcuda.utils.ring_forcing_spectrum(g, 14.0, 1.5, 1e-3)
    f = gfcuda.Forcing("stochastic", spectrum=spec, seed=1234)
    return gfcuda.SingleLayerQG.Problem("GPU", nx=w["nx"], beta=w["beta"], mu=w["mu"], dt=w["dt"],
                                        stepper=w["stepper"], forcing=f, T=T, precision=precision)


def set_initial_state(prob, w):
    """The workload's initial condition at t = 0, made by the library (peaked isotropic
    vorticity on the device) or from a seeded generator (MultiLayerQG white noise);
    SingleLayerQG starts at rest."""
    import gfcuda
    if w["module"] == "TwoDNavierStokes":
        z0 = gfcuda.peakedisotropicspectrum(prob.grid, 6, 0.5, mask=prob.timestepper.filter, seed=1234)
        gfcuda.TwoDNavierStokes.set_zeta(prob, z0)
    elif w["module"] == "MultiLayerQG":
        q0 = 1e-2 * np.random.default_rng(1234).standard_normal((w["nlayers"], w["ny"], w["nx"]))
        gfcuda.MultiLayerQG.set_q(prob, q0)
    else:
        gfcuda.SingleLayerQG.set_q(prob, np.zeros((w["ny"], w["nx"])))
    prob.set_clock(0.0, 0)


def initial_state_oracle(w):
    """The same initial condition from the oracle, for the CPU legs."""
    import gf_oracle as O
    if w["module"] == "TwoDNavierStokes":
        g = O.Grid(w["nx"])
        return O.peakedisotropicspectrum(g, 6, 0.5, mask=O.makefilter(g), seed=1234)
    if w["module"] == "MultiLayerQG":
        return 1e-2 * np.random.default_rng(1234).standard_normal((w["nlayers"], w["ny"], w["nx"]))
    return np.zeros((w["ny"], w["nx"]))


def points(w):
    return w["nx"] * w["ny"] * w.get("nlayers", 1)


def _events(n):
    import torch
    return [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(n)]


def call_plan(steps, call_steps):
    """stepforward! calls covering exactly `steps` model steps: calls of call_steps steps,
    the last one shorter when call_steps does not divide steps."""
    calls = [call_steps] * (steps // call_steps)
    if steps % call_steps:
        calls.append(steps % call_steps)
    return calls


def time_arm(w, T, steps, warmup, flush, with_e2e, precision=None, graph=True, tune=True, shape=None,
             call_steps=CALL_STEPS, tma=None):
    """Run one precision arm: `warmup` model steps, then exactly `steps` timed model steps as
    stepforward! calls of call_steps steps each (CUDA events on the legacy default stream,
    which orders with the library's blocking stream; L2 flushed before every call) -- each call
    one replay of the context's captured call_steps-step graph, as a user's stepforward! runs;
    then the same calls again with the library's per-launch events on (per-kernel times for
    the roofline; no graphs); then `steps` single-step calls (every step observed, L2 flushed
    before each), plain and with per-launch events; then one call of `steps` steps replayed
    from captured CUDA graphs of call_steps steps (one event pair); then optionally the
    end-to-end timing through the host-buffer API (`steps` single-step calls).  Every timed leg starts from the
    initial condition at t = 0 (the SingleLayerQG workload, nu = 0 and no filter, grows to the
    grid scale and overflows after ~220 steps in the reference algorithm too), so the state
    returned is the one after `steps` steps in every arm."""
    import ctypes as C
    import torch
    import gfcuda
    prob = make_problem(w, T, precision)
    set_initial_state(prob, w)
    if shape is not None:
        prob.launch_shape = shape
        if tma is not None:
            prob.tma_columns = tma
    elif tune:
        shape = prob.autotune(reps=3)  # the library's launch-shape autotuner
    prob.set_graph_steps(call_steps)
    gfcuda.stepforward(prob, warmup)
    prob.synchronize()
    lib, ctx = prob._lib, prob._ctx
    ms2 = (C.c_double * 2)()
    n2 = (C.c_int64 * 2)()
    nl = C.c_int64()

    def timed_calls(calls, profile):
        """the calls, each timed with one event pair (L2 flushed before each); profile: with
        the library's per-launch events (per-kernel times; no graphs)"""
        lib.gf_profile_read(ctx, ms2, n2, C.byref(nl))  # reset counters
        lib.gf_profile_enable(ctx, 1 if profile else 0)
        ev = _events(len(calls))
        for i, nsteps in enumerate(calls):
            flush.zero_()
            ev[i][0].record()
            prob._c(lib.gf_step(ctx, nsteps))
            ev[i][1].record()
        torch.cuda.synchronize()
        ms = sum(a.elapsed_time(b) for a, b in ev) / sum(calls)
        prob._c(lib.gf_profile_read(ctx, ms2, n2, C.byref(nl)))
        lib.gf_profile_enable(ctx, 0)
        return ms, ms2[0] / max(n2[0], 1), ms2[1] / max(n2[1], 1), nl.value

    plan = call_plan(steps, call_steps)
    set_initial_state(prob, w)
    ms, _, _, launches = timed_calls(plan, False)         # the headline: stepforward! calls as a user runs them
    set_initial_state(prob, w)
    msi, mrow, mcol, _ = timed_calls(plan, True)          # the same calls with per-launch events
    set_initial_state(prob, w)
    mso, _, _, _ = timed_calls([1] * steps, False)
    set_initial_state(prob, w)
    _, mrowo, mcolo, _ = timed_calls([1] * steps, True)
    res = {"ms_per_step": ms, "ms_row": mrow, "ms_col": mcol, "launches": launches, "call_steps": call_steps,
           "ms_per_step_instrumented": msi,
           "ms_per_step_observed": mso, "ms_row_observed": mrowo, "ms_col_observed": mcolo,
           "launch_shape": shape, "steps": steps}
    if graph:
        gfcuda.stepforward(prob, call_steps)  # captures the graph outside the timed region
        set_initial_state(prob, w)
        prob.synchronize()
        (e0, e1), = _events(1)
        flush.zero_()
        e0.record()
        prob._c(lib.gf_step(ctx, steps))
        e1.record()
        torch.cuda.synchronize()
        res["ms_per_step_graph"] = e0.elapsed_time(e1) / steps
    res["sol"] = prob.sol   # the state after the same number of steps in every arm
    if with_e2e:
        sshape = prob.spec_shape
        hin = torch.empty(int(np.prod(sshape)) * 2, dtype=torch.float32 if T == np.float32 else torch.float64,
                          pin_memory=True)
        hout = torch.empty_like(hin, pin_memory=True)
        hin_np, hout_np = hin.numpy(), hout.numpy()
        prob._c(lib.gf_get_state(ctx, hin_np.ctypes.data, 0))
        tot = 0.0
        for i in range(steps):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            prob._c(lib.gf_set_state(ctx, hin_np.ctypes.data, 0))
            prob._c(lib.gf_step(ctx, 1))
            prob._c(lib.gf_get_state(ctx, hout_np.ctypes.data, 0))
            tot += time.perf_counter() - t0
            hin_np[:] = hout_np
        res["e2e_s_per_step"] = tot / steps
        res["state_bytes"] = hin.numel() * hin.element_size()
    prob.close()
    return res


def accuracy_100_steps(w, nsteps=100):
    """FP32 and FP64 (IEEE and df64) runs of the same workload from the same initial state:
    relative L2 difference of the FP32 and df64 states from the IEEE FP64 state after
    nsteps steps (the FP64 path itself matches the FP64 oracle to 1e-12 per step)."""
    import gfcuda
    sols = {}
    for key, T, prec in (("f32", np.float32, None), ("df64", np.float64, "DF64"), ("f64", np.float64, None)):
        p = make_problem(w, T, prec)
        set_initial_state(p, w)
        gfcuda.stepforward(p, nsteps)
        sols[key] = p.sol
        p.close()
    return {"steps": nsteps, "fp32_vs_fp64": relerr(sols["f32"], sols["f64"]),
            "df64_vs_fp64": relerr(sols["df64"], sols["f64"])}


def run_decaying128(cpu=True):
    """TwoDNavierStokes decaying 128^2, nu = 0, FilteredRK4 dt = 0.005, 1000 steps from the
    peaked isotropic state (k0 = 6, E = 0.5), with zeta, energy and enstrophy read back to
    the host every 100 steps: wall time of the whole run (host outputs included) in IEEE
    FP64 and FP64-plain (df64), the FP64 CPU restatement on the same run, and the final-state
    difference from it."""
    import gfcuda
    out = {"workload": "TwoDNavierStokes 128^2 decaying, nu=0, FilteredRK4 dt=0.005, 1000 steps, zeta/E/Z "
                       "every 100 steps (gf_step_output: device rings, one host wait)"}
    sols = {}
    for key, prec in (("fp64", None), ("df64", "DF64")):
        p = gfcuda.TwoDNavierStokes.Problem("GPU", nx=128, dt=0.005, stepper="FilteredRK4", precision=prec)
        z0 = gfcuda.peakedisotropicspectrum(p.grid, 6, 0.5, mask=p.timestepper.filter, seed=1234)
        TD = gfcuda.TwoDNavierStokes
        for rep in range(2):  # the second run is timed
            TD.set_zeta(p, z0)
            p.set_clock(0.0, 0)
            p.synchronize()
            t0 = time.perf_counter()
            d, f = gfcuda.stepforward_output(p, 1000, 100, diagnostics=[TD.energy, TD.enstrophy], fields=["zeta"])
            dt = time.perf_counter() - t0
        # 1000 steps: the total in seconds equals the time per step in milliseconds
        out[key] = {"s_total": dt, "ms_per_step": dt, "E_final": float(d[-1, 0]), "Z_final": float(d[-1, 1]),
                    "outputs": int(f["zeta"].shape[0])}
        sols[key] = p.sol
        p.close()
    if cpu:
        import gf_oracle as O
        O.set_fft_workers(os.cpu_count() or 1)
        try:
            r = O.TwoDNavierStokes(nx=128, dt=0.005, stepper="FilteredRK4")
            g = r.grid
            z0 = O.peakedisotropicspectrum(g, 6, 0.5, mask=O.makefilter(g), seed=1234)
            r.set_zeta(z0)
            t0 = time.perf_counter()
            for k in range(10):
                r.stepforward(100)
                r.energy(), r.enstrophy()
                r.updatevars()
            dt = time.perf_counter() - t0
        finally:
            O.set_fft_workers(None)
        out["cpu_restatement"] = {"s_total": dt, "cores": os.cpu_count() or 1, "kind": "port"}
        out["fp64_vs_cpu_rel_l2_after_1000_steps"] = relerr(sols["fp64"], r.sol)
        out["df64_vs_cpu_rel_l2_after_1000_steps"] = relerr(sols["df64"], r.sol)
        out["speedup_fp64_vs_cpu"] = dt / out["fp64"]["s_total"]
    return out


def time_ensemble(steps, warmup, flush, tune=True):
    """The 1536-run ensemble: one batched Problem per size class (instance i of a class
    draws its forcing with seed + i), all stepped by gf_ensemble_step; each class runs on its
    own stream, concurrently.  `warmup` model steps, then exactly `steps` timed model steps
    as calls of CALL_STEPS steps with L2 flushes before each, then the same steps from one
    graph over all classes replayed."""
    import torch
    import gfcuda
    from gfcuda.core import Grid
    e = ENSEMBLE
    probs = []
    for n, B in e["classes"]:
        g = Grid(n, n, 2 * np.pi, 2 * np.pi, 1 / 3, np.float64)
        spec = gfcuda.utils.ring_forcing_spectrum(g, e["kf"], e["dkf"], e["eps"])
        probs.append(gfcuda.TwoDNavierStokes.Problem(
            "GPU", nx=n, dt=e["dt"], nu=e["nu"], nnu=e["nnu"], stepper=e["stepper"], T=np.float32, batch=B,
            forcing=gfcuda.Forcing("stochastic", spectrum=spec, seed=1000 * n)))
    # FFT radix and tiles per size class (tune=False: the built-in block-shape rule)
    shapes = [p.autotune(reps=3) for p in probs] if tune else None
    for p in probs:
        p.set_graph_steps(0)
    gfcuda.ensemble_step(probs, warmup)
    torch.cuda.synchronize()
    calls = call_plan(steps, CALL_STEPS)
    ev = _events(len(calls))
    for i, nsteps in enumerate(calls):
        flush.zero_()
        ev[i][0].record()
        gfcuda.ensemble_step(probs, nsteps)
        ev[i][1].record()
    torch.cuda.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in ev) / steps
    for p in probs:
        p.set_graph_steps(CALL_STEPS)
    gfcuda.ensemble_step(probs, CALL_STEPS)  # captures the ensemble graph
    (e0, e1), = _events(1)
    flush.zero_()
    e0.record()
    gfcuda.ensemble_step(probs, steps)
    e1.record()
    torch.cuda.synchronize()
    ms_graph = e0.elapsed_time(e1) / steps
    # the same steps through the persistent ensemble launches (one row and one column launch
    # per stage for all classes, blocks walking the work list of every class's tiles)
    gfcuda.ensemble_step(probs, CALL_STEPS, persistent=True)  # captures that graph
    (e2, e3), = _events(1)
    flush.zero_()
    e2.record()
    gfcuda.ensemble_step(probs, steps, persistent=True)
    e3.record()
    torch.cuda.synchronize()
    ms_persistent = e2.elapsed_time(e3) / steps
    E = [float(np.mean(p.diagnostics([0])[:, 0])) for p in probs]
    for p in probs:
        p.close()
    pts = sum(n * n * B for n, B in e["classes"])
    return {"ms_per_step": ms, "ms_per_step_graph": ms_graph, "ms_per_step_persistent": ms_persistent, "points": pts,
            "mean_energy": E, "launch_shapes": shapes}


def cpu_baseline(w, seconds=20.0, max_steps=5):
    """The FP64 restatement (oracle) stepping the same workload on the host cores."""
    import gf_oracle as O
    cores = os.cpu_count() or 1
    O.set_fft_workers(cores)
    try:
        if w["module"] == "TwoDNavierStokes":
            r = O.TwoDNavierStokes(nx=w["nx"], dt=w["dt"], stepper=w["stepper"])
            r.set_zeta(initial_state_oracle(w))
        else:
            g = O.Grid(w["nx"])
            spec = O.ring_forcing_spectrum(g, 14.0, 1.5, 1e-3)
            r = O.SingleLayerQG(nx=w["nx"], beta=w["beta"], mu=w["mu"], dt=w["dt"], stepper=w["stepper"],
                                forcing=O.Forcing("stochastic", spectrum=spec, seed=1234))
        r.stepforward(1)
        n, t0 = 0, time.perf_counter()
        while n < max_steps and time.perf_counter() - t0 < seconds:
            r.stepforward(1)
            n += 1
        dt = time.perf_counter() - t0
    finally:
        O.set_fft_workers(None)
    return {"value": w["nx"] * w["ny"] * n / dt, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{n} {w['stepper']} steps of {w['module']} {w['nx']}x{w['ny']} FP64 (numpy/scipy.fft "
                      f"restatement, {cores} FFT threads), {dt:.1f} s"}


def run_reference(args):
    if not is_rank0():
        return 0
    w = HEADLINE
    import gf_oracle as O
    cores = os.cpu_count() or 1
    O.set_fft_workers(cores)
    r = O.TwoDNavierStokes(nx=w["nx"], dt=w["dt"], stepper=w["stepper"])
    r.set_zeta(initial_state_oracle(w))
    r.stepforward(args.warmup)
    t0 = time.perf_counter()
    r.stepforward(args.steps)
    dt = time.perf_counter() - t0
    v = w["nx"] * w["ny"] * args.steps / dt
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "TwoDNavierStokes 2048^2 FilteredRK4 dt=5e-4 nu=0, peaked isotropic IC (k0=6, E=0.5)",
                       "nx": w["nx"], "ny": w["ny"], "stepper": w["stepper"]},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{args.steps} steps after {args.warmup} warm-up, FP64 restatement of the "
                                       f"reference (numpy/scipy.fft, {cores} threads)"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def time_adjoint(flush, T=np.float32, precision=None, reps=2):
    """Forward stepforward!(prob, 500) against gf_grad over the same 500 steps (forward
    with checkpoints + loss + reverse sweep) with device-resident gradients, CUDA events on
    the legacy default stream; best of `reps` after one untimed run of each."""
    import torch
    import gfcuda
    from gfcuda.core import Grid
    w = ADJOINT256
    g = Grid(w["nx"], w["ny"], 2 * np.pi, 2 * np.pi, 1 / 3, np.float64)
    eta = gfcuda.utils.random_topography(g, 8, 0.1, seed=3)
    p = gfcuda.SingleLayerQG.Problem("GPU", nx=w["nx"], deformation_radius=w["ell"], eta=eta, dt=w["dt"],
                                     stepper=w["stepper"], T=T, precision=precision)
    q0 = gfcuda.peakedisotropicspectrum(p.grid, 6, 0.5, seed=1234)
    gfcuda.SingleLayerQG.set_q(p, q0)
    p.autotune(reps=3)
    gfcuda.adjoint.setup(p, w["nsteps"], w["every"])
    tdt = torch.float32 if T == np.float32 else torch.float64
    dq0 = torch.empty((w["ny"], w["nx"]), dtype=tdt, device="cuda")
    deta = torch.empty_like(dq0)
    import ctypes as C
    loss = C.c_double()
    lib, ctx = p._lib, p._ctx

    def fwd():
        gfcuda.SingleLayerQG.set_q(p, q0)
        flush.zero_()
        (e0, e1), = _events(1)
        e0.record()
        p._c(lib.gf_step(ctx, w["nsteps"]))
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    def grad():
        gfcuda.SingleLayerQG.set_q(p, q0)
        flush.zero_()
        (e0, e1), = _events(1)
        e0.record()
        p._c(lib.gf_grad(ctx, 0, C.c_void_p(dq0.data_ptr()), C.c_void_p(deta.data_ptr()), None, 1))
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    fwd(), grad()
    tf = min(fwd() for _ in range(reps))
    tg = min(grad() for _ in range(reps))
    p.close()
    n = w["nsteps"]
    return {"forward_ms_per_step": tf / n, "grad_ms_per_step": tg / n,
            "adjoint_over_forward": (tg - tf) / tf, "grad_over_forward": tg / tf}


def reduce_max(dist, vals):
    """Element-wise maximum of `vals` over ranks (the slowest replica sets each time)."""
    if not dist:
        return [float(v) for v in vals]
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(v) for v in vals], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()


def whole_job(points_per_rank, world, ms_max):
    """Grid-point*steps/s of all replicas: every rank advanced points_per_rank points per
    step, and the job took the slowest rank's time."""
    return world * points_per_rank / (ms_max * 1e-3)


def roofline(w, res, cb, tag, peaks, peak_src):
    """HBM roofline of the dominant kernel of an arm: its share of the two-sweep model's
    bytes per launch (model_launch_bytes, every mode of every array once, word = half the
    complex element size) over the average duration of its launches in the timed
    stepforward! calls, timed with CUDA events on the library stream.  Beside it the exact
    byte count of what the launches touch (launch_bytes: pruned columns and modes, averaged
    over the launches of a call) and the same figures for single observed steps."""
    row_b, col_b = call_bytes(w, cb, res["call_steps"])
    dom = "col_stage" if res["ms_col"] >= res["ms_row"] else "row_nl"
    ix = 1 if dom == "col_stage" else 0
    model = model_launch_bytes(w, cb // 2)[ix]
    exact = col_b if dom == "col_stage" else row_b
    t = res["ms_col"] if dom == "col_stage" else res["ms_row"]
    ach = model / (t * 1e-3) / 1e9
    ach_exact = exact / (t * 1e-3) / 1e9
    ob = launch_bytes(w, cb, True)[ix]
    to = res["ms_col_observed"] if dom == "col_stage" else res["ms_row_observed"]
    return {"kernel": dom, "bound": "hbm", "achieved": ach, "peak": peaks["hbm_gbs"], "unit": "GB/s",
            "frac": ach / peaks["hbm_gbs"], "peak_source": peak_src, "traffic": ncu_traffic(dom, tag),
            "algorithmic_bytes_per_launch": model, "bytes_model": "two-sweep words/pt per kernel",
            "launch_ms": t, "row_ms": res["ms_row"], "col_ms": res["ms_col"], "calls_of_steps": res["call_steps"],
            "exact_bytes_per_launch": exact, "achieved_exact": ach_exact, "frac_exact": ach_exact / peaks["hbm_gbs"],
            "observed_step": {"model_bytes_per_launch": model, "exact_bytes_per_launch": ob, "launch_ms": to,
                              "achieved": model / (to * 1e-3) / 1e9,
                              "frac": model / (to * 1e-3) / 1e9 / peaks["hbm_gbs"],
                              "frac_exact": ob / (to * 1e-3) / 1e9 / peaks["hbm_gbs"]}}


def relerr(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def run_ours(args):
    import torch
    dist = dist_setup(args.gpus)
    world = dist.get_world_size() if dist else 1
    if not torch.cuda.is_available():
        raise RuntimeError("bench.py needs a GPU")
    import gfcuda
    gfcuda.load()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MiB > L2
    peaks, peak_src = measured_peaks()
    w = HEADLINE
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with Clocks() as clk:
        r32 = time_arm(w, np.float32, args.steps, args.warmup, flush, with_e2e=True)
        rdf = time_arm(w, np.float64, args.steps, args.warmup, flush, with_e2e=True, precision="DF64")
        r64 = time_arm(w, np.float64, args.steps, args.warmup, flush, with_e2e=True)
        # the workloads beside the headline: at most 200 steps per timed leg (the SingleLayerQG
        # workload as specified overflows after ~220 steps from rest)
        ks = min(args.steps, 200)
        c32 = time_arm(SLQG512, np.float32, ks, args.warmup, flush, with_e2e=False)
        cdf = time_arm(SLQG512, np.float64, ks, args.warmup, flush, with_e2e=False, precision="DF64")
        c64 = time_arm(SLQG512, np.float64, ks, args.warmup, flush, with_e2e=False)
        m32 = time_arm(MLQG1024X3, np.float32, ks, args.warmup, flush, with_e2e=False)
        mdf = time_arm(MLQG1024X3, np.float64, ks, args.warmup, flush, with_e2e=False, precision="DF64")
        ens = time_ensemble(ks, args.warmup, flush)
        adj32 = time_adjoint(flush)
        adj64 = time_adjoint(flush, np.float64)
    fp64_peak = fp64_gemm_peak_tflops()
    acc = accuracy_100_steps(w)
    acc1 = accuracy_100_steps(SLQG512)
    acc2 = accuracy_100_steps(MLQG1024X3)
    dec128 = run_decaying128(cpu=is_rank0())
    ms, msg, msdf, ms64, e2e_s, e2e_df, e2e_64, mso = reduce_max(dist, [
        r32["ms_per_step"], r32["ms_per_step_graph"], rdf["ms_per_step"], r64["ms_per_step"],
        1e3 * r32["e2e_s_per_step"], 1e3 * rdf["e2e_s_per_step"], 1e3 * r64["e2e_s_per_step"],
        r32["ms_per_step_observed"]])
    if dist:
        dist.barrier()
    if not is_rank0():
        return 0
    pts = points(w)
    value = whole_job(pts, world, ms)
    vdf = whole_job(pts, world, msdf)
    v64 = whole_job(pts, world, ms64)
    err = relerr(r32["sol"], r64["sol"])
    dferr = relerr(rdf["sol"], r64["sol"])
    cerr = relerr(c32["sol"], c64["sol"])
    cdferr = relerr(cdf["sol"], c64["sol"])
    merr = relerr(m32["sol"], mdf["sol"])
    cpu = cpu_baseline(w)
    c1p, c2p = points(SLQG512), points(MLQG1024X3)
    rf_df = roofline(w, rdf, 16, "twodns2048_df64", peaks, peak_src)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": "TwoDNavierStokes 2048^2 FilteredRK4 dt=5e-4 nu=0, peaked isotropic IC (k0=6, E=0.5)",
                   "nx": w["nx"], "ny": w["ny"], "stepper": w["stepper"], "precision": "FP32 bulk",
                   "l2": f"flushed before every timed stepforward! call of {CALL_STEPS} steps (256 MiB write)",
                   "parallelism": f"replicas x{world}", "steps_per_call": CALL_STEPS,
                   "steps_counted": "model time steps (4 FilteredRK4 stages each), timed as stepforward! "
                                    f"calls of {CALL_STEPS} steps",
                   "ms_per_step_graph": msg, "ms_per_step_instrumented": r32["ms_per_step_instrumented"],
                   "launch_shape": r32["launch_shape"]},
        "roofline": roofline(w, r32, 8, "twodns2048_fp32", peaks, peak_src),
        "roofline_step_two_sweep": step_roofline(w, ms, 4, peaks),
        "cpu_baseline": cpu,
        "e2e": {"value": whole_job(pts, world, e2e_s), "unit": UNIT, "h2d_bytes_per_step": r32["state_bytes"],
                "d2h_bytes_per_step": r32["state_bytes"]},
        "gpu_launches": r32["launches"],
        "clocks": clk.summary(int(os.environ.get("LOCAL_RANK", "0"))),
        # the same workload, every step its own stepforward!(prob, 1) call (every mode computed)
        "value_single_step_calls": whole_job(pts, world, mso), "ms_per_step_single_step_calls": mso,
        # precision-matched arms of the same workload (FP64 inputs and outputs)
        "value_fp64_plain": vdf, "ms_per_step_fp64_plain": msdf, "e2e_fp64_plain": whole_job(pts, world, e2e_df),
        "value_fp64_ieee": v64, "ms_per_step_fp64_ieee": ms64, "e2e_fp64_ieee": whole_job(pts, world, e2e_64),
        "fp32_vs_fp64_rel_l2_100_steps": acc["fp32_vs_fp64"],
        "fp64_plain": {"arithmetic": "df64 (double-float pairs, 48-bit significand, FP32 pipes)", "value": vdf,
                       "ms_per_step": msdf, "ms_per_step_graph": rdf["ms_per_step_graph"],
                       "roofline": rf_df,
                       "compute_roofline": compute_roofline(rf_df, "twodns2048_df64"),
                       "roofline_step_two_sweep": step_roofline(w, msdf, 8, peaks),
                       "e2e": {"value": whole_job(pts, world, e2e_df), "unit": UNIT},
                       "rel_l2_vs_ieee_fp64": dferr},
        "fp64_ieee": {"value": v64, "ms_per_step": ms64, "e2e": {"value": whole_job(pts, world, e2e_64), "unit": UNIT},
                      "roofline": roofline(w, r64, 16, "twodns2048_fp64", peaks, peak_src),
                      "compute_roofline": fp64_compute_roofline(w, ms64, fp64_peak),
                      "roofline_step_two_sweep": step_roofline(w, ms64, 8, peaks)},
        "fp32_over_fp64": value / vdf,
        "fp32_over_ieee_fp64": value / v64,
        "fp32_vs_fp64_rel_l2": acc["fp32_vs_fp64"],
        "fp32_vs_fp64_steps": acc["steps"],
        "df64_vs_fp64_rel_l2_100_steps": acc["df64_vs_fp64"],
        "fp32_vs_fp64_rel_l2_after_timed_steps": err,
        "states_compared_after_steps": args.steps,
        "slqg512": {"workload": "SingleLayerQG 512^2 beta=10 mu=0.01 ETDRK4 dt=0.05, stochastic ring forcing "
                                "kf=14 eps=1e-3, q0=0 (L2-resident: latency, no HBM fraction)",
                    "fp32": c1p / (c32["ms_per_step"] * 1e-3),
                    "fp64_plain_df64": c1p / (cdf["ms_per_step"] * 1e-3),
                    "fp64_ieee": c1p / (c64["ms_per_step"] * 1e-3),
                    "ms_per_step_fp32": c32["ms_per_step"], "ms_per_step_graph_fp32": c32["ms_per_step_graph"],
                    "ms_per_step_df64": cdf["ms_per_step"], "ms_per_step_fp64": c64["ms_per_step"],
                    "fp32_vs_fp64_rel_l2": cerr, "df64_vs_fp64_rel_l2": cdferr,
                    "states_compared_after_steps": ks,
                    "fp32_vs_fp64_rel_l2_100_steps": acc1["fp32_vs_fp64"],
                    "df64_vs_fp64_rel_l2_100_steps": acc1["df64_vs_fp64"]},
        "mlqg1024x3": {"workload": "MultiLayerQG 3 layers 1024^2 ETDRK4 dt=2.5e-3, H=[.2,.3,.5], "
                                   "b from rho=[4,5,5.5] (g=1), f0=1, beta=5, U=[1,.5,0], mu=0.05, q0 white noise 1e-2",
                       "points": c2p, "fp32": c2p / (m32["ms_per_step"] * 1e-3),
                       "fp64_plain_df64": c2p / (mdf["ms_per_step"] * 1e-3),
                       "ms_per_step_fp32": m32["ms_per_step"], "ms_per_step_graph_fp32": m32["ms_per_step_graph"],
                       "ms_per_step_df64": mdf["ms_per_step"],
                       "fp32_vs_df64_rel_l2": merr, "steps_compared": ks,
                       "fp32_vs_fp64_rel_l2_100_steps": acc2["fp32_vs_fp64"],
                       "df64_vs_fp64_rel_l2_100_steps": acc2["df64_vs_fp64"],
                       "roofline_fp32": roofline(MLQG1024X3, m32, 8, "mlqg1024x3_fp32", peaks, peak_src)},
        "ensemble1536": {"workload": "1536 TwoDNavierStokes runs: 1024 x 64^2 + 384 x 128^2 + 128 x 256^2, "
                                     "FilteredRK4 dt=0.01 nu=1e-4 (nnu=1), per-instance stochastic ring forcing "
                                     "kf=8 eps=1e-3, zeta0=0, FP32, three batched contexts on concurrent streams",
                         "points": ens["points"], "value": ens["points"] / (ens["ms_per_step"] * 1e-3),
                         "value_graph": ens["points"] / (ens["ms_per_step_graph"] * 1e-3),
                         "value_persistent_launch": ens["points"] / (ens["ms_per_step_persistent"] * 1e-3),
                         "ms_per_step_persistent_launch": ens["ms_per_step_persistent"],
                         "ms_per_step": ens["ms_per_step"], "ms_per_step_graph": ens["ms_per_step_graph"],
                         "mean_energy_per_class": ens["mean_energy"], "launch_shapes": ens["launch_shapes"]},
        "twodns128_decaying": dec128,
        "adjoint_slqg256": {"workload": "gradient of the final kinetic energy w.r.t. q0 and topography: "
                                        "SingleLayerQG 256^2, deformation radius 0.35, topography |k|<=8 amp 0.1, "
                                        "ETDRK4 dt=0.01, 500 steps, checkpoint every 25",
                            "fp32": adj32, "fp64": adj64,
                            "adjoint_over_forward_definition": "(gf_grad time - forward time) / forward time: the "
                            "reverse sweep (segment recomputation + transposed stages) per forward step"},
        # the same figures at the top level of the line (the small decaying run and the adjoint)
        "ms_per_step_twodns128_fp64": dec128["fp64"]["ms_per_step"],
        "ms_per_step_twodns128_df64": dec128["df64"]["ms_per_step"],
        "speedup_twodns128_fp64_vs_cpu": dec128.get("speedup_fp64_vs_cpu"),
        "adjoint_grad_over_forward_fp32": adj32["grad_over_forward"],
        "adjoint_grad_over_forward_fp64": adj64["grad_over_forward"],
    }
    print(json.dumps(line), flush=True)
    return 0


SINGLE = {"twodns2048_fp32": (HEADLINE, np.float32, None), "twodns2048_fp64": (HEADLINE, np.float64, None),
          "twodns2048_df64": (HEADLINE, np.float64, "DF64"), "slqg512_fp32": (SLQG512, np.float32, None),
          "slqg512_fp64": (SLQG512, np.float64, None), "slqg512_df64": (SLQG512, np.float64, "DF64"),
          "mlqg1024x3_fp32": (MLQG1024X3, np.float32, None), "mlqg1024x3_df64": (MLQG1024X3, np.float64, "DF64"),
          "ensemble1536_fp32": (ENSEMBLE, np.float32, None), "adjoint256_fp32": (ADJOINT256, np.float32, None),
          "adjoint256_fp64": (ADJOINT256, np.float64, None), "twodns128_fp64": (DECAY128, np.float64, None),
          "twodns128_df64": (DECAY128, np.float64, "DF64")}


def run_single(args):
    """One arm only (for profiler captures and quick checks); not the benchmark line."""
    import torch
    import gfcuda
    gfcuda.load()
    w, T, prec = SINGLE[args.single]
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    if w is ENSEMBLE:
        r = time_ensemble(args.steps, args.warmup, flush, tune=not args.no_tune)
        r["pt_steps_per_s"] = r["points"] / (r["ms_per_step"] * 1e-3)
    elif w is ADJOINT256:
        r = time_adjoint(flush, T, reps=1)
    else:
        shape = tuple(int(v) for v in args.shape.split(",")) if args.shape else None
        r = time_arm(w, T, args.steps, args.warmup, flush, with_e2e=False, precision=prec,
                     tune=not (args.no_tune or shape), shape=shape, call_steps=args.call_steps, tma=args.tma)
        r.pop("sol")
        r["pt_steps_per_s"] = points(w) / (r["ms_per_step"] * 1e-3)
    r["workload"] = args.single
    print(json.dumps(r), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200, help="model time steps timed per arm")
    ap.add_argument("--warmup", type=int, default=20, help="untimed model time steps before them")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--single", choices=sorted(SINGLE), help="time one arm only (profiling mode)")
    ap.add_argument("--no-tune", action="store_true", help="single mode: built-in block shapes, no autotuner")
    ap.add_argument("--call-steps", type=int, default=CALL_STEPS, help="single mode: steps per timed call")
    ap.add_argument("--shape", help="single mode: launch shape row_radix,row_pairs,col_radix,col_columns "
                                    "instead of the autotuner (e.g. a shape it chose, for profiling)")
    ap.add_argument("--tma", type=int, help="single mode with --shape: TMA column stage with this many columns "
                                             "per block (0: the per-thread-copy column kernel)")
    args = ap.parse_args()
    if args.single:
        return run_single(args)
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
