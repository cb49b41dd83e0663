"""Reverse-mode derivative of stepforward! (the host-side counterpart of a
ChainRulesCore.rrule on stepforward!), over libgfcuda's adjoint entry points.

    loss, dq0, deta = grad(prob, nsteps, checkpoint_every=25)     # final kinetic energy
    pullback = stepforward_with_pullback(prob, nsteps)           # rrule-style
    sol0_bar, eta_bar = pullback(sol_bar)

TwoDNavierStokes, SingleLayerQG (constant U or U(y)), MultiLayerQG and SurfaceQG with ETDRK4, FilteredETDRK4,
RK4 or FilteredRK4.  The
gradients are those of the discrete step the library computes, in the Problem's precision.
"""
import ctypes as C

import numpy as np

from . import _abi as A


def setup(prob, nsteps, checkpoint_every=25, snapshots=None):
    """Allocate for nsteps steps recomputed in units of checkpoint_every steps; `snapshots`
    bounds the stored states (binomial checkpointing; default one per unit)."""
    prob._c(prob._lib.gf_adjoint_setup(prob._ctx, int(nsteps), int(checkpoint_every)))
    if snapshots is not None:
        prob._c(prob._lib.gf_adjoint_set_snapshots(prob._ctx, int(snapshots)))
    prob._adj_steps = int(nsteps)


def info(prob):
    """(units, snapshot slots, unit advances the last reverse sweep added to the forward pass)"""
    u, s, a = C.c_int32(), C.c_int32(), C.c_int64()
    prob._c(prob._lib.gf_adjoint_info(prob._ctx, C.byref(u), C.byref(s), C.byref(a)))
    return u.value, s.value, a.value


def grad(prob, nsteps=None, checkpoint_every=25, topography=None):
    """Step prob forward nsteps from its current state and return (loss, dq0, deta): the
    final kinetic energy (MultiLayerQG: the total of energies(prob)[0]) and its gradients with
    respect to the physical initial field (as given to set_q!/set_zeta!; every layer) and to
    the topography eta (SingleLayerQG, MultiLayerQG; None otherwise unless topography=True is
    asked)."""
    if nsteps is not None and getattr(prob, "_adj_steps", None) != int(nsteps):
        setup(prob, nsteps, checkpoint_every)
    g = prob.grid
    nl = getattr(prob, "nlayers", 1)
    dq0 = np.empty((nl, g.ny, g.nx) if prob.module == "MultiLayerQG" else (g.ny, g.nx), dtype=prob.T)
    want_eta = prob.module in ("SingleLayerQG", "MultiLayerQG") if topography is None else topography
    deta = np.empty((g.ny, g.nx), dtype=prob.T) if want_eta else None
    loss = C.c_double()
    prob._c(prob._lib.gf_grad(prob._ctx, A.LOSS_KINETIC_ENERGY, dq0.ctypes.data,
                              None if deta is None else deta.ctypes.data, C.byref(loss), A.HOST))
    return loss.value, dq0, deta


def stepforward_with_pullback(prob, nsteps, checkpoint_every=25):
    """stepforward!(prob, nsteps) keeping checkpoints; returns pullback(sol_bar) ->
    (sol0_bar, eta_bar), the cotangents of the initial state and (SingleLayerQG, MultiLayerQG)
    of eta."""
    setup(prob, nsteps, checkpoint_every)
    prob._c(prob._lib.gf_adjoint_forward(prob._ctx))

    def pullback(sol_bar):
        g = prob.grid
        sb = np.ascontiguousarray(np.broadcast_to(sol_bar, prob.spec_shape), dtype=prob.CT)
        s0 = np.empty(prob.spec_shape, dtype=prob.CT)
        eb = np.empty((g.ny, g.nx), dtype=prob.T) if prob.module in ("SingleLayerQG", "MultiLayerQG") else None
        prob._c(prob._lib.gf_adjoint_backward(prob._ctx, sb.ctypes.data, s0.ctypes.data,
                                              None if eb is None else eb.ctypes.data, A.HOST))
        return s0, eb

    return pullback
