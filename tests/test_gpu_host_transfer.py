"""State transfers with page-locked host buffers.

gf_set_state / gf_get_state read or write a page-locked (pinned) caller buffer directly from
the re-pitch kernel, and pageable buffers through a copy-engine transfer into the staging
buffer; both must move exactly the same values, in every precision, for several layers and
for a batch, for a buffer that starts inside a larger pinned block, and for memory page-locked
by cudaHostRegister (read-write, and read-only for gf_set_state, which only reads it).  A
runtime error the caller left pending in its thread is not reported as the library's."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
gfcuda = pytest.importorskip("gfcuda")
from gfcuda import MultiLayerQG as ML, TwoDNavierStokes as TD  # noqa: E402
from gfcuda import stepforward  # noqa: E402
from gfcuda import _abi as A  # noqa: E402


def make(kind, T, precision):
    if kind == "twodns":
        p = TD.Problem("GPU", nx=128, ny=64, dt=1e-3, stepper="RK4", T=T, precision=precision)
    elif kind == "batch":
        p = TD.Problem("GPU", nx=64, dt=1e-3, stepper="RK4", T=T, precision=precision, batch=3)
    else:
        p = ML.Problem(3, "GPU", nx=64, f0=1.0, beta=0.1, H=[0.2, 0.3, 0.5], b=[-1.0, -1.2, -1.5],
                       U=[0.05, 0.02, 0.0], dt=1e-3, stepper="RK4", T=T, precision=precision)
    rng = np.random.default_rng(7)
    shape = p.spec_shape
    p.sol = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) * 1e-2
    stepforward(p, 3)
    return p


def pinned_view(shape, dtype, offset_bytes=0):
    """a numpy array on page-locked memory, offset_bytes into a larger pinned block"""
    n = int(np.prod(shape)) * np.dtype(dtype).itemsize
    blk = torch.empty(n + offset_bytes + 256, dtype=torch.uint8, pin_memory=True)
    a = blk.numpy()[offset_bytes:offset_bytes + n].view(dtype).reshape(shape)
    return blk, a


@pytest.mark.parametrize("kind", ["twodns", "batch", "mlqg"])
@pytest.mark.parametrize("T,precision", [(np.float32, None), (np.float64, None), (np.float64, "DF64")])
@pytest.mark.parametrize("offset", [0, 64])
def test_pinned_state_transfers_match_pageable(kind, T, precision, offset):
    p = make(kind, T, precision)
    try:
        CT = p.CT
        ref = p.sol  # pageable path
        blk, out = pinned_view(p.spec_shape, CT, offset)
        out[...] = 0
        p._c(p._lib.gf_get_state(p._ctx, out.ctypes.data, A.HOST))
        np.testing.assert_array_equal(out, ref)

        rng = np.random.default_rng(11)
        new = (rng.standard_normal(p.spec_shape) + 1j * rng.standard_normal(p.spec_shape)).astype(CT)
        blk2, src = pinned_view(p.spec_shape, CT, offset)
        src[...] = new
        p._c(p._lib.gf_set_state(p._ctx, src.ctypes.data, A.HOST))
        via_pinned = p.sol
        p.sol = new  # pageable path
        np.testing.assert_array_equal(via_pinned, p.sol)
        if precision is None:
            np.testing.assert_array_equal(via_pinned, new)
        else:  # double-float keeps 48 significand bits
            assert np.max(np.abs(via_pinned - new)) <= 1e-13 * np.max(np.abs(new))
        del blk, blk2
    finally:
        p.close()


def _register(a, flags):
    """page-lock numpy array a with cudaHostRegister(flags); False when the platform refuses"""
    rt = torch.cuda.cudart()
    if not hasattr(rt, "cudaHostRegister"):
        pytest.skip("torch's cudart binding has no cudaHostRegister")
    err = rt.cudaHostRegister(a.ctypes.data, a.nbytes, flags)
    return int(err) == 0


@pytest.mark.parametrize("T,precision", [(np.float32, None), (np.float64, "DF64")])
def test_registered_host_memory(T, precision):
    p = make("twodns", T, precision)
    rt = torch.cuda.cudart()
    try:
        ref = p.sol
        rng = np.random.default_rng(5)
        new = (rng.standard_normal(p.spec_shape) + 1j * rng.standard_normal(p.spec_shape)).astype(p.CT)
        # read-write registration: both directions
        buf = np.zeros(p.spec_shape, dtype=p.CT)
        if not _register(buf, 0):
            pytest.skip("cudaHostRegister refused")
        try:
            p._c(p._lib.gf_get_state(p._ctx, buf.ctypes.data, A.HOST))
            np.testing.assert_array_equal(buf, ref)
            buf[...] = new
            p._c(p._lib.gf_set_state(p._ctx, buf.ctypes.data, A.HOST))
            via_registered = p.sol
        finally:
            rt.cudaHostUnregister(buf.ctypes.data)
        p.sol = new
        np.testing.assert_array_equal(via_registered, p.sol)
        # read-only registration (cudaHostRegisterReadOnly = 8): gf_set_state reads it
        ro = new[::-1].copy()
        if _register(ro, 8):
            try:
                p._c(p._lib.gf_set_state(p._ctx, ro.ctypes.data, A.HOST))
                via_ro = p.sol
            finally:
                rt.cudaHostUnregister(ro.ctypes.data)
            p.sol = ro
            np.testing.assert_array_equal(via_ro, p.sol)
    finally:
        p.close()


def test_pending_runtime_error_of_the_caller_is_not_reported_as_the_librarys():
    # a refused host-side runtime call (unregistering memory that was never registered) leaves
    # a non-sticky error pending in the thread; the library's next calls must still succeed
    rt = torch.cuda.cudart()
    if not hasattr(rt, "cudaHostUnregister"):
        pytest.skip("torch's cudart binding has no cudaHostUnregister")
    p = make("twodns", np.float32, None)
    try:
        a = np.zeros(64)
        assert int(rt.cudaHostUnregister(a.ctypes.data)) != 0
        stepforward(p, 2)
        s1 = p.sol
        assert int(rt.cudaHostUnregister(a.ctypes.data)) != 0
        p.sol = s1
        np.testing.assert_array_equal(p.sol, s1)
    finally:
        p.close()
