"""State transfers with page-locked host buffers.

gf_set_state / gf_get_state read or write a page-locked (pinned) caller buffer directly from
the re-pitch kernel, and pageable buffers through a copy-engine transfer into the staging
buffer; both must move exactly the same values, in every precision, for several layers and
for a batch, and also for a buffer that starts inside a larger pinned block."""
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
