"""The allocation-free forward transform gf_rfft2_noalloc, called through the C ABI with
caller-owned device buffers, must give the same spectrum as the context-based
gf_fwdtransform, on two calls in a row (the calls share the library's fixed scratch array).

This file is collected last so that a stop-at-first-failure run has already run every
other test; it passes alone in a fresh process as well."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.mark.parametrize("T,tol", [(np.float64, 1e-13), (np.float32, 2e-6)])
@pytest.mark.parametrize("nx,ny", [(512, 512), (64, 256)])
def test_rfft2_noalloc_matches_fwdtransform(lib, T, tol, nx, ny):
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    import gfcuda
    tdt = torch.float64 if T == np.float64 else torch.float32
    cdt = torch.complex128 if T == np.float64 else torch.complex64
    prec = 1 if T == np.float64 else 0
    rng = np.random.default_rng(11)
    prob = gfcuda.TwoDNavierStokes.Problem("GPU", nx=nx, ny=ny, T=T)
    for call in range(2):
        f = rng.standard_normal((ny, nx))
        ref = prob.fwdtransform(f)                        # existing entry point
        fd = torch.tensor(f, dtype=tdt, device="cuda")    # caller-owned device buffers
        out = torch.zeros((ny, nx // 2 + 1), dtype=cdt, device="cuda")
        torch.cuda.synchronize()
        rc = lib.gf_rfft2_noalloc(C.c_void_p(fd.data_ptr()), C.c_void_p(out.data_ptr()), nx, ny, prec, None)
        assert rc == 0, lib.gf_last_error(None)
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert np.linalg.norm(got - ref) <= tol * np.linalg.norm(ref), call
        assert np.linalg.norm(got - np.fft.rfft2(f)) <= tol * np.linalg.norm(ref), call
    prob.close()


_FRESH = r"""
import ctypes as C, sys
import numpy as np, torch
sys.path.insert(0, {pkg!r})
import gfcuda
lib = gfcuda.load()
# no Problem exists in this process: the call below does the device set-up itself, and it
# runs on a caller-created non-blocking stream, not the legacy default stream
st = torch.cuda.Stream()
rng = np.random.default_rng(5)
for T, tdt, cdt, prec, tol in ((np.float64, torch.float64, torch.complex128, 1, 1e-13),
                               (np.float32, torch.float32, torch.complex64, 0, 2e-6)):
    for call in range(2):
        f = rng.standard_normal((128, 256))
        with torch.cuda.stream(st):
            fd = torch.tensor(f, dtype=tdt, device="cuda")
            out = torch.zeros((128, 129), dtype=cdt, device="cuda")
        st.synchronize()
        rc = lib.gf_rfft2_noalloc(C.c_void_p(fd.data_ptr()), C.c_void_p(out.data_ptr()), 256, 128, prec,
                                  C.c_void_p(st.cuda_stream))
        assert rc == 0, lib.gf_last_error(None)
        st.synchronize()
        ref = np.fft.rfft2(f)
        err = np.linalg.norm(out.cpu().numpy() - ref) / np.linalg.norm(ref)
        assert err <= tol, (T, call, err)
print("fresh-ok")
"""


def test_rfft2_noalloc_first_call_in_a_fresh_process_on_a_nonblocking_stream():
    """The first call of a process that never built a context, made on a non-blocking
    stream: the device set-up must finish copying the twiddle tables before any kernel of
    that stream reads them."""
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    import os
    import subprocess
    import sys
    pkg = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "geophysicalflows.jl_gb300")
    r = subprocess.run([sys.executable, "-c", _FRESH.format(pkg=pkg)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and "fresh-ok" in r.stdout, r.stdout + r.stderr


def test_rfft2_noalloc_rejects_sizes_beyond_the_maximum(lib):
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    fd = torch.zeros((1024, 1024), dtype=torch.float64, device="cuda")
    out = torch.zeros((1024, 513), dtype=torch.complex128, device="cuda")
    rc = lib.gf_rfft2_noalloc(C.c_void_p(fd.data_ptr()), C.c_void_p(out.data_ptr()), 1024, 1024, 1, None)
    assert rc == -2
    assert b"GF_NOALLOC_MAX_N" in lib.gf_last_error(None)
    rc = lib.gf_rfft2_noalloc(C.c_void_p(fd.data_ptr()), C.c_void_p(out.data_ptr()), 100, 64, 1, None)
    assert rc == -2
