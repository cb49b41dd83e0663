"""CPU tests of the C ABI: the library loads, exports every declared symbol, the config
struct layout matches the header, and argument validation fails loudly before any GPU work."""
import ctypes as C
import os
import re
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gfcuda.h")


def declared_symbols():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(gf_\w+)\s*\(", txt, re.M)))


def test_library_exports_every_declared_symbol(lib):
    syms = declared_symbols()
    assert len(syms) >= 20
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    import gfcuda._abi as A
    assert sorted(A.EXPORTS) == syms


def test_abi_version(lib):
    assert lib.gf_abi_version() == 1


def test_config_struct_layout_matches_header(tmp_path):
    import gfcuda._abi as A
    fields = [f for f, _ in A.gf_config._fields_]
    src = tmp_path / "layout.c"
    body = "\n".join(f'  printf("%s %zu\\n", "{f}", offsetof(gf_config, {f}));' for f in fields)
    src.write_text(f'#include <stdio.h>\n#include <stddef.h>\n#include "gfcuda.h"\nint main(void) {{\n'
                   f'  printf("sizeof %zu\\n", sizeof(gf_config));\n{body}\n  return 0;\n}}\n')
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.dirname(HEADER), str(src), "-o", str(exe)], check=True)
    out = dict(line.split() for line in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split("\n") if line)
    assert int(out["sizeof"]) == C.sizeof(A.gf_config)
    for f in fields:
        assert int(out[f]) == getattr(A.gf_config, f).offset, f


def _cfg(**kw):
    import gfcuda._abi as A
    c = A.gf_config()
    c.module, c.precision, c.stepper = 0, A.F64, A.STEPPERS["RK4"]
    c.nx, c.ny, c.nlayers = 64, 64, 1
    c.Lx = c.Ly = 2 * np.pi
    c.dt, c.aliased_fraction = 0.01, 1 / 3
    for k, v in kw.items():
        setattr(c, k, v)
    return c


@pytest.mark.parametrize("kw,code", [
    (dict(nx=101), -2), (dict(nx=2 * 67), -2), (dict(ny=2), -2), (dict(nx=4096), -2), (dict(nx=8192, precision=0), -2),
    (dict(stepper=9), -1), (dict(module=7), -1),
    (dict(dt=0.0), -1), (dict(aliased_fraction=1.0), -1), (dict(precision=5), -1),
    (dict(module=2, nlayers=9), -2), (dict(module=0, nlayers=2), -1), (dict(forcing_kind=9), -1),
])
def test_create_rejects_bad_configs_before_touching_the_gpu(lib, kw, code):
    ctx = C.c_void_p()
    cfg = _cfg(**kw)
    assert lib.gf_create(C.byref(cfg), None, C.byref(ctx)) == code
    assert ctx.value is None
    assert lib.gf_last_error(None)


def test_null_arguments(lib):
    assert lib.gf_create(None, None, None) == -1
    assert lib.gf_step(None, 1) == -1
    assert lib.gf_destroy(None) == 0
    # launch-shape, field-parallel, TMA, ensemble and adjoint entry points refuse a null context
    out = (C.c_int32 * 4)()
    assert lib.gf_set_field_parallel(None, 4, 4, 1) == -1
    assert lib.gf_get_field_parallel(None, out) == -1
    assert lib.gf_set_tma_columns(None, 2) == -1
    assert lib.gf_set_ensemble_mode(None, 1) == -1
    assert lib.gf_set_launch_shape(None, out) == -1
    assert lib.gf_autotune(None, 2, out) == -1
    assert lib.gf_adjoint_setup(None, 10, 5) == -1
    assert lib.gf_grad(None, 0, None, None, None, 0) == -1


def test_python_mirror_validates(lib):
    import gfcuda
    with pytest.raises(ValueError):
        gfcuda.TwoDNavierStokes.Problem("CPU", nx=64)
    with pytest.raises(ValueError):
        gfcuda.TwoDNavierStokes.Problem("GPU", nx=64, stepper="RK5")
    with pytest.raises(ValueError):
        gfcuda.Forcing("magic")
