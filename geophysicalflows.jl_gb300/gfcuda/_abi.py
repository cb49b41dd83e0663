"""ctypes binding of libgfcuda (declarations in include/gfcuda.h)."""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "libgfcuda.so")

# enums (include/gfcuda.h)
GF_OK, GF_ERR_ARG, GF_ERR_UNSUPPORTED, GF_ERR_CUDA, GF_ERR_NOMEM, GF_ERR_STATE, GF_ERR_NOT_IMPLEMENTED = 0, -1, -2, -3, -4, -5, -6
MODULES = {"TwoDNavierStokes": 0, "SingleLayerQG": 1, "MultiLayerQG": 2, "SurfaceQG": 3, "BarotropicQGQL": 4}
STEPPERS = {"ForwardEuler": 0, "FilteredForwardEuler": 1, "RK4": 2, "FilteredRK4": 3,
            "ETDRK4": 4, "FilteredETDRK4": 5, "AB3": 6, "FilteredAB3": 7}
F32, F64, DF64 = 0, 1, 2
FORCING = {None: 0, "static": 1, "harmonic": 2, "stochastic": 3, "stochastic_phase": 4}
HOST, DEVICE = 0, 1
LOSS_KINETIC_ENERGY = 0
# int fn(double t, int64_t step, int32_t stage, void* Fh, void* user)
FORCING_FN = C.CFUNCTYPE(C.c_int, C.c_double, C.c_int64, C.c_int32, C.c_void_p, C.c_void_p)
FIELD_Q, FIELD_PSI, FIELD_U, FIELD_V = 0, 1, 2, 3
FIELD_ZETA_MEAN, FIELD_PSI_MEAN, FIELD_U_MEAN = 4, 5, 6

EXPORTS = ["gf_create", "gf_destroy", "gf_last_error", "gf_abi_version", "gf_get_dims", "gf_set_state",
           "gf_get_state", "gf_get_clock", "gf_set_clock", "gf_set_physical", "gf_step", "gf_step_diags",
           "gf_calcN", "gf_updatevars", "gf_get_field", "gf_fwdtransform", "gf_invtransform",
           "gf_diagnostics", "gf_set_forcing", "gf_synchronize", "gf_profile_enable", "gf_profile_read",
           "gf_rfft2_noalloc", "gf_get_batch", "gf_set_graph_steps", "gf_ensemble_step",
           "gf_peakedisotropicspectrum", "gf_get_filter", "gf_adjoint_setup", "gf_adjoint_forward",
           "gf_adjoint_backward", "gf_grad", "gf_autotune", "gf_set_launch_shape", "gf_get_launch_shape",
           "gf_fluxes", "gf_step_callback", "gf_adjoint_set_snapshots", "gf_adjoint_info",
           "gf_step_output", "gf_set_tma_columns", "gf_get_tma_columns", "gf_set_ensemble_mode",
           "gf_set_field_parallel", "gf_get_field_parallel"]


class gf_config(C.Structure):
    _fields_ = [
        ("module", C.c_int32), ("precision", C.c_int32), ("stepper", C.c_int32),
        ("nx", C.c_int32), ("ny", C.c_int32), ("nlayers", C.c_int32),
        ("Lx", C.c_double), ("Ly", C.c_double), ("dt", C.c_double), ("aliased_fraction", C.c_double),
        ("nu", C.c_double), ("mu", C.c_double), ("nnu", C.c_int32), ("nmu", C.c_int32),
        ("beta", C.c_double), ("deformation_radius", C.c_double), ("U", C.c_double),
        ("U_y", C.POINTER(C.c_double)), ("eta", C.POINTER(C.c_double)),
        ("f0", C.c_double), ("H", C.POINTER(C.c_double)), ("b", C.POINTER(C.c_double)),
        ("topographic_pv_gradient", C.c_double * 2), ("linear", C.c_int32),
        ("H_sqg", C.c_double),
        ("forcing_kind", C.c_int32), ("seed", C.c_uint64), ("forcing_omega", C.c_double), ("forcing_phase", C.c_double),
        ("filter_order", C.c_double), ("filter_innerK", C.c_double), ("filter_outerK", C.c_double),
        ("etdrk4_ncirc", C.c_int32), ("etdrk4_rcirc", C.c_double),
        ("batch", C.c_int32),
    ]


_lib = None


def load(path=None):
    """Load libgfcuda.so (built in-tree; GFCUDA_LIB may name another build of it, e.g. a
    variant compiled with different tuning macros).  Raises if it is missing: there is no
    fallback."""
    global _lib
    path = path or os.environ.get("GFCUDA_LIB") or LIBPATH
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"libgfcuda.so not built ({path}); run __graft_entry__.build()")
    lib = C.CDLL(path)
    vp, i32, i64, dbl = C.c_void_p, C.c_int32, C.c_int64, C.c_double
    sig = {
        "gf_create": ([C.POINTER(gf_config), vp, C.POINTER(vp)], C.c_int),
        "gf_destroy": ([vp], C.c_int),
        "gf_last_error": ([vp], C.c_char_p),
        "gf_abi_version": ([], C.c_int),
        "gf_get_dims": ([vp, C.POINTER(i32), C.POINTER(i32), C.POINTER(i32), C.POINTER(i32)], C.c_int),
        "gf_set_state": ([vp, vp, C.c_int], C.c_int),
        "gf_get_state": ([vp, vp, C.c_int], C.c_int),
        "gf_get_clock": ([vp, C.POINTER(dbl), C.POINTER(i64)], C.c_int),
        "gf_set_clock": ([vp, dbl, i64], C.c_int),
        "gf_set_physical": ([vp, C.c_int, vp, C.c_int], C.c_int),
        "gf_step": ([vp, i64], C.c_int),
        "gf_step_diags": ([vp, i64, C.POINTER(i32), i32, C.POINTER(dbl)], C.c_int),
        "gf_calcN": ([vp, vp, vp, dbl, C.c_int], C.c_int),
        "gf_updatevars": ([vp], C.c_int),
        "gf_get_field": ([vp, C.c_int, vp, C.c_int], C.c_int),
        "gf_fwdtransform": ([vp, vp, vp, C.c_int], C.c_int),
        "gf_invtransform": ([vp, vp, vp, C.c_int], C.c_int),
        "gf_diagnostics": ([vp, C.POINTER(i32), i32, C.POINTER(dbl)], C.c_int),
        "gf_set_forcing": ([vp, vp, C.c_int], C.c_int),
        "gf_synchronize": ([vp], C.c_int),
        "gf_profile_enable": ([vp, C.c_int], C.c_int),
        "gf_profile_read": ([vp, C.POINTER(dbl), C.POINTER(i64), C.POINTER(i64)], C.c_int),
        "gf_rfft2_noalloc": ([vp, vp, i32, i32, i32, vp], C.c_int),
        "gf_get_batch": ([vp, C.POINTER(i32)], C.c_int),
        "gf_set_graph_steps": ([vp, i32], C.c_int),
        "gf_ensemble_step": ([C.POINTER(vp), i32, i64], C.c_int),
        "gf_peakedisotropicspectrum": ([vp, C.c_double, C.c_double, vp, i32, C.c_uint64, vp, C.c_int], C.c_int),
        "gf_get_filter": ([vp, vp], C.c_int),
        "gf_adjoint_setup": ([vp, i64, i32], C.c_int),
        "gf_adjoint_forward": ([vp], C.c_int),
        "gf_adjoint_backward": ([vp, vp, vp, vp, C.c_int], C.c_int),
        "gf_grad": ([vp, C.c_int, vp, vp, C.POINTER(dbl), C.c_int], C.c_int),
        "gf_autotune": ([vp, i32, C.POINTER(i32)], C.c_int),
        "gf_fluxes": ([vp, vp, vp], C.c_int),
        "gf_step_callback": ([vp, i64, FORCING_FN, vp], C.c_int),
        "gf_adjoint_set_snapshots": ([vp, i32], C.c_int),
        "gf_step_output": ([vp, i64, i32, C.POINTER(i32), i32, C.POINTER(dbl), C.POINTER(i32), i32, vp], C.c_int),
        "gf_adjoint_info": ([vp, C.POINTER(i32), C.POINTER(i32), C.POINTER(i64)], C.c_int),
        "gf_set_launch_shape": ([vp, C.POINTER(i32)], C.c_int),
        "gf_get_launch_shape": ([vp, C.POINTER(i32)], C.c_int),
        "gf_set_tma_columns": ([vp, i32], C.c_int),
        "gf_get_tma_columns": ([vp, C.POINTER(i32)], C.c_int),
        "gf_set_ensemble_mode": ([vp, i32], C.c_int),
        "gf_set_field_parallel": ([vp, i32, i32, i32], C.c_int),
        "gf_get_field_parallel": ([vp, C.POINTER(i32)], C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(lib, name)
        f.argtypes, f.restype = args, res
    _lib = lib
    return lib


class GFError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"libgfcuda error {code}: {msg}")
        self.code = code


class GFNotImplemented(GFError, NotImplementedError):
    pass


def check(lib, ctx, code):
    if code != GF_OK:
        msg = lib.gf_last_error(ctx).decode(errors="replace")
        if code == GF_ERR_NOT_IMPLEMENTED:
            raise GFNotImplemented(code, msg)
        if code == GF_ERR_ARG:
            raise ValueError(msg)
        raise GFError(code, msg)
