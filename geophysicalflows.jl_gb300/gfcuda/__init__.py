"""gfcuda: GB300 (sm_103a) pseudospectral time step of GeophysicalFlows.jl behind a C ABI.

Host-side mirror of the reference's module API; every computation runs in libgfcuda.so.
"""
from . import _abi
from ._abi import load, GFError, GFNotImplemented
from .core import Diagnostic, Forcing, ensemble_step, stepforward, stepforward_output
from . import TwoDNavierStokes, SingleLayerQG, MultiLayerQG, SurfaceQG, BarotropicQGQL
from . import utils
from . import adjoint
from .utils import lambdipole, peakedisotropicspectrum

__all__ = ["load", "GFError", "GFNotImplemented", "Diagnostic", "Forcing", "ensemble_step", "stepforward", "stepforward_output", "TwoDNavierStokes",
           "SingleLayerQG", "MultiLayerQG", "SurfaceQG", "BarotropicQGQL", "utils", "adjoint", "lambdipole", "peakedisotropicspectrum"]
