"""GeophysicalFlows.SurfaceQG (src/surfaceqg.jl) on libgfcuda."""
import numpy as np

from . import _abi as A
from .core import Problem as _Problem, _check_dev


class Problem(_Problem):
    """Problem(dev; nx, ny, Lx, Ly, H, nu, nnu, dt, stepper, forcing, aliased_fraction, T)
    (src/surfaceqg.jl:76-100)."""

    module = "SurfaceQG"
    field_names = {A.FIELD_Q: "b", A.FIELD_PSI: "psi", A.FIELD_U: "u", A.FIELD_V: "v"}

    def __init__(self, dev="GPU", nx=256, ny=None, Lx=2 * np.pi, Ly=None, H=np.inf, nu=0.0, nnu=1, dt=0.01,
                 stepper="RK4", forcing=None, aliased_fraction=1 / 3, T=np.float64, stream=None, precision=None, batch=1):
        _check_dev(dev)
        ny = nx if ny is None else ny
        Ly = Lx if Ly is None else Ly
        super().__init__(dict(nu=float(nu), nnu=int(nnu), H_sqg=(0.0 if np.isinf(H) else float(H))), nx, ny, Lx,
                         Ly, dt, stepper, T, aliased_fraction, forcing, stream=stream, precision=precision, batch=batch)
        self.H = H


def set_b(prob, b):
    """set_b! (src/surfaceqg.jl:356-364)"""
    prob._set_physical(A.FIELD_Q, b)


def updatevars(prob):
    prob.updatevars()


def get_streamfunction(prob):
    """src/surfaceqg.jl:372-377 (psi = irfft(psihfrombh b-hat); sign as the reference)"""
    prob.updatevars()
    return -prob.vars.psi


def _d(prob, k):
    return float(prob.diagnostics([k])[0])


def kinetic_energy(prob): return _d(prob, 0)
def buoyancy_variance(prob): return _d(prob, 1)
def total_3D_energy(prob): return _d(prob, 2)
def buoyancy_dissipation(prob): return _d(prob, 3)


def buoyancy_work(prob):
    if prob.forcing.kind is None:
        raise TypeError("buoyancy_work needs a forced problem")
    return _d(prob, 4)


# library diagnostic ids: stepforward(prob, diags, n) streams these from the device
for _f, _k in ((kinetic_energy, 0), (buoyancy_variance, 1), (total_3D_energy, 2), (buoyancy_dissipation, 3)):
    _f.diag_id = _k
