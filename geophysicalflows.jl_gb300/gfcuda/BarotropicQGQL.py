"""GeophysicalFlows.BarotropicQGQL (src/barotropicqgql.jl) on libgfcuda: quasi-linear
barotropic QG, the zonal mean (kr = 0) and the eddies (kr > 0) advected quasi-linearly."""
import numpy as np

from . import _abi as A
from .core import Problem as _Problem, _check_dev


class Params:
    """src/barotropicqgql.jl:121-147"""

    def __init__(self, beta, eta, mu, nu, nnu):
        self.beta, self.eta, self.mu, self.nu, self.nnu = beta, eta, mu, nu, nnu


class Problem(_Problem):
    """Problem(dev; nx, ny, Lx, Ly, beta, eta, nu, nnu, mu, dt, stepper, forcing,
    aliased_fraction, T) (src/barotropicqgql.jl:75-110).  `forcing` replaces
    calcF/stochastic.  eta is kept in params; the reference's advection does not use it."""

    module = "BarotropicQGQL"
    field_names = {A.FIELD_Q: "zeta", A.FIELD_PSI: "psi", A.FIELD_U: "u", A.FIELD_V: "v",
                   A.FIELD_ZETA_MEAN: "Zeta", A.FIELD_PSI_MEAN: "Psi", A.FIELD_U_MEAN: "U"}

    def __init__(self, dev="GPU", nx=256, ny=None, Lx=2 * np.pi, Ly=None, beta=0.0, eta=None, nu=0.0, nnu=1,
                 mu=0.0, dt=0.01, stepper="RK4", forcing=None, aliased_fraction=1 / 3, T=np.float64, stream=None,
                 precision=None, batch=1):
        _check_dev(dev)
        ny = nx if ny is None else ny
        Ly = Lx if Ly is None else Ly
        super().__init__(dict(beta=float(beta), nu=float(nu), nnu=int(nnu), mu=float(mu)), nx, ny, Lx, Ly, dt,
                         stepper, T, aliased_fraction, forcing, stream=stream, precision=precision, batch=batch)
        eta = np.zeros((ny, nx)) if eta is None else np.asarray(eta, dtype=np.float64).reshape(ny, nx)
        self.params = Params(beta, eta, mu, nu, nnu)


def set_zeta(prob, zeta):
    """set_zeta! (src/barotropicqgql.jl:409-423): sol = rfft(zeta), sol[0,0] = 0, updatevars!"""
    prob._set_physical(A.FIELD_Q, zeta)


def updatevars(prob):
    prob.updatevars()


def _d(prob, k):
    return float(prob.diagnostics([k])[0])


def energy(prob): return _d(prob, 0)
def enstrophy(prob): return _d(prob, 1)
def dissipation(prob): return _d(prob, 2)
def drag(prob): return _d(prob, 4)


def work(prob):
    if prob.forcing.kind is None:
        raise TypeError("work needs a forced problem")
    return _d(prob, 3)


# library diagnostic ids: stepforward(prob, diags, n) streams these from the device
for _f, _k in ((energy, 0), (enstrophy, 1), (dissipation, 2), (drag, 4)):
    _f.diag_id = _k
