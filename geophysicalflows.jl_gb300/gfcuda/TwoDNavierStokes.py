"""GeophysicalFlows.TwoDNavierStokes (src/twodnavierstokes.jl) on libgfcuda."""
import numpy as np

from . import _abi as A
from .core import Forcing, Problem as _Problem, _check_dev


class Params:
    """src/twodnavierstokes.jl:117-128"""

    def __init__(self, nu, nnu, mu=0.0, nmu=0):
        self.nu, self.nnu, self.mu, self.nmu = nu, nnu, mu, nmu

    def __eq__(self, o):
        return (self.nu, self.nnu, self.mu, self.nmu) == (o.nu, o.nnu, o.mu, o.nmu)


class Problem(_Problem):
    """Problem(dev; nx, ny, Lx, Ly, nu, nnu, mu, nmu, dt, stepper, forcing, aliased_fraction, T)
    (src/twodnavierstokes.jl:71-100).  `forcing` replaces calcF/stochastic."""

    module = "TwoDNavierStokes"
    field_names = {A.FIELD_Q: "zeta", A.FIELD_PSI: "psi", A.FIELD_U: "u", A.FIELD_V: "v"}

    def __init__(self, dev="GPU", nx=256, ny=None, Lx=2 * np.pi, Ly=None, nu=0.0, nnu=1, mu=0.0, nmu=0,
                 dt=0.01, stepper="RK4", forcing=None, aliased_fraction=1 / 3, T=np.float64, stream=None, precision=None, batch=1):
        _check_dev(dev)
        ny = nx if ny is None else ny
        Ly = Lx if Ly is None else Ly
        super().__init__(dict(nu=float(nu), nnu=int(nnu), mu=float(mu), nmu=int(nmu)), nx, ny, Lx, Ly, dt,
                         stepper, T, aliased_fraction, forcing, stream=stream, precision=precision, batch=batch)
        self.params = Params(nu, nnu, mu, nmu)


def set_zeta(prob, zeta):
    """set_ζ! (src/twodnavierstokes.jl:352-360)"""
    prob._set_physical(A.FIELD_Q, zeta)


set_ζ = set_zeta


def updatevars(prob):
    prob.updatevars()


def _d(prob, k):
    return float(prob.diagnostics([k])[0])


def energy(prob): return _d(prob, 0)
def enstrophy(prob): return _d(prob, 1)
def palinstrophy(prob): return _d(prob, 2)
def energy_dissipation_hyperviscosity(prob): return _d(prob, 3)
def energy_dissipation_hypoviscosity(prob): return _d(prob, 4)
def enstrophy_dissipation_hyperviscosity(prob): return _d(prob, 5)
def enstrophy_dissipation_hypoviscosity(prob): return _d(prob, 6)


def energy_work(prob):
    _need_forcing(prob)
    return _d(prob, 7)


def enstrophy_work(prob):
    _need_forcing(prob)
    return _d(prob, 8)


def _need_forcing(prob):
    if prob.forcing.kind is None:
        raise TypeError("work diagnostics need a forced problem")


# library diagnostic ids: stepforward(prob, diags, n) streams these from the device
for _f, _k in ((energy, 0), (enstrophy, 1), (palinstrophy, 2), (energy_dissipation_hyperviscosity, 3),
               (energy_dissipation_hypoviscosity, 4), (enstrophy_dissipation_hyperviscosity, 5),
               (enstrophy_dissipation_hypoviscosity, 6)):
    _f.diag_id = _k
