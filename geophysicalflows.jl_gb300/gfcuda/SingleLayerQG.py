"""GeophysicalFlows.SingleLayerQG (src/singlelayerqg.jl) on libgfcuda."""
import numpy as np

from . import _abi as A
from .core import Problem as _Problem, _check_dev


class Problem(_Problem):
    """Problem(dev; nx, ny, Lx, Ly, beta, deformation_radius, U, eta, nu, nnu, mu, dt, stepper,
    forcing, aliased_fraction, T) (src/singlelayerqg.jl:91-126).  U is a number or a length-ny
    profile U(y); eta is None, an (ny, nx) array or a function eta(x, y)."""

    module = "SingleLayerQG"
    field_names = {A.FIELD_Q: "q", A.FIELD_PSI: "psi", A.FIELD_U: "u", A.FIELD_V: "v"}

    def __init__(self, dev="GPU", nx=256, ny=None, Lx=2 * np.pi, Ly=None, beta=0.0, deformation_radius=np.inf,
                 U=0.0, eta=None, nu=0.0, nnu=1, mu=0.0, dt=0.01, stepper="RK4", forcing=None,
                 aliased_fraction=1 / 3, T=np.float64, stream=None, precision=None, batch=1):
        _check_dev(dev)
        ny = nx if ny is None else ny
        Ly = Lx if Ly is None else Ly
        kw = dict(beta=float(beta), nu=float(nu), nnu=int(nnu), mu=float(mu))
        ell = deformation_radius
        kw["deformation_radius"] = 0.0 if (ell is None or np.isinf(ell)) else float(ell)
        self.deformation_radius = ell
        if np.isscalar(U):
            kw["U"] = float(U)
        else:
            kw["U_y"] = np.asarray(U, dtype=np.float64).reshape(ny)
        if eta is not None:
            if callable(eta):
                x = -Lx / 2 + Lx / nx * np.arange(nx)
                y = -Ly / 2 + Ly / ny * np.arange(ny)
                X, Y = np.meshgrid(x, y, indexing="xy")
                eta = np.asarray(eta(X, Y), dtype=np.float64) * np.ones((ny, nx))
            kw["eta"] = np.asarray(eta, dtype=np.float64).reshape(ny, nx)
        super().__init__(kw, nx, ny, Lx, Ly, dt, stepper, T, aliased_fraction, forcing, stream=stream, precision=precision, batch=batch)
        self.beta, self.U, self.mu, self.nu, self.nnu = beta, U, mu, nu, nnu


def set_q(prob, q):
    """set_q! (src/singlelayerqg.jl:525-534)"""
    prob._set_physical(A.FIELD_Q, q)


def updatevars(prob):
    prob.updatevars()


def _d(prob, k):
    return float(prob.diagnostics([k])[0])


def kinetic_energy(prob): return _d(prob, 0)


def potential_energy(prob):
    ell = prob.deformation_radius
    if ell is None or np.isinf(ell):
        return 0
    return _d(prob, 1)


def energy(prob): return _d(prob, 9)
def enstrophy(prob): return _d(prob, 2)
def energy_dissipation(prob): return _d(prob, 3)
def enstrophy_dissipation(prob): return _d(prob, 4)
def energy_work(prob): return _d(prob, 5)
def enstrophy_work(prob): return _d(prob, 6)
def energy_drag(prob): return _d(prob, 7)
def enstrophy_drag(prob): return _d(prob, 8)


# library diagnostic ids: stepforward(prob, diags, n) streams these from the device
for _f, _k in ((kinetic_energy, 0), (energy, 9), (enstrophy, 2)):
    _f.diag_id = _k
