"""GeophysicalFlows.MultiLayerQG (src/multilayerqg.jl) on libgfcuda."""
import numpy as np

from . import _abi as A
from .core import Problem as _Problem, _check_dev


class Problem(_Problem):
    """Problem(nlayers, dev; nx, ny, Lx, Ly, f0, beta, U, H, b, eta, topographic_pv_gradient, mu,
    nu, nnu, dt, stepper, forcing, linear, aliased_fraction, T) (src/multilayerqg.jl:87-135).
    U: a number, a length-nlayers vector (one constant per layer), a length-ny profile
    (one layer) or an (ny, nlayers) matrix, as convert_U_to_U3D (src/multilayerqg.jl:219-250)."""

    module = "MultiLayerQG"
    field_names = {A.FIELD_Q: "q", A.FIELD_PSI: "psi", A.FIELD_U: "u", A.FIELD_V: "v"}

    def __init__(self, nlayers, dev="GPU", nx=128, ny=None, Lx=2 * np.pi, Ly=None, f0=1.0, beta=0.0, U=None,
                 H=None, b=None, eta=None, topographic_pv_gradient=(0.0, 0.0), mu=0.0, nu=0.0, nnu=1, dt=0.01,
                 stepper="RK4", forcing=None, linear=False, aliased_fraction=1 / 3, T=np.float64, stream=None, precision=None, batch=1):
        _check_dev(dev)
        ny = nx if ny is None else ny
        Ly = Lx if Ly is None else Ly
        n = int(nlayers)
        H = np.full(n, 1 / n) if H is None else np.asarray(H, dtype=np.float64)
        b = -(1 + np.arange(n) / n) if b is None else np.asarray(b, dtype=np.float64)
        if U is None:
            Uy = np.zeros((n, ny))
        elif np.isscalar(U):
            Uy = np.full((n, ny), float(U))
        else:
            Ua = np.asarray(U, dtype=np.float64)
            if Ua.ndim == 1 and Ua.size == n and not (n == 1 and ny == 1):
                Uy = np.repeat(Ua[:, None], ny, axis=1)
            elif Ua.ndim == 1:
                Uy = np.repeat(Ua.reshape(1, ny), n, axis=0)
            else:
                Uy = Ua.reshape(ny, n).T.copy()
        kw = dict(f0=float(f0), beta=float(beta), H=H, b=b, U_y=np.ascontiguousarray(Uy).ravel(), mu=float(mu),
                  nu=float(nu), nnu=int(nnu), linear=int(bool(linear)),
                  topographic_pv_gradient=tuple(float(v) for v in topographic_pv_gradient))
        if eta is not None:
            kw["eta"] = np.asarray(eta, dtype=np.float64).reshape(ny, nx)
        super().__init__(kw, nx, ny, Lx, Ly, dt, stepper, T, aliased_fraction, forcing, nlayers=n, stream=stream, precision=precision, batch=batch)
        self.H, self.b, self.f0, self.Uy = H, b, f0, Uy


def set_q(prob, q):
    """set_q! (src/multilayerqg.jl:842-870)"""
    prob._set_physical(A.FIELD_Q, q)


def set_psi(prob, psi):
    """set_ψ! (src/multilayerqg.jl:872-894)"""
    prob._set_physical(A.FIELD_PSI, psi)


set_ψ = set_psi


def updatevars(prob):
    prob.updatevars()


def fwdtransform(prob, field):
    return prob.fwdtransform(field)


def invtransform(prob, fieldh):
    return prob.invtransform(fieldh)


def fluxes(prob):
    """Lateral eddy fluxes per layer and vertical eddy fluxes per interface
    (src/multilayerqg.jl:977-1022); one layer: the lateral flux only.  Batched problems:
    arrays with a leading instance axis."""
    n, B = prob.nlayers, prob.batch
    lat = np.empty((B, n))
    ver = np.empty((B, max(n - 1, 1)))
    prob._c(prob._lib.gf_fluxes(prob._ctx, lat.ctypes.data, ver.ctypes.data))
    prob._pull_vars()
    ver = ver[:, : n - 1]
    if n == 1:
        return float(lat[0, 0]) if B == 1 else lat[:, 0].copy()
    return (lat[0].copy(), ver[0].copy()) if B == 1 else (lat, ver)


def energies(prob):
    """KE per layer and PE per interface (src/multilayerqg.jl:918-951)."""
    n = prob.nlayers
    if n == 1:
        return float(prob.diagnostics([0])[0])
    v = prob.diagnostics(list(range(n)) + [8 + j for j in range(n - 1)])
    return v[:n].copy(), v[n:].copy()
