"""Host-side set-up helpers of the package (no GPU): the forcing-spectrum normalisation and
parsevalsum against the oracle."""
import numpy as np
import pytest

import gf_oracle as O
from gfcuda import utils
from gfcuda.core import Grid


@pytest.mark.parametrize("n,kf", [(64, 8.0), (128, 14.0), (96, 5.0)])
def test_ring_forcing_spectrum_matches_oracle(n, kf):
    g, go = Grid(n, n, 2 * np.pi, 2 * np.pi, 1 / 3, np.float64), O.Grid(n)
    a, b = utils.ring_forcing_spectrum(g, kf, 1.5, 1e-3), O.ring_forcing_spectrum(go, kf, 1.5, 1e-3)
    assert np.max(np.abs(a - b)) <= 1e-15 * np.max(np.abs(b))


def test_parsevalsum_matches_oracle():
    rng = np.random.default_rng(2)
    for nx, ny in ((64, 64), (63, 32)):
        g, go = Grid(nx, ny, 2 * np.pi, 3.0, 1 / 3, np.float64), O.Grid(nx, 2 * np.pi, ny, 3.0)
        fh = rng.standard_normal((ny, nx // 2 + 1)) + 1j * rng.standard_normal((ny, nx // 2 + 1))
        assert abs(utils.parsevalsum(fh, g) - O.parsevalsum(fh, go)) <= 1e-12 * abs(O.parsevalsum(fh, go))


def test_radialspectrum_slope_of_peaked_spectrum():
    """test/test_utils.jl:1-16: the radial spectrum of psi_hat for peakedisotropicspectrum
    (allones) falls off as rho^-2 for 15 < rho <= 17.5 (rtol 5e-3)"""
    from test_oracle_reference import isapprox
    g, go = Grid(128, 128, 2 * np.pi, 2 * np.pi, 1 / 3, np.float64), O.Grid(128)
    qi = O.peakedisotropicspectrum(go, 6, 0.5, allones=True)
    rho, F = utils.radialspectrum(np.fft.rfft2(qi) * go.invKrsq, g)
    sel = (rho > 15.0) & (rho <= 17.5)
    assert sel.sum() >= 5
    assert isapprox(np.abs(F[sel]) / abs(F[sel][0]), (rho[sel] / rho[sel][0]) ** -2, 5e-3)


def test_radialspectrum_of_isotropic_field():
    """an isotropic Gaussian spectrum exp(-K^2 / 2 s^2) integrates to 2 pi rho exp(-rho^2 / 2 s^2)"""
    g = Grid(128, 128, 2 * np.pi, 2 * np.pi, 1 / 3, np.float64)
    s = 6.0
    fh = np.exp(-g.Krsq / (2 * s * s))
    rho, F = utils.radialspectrum(fh, g)
    exact = 2 * np.pi * rho * np.exp(-rho ** 2 / (2 * s * s))
    sel = rho < 40
    assert np.max(np.abs(F[sel] - exact[sel])) <= 2e-2 * np.max(exact)
