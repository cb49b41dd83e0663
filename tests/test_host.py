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
