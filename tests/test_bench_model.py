"""The benchmark's byte models (CPU only): the kept-mode geometry of the per-launch model
agrees with the oracle's dealias mask, the two-sweep model gives the words per point of the
reference model (2DNS FilteredRK4 64, SLQG ETDRK4 71, MLQG ETDRK4 79), and an unobserved
launch moves fewer bytes than an observed one; the transforms' flop model of the FP64 compute
roofline."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402
import gf_oracle as O  # noqa: E402


@pytest.mark.parametrize("nx,ny", [(2048, 2048), (512, 512), (1024, 1024), (128, 64), (64, 256)])
def test_kept_geometry_matches_the_dealias_mask(nx, ny):
    nkr, kcut, rows = bench.dealias_geometry(nx, ny)
    mask = O.Grid(nx, 2 * np.pi, ny, 2 * np.pi).dealias_mask()
    assert mask.shape == (ny, nkr)
    assert int(mask.sum()) == kcut * rows
    assert np.all(mask[:, kcut:] == 0) and np.all(mask[:, :kcut].sum(axis=0) == rows)


def test_two_sweep_words_per_point():
    assert bench.algorithmic_bytes(bench.HEADLINE, 4) == 256 * bench.points(bench.HEADLINE)
    assert bench.algorithmic_bytes(bench.HEADLINE, 8) == 512 * bench.points(bench.HEADLINE)
    assert bench.algorithmic_bytes(bench.SLQG512, 4) == 284 * bench.points(bench.SLQG512)
    assert bench.algorithmic_bytes(bench.MLQG1024X3, 4) == 316 * bench.points(bench.MLQG1024X3)


@pytest.mark.parametrize("w", [bench.HEADLINE, bench.SLQG512, bench.MLQG1024X3])
@pytest.mark.parametrize("cb", [8, 16])
def test_unobserved_launches_move_fewer_bytes(w, cb):
    ro, co = bench.launch_bytes(w, cb, True)
    ru, cu = bench.launch_bytes(w, cb, False)
    assert 0 < ru < ro and 0 < cu < co
    rc, cc = bench.call_bytes(w, cb, 10)
    assert ru < rc < ro and cu < cc < co
    # complex element size scales every term
    r8, c8 = bench.launch_bytes(w, 8, True)
    r16, c16 = bench.launch_bytes(w, 16, True)
    assert r16 == pytest.approx(2 * r8) and c16 > c8


def test_fft_flop_model():
    # single-step calls: every column in every stage; 5 n log2 n per complex transform
    w = bench.HEADLINE
    f = 5 * 2048 * 11
    assert bench.fft_flops_per_step(w, 1) == 4 * 5 * (1024 + 1025) * f
    # calls of 10 steps: the kept 682 columns in 9 of them
    assert bench.fft_flops_per_step(w, 10) == pytest.approx(4 * 5 * (1024 + (9 * 682 + 1025) / 10) * f)
    r = bench.fp64_compute_roofline(w, 5.0, 1.0)
    assert r["unit"] == "TFLOP/s" and r["frac"] == pytest.approx(r["achieved"])
