"""The bench's byte and flop counts behind the reported roofline fractions (no GPU)."""
import importlib.util
import math
import os

import pytest

from tdda import lattice

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_canonical_aproduct_bytes(bench):
    """(84 B + 48) N s: cfg 2 FP64 138.4 MB, FP32 69.2 MB; cfg 3 FP32 with 8 RHS 1.274 GB."""
    assert bench.pass_bytes_total(65536, 1, 16) == 138412032
    assert bench.pass_bytes_total(65536, 1, 8) == 69206016
    assert bench.pass_bytes_total(221184, 8, 8) == 1274019840


def test_pass_bytes_of_the_fused_kernels(bench):
    """Fused z+y kernels move the 3N vector and the 3 Nx My Mz plane; the x pass moves the
    plane in and out plus the canonical full-grid Green count, once per launch."""
    w = lattice.config(3)
    grid = (192, 192, 48)
    plane = 3 * w.Nx * 192 * 48
    green = 6 * 192 * 192 * 48
    per = bench.pass_bytes(grid, w.Nx, w.Ny, w.Nz, w.N, 8, fused=True)
    assert per == [(3 * w.N + plane) * 8, 0, (2 * plane + green) * 8, (3 * w.N + plane) * 8, 0]
    b8 = bench.pass_bytes_batch(w, grid, 8, True, 8)
    assert b8[2] == 8 * 2 * plane * 8 + green * 8 == 424673280
    assert b8[0] == 8 * (3 * w.N + plane) * 8


def test_pass_rooflines_skip_fused_slots_and_sum_the_product(bench):
    w = lattice.config(2)
    prof = [0.010, 0.002, 0.012, 0.008, 0.002]
    names = ["k_zyfwd", "-", "k_xpass2", "k_yzinv", "-"]
    passes, whole = bench.pass_rooflines(w, (128, 128, 32), prof, names, 8, True, 1, 6785.9)
    assert [p["kernel"] for p in passes] == ["k_zyfwd", "k_xpass2", "k_yzinv"]
    assert whole["avg_ms"] == pytest.approx(0.030)
    assert whole["canonical_bytes"] == 69206016
    assert whole["frac"] == pytest.approx(69206016 / 0.030e-3 / 1e9 / 6785.9)
    x = passes[1]
    assert x["algorithmic_bytes"] == 37748736
    assert x["frac"] == pytest.approx(37748736 / 0.012e-3 / 1e9 / 6785.9)


def test_fp64_flop_count(bench):
    """Six unpruned complex 3-D FFTs at 5 G log2 G plus the 72 G spectral product."""
    G = 128 * 128 * 32
    assert bench.aprod_flops((128, 128, 32)) == pytest.approx(6 * 5 * G * math.log2(G) + 72 * G)
    assert bench.aprod_flops((128, 128, 32)) / 1e6 == pytest.approx(336.5, abs=0.1)
