"""Host-side workload generation (no GPU)."""
import math

import numpy as np

from tdda import lattice


def test_bulk_order_matches_build_a_bulk():
    R = lattice.bulk(3, 4, 5).reshape(-1, 3)
    # tools.cpp:497-510: position = z + Nz*(y + Ny*x)
    for x in range(3):
        for y in range(4):
            for z in range(5):
                assert tuple(R[z + 5 * (y + 4 * x)]) == (x, y, z)


def test_smooth_sizes_of_the_workloads():
    assert [lattice.smooth_size(2 * n - 1) for n in (20, 10, 64, 16, 96, 24, 80)] == [40, 20, 128, 32, 192, 48, 160]
    assert lattice.smooth_size(2 * 37 - 1) == 75
    assert lattice.smooth_size(1) == 1


def test_perpendicular_polarisation():
    for deg in (0, 15, 30, 45):
        th = math.radians(deg)
        nE = lattice.n_e_perp_in_xz(th)
        k = np.array([math.sin(th), 0, math.cos(th)])
        assert abs(k @ nE) < 1e-12 and abs(np.linalg.norm(nE) - 1) < 1e-12 and nE[0] >= 0


def test_configs_are_seeded_and_in_range():
    for idx in (1, 2, 3, 4):
        w = lattice.config(idx)
        w2 = lattice.config(idx)
        assert np.array_equal(w.rho, w2.rho)
        assert w.rho.min() >= 0 and w.rho.max() <= 1
        assert w.R.size == 3 * w.Nx * w.Ny * w.Nz
    assert len(lattice.config(3).incidences) == 8
    w4 = lattice.config(4).rho.reshape(80, 80, 20)
    assert np.allclose(w4, w4[::-1, :, :]) and np.allclose(w4, w4[:, ::-1, :])


def test_fft_lengths_round_up_to_compiled_lengths():
    """The core's axis lengths: the compiled length when it costs at most 25% more points."""
    assert [lattice.fft_length(n, False) for n in (20, 64, 80, 96)] == [40, 128, 160, 192]
    assert [lattice.fft_length(n, True) for n in (10, 16, 20, 24)] == [20, 32, 40, 48]
    assert lattice.fft_length(32, True) == 64        # 63 -> 64
    assert lattice.fft_length(18, False) == 40       # 35 -> 40
    assert lattice.fft_length(50, False) == 112      # 99 -> 100 -> 112
    assert lattice.fft_length(25, False) == 56 and lattice.fft_length(25, True) == 56  # 49 -> 56
    assert lattice.fft_length(100, False) == 224     # 199 -> 200 -> 224
    assert lattice.fft_length(66, False) == 160      # 131 -> 135 -> 160 (18% more)
    assert lattice.fft_length(110, False) == 224     # 219 -> 224
    assert lattice.fft_length(120, False) == 256     # 239 -> 240 -> 256
    assert lattice.fft_length(6, False) == 12 and lattice.fft_length(4, True) == 7
