"""Early launch of the fused FP32 pass kernels (programmatic dependent launch, TDDA_EARLY_LAUNCH):
a kernel's blocks start while the previous kernel of the stream runs, stage their twiddles, and
wait for the previous kernel's completion before they touch the grid, the vectors or the solve
states.  Only the timing changes, so every result must be bit-identical to the ordinary launch
(mode 0), for each release point: 1 (right after the wait), 2 (before the last stage) and 3 (the
default: 1 for launches of at most one block per SM, else 2).

Checked: single FP32+refine and Jacobi solves of the reference's cfg 1 lattice, the 64 x 64 x 16
lattice, and a batch of three right-hand sides; each against mode 0, bit for bit, with the same
inner and outer step counts.  The mode is read when a core is created."""
import os

import numpy as np
import pytest

import tdda
from conftest import golden
from tdda import lattice

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if tdda.device_count() < 1:
        pytest.skip("no CUDA device")


def _with_mode(mode, fn):
    old = os.environ.get("TDDA_EARLY_LAUNCH")
    os.environ["TDDA_EARLY_LAUNCH"] = str(mode)
    try:
        return fn()
    finally:
        if old is None:
            del os.environ["TDDA_EARLY_LAUNCH"]
        else:
            os.environ["TDDA_EARLY_LAUNCH"] = old


def _solve(box, R, d, lam, mat, nback, diel, incs, precision):
    c = tdda.AProductCore(*box, R, d, lam, mat, nback, max_rhs=len(incs))
    ms = [tdda.DDAModel(c, i[0], i[1], i[2], diel) for i in incs]
    infos = tdda.solve_batch(ms, precision, 10000, 1e-5)
    out = [(m.get_P(), info) for m, info in zip(ms, infos)]
    for m in ms:
        m.close()
    c.close()
    return out


def _cases():
    g = golden("solve_cfg1.npz")
    R = np.asarray(g["R"], np.int32).reshape(-1)
    box = tuple(int(v) for v in g["box"])
    cfg1 = (box, R, float(g["d"]), float(g["lam"]), g["material"], float(g["nback"]), g["diel_old"],
            [(g["nK"], float(g["E0"]), g["nE0"])])
    w = lattice.config(2)
    i0 = w.incidences[0]
    cfg2 = ((w.Nx, w.Ny, w.Nz), w.R, w.d, w.lam, w.material, w.nback, w.diel_old, [(i0.nK, i0.E0, i0.nE0)])
    rng = np.random.Generator(np.random.PCG64(11))
    Rb = lattice.bulk(20, 20, 10)
    diel = np.repeat(rng.random(Rb.size // 3), 3)
    th = [0.0, 0.3, 0.7]
    incs = [(np.array([np.sin(t), 0.0, np.cos(t)]), 1.0, lattice.n_e_perp_in_xz(t)) for t in th]
    batch = ((20, 20, 10), Rb, 10.0, 560.0, np.array([1.0, 4.0 + 0.1j]), 1.0, diel, incs)
    return {"cfg1": cfg1, "cfg2": cfg2, "batch3": batch}


@pytest.mark.parametrize("precision", [tdda.FP32_REFINE, tdda.FP32_JACOBI])
def test_early_launch_is_bit_identical_to_the_ordinary_launch(precision):
    for name, case in _cases().items():
        base = _with_mode(0, lambda: _solve(*case, precision))
        for mode in (1, 2, 3):
            got = _with_mode(mode, lambda: _solve(*case, precision))
            for k, ((P0, i0), (P1, i1)) in enumerate(zip(base, got)):
                assert i1["status"] == tdda.OK, (name, mode, k, i1)
                assert i1["inner_iterations"] == i0["inner_iterations"], (name, mode, k)
                assert i1["outer_iterations"] == i0["outer_iterations"], (name, mode, k)
                assert np.array_equal(P1, P0), (name, mode, k)
