"""Cross-lattice batches (tdda_solve_multi): FP32+refine solves of different lattices that share
one FFT grid shape, with the inner solves' passes of all of them in one launch per pass kernel.

The reference solves one structure at a time with one core (main.cpp:577-598); here several
structures -- different boxes, dipole sets, spacings, wavelengths and materials -- share the
launches.  Every right-hand side reads its own lattice, cellmap and Green spectrum, and follows
the arithmetic of its own solve alone, so each result is bit-identical to that model's
tdda_model_solve_mixed.  Two grid shapes: 64 x 64 x 32 (the five-pass FP32 kernels) and
40 x 40 x 20 (the fused z+y kernels).
"""
import math

import numpy as np
import pytest

import oracle as O
import tdda
from conftest import rel
from tdda import lattice

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if tdda.device_count() < 1:
        pytest.skip("no CUDA device")


def _lattices(boxes, seed):
    """(box, R, d, lam, material, diel, incidence) per lattice: full boxes, and a box with
    holes whose dipoles are listed in a shuffled order."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    mats = [4.0 + 0.1j, 6.25 + 0.05j, 2.25 + 0.0j]
    for k, (box, holes) in enumerate(boxes):
        R = lattice.bulk(*box).reshape(-1, 3)
        if holes:
            R = R[rng.random(R.shape[0]) < 0.7]
            R = R[rng.permutation(R.shape[0])]
        R = np.ascontiguousarray(R.ravel(), np.int32)
        n = R.size // 3
        d = [10.0, 8.0, 12.0][k % 3]
        lam = float(rng.uniform(450.0, 700.0))
        diel = np.repeat(rng.random(n), 3)
        th = math.radians(15.0 * k)
        inc = lattice.Incidence(np.array([math.sin(th), 0.0, math.cos(th)]), lattice.n_e_perp_in_xz(th))
        out.append((box, R, d, lam, np.array([1.0, mats[k % 3]]), diel, inc))
    return out


@pytest.mark.parametrize("grid,boxes", [
    ((64, 64, 32), [((32, 32, 16), False), ((30, 29, 14), False), ((29, 31, 14), True), ((32, 30, 15), False)]),
    ((40, 40, 20), [((20, 20, 10), False), ((18, 19, 9), False), ((17, 20, 10), True)]),
])
def test_cross_lattice_batch_equals_each_solve_alone(grid, boxes):
    lats = _lattices(boxes, seed=sum(grid))
    cores, alone, models = [], [], []
    for (box, R, d, lam, mat, diel, inc) in lats:
        c = tdda.AProductCore(*box, R, d, lam, mat)
        assert c.grid == grid, (box, c.grid)
        m = tdda.DDAModel(c, inc.nK, inc.E0, inc.nE0, diel)
        info = m.solve_mixed(10000, 1e-5)
        assert info["status"] == tdda.OK
        alone.append((m.get_P(), info))
        m.close()
        cores.append(c)
        models.append(tdda.DDAModel(c, inc.nK, inc.E0, inc.nE0, diel))
    infos = tdda.solve_multi(models, 10000, 1e-5)
    for k, (m, info, (P, ia)) in enumerate(zip(models, infos, alone)):
        assert info["status"] == tdda.OK, (k, info)
        assert info["inner_iterations"] == ia["inner_iterations"], (k, info, ia)
        assert info["outer_iterations"] == ia["outer_iterations"]
        assert np.array_equal(m.get_P(), P), k
    # the shape is kept: a second batch in another order gives the same results
    for m in models:
        m.InitializeP()
    infos2 = tdda.solve_multi(models[::-1], 10000, 1e-5)
    for m, (P, _) in zip(models, alone):
        assert np.array_equal(m.get_P(), P)
    assert all(i["status"] == tdda.OK for i in infos2)
    # one lattice checked against the oracle's FP64 product: converged to the tolerance
    box, R, d, lam, mat, diel, inc = lats[2]
    oc = O.OracleCore(*box, R, d, lam, mat, grid=grid)
    om = O.OracleModel(oc, inc.nK, inc.E0, inc.nE0, diel)
    E = models[2].get_E()
    assert rel(om.Aproductwithalb(models[2].get_P()), E) <= 1e-5
    for m in models:
        m.close()
    for c in cores:
        c.close()


def test_cross_lattice_batch_rejects_another_grid_shape():
    a = tdda.AProductCore(20, 20, 10, lattice.bulk(20, 20, 10), 10.0, 500.0, np.array([1.0, 4.0 + 0.1j]))
    b = tdda.AProductCore(32, 32, 16, lattice.bulk(32, 32, 16), 10.0, 500.0, np.array([1.0, 4.0 + 0.1j]))
    ma = tdda.DDAModel(a, [0, 0, 1], 1.0, [1, 0, 0], np.full(3 * a.N, 0.5))
    mb = tdda.DDAModel(b, [0, 0, 1], 1.0, [1, 0, 0], np.full(3 * b.N, 0.5))
    with pytest.raises(tdda.TddaError) as e:
        tdda.solve_multi([ma, mb])
    assert e.value.status == tdda.ERR_INVALID_ARGUMENT and "grid shape" in str(e.value)
    ma.close()
    mb.close()
    a.close()
    b.close()
