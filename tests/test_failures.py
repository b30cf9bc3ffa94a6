"""Failure paths, injected on the host: a right-hand side whose incident field holds a NaN.

No GPU fault is involved: the NaN enters through the C ABI's change_E (or a request's
incident amplitude), the solver's scalars turn NaN, and the solve of that right-hand side
stops with TDDA_ERR_NAN.  The reference iterates on NaN to its iteration limit
(DDAModel.cpp:186-255 has no finiteness test); here the stop is reported per right-hand
side, and the other right-hand sides of the same batched launches are unaffected: their
results are bit-identical to their solves alone.
"""
import time

import numpy as np
import pytest

import tdda
from tdda import lattice

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if tdda.device_count() < 1:
        pytest.skip("no CUDA device")


INCS = [lattice.XPOL_Z,
        lattice.Incidence(np.array([0.0, 0.0, 1.0]), np.array([0.0, 1.0, 0.0])),
        lattice.Incidence(np.array([np.sin(0.5), 0.0, np.cos(0.5)]), lattice.n_e_perp_in_xz(0.5))]


@pytest.mark.parametrize("precision", [tdda.FP64, tdda.FP32_REFINE])
def test_nan_right_hand_side_is_isolated_in_a_batch(precision):
    w = lattice.config(1)
    core = tdda.AProductCore(w.Nx, w.Ny, w.Nz, w.R, w.d, w.lam, w.material, max_rhs=3)
    alone = []
    for inc in INCS:
        m = tdda.DDAModel(core, inc.nK, 1.0, inc.nE0, w.diel_old)
        tdda.solve_batch([m], precision, 10000, 1e-5)
        alone.append((m.get_P(), m.last_info))
        m.close()
    ms = [tdda.DDAModel(core, inc.nK, 1.0, inc.nE0, w.diel_old) for inc in INCS]
    E = ms[1].get_E()
    E[3 * 17 + 1] = complex(np.nan, 0.0)  # one entry of dipole 17's y component
    ms[1].change_E(E)
    infos = tdda.solve_batch(ms, precision, 10000, 1e-5)
    assert infos[1]["status"] == tdda.ERR_NAN
    for k in (0, 2):
        P, ia = alone[k]
        assert infos[k]["status"] == tdda.OK and ia["status"] == tdda.OK
        assert infos[k]["iterations"] == ia["iterations"]
        assert np.array_equal(ms[k].get_P(), P)
    # the failed model is usable again once its right-hand side is restored
    ms[1].reset_E()
    ms[1].InitializeP()
    info = tdda.solve_batch([ms[1]], precision, 10000, 1e-5)[0]
    assert info["status"] == tdda.OK
    assert np.array_equal(ms[1].get_P(), alone[1][0])
    for m in ms:
        m.close()
    core.close()


@pytest.mark.parametrize("precision", [tdda.FP32_REFINE, tdda.FP32_JACOBI])
def test_zero_right_hand_side_in_a_mixed_batch(precision):
    """E = 0 in one right-hand side of a mixed-precision batch started from P = 0: the first
    inner solve starts before the first residual is read back, so the zero right-hand side
    must still end as converged with P = 0 and no steps, and the others must equal their solves
    alone, bit for bit."""
    w = lattice.config(1)
    core = tdda.AProductCore(w.Nx, w.Ny, w.Nz, w.R, w.d, w.lam, w.material, max_rhs=3)
    alone = []
    for inc in INCS:
        m = tdda.DDAModel(core, inc.nK, 1.0, inc.nE0, w.diel_old)
        tdda.solve_batch([m], precision, 10000, 1e-5)
        alone.append((m.get_P(), m.last_info))
        m.close()
    ms = [tdda.DDAModel(core, inc.nK, 1.0, inc.nE0, w.diel_old) for inc in INCS]
    ms[1].change_E(np.zeros(3 * core.N, np.complex128))
    infos = tdda.solve_batch(ms, precision, 10000, 1e-5)
    assert infos[1]["status"] == tdda.OK, infos[1]
    assert infos[1]["inner_iterations"] == 0 and infos[1]["outer_iterations"] == 0
    assert infos[1]["error"] == 0.0
    assert not np.any(ms[1].get_P())
    for k in (0, 2):
        P, ia = alone[k]
        assert infos[k]["status"] == tdda.OK
        assert infos[k]["inner_iterations"] == ia["inner_iterations"]
        assert np.array_equal(ms[k].get_P(), P)
    for m in ms:
        m.close()
    core.close()


@pytest.mark.parametrize("precision", [tdda.FP64, tdda.FP32_REFINE])
def test_server_fails_the_nan_request_and_completes_the_others(precision):
    rng = np.random.Generator(np.random.PCG64(9))
    n = 8
    R = lattice.bulk(n, n, n)
    mat = np.array([1.0, 4.0 + 0.1j])
    diel = np.repeat(rng.random(n ** 3), 3)
    good = ([0.0, 0.0, 1.0], [1.0, 0.0, 0.0], 1.0)
    bad = ([0.0, 0.0, 1.0], [0.0, 1.0, 0.0], float("nan"))
    s = tdda.Server(hbm_budget_bytes=150e9, workers=1, precision=precision, max_group=8)
    ids = [s.submit(n, n, n, R, 10.0, 500.0, mat, diel, [good]),
           s.submit(n, n, n, R, 10.0, 500.0, mat, diel, [bad]),
           s.submit(n, n, n, R, 10.0, 500.0, mat, diel, [good, bad]),
           s.submit(n, n, n, R, 10.0, 520.0, mat, diel, [good])]
    out = [s.result(i) for i in ids]
    s.close()
    assert out[0][0]["state"] == tdda.REQ_DONE and out[0][0]["status"] == tdda.OK
    assert out[3][0]["state"] == tdda.REQ_DONE and out[3][0]["status"] == tdda.OK
    for k in (1, 2):
        assert out[k][0]["state"] == tdda.REQ_FAILED and out[k][0]["status"] == tdda.ERR_NAN
    for k, lam in ((0, 500.0), (3, 520.0)):
        core = tdda.AProductCore(n, n, n, R, 10.0, lam, mat)
        m = tdda.DDAModel(core, good[0], good[2], good[1], diel)
        tdda.solve_batch([m], precision, 10000, 1e-5)
        assert np.array_equal(out[k][1][0], m.get_P())
        m.close()
        core.close()
    # the good right-hand side of the mixed request is solved like the others
    assert np.array_equal(out[2][1][0], out[0][1][0])
