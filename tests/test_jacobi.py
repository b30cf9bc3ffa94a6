"""FP32+refine with a Jacobi right preconditioner (TDDA_FP32_JACOBI): the inner BiCGSTAB solves
(A D^-1) y = r with D = diag(al) and corrects P by D^-1 y; the outer FP64 residual check is the
refinement's, so every result meets the tolerance by the FP64 product.  The reference runs its
BiCGSTAB unpreconditioned (DDAModel.cpp:131-260); the solution it converges to is the same, and
the tests bound the distance to the reference's own solve.

Checked: the tolerance by the oracle's FP64 product and the distance to the reference's cfg 1
solve; far fewer inner steps than the unpreconditioned FP32 solve on a lattice of random
densities (al over two decades); a batch equal to each right-hand side alone, bit for bit; a
cross-lattice batch equal to each solve alone; the served stream equal to each request alone."""
import time

import numpy as np
import pytest

import oracle as O
import tdda
from conftest import golden, rel
from tdda import lattice

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if tdda.device_count() < 1:
        pytest.skip("no CUDA device")


def _core_model(g):
    R = np.asarray(g["R"], np.int32).reshape(-1)
    Nx, Ny, Nz = (int(v) for v in g["box"])
    c = tdda.AProductCore(Nx, Ny, Nz, R, float(g["d"]), float(g["lam"]), g["material"], float(g["nback"]))
    m = tdda.DDAModel(c, g["nK"], float(g["E0"]), g["nE0"], g["diel_old"])
    return c, m


def test_jacobi_solve_meets_the_tolerance_in_fewer_steps():
    g = golden("solve_cfg1.npz")
    c, m = _core_model(g)
    [info] = tdda.solve_batch([m], tdda.FP32_JACOBI, 10000, 1e-5)
    m.update_E_in_structure()
    assert info["status"] == tdda.OK and info["true_residual"] <= 1e-5
    # the residual by the oracle's FP64 product on the same grid
    R = np.asarray(g["R"], np.int32).reshape(-1)
    Nx, Ny, Nz = (int(v) for v in g["box"])
    oc = O.OracleCore(Nx, Ny, Nz, R, float(g["d"]), float(g["lam"]), g["material"], float(g["nback"]), grid=c.grid)
    om = O.OracleModel(oc, g["nK"], float(g["E0"]), g["nE0"], g["diel_old"])
    E = m.get_E()
    res = rel(om.Aproductwithalb(m.get_P()), E)
    assert res <= 1e-5
    # the reference's own solve at tol 1e-5 is itself within ~1e-5 of the exact solution
    d_ref = rel(m.get_P(), g["P"])
    assert d_ref <= 2e-4
    # unpreconditioned FP32+refine on the same lattice
    m2 = tdda.DDAModel(c, g["nK"], float(g["E0"]), g["nE0"], g["diel_old"])
    [info2] = tdda.solve_batch([m2], tdda.FP32_REFINE, 10000, 1e-5)
    al = np.abs(m.get_al())
    print(f"\ncfg1: Jacobi {info['inner_iterations']} inner steps, plain FP32 {info2['inner_iterations']}; "
          f"|al| {al.min():.3g}..{al.max():.3g}; residual {res:.2e} (oracle), vs reference P {d_ref:.2e}")
    assert info["inner_iterations"] * 3 <= info2["inner_iterations"]
    for x in (m, m2):
        x.close()
    c.close()


def test_jacobi_batch_equals_each_right_hand_side_alone():
    w = lattice.config(1)
    incs = lattice.config(3).incidences[:3]
    keep = np.random.Generator(np.random.PCG64(9)).random(w.N) < 0.8  # a lattice with holes
    R = w.R.reshape(-1, 3)[keep].reshape(-1)
    diel = w.diel_old.reshape(-1, 3)[keep].reshape(-1)
    c = tdda.AProductCore(w.Nx, w.Ny, w.Nz, R, w.d, w.lam, w.material, w.nback, max_rhs=3)
    ms = [tdda.DDAModel(c, i.nK, i.E0, i.nE0, diel) for i in incs]
    infos = tdda.solve_batch(ms, tdda.FP32_JACOBI, 10000, 1e-5)
    assert all(i["status"] == tdda.OK and i["true_residual"] <= 1e-5 for i in infos)
    for m, info, inc in zip(ms, infos, incs):
        a = tdda.DDAModel(c, inc.nK, inc.E0, inc.nE0, diel)
        [ia] = tdda.solve_batch([a], tdda.FP32_JACOBI, 10000, 1e-5)
        assert ia["inner_iterations"] == info["inner_iterations"]
        assert np.array_equal(a.get_P(), m.get_P())
        a.close()
    for m in ms:
        m.close()
    c.close()


def test_jacobi_cross_lattice_batch_equals_each_solve_alone():
    rng = np.random.Generator(np.random.PCG64(31))
    boxes = [(20, 20, 10), (18, 19, 9), (17, 20, 10)]
    cores, models, alone = [], [], []
    for k, box in enumerate(boxes):
        n = int(np.prod(box))
        R = lattice.bulk(*box)
        mat = np.array([1.0, [2.25, 4.0 + 0.1j, 6.25 + 0.05j][k]])
        diel = np.repeat(rng.random(n), 3)
        lam = float(rng.uniform(450, 650))
        c = tdda.AProductCore(*box, R, 10.0, lam, mat)
        assert c.grid == (40, 40, 20)
        a = tdda.DDAModel(c, (0.0, 0.0, 1.0), 1.0, (1.0, 0.0, 0.0), diel)
        [ia] = tdda.solve_batch([a], tdda.FP32_JACOBI, 10000, 1e-5)
        alone.append((a.get_P(), ia))
        a.close()
        cores.append(c)
        models.append(tdda.DDAModel(c, (0.0, 0.0, 1.0), 1.0, (1.0, 0.0, 0.0), diel))
    infos = tdda.solve_multi(models, 10000, 1e-5, precision=tdda.FP32_JACOBI)
    for m, info, (P, ia) in zip(models, infos, alone):
        assert info["status"] == tdda.OK and info["inner_iterations"] == ia["inner_iterations"]
        assert np.array_equal(m.get_P(), P)
    for m in models:
        m.close()
    for c in cores:
        c.close()


def test_served_jacobi_requests_equal_each_request_alone():
    rng = np.random.Generator(np.random.PCG64(43))
    reqs = []
    for k in range(8):
        Nx, Ny, Nz = (int(v) for v in rng.integers(4, 12, 3))
        lam = float(rng.uniform(400, 800))
        em = [2.25, 4.0 + 0.1j, 6.25 + 0.05j][k % 3]
        diel = np.repeat(rng.random(Nx * Ny * Nz), 3)
        incs = [((0.0, 0.0, 1.0), (1.0, 0.0, 0.0), 1.0), ((0.0, 0.0, 1.0), (0.0, 1.0, 0.0), 1.0)][: 1 + k % 2]
        reqs.append((Nx, Ny, Nz, lam, np.array([1.0, em]), diel, incs))
    s = tdda.Server(hbm_budget_bytes=150e9, workers=3, precision=tdda.FP32_JACOBI)
    ids = []
    for Nx, Ny, Nz, lam, mat, diel, incs in reqs:
        ids.append(s.submit(Nx, Ny, Nz, lattice.bulk(Nx, Ny, Nz), 10.0, lam, mat, diel, incs))
        time.sleep(float(rng.exponential(0.002)))
    out = [s.result(i) for i in ids]
    s.close()
    for (Nx, Ny, Nz, lam, mat, diel, incs), (info, P) in zip(reqs, out):
        assert info["state"] == tdda.REQ_DONE, info
        core = tdda.AProductCore(Nx, Ny, Nz, lattice.bulk(Nx, Ny, Nz), 10.0, lam, mat, max_rhs=len(incs))
        models = [tdda.DDAModel(core, i[0], i[2], i[1], diel) for i in incs]
        tdda.solve_batch(models, tdda.FP32_JACOBI, 10000, 1e-5)
        for k, m in enumerate(models):
            assert np.array_equal(P[k], m.get_P())
            m.close()
        core.close()


def test_auto_takes_jacobi_where_al_varies():
    """TDDA_FP32_AUTO per right-hand side: Jacobi on cfg 1's random densities (|al| over two
    decades), plain FP32+refine on cfg 2's box-filtered ones (|al| within 2x); each result is
    bit-identical to the solve with the explicit choice."""
    for cfg, expect in ((1, tdda.FP32_JACOBI), (2, tdda.FP32_REFINE)):
        w = lattice.config(cfg)
        inc = w.incidences[0]
        c = tdda.AProductCore(w.Nx, w.Ny, w.Nz, w.R, w.d, w.lam, w.material, w.nback)
        out = {}
        for prec in (tdda.FP32_AUTO, expect):
            m = tdda.DDAModel(c, inc.nK, inc.E0, inc.nE0, w.diel_old)
            [info] = tdda.solve_batch([m], prec, 10000, 1e-5)
            assert info["status"] == tdda.OK and info["true_residual"] <= 1e-5
            out[prec] = (m.get_P(), info["inner_iterations"])
            m.close()
        assert out[tdda.FP32_AUTO][1] == out[expect][1]
        assert np.array_equal(out[tdda.FP32_AUTO][0], out[expect][0]), cfg
        c.close()
