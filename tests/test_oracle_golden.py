"""The oracle (C restatement of the reference's path) against the reference's own outputs.

The fixtures under tests/golden/ were produced by the reference's sources run
unchanged (tests/golden/make_golden.py).  These tests pin the oracle before
anything is checked against it.  CPU only.
"""
import numpy as np
import pytest

import oracle as O
from conftest import golden, rel


def test_ldr_known_answer():
    """LDR_inter(10,0,0) at K=2*pi/500 (AProductCore.cpp:588-623)."""
    K = 2 * np.pi / 500.0
    t = O.ldr_inter(K, 10.0, 0.0, 0.0)
    assert t[0] == pytest.approx(-2.01573e-3 - 1.32085e-6j, rel=1e-5)
    assert t[3] == pytest.approx(9.92198e-4 - 1.31876e-6j, rel=1e-5)
    assert t[5] == pytest.approx(9.92198e-4 - 1.31876e-6j, rel=1e-5)
    assert t[1] == 0 and t[2] == 0 and t[4] == 0


def test_ldr_self_term_is_zero():
    assert np.all(O.ldr_inter(0.0125, 0.0, 0.0, 0.0) == 0)


def test_ldr_matches_reference():
    g = golden("ldr.npz")
    for p, t in zip(g["points"], g["tensors"]):
        o = O.ldr_inter(float(g["K"]), *p)
        assert np.max(np.abs(o - t)) <= 1e-15 * max(np.max(np.abs(t)), 1e-300)


@pytest.mark.parametrize("name", ["box6x5x4", "sparse8x7x5", "box14x12x8"])
def test_aproduct_matches_reference(name):
    g = golden(f"aprod_{name}.npz")
    Nx, Ny, Nz = (int(v) for v in g["box"])
    core = O.OracleCore(Nx, Ny, Nz, g["R"], float(g["d"]), float(g["lam"]), g["material"], float(g["nback"]))
    model = O.OracleModel(core, g["nK"], float(g["E0"]), g["nE0"], g["diel_old"])
    assert rel(model.al, g["al"]) <= 1e-15
    for b, y, yw in zip(g["b"], g["y"], g["y_alb"]):
        assert rel(core.Aproduct(b), y) <= 1e-14
        assert rel(model.Aproductwithalb(b), yw) <= 1e-14


@pytest.mark.parametrize("name", ["box6x5x4", "sparse8x7x5"])
def test_aproduct_equals_direct_sum(name):
    """FFT convolution == the O(N^2) sum of LDR tensors, on any grid >= 2N-1."""
    g = golden(f"aprod_{name}.npz")
    Nx, Ny, Nz = (int(v) for v in g["box"])
    b = g["b"][0]
    core = O.OracleCore(Nx, Ny, Nz, g["R"], float(g["d"]), float(g["lam"]), g["material"], float(g["nback"]))
    yd = O.aproduct_direct(g["R"], float(g["d"]), core.K, b)
    assert rel(core.Aproduct(b), yd) <= 1e-13
    for grid, pruned in (((2 * Nx, 2 * Ny, 2 * Nz), True), ((2 * Nx + 3, 2 * Ny + 1, 2 * Nz), False)):
        c2 = O.OracleCore(Nx, Ny, Nz, g["R"], float(g["d"]), float(g["lam"]), g["material"],
                          float(g["nback"]), grid=grid, pruned=pruned)
        assert rel(c2.Aproduct(b), yd) <= 1e-13


def _solve(g, grid=None, tol=None):
    Nx, Ny, Nz = (int(v) for v in g["box"])
    core = O.OracleCore(Nx, Ny, Nz, g["R"], float(g["d"]), float(g["lam"]), g["material"],
                        float(g["nback"]), grid=grid, pruned=grid is not None)
    m = O.OracleModel(core, g["nK"], float(g["E0"]), g["nE0"], g["diel_old"])
    if "P0" in g:
        m.InitializeP(g["P0"])
    if "E_rhs" in g:
        m.change_E(g["E_rhs"])
    st = m.bicgstab(int(g["max_it"]), float(tol if tol is not None else g["max_err"]))
    m.update_E_in_structure()
    return st, m


@pytest.mark.parametrize("name", ["adj8x8x4", "sparse10x9x6", "cfg1", "cfg1_tight"])
def test_solve_matches_reference(name):
    """On the reference's own grid the restated BiCGSTAB reproduces the reference's run:
    same iteration count, same printed error, P and Einternal to rounding."""
    g = golden(f"solve_{name}.npz")
    st, m = _solve(g)
    assert st == O.CONVERGED
    assert m.ITERATION == int(g["iterations"])
    assert m.Error == pytest.approx(float(g["error"]), rel=1e-5)
    assert rel(m.P, g["P"]) <= 1e-12
    assert rel(m.Einternal, g["Einternal"]) <= 1e-12


def test_solve_rounding_sensitivity():
    """Why parity at tol 1e-5 is stated against the tolerance and the 1e-9 bar is taken at
    tol 1e-10: a product that differs from the reference only in rounding (the same
    convolution on a 2N grid) moves the 1e-5 solution by O(1e-5) and the iteration count by
    several, while the 1e-10 solutions agree to better than 1e-9."""
    g = golden("solve_cfg1.npz")
    Nx, Ny, Nz = (int(v) for v in g["box"])
    st, m = _solve(g, grid=(2 * Nx, 2 * Ny, 2 * Nz))
    assert st == O.CONVERGED and m.Error <= 1e-5
    d = rel(m.P, g["P"])
    assert 1e-7 < d < 1e-4
    gt = golden("solve_cfg1_tight.npz")
    st, mt = _solve(gt, grid=(2 * Nx, 2 * Ny, 2 * Nz))
    assert st == O.CONVERGED
    assert rel(mt.P, gt["P"]) <= 1e-9
    assert rel(mt.Einternal, gt["Einternal"]) <= 1e-9


@pytest.mark.parametrize("name", ["cfg1", "sparse10x9x6"])
def test_point_field_matches_reference(name):
    """E at off-lattice points from the solved P (ObjPointEDDAModel::GetVal,
    ObjDDAModel.cpp:20-96): the restated sum reproduces the reference's |E|."""
    g = golden(f"field_{name}.npz")
    Nx, Ny, Nz = (int(v) for v in g["box"])
    core = O.OracleCore(Nx, Ny, Nz, g["R"], float(g["d"]), float(g["lam"]), g["material"], float(g["nback"]))
    m = O.OracleModel(core, g["nK"], float(g["E0"]), g["nE0"], g["diel_old"])
    m.InitializeP(g["P"])
    E = m.field_at(g["points"])
    absE = np.sqrt(np.sum(np.abs(E) ** 2, axis=1))
    assert np.max(np.abs(absE - g["absE"]) / g["absE"]) <= 1e-13


@pytest.mark.parametrize("name", ["cell6x5x3", "sparse5x4x3"])
def test_periodic_aproduct_matches_reference(name):
    """The periodic constructor's image sums (AProductCore.cpp:251-536, 573-586)."""
    g = golden(f"aprodper_{name}.npz")
    Nx, Ny, Nz = (int(v) for v in g["box"])
    mm, mn, Lm, Ln = g["periodic"]
    core = O.OracleCore(Nx, Ny, Nz, g["R"], float(g["d"]), float(g["lam"]), g["material"], float(g["nback"]),
                        periodic=(int(mm), int(mn), float(Lm), float(Ln)))
    model = O.OracleModel(core, g["nK"], float(g["E0"]), g["nE0"], g["diel_old"])
    assert rel(model.al, g["al"]) <= 1e-15
    for b, y, yw in zip(g["b"], g["y"], g["y_alb"]):
        assert rel(core.Aproduct(b), y) <= 1e-14
        assert rel(model.Aproductwithalb(b), yw) <= 1e-14


def test_sici_matches_scipy():
    """Si, Ci of the restatement (A&S series and continued fraction) against scipy's."""
    special = pytest.importorskip("scipy.special")
    xs = np.concatenate([np.linspace(0.1, 4.0, 391), np.linspace(4.0, 60.0, 561), np.geomspace(60.0, 1e5, 300)])
    S, C = special.sici(xs)
    for x, s_ref, c_ref in zip(xs, S, C):
        s, c = O.sici(float(x))
        assert abs(s - s_ref) <= 2e-15 * max(1.0, abs(s_ref))
        assert abs(c - c_ref) <= 2e-15 * max(1.0, abs(c_ref))


@pytest.mark.parametrize("name", ["box6x5x4", "sparse7x6x4"])
def test_fcd_aproduct_matches_reference(name):
    """The FCD tensor (AProductCore.cpp:625-695) with interpolated Si/Ci tables: the oracle's
    tables are its own Si/Ci at the nodes; the reference's were written by scipy, as
    SiCi/SiCi.py does."""
    g = golden(f"aprodfcd_{name}.npz")
    Nx, Ny, Nz = (int(v) for v in g["box"])
    core = O.OracleCore(Nx, Ny, Nz, g["R"], float(g["d"]), float(g["lam"]), g["material"], float(g["nback"]),
                        method="FCD")
    model = O.OracleModel(core, g["nK"], float(g["E0"]), g["nE0"], g["diel_old"])
    assert rel(model.al, g["al"]) <= 1e-15
    for b, y, yw in zip(g["b"], g["y"], g["y_alb"]):
        assert rel(core.Aproduct(b), y) <= 1e-13
        assert rel(model.Aproductwithalb(b), yw) <= 1e-13
