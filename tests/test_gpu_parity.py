"""CUDA product path against the oracle and the reference's golden outputs.

Every call goes through libtdda's C ABI.  Tolerances:
  * FFT engine / A-product, FP64: 1e-12 relative (norm-wise) -- rounding of two FFTs;
  * polarisability al: 1e-14 (device FP64 complex division against the host's);
  * A-product, FP32 convolution: 1e-5 relative;
  * FP64 solve at the reference's tolerance 1e-5: converged, |E - A P|/|E| <= 1e-5 checked
    with the oracle, P and Einternal within 2e-4 of the reference's and the iteration
    count inside the spread the reference's own count shows under rounding-level changes
    (measured: cfg 1 55-71 around the reference's 61; tests/golden/iters_spread.npz) -- the
    reference's own solve moves by O(1e-5) and several iterations under a rounding-level
    change of its product (test_oracle_golden.py);
  * FP64 solve at 1e-10: P and Einternal within 1e-9 of the reference's run at 1e-10.
"""
import numpy as np
import pytest

import oracle as O
import tdda
from conftest import golden, rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if tdda.device_count() < 1:
        pytest.skip("no CUDA device")


def _core(g, **kw):
    Nx, Ny, Nz = (int(v) for v in g["box"])
    return tdda.AProductCore(Nx, Ny, Nz, g["R"], float(g["d"]), float(g["lam"]), g["material"],
                             float(g["nback"]), **kw)


def _ocore(g, **kw):
    Nx, Ny, Nz = (int(v) for v in g["box"])
    return O.OracleCore(Nx, Ny, Nz, g["R"], float(g["d"]), float(g["lam"]), g["material"], float(g["nback"]), **kw)


@pytest.mark.parametrize("shape", [(8, 12, 10), (40, 40, 20), (5, 7, 3), (1, 16, 9), (64, 30, 14), (21, 1, 1)])
def test_fft_engine_matches_numpy(shape):
    torch = pytest.importorskip("torch")
    rng = np.random.Generator(np.random.PCG64(sum(shape)))
    a = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    for sign, ref in ((-1, np.fft.fftn(a)), (+1, np.fft.ifftn(a) * a.size)):
        t = torch.from_numpy(a.copy()).to("cuda")
        torch.cuda.synchronize()
        tdda.fft3d_device(t.data_ptr(), *shape, sign)
        out = t.cpu().numpy()
        assert rel(out, ref) <= 1e-14


def test_core_reports_reference_quantities():
    g = golden("aprod_box6x5x4.npz")
    c = _core(g)
    oc = _ocore(g)
    assert c.get_K() == oc.K
    assert np.array_equal(c.get_material(), oc.material)  # 1.0 -> 1.01 (AProductCore.cpp:21-23)
    assert c.grid == (12, 9, 7)  # smallest 7-smooth lengths >= 2N-1
    t = c.LDR_inter(10.0, 0.0, 0.0)
    assert t[0, 0] == pytest.approx(-2.01573e-3 - 1.32085e-6j, rel=1e-5)


@pytest.mark.parametrize("name", ["box6x5x4", "sparse8x7x5", "box14x12x8"])
def test_aproduct_matches_reference(name):
    g = golden(f"aprod_{name}.npz")
    c = _core(g)
    Nx, Ny, Nz = (int(v) for v in g["box"])
    m = tdda.DDAModel(c, g["nK"], float(g["E0"]), g["nE0"], g["diel_old"])
    assert rel(m.get_al(), g["al"]) <= 1e-14  # device FP64 complex division vs the host's
    for b, y, yw in zip(g["b"], g["y"], g["y_alb"]):
        assert rel(c.Aproduct(b), y) <= 1e-12
        assert rel(m.Aproductwithalb(b), yw) <= 1e-12
        assert rel(c.Aproduct(b, precision=tdda.FP32_REFINE), y) <= 1e-5


def test_aproduct_equals_direct_sum_on_odd_boxes():
    rng = np.random.Generator(np.random.PCG64(77))
    for (Nx, Ny, Nz) in ((5, 3, 7), (1, 1, 6), (9, 2, 1), (4, 4, 4)):
        R = tdda.lattice.bulk(Nx, Ny, Nz)
        c = tdda.AProductCore(Nx, Ny, Nz, R, 7.0, 480.0, np.array([1.0, 2.25]))
        b = rng.standard_normal(R.size) + 1j * rng.standard_normal(R.size)
        yd = O.aproduct_direct(R, 7.0, c.K, b)
        assert rel(c.Aproduct(b), yd) <= 1e-12


def test_aproduct_config_shapes_against_oracle():
    """Every compiled FFT length (x/y 40, 128, 160, 192; z 20, 32, 40, 48) against the oracle."""
    rng = np.random.Generator(np.random.PCG64(3))
    for idx in (1, 2, 3, 4):
        w = tdda.lattice.config(idx)
        c = tdda.AProductCore(w.Nx, w.Ny, w.Nz, w.R, w.d, w.lam, w.material)
        oc = O.OracleCore(w.Nx, w.Ny, w.Nz, w.R, w.d, w.lam, w.material, grid=c.grid, pruned=True)
        b = rng.standard_normal(w.R.size) + 1j * rng.standard_normal(w.R.size)
        y = oc.Aproduct(b)
        assert rel(c.Aproduct(b), y) <= 1e-12
        assert rel(c.Aproduct(b, precision=tdda.FP32_REFINE), y) <= 1e-5


@pytest.mark.parametrize("box,grid", [((16, 24, 32), (32, 48, 64)), ((40, 48, 28), (80, 96, 56)),
                                      ((120, 10, 10), (256, 20, 20)), ((30, 60, 12), (64, 128, 24)),
                                      ((25, 50, 25), (56, 112, 56)), ((100, 8, 8), (224, 15, 15)),
                                      ((28, 64, 16), (56, 128, 32)), ((40, 80, 20), (80, 160, 40))])
def test_rounded_up_lengths_against_oracle(box, grid):
    """Axes rounded up to the further compiled lengths (32, 48, 56, 64, 80, 96, 112, 224,
    256; z 56, 64), also as the x length beside fused (My, Mz) planes:
    products in both precisions against the oracle on the same grid, and a refined solve."""
    Nx, Ny, Nz = box
    R = tdda.lattice.bulk(Nx, Ny, Nz)
    mat = np.array([1.0, 4.0 + 0.1j])
    c = tdda.AProductCore(Nx, Ny, Nz, R, 8.0, 550.0, mat)
    assert tuple(c.grid) == grid
    oc = O.OracleCore(Nx, Ny, Nz, R, 8.0, 550.0, mat, grid=c.grid, pruned=True)
    rng = np.random.Generator(np.random.PCG64(sum(box)))
    b = rng.standard_normal(R.size) + 1j * rng.standard_normal(R.size)
    y = oc.Aproduct(b)
    assert rel(c.Aproduct(b), y) <= 1e-12
    assert rel(c.Aproduct(b, precision=tdda.FP32_REFINE), y) <= 1e-5
    rho = np.repeat(rng.random(R.size // 3), 3)
    m = tdda.DDAModel(c, (0.0, 0.0, 1.0), 1.0, (1.0, 0.0, 0.0), rho)
    info = m.solve_mixed(10000, 1e-5)
    assert info["status"] == tdda.OK and info["true_residual"] <= 1e-5


def test_xpass_tile_and_form_and_the_autotuner():
    """The FP32 x pass's z-tile changes no result (products and refined solves bit-identical,
    the captured solve steps taken again), the shared-memory form matches the oracle at the
    FP32 level, and the autotuner keeps its fastest timed candidate."""
    Nx, Ny, Nz = 64, 64, 16
    R = tdda.lattice.bulk(Nx, Ny, Nz)
    mat = np.array([1.0, 6.25 + 0.05j])
    c = tdda.AProductCore(Nx, Ny, Nz, R, 10.0, 600.0, mat)
    oc = O.OracleCore(Nx, Ny, Nz, R, 10.0, 600.0, mat, grid=c.grid, pruned=True)
    rng = np.random.Generator(np.random.PCG64(77))
    b = rng.standard_normal(R.size) + 1j * rng.standard_normal(R.size)
    y = oc.Aproduct(b)
    rho = np.repeat(rng.random(R.size // 3), 3)
    m = tdda.DDAModel(c, (0.0, 0.0, 1.0), 1.0, (1.0, 0.0, 0.0), rho)
    zero = np.zeros(R.size, np.complex128)
    out = {}
    for form, tile in ((0, 8), (0, 16), (1, 0)):
        c.set_xpass(form, tile)
        assert c.pass_names(tdda.FP32_REFINE)[2] == ("k_xpass2" if form == 0 else "k_xpass")
        yk = c.Aproduct(b, precision=tdda.FP32_REFINE)
        assert rel(yk, y) <= 1e-5
        m.InitializeP(zero)
        info = m.solve_mixed(10000, 1e-5)
        assert info["status"] == tdda.OK and info["true_residual"] <= 1e-5
        out[(form, tile)] = (yk, m.get_P(), info["inner_iterations"])
    assert np.array_equal(out[(0, 8)][0], out[(0, 16)][0])
    assert np.array_equal(out[(0, 8)][1], out[(0, 16)][1])
    assert out[(0, 8)][2] == out[(0, 16)][2]
    t = c.autotune(nrhs=1, reps=3)
    cands = t["candidates"]
    assert [(k["form"], k["tile"]) for k in cands] == [(0, 8), (0, 16), (1, 0)]
    assert all(k["ms"] > 0 for k in cands)
    fastest = min(cands, key=lambda k: k["ms"])
    assert (t["x_form"], t["x_tile"]) == (fastest["form"], fastest["tile"])
    m.InitializeP(zero)
    info = m.solve_mixed(10000, 1e-5)
    assert info["status"] == tdda.OK and info["true_residual"] <= 1e-5
    assert np.array_equal(m.get_P(), out[(t["x_form"], t["x_tile"])][1])
    with pytest.raises(tdda.TddaError):
        c.set_xpass(1, 8)
    # an x length without a two-stage plan has one candidate, the shared-memory form
    c2 = tdda.AProductCore(100, 8, 8, tdda.lattice.bulk(100, 8, 8), 8.0, 550.0, np.array([1.0, 4.0 + 0.1j]))
    t2 = c2.autotune(nrhs=1, reps=2)
    assert [(k["form"], k["tile"]) for k in t2["candidates"]] == [(1, 0)] and t2["x_form"] == 1


def test_batch_schedule_groups_and_its_autotuner():
    """Right-hand sides per launch (the batch schedule) change no result: a batched FP32+refine
    solve of 6 incidences run as one launch per pass, as groups of 4 (with a ragged last group)
    and of 1 gives bit-identical P and iteration counts; the tuner keeps its fastest candidate."""
    w = tdda.lattice.config(1)
    incs = tdda.lattice.config(3).incidences[:6]
    c = tdda.AProductCore(w.Nx, w.Ny, w.Nz, w.R, w.d, w.lam, w.material, w.nback, max_rhs=6)
    ms = [tdda.DDAModel(c, i.nK, i.E0, i.nE0, w.diel_old) for i in incs]
    zero = np.zeros(3 * w.N, np.complex128)
    out = {}
    for group in (0, 4, 1):
        c.set_batch_group(group)
        for m in ms:
            m.InitializeP(zero)
        infos = tdda.solve_batch(ms, tdda.FP32_REFINE, 10000, 1e-5)
        assert all(i["status"] == tdda.OK and i["true_residual"] <= 1e-5 for i in infos)
        out[group] = ([m.get_P() for m in ms], [i["inner_iterations"] for i in infos])
    for group in (4, 1):
        assert out[group][1] == out[0][1]
        for a, b in zip(out[group][0], out[0][0]):
            assert np.array_equal(a, b)
    t = c.autotune_batch(nrhs=6, reps=2)
    assert [k["group"] for k in t["candidates"]] == [0, 3, 1]
    assert all(k["ms"] > 0 for k in t["candidates"])
    assert t["group"] == min(t["candidates"], key=lambda k: k["ms"])["group"]
    with pytest.raises(tdda.TddaError):
        c.set_batch_group(7)
    for m in ms:
        m.close()
    c.close()


def _model(g, core):
    m = tdda.DDAModel(core, g["nK"], float(g["E0"]), g["nE0"], g["diel_old"])
    if "P0" in g:
        m.InitializeP(g["P0"])
    if "E_rhs" in g:
        m.change_E(g["E_rhs"])
    return m


def _true_residual(g, P, E):
    oc = _ocore(g)
    om = O.OracleModel(oc, g["nK"], float(g["E0"]), g["nE0"], g["diel_old"])
    return rel(om.Aproductwithalb(P), E)


@pytest.mark.parametrize("name", ["cfg1", "sparse10x9x6", "adj8x8x4"])
def test_fp64_solve_matches_reference_at_its_tolerance(name):
    g = golden(f"solve_{name}.npz")
    c = _core(g)
    m = _model(g, c)
    info = m.bicgstab(int(g["max_it"]), float(g["max_err"]))
    m.update_E_in_structure()
    assert info["status"] == tdda.OK
    assert info["error"] <= float(g["max_err"])
    it_ref = int(g["iterations"])
    # the window is the measured spread of the reference's own count under rounding-level
    # changes (its 2N-1 grid and the GPU's grid, E and 16 one-ulp perturbations of E each;
    # tests/golden/make_golden_configs.py)
    spread = golden("iters_spread.npz")[name][:, 2]
    print(f"\n{name}: GPU FP64 {m.get_ITERATION()} iterations, reference {it_ref}, "
          f"reference under rounding changes {int(spread.min())}-{int(spread.max())}")
    assert int(spread.min()) <= it_ref <= int(spread.max())
    assert int(spread.min()) <= m.get_ITERATION() <= int(spread.max())
    assert _true_residual(g, m.get_P(), m.get_E()) <= 1.5 * float(g["max_err"])
    assert rel(m.get_P(), g["P"]) <= 2e-4
    assert rel(m.get_Einternal(), g["Einternal"]) <= 2e-4


def test_fp64_solve_matches_reference_to_1e9_at_tight_tolerance():
    g = golden("solve_cfg1_tight.npz")
    c = _core(g)
    m = _model(g, c)
    info = m.bicgstab(int(g["max_it"]), float(g["max_err"]))
    m.update_E_in_structure()
    assert info["status"] == tdda.OK
    assert rel(m.get_P(), g["P"]) <= 1e-9
    assert rel(m.get_Einternal(), g["Einternal"]) <= 1e-9


def test_mixed_precision_reaches_tolerance_with_fp64_residual():
    g = golden("solve_cfg1.npz")
    c = _core(g)
    m = _model(g, c)
    info = m.solve_mixed(10000, 1e-5)
    m.update_E_in_structure()
    assert info["status"] == tdda.OK and info["outer_iterations"] >= 1
    assert info["true_residual"] <= 1e-5
    assert _true_residual(g, m.get_P(), m.get_E()) <= 1e-5
    assert rel(m.get_P(), g["P"]) <= 2e-4


@pytest.mark.parametrize("steps", [1, 2, 3, 4, 5, 6, 9])
def test_mixed_inner_steps_follow_the_reference_recurrence(steps):
    """The FP32 inner solve stopped by its step limit: the first correction after k steps
    is the reference's BiCGSTAB iterate after k iterations from P = 0 (DDAModel.cpp:164-255),
    up to FP32 rounding (tolerance 1e-3; a step applied one iteration early or late moves P
    by O(1) here).  Limits inside and at the end of the 4-step launch chunks."""
    g = golden("solve_cfg1.npz")
    c = _core(g)
    m = _model(g, c)
    info = m.solve_mixed(steps, 1e-12)
    assert info["status"] == tdda.NOT_CONVERGED
    assert info["inner_iterations"] == steps and info["outer_iterations"] == 1
    oc = _ocore(g)
    om = O.OracleModel(oc, g["nK"], float(g["E0"]), g["nE0"], g["diel_old"])
    om.bicgstab(steps, 1e-12)
    assert rel(m.get_P(), om.P) <= 1e-3


def test_mixed_residual_in_double_float_matches_the_fp64_product():
    """The refinement's residual on the 64x64x16 lattice comes from the double-float
    product (FP32 pairs, about 44 bits).  It equals |E - (A P + al P)| / |E| formed with
    the FP64 product to 1e-6 of itself: the double-float error is ~1e-13 |E|."""
    w = tdda.lattice.config(2)
    c = tdda.AProductCore(w.Nx, w.Ny, w.Nz, w.R, w.d, w.lam, w.material, w.nback)
    inc = w.incidences[0]
    m = tdda.DDAModel(c, inc.nK, inc.E0, inc.nE0, w.diel_old)
    info = m.solve_mixed(10000, 1e-5)
    assert info["status"] == tdda.OK
    E = m.get_E()
    res64 = np.linalg.norm(E - m.Aproductwithalb(m.get_P())) / np.linalg.norm(E)
    assert res64 <= 1e-5
    assert abs(info["true_residual"] - res64) <= 1e-6 * res64


def test_mixed_solve_on_a_lattice_with_holes_uses_the_double_float_residual():
    """A sphere of dipoles inside a 20x20x10 box (grid 40x40x20, a double-float grid): the
    gather and scatter go through the cell map.  The refined solve reaches tol by the
    oracle's FP64 product, and its reported residual equals that product's."""
    Nx, Ny, Nz = 20, 20, 10
    x, y, z = np.meshgrid(np.arange(Nx), np.arange(Ny), np.arange(Nz), indexing="ij")
    keep = ((x - 9.5) / 9.5) ** 2 + ((y - 9.5) / 9.5) ** 2 + ((z - 4.5) / 4.5) ** 2 <= 1.0
    R = np.stack([x[keep], y[keep], z[keep]], axis=1).astype(np.int32).ravel()
    N = R.size // 3
    rho = np.repeat(np.random.Generator(np.random.PCG64(11)).random(N), 3)
    mat = np.array([1.0, 4.0 + 0.1j])
    c = tdda.AProductCore(Nx, Ny, Nz, R, 10.0, 500.0, mat)
    assert tuple(c.grid) == (40, 40, 20)
    m = tdda.DDAModel(c, (0.0, 0.0, 1.0), 1.0, (1.0, 0.0, 0.0), rho)
    info = m.solve_mixed(10000, 1e-5)
    assert info["status"] == tdda.OK
    oc = O.OracleCore(Nx, Ny, Nz, R, 10.0, 500.0, mat, grid=c.grid)
    om = O.OracleModel(oc, (0.0, 0.0, 1.0), 1.0, (1.0, 0.0, 0.0), rho)
    E = om.E
    res = np.linalg.norm(E - om.Aproductwithalb(m.get_P())) / np.linalg.norm(E)
    assert res <= 1e-5
    assert abs(info["true_residual"] - res) <= 1e-6 * res


def test_host_launched_chunks_equal_the_device_side_loop(monkeypatch):
    """TDDA_DEVICE_LOOP=0 (cores created while it is set) launches each 4-step chunk from the
    host instead of the conditional graph node: the same kernels in the same order, so P and
    the step counts are bit-identical."""
    w = tdda.lattice.config(1)
    out = []
    for mode in ("1", "0"):
        monkeypatch.setenv("TDDA_DEVICE_LOOP", mode)
        c = tdda.AProductCore(w.Nx, w.Ny, w.Nz, w.R, w.d, w.lam, w.material, max_rhs=2)
        ms = [tdda.DDAModel(c, inc.nK, 1.0, inc.nE0, w.diel_old)
              for inc in (tdda.lattice.XPOL_Z,
                          tdda.lattice.Incidence(np.array([0.0, 0.0, 1.0]), np.array([0.0, 1.0, 0.0])))]
        infos = tdda.solve_batch(ms, tdda.FP32_REFINE, 10000, 1e-5)
        out.append(([m.get_P() for m in ms], [i["inner_iterations"] for i in infos]))
    assert out[0][1] == out[1][1]
    for a, b in zip(out[0][0], out[1][0]):
        assert np.array_equal(a, b)


def test_batch_equals_alone():
    w = tdda.lattice.config(1)
    incs = [tdda.lattice.XPOL_Z,
            tdda.lattice.Incidence(np.array([0.0, 0.0, 1.0]), np.array([0.0, 1.0, 0.0])),
            tdda.lattice.Incidence(np.array([np.sin(0.5), 0.0, np.cos(0.5)]), tdda.lattice.n_e_perp_in_xz(0.5))]
    for prec in (tdda.FP64, tdda.FP32_REFINE):
        core = tdda.AProductCore(w.Nx, w.Ny, w.Nz, w.R, w.d, w.lam, w.material, max_rhs=4)
        alone = []
        for inc in incs:
            m = tdda.DDAModel(core, inc.nK, 1.0, inc.nE0, w.diel_old)
            info = m.bicgstab(10000, 1e-5) if prec == tdda.FP64 else m.solve_mixed(10000, 1e-5)
            alone.append((m.get_P(), info))
        ms = [tdda.DDAModel(core, inc.nK, 1.0, inc.nE0, w.diel_old) for inc in incs]
        infos = tdda.solve_batch(ms, prec, 10000, 1e-5)
        for m, info, (P, ia) in zip(ms, infos, alone):
            assert info["status"] == tdda.OK
            assert info["iterations"] == ia["iterations"]
            assert np.array_equal(m.get_P(), P)


def test_zero_rhs_breaks_down_like_the_reference():
    """E = 0: r0.rl = 0 at the first loop iteration, ITERATION = 1 (DDAModel.cpp:193-215)."""
    g = golden("aprod_box6x5x4.npz")
    c = _core(g)
    m = tdda.DDAModel(c, g["nK"], float(g["E0"]), g["nE0"], g["diel_old"])
    m.change_E(np.zeros(3 * c.N, np.complex128))
    info = m.bicgstab(100, 1e-5)
    oc = _ocore(g)
    om = O.OracleModel(oc, g["nK"], float(g["E0"]), g["nE0"], g["diel_old"])
    om.change_E(np.zeros(3 * c.N, np.complex128))
    assert om.bicgstab(100, 1e-5) == O.BREAKDOWN and om.ITERATION == 1
    assert info["status"] == tdda.BREAKDOWN and m.get_ITERATION() == 1


def test_iteration_limit_keeps_previous_iteration_count():
    """Non-convergence leaves ITERATION at its previous value (DDAModel.cpp:256-259)."""
    g = golden("solve_cfg1.npz")
    c = _core(g)
    m = _model(g, c)
    info = m.bicgstab(3, 1e-5)
    assert info["status"] == tdda.NOT_CONVERGED and m.get_ITERATION() == 0
    m2 = _model(g, c)
    m2.bicgstab(10000, 1e-5)
    it = m2.get_ITERATION()
    m2.bicgstab(2, 1e-12)
    assert m2.get_ITERATION() == it


def test_densities_outside_the_material_table_are_rejected():
    """A density whose interpolation would index outside material (DDAModel.cpp:54-63)
    is refused before anything changes: 0 <= rho < len(material), NaN refused."""
    g = golden("aprod_box6x5x4.npz")
    c = _core(g)
    m = _model(g, c)
    al0 = m.get_al()
    for bad in (-0.1, 2.0, np.nan):
        d = g["diel_old"].copy()
        d[7] = bad
        with pytest.raises(tdda.TddaError):
            m.UpdateAlpha(d)
        assert np.array_equal(m.get_al(), al0)
        with pytest.raises(tdda.TddaError):
            tdda.DDAModel(c, g["nK"], float(g["E0"]), g["nE0"], d)
    d = g["diel_old"].copy()
    d[7] = np.nextafter(2.0, 0.0)  # the last density inside the table
    m.UpdateAlpha(d)
    assert np.isfinite(m.get_al()).all()


def test_update_alpha_matches_oracle():
    g = golden("aprod_box6x5x4.npz")
    c = _core(g)
    m = tdda.DDAModel(c, g["nK"], float(g["E0"]), g["nE0"], g["diel_old"])
    d2 = np.clip(g["diel_old"] * 0.5 + 0.25, 0, 1)
    m.UpdateAlpha(d2)
    om = O.OracleModel(_ocore(g), g["nK"], float(g["E0"]), g["nE0"], d2)
    assert rel(m.get_al(), om.al) <= 1e-14
    assert rel(m.get_diel(), om.diel) <= 1e-15
    m.UpdateAlphaSingle(3, 1.0)
    d3 = d2.copy()
    d3[9:12] = 1.0
    om.UpdateAlpha(d3)
    assert rel(m.get_al(), om.al) <= 1e-14
    m.reset_E()
    assert rel(m.get_E(), om.E) <= 1e-14  # device sincos against the host libm


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["cfg1", "sparse10x9x6"])
def test_point_field_matches_reference(name):
    """E at off-lattice points (tdda_model_field_at) from the reference's solved P:
    |E| against ObjPointEDDAModel::GetVal run by the reference, the components against the
    oracle's sum (ObjDDAModel.cpp:20-96)."""
    g = golden(f"field_{name}.npz")
    Nx, Ny, Nz = (int(v) for v in g["box"])
    core = tdda.AProductCore(Nx, Ny, Nz, g["R"], float(g["d"]), float(g["lam"]), g["material"], float(g["nback"]))
    m = tdda.DDAModel(core, g["nK"], float(g["E0"]), g["nE0"], g["diel_old"])
    m.InitializeP(g["P"])
    E = m.field_at(g["points"])
    absE = np.sqrt(np.sum(np.abs(E) ** 2, axis=1))
    assert np.max(np.abs(absE - g["absE"]) / g["absE"]) <= 1e-12
    oc = O.OracleCore(Nx, Ny, Nz, g["R"], float(g["d"]), float(g["lam"]), g["material"], float(g["nback"]))
    om = O.OracleModel(oc, g["nK"], float(g["E0"]), g["nE0"], g["diel_old"])
    om.InitializeP(g["P"])
    assert rel(E.ravel(), om.field_at(g["points"]).ravel()) <= 1e-12
    m.close()
    core.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["cell6x5x3", "sparse5x4x3"])
def test_periodic_aproduct_matches_reference(name):
    """tdda_core_create_periodic: the image sums on the device (AProductCore.cpp:251-536)
    against the reference's periodic A-products."""
    g = golden(f"aprodper_{name}.npz")
    Nx, Ny, Nz = (int(v) for v in g["box"])
    mm, mn, Lm, Ln = g["periodic"]
    core = tdda.AProductCore(Nx, Ny, Nz, g["R"], float(g["d"]), float(g["lam"]), g["material"], float(g["nback"]),
                             periodic=(int(mm), int(mn), float(Lm), float(Ln)))
    m = tdda.DDAModel(core, g["nK"], float(g["E0"]), g["nE0"], g["diel_old"])
    for b, y, yw in zip(g["b"], g["y"], g["y_alb"]):
        assert rel(core.Aproduct(b), y) <= 1e-12
        assert rel(core.Aproduct(b, tdda.FP32_REFINE), y) <= 1e-5
        assert rel(m.Aproductwithalb(b), yw) <= 1e-12
    m.close()
    core.close()


@pytest.mark.gpu
def test_periodic_solve_matches_oracle():
    """A BiCGSTAB solve on a periodic core, FP64 to 1e-10 and FP32+refine to 1e-5, against
    the oracle's periodic solve."""
    Nx, Ny, Nz, d, lam = 7, 6, 3, 10.0, 540.0
    R = tdda.lattice.bulk(Nx, Ny, Nz)
    rho = np.repeat(0.5 + 0.5 * np.cos(0.21 * np.arange(Nx * Ny * Nz)), 3)
    per = (4, 4, 70.0, 60.0)
    mat = np.array([1.0, 2.25 + 0.02j])
    oc = O.OracleCore(Nx, Ny, Nz, R, d, lam, mat, periodic=per)
    om = O.OracleModel(oc, [0, 0, 1], 1.0, [1, 0, 0], rho)
    assert om.bicgstab(10000, 1e-12) == O.CONVERGED
    core = tdda.AProductCore(Nx, Ny, Nz, R, d, lam, mat, periodic=per)
    for prec, tol, bound in ((tdda.FP64, 1e-10, 1e-9), (tdda.FP32_REFINE, 1e-5, 2e-4)):
        m = tdda.DDAModel(core, [0, 0, 1], 1.0, [1, 0, 0], rho)
        info = m.bicgstab(10000, tol) if prec == tdda.FP64 else m.solve_mixed(10000, tol)
        assert info["status"] == 0
        assert rel(m.get_P(), om.P) <= bound
        m.close()
    core.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["box6x5x4", "sparse7x6x4"])
def test_fcd_aproduct_matches_reference(name):
    """The FCD tensor on the device (Si/Ci tables built by k_sici_table, interpolated as
    SiCi.cpp:27-47) against the reference's FCD A-products."""
    g = golden(f"aprodfcd_{name}.npz")
    Nx, Ny, Nz = (int(v) for v in g["box"])
    core = tdda.AProductCore(Nx, Ny, Nz, g["R"], float(g["d"]), float(g["lam"]), g["material"], float(g["nback"]),
                             method="FCD")
    m = tdda.DDAModel(core, g["nK"], float(g["E0"]), g["nE0"], g["diel_old"])
    for b, y, yw in zip(g["b"], g["y"], g["y_alb"]):
        assert rel(core.Aproduct(b), y) <= 1e-12
        assert rel(core.Aproduct(b, tdda.FP32_REFINE), y) <= 1e-5
        assert rel(m.Aproductwithalb(b), yw) <= 1e-12
    m.close()
    core.close()


@pytest.mark.gpu
def test_fcd_tensor_field_and_solve_match_oracle():
    """A_dic_generator, the off-lattice field and an FP64 solve on an FCD core (periodic
    images included) against the oracle."""
    Nx, Ny, Nz, d, lam = 6, 5, 3, 12.0, 560.0
    R = tdda.lattice.bulk(Nx, Ny, Nz)
    rho = np.repeat(0.5 + 0.5 * np.sin(0.33 * np.arange(Nx * Ny * Nz)), 3)
    mat = np.array([1.0, 3.0 + 0.05j])
    oc = O.OracleCore(Nx, Ny, Nz, R, d, lam, mat, method="FCD")
    core = tdda.AProductCore(Nx, Ny, Nz, R, d, lam, mat, method="FCD")
    for p in ((12.0, 0.0, 0.0), (24.0, -12.0, 36.0), (7.3, 15.1, -3.3)):
        t = O.fcd_inter(oc.K, d, *p)
        full = np.array([[t[0], t[1], t[2]], [t[1], t[3], t[4]], [t[2], t[4], t[5]]])
        assert np.max(np.abs(core.A_dic_generator(*p) - full)) <= 1e-13 * np.max(np.abs(full))
    om = O.OracleModel(oc, [0, 0, 1], 1.0, [1, 0, 0], rho)
    assert om.bicgstab(10000, 1e-12) == O.CONVERGED
    m = tdda.DDAModel(core, [0, 0, 1], 1.0, [1, 0, 0], rho)
    assert m.bicgstab(10000, 1e-10)["status"] == 0
    assert rel(m.get_P(), om.P) <= 1e-9
    m.InitializeP(om.P)
    pts = np.array([[30.0, 24.0, 90.0], [-20.0, 10.0, 18.0]])
    assert rel(m.field_at(pts).ravel(), om.field_at(pts).ravel()) <= 1e-12
    m.close()
    core.close()
    per = (2, 2, Nx * d, Ny * d)
    opc = O.OracleCore(Nx, Ny, Nz, R, d, lam, mat, method="FCD", periodic=per)
    pcore = tdda.AProductCore(Nx, Ny, Nz, R, d, lam, mat, method="FCD", periodic=per)
    b = (np.cos(np.arange(3 * R.size // 3)) + 1j * np.sin(0.5 * np.arange(3 * R.size // 3))).astype(np.complex128)
    assert rel(pcore.Aproduct(b), opc.Aproduct(b)) <= 1e-12
    pcore.close()
