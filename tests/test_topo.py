"""The topology-optimisation loop (tdda/topo.py): the caller of the solve path.

CPU: the LDR tensor restated with numpy equals the oracle's; the design map's transpose
is its adjoint; dal/deps equals a finite difference of 1/alpha_LDR; the optimiser moments
follow EvoDDAModel.cpp:673-731; the projection and its beta schedule follow
FilterOption.cpp:23-62, and the reference's diagonal chain form restates gradients_filtered
(EvoDDAModel.cpp:1177-1225).  GPU: the device objective and sensitivity equal their host
restatement from the downloaded fields; the adjoint gradient (forward + 3 basis adjoints
batched) equals central finite differences of the objective, also through the projection;
gradient ascent raises the objective.
"""
import math
from types import SimpleNamespace

import numpy as np
import pytest

import oracle as O
import tdda
from tdda import topo
from conftest import rel


def test_ldr_tensor_matches_oracle():
    rng = np.random.Generator(np.random.PCG64(3))
    K = 2 * math.pi / 530.0
    pts = rng.uniform(-200, 200, (20, 3))
    t = topo.ldr_tensor(K, pts[:, 0], pts[:, 1], pts[:, 2])
    for i, p in enumerate(pts):
        assert np.max(np.abs(t[:, i] - O.ldr_inter(K, *p))) <= 1e-15 * np.max(np.abs(t[:, i]))
    assert np.all(topo.ldr_tensor(K, [0.0], [0.0], [0.0]) == 0)


def test_design_map_transpose_is_adjoint():
    rng = np.random.Generator(np.random.PCG64(4))
    for Nx, Ny in ((10, 10), (9, 12)):
        dm = topo.DesignMap(Nx, Ny, 2.0)
        th = rng.random((dm.hx, dm.hy))
        v = rng.standard_normal((Nx, Ny))
        assert abs(np.sum(dm.rho(th) * v) - np.sum(th * dm.grad_theta(v))) < 1e-12
        rho = dm.rho(th)
        assert np.allclose(rho, rho[::-1, :]) and np.allclose(rho, rho[:, ::-1])


def test_dal_deps_matches_finite_difference():
    K, d, S = 2 * math.pi / 500.0, 10.0, 0.3
    nE0, nK = np.array([1.0, 0.0, 0.0]), np.array([math.sqrt(0.3), 0.0, math.sqrt(0.7)])
    assert abs(float(np.sum((nE0 * nK) ** 2)) - S) < 1e-12
    for eps in (1.01 + 0j, 2.5 + 0.3j, 4.0 + 0.1j):
        h = 1e-6
        al = lambda e: 1.0 / O.get_alpha(500.0, K, d, e, nE0, nK)
        fd = (al(eps + h) - al(eps - h)) / (2 * h)
        assert abs(topo.dal_deps(np.array([eps]), K, d, S)[0] - fd) <= 1e-6 * abs(fd)


@pytest.mark.gpu
def test_adjoint_gradient_equals_finite_differences():
    if tdda.device_count() < 1:
        pytest.skip("no CUDA device")
    Nx, Ny, Nz, d = 6, 6, 4, 10.0
    rng = np.random.Generator(np.random.PCG64(8))
    th0 = 0.4 + 0.2 * rng.random((3, 3))
    r_obs = (d * (Nx - 1) / 2, d * (Ny - 1) / 2, d * (Nz - 1) + 100.0)
    loop = topo.TopoLoop(Nx, Ny, Nz, d, 500.0, np.array([1.0, 4.0 + 0.1j]), th0, r_obs, precision=tdda.FP64,
                         tol=1e-12)
    g = loop.evaluate().grad_theta
    h = 1e-5
    for (i, j) in ((0, 0), (1, 2), (2, 1)):
        fs = []
        for s in (+1, -1):
            loop.theta = th0.copy()
            loop.theta[i, j] += s * h
            fs.append(loop.evaluate().objective)
        fd = (fs[0] - fs[1]) / (2 * h)
        assert abs(g[i, j] - fd) <= 1e-5 * max(abs(fd), 1e-30) + 1e-12, (i, j, g[i, j], fd)
    loop.close()


@pytest.mark.gpu
def test_gradient_ascent_raises_the_objective():
    if tdda.device_count() < 1:
        pytest.skip("no CUDA device")
    Nx, Ny, Nz, d = 10, 10, 4, 10.0
    rng = np.random.Generator(np.random.PCG64(9))
    th0 = 0.4 + 0.2 * rng.random((5, 5))
    r_obs = (d * (Nx - 1) / 2, d * (Ny - 1) / 2, d * (Nz - 1) + 100.0)
    loop = topo.TopoLoop(Nx, Ny, Nz, d, 500.0, np.array([1.0, 4.0 + 0.1j]), th0, r_obs)
    f = [loop.step().objective for _ in range(6)]
    loop.close()
    assert f[-1] > f[0]


@pytest.mark.gpu
def test_heritage_starts_from_the_last_solutions():
    """origin_heritage / adjoint_heritage (EvoDDAModel.cpp:435-440, 598-604): each step's solves
    start from the previous step's solutions.  The objectives follow the cold-started loop's to
    the solves' tolerance, and the warm-started solves take fewer BiCGSTAB steps."""
    if tdda.device_count() < 1:
        pytest.skip("no CUDA device")
    Nx, Ny, Nz, d = 12, 12, 4, 10.0
    rng = np.random.Generator(np.random.PCG64(19))
    th0 = 0.4 + 0.2 * rng.random((6, 6))
    r_obs = (d * (Nx - 1) / 2, d * (Ny - 1) / 2, d * (Nz - 1) + 100.0)
    out = {}
    for her in (False, True):
        loop = topo.TopoLoop(Nx, Ny, Nz, d, 500.0, np.array([1.0, 4.0 + 0.1j]), th0, r_obs, precision=tdda.FP64,
                             tol=1e-8, origin_heritage=her, adjoint_heritage=her)
        rs = [loop.step() for _ in range(5)]
        loop.close()
        out[her] = ([r.objective for r in rs], [sum(r.iterations) for r in rs])
    (f0, i0), (f1, i1) = out[False], out[True]
    assert i1[0] == i0[0]  # the first step starts from P = 0 in both
    assert sum(i1[1:]) < sum(i0[1:])
    for a, b in zip(f0, f1):
        assert abs(a - b) <= 1e-6 * abs(a)


def test_adam_moments_follow_the_reference():
    """EvoDDAModel.cpp:673-690: bias correction inside the moving averages, beta2 = 1 - (1-beta1)^2."""
    st = SimpleNamespace(iteration=0, method="Adam", epsilon=0.05, V=None, S_ad=None, gsq=None)
    g0 = np.array([[0.3, -2.0]])
    out0, eps0 = topo.TopoLoop._moments(st, g0.copy())
    assert np.allclose(out0, g0 / (np.abs(g0) + 1e-8)) and eps0 == 0.1
    st.iteration = 4
    g1 = np.array([[-0.1, 1.0]])
    b1, b2 = 0.9, 1 - 0.1 ** 2
    V = b1 * g0 + (1 - b1) * g1 / (1 - b1 ** 5)
    S = b2 * g0 ** 2 + (1 - b2) * g1 ** 2 / (1 - b2 ** 5)
    out1, eps1 = topo.TopoLoop._moments(st, g1.copy())
    assert np.allclose(out1, V / (np.sqrt(S) + 1e-8)) and eps1 == 0.05
    ag = SimpleNamespace(iteration=0, method="Adagrad", epsilon=0.1, gsq=np.zeros((1, 2)))
    out, _ = topo.TopoLoop._moments(ag, g0.copy())
    assert np.allclose(out, g0 / np.sqrt(g0 ** 2 / 100000 + 1))


@pytest.mark.gpu
def test_device_glue_equals_host_restatement():
    """tdda_model_field_at and tdda_model_density_gradient against the same quantities
    formed on the host from the downloaded forward and adjoint fields."""
    if tdda.device_count() < 1:
        pytest.skip("no CUDA device")
    Nx, Ny, Nz, d = 8, 6, 4, 10.0
    rng = np.random.Generator(np.random.PCG64(10))
    dm = topo.DesignMap(Nx, Ny, 2.0)
    th0 = 0.3 + 0.4 * rng.random((dm.hx, dm.hy))
    r_obs = (d * (Nx - 1) / 2 + 3.0, d * (Ny - 1) / 2, d * (Nz - 1) + 80.0)
    mat = np.array([1.0, 6.25 + 0.05j])
    loop = topo.TopoLoop(Nx, Ny, Nz, d, 550.0, mat, th0, r_obs, precision=tdda.FP64, tol=1e-11,
                         nK=(math.sin(0.3), 0.0, math.cos(0.3)), nE0=(math.cos(0.3), 0.0, -math.sin(0.3)))
    r = loop.evaluate()
    P = loop.fwd.get_P()
    lams = [a.get_P() for a in loop.adj]
    E_obs = loop.Einc_obs + loop.b @ P
    assert r.objective == pytest.approx(float(np.sum(np.abs(E_obs) ** 2)), rel=1e-12)
    lam = sum(np.conj(E_obs[k]) * lams[k] for k in range(3))
    diel = loop._diel()
    m = loop.mat
    eps = m[0] + diel * (m[1] - m[0])
    dal = topo.dal_deps(eps, loop.K, d, loop.S) * (m[1] - m[0])
    g_dip = -2.0 * np.real((lam * dal * P).reshape(-1, 3).sum(axis=1))
    g_host = dm.grad_theta(g_dip.reshape(Nx, Ny, Nz).sum(axis=2))
    assert rel(r.grad_theta, g_host) <= 1e-10
    loop.close()


def _smooth_density_restated(x, ita, beta):
    """FilterOption::SmoothDensity (FilterOption.cpp:48-62), one value at a time."""
    if 0.0 <= x <= ita:
        return ita * (math.exp(-beta * (1 - x / ita)) - (1 - x / ita) * math.exp(-beta))
    if ita < x <= 1.0:
        return (1 - ita) * (1 - math.exp(-beta * (x - ita) / (1 - ita)) + (x - ita) / (1 - ita) * math.exp(-beta)) + ita
    raise ValueError


def test_projection_follows_the_reference():
    for ita in (0.5, 0.3):
        p = topo.Projection(1.0, 40.0, ita, "exp")
        for it in (0, 37, 99):
            beta = p.update_beta(it, 99)
            assert beta == pytest.approx(1.0 + 39.0 * math.exp(it / 99 - 1.0), rel=1e-15)
            x = np.linspace(0.0, 1.0, 41)
            h = p(x)
            assert np.allclose(h, [_smooth_density_restated(v, ita, beta) for v in x], rtol=1e-14, atol=1e-15)
            assert h[0] == pytest.approx(0.0, abs=1e-15) and h[-1] == pytest.approx(1.0, abs=1e-15)
            xi = np.linspace(0.01, 0.99, 17)
            xi = xi[np.abs(xi - ita) > 1e-3]
            fd = (p(xi + 1e-7) - p(xi - 1e-7)) / 2e-7
            assert np.allclose(p.derivative(xi), fd, rtol=1e-6)
    with pytest.raises(ValueError):
        topo.Projection(1.0, 10.0)(np.array([1.2]))
    with pytest.raises(ValueError):
        topo.Projection(1.0, 10.0, kind="cubic")
    # tools.cpp:780-798
    assert topo.beta_schedule("piecewise", 50, 100, 1, 41) == 1
    assert topo.beta_schedule("piecewise", 60, 100, 1, 41) == 3
    assert topo.beta_schedule("piecewise", 75, 100, 1, 41) == 5
    assert topo.beta_schedule("piecewise", 81, 100, 1, 41) == 41
    assert topo.beta_schedule("linear", 25, 100, 1, 41) == 11
    # fixit: the schedule runs over MAX_ITERATION_FIXED steps (FilterOption.cpp:23-27)
    pf = topo.Projection(1.0, 41.0, kind="linear", fixed_steps=50)
    assert pf.update_beta(25, 200) == 21


def test_reference_chain_form_restates_gradients_filtered():
    """The "reference" chain rule against a literal restatement of gradients_filtered's loops
    (EvoDDAModel.cpp:1177-1225) over the design map's filter weights, one free parameter per
    (x, y) column and no mirror (a 1 x 1 quadrant would hide the structure, so the map's mirror
    is bypassed by comparing before mirror_t)."""
    Nx, Ny = 7, 6
    dm = topo.DesignMap(Nx, Ny, 2.0)
    rng = np.random.Generator(np.random.PCG64(12))
    rf = rng.uniform(0.05, 0.95, (Nx, Ny))
    g = rng.standard_normal((Nx, Ny))
    proj = topo.Projection(2.0, 30.0, 0.5)
    proj.update_beta(10, 99)
    # FreeWeight[i]: (position, weight) of the parameters filtered into parameter i
    free_weight = []
    for x in range(Nx):
        for y in range(Ny):
            lst = []
            for dx, dy, w in dm.taps:
                xs, ys = x + dx, y + dy
                if 0 <= xs < Nx and 0 <= ys < Ny:
                    lst.append((xs * Ny + ys, w))
            free_weight.append(lst)
    n = Nx * Ny
    result = np.zeros(n)
    for lst in free_weight:
        s = sum(w for _, w in lst)
        for pos, w in lst:
            result[pos] += w / s
    gf = g.ravel()
    for i in range(n):
        result[i] = result[i] * proj.derivative(rf.ravel()[i]) * gf[i]
    colsum = dm.filter_t(np.ones((Nx, Ny)))
    ours = colsum * proj.derivative(rf) * g
    assert np.allclose(ours.ravel(), result, rtol=1e-13, atol=1e-15)


@pytest.mark.gpu
def test_adjoint_gradient_through_the_projection_equals_finite_differences():
    if tdda.device_count() < 1:
        pytest.skip("no CUDA device")
    Nx, Ny, Nz, d = 6, 6, 4, 10.0
    rng = np.random.Generator(np.random.PCG64(18))
    th0 = 0.3 + 0.4 * rng.random((3, 3))
    r_obs = (d * (Nx - 1) / 2, d * (Ny - 1) / 2, d * (Nz - 1) + 100.0)
    proj = topo.Projection(2.0, 20.0, 0.5, "exp")
    loop = topo.TopoLoop(Nx, Ny, Nz, d, 500.0, np.array([1.0, 4.0 + 0.1j]), th0, r_obs, precision=tdda.FP64,
                         tol=1e-12, projection=proj, max_steps=50)
    loop.iteration = 30  # beta = update_beta(29, 49), well above beta_min
    g = loop.evaluate().grad_theta
    assert loop.projection.beta == pytest.approx(2.0 + 18.0 * math.exp(29 / 49 - 1.0))
    h = 1e-6
    for (i, j) in ((0, 0), (1, 2), (2, 1)):
        fs = []
        for s in (+1, -1):
            loop.theta = th0.copy()
            loop.theta[i, j] += s * h
            fs.append(loop.evaluate().objective)
        fd = (fs[0] - fs[1]) / (2 * h)
        assert abs(g[i, j] - fd) <= 1e-5 * max(abs(fd), 1e-30) + 1e-12, (i, j, g[i, j], fd)
    loop.close()
