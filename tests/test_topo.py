"""The topology-optimisation loop (tdda/topo.py): the caller of the solve path.

CPU: the LDR tensor restated with numpy equals the oracle's; the design map's transpose
is its adjoint; dal/deps equals a finite difference of 1/alpha_LDR.  GPU: the adjoint
gradient (forward + 3 basis adjoints batched) equals central finite differences of the
objective, and gradient ascent raises the objective.
"""
import math

import numpy as np
import pytest

import oracle as O
import tdda
from tdda import topo


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
