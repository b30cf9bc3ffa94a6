"""Topology-optimisation loop around the batched solver (the caller of the hot path).

The reference's EvoDDAModel::EvoOptimization (EvoDDAModel.cpp:393-765) runs, per
iteration, a forward solve, a finite-difference objective derivative, an adjoint
solve with the same matrix (A is complex symmetric), gradient assembly, an
optimiser step and a density update.  This loop keeps that structure for a point
objective f = |E(r_obs)|^2 (ObjPointEDDAModel, ObjDDAModel.cpp:20-96, evaluates
E(r_obs) = E_inc(r_obs) - sum_j A(r_obs - r_j) P_j) and makes two changes:

* the adjoint source is exact instead of finite differences.  With
  E_obs = E_inc(r_obs) + sum_k b_k . P and b_k[j] = -A(r_obs - r_j) e_k,
  df/dP = sum_k conj(E_obs,k) b_k, so the adjoint solution is
  lambda = sum_k conj(E_obs,k) lambda_k with A lambda_k = b_k.  The three
  lambda_k and the forward P are solved together, four right-hand sides in one
  batched solve per iteration (tdda_solve_batch);
* dal/drho is analytic: 1/alpha_LDR(eps) = 1/a1 + T/d^3 (tools.cpp:617-630),
  so dal/deps = -3/(c (eps-1)^2) + (b2 + b3 S)(K d)^2/d^3.

Design parameters theta live on one xy quadrant; rho = filter(mirror4(theta)),
extruded along z (the reference's 2-D extruded design with 4-fold symmetry,
SpacePara.cpp:8-48, and its linear cone filter).  df/dtheta follows by the
transposed chain.  The step is gradient ascent: the gradient is scaled so that
its mean magnitude is at least 0.1 (EvoDDAModel.cpp:734-738) and multiplied by
epsilon = 0.1, so the mean step is 0.01; theta is clipped to [0, 1].

With a Projection, rho = H_beta(filter(mirror4(theta))): the reference's smooth Heaviside
(FilterOption::SmoothDensity, FilterOption.cpp:48-62) with beta on its exp / piecewise /
linear schedule (FilterOption.cpp:23-46), and the gradient passes through H' on the way back
(EvoDDAModel.cpp:1177-1225), either exactly or in the reference's diagonal form.

The step follows EvoDDAModel.cpp:640-735: optional Adam / Adamdecay / Adagrad
moments on the parameter gradient, the mean-magnitude normalisation and the
step epsilon * g.

Everything O(N) runs on the GPU through libtdda: the batched solves, the
objective (tdda_model_field_at at r_obs) and the per-column adjoint sensitivity
(tdda_model_density_gradient); P never leaves the device.  The host keeps the
O(Nx Ny) design map (mirror, filter and their transposes) and the optimiser.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from . import FP32_REFINE, AProductCore, DDAModel, lattice, solve_batch

B1, B2, B3 = -1.891531, 0.1648469, -1.7700004  # LDR coefficients (tools.cpp:618-620)


def ldr_tensor(K: float, x, y, z) -> np.ndarray:
    """LDR interaction tensor (AProductCore.cpp:588-623) at offsets (x, y, z) in nm.
    Returns (6, n) complex: xx, xy, xz, yy, yz, zz; zero at r = 0."""
    x, y, z = (np.asarray(v, np.float64) for v in (x, y, z))
    xs, ys, zs = x * x, y * y, z * z
    rn = np.sqrt(xs + ys + zs)
    out = np.zeros((6,) + rn.shape, np.complex128)
    ok = rn != 0
    r = rn[ok]
    rsq, rcu = r * r, r * r * r
    c1 = np.exp(1j * K * r) / rcu
    c2 = (1.0 - 1j * K * r) / rsq
    c3 = K * K - 3.0 * c2
    out[0, ok] = c1 * (c2 * (rsq - 3 * xs[ok]) - K * K * (ys[ok] + zs[ok]))
    out[1, ok] = c1 * (x[ok] * y[ok] * c3)
    out[2, ok] = c1 * (z[ok] * x[ok] * c3)
    out[3, ok] = c1 * (c2 * (rsq - 3 * ys[ok]) - K * K * (zs[ok] + xs[ok]))
    out[4, ok] = c1 * (y[ok] * z[ok] * c3)
    out[5, ok] = c1 * (c2 * (rsq - 3 * zs[ok]) - K * K * (xs[ok] + ys[ok]))
    return out


def point_sources(R: np.ndarray, d: float, K: float, r_obs) -> np.ndarray:
    """b_k[j] = -A(r_obs - d R_j) e_k for k = x, y, z: (3, 3N) complex."""
    R = np.asarray(R).reshape(-1, 3)
    t = ldr_tensor(K, r_obs[0] - d * R[:, 0], r_obs[1] - d * R[:, 1], r_obs[2] - d * R[:, 2])
    # symmetric tensor: column k = row k
    rows = [(0, 1, 2), (1, 3, 4), (2, 4, 5)]
    b = np.zeros((3, R.shape[0], 3), np.complex128)
    for k, (a0, a1, a2) in enumerate(rows):
        b[k, :, 0], b[k, :, 1], b[k, :, 2] = -t[a0], -t[a1], -t[a2]
    return b.reshape(3, -1)


def dal_deps(eps: np.ndarray, K: float, d: float, S: float) -> np.ndarray:
    c = 3 * d ** 3 / (4 * math.pi)
    return -3.0 / (c * (eps - 1.0) ** 2) + (B2 + B3 * S) * (K * d) ** 2 / d ** 3


class DesignMap:
    """theta (quadrant, hx x hy) -> rho (Nx x Ny, extruded along z) and its transpose."""

    def __init__(self, Nx: int, Ny: int, r: float = 2.0):
        self.Nx, self.Ny, self.r = Nx, Ny, r
        self.hx, self.hy = (Nx + 1) // 2, (Ny + 1) // 2
        self.ix = np.minimum(np.arange(Nx), Nx - 1 - np.arange(Nx))
        self.iy = np.minimum(np.arange(Ny), Ny - 1 - np.arange(Ny))
        ri = int(math.ceil(r))
        self.taps = [(dx, dy, r - math.sqrt(dx * dx + dy * dy)) for dx in range(-ri, ri + 1)
                     for dy in range(-ri, ri + 1) if dx * dx + dy * dy <= r * r - 0.01]
        wsum = np.zeros((Nx, Ny))
        for dx, dy, w in self.taps:
            wsum[self._dst(dx, Nx), self._dst(dy, Ny)] += w
        self.wsum = wsum

    @staticmethod
    def _src(dd, n):
        return slice(max(0, dd), n + min(0, dd))

    @staticmethod
    def _dst(dd, n):
        return slice(max(0, -dd), n + min(0, -dd))

    def mirror(self, theta):
        return theta[self.ix][:, self.iy]

    def mirror_t(self, g):
        out = np.zeros((self.hx, self.hy))
        np.add.at(out, (self.ix[:, None], self.iy[None, :]), g)
        return out

    def filter(self, a):
        acc = np.zeros_like(a)
        for dx, dy, w in self.taps:
            acc[self._dst(dx, self.Nx), self._dst(dy, self.Ny)] += w * a[self._src(dx, self.Nx), self._src(dy, self.Ny)]
        return acc / self.wsum

    def filter_t(self, g):
        gw = g / self.wsum
        out = np.zeros_like(g)
        for dx, dy, w in self.taps:
            out[self._src(dx, self.Nx), self._src(dy, self.Ny)] += w * gw[self._dst(dx, self.Nx), self._dst(dy, self.Ny)]
        return out

    def rho(self, theta):
        return self.filter(self.mirror(theta))

    def grad_theta(self, g_xy):
        return self.mirror_t(self.filter_t(g_xy))


def beta_schedule(kind: str, x: float, x_max: float, beta_min: float, beta_max: float) -> float:
    """The projection sharpness at optimisation step x of x_max (FilterOption::update_beta,
    FilterOption.cpp:23-46, with tools.cpp:776-798): "exp", "piecewise" or "linear"."""
    if kind == "exp":
        return beta_min + (beta_max - beta_min) * math.exp(x / x_max - 1.0)
    if kind == "piecewise":
        if x <= 0.5 * x_max:
            return beta_min
        if x <= 0.7 * x_max:
            return beta_min + (beta_max - beta_min) / 20
        if x <= 0.8 * x_max:
            return beta_min + (beta_max - beta_min) / 10
        return beta_max
    if kind == "linear":
        return beta_min + (beta_max - beta_min) * x / x_max
    raise ValueError(f"beta schedule {kind!r} is not defined")


class Projection:
    """Smooth Heaviside projection of the filtered density (FilterOption, FilterOption.cpp:5-62):

        H(x) = ita (exp(-beta (1 - x/ita)) - (1 - x/ita) exp(-beta))                     x <= ita
        H(x) = (1-ita) (1 - exp(-beta (x-ita)/(1-ita)) + (x-ita)/(1-ita) exp(-beta)) + ita  x > ita

    for x in [0, 1] (SmoothDensity, :48-62), and its derivative
    H'(x) = beta exp(-beta (1 - x/ita)) + exp(-beta) below ita, beta exp(-beta (x-ita)/(1-ita)) +
    exp(-beta) above (PtoFderivative, EvoDDAModel.cpp:1163-1175).  beta follows the schedule of
    update_beta from beta_min at step 0 to beta_max at step x_max; with fixit the schedule runs
    over MAX_ITERATION_FIXED steps instead (FilterOption.cpp:23-27)."""

    def __init__(self, beta_min: float, beta_max: float, ita: float = 0.5, kind: str = "exp",
                 fixed_steps: int = 0):
        beta_schedule(kind, 0.0, 1.0, beta_min, beta_max)  # rejects an unknown schedule
        self.beta_min, self.beta_max, self.ita, self.kind = float(beta_min), float(beta_max), float(ita), kind
        self.fixed_steps = int(fixed_steps)
        self.beta = self.beta_min

    def update_beta(self, iteration: int, max_iteration: int) -> float:
        x_max = self.fixed_steps if self.fixed_steps > 0 else max_iteration
        self.beta = beta_schedule(self.kind, float(iteration), float(x_max), self.beta_min, self.beta_max)
        return self.beta

    def _check(self, x):
        x = np.asarray(x, np.float64)
        if np.any(x < 0.0) or np.any(x > 1.0) or np.any(np.isnan(x)):
            raise ValueError("SmoothDensity: input out of range [0, 1]")
        return x

    def __call__(self, x):
        x = self._check(x)
        b, it = self.beta, self.ita
        lo = it * (np.exp(-b * (1 - x / it)) - (1 - x / it) * math.exp(-b))
        hi = (1 - it) * (1 - np.exp(-b * (x - it) / (1 - it)) + (x - it) / (1 - it) * math.exp(-b)) + it
        return np.where(x <= it, lo, hi)

    def derivative(self, x):
        x = self._check(x)
        b, it = self.beta, self.ita
        lo = b * np.exp(-b * (1 - x / it)) + math.exp(-b)
        hi = b * np.exp(-b * (x - it) / (1 - it)) + math.exp(-b)
        return np.where(x <= it, lo, hi)


@dataclass
class StepResult:
    objective: float
    iterations: list
    grad_theta: np.ndarray


class TopoLoop:
    """Point-|E|^2 topology optimisation with forward + 3 adjoint solves batched per step."""

    def __init__(self, Nx, Ny, Nz, d, lam, material, theta0, r_obs, precision=FP32_REFINE, tol=1e-5,
                 max_it=10000, nK=(0.0, 0.0, 1.0), nE0=(1.0, 0.0, 0.0), E0=1.0, filter_r=2.0, epsilon=0.1,
                 method="grad", projection: Projection = None, max_steps: int = 200, chain: str = "exact",
                 origin_heritage: bool = False, adjoint_heritage: bool = False):
        """origin_heritage / adjoint_heritage: start each step's forward / adjoint solves from
        the previous step's solutions instead of P = 0 (the reference's HaveOriginHeritage and
        HaveAdjointHeritage, EvoDDAModel.cpp:435-440, 598-604; its main.cpp sets both false,
        the default here).
        projection: the smooth Heaviside applied after the filter, its beta scheduled over
        max_steps steps (the reference's MAX_ITERATION_EVO); chain "exact" (the transposed
        chain rule through filter and projection, checked against finite differences) or
        "reference" (the reference's diagonal form of gradients_filtered,
        EvoDDAModel.cpp:1177-1225: each column's gradient times the column sum of the
        normalised filter weights and the projection's slope at that column)."""
        self.Nx, self.Ny, self.Nz, self.d = Nx, Ny, Nz, d
        self.R = lattice.bulk(Nx, Ny, Nz)
        self.map = DesignMap(Nx, Ny, filter_r)
        self.theta = np.array(theta0, np.float64).reshape(self.map.hx, self.map.hy)
        self.precision, self.tol, self.max_it, self.epsilon = precision, tol, max_it, epsilon
        self.nK, self.nE0, self.E0 = np.array(nK, float), np.array(nE0, float), float(E0)
        self.r_obs = np.array(r_obs, float)
        if chain not in ("exact", "reference"):
            raise ValueError(f"unknown chain rule {chain!r}")
        self.projection, self.max_steps, self.chain = projection, int(max_steps), chain
        self.origin_heritage, self.adjoint_heritage = bool(origin_heritage), bool(adjoint_heritage)
        self.iteration = 0
        self.core = AProductCore(Nx, Ny, Nz, self.R, d, lam, material, max_rhs=4)
        self.K = self.core.K
        self.mat = self.core.get_material()  # normalised (vacuum -> 1.01)
        self.S = float(np.sum((self.nE0 * self.nK) ** 2))
        diel = self._diel()
        self.fwd = DDAModel(self.core, self.nK, self.E0, self.nE0, diel)
        self.b = point_sources(self.R, d, self.K, self.r_obs)
        self.adj = []
        for k in range(3):
            m = DDAModel(self.core, self.nK, self.E0, self.nE0, diel)
            m.change_E(self.b[k])
            self.adj.append(m)
        self.Einc_obs = self.E0 * self.nE0 * np.exp(1j * self.K * float(self.nK @ self.r_obs))
        # design parameter of the sensitivity sum: the (x, y) column; in build_a_bulk order the
        # dipoles of column x Ny + y are (x Ny + y) Nz + z, z < Nz
        N = Nx * Ny * Nz
        self.col_off = np.arange(0, N + 1, Nz, dtype=np.int32)
        self.col_dip = np.arange(N, dtype=np.int32)
        if method not in ("grad", "Adam", "Adamdecay", "Adagrad"):
            raise ValueError(f"unknown optimiser {method!r}")
        self.method = method
        self.V = self.S_ad = None
        self.gsq = np.zeros_like(self.theta)  # Adagrad accumulator (EvoDDAModel.cpp:36)

    def _beta(self):
        """The projection's beta for the current step: the structure of step it was projected
        with update_beta(it - 1, MAX - 1) (CoreStructure.cpp:46, EvoDDAModel.cpp:750), and its
        gradient uses the same beta (EvoDDAModel.cpp:645-648)."""
        return self.projection.update_beta(max(self.iteration - 1, 0), self.max_steps - 1)

    def _filtered(self):
        return np.clip(self.map.rho(self.theta), 0.0, 1.0)

    def _rho(self):
        rf = self._filtered()
        if self.projection is None:
            return rf
        self._beta()
        return self.projection(rf)

    def _diel(self):
        rho_xy = self._rho()
        rho = np.repeat(rho_xy[:, :, None], self.Nz, axis=2).ravel()
        return np.repeat(rho, 3)

    def evaluate(self):
        """Solve forward + adjoints at the current theta; return f and df/dtheta."""
        diel = self._diel()
        models = [self.fwd] + self.adj
        for k, m in enumerate(models):
            m.UpdateAlpha(diel)
            # a model keeps its last solution on the device: heritage starts from it
            if not (self.origin_heritage if k == 0 else self.adjoint_heritage):
                m.InitializeP()
        infos = solve_batch(models, self.precision, self.max_it, self.tol)
        E_obs = self.fwd.field_at(self.r_obs[None, :])[0]  # E_inc(r_obs) - sum_j A(r_obs - r_j) P_j
        f = float(np.sum(np.abs(E_obs) ** 2))
        # df/drho_j = 2 Re(conj(E_obs) . dE_obs/drho_j) = -2 Re(lambda_j dal_j P_j), lambda = sum_k conj(E_k) lambda_k
        s = self.fwd.density_gradient(self.adj, np.conj(E_obs), self.col_off, self.col_dip)
        g_xy = (-2.0 * s).reshape(self.Nx, self.Ny)
        # rho is clipped to [0, 1]; the filter keeps it inside, so the clip is inactive
        return StepResult(f, [i["iterations"] for i in infos], self.grad_theta(g_xy))

    def grad_theta(self, g_xy):
        """df/dtheta from df/drho per (x, y) column through projection, filter and mirror."""
        if self.projection is None:
            return self.map.grad_theta(g_xy)
        rf = self._filtered()
        self._beta()
        slope = self.projection.derivative(rf)
        if self.chain == "exact":
            return self.map.mirror_t(self.map.filter_t(slope * g_xy))
        # EvoDDAModel.cpp:1199-1221: result(p) = (sum_i w_ip / sum_j w_ij) H'(rho_f(p)) g(p)
        colsum = self.map.filter_t(np.ones_like(g_xy))
        return self.map.mirror_t(colsum * slope * g_xy)

    def _moments(self, g):
        """Adam / Adamdecay / Adagrad of EvoDDAModel.cpp:673-731 (beta1 = 0.9,
        beta2 = 1 - (1 - beta1)^2, bias correction inside the moving averages as there)."""
        it, b1 = self.iteration, 0.9
        b2 = 1 - (1 - b1) ** 2
        eps = self.epsilon
        if self.method in ("Adam", "Adamdecay"):
            if it == 0:
                self.V = (1 - b1) * g / (1 - b1 ** (it + 1))
                self.S_ad = (1 - b2) * g ** 2 / (1 - b2 ** (it + 1))
            else:
                self.V = b1 * self.V + (1 - b1) * g / (1 - b1 ** (it + 1))
                self.S_ad = b2 * self.S_ad + (1 - b2) * g ** 2 / (1 - b2 ** (it + 1))
            g = self.V / (np.sqrt(self.S_ad) + 1e-8)
            if it <= 3:
                eps = 0.1
            elif self.method == "Adamdecay" and it >= 150:
                eps = self.epsilon * math.exp(-(it - 150) / 10.0)
        elif self.method == "Adagrad":
            self.gsq += g ** 2 / 100000
            g = g / np.sqrt(self.gsq + 1)
        return g, eps

    def step(self) -> StepResult:
        r = self.evaluate()
        g, eps = self._moments(r.grad_theta.copy())
        mean = float(np.mean(np.abs(g)))
        if 0 < mean < 0.1:  # EvoDDAModel.cpp:734-736
            g /= mean / 0.1
        self.theta = np.clip(self.theta + eps * g, 0.0, 1.0)
        self.iteration += 1
        return r

    def close(self):
        for m in [self.fwd] + self.adj:
            m.close()
        self.core.close()
