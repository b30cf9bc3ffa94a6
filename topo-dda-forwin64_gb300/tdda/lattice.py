"""Seeded synthetic lattices and incidence sets for the DDA solve workloads.

The reference builds a full box with ``build_a_bulk`` (tools.cpp:497-510: x
slowest, z fastest, dipole index ``z + Nz*(y + Ny*x)``), takes a per-dipole
density ``diel_old`` in [0, 1] (3 equal entries per dipole,
CoreStructure.cpp:22-27) and interpolates eps between ``material(0)`` and
``material(1)`` (DDAModel.cpp:54-63).  No public dataset is involved: every
workload below is drawn from a fixed seed with numpy's PCG64 generator.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


def bulk(Nx: int, Ny: int, Nz: int) -> np.ndarray:
    """Lattice indices of a full Nx x Ny x Nz box in build_a_bulk order (3N int32)."""
    x, y, z = np.meshgrid(np.arange(Nx), np.arange(Ny), np.arange(Nz), indexing="ij")
    return np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1).astype(np.int32).ravel()


def smooth_size(n: int) -> int:
    """Smallest 2^a 3^b 5^c 7^d >= n, the FFT length used per axis.

    Any length >= 2N-1 gives the reference's linear convolution exactly
    (AProductCore.cpp:41-44 uses 2N-1); a 7-smooth length keeps the FFT
    radices small."""
    m = max(1, n)
    while True:
        k = m
        for p in (2, 3, 5, 7):
            while k % p == 0:
                k //= p
        if k == 1:
            return m
        m += 1


FAST_Z = (20, 32, 40, 48, 56, 64)
FAST_XY = (32, 40, 48, 56, 64, 80, 96, 112, 128, 160, 192, 224, 256)


def fft_length(n: int, z_axis: bool) -> int:
    """FFT length a core uses for an axis of n cells: smooth_size(2n-1), or the next length
    with compiled passes (FAST_Z / FAST_XY) when that holds at most 25% more points."""
    m = smooth_size(2 * n - 1)
    for f in (FAST_Z if z_axis else FAST_XY):
        if f >= m:
            return f if 4 * f <= 5 * m else m
    return m


def n_e_perp_in_xz(theta: float, phi: float = 0.0) -> np.ndarray:
    """Unit polarisation perpendicular to k in the xz-plane (tools.cpp:686-704)."""
    tmp = math.cos(theta) / math.sqrt(math.sin(theta) ** 2 * math.cos(phi) ** 2 + math.cos(theta) ** 2)
    k = np.array([math.sin(theta) * math.cos(phi), math.sin(theta) * math.sin(phi), math.cos(theta)])
    for xv in (-tmp, tmp):
        for zv in (-math.sqrt(1 - tmp * tmp), math.sqrt(1 - tmp * tmp)):
            nE = np.array([xv, 0.0, zv])
            if abs(float(k @ nE)) < 1e-10 and xv >= 0.0:
                return nE
    raise ValueError("no perpendicular polarisation in the xz-plane")


def box_filter3(rho: np.ndarray) -> np.ndarray:
    """3x3x3 mean with edge replication."""
    p = np.pad(rho, 1, mode="edge")
    out = np.zeros_like(rho)
    nx, ny, nz = rho.shape
    for dx in range(3):
        for dy in range(3):
            for dz in range(3):
                out += p[dx:dx + nx, dy:dy + ny, dz:dz + nz]
    return out / 27.0


def linear_filter_xy(rho: np.ndarray, r: float) -> np.ndarray:
    """Linear 'cone' density filter in the xy-plane, weight r - dist for
    dist^2 <= r^2 - 0.01 (SpacePara.cpp:37-48), normalised per cell."""
    nx, ny, nz = rho.shape
    ri = int(math.ceil(r))
    out = np.zeros_like(rho)
    wsum = np.zeros((nx, ny))
    acc = np.zeros_like(rho)
    for dx in range(-ri, ri + 1):
        for dy in range(-ri, ri + 1):
            dist2 = dx * dx + dy * dy
            if dist2 > r * r - 0.01:
                continue
            w = r - math.sqrt(dist2)
            xs = slice(max(0, dx), nx + min(0, dx))
            xd = slice(max(0, -dx), nx + min(0, -dx))
            ys = slice(max(0, dy), ny + min(0, dy))
            yd = slice(max(0, -dy), ny + min(0, -dy))
            acc[xd, yd, :] += w * rho[xs, ys, :]
            wsum[xd, yd] += w
    out = acc / wsum[:, :, None]
    return out


def mirror4_xy(rho: np.ndarray) -> np.ndarray:
    """4-fold mirror symmetry in x and y: the lower-left quadrant is copied."""
    nx, ny, _ = rho.shape
    ix = np.minimum(np.arange(nx), nx - 1 - np.arange(nx))
    iy = np.minimum(np.arange(ny), ny - 1 - np.arange(ny))
    return rho[ix][:, iy].copy()


@dataclass
class Incidence:
    nK: np.ndarray
    nE0: np.ndarray
    E0: float = 1.0


@dataclass
class Workload:
    """One lattice + the right-hand sides solved on it."""
    name: str
    Nx: int
    Ny: int
    Nz: int
    d: float
    lam: float
    material: np.ndarray          # complex, [background, design]
    rho: np.ndarray               # per-dipole density (N)
    R: np.ndarray                 # 3N int32
    incidences: list = field(default_factory=list)
    nback: float = 1.0
    tol: float = 1e-5
    max_it: int = 10000

    @property
    def N(self) -> int:
        return self.R.size // 3

    @property
    def diel_old(self) -> np.ndarray:
        """3N density vector, the same value for the 3 components."""
        return np.repeat(self.rho, 3).astype(np.float64)


XPOL_Z = Incidence(np.array([0.0, 0.0, 1.0]), np.array([1.0, 0.0, 0.0]))


def config(idx: int, seed: int = 1234) -> Workload:
    """The five solve workloads.  idx is 1-based:

    1  plain FP64 single solve       20x20x10, d=10 nm, lam=500 nm, rho~U[0,1], eps_m=4+0.1i
    2  mixed-precision single solve  64x64x16, d=10 nm, lam=600 nm, rho~U[0,1] then 3x3x3 box filter,
                                     eps_m=6.25+0.05i
    3  batched right-hand sides      96x96x24, d=8 nm, lam=550 nm, rho~Bernoulli(0.4), eps_m=4+0.1i,
                                     8 RHS: x/y polarisation x polar angle {0,15,30,45} deg in xz
    4  topology-optimisation lattice 80x80x20, d=10 nm, lam=500 nm, rho~U[0.4,0.6], radius-2 linear
                                     filter, 4-fold xy mirror symmetry, eps_m=4+0.1i
    All use material(0)=1.0 (the AProductCore ctor bumps it to 1.01), LDR polarisability, a
    unit plane wave and tol 1e-5.
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    if idx == 1:
        Nx, Ny, Nz, d, lam, em = 20, 20, 10, 10.0, 500.0, 4.0 + 0.1j
        rho = rng.random(Nx * Ny * Nz)
        inc = [XPOL_Z]
    elif idx == 2:
        Nx, Ny, Nz, d, lam, em = 64, 64, 16, 10.0, 600.0, 6.25 + 0.05j
        rho = box_filter3(rng.random((Nx, Ny, Nz))).ravel()
        inc = [XPOL_Z]
    elif idx == 3:
        Nx, Ny, Nz, d, lam, em = 96, 96, 24, 8.0, 550.0, 4.0 + 0.1j
        rho = (rng.random(Nx * Ny * Nz) < 0.4).astype(np.float64)
        inc = []
        for deg in (0.0, 15.0, 30.0, 45.0):
            th = math.radians(deg)
            nK = np.array([math.sin(th), 0.0, math.cos(th)])
            inc.append(Incidence(nK, n_e_perp_in_xz(th)))
            inc.append(Incidence(nK, np.array([0.0, 1.0, 0.0])))
    elif idx == 4:
        Nx, Ny, Nz, d, lam, em = 80, 80, 20, 10.0, 500.0, 4.0 + 0.1j
        raw = 0.4 + 0.2 * rng.random((Nx, Ny, Nz))
        rho = mirror4_xy(linear_filter_xy(mirror4_xy(raw), 2.0)).ravel()
        inc = [XPOL_Z]
    else:
        raise ValueError(f"no workload {idx}")
    return Workload(name=f"cfg{idx}", Nx=Nx, Ny=Ny, Nz=Nz, d=d, lam=lam,
                    material=np.array([1.0 + 0j, em]), rho=np.clip(rho, 0.0, 1.0),
                    R=bulk(Nx, Ny, Nz), incidences=inc)


@dataclass
class ServeRequest:
    t_arrival: float
    Nx: int
    Ny: int
    Nz: int
    lam: float
    eps_m: complex
    seed: int
    incidences: list

    @property
    def N(self) -> int:
        return self.Nx * self.Ny * self.Nz

    def diel_old(self) -> np.ndarray:
        rng = np.random.Generator(np.random.PCG64(self.seed))
        return np.repeat(rng.random(self.N), 3)


def serving_stream(n: int = 512, rate: float = 200.0, seed: int = 5, lo: int = 16, hi: int = 128,
                   zhi: int = 32) -> list:
    """The serving workload: n solve requests with Poisson arrivals (mean `rate` per s),
    lattice dims log-uniform per axis in [lo, hi] (z capped at zhi), d = 10 nm,
    wavelength U[400, 800] nm, eps_m in {2.25, 4.0+0.1i, 6.25+0.05i}, rho ~ U[0, 1],
    1-4 right-hand sides drawn from x/y polarisation x polar angles 0/15/30/45 deg."""
    rng = np.random.Generator(np.random.PCG64(seed))
    pool = config(3).incidences  # the 8 incidences of the batched workload
    t = 0.0
    out = []
    for k in range(n):
        t += float(rng.exponential(1.0 / rate))
        dims = [int(round(math.exp(rng.uniform(math.log(lo), math.log(hi))))) for _ in range(3)]
        dims[2] = min(dims[2], zhi)
        lam = float(rng.uniform(400.0, 800.0))
        em = [2.25 + 0j, 4.0 + 0.1j, 6.25 + 0.05j][int(rng.integers(0, 3))]
        nrhs = int(rng.integers(1, 5))
        pick = rng.choice(len(pool), size=nrhs, replace=False)
        incs = [(pool[i].nK, pool[i].nE0, pool[i].E0) for i in pick]
        out.append(ServeRequest(t, dims[0], dims[1], dims[2], lam, em, int(rng.integers(0, 2**31)), incs))
    return out
