"""Generate the solve-level fixtures of the benchmarked lattices (configs 1-4).

The lattices are too large to commit whole (cfg 3 holds 663,552 complex unknowns), so each
fixture keeps what a size-independent comparison needs:
  * a seeded sample of 4,096 entries of P and of Einternal (indices stored), against which
    the GPU's solution is compared norm-wise over the sample;
  * the norms |P| and |Einternal| of the full vectors;
  * the iteration count and the final recursive residual;
  * a fingerprint of the inputs (sum and norm of the densities) so a changed workload
    generator is caught.

solve_cfg2_ref.npz       the reference itself (oracle/_ref/ref_driver: the reference's own
                         AProductCore.cpp / DDAModel.cpp with the CPU FFT stand-in) on
                         cfg 2 at tol 1e-10, on its own 127 x 127 x 31 grid
                         (AProductCore.cpp:41-44)
solve_cfg{2,3,4}_tight.npz  the oracle (the C restatement pinned bit-exact to the
                         reference on the smaller fixtures) on the 2N grid the GPU uses, FP64
                         BiCGSTAB to 1e-10; cfg 3 for incidences 0 (x-pol, 0 deg) and 7
                         (y-pol, 45 deg), cfg 2 and 4 for the x-polarised wave along +z.
                         Each also stores the same solve stopped at tol 1e-5, sampled, and
                         its distance from the tol-1e-10 solution (the error a converged
                         solve at the workloads' own tolerance carries)
iters_spread_cfg3_tight.npz  the same at tol 1e-10 for cfg 3 (incidences 0 and 7, the GPU's
                         grid, E and 5 one-ulp perturbations each)
iters_spread.npz         how far the reference's iteration count at tol 1e-5 moves under
                         rounding-level changes, for the three tol-1e-5 solve fixtures
                         (cfg 1, sparse10x9x6, adj8x8x4): the oracle's BiCGSTAB on the
                         reference's 2N-1 grid and on the GPU's grid, each for E and for 16
                         perturbations of E by at most one unit in the last place per entry

Run from the repository root:  python tests/golden/make_golden_configs.py [names...]
The reference solve needs the reference checkout (oracle/Makefile's REF_ROOT); the oracle
solves need only oracle/liboracle.so.  Total time here: about ten minutes on one core.
"""
from __future__ import annotations

import os
import struct
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "topo-dda-forwin64_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, HERE)
from tdda import lattice  # noqa: E402

NSAMPLE = 4096
SAMPLE_SEED = 2024


def sample_index(n3: int) -> np.ndarray:
    rng = np.random.Generator(np.random.PCG64(SAMPLE_SEED + n3))
    return np.sort(rng.choice(n3, size=min(NSAMPLE, n3), replace=False)).astype(np.int64)


def fingerprint(w: lattice.Workload) -> np.ndarray:
    return np.array([w.rho.sum(), np.linalg.norm(w.rho), float(w.N)])


def _save(name, w, inc_index, P, Ein, iterations, error, tol, grid, source, extra=None):
    idx = sample_index(3 * w.N)
    out = dict(cfg=int(w.name[3:]), incidence=int(inc_index), tol=float(tol), iterations=int(iterations),
               error=float(error), idx=idx, P_s=np.asarray(P)[idx], Ein_s=np.asarray(Ein)[idx],
               normP=float(np.linalg.norm(P)), normEin=float(np.linalg.norm(Ein)), grid=np.array(grid, np.int32),
               fingerprint=fingerprint(w), source=source)
    if extra:
        out.update(extra)
    np.savez_compressed(os.path.join(HERE, name), **out)
    print(f"{name}: cfg {out['cfg']} inc {inc_index} iterations {iterations} error {error:.3e} "
          f"|P| {out['normP']:.6e} ({source})", flush=True)


def oracle_tight(name, idx, inc_index):
    import oracle as O
    w = lattice.config(idx)
    inc = w.incidences[inc_index]
    grid = tuple(2 * n for n in (w.Nx, w.Ny, w.Nz))
    t0 = time.time()
    oc = O.OracleCore(w.Nx, w.Ny, w.Nz, w.R, w.d, w.lam, w.material, w.nback, grid=grid, pruned=True)
    om = O.OracleModel(oc, inc.nK, inc.E0, inc.nE0, w.diel_old)
    st = om.bicgstab(100000, 1e-5)
    assert st == O.CONVERGED, st
    it5, err5, P5 = om.ITERATION, om.Error, om.P
    om.update_E_in_structure()
    Ein5 = om.Einternal
    om.InitializeP(np.zeros(3 * w.N, np.complex128))
    st = om.bicgstab(100000, 1e-10)
    assert st == O.CONVERGED, st
    om.update_E_in_structure()
    P, Ein = om.P, om.Einternal
    idx_s = sample_index(3 * w.N)
    extra = dict(it_tol5=int(it5), err_tol5=float(err5), P5_s=P5[idx_s], Ein5_s=Ein5[idx_s],
                 dist_tol5=float(np.linalg.norm(P5 - P) / np.linalg.norm(P)))
    _save(name, w, inc_index, P, Ein, om.ITERATION, om.Error, 1e-10, grid, "oracle", extra)
    print(f"   tol 1e-5: {it5} iterations, |P5 - P|/|P| = {extra['dist_tol5']:.3e} ({time.time() - t0:.0f} s)",
          flush=True)
    om.close()
    oc.close()


def reference_cfg2():
    import make_golden as MG
    MG.build_driver()
    w = lattice.config(2)
    t0 = time.time()
    raw, out = MG.run(1, **MG.case_kw(w, None, 10000, 1e-10), vecs=[])
    N = w.N
    off = 12 * N + 48 * N
    it = struct.unpack_from("<i", raw, off)[0]
    off += 4
    P = np.frombuffer(raw, "<c16", count=3 * N, offset=off)
    off += 48 * N
    Ein = np.frombuffer(raw, "<c16", count=3 * N, offset=off)
    import re
    m = re.findall(r"Error:\s*([-+0-9.eE]+)", out)
    err = float(m[-1]) if m else float("nan")
    grid = tuple(2 * n - 1 for n in (w.Nx, w.Ny, w.Nz))
    _save("solve_cfg2_ref.npz", w, 0, P, Ein, it, err, 1e-10, grid, "reference")
    print(f"   ({time.time() - t0:.0f} s)", flush=True)


def _spread_rows(Nx, Ny, Nz, R, d, lam, material, nback, nK, E0, nE0, diel, P0=None, E_rhs=None, nperturb=16):
    """Iteration counts of the oracle's BiCGSTAB at tol 1e-5 on the reference's 2N-1 grid and
    on the GPU's grid, for E and nperturb perturbations of E by at most one unit in the last
    place per entry."""
    import oracle as O
    grids = [tuple(2 * n - 1 for n in (Nx, Ny, Nz)),
             (lattice.fft_length(Nx, False), lattice.fft_length(Ny, False), lattice.fft_length(Nz, True))]
    rows = []
    for gi, grid in enumerate(grids):
        oc = O.OracleCore(Nx, Ny, Nz, R, d, lam, material, nback, grid=grid)
        om = O.OracleModel(oc, nK, E0, nE0, diel)
        E = om.E if E_rhs is None else np.asarray(E_rhs, np.complex128)
        for k in range(nperturb + 1):
            Ek = E.copy()
            if k > 0:
                rng = np.random.Generator(np.random.PCG64(700 + k))
                re_, im_ = E.real.copy(), E.imag.copy()
                for part in (re_, im_):
                    s = rng.integers(-1, 2, part.size)
                    part[s > 0] = np.nextafter(part[s > 0], np.inf)
                    part[s < 0] = np.nextafter(part[s < 0], -np.inf)
                Ek = re_ + 1j * im_
            om.change_E(Ek)
            om.InitializeP(np.zeros(3 * (R.size // 3), np.complex128) if P0 is None else P0)
            om.ITERATION = 0
            st = om.bicgstab(10000, 1e-5)
            assert st == O.CONVERGED
            rows.append((gi, k, om.ITERATION))
        om.close()
        oc.close()
    return np.array(rows, np.int32)


def iteration_spread():
    """The spread for the three tol-1e-5 solve fixtures of make_golden.py."""
    out = {}
    for name in ("cfg1", "sparse10x9x6", "adj8x8x4"):
        g = np.load(os.path.join(HERE, f"solve_{name}.npz"))
        Nx, Ny, Nz = (int(v) for v in g["box"])
        rows = _spread_rows(Nx, Ny, Nz, np.asarray(g["R"], np.int32), float(g["d"]), float(g["lam"]),
                            g["material"], float(g["nback"]), g["nK"], float(g["E0"]), g["nE0"], g["diel_old"],
                            g["P0"] if "P0" in g else None, g["E_rhs"] if "E_rhs" in g else None)
        out[name] = rows
        its = rows[:, 2]
        print(f"spread {name}: reference {int(g['iterations'])}; {sorted(its.tolist())} "
              f"(min {its.min()}, max {its.max()})", flush=True)
    np.savez_compressed(os.path.join(HERE, "iters_spread.npz"), tol=1e-5, **out)


def _tight_count(args):
    """Iterations of the oracle's FP64 BiCGSTAB to 1e-10 on cfg 3's 2N grid for incidence inc,
    with E perturbed by at most one unit in the last place per entry (k > 0)."""
    inc_index, k = args
    import oracle as O
    w = lattice.config(3)
    inc = w.incidences[inc_index]
    grid = tuple(2 * n for n in (w.Nx, w.Ny, w.Nz))
    oc = O.OracleCore(w.Nx, w.Ny, w.Nz, w.R, w.d, w.lam, w.material, w.nback, grid=grid, pruned=True)
    om = O.OracleModel(oc, inc.nK, inc.E0, inc.nE0, w.diel_old)
    if k > 0:
        E = om.E
        rng = np.random.Generator(np.random.PCG64(900 + k))
        re_, im_ = E.real.copy(), E.imag.copy()
        for part in (re_, im_):
            sgn = rng.integers(-1, 2, part.size)
            part[sgn > 0] = np.nextafter(part[sgn > 0], np.inf)
            part[sgn < 0] = np.nextafter(part[sgn < 0], -np.inf)
        om.change_E(re_ + 1j * im_)
    st = om.bicgstab(100000, 1e-10)
    assert st == O.CONVERGED
    it = om.ITERATION
    om.close()
    oc.close()
    return inc_index, k, it


def cfg3_tight_spread(nperturb=5, workers=6):
    """The spread of the tol-1e-10 iteration count of cfg 3 (incidences 0 and 7) under
    one-ulp perturbations of E, on the GPU's grid."""
    import multiprocessing as mp
    jobs = [(i, k) for i in (0, 7) for k in range(nperturb + 1)]
    with mp.get_context("spawn").Pool(workers) as pool:
        rows = pool.map(_tight_count, jobs)
    arr = np.array(rows, np.int32)
    np.savez_compressed(os.path.join(HERE, "iters_spread_cfg3_tight.npz"), rows=arr, tol=1e-10)
    for i in (0, 7):
        its = arr[arr[:, 0] == i, 2]
        print(f"cfg3 incidence {i} at tol 1e-10: {sorted(its.tolist())}", flush=True)


JOBS = {
    "cfg3_spread": cfg3_tight_spread,
    "spread": iteration_spread,
    "cfg2_ref": reference_cfg2,
    "cfg2": lambda: oracle_tight("solve_cfg2_tight.npz", 2, 0),
    "cfg4": lambda: oracle_tight("solve_cfg4_tight.npz", 4, 0),
    "cfg3_0": lambda: oracle_tight("solve_cfg3_inc0_tight.npz", 3, 0),
    "cfg3_7": lambda: oracle_tight("solve_cfg3_inc7_tight.npz", 3, 7),
}


def main(names):
    for n in names or list(JOBS):
        JOBS[n]()


if __name__ == "__main__":
    main(sys.argv[1:])
