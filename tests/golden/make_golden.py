"""Generate the golden fixtures in this folder from the reference itself.

Builds oracle/_ref/ref_driver -- the reference's own AProductCore.cpp,
DDAModel.cpp, tools.cpp, ... compiled unchanged from the reference checkout
(oracle/Makefile's REF_ROOT, which the environment may set) with the
CPU stand-ins for cuFFT and the CUDA runtime in oracle/ref_shim -- and runs it
on seeded inputs.  Each fixture stores its inputs and the reference's outputs:

  ldr.npz          LDR_inter (AProductCore.cpp:588-623) at a set of offsets
  aprod_*.npz      Aproduct / Aproductwithalb (AProductCore.cpp:697-758,
                   DDAModel.cpp:577-586) of seeded vectors
  aprodper_*.npz   the same on the periodic core (AProductCore.cpp:251-536)
  aprodfcd_*.npz   the same with the FCD tensor (AProductCore.cpp:625-695); its
                   Si/Ci tables are written the way SiCi/SiCi.py writes them
  solve_*.npz      bicgstab + update_E_in_structure (DDAModel.cpp:131-260,
                   567-575): ITERATION, the printed Error, P, Einternal
  text_*/          the reference's text files of a solved structure
                   (CoreStructure.cpp:155-185, DDAModel.cpp:589-697,
                   main.cpp:282-289) with text_*.npz holding what they print
  field_*.npz      a solve, then the point-field objective
                   ObjPointEDDAModel::GetVal (ObjDDAModel.cpp:20-96) at
                   off-lattice points: |E_ext(r) - sum_i A(r - d R_i) P_i|

Run from the repository root:  python tests/golden/make_golden.py
It needs the reference checkout, so it runs where that checkout exists; the
fixtures it writes are committed and travel with the tests.
"""
from __future__ import annotations

import math
import os
import re
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "topo-dda-forwin64_gb300"))
from tdda import lattice  # noqa: E402

DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_driver")


def build_driver():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)


def write_input(path, mode, Nx, Ny, Nz, R, d, lam, nback, material, nK, E0, nE0, max_it, max_err,
                diel_old, vecs):
    R = np.ascontiguousarray(R, np.int32).reshape(-1)
    N = R.size // 3
    material = np.asarray(material, np.complex128)
    with open(path, "wb") as f:
        f.write(struct.pack("<5i", mode, Nx, Ny, Nz, N))
        f.write(struct.pack("<3d", d, lam, nback))
        f.write(struct.pack("<i", material.size))
        f.write(material.astype("<c16").tobytes())
        f.write(np.asarray(nK, "<f8").tobytes())
        f.write(struct.pack("<d", E0))
        f.write(np.asarray(nE0, "<f8").tobytes())
        f.write(struct.pack("<id", max_it, max_err))
        f.write(R.astype("<i4").tobytes())
        f.write(np.asarray(diel_old, "<f8").tobytes())
        f.write(struct.pack("<i", len(vecs)))
        for v in vecs:
            f.write(np.asarray(v).astype("<c16" if mode != 2 else "<f8").tobytes())


def write_sici_tables(folder):
    """The tables SiCi.cpp:8-25 reads (from .\\SiCi\\Si.txt and .\\SiCi\\Ci.txt relative to the
    working directory, backslashes included), produced as SiCi/SiCi.py does: scipy's sici at
    0.1, 0.2, ..., 0.1 * 999999, written with str()."""
    from scipy.special import sici
    number, dis = 1000000, 0.1
    pos = np.linspace(dis, dis * (number - 1), number - 1)
    si, ci = sici(pos)
    for name, vals in (("Si", si), ("Ci", ci)):
        with open(os.path.join(folder, ".\\SiCi\\%s.txt" % name), "w") as f:
            f.write(str(number - 1) + "\n" + str(dis) + "\n")
            f.write("\n".join(str(v) for v in vals.tolist()))
            f.write("\n")


def run(mode, points=None, periodic=None, keep=None, **kw):
    with tempfile.TemporaryDirectory() as td:
        if mode == 5:
            write_sici_tables(td)
        fin, fout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        write_input(fin, mode, **kw)
        if periodic is not None:
            with open(fin, "ab") as f:
                f.write(struct.pack("<2i2d", int(periodic[0]), int(periodic[1]), float(periodic[2]),
                                    float(periodic[3])))
        if points is not None:
            pts = np.ascontiguousarray(points, "<f8").reshape(-1, 3)
            with open(fin, "ab") as f:
                f.write(struct.pack("<i", pts.shape[0]))
                f.write(pts.tobytes())
        pr = subprocess.run([DRIVER, fin, fout], capture_output=True, text=True, check=True, cwd=td)
        with open(fout, "rb") as f:
            raw = f.read()
        if keep is not None:  # copy the files the reference wrote into its working directory
            import shutil
            os.makedirs(keep, exist_ok=True)
            for name in os.listdir(td):
                if name.endswith(".txt") and "SiCi" not in name:
                    shutil.copy(os.path.join(td, name), os.path.join(keep, name))
    return raw, pr.stdout


def case_kw(w: lattice.Workload, inc=None, max_it=10000, max_err=1e-5):
    inc = inc or w.incidences[0]
    return dict(Nx=w.Nx, Ny=w.Ny, Nz=w.Nz, R=w.R, d=w.d, lam=w.lam, nback=w.nback,
                material=w.material, nK=inc.nK, E0=inc.E0, nE0=inc.nE0, max_it=max_it,
                max_err=max_err, diel_old=w.diel_old)


def inputs_dict(w: lattice.Workload, inc=None):
    inc = inc or w.incidences[0]
    return dict(box=np.array([w.Nx, w.Ny, w.Nz], np.int32), R=w.R, d=w.d, lam=w.lam, nback=w.nback,
                material=w.material, nK=inc.nK, E0=inc.E0, nE0=inc.nE0, diel_old=w.diel_old)


def small_workload(name, Nx, Ny, Nz, seed, em=4.0 + 0.1j, d=10.0, lam=500.0, keep=1.0,
                   shuffle=False):
    rng = np.random.Generator(np.random.PCG64(seed))
    R = lattice.bulk(Nx, Ny, Nz).reshape(-1, 3)
    if keep < 1.0:
        R = R[rng.random(R.shape[0]) < keep]
    if shuffle:
        R = R[rng.permutation(R.shape[0])]
    rho = rng.random(R.shape[0])
    return lattice.Workload(name=name, Nx=Nx, Ny=Ny, Nz=Nz, d=d, lam=lam,
                            material=np.array([1.0 + 0j, em]), rho=rho,
                            R=np.ascontiguousarray(R.ravel(), np.int32),
                            incidences=[lattice.XPOL_Z])


def rand_vec(n, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    return (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex128)


def gen_ldr():
    pts = np.array([[10, 0, 0], [0, 0, 0], [0, 10, 0], [0, 0, 10], [10, 20, -30], [-50, 30, 70],
                    [3.5, -7.25, 11.0], [190, -190, 90], [-10, -10, -10], [400, 0, 0]], np.float64)
    w = small_workload("ldr", 2, 2, 2, 7)
    raw, _ = run(2, **case_kw(w), vecs=list(pts))
    K = struct.unpack_from("<d", raw, 0)[0]
    vals = np.frombuffer(raw, "<c16", offset=8).reshape(-1, 6)
    np.savez(os.path.join(HERE, "ldr.npz"), lam=w.lam, K=K, points=pts, tensors=vals)
    print("ldr: K=%.12g xx(10,0,0)=%s" % (K, vals[0, 0]))


def gen_aprod(name, w: lattice.Workload, nvec, seed):
    N = w.N
    vecs = [rand_vec(3 * N, seed + v) for v in range(nvec)]
    raw, _ = run(0, **case_kw(w), vecs=vecs)
    off = 0
    Rout = np.frombuffer(raw, "<i4", count=3 * N, offset=off)
    off += 12 * N
    al = np.frombuffer(raw, "<c16", count=3 * N, offset=off)
    off += 48 * N
    ys, yws = [], []
    for _ in range(nvec):
        ys.append(np.frombuffer(raw, "<c16", count=3 * N, offset=off))
        off += 48 * N
        yws.append(np.frombuffer(raw, "<c16", count=3 * N, offset=off))
        off += 48 * N
    assert np.array_equal(Rout, w.R), "reference reordered the dipoles"
    np.savez_compressed(os.path.join(HERE, f"aprod_{name}.npz"), **inputs_dict(w), al=al, b=np.array(vecs),
             y=np.array(ys), y_alb=np.array(yws))
    print(f"aprod_{name}: N={N} |y|={np.linalg.norm(ys[0]):.6g}")


def gen_text(name, w: lattice.Workload):
    N = w.N
    folder = os.path.join(HERE, f"text_{name}")
    raw, _ = run(6, keep=folder, **case_kw(w), vecs=[])
    off = 12 * N + 48 * N
    it = struct.unpack_from("<i", raw, off)[0]
    off += 4
    P = np.frombuffer(raw, "<c16", count=3 * N, offset=off)
    off += 48 * N
    Ein = np.frombuffer(raw, "<c16", count=3 * N, offset=off)
    inc = w.incidences[0]
    np.savez_compressed(os.path.join(HERE, f"text_{name}.npz"), box=np.array([w.Nx, w.Ny, w.Nz], np.int32),
                        R=w.R, diel_old=w.diel_old, d=w.d, nK=inc.nK, nE0=inc.nE0, P=P, Einternal=Ein)
    print(f"text_{name}: N={N} files={sorted(os.listdir(folder))}")


def gen_aprod_fcd(name, w: lattice.Workload, nvec, seed):
    N = w.N
    vecs = [rand_vec(3 * N, seed + v) for v in range(nvec)]
    raw, _ = run(5, **case_kw(w), vecs=vecs)
    off = 12 * N
    al = np.frombuffer(raw, "<c16", count=3 * N, offset=off)
    off += 48 * N
    ys, yws = [], []
    for _ in range(nvec):
        ys.append(np.frombuffer(raw, "<c16", count=3 * N, offset=off))
        off += 48 * N
        yws.append(np.frombuffer(raw, "<c16", count=3 * N, offset=off))
        off += 48 * N
    np.savez_compressed(os.path.join(HERE, f"aprodfcd_{name}.npz"), **inputs_dict(w), al=al, b=np.array(vecs),
                        y=np.array(ys), y_alb=np.array(yws))
    print(f"aprodfcd_{name}: N={N} |y|={np.linalg.norm(ys[0]):.6g}")


def gen_aprod_periodic(name, w: lattice.Workload, periodic, nvec, seed):
    N = w.N
    vecs = [rand_vec(3 * N, seed + v) for v in range(nvec)]
    raw, _ = run(4, periodic=periodic, **case_kw(w), vecs=vecs)
    off = 12 * N
    al = np.frombuffer(raw, "<c16", count=3 * N, offset=off)
    off += 48 * N
    ys, yws = [], []
    for _ in range(nvec):
        ys.append(np.frombuffer(raw, "<c16", count=3 * N, offset=off))
        off += 48 * N
        yws.append(np.frombuffer(raw, "<c16", count=3 * N, offset=off))
        off += 48 * N
    np.savez_compressed(os.path.join(HERE, f"aprodper_{name}.npz"), **inputs_dict(w), al=al, b=np.array(vecs),
                        y=np.array(ys), y_alb=np.array(yws), periodic=np.array(periodic, np.float64))
    print(f"aprodper_{name}: N={N} periodic={periodic} |y|={np.linalg.norm(ys[0]):.6g}")


def gen_solve(name, w: lattice.Workload, inc=None, P0=None, Ein=None, max_it=10000, max_err=1e-5):
    N = w.N
    vecs = []
    if P0 is not None:
        vecs.append(P0)
    if Ein is not None:
        vecs.append(Ein)
    raw, out = run(1, **case_kw(w, inc, max_it, max_err), vecs=vecs)
    off = 12 * N
    al = np.frombuffer(raw, "<c16", count=3 * N, offset=off)
    off += 48 * N
    it = struct.unpack_from("<i", raw, off)[0]
    off += 4
    P = np.frombuffer(raw, "<c16", count=3 * N, offset=off)
    off += 48 * N
    Ein_out = np.frombuffer(raw, "<c16", count=3 * N, offset=off)
    m = re.findall(r"Error:\s*([-+0-9.eE]+)", out)
    err = float(m[-1]) if m else float("nan")
    extra = {}
    if P0 is not None:
        extra["P0"] = P0
    if Ein is not None:
        extra["E_rhs"] = Ein
    np.savez_compressed(os.path.join(HERE, f"solve_{name}.npz"), **inputs_dict(w, inc), iterations=it,
             error=err, P=P, Einternal=Ein_out, max_it=max_it, max_err=max_err, **extra)
    print(f"solve_{name}: N={N} iterations={it} error={err:.6g} P[0]={P[0]}")


def gen_field(name, w: lattice.Workload, points, inc=None):
    N = w.N
    pts = np.asarray(points, np.float64).reshape(-1, 3)
    raw, _ = run(3, points=pts, **case_kw(w, inc), vecs=[])
    off = 12 * N + 48 * N
    it = struct.unpack_from("<i", raw, off)[0]
    off += 4
    P = np.frombuffer(raw, "<c16", count=3 * N, offset=off)
    off += 96 * N
    absE = np.frombuffer(raw, "<f8", count=pts.shape[0], offset=off)
    np.savez_compressed(os.path.join(HERE, f"field_{name}.npz"), **inputs_dict(w, inc), iterations=it, P=P,
                        points=pts, absE=absE)
    print(f"field_{name}: N={N} iterations={it} |E|={absE}")


def main():
    build_driver()
    gen_ldr()
    gen_aprod("box6x5x4", small_workload("box6x5x4", 6, 5, 4, 11), 2, 100)
    gen_aprod("sparse8x7x5", small_workload("sparse8x7x5", 8, 7, 5, 12, keep=0.6, shuffle=True), 1, 200)
    gen_aprod("box14x12x8", small_workload("box14x12x8", 14, 12, 8, 13, em=6.25 + 0.05j, lam=600.0), 1, 300)
    # the plain FP64 parity workload: 20x20x10, rho~U[0,1], eps_m=4+0.1i, x-pol along +z, tol 1e-5
    gen_solve("cfg1", lattice.config(1))
    # the same workload solved to 1e-10: the regime where solutions of two implementations
    # that differ only in rounding agree to ~1e-10 (at 1e-5 they differ by O(1e-5))
    gen_solve("cfg1_tight", lattice.config(1), max_err=1e-10)
    # oblique incidence on a sparse, shuffled lattice with a real-valued material
    ws = small_workload("sparse10x9x6", 10, 9, 6, 14, em=2.25 + 0j, keep=0.7, shuffle=True)
    th = math.radians(30.0)
    inc = lattice.Incidence(np.array([math.sin(th), 0.0, math.cos(th)]), lattice.n_e_perp_in_xz(th))
    gen_solve("sparse10x9x6", ws, inc)
    # warm start + a replaced right-hand side (the adjoint's change_E / InitializeP)
    wa = small_workload("adj8x8x4", 8, 8, 4, 15)
    gen_solve("adj8x8x4", wa, P0=0.01 * rand_vec(3 * wa.N, 400), Ein=rand_vec(3 * wa.N, 500))
    # periodic cores: a unit cell repeated with its own period, and a sparse cell in a wider
    # non-square array
    gen_aprod_periodic("cell6x5x3", small_workload("cell6x5x3", 6, 5, 3, 16), (3, 3, 60.0, 50.0), 2, 600)
    gen_aprod_periodic("sparse5x4x3", small_workload("sparse5x4x3", 5, 4, 3, 17, keep=0.7, shuffle=True),
                       (5, 2, 75.0, 52.0), 1, 700)
    # the FCD tensor on a box and on a sparse lattice
    gen_aprod_fcd("box6x5x4", small_workload("box6x5x4", 6, 5, 4, 11), 1, 800)
    gen_aprod_fcd("sparse7x6x4", small_workload("sparse7x6x4", 7, 6, 4, 18, em=2.25 + 0.0j, lam=620.0, keep=0.6,
                                                  shuffle=True), 1, 900)
    # the reference's text files of a small solved structure (densities with many digits, a
    # shuffled sparse lattice)
    gen_text("sparse4x3x2", small_workload("sparse4x3x2", 4, 3, 2, 19, keep=0.8, shuffle=True))
    # the point field of the solved cfg 1 structure: above the centre (the topology objective's
    # point), beside, below, far off, and inside the box between lattice sites
    gen_field("cfg1", lattice.config(1), [[95.0, 95.0, 190.0], [-50.0, 95.0, 45.0], [95.0, 95.0, -80.0],
                                          [300.0, -100.0, 400.0], [95.0, 95.0, 45.0], [12.5, 3.0, 51.0]])
    # the same on the sparse lattice under oblique incidence (every n_K component in E_ext)
    gen_field("sparse10x9x6", ws, [[45.0, 40.0, 150.0], [-30.0, 0.0, 25.0], [140.0, 100.0, -40.0],
                                   [47.5, 42.5, 27.5]], inc)


if __name__ == "__main__":
    main()
