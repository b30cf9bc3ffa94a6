"""Timing runs of the reference's own code (test and measurement infrastructure only).

Two builds of the reference's solve path, made by oracle/Makefile (`timers-if-present`)
from its sources (the checkout, or the copy `make -C oracle stage` leaves in
baseline/_ref):

  oracle/_ref/ref_timer   AProductCore.cpp, DDAModel.cpp, ... against the CPU stand-ins of
                          oracle/ref_shim, with Bluestein's algorithm for the prime lengths
                          of the reference's 2N - 1 FFT grid: the reference's host path on
                          one core;
  oracle/_ref/ref_cufft   the same sources against the CUDA runtime and cuFFT, kernel.cu
                          built for sm_103a: the reference's own GPU build, with its
                          host<->device copies per product (AProductCore.cpp:697-758).

Both run ref_driver.cpp's mode 7: the constructor AProductCore + DDAModel, `reps`
A-products of a seeded vector, then optionally one BiCGSTAB solve from P = 0
(DDAModel.cpp:131-260).  Only bench.py's reference arm uses this module.
"""
from __future__ import annotations

import os
import re
import struct
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TIMER = os.path.join(HERE, "_ref", "ref_timer")
CUFFT = os.path.join(HERE, "_ref", "ref_cufft")


def available(path: str) -> bool:
    return os.path.isfile(path) and os.access(path, os.X_OK)


def write_input(path, w, inc, max_it, tol, vec, reps, solve):
    """ref_driver.cpp's input layout (mode 7): box, spacing, wavelength, materials,
    incidence, stopping rule, lattice R, densities, one vector, reps, solve flag."""
    R = np.ascontiguousarray(w.R, np.int32).reshape(-1)
    N = R.size // 3
    mat = np.asarray(w.material, np.complex128)
    with open(path, "wb") as f:
        f.write(struct.pack("<5i", 7, w.Nx, w.Ny, w.Nz, N))
        f.write(struct.pack("<3d", w.d, w.lam, w.nback))
        f.write(struct.pack("<i", mat.size))
        f.write(mat.astype("<c16").tobytes())
        f.write(np.asarray(inc.nK, "<f8").tobytes())
        f.write(struct.pack("<d", inc.E0))
        f.write(np.asarray(inc.nE0, "<f8").tobytes())
        f.write(struct.pack("<id", max_it, tol))
        f.write(R.astype("<i4").tobytes())
        f.write(np.asarray(w.diel_old, "<f8").tobytes())
        f.write(struct.pack("<i", 1))
        f.write(np.asarray(vec, np.complex128).astype("<c16").tobytes())
        f.write(struct.pack("<2i", reps, 1 if solve else 0))


def seeded_vector(n3: int, seed: int = 7) -> np.ndarray:
    rng = np.random.Generator(np.random.PCG64(seed))
    return rng.standard_normal(n3) + 1j * rng.standard_normal(n3)


class Run:
    """One prepared input; start() launches the binary, finish() waits and parses."""

    def __init__(self, binary, w, inc, max_it, tol, reps, solve, env=None):
        self.td = tempfile.TemporaryDirectory()
        self.fin = os.path.join(self.td.name, "in.bin")
        self.fout = os.path.join(self.td.name, "out.bin")
        write_input(self.fin, w, inc, max_it, tol, seeded_vector(3 * w.N), reps, solve)
        self.binary, self.reps, self.env = binary, reps, env
        self.proc = None

    def start(self):
        self.proc = subprocess.Popen([self.binary, self.fin, self.fout], cwd=self.td.name, env=self.env,
                                     stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)

    def finish(self, timeout=None) -> dict:
        out, err = self.proc.communicate(timeout=timeout)
        try:
            if self.proc.returncode != 0:
                raise RuntimeError(f"{os.path.basename(self.binary)} exited {self.proc.returncode}: {err[-500:]}")
            with open(self.fout, "rb") as f:
                raw = f.read()
        finally:
            self.td.cleanup()
        ctor = struct.unpack_from("<d", raw, 0)[0]
        aprod = list(struct.unpack_from(f"<{self.reps}d", raw, 8))
        it, solve_s = struct.unpack_from("<id", raw, 8 + 8 * self.reps)
        m = re.findall(r"Error:\s*([0-9.eE+-]+)", out)
        return {"ctor_s": ctor, "aprod_s": aprod, "iterations": it, "solve_s": solve_s,
                "error": float(m[-1]) if m else None}


def run_many(binary, w, inc, max_it, tol, reps, solve, copies, timeout=None) -> list:
    """`copies` independent processes of the binary at once (one per host core)."""
    env = dict(os.environ, OMP_NUM_THREADS="1")
    runs = [Run(binary, w, inc, max_it, tol, reps, solve, env) for _ in range(copies)]
    for r in runs:
        r.start()
    return [r.finish(timeout) for r in runs]
