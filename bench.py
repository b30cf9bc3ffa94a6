"""Benchmark of the DDA solve hot path: converged solves/s at rel. residual 1e-5.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (one step = one converged solve): the mixed-precision single-solve lattice
64x64x16 dipoles (65,536; FFT grid 128x128x32), d = 10 nm, lambda = 600 nm, rho ~ U[0,1]
seeded then 3x3x3 box filtered, eps_m = 6.25+0.05i, x-polarised plane wave along +z,
LDR polarisability, BiCGSTAB to |r|/|E| <= 1e-5.  Data are seeded synthetic (no dataset).

ours       FP32 FFT convolution + Krylov vectors, double-float dot sums, the residual of
           the FP64 vectors from a double-float (~44-bit) product, iterative refinement
           (value); the plain FP64 solve of the same lattice is
           timed beside it (fp64).  Inputs are resident in HBM in the device-timed region;
           `e2e` is the same solve through the C ABI with host buffers.
reference  the reference's solve path run on the host cores: its own AProductCore.cpp /
           DDAModel.cpp sources (oracle/_ref/ref_timer, built from the reference's sources
           with CPU stand-ins for cuFFT), one process per core, one full converged solve in
           each; beside it the reference's own GPU build with cuFFT on this GPU
           (oracle/_ref/ref_cufft).  Where the reference's sources were not built, the
           oracle port of AProductCore::Aproduct + DDAModel::bicgstab, all host threads.

Multi-GPU: the solve does not shard; N ranks run N independent replicas (weak scaling).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "topo-dda-forwin64_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from tdda import lattice  # noqa: E402

METRIC = "solves/s & p99 latency, FP32+refine vs FP64 plain, same GB300, rel.res 1e-5"
UNIT = "solves/s"
TOL = 1e-5
MAX_IT = 10000
WORKLOAD = "mixed-precision single solve 64x64x16 (cfg 2)"


# --------------------------------------------------------------------------- helpers
def env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0")), \
        int(os.environ.get("WORLD_SIZE", "1"))


class Dist:
    """Barrier and max-reduction over ranks (torch.distributed when WORLD_SIZE > 1)."""

    def __init__(self):
        self.rank, self.local_rank, self.world = env_rank()
        self.pg = None
        if self.world > 1:
            import torch.distributed as td
            td.init_process_group("gloo")
            self.td = td

    def barrier(self):
        if self.world > 1:
            self.td.barrier()

    def max(self, x: float) -> float:
        if self.world == 1:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.td.destroy_process_group()


class Clocks:
    """nvidia-smi SM clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def pass_bytes(grid, Nx, Ny, Nz, N, s, fused=False):
    """Algorithmic bytes of the five A-product passes for one right-hand side.

    The canonical pass model, on the grid (Mx, My, Mz) actually used:
    the z-forward pass reads the 3N vector and writes 3 Nx Ny Mz grid entries, the
    y-forward pass reads those and writes 3 Nx My Mz, the x pass reads and writes
    3 Nx My Mz and reads the six Green components on the full grid (6 Mx My Mz,
    the canonical count; the folded layout actually stores 6 Hx Hy Hz), the inverse
    passes mirror the forward ones.  s = bytes per complex entry.  With fused z+y
    passes (3 kernels per product) entries 0 and 3 are the fused kernels."""
    Mx, My, Mz = grid
    zf = 3 * N + 3 * Nx * Ny * Mz
    yf = 3 * Nx * Ny * Mz + 3 * Nx * My * Mz
    xp = 2 * 3 * Nx * My * Mz + 6 * Mx * My * Mz
    if fused:  # k_zyfwd / k_yzinv: the 3N vector in, the 3 Nx My Mz plane out (and back)
        zy = 3 * N + 3 * Nx * My * Mz
        return [zy * s, 0, xp * s, zy * s, 0]
    return [zf * s, yf * s, xp * s, yf * s, zf * s]


# GB300 FP64 (CUDA-core) rate, nominal: the measured-peaks file holds no FP64 figure
FP64_NOMINAL_TFLOPS = 1.25


def aprod_flops(grid):
    """Canonical FP64 flops of one A-product for one right-hand side: six complex 3-D FFTs
    counted unpruned at 5 G log2 G each, plus the symmetric 3x3 spectral product at 72 G,
    G = Mx My Mz (the grid actually used)."""
    G = grid[0] * grid[1] * grid[2]
    return 6 * 5 * G * math.log2(G) + 72 * G


def pass_bytes_total(N, B, s):
    """Canonical bytes of one A-product over B right-hand sides: (84 B + 48) N s."""
    return (84 * B + 48) * N * s


def ncu_traffic(key):
    """DRAM bytes per launch of a kernel from the committed ncu summary table, or None."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        for line in f:
            parts = line.split("#")[0].split()
            if len(parts) == 2 and parts[0] == key:
                return int(parts[1])
    return None


def pass_names(core, precision):
    """Kernel of each profile slot, from the library ("-" where a fused kernel covers it)."""
    return [n or "-" for n in core.pass_names(precision)]


# ------------------------------------------------------------------ CPU baseline
def cpu_model() -> str:
    """The host CPU's model name (lscpu / /proc/cpuinfo), or the platform's machine name."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.lower().startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for ln in f:
                if ln.lower().startswith(("model name", "cpu model")):
                    return ln.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.machine()


class CpuBaseline:
    """The reference's solve path on the host cores: `threads` independent solves of the
    workload (one per thread, the oracle's FP64 restatement of AProductCore::Aproduct +
    DDAModel::bicgstab, pinned bit-exact to the reference's own sources on the smaller
    fixtures), each a full converged BiCGSTAB solve to tol 1e-5 from P = 0.  The FFT grid
    is the smooth 2N grid with the zero halves pruned, which makes the port faster than
    the reference's own host path (prime 2N-1 lengths and an O(M) host scatter/gather per
    product, AProductCore.cpp:697-758).  The operators (Green spectra) are built once,
    outside the sample, as the GPU path builds its core once."""

    def __init__(self, w, threads: int):
        import oracle as O

        self.O = O
        self.w = w
        self.threads = threads
        grid = tuple(lattice.smooth_size(2 * n - 1) for n in (w.Nx, w.Ny, w.Nz))
        inc = w.incidences[0]
        self.cores = [O.OracleCore(w.Nx, w.Ny, w.Nz, w.R, w.d, w.lam, w.material, grid=grid, pruned=True)
                      for _ in range(threads)]
        self.models = [O.OracleModel(c, inc.nK, inc.E0, inc.nE0, w.diel_old) for c in self.cores]
        self.zero = np.zeros(3 * w.N, np.complex128)

    def sample(self, iters: int = 0) -> dict:
        """One step: every thread runs one solve at once.  iters = 0: each solve runs to
        convergence (the measured sample); iters > 0: each stops after `iters` iterations
        (warm-up only)."""
        for m in self.models:
            m.InitializeP(self.zero)
            m.ITERATION = 0
        status = [None] * self.threads

        def run(k):
            status[k] = self.models[k].bicgstab(iters if iters > 0 else MAX_IT, TOL)  # releases the GIL

        th = [threading.Thread(target=run, args=(k,)) for k in range(self.threads)]
        t0 = time.perf_counter()
        for t in th:
            t.start()
        for t in th:
            t.join()
        wall = time.perf_counter() - t0
        if iters == 0 and any(st != self.O.CONVERGED for st in status):
            raise RuntimeError(f"CPU baseline solve did not converge: {status}")
        its = self.models[0].ITERATION
        return {"value": self.threads / wall, "unit": UNIT, "cores": self.threads, "kind": "port",
                "cpu_model": cpu_model(),
                "sample": (f"{self.threads} threads x one full FP64 BiCGSTAB solve each of the same lattice "
                           f"to tol {TOL:g} ({its} iterations, {wall:.2f} s wall); the oracle port of "
                           f"the reference's solve path on the 2N grid with pruned zero halves"),
                "sample_wall_s": wall, "iterations": its}


def run_reference_code(args, w, threads: int) -> dict:
    """The reference's own code (oracle/_ref/ref_timer: its AProductCore.cpp, DDAModel.cpp, ...
    compiled unchanged against the CPU stand-ins for cuFFT and the CUDA runtime), timed on
    the host cores with one independent process per core.  Each warm-up and timed step runs,
    in every process, the constructor and one A-product of the workload; a last step runs,
    in every process, the constructor and one full BiCGSTAB solve to tol 1e-5 from P = 0.
    The line's value is that full step's: processes / median solve time (measured, not
    extrapolated).  The product steps give the extrapolated rate beside it, processes /
    (median product time x the 2 its + 3 products of the reference's solve).  Then, where
    it was built, the reference's GPU build (oracle/_ref/ref_cufft: kernel.cu for sm_103a
    with cuFFT) runs the same constructor, products and solve on the GPU."""
    import ref_timing as RT

    inc = w.incidences[0]
    for _ in range(args.warmup):
        RT.run_many(RT.TIMER, w, inc, MAX_IT, TOL, 1, False, threads)
    prods, step_s = [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        rs = RT.run_many(RT.TIMER, w, inc, MAX_IT, TOL, 1, False, threads)
        step_s.append(time.perf_counter() - t0)
        prods += [r["aprod_s"][0] for r in rs]
    t0 = time.perf_counter()
    full = RT.run_many(RT.TIMER, w, inc, MAX_IT, TOL, 0, True, threads)
    full_wall = time.perf_counter() - t0
    its = full[0]["iterations"]
    solve_s = statistics.median(r["solve_s"] for r in full)
    value = threads / solve_s
    extrap = threads / (statistics.median(prods) * (2 * its + 3))
    sample = (f"reference's own AProductCore/DDAModel sources (oracle/_ref/ref_timer, CPU stand-ins for cuFFT "
              f"with Bluestein on its {2 * w.Nx - 1}x{2 * w.Ny - 1}x{2 * w.Nz - 1} grid), {threads} processes, one per "
              f"core: one full BiCGSTAB solve each to tol {TOL:g} from P = 0 ({its} iterations, median "
              f"{solve_s:.1f} s, {full_wall:.1f} s wall); {args.steps} steps of one A-product per process "
              f"(median {1e3 * statistics.median(prods):.0f} ms) give {extrap:.3f} solves/s extrapolated")
    out = {"value": value, "kind": "reference", "cores": threads, "cpu_model": cpu_model(), "sample": sample,
           "iterations": its, "error": full[0]["error"], "solve_s_median": solve_s,
           "aprod_ms_median": 1e3 * statistics.median(prods), "extrapolated_value": extrap,
           "ms_per_step": 1e3 * statistics.median(step_s)}
    import torch
    if RT.available(RT.CUFFT) and torch.cuda.is_available():
        g = RT.run_many(RT.CUFFT, w, inc, MAX_IT, TOL, 20, True, 1)[0]
        out["gpu_cufft_build"] = {
            "what": "the reference's AProductCore.cpp + DDAModel.cpp + kernel.cu built for sm_103a with cuFFT "
                    "(oracle/_ref/ref_cufft), one solve on this GPU; host<->device copies per product included "
                    "(its design)",
            "value": 1.0 / g["solve_s"], "unit": UNIT, "solve_s": g["solve_s"], "iterations": g["iterations"],
            "error": g["error"], "aprod_ms_median": 1e3 * statistics.median(g["aprod_s"][1:]),
            "ctor_s": g["ctor_s"]}
    return out


def run_reference(args, dist: Dist):
    """The reference's CPU solve path timed on the host cores (rank 0 only): the reference's
    own code where it was built on this host (run_reference_code), else the oracle port."""
    if dist.rank != 0:
        return
    w = lattice.config(2)
    threads = os.cpu_count() or 1
    import ref_timing as RT
    if RT.available(RT.TIMER):
        r = run_reference_code(args, w, threads)
        line = {"impl": "reference", "metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms_per_step"],
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
                "data": "synthetic (seeded)",
                "config": {"workload": WORKLOAD, "lattice": [w.Nx, w.Ny, w.Nz], "dipoles": w.N, "tol": TOL,
                           "grid": [2 * n - 1 for n in (w.Nx, w.Ny, w.Nz)]},
                "cpu_baseline": {k: r[k] for k in ("value", "kind", "cores", "cpu_model", "sample")},
                "reference_solve": {k: r[k] for k in ("iterations", "error", "solve_s_median", "aprod_ms_median",
                                                      "extrapolated_value")},
                "e2e": {"value": r["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        line["cpu_baseline"]["unit"] = UNIT
        if "gpu_cufft_build" in r:
            line["gpu_cufft_build"] = r["gpu_cufft_build"]
        print(json.dumps(line), flush=True)
        return
    iters = max(1, args.cpu_iters)
    cpu = CpuBaseline(w, threads)
    for _ in range(args.warmup):
        cpu.sample(iters)
    vals = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        r = cpu.sample(0)
        vals.append(r["value"])
    total = time.perf_counter() - t0
    v = statistics.median(vals)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
            "data": "synthetic (seeded)",
            "config": {"workload": WORKLOAD, "lattice": [w.Nx, w.Ny, w.Nz], "dipoles": w.N, "tol": TOL,
                       "grid": [lattice.smooth_size(2 * n - 1) for n in (w.Nx, w.Ny, w.Nz)]},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "cpu_model": r["cpu_model"], "sample": r["sample"]},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------- ours
def pinned_c128(n: int) -> np.ndarray:
    import torch
    return torch.zeros(n, dtype=torch.complex128, pin_memory=True).numpy()


def pinned_f64(n: int) -> np.ndarray:
    import torch
    return torch.zeros(n, dtype=torch.float64, pin_memory=True).numpy()


def time_batch(tdda, torch, w, incs, precision, steps, dev, flush_l2, keep_P=False):
    """Solve len(incs) right-hand sides of one lattice in one batched solve per step
    (keep_P: the result's polarisations in out["P"])."""
    core = tdda.AProductCore(w.Nx, w.Ny, w.Nz, w.R, w.d, w.lam, w.material, w.nback, max_rhs=len(incs), device=dev)
    fp32 = precision in (tdda.FP32_REFINE, tdda.FP32_JACOBI)
    tune = core.autotune(nrhs=len(incs), reps=10) if fp32 else None
    # the batch schedule (right-hand sides per launch), timed on this core's FP32 products
    btune = core.autotune_batch(nrhs=len(incs), reps=5) if fp32 else None
    models = [tdda.DDAModel(core, inc.nK, inc.E0, inc.nE0, w.diel_old) for inc in incs]
    stream = torch.cuda.ExternalStream(core.stream(), device=dev)
    zero = pinned_c128(3 * w.N)

    def step():
        for m in models:
            m.InitializeP(zero)
        flush_l2()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        infos = tdda.solve_batch(models, precision, MAX_IT, TOL)
        e1.record(stream)
        e1.synchronize()
        if any(i["status"] != tdda.OK for i in infos):
            raise RuntimeError(f"batched solve did not converge: {infos}")
        return e0.elapsed_time(e1), infos

    step()
    runs = [step() for _ in range(steps)]
    ms = [r[0] for r in runs]
    infos = runs[-1][1]
    n32 = 2 * max(i["inner_iterations"] for i in infos) + 2 * max(i["outer_iterations"] for i in infos)
    prof = core.profile_aproduct(tdda.FP32_REFINE if fp32 else tdda.FP64, len(incs), 5)
    out = {"rhs": len(incs), "value": len(incs) * steps / (sum(ms) / 1000.0), "unit": UNIT, "steps": steps,
           "ms_per_batch": sum(ms) / steps, "iterations": [i["iterations"] for i in infos],
           "pass_ms": prof, "kernels": pass_names(core, tdda.FP32_REFINE if fp32 else tdda.FP64),
           "grid": list(core.grid)}
    if tune:
        out["x_pass_autotune"] = tune
    if btune:
        out["batch_schedule_autotune"] = btune
    if keep_P:
        out["P"] = [m.get_P() for m in models]
    for m in models:
        m.close()
    core.close()
    return out, prof, n32


def required_bytes(grid, Nx, N, s, fused, nrhs):
    """Bytes each kernel of one A-product over nrhs right-hand sides must move, as stored:
    the same grid and vector terms as pass_bytes, but the x pass reads the folded Green
    table (6 Hx Hy Hz entries, H = M/2 + 1) once per launch instead of the canonical
    6 Mx My Mz.  Fused forms only (the compiled FP32 planes) and the five-pass form."""
    Mx, My, Mz = grid
    H = (Mx // 2 + 1) * (My // 2 + 1) * (Mz // 2 + 1)
    plane = 3 * Nx * My * Mz
    if fused:
        zy = (3 * N + plane) * s * nrhs
        return [zy, 0, (2 * plane * nrhs + 6 * H) * s, zy, 0]
    per = pass_bytes(grid, Nx, 0, 0, N, s, False)
    return [per[0] * nrhs, per[1] * nrhs, (2 * plane * nrhs + 6 * H) * s, per[3] * nrhs, per[4] * nrhs]


def pass_bytes_batch(w, grid, s, fused, nrhs):
    """Algorithmic bytes of each pass kernel of one A-product over nrhs right-hand sides:
    the grid and vector terms once per right-hand side, the Green read once per launch."""
    Mx, My, Mz = grid
    per = pass_bytes(grid, w.Nx, w.Ny, w.Nz, w.N, s, fused)
    green = 6 * Mx * My * Mz * s
    return [(b - green) * nrhs + green if k == 2 else b * nrhs for k, b in enumerate(per)]


def pass_rooflines(w, grid, prof, names, s, fused, nrhs, peak):
    """Every pass kernel of one A-product against the HBM roof (the bytes each kernel must
    move, over its CUDA-event time), and the whole product on the canonical five-pass
    count (84 B + 48) N s, over the summed time of the kernels that run it."""
    bk = pass_bytes_batch(w, grid, s, fused, nrhs)
    passes = []
    live = [k for k, name in enumerate(names) if name not in ("", "-")]
    for k in live:
        name = names[k]
        ach = bk[k] / (prof[k] * 1e-3) / 1e9
        passes.append({"kernel": name, "algorithmic_bytes": bk[k], "avg_ms": prof[k], "achieved": ach,
                       "frac": ach / peak})
    t = sum(prof[k] for k in live)
    canon = pass_bytes_total(w.N, nrhs, s)
    ach = canon / (t * 1e-3) / 1e9
    return passes, {"canonical_bytes": canon, "avg_ms": t, "achieved": ach, "frac": ach / peak,
                    "kernels": [names[k] for k in live]}


def batched_roofline(w, grid, prof, nrhs, s, peak, kernel, names):
    """Roofline of the x pass (the largest) for nrhs right-hand sides: the Green tensor is
    read once per launch, the grid once per right-hand side.  `passes` and `aproduct`
    give the other pass kernels and the whole product."""
    b = pass_bytes_batch(w, grid, s, True, nrhs)[2]
    t = prof[2]
    ach = b / (t * 1e-3) / 1e9
    req = required_bytes(grid, w.Nx, w.N, s, True, nrhs)[2]
    passes, whole = pass_rooflines(w, grid, prof, names, s, names[1] == "-", nrhs, peak)
    return {"kernel": kernel, "bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
            "algorithmic_bytes": b, "avg_ms": t, "required_bytes": req,
            "frac_required": req / (t * 1e-3) / 1e9 / peak, "traffic": ncu_traffic(f"{kernel}:fp32:cfg3x{nrhs}"),
            "passes": passes, "aproduct": whole}


def run_serving(tdda, stream, precision, workers, budget, dev):
    """Replay the request stream in real time through the serving loop."""
    srv = tdda.Server(hbm_budget_bytes=budget, workers=workers, precision=precision, max_it=MAX_IT, tol=TOL,
                      max_group=8, device=dev)
    t0 = srv.clock()
    ids = []
    for r in stream:
        diel = r.diel_old()
        delay = t0 + r.t_arrival - srv.clock()
        if delay > 0:
            time.sleep(delay)
        ids.append(srv.submit(r.Nx, r.Ny, r.Nz, lattice.bulk(r.Nx, r.Ny, r.Nz), 10.0, r.lam,
                              np.array([1.0, r.eps_m]), diel, r.incidences))
    infos = [srv.result(i, with_P=False)[0] for i in ids]
    peak = srv.stats()["peak_bytes"]
    counters = srv.counters()
    srv.close()
    ok = [i["state"] == tdda.REQ_DONE for i in infos]
    lat = np.array([(i["t_done"] - i["t_submit"]) * 1e3 for i in infos])
    span = max(i["t_done"] for i in infos) - min(i["t_submit"] for i in infos)
    rhs = sum(len(r.incidences) for r in stream)
    classes = {"N<32k": lambda n: n < 32768, "32k<=N<128k": lambda n: 32768 <= n < 131072,
               "N>=128k": lambda n: n >= 131072}
    per = {}
    for name, f in classes.items():
        sel = [l for l, r in zip(lat, stream) if f(r.N)]
        if sel:
            per[name] = {"requests": len(sel), "p50_ms": float(np.percentile(sel, 50)),
                         "p99_ms": float(np.percentile(sel, 99))}
    # steady state: right-hand sides completed between the 10th and the 90th percentile of the
    # completion times, over that window (the ramp-up and the tail of slow requests excluded)
    done = sorted((i["t_done"], len(r.incidences)) for i, r in zip(infos, stream))
    lo, hi = done[len(done) // 10], done[(9 * len(done)) // 10]
    window = hi[0] - lo[0]
    mid = sum(n for t, n in done if lo[0] < t <= hi[0])
    shared = sum(1 for i, r in zip(infos, stream) if i["group"] > len(r.incidences))
    return {"requests": len(stream), "failed": int(len(ok) - sum(ok)), "rhs_solves": rhs,
            "value": rhs / span, "unit": UNIT, "requests_per_s": len(stream) / span, "makespan_s": span,
            "steady_state": {"value": mid / window if window > 0 else None, "unit": UNIT,
                             "window_s": window, "rhs_solves": mid},
            "requests_sharing_launches": shared, "counters": counters,
            "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99))},
            "latency_by_size": per, "peak_admitted_bytes": peak,
            "max_iterations": max(i["iterations"] for i in infos)}


def run_cfg1(tdda, torch, dev, steps=10):
    """The plain FP64 single-solve workload (20x20x10, rho ~ U[0,1]), solved with each
    precision: solves/s over `steps` solves after 3 warm-up solves (CUDA events)."""
    w = lattice.config(1)
    inc = w.incidences[0]
    core = tdda.AProductCore(w.Nx, w.Ny, w.Nz, w.R, w.d, w.lam, w.material, w.nback, device=dev)
    m = tdda.DDAModel(core, inc.nK, inc.E0, inc.nE0, w.diel_old)
    stream = torch.cuda.ExternalStream(core.stream(), device=dev)
    zero = np.zeros(3 * w.N, np.complex128)
    out = {"workload": "plain single solve 20x20x10 (cfg 1)", "dipoles": w.N}
    for name, prec in (("fp64", tdda.FP64), ("fp32_refine", tdda.FP32_REFINE), ("fp32_jacobi", tdda.FP32_JACOBI)):
        ms = []
        for k in range(3 + steps):
            m.InitializeP(zero)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            [info] = tdda.solve_batch([m], prec, MAX_IT, TOL)
            e1.record(stream)
            e1.synchronize()
            if k >= 3:
                ms.append(e0.elapsed_time(e1))
        out[name] = {"value": 1000.0 * steps / sum(ms), "unit": UNIT, "ms_p50": float(np.percentile(ms, 50)),
                     "iterations": info["iterations"], "true_residual": info.get("true_residual")}
    m.close()
    core.close()
    return out


def run_topo(tdda, iters):
    """The topology-optimisation workload: 80x80x20, forward + 3 adjoint solves batched per
    iteration, point |E|^2 objective 100 nm above the top centre, gradient ascent.  The loop
    runs `iters` steps with the FP32+refine solves; the design it reaches is then evaluated
    (forward + adjoint solves, gradient) once with each precision, so both are timed on the
    same structure."""
    from tdda import topo

    w = lattice.config(4)
    rng = np.random.Generator(np.random.PCG64(1234))
    dm = topo.DesignMap(w.Nx, w.Ny, 2.0)
    th0 = 0.4 + 0.2 * rng.random((dm.hx, dm.hy))
    r_obs = (w.d * (w.Nx - 1) / 2, w.d * (w.Ny - 1) / 2, w.d * (w.Nz - 1) + 100.0)
    loop = topo.TopoLoop(w.Nx, w.Ny, w.Nz, w.d, w.lam, w.material, th0, r_obs, precision=tdda.FP32_REFINE, tol=TOL)
    t0 = time.perf_counter()
    f, its = [], []
    for _ in range(iters):
        r = loop.step()
        f.append(r.objective)
        its.append(r.iterations)
    dt = time.perf_counter() - t0
    # the same loop with the Jacobi-preconditioned inner solves, from the same start, cold
    # and with the reference's heritage option (each step's solves start from the last ones)
    loops = {}
    for name, her in (("fp32_jacobi_loop", False), ("fp32_jacobi_heritage_loop", True)):
        jloop = topo.TopoLoop(w.Nx, w.Ny, w.Nz, w.d, w.lam, w.material, th0, r_obs, precision=tdda.FP32_JACOBI,
                              tol=TOL, origin_heritage=her, adjoint_heritage=her)
        t0 = time.perf_counter()
        fj, itj = [], []
        for _ in range(iters):
            rj = jloop.step()
            fj.append(rj.objective)
            itj.append(rj.iterations)
        dtj = time.perf_counter() - t0
        jloop.close()
        loops[name] = {"s_per_step": dtj / iters, "solves_per_s": 4 * iters / dtj, "objective_last": fj[-1],
                       "bicgstab_iterations_last": itj[-1]}
    final = {}
    for name, prec in (("fp32_refine", tdda.FP32_REFINE), ("fp32_jacobi", tdda.FP32_JACOBI), ("fp64", tdda.FP64)):
        loop.precision = prec
        loop.evaluate()  # warm-up: graphs and buffers of this precision
        t1 = time.perf_counter()
        e = loop.evaluate()
        final[name] = {"evaluate_s": time.perf_counter() - t1, "objective": e.objective,
                       "bicgstab_iterations": e.iterations}
    loop.close()
    return {"steps": iters, "s_per_step": dt / iters, "solves_per_s": 4 * iters / dt,
            "objective_first": f[0], "objective_last": f[-1], "bicgstab_iterations_last": its[-1],
            "final_design": final,
            **loops,
            "speedup_fp32_refine": final["fp64"]["evaluate_s"] / final["fp32_refine"]["evaluate_s"],
            "speedup_fp32_jacobi": final["fp64"]["evaluate_s"] / final["fp32_jacobi"]["evaluate_s"]}


def run_ours(args, dist: Dist):
    import torch

    import tdda

    dev = dist.local_rank
    torch.cuda.set_device(dev)
    w = lattice.config(2)
    inc = w.incidences[0]
    n3 = 3 * w.N
    core = tdda.AProductCore(w.Nx, w.Ny, w.Nz, w.R, w.d, w.lam, w.material, w.nback, max_rhs=1, device=dev)
    tune = core.autotune(nrhs=1, reps=20)  # the FP32 x pass's form and tile, timed on this core
    model = tdda.DDAModel(core, inc.nK, inc.E0, inc.nE0, w.diel_old)
    stream = torch.cuda.ExternalStream(core.stream(), device=dev)
    zero = pinned_c128(n3)
    P_host = pinned_c128(n3)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{dev}")  # > 129 MB of L2

    def flush_l2():
        flush.zero_()
        torch.cuda.synchronize(dev)

    def solve(prec):
        model.InitializeP(zero)  # P = 0, as a fresh DDAModel starts (DDAModel.cpp:42)
        flush_l2()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        info = model.solve_mixed(MAX_IT, TOL) if prec == tdda.FP32_REFINE else model.bicgstab(MAX_IT, TOL)
        e1.record(stream)
        e1.synchronize()
        if info["status"] != tdda.OK:
            raise RuntimeError(f"solve did not converge: {info}")
        return e0.elapsed_time(e1), info

    for _ in range(args.warmup):
        solve(tdda.FP32_REFINE)
    dist.barrier()
    torch.cuda.synchronize(dev)
    l0 = tdda.kernel_launches()
    with Clocks(dev) as ck:
        runs = [solve(tdda.FP32_REFINE) for _ in range(args.steps)]
    launches = tdda.kernel_launches() - l0
    ms = [r[0] for r in runs]
    info = runs[-1][1]
    t_max = dist.max(sum(ms))
    value = dist.world * args.steps / (t_max / 1000.0)
    P32 = model.get_P()  # the last timed FP32+refine solve

    # the plain FP64 solve of the same lattice, same timing rules
    k64 = max(3, min(args.steps, args.fp64_steps))
    solve(tdda.FP64)
    r64 = [solve(tdda.FP64) for _ in range(k64)]
    ms64 = [r[0] for r in r64]
    fp64_value = dist.world * k64 / (dist.max(sum(ms64)) / 1000.0)
    # the FP32+refine result's error against the FP64 solution of the same lattice (FP64
    # BiCGSTAB to 1e-10, untimed), beside the error the FP64 solve itself carries at tol 1e-5
    P64_tol = model.get_P()
    model.InitializeP(zero)
    model.bicgstab(MAX_IT, 1e-10)
    P64 = model.get_P()
    n64 = np.linalg.norm(P64)
    error_vs_fp64 = {"fp32_refine": float(np.linalg.norm(P32 - P64) / n64),
                     "fp64_at_tol": float(np.linalg.norm(P64_tol - P64) / n64),
                     "reference_solution": "FP64 BiCGSTAB of the same lattice to 1e-10"}

    # end to end through the C ABI with pinned host buffers: new densities and P0 in, P out
    rho_host = pinned_f64(n3)
    rho_host[:] = w.diel_old
    zero = pinned_c128(n3)
    h2d = n3 * 8 + n3 * 16    # the 3N densities uploaded by UpdateAlpha, P0 by InitializeP
    d2h = n3 * 16             # P
    for _ in range(1):
        model.UpdateAlpha(rho_host)
    e2e_s = []
    for _ in range(args.steps):
        flush_l2()
        t0 = time.perf_counter()
        model.UpdateAlpha(rho_host)
        model.InitializeP(zero)
        model.solve_mixed(MAX_IT, TOL)
        model._get(tdda.FIELD_P, out=P_host)
        e2e_s.append(time.perf_counter() - t0)
    e2e_value = dist.world * args.steps / dist.max(sum(e2e_s))

    # roofline of the dominant pass kernel (per-pass CUDA events on the core's stream)
    prof32 = core.profile_aproduct(tdda.FP32_REFINE, 1, 20)
    prof64 = core.profile_aproduct(tdda.FP64, 1, 5)
    n32 = 2 * info["inner_iterations"] + 2 * info["outer_iterations"]   # FP32 products per solve
    n64 = info["outer_iterations"] + 1                                  # FP64 residual products
    shares = [(n32 * t, "fp32", k) for k, t in enumerate(prof32)] + [(n64 * t, "fp64", k) for k, t in enumerate(prof64)]
    _, prec, k = max(shares)
    s = 8 if prec == "fp32" else 16
    pprec = tdda.FP32_REFINE if prec == "fp32" else tdda.FP64
    fused = core.pass_count(pprec) == 3
    names = pass_names(core, pprec)
    bytes_k = pass_bytes(core.grid, w.Nx, w.Ny, w.Nz, w.N, s, fused)[k]
    t_k = (prof32 if prec == "fp32" else prof64)[k]
    peaks = measured_peaks()
    achieved = bytes_k / (t_k * 1e-3) / 1e9
    req_k = required_bytes(core.grid, w.Nx, w.N, s, fused, 1)[k]
    traffic = ncu_traffic(f"{names[k]}:{prec}:cfg2")
    names32 = pass_names(core, tdda.FP32_REFINE)
    passes32, whole32 = pass_rooflines(w, core.grid, prof32, names32, 8, core.pass_count(tdda.FP32_REFINE) == 3, 1,
                                       peaks["hbm_gbs"])
    # the FP64 product against the FP64 ALU roof (its HBM bytes are far below that roof)
    f64 = aprod_flops(core.grid)
    t64 = sum(prof64)
    fp64_achieved = f64 / (t64 * 1e-3) / 1e12
    fp64_roof = {"kernels": "A-product (5 passes)", "bound": "fp64", "achieved": fp64_achieved,
                 "peak": FP64_NOMINAL_TFLOPS, "unit": "TFLOP/s", "frac": fp64_achieved / FP64_NOMINAL_TFLOPS,
                 "peak_source": "nominal", "canonical_flops": f64, "avg_ms": t64,
                 "hbm_bytes_canonical": pass_bytes_total(w.N, 1, 16),
                 "hbm_frac": pass_bytes_total(w.N, 1, 16) / (t64 * 1e-3) / 1e9 / peaks["hbm_gbs"]}

    # batched right-hand sides: the 96x96x24 lattice with its 8 incidences in one solve
    batched = None
    if not args.no_batched:
        w3 = lattice.config(3)
        b32, prof_b, _ = time_batch(tdda, torch, w3, w3.incidences, tdda.FP32_REFINE, args.batched_steps, dev, flush_l2,
                                    keep_P=True)
        b32["roofline"] = batched_roofline(w3, tuple(b32["grid"]), prof_b, len(w3.incidences), 8, peaks["hbm_gbs"],
                                           b32["kernels"][2], b32["kernels"])
        j32, _, _ = time_batch(tdda, torch, w3, w3.incidences, tdda.FP32_JACOBI, args.batched_steps, dev, flush_l2,
                               keep_P=True)
        b64, _, _ = time_batch(tdda, torch, w3, w3.incidences, tdda.FP64, 1, dev, flush_l2)
        # error of each FP32+refine result against the FP64 solution to 1e-10 (untimed)
        c3 = tdda.AProductCore(w3.Nx, w3.Ny, w3.Nz, w3.R, w3.d, w3.lam, w3.material, w3.nback,
                               max_rhs=len(w3.incidences), device=dev)
        m3 = [tdda.DDAModel(c3, i.nK, i.E0, i.nE0, w3.diel_old) for i in w3.incidences]
        tdda.solve_batch(m3, tdda.FP64, MAX_IT, 1e-10)
        for bx in (b32, j32):
            bx["error_vs_fp64"] = [float(np.linalg.norm(p32 - m.get_P()) / np.linalg.norm(m.get_P()))
                                   for p32, m in zip(bx.pop("P"), m3)]
        for m in m3:
            m.close()
        c3.close()
        batched = {"workload": "batched 8 RHS 96x96x24 (cfg 3)", "dipoles": w3.N, "fp32_refine": b32,
                   "fp64": {"value": b64["value"], "unit": UNIT, "iterations": b64["iterations"],
                            "ms_per_batch": b64["ms_per_batch"]},
                   "speedup_fp32_refine": b32["value"] / b64["value"],
                   "fp32_jacobi": {k: j32[k] for k in ("value", "unit", "ms_per_batch", "iterations", "error_vs_fp64")},
                   "speedup_fp32_jacobi": j32["value"] / b64["value"]}

    # serving: the request stream through the continuous-batching loop
    serving = None
    if args.serve_requests > 0:
        stream = lattice.serving_stream(n=args.serve_requests, rate=200.0, seed=5)
        s32 = run_serving(tdda, stream, tdda.FP32_REFINE, args.serve_workers, 150e9, dev)
        sj = run_serving(tdda, stream, tdda.FP32_JACOBI, args.serve_workers, 150e9, dev)
        n64 = min(args.serve_requests, args.serve_fp64_requests or args.serve_requests)
        s64 = run_serving(tdda, stream[:n64], tdda.FP64, args.serve_workers, 150e9, dev) if n64 > 0 else None
        serving = {"workload": f"serving stream {args.serve_requests} requests, Poisson 200/s, dims 16-128 "
                               "log-uniform (z<=32), 1-4 RHS (cfg 5)", "hbm_budget_bytes": 150e9,
                   "workers": args.serve_workers, "fp32_refine": s32, "fp32_jacobi": sj, "fp64": s64,
                   "speedup_fp32_refine": s32["value"] / s64["value"] if s64 and n64 == len(stream) else None,
                   "speedup_fp32_jacobi": sj["value"] / s64["value"] if s64 and n64 == len(stream) else None}

    cfg1 = run_cfg1(tdda, torch, dev)

    # topology optimisation: forward + adjoint solves batched per iteration
    topo_line = None
    if args.topo_iters > 0:
        topo_line = {"workload": "topology optimisation 80x80x20 (cfg 4), point |E|^2, fwd + 3 adjoint RHS batched",
                     **run_topo(tdda, args.topo_iters)}

    cpu = None
    if dist.rank == 0:
        threads = args.cpu_threads or (os.cpu_count() or 1)
        import ref_timing as RT
        if RT.available(RT.TIMER) and not args.cpu_port:
            # the reference's own code (its sources with the CPU stand-ins for cuFFT): one full
            # converged solve per process, one process per core
            t0 = time.perf_counter()
            rs = RT.run_many(RT.TIMER, w, inc, MAX_IT, TOL, 0, True, threads)
            wall = time.perf_counter() - t0
            solve_s = statistics.median(r["solve_s"] for r in rs)
            cpu = {"value": threads / solve_s, "unit": UNIT, "cores": threads, "kind": "reference",
                   "cpu_model": cpu_model(), "iterations": rs[0]["iterations"],
                   "sample": (f"{threads} processes, one per core, of the reference's own AProductCore/DDAModel "
                              f"sources (oracle/_ref/ref_timer: CPU stand-ins for cuFFT, Bluestein on its "
                              f"{2 * w.Nx - 1}x{2 * w.Ny - 1}x{2 * w.Nz - 1} grid): one full FP64 BiCGSTAB solve "
                              f"each to tol {TOL:g} ({rs[0]['iterations']} iterations, median {solve_s:.1f} s, "
                              f"{wall:.1f} s wall)")}
        else:
            base = CpuBaseline(w, threads)
            base.sample(1)  # warm-up
            cpu = base.sample(0)
            cpu.pop("sample_wall_s", None)
    clocks = ck.summary()
    if dist.rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c64/f64", "data": "synthetic (seeded)",
            "config": {"workload": WORKLOAD, "lattice": [w.Nx, w.Ny, w.Nz], "dipoles": w.N,
                       "grid": list(core.grid), "tol": TOL, "precision": "FP32+refine",
                       "l2": "flushed between steps (256 MiB write)", "parallelism": f"replicas x{dist.world}"},
            "latency_ms": {"p50": float(np.percentile(ms, 50)), "p99": float(np.percentile(ms, 99))},
            "solve": {"inner_iterations": info["inner_iterations"], "outer_iterations": info["outer_iterations"],
                      "true_residual": info["true_residual"], "error_vs_fp64": error_vs_fp64},
            "fp64": {"value": fp64_value, "unit": UNIT, "steps": k64,
                     "latency_ms": {"p50": float(np.percentile(ms64, 50)), "p99": float(np.percentile(ms64, 99))},
                     "iterations": r64[-1][1]["iterations"], "speedup_fp32_refine": value / fp64_value,
                     "roofline": fp64_roof},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "roofline": {"kernel": f"{names[k]} ({prec})", "bound": "hbm", "achieved": achieved,
                         "peak": peaks["hbm_gbs"], "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"],
                         "peak_source": peaks["source"], "algorithmic_bytes": bytes_k, "avg_ms": t_k,
                         "required_bytes": req_k, "frac_required": req_k / (t_k * 1e-3) / 1e9 / peaks["hbm_gbs"],
                         "traffic": traffic,
                         "pass_ms_fp32": prof32, "pass_ms_fp64": prof64,
                         "kernels_fp32": pass_names(core, tdda.FP32_REFINE),
                         "kernels_fp64": pass_names(core, tdda.FP64),
                         "passes_fp32": passes32, "aproduct_fp32": whole32, "x_pass_autotune": tune},
            "batched": batched,
            "serving": serving,
            "cfg1": cfg1,
            "topo": topo_line,
            "gpu_launches": launches,
            "clocks": clocks,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)


def run_aprod_only(args):
    """Only A-products of one workload (for profiler captures): --aprod-only CFG runs
    `--reps` plain products of all of the workload's right-hand sides at once."""
    import tdda

    w = lattice.config(args.aprod_only)
    nrhs = len(w.incidences)
    core = tdda.AProductCore(w.Nx, w.Ny, w.Nz, w.R, w.d, w.lam, w.material, w.nback, max_rhs=nrhs)
    prec = tdda.FP64 if args.aprod_precision == "fp64" else tdda.FP32_REFINE
    ms = core.profile_aproduct(prec, nrhs, args.reps)
    print(json.dumps({"aprod_only": f"cfg{args.aprod_only}", "rhs": nrhs, "grid": list(core.grid),
                      "precision": args.aprod_precision, "pass_ms": ms}), flush=True)


def run_solve_only(args):
    """Only solves of one workload (for launch-list captures): --solve-only CFG runs two
    batched FP32+refine solves of all of the workload's right-hand sides."""
    import tdda

    w = lattice.config(args.solve_only)
    core = tdda.AProductCore(w.Nx, w.Ny, w.Nz, w.R, w.d, w.lam, w.material, w.nback, max_rhs=len(w.incidences))
    models = [tdda.DDAModel(core, i.nK, i.E0, i.nE0, w.diel_old) for i in w.incidences]
    zero = np.zeros(3 * w.N, np.complex128)
    for _ in range(2):
        for m in models:
            m.InitializeP(zero)
        infos = tdda.solve_batch(models, tdda.FP32_REFINE, MAX_IT, TOL)
    print(json.dumps({"solve_only": f"cfg{args.solve_only}", "rhs": len(models),
                      "inner_iterations": [i["inner_iterations"] for i in infos],
                      "outer_iterations": [i["outer_iterations"] for i in infos]}), flush=True)
    for m in models:
        m.close()
    core.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--fp64-steps", type=int, default=5)
    ap.add_argument("--cpu-iters", type=int, default=4)
    ap.add_argument("--cpu-threads", type=int, default=0)
    ap.add_argument("--cpu-port", action="store_true",
                    help="time the oracle port for cpu_baseline even where the reference's own code was built")
    ap.add_argument("--batched-steps", type=int, default=3)
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--serve-requests", type=int, default=64)
    ap.add_argument("--serve-workers", type=int, default=8)
    ap.add_argument("--serve-fp64-requests", type=int, default=0,
                    help="replay only the first n requests with plain FP64 (0: all of them)")
    ap.add_argument("--topo-iters", type=int, default=200)
    ap.add_argument("--aprod-only", type=int, default=0)
    ap.add_argument("--aprod-precision", choices=["fp32", "fp64"], default="fp32")
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--solve-only", type=int, default=0)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.aprod_only:
        run_aprod_only(args)
        return
    if args.solve_only:
        run_solve_only(args)
        return
    dist = Dist()
    try:
        if args.impl == "reference":
            run_reference(args, dist)
        else:
            run_ours(args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
