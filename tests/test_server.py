"""The continuous-batching solve loop (tdda_server_*).

Scheduler behaviour is tested without a GPU in the server's dry-run mode (the same
scheduler; each request sleeps instead of solving): admission never exceeds the HBM
budget, a request that does not fit waits while smaller ones behind it run, requests
sharing an operator are grouped, a request larger than the whole budget fails.  The GPU
test checks that each result in a mixed stream equals the same request solved alone.
"""
import time

import numpy as np
import pytest

import tdda
from tdda import lattice

MAT = np.array([1.0, 4.0 + 0.1j])
XPOL = ([0.0, 0.0, 1.0], [1.0, 0.0, 0.0], 1.0)
YPOL = ([0.0, 0.0, 1.0], [0.0, 1.0, 0.0], 1.0)


def _req(server, n, lam=500.0, seed=0, incs=(XPOL,)):
    rng = np.random.Generator(np.random.PCG64(seed))
    R = lattice.bulk(n, n, n)
    diel = np.repeat(rng.random(n ** 3), 3)
    return server.submit(n, n, n, R, 10.0, lam, MAT, diel, list(incs))


def test_dry_run_respects_the_budget_and_first_fit():
    small = tdda.request_bytes(6, 6, 6, 216, 1)
    big = tdda.request_bytes(12, 12, 12, 1728, 1)
    budget = big + 0.5 * small  # the big request fits alone, not with a small one beside it
    s = tdda.Server(hbm_budget_bytes=budget, workers=3, dry_run_ms=40.0)
    ids = [_req(s, 6, seed=1), _req(s, 12, seed=2), _req(s, 6, seed=3, lam=510.0), _req(s, 6, seed=4, lam=520.0)]
    peak_seen = 0.0
    t0 = time.time()
    while time.time() - t0 < 10:
        st = s.stats()
        peak_seen = max(peak_seen, st["bytes"])
        if st["queued"] == 0 and st["running"] == 0:
            break
        time.sleep(0.005)
    infos = [s.result(i, with_P=False)[0] for i in ids]
    s.close()
    assert all(i["state"] == tdda.REQ_DONE for i in infos)
    assert peak_seen <= budget and s is not None
    # the big request could not start beside the first small one: the small ones behind it ran first
    assert infos[1]["t_start"] >= infos[0]["t_done"] - 1e-3
    assert infos[2]["t_start"] < infos[1]["t_start"]


def test_dry_run_groups_requests_sharing_an_operator():
    s = tdda.Server(hbm_budget_bytes=1e12, workers=1, dry_run_ms=30.0, max_group=4)
    a = _req(s, 6, seed=1)           # occupies the single worker
    b = _req(s, 7, seed=2)           # same operator as c: both queued while a runs
    c = _req(s, 7, seed=2, incs=(XPOL, YPOL))
    d = _req(s, 7, seed=2, lam=600.0)
    infos = [s.result(i, with_P=False)[0] for i in (a, b, c, d)]
    s.close()
    assert infos[1]["group"] == 3 and infos[2]["group"] == 3 and infos[1]["t_start"] == infos[2]["t_start"]
    assert infos[3]["group"] == 1


def test_request_larger_than_the_budget_fails():
    s = tdda.Server(hbm_budget_bytes=1e6, workers=1, dry_run_ms=1.0)
    i = _req(s, 10)
    info, _ = s.result(i, with_P=False)
    s.close()
    assert info["state"] == tdda.REQ_FAILED and info["status"] == tdda.ERR_OUT_OF_MEMORY


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [tdda.FP64, tdda.FP32_REFINE])
def test_each_result_equals_the_request_alone(precision):
    if tdda.device_count() < 1:
        pytest.skip("no CUDA device")
    rng = np.random.Generator(np.random.PCG64(42))
    reqs = []
    for k in range(10):
        Nx, Ny, Nz = (int(v) for v in rng.integers(4, 12, 3))
        lam = float(rng.uniform(400, 800))
        em = [2.25, 4.0 + 0.1j, 6.25 + 0.05j][k % 3]
        diel = np.repeat(rng.random(Nx * Ny * Nz), 3)
        incs = [XPOL, YPOL][: 1 + k % 2]
        reqs.append((Nx, Ny, Nz, lam, np.array([1.0, em]), diel, incs))
    s = tdda.Server(hbm_budget_bytes=150e9, workers=3, precision=precision)
    ids = []
    for r in reqs:
        Nx, Ny, Nz, lam, mat, diel, incs = r
        ids.append(s.submit(Nx, Ny, Nz, lattice.bulk(Nx, Ny, Nz), 10.0, lam, mat, diel, incs))
        time.sleep(float(rng.exponential(0.002)))
    out = [s.result(i) for i in ids]
    s.close()
    for (Nx, Ny, Nz, lam, mat, diel, incs), (info, P) in zip(reqs, out):
        assert info["state"] == tdda.REQ_DONE, info
        core = tdda.AProductCore(Nx, Ny, Nz, lattice.bulk(Nx, Ny, Nz), 10.0, lam, mat, max_rhs=len(incs))
        models = [tdda.DDAModel(core, i[0], i[2], i[1], diel) for i in incs]
        tdda.solve_batch(models, precision, 10000, 1e-5)
        for k, m in enumerate(models):
            assert np.array_equal(P[k], m.get_P())


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [tdda.FP64, tdda.FP32_REFINE])
def test_operators_stay_resident(precision):
    """Requests of one operator (lattice, spacing, wavelength, material) after one another:
    the core and its models are built once and reused; results equal the request alone."""
    if tdda.device_count() < 1:
        pytest.skip("no CUDA device")
    n = 9
    R = lattice.bulk(n, n, n)
    s = tdda.Server(hbm_budget_bytes=150e9, workers=1, precision=precision, max_group=4)
    outs = []
    for k in range(4):
        rng = np.random.Generator(np.random.PCG64(60 + k))
        diel = np.repeat(rng.random(n ** 3), 3)  # new densities: same operator, new models' al
        rid = s.submit(n, n, n, R, 10.0, 500.0, MAT, diel, [XPOL, YPOL][: 1 + k % 2])
        outs.append((diel, k, s.result(rid)))
    c = s.counters()
    s.close()
    assert c["operators_built"] == 1 and c["operator_hits"] == 3 and c["resident_operators"] == 1
    core = tdda.AProductCore(n, n, n, R, 10.0, 500.0, MAT, max_rhs=2)
    for diel, k, (info, P) in outs:
        assert info["state"] == tdda.REQ_DONE
        incs = [XPOL, YPOL][: 1 + k % 2]
        ms = [tdda.DDAModel(core, i[0], i[2], i[1], diel) for i in incs]
        tdda.solve_batch(ms, precision, 10000, 1e-5)
        for j, m in enumerate(ms):
            assert np.array_equal(P[j], m.get_P())
            m.close()
    core.close()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [tdda.FP64, tdda.FP32_JACOBI])
def test_idle_operators_are_capped(precision):
    """A stream of 44 operators that never return: at most 32 idle operators stay resident
    (hundreds of idle cores alive at once slowed every later request of the process), the
    rest are evicted least recently used first, and every request still completes."""
    if tdda.device_count() < 1:
        pytest.skip("no CUDA device")
    s = tdda.Server(hbm_budget_bytes=150e9, workers=2, precision=precision, max_group=4)
    ids = [_req(s, 6, lam=450.0 + 5.0 * k, seed=k) for k in range(44)]
    infos = [s.result(i, with_P=False)[0] for i in ids]
    c = s.counters()
    s.close()
    assert all(i["state"] == tdda.REQ_DONE for i in infos)
    assert c["operators_built"] == 44
    assert c["resident_operators"] <= 32
    assert c["operators_evicted"] >= 12


@pytest.mark.gpu
def test_requests_join_running_work_across_lattices():
    """FP32+refine continuous batching: one worker, a session of 4 slots.  A slow request
    (a 14^3 lattice at a high contrast) is running when requests of other lattices of the
    same FFT grid shape arrive; they join its launches as slots are free, and every result
    equals its request alone."""
    if tdda.device_count() < 1:
        pytest.skip("no CUDA device")
    rng = np.random.Generator(np.random.PCG64(77))
    boxes = [(14, 14, 14), (15, 14, 16), (16, 15, 14), (14, 16, 15), (15, 15, 15)]
    grids = {tuple(lattice.fft_length(b[a], a == 2) for a in range(3)) for b in boxes}
    assert len(grids) == 1
    reqs = []
    for k, b in enumerate(boxes):
        mat = np.array([1.0, 12.0 + 0.05j]) if k == 0 else np.array([1.0, [2.25, 4.0 + 0.1j][k % 2]])
        reqs.append((b, 10.0 - k, float(rng.uniform(450, 650)), mat, np.repeat(rng.random(int(np.prod(b))), 3)))
    s = tdda.Server(hbm_budget_bytes=150e9, workers=1, precision=tdda.FP32_REFINE, max_group=4)
    ids = []
    for k, (b, d, lam, mat, diel) in enumerate(reqs):
        ids.append(s.submit(*b, lattice.bulk(*b), d, lam, mat, diel, [XPOL]))
        if k == 0:
            time.sleep(0.05)  # the first request is running when the others arrive
    out = [s.result(i) for i in ids]
    c = s.counters()
    s.close()
    assert c["joined_running"] >= 1 and c["max_lattices_in_use"] >= 2, c
    for (b, d, lam, mat, diel), (info, P) in zip(reqs, out):
        assert info["state"] == tdda.REQ_DONE, info
        core = tdda.AProductCore(*b, lattice.bulk(*b), d, lam, mat)
        m = tdda.DDAModel(core, XPOL[0], XPOL[2], XPOL[1], diel)
        m.solve_mixed(10000, 1e-5)
        assert np.array_equal(P[0], m.get_P())
        m.close()
        core.close()


@pytest.mark.gpu
def test_request_bytes_bound_the_device_memory_a_request_takes():
    """tdda_request_bytes against the device memory a core and its models take (the drop in
    free memory while they exist, in a fresh process so the memory pool starts empty)."""
    if tdda.device_count() < 1:
        pytest.skip("no CUDA device")
    import subprocess
    import sys
    code = (
        "import sys, numpy as np; sys.path.insert(0, 'topo-dda-forwin64_gb300'); import tdda, torch\n"
        "from tdda import lattice\n"
        "torch.cuda.init(); torch.zeros(1, device='cuda'); torch.cuda.synchronize()\n"
        "out = []\n"
        "for (nx, ny, nz, nrhs) in ((40, 40, 20, 1), (48, 40, 24, 2)):\n"
        "    f0 = torch.cuda.mem_get_info()[0]\n"
        "    R = lattice.bulk(nx, ny, nz)\n"
        "    c = tdda.AProductCore(nx, ny, nz, R, 10.0, 500.0, np.array([1.0, 4.0 + 0.1j]), max_rhs=nrhs)\n"
        "    ms = [tdda.DDAModel(c, [0, 0, 1], 1.0, [1, 0, 0], np.full(R.size, 0.5)) for _ in range(nrhs)]\n"
        "    tdda.solve_batch(ms, tdda.FP32_REFINE, 10000, 1e-5)\n"
        "    torch.cuda.synchronize()\n"
        "    f1 = torch.cuda.mem_get_info()[0]\n"
        "    out.append((f0 - f1, tdda.request_bytes(nx, ny, nz, R.size // 3, nrhs)))\n"
        "print(out)\n")
    import os
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, cwd=root, timeout=300)
    assert r.returncode == 0, r.stderr
    pairs = eval(r.stdout.strip().splitlines()[-1])
    for used, est in pairs:
        print(f"\ndevice memory taken {used / 1e6:.1f} MB, tdda_request_bytes {est / 1e6:.1f} MB")
        # the estimate bounds what a request takes (pool granularity: up to 64 MB more per request)
        assert used <= est + 64e6
        assert est <= 3 * used + 64e6
