"""The C++ drop-in (topo-dda-forwin64_gb300/cpp/tdda.hpp) used with the reference's call sequence.

tests/cpp/mirror_solve.cpp builds a structure with the reference CoreStructure's getters,
constructs AProductCore / DDAModel (with RResult points), runs bicgstab +
update_E_in_structure + solve_E and dumps the results; here they are compared with the oracle.  Compiling is a CPU test; running is a
GPU test.  tests/cpp/dropin_reference.cpp compiles the reference's own callers (its
ObjDDAModel.cpp and structure classes, unchanged) against the drop-in with Eigen types.
"""
import math
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle as O
import tdda
from conftest import ROOT, rel

SRC = os.path.join(ROOT, "tests", "cpp", "mirror_solve.cpp")
PKG = os.path.join(ROOT, "topo-dda-forwin64_gb300")


def _build(tmp_path) -> str:
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "mirror_solve")
    subprocess.run([cxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe, "-L", PKG,
                    "-ltdda", f"-Wl,-rpath,{PKG}"], check=True, capture_output=True, text=True)
    return exe


def test_mirror_header_compiles_against_the_abi(tmp_path):
    tdda.load()  # libtdda.so must exist to link
    assert os.path.exists(_build(tmp_path))


def test_reference_callers_compile_against_the_dropin():
    """The reference's ObjDDAModel.cpp, CoreStructure.cpp, Space*.cpp, Structure.cpp, tools.cpp
    and FilterOption.cpp, unchanged, with the drop-in in place of AProductCore.h / DDAModel.h
    (tests/cpp/dropin_reference.cpp: the "DDA input" sequence of main.cpp:165-251 and the
    point objective), built and linked with libtdda.  Matrix3cd A = Core.A_dic_generator(...)
    (ObjDDAModel.cpp:60) and R = Core.get_R() into a VectorXi* (ObjDDAModel.cpp:37) compile.
    Skipped where the reference checkout is absent; running it needs a CUDA device."""
    tdda.load()
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "dropin-if-present"], capture_output=True,
                       text=True)
    if "reference sources absent" in r.stdout:
        pytest.skip("reference checkout absent")
    assert r.returncode == 0, r.stdout + r.stderr
    assert os.path.exists(os.path.join(ROOT, "oracle", "_ref", "dropin_reference"))


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol,bound", [(0, 1e-10, 1e-9), (1, 1e-5, 1e-4), (2, 1e-5, 1e-4)])
def test_mirror_solve_matches_oracle(tmp_path, precision, tol, bound):
    if tdda.device_count() < 1:
        pytest.skip("no CUDA device")
    exe = _build(tmp_path)
    Nx, Ny, Nz, d, lam, em = 9, 8, 6, 10.0, 520.0, 4.0 + 0.1j
    out = str(tmp_path / "out.bin")
    r = subprocess.run([exe, str(Nx), str(Ny), str(Nz), str(d), str(lam), str(em.real), str(em.imag), repr(tol),
                        str(precision), out], check=True, capture_output=True, text=True)
    N = Nx * Ny * Nz
    raw = open(out, "rb").read()
    it = int(np.frombuffer(raw, "<i4", count=1)[0])
    P = np.frombuffer(raw, "<c16", count=3 * N, offset=4)
    Ein = np.frombuffer(raw, "<c16", count=3 * N, offset=4 + 48 * N)
    rho = np.array([0.5 + 0.5 * math.sin(0.37 * i) for i in range(N)])
    R = tdda.lattice.bulk(Nx, Ny, Nz)
    oc = O.OracleCore(Nx, Ny, Nz, R, d, lam, np.array([1.0, em]))
    om = O.OracleModel(oc, [0, 0, 1], 1.0, [1, 0, 0], np.repeat(rho, 3))
    assert om.bicgstab(100000, 1e-12) == O.CONVERGED
    om.update_E_in_structure()
    assert it > 0, r.stdout
    EResult = np.frombuffer(raw, "<c16", count=12, offset=4 + 96 * N)
    RResult = np.array([[Nx // 2, Ny // 2, Nz + 10], [-5, Ny // 2, Nz // 2], [Nx + 3, -2, -4],
                        [2 * Nx, 2 * Ny, 2 * Nz]], np.float64)
    assert rel(P, om.P) <= bound
    assert rel(Ein, om.Einternal) <= bound
    assert rel(EResult, om.field_at(d * RResult).ravel()) <= bound
    # DDAModel::output_to_file: the same bytes as the reference's writer (tdda.io, pinned to it)
    ref_txt = str(tmp_path / "ref.txt")
    tdda.io.write_model_results(ref_txt, EResult, P)
    assert open(out + ".Model_results1it3.txt", "rb").read() == open(ref_txt, "rb").read()
    # periodic core (MAXm 2, MAXn 1, periods of the box): the product of the solved P, and the
    # image tensor A_dic_generator(10, 20, 5, m=1, n=-1)
    off = 4 + 96 * N + 12 * 16
    y = np.frombuffer(raw, "<c16", count=3 * N, offset=off)
    A = np.frombuffer(raw, "<c16", count=9, offset=off + 48 * N).reshape(3, 3)
    opc = O.OracleCore(Nx, Ny, Nz, R, d, lam, np.array([1.0, em]), periodic=(2, 1, Nx * d, Ny * d))
    assert rel(y, opc.Aproduct(P)) <= 1e-12
    x_, y_, z_ = 10.0 + Nx * d, 20.0 - Ny * d, 5.0
    t = O.ldr_inter(opc.K, x_, y_, z_) * math.exp(-(0.01 * opc.K * math.sqrt(x_ ** 2 + y_ ** 2 + z_ ** 2)) ** 4)
    full = np.array([[t[0], t[1], t[2]], [t[1], t[3], t[4]], [t[2], t[4], t[5]]])
    assert np.max(np.abs(A - full)) <= 1e-15 * np.max(np.abs(full))
