"""The reference's text files (tdda/io.py) against files the reference's own writers produced
(tests/golden/text_*: CoreStructure.cpp:155-185, DDAModel.cpp:589-697, main.cpp:282-289).
CPU only."""
import os

import numpy as np
import pytest

from conftest import ROOT, golden
from tdda import io

FOLDER = os.path.join(ROOT, "tests", "golden", "text_sparse4x3x2")


def _bytes(path):
    with open(path, "rb") as f:
        return f.read()


@pytest.fixture(scope="module")
def g():
    return golden("text_sparse4x3x2.npz")


def test_core_structure_files_are_byte_identical(g, tmp_path):
    Nx, Ny, Nz = (int(v) for v in g["box"])
    p = tmp_path / "CoreStructure7.txt"
    io.write_core_structure(str(p), Nx, Ny, Nz, g["R"], g["diel_old"], float(g["d"]), "normal")
    assert _bytes(p) == _bytes(os.path.join(FOLDER, "CoreStructure7.txt"))
    q = tmp_path / "sCoreStructure8.txt"
    io.write_core_structure(str(q), Nx, Ny, Nz, g["R"], g["diel_old"], float(g["d"]), "simple")
    assert _bytes(q) == _bytes(os.path.join(FOLDER, "sCoreStructure8.txt"))
    r = io.read_core_structure(str(p))
    assert (r["Nx"], r["Ny"], r["Nz"], r["N"]) == (Nx, Ny, Nz, g["R"].size // 3)
    assert np.array_equal(r["R"], g["R"]) and r["d"] == float(g["d"])
    assert np.allclose(r["diel_old"], g["diel_old"], rtol=1e-5, atol=0)


def test_model_results_file_is_byte_identical(g, tmp_path):
    p = tmp_path / io.model_results_path("", 3, 1)
    io.write_model_results(str(p), g["Einternal"], g["P"])
    assert _bytes(p) == _bytes(os.path.join(FOLDER, "Model_results1it3.txt"))
    E, P = io.read_model_results(str(p), g["P"].size)
    assert np.allclose(E, g["Einternal"], rtol=1e-5, atol=1e-12)
    assert np.allclose(P, g["P"], rtol=1e-5, atol=1e-12)


def test_commondata_file_is_byte_identical(g, tmp_path):
    Nx, Ny, Nz = (int(v) for v in g["box"])
    p = tmp_path / "commondata.txt"
    io.write_commondata(str(p), Nx, Ny, Nz, g["R"], float(g["d"]), g["nE0"], g["nK"])
    assert _bytes(p) == _bytes(os.path.join(FOLDER, "commondata.txt"))
    c = io.read_commondata(str(p))
    assert np.array_equal(c["geometry"], g["R"]) and np.allclose(c["nK"], g["nK"])


def test_number_formats_follow_the_cpp_stream():
    assert io.fmt_real(0.5) == "0.5" and io.fmt_real(1e-7) == "1e-07" and io.fmt_real(123456789.0) == "1.23457e+08"
    assert io.fmt_real(-0.0) == "-0" and io.fmt_real(10.0) == "10"
    assert io.fmt_complex(1.5 - 2j) == "1.5-2j" and io.fmt_complex(1.5 + 2j) == "1.5+2j"
    assert io.fmt_complex(complex(1.0, -0.0)) == "1+-0j"
    for z in (1.5 - 2j, 3e-9 + 4.25e10j, complex(1.0, -0.0), -7e-5 - 1e-300j):
        assert io.parse_complex(io.fmt_complex(z)) == pytest.approx(z, rel=1e-5)
    assert io.eigen_vector([1, 10, 100], ints=True) == "  1\n 10\n100"
