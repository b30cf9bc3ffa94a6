"""The reference's text files: writers that produce them byte for byte, and readers.

* ``CoreStructure<it>.txt`` (CoreStructure::output_to_file, CoreStructure.cpp:155-185):
  mode "normal" writes Nx, Ny, Nz, N, the lattice R (3N integers), the densities diel_old
  (3N) and d; mode "simple" writes diel_old only.
* ``Model_results<label>it<it>.txt`` / ``Model_results<it>.txt`` (DDAModel::output_to_file,
  DDAModel.cpp:589-697): the field EResult, then (with a model label) P, one complex number
  per line as ``re+imj`` / ``re-imj``.
* ``commondata.txt`` (main.cpp:282-289): Nx, Ny, Nz, N, the geometry (3N integers), d,
  n_E0 and n_K.

Numbers are printed as a C++ ostream prints them by default (6 significant digits, the
shortest of fixed and scientific notation).  A vector is printed as Eigen prints it: one
coefficient per line, right-aligned to the widest coefficient of the vector.
"""
from __future__ import annotations

import os

import numpy as np


def fmt_real(v: float) -> str:
    """A double as std::ostream << prints it with its default precision of 6."""
    v = float(v)
    if v != v:
        return "nan" if np.copysign(1.0, v) > 0 else "-nan"
    if v in (float("inf"), float("-inf")):
        return "inf" if v > 0 else "-inf"
    return format(v, ".6g")


def fmt_complex(z: complex) -> str:
    """``re`` then ``im`` then ``j``, with a ``+`` when the imaginary part is not negative
    (DDAModel.cpp:633-641; a negative zero imaginary part prints as ``+-0``)."""
    z = complex(z)
    re, im = fmt_real(z.real), fmt_real(z.imag)
    return f"{re}{im}j" if z.imag < 0 else f"{re}+{im}j"


def eigen_vector(values, ints: bool = False) -> str:
    """An Eigen column vector as operator<< prints it (no trailing newline)."""
    strs = [str(int(v)) for v in values] if ints else [fmt_real(v) for v in values]
    width = max((len(s) for s in strs), default=0)
    return "\n".join(s.rjust(width) for s in strs)


def write_core_structure(path: str, Nx: int, Ny: int, Nz: int, R, diel_old, d: float, mode: str = "normal"):
    """CoreStructure::output_to_file(save_position, iteration, mode) into `path`."""
    R = np.asarray(R).reshape(-1)
    diel_old = np.asarray(diel_old, np.float64).reshape(-1)
    with open(path, "w", newline="\n") as f:
        if mode == "normal":
            N = R.size // 3
            f.write(f"{Nx}\n{Ny}\n{Nz}\n{N}\n")
            f.write(eigen_vector(R, ints=True) + "\n")
            f.write(eigen_vector(diel_old) + "\n")
            f.write(fmt_real(d) + "\n")
        else:
            f.write(eigen_vector(diel_old) + "\n")


def core_structure_path(save_position: str, iteration: int) -> str:
    return f"{save_position}CoreStructure{iteration}.txt"


def read_core_structure(path: str, mode: str = "normal") -> dict:
    """The fields of a CoreStructure file (values rounded to 6 digits, as written)."""
    with open(path) as f:
        tok = f.read().split()
    if mode != "normal":
        return {"diel_old": np.array([float(t) for t in tok])}
    Nx, Ny, Nz, N = (int(t) for t in tok[:4])
    R = np.array([int(t) for t in tok[4:4 + 3 * N]], np.int32)
    diel = np.array([float(t) for t in tok[4 + 3 * N:4 + 6 * N]])
    d = float(tok[4 + 6 * N])
    return {"Nx": Nx, "Ny": Ny, "Nz": Nz, "N": N, "R": R, "diel_old": diel, "d": d}


def write_model_results(path: str, EResult, P=None):
    """DDAModel::output_to_file: EResult, then P when given (the model-label form)."""
    with open(path, "w", newline="\n") as f:
        for z in np.asarray(EResult).reshape(-1):
            f.write(fmt_complex(z) + "\n")
        if P is not None:
            for z in np.asarray(P).reshape(-1):
                f.write(fmt_complex(z) + "\n")


def model_results_path(save_position: str, iteration: int, label: int | None = None) -> str:
    if label is None:
        return f"{save_position}Model_resultsit{iteration}.txt"
    return f"{save_position}Model_results{label}it{iteration}.txt"


def parse_complex(s: str) -> complex:
    """The inverse of fmt_complex (also reads ``+-0``)."""
    s = s.strip()
    if not s.endswith("j"):
        raise ValueError(f"not a complex number: {s!r}")
    body = s[:-1]
    # the split is the last sign that is not an exponent's and not the leading one
    for i in range(len(body) - 1, 0, -1):
        if body[i] in "+-" and body[i - 1] not in "eE":
            if body[i] == "-" and body[i - 1] == "+":  # "+-": a negative zero imaginary part
                i -= 1
            re, im = body[:i], body[i:]
            if im.startswith("+-"):
                im = im[1:]
            return complex(float(re), float(im))
    raise ValueError(f"not a complex number: {s!r}")


def read_model_results(path: str, n3: int | None = None):
    """All complex numbers of a Model_results file; with n3, (EResult, P) split after the
    first n3 entries."""
    with open(path) as f:
        vals = np.array([parse_complex(line) for line in f if line.strip()], np.complex128)
    if n3 is None:
        return vals
    return vals[:n3], vals[n3:]


def write_commondata(path: str, Nx: int, Ny: int, Nz: int, geometry, d: float, nE0, nK):
    """The commondata.txt lines of main.cpp:282-289."""
    geometry = np.asarray(geometry).reshape(-1)
    with open(path, "w", newline="\n") as f:
        f.write(f"{Nx}\n{Ny}\n{Nz}\n{geometry.size // 3}\n")
        f.write(eigen_vector(geometry, ints=True) + "\n")
        f.write(fmt_real(d) + "\n")
        f.write(eigen_vector(nE0) + "\n")
        f.write(eigen_vector(nK) + "\n")


def read_commondata(path: str) -> dict:
    with open(path) as f:
        tok = f.read().split()
    Nx, Ny, Nz, N = (int(t) for t in tok[:4])
    geo = np.array([int(t) for t in tok[4:4 + 3 * N]], np.int32)
    rest = [float(t) for t in tok[4 + 3 * N:]]
    return {"Nx": Nx, "Ny": Ny, "Nz": Nz, "N": N, "geometry": geo, "d": rest[0],
            "nE0": np.array(rest[1:4]), "nK": np.array(rest[4:7])}


def ensure_folder(save_position: str):
    """The reference writes into folders it expects to exist; create them."""
    folder = os.path.dirname(save_position)
    if folder:
        os.makedirs(folder, exist_ok=True)
