"""ctypes wrapper of liboracle.so, the CPU restatement of the reference's solve path.

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py``, as the checker.  The product never routes
through it.  The functions it wraps cite the reference lines they restate in
oracle/tdda_oracle.h.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

CONVERGED, BREAKDOWN, MAXITER = 0, 1, 2


def build(force: bool = False) -> str:
    """Compile liboracle.so with the Makefile next to this file."""
    path = os.path.join(_HERE, "liboracle.so")
    if force or not os.path.exists(path):
        subprocess.run(["make", "-s", "-C", _HERE, "liboracle.so"], check=True)
    return path


def lib() -> ctypes.CDLL:
    global _LIB
    if _LIB is None:
        L = ctypes.CDLL(build())
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        vp = ctypes.c_void_p
        L.or_ldr_inter.argtypes = [ctypes.c_double] * 4 + [dp]
        L.or_get_alpha.argtypes = [ctypes.c_double] * 5 + [dp, dp, dp]
        L.or_normalize_material.argtypes = [ctypes.c_int, dp, ctypes.c_double, dp]
        L.or_core_create.restype = vp
        L.or_core_create.argtypes = [ctypes.c_int] * 4 + [ip] + [ctypes.c_double] * 3 + [
            ctypes.c_int, dp, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.or_core_create_periodic.restype = vp
        L.or_core_create_periodic.argtypes = [ctypes.c_int] * 4 + [ip] + [ctypes.c_double] * 3 + [
            ctypes.c_int, dp, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int,
            ctypes.c_int, ctypes.c_int]
        L.or_core_create_method.restype = vp
        L.or_core_create_method.argtypes = [ctypes.c_int] * 4 + [ip] + [ctypes.c_double] * 3 + [
            ctypes.c_int, dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
            ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.or_fcd_inter.argtypes = [ctypes.c_double] * 5 + [dp]
        L.or_core_destroy.argtypes = [vp]
        L.or_core_set_pruned.argtypes = [vp, ctypes.c_int]
        L.or_core_K.restype = ctypes.c_double
        L.or_core_K.argtypes = [vp]
        L.or_core_material.argtypes = [vp, dp]
        L.or_core_grid.argtypes = [vp, ip]
        L.or_aproduct.argtypes = [vp, dp, dp]
        L.or_aproduct_direct.argtypes = [ctypes.c_int, ip, ctypes.c_double, ctypes.c_double, dp, dp]
        L.or_model_create.restype = vp
        L.or_model_create.argtypes = [vp, dp, ctypes.c_double, dp, dp]
        L.or_model_destroy.argtypes = [vp]
        L.or_model_update_alpha.argtypes = [vp, dp]
        L.or_model_change_E.argtypes = [vp, dp]
        L.or_model_reset_E.argtypes = [vp]
        L.or_model_initialize_P.argtypes = [vp, dp]
        L.or_model_aproduct_with_alb.argtypes = [vp, dp, dp]
        L.or_model_bicgstab.argtypes = [vp, ctypes.c_int, ctypes.c_double, ip, dp]
        L.or_model_update_E_in_structure.argtypes = [vp]
        L.or_model_get.argtypes = [vp, ctypes.c_int, dp]
        L.or_model_field_at.argtypes = [vp, ctypes.c_int, dp, dp]
        L.or_sici.argtypes = [ctypes.c_double, dp, dp]
        _LIB = L
    return _LIB


def _dp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def _c128(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.complex128))


def ldr_inter(K: float, x: float, y: float, z: float) -> np.ndarray:
    out = np.zeros(6, np.complex128)
    lib().or_ldr_inter(K, x, y, z, _dp(out.view(np.float64)))
    return out


def fcd_inter(K: float, d: float, x: float, y: float, z: float) -> np.ndarray:
    """FCD tensor (AProductCore.cpp:625-695): xx, xy, xz, yy, yz, zz."""
    out = np.zeros(12)
    lib().or_fcd_inter(K, d, x, y, z, _dp(out))
    return out.view(np.complex128)


def sici(x: float):
    """(Si(x), Ci(x)) for x > 0."""
    s, c = ctypes.c_double(), ctypes.c_double()
    lib().or_sici(float(x), ctypes.byref(s), ctypes.byref(c))
    return s.value, c.value


def get_alpha(lam, K, d, eps, nE0, nK) -> complex:
    out = np.zeros(2)
    nE0 = np.ascontiguousarray(nE0, np.float64)
    nK = np.ascontiguousarray(nK, np.float64)
    lib().or_get_alpha(lam, K, d, float(np.real(eps)), float(np.imag(eps)), _dp(nE0), _dp(nK), _dp(out))
    return complex(out[0], out[1])


def aproduct_direct(R: np.ndarray, d: float, K: float, b) -> np.ndarray:
    R = np.ascontiguousarray(R, np.int32).reshape(-1)
    b = _c128(b)
    y = np.zeros_like(b)
    lib().or_aproduct_direct(R.size // 3, _ip(R), d, K, _dp(b.view(np.float64)), _dp(y.view(np.float64)))
    return y


class OracleCore:
    """AProductCore restated (AProductCore.cpp:12-249, 697-758)."""

    def __init__(self, Nx, Ny, Nz, R, d, lam, material, nback=1.0, grid=None, pruned=False, periodic=None,
                 method="LDR"):
        """periodic = (MAXm, MAXn, Lm, Ln) selects the periodic constructor (AProductCore.cpp:251-536);
        method "LDR" or "FCD" the interaction tensor (AProductCore.cpp:560-571)."""
        self.R = np.ascontiguousarray(R, np.int32).reshape(-1)
        self.N = self.R.size // 3
        mat = _c128(material)
        M = grid or (0, 0, 0)
        if method != "LDR":
            mm, mn, Lm, Ln = periodic if periodic is not None else (0, 0, 0.0, 0.0)
            h = lib().or_core_create_method(Nx, Ny, Nz, self.N, _ip(self.R), d, lam, nback, mat.size,
                                            _dp(mat.view(np.float64)), {"FCD": 1}[method], int(periodic is not None),
                                            int(mm), int(mn), float(Lm), float(Ln), int(M[0]), int(M[1]), int(M[2]))
        elif periodic is None:
            h = lib().or_core_create(Nx, Ny, Nz, self.N, _ip(self.R), d, lam, nback, mat.size,
                                     _dp(mat.view(np.float64)), int(M[0]), int(M[1]), int(M[2]))
        else:
            mm, mn, Lm, Ln = periodic
            h = lib().or_core_create_periodic(Nx, Ny, Nz, self.N, _ip(self.R), d, lam, nback, mat.size,
                                              _dp(mat.view(np.float64)), int(mm), int(mn), float(Lm), float(Ln),
                                              int(M[0]), int(M[1]), int(M[2]))
        if not h:
            raise ValueError("oracle core rejected its arguments")
        self.h = h
        self.nmat = mat.size
        self.d = d
        lib().or_core_set_pruned(h, int(bool(pruned)))

    @property
    def K(self) -> float:
        return lib().or_core_K(self.h)

    @property
    def material(self) -> np.ndarray:
        out = np.zeros(self.nmat, np.complex128)
        lib().or_core_material(self.h, _dp(out.view(np.float64)))
        return out

    @property
    def grid(self):
        out = np.zeros(3, np.int32)
        lib().or_core_grid(self.h, _ip(out))
        return tuple(int(v) for v in out)

    def Aproduct(self, b) -> np.ndarray:
        b = _c128(b)
        y = np.zeros_like(b)
        lib().or_aproduct(self.h, _dp(b.view(np.float64)), _dp(y.view(np.float64)))
        return y

    def close(self):
        if getattr(self, "h", None):
            lib().or_core_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class OracleModel:
    """DDAModel restated (DDAModel.cpp:12-69, 131-260, 470-586)."""

    def __init__(self, core: OracleCore, nK, E0, nE0, diel_old):
        self.core = core
        self.n3 = 3 * core.N
        nK = np.ascontiguousarray(nK, np.float64)
        nE0 = np.ascontiguousarray(nE0, np.float64)
        diel = np.ascontiguousarray(diel_old, np.float64)
        h = lib().or_model_create(core.h, _dp(nK), float(E0), _dp(nE0), _dp(diel))
        if not h:
            raise ValueError("oracle model rejected its arguments")
        self.h = h
        self.ITERATION = 0
        self.Error = 0.0

    def _get(self, what: int) -> np.ndarray:
        out = np.zeros(self.n3, np.complex128)
        lib().or_model_get(self.h, what, _dp(out.view(np.float64)))
        return out

    P = property(lambda self: self._get(0))
    E = property(lambda self: self._get(1))
    al = property(lambda self: self._get(2))
    diel = property(lambda self: self._get(3))
    Einternal = property(lambda self: self._get(4))

    def UpdateAlpha(self, diel_old):
        diel = np.ascontiguousarray(diel_old, np.float64)
        if lib().or_model_update_alpha(self.h, _dp(diel)):
            raise ValueError("density outside the material table")

    def change_E(self, E):
        E = _c128(E)
        lib().or_model_change_E(self.h, _dp(E.view(np.float64)))

    def reset_E(self):
        lib().or_model_reset_E(self.h)

    def InitializeP(self, P):
        P = _c128(P)
        lib().or_model_initialize_P(self.h, _dp(P.view(np.float64)))

    def field_at(self, points) -> np.ndarray:
        """E at off-lattice points (npts x 3, nm) -> npts x 3 complex (ObjDDAModel.cpp:83-96)."""
        pts = np.ascontiguousarray(points, np.float64).reshape(-1, 3)
        out = np.zeros((pts.shape[0], 3), np.complex128)
        lib().or_model_field_at(self.h, pts.shape[0], _dp(pts), _dp(out.view(np.float64)))
        return out

    def Aproductwithalb(self, b) -> np.ndarray:
        b = _c128(b)
        y = np.zeros_like(b)
        lib().or_model_aproduct_with_alb(self.h, _dp(b.view(np.float64)), _dp(y.view(np.float64)))
        return y

    def bicgstab(self, max_it: int, max_err: float) -> int:
        it = ctypes.c_int(self.ITERATION)
        err = ctypes.c_double(self.Error)
        st = lib().or_model_bicgstab(self.h, int(max_it), float(max_err), ctypes.byref(it),
                                     ctypes.byref(err))
        self.ITERATION, self.Error = it.value, err.value
        return st

    def update_E_in_structure(self):
        lib().or_model_update_E_in_structure(self.h)

    def close(self):
        if getattr(self, "h", None):
            lib().or_model_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
