"""Python binding of libtdda (the C ABI in include/tdda.h), shaped like the reference.

``AProductCore`` and ``DDAModel`` keep the method names and argument meaning of the
reference's classes (AProductCore.h:51-80, DDAModel.h:34-74) so that tests and
benchmarks read like the reference's own call sequence (main.cpp:245-251):

    core = AProductCore(Nx, Ny, Nz, R, d, lam, material, nback)
    model = DDAModel(core, n_K, E0, n_E0, diel_old)
    model.bicgstab(MAX_ITERATION, MAX_ERROR)
    model.update_E_in_structure()
    P, Ein = model.get_P(), model.get_Einternal()

Every call goes through the CUDA library; there is no CPU path.  Loading fails
loudly when libtdda.so has not been built (``python topo-dda-forwin64_gb300/build.py``).
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

from . import io, lattice  # noqa: F401

_PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(_PKG, "libtdda.so")

OK, ERR_INVALID_ARGUMENT, ERR_CUDA, ERR_OUT_OF_MEMORY, ERR_UNSUPPORTED = 0, 1, 2, 3, 4
NOT_CONVERGED, BREAKDOWN, ERR_NAN, ERR_NO_DEVICE = 5, 6, 7, 8
STATUS_NAMES = {0: "ok", 1: "invalid argument", 2: "cuda error", 3: "out of memory", 4: "unsupported",
                5: "not converged", 6: "breakdown", 7: "nan", 8: "no device"}
FP64, FP32_REFINE, FP32_JACOBI, FP32_AUTO = 0, 1, 2, 3
MEM_HOST, MEM_DEVICE = 0, 1
FIELD_P, FIELD_E, FIELD_AL, FIELD_DIEL, FIELD_EINTERNAL = 0, 1, 2, 3, 4
METHODS = {"LDR": 0, "FCD": 1}

# every entry point declared in include/tdda.h
EXPORTS = [
    "tdda_abi_version", "tdda_last_error", "tdda_device_count", "tdda_core_create", "tdda_core_create_periodic",
    "tdda_core_interaction",
    "tdda_core_destroy",
    "tdda_core_info", "tdda_aproduct", "tdda_core_ldr_inter", "tdda_model_create", "tdda_model_destroy",
    "tdda_model_update_alpha", "tdda_model_update_alpha_single", "tdda_model_change_E", "tdda_model_reset_E",
    "tdda_model_initialize_P", "tdda_model_aproduct_with_alb", "tdda_model_bicgstab", "tdda_model_solve_mixed",
    "tdda_model_update_E_in_structure", "tdda_model_get", "tdda_model_iterations", "tdda_model_field_at",
    "tdda_model_density_gradient",
    "tdda_solve_batch", "tdda_solve_multi",
    "tdda_fft3d", "tdda_core_stream", "tdda_kernel_launches", "tdda_profile_aproduct", "tdda_core_pass_count",
    "tdda_core_pass_name", "tdda_core_set_xpass", "tdda_core_autotune",
    "tdda_core_set_batch_group", "tdda_core_autotune_batch", "tdda_solve_multi_precision", "tdda_aproduct_noalloc", "tdda_server_create", "tdda_server_submit", "tdda_server_result",
    "tdda_server_stats", "tdda_server_counters_get", "tdda_server_clock", "tdda_server_destroy",
    "tdda_request_bytes",
]
REQ_QUEUED, REQ_RUNNING, REQ_DONE, REQ_FAILED = 0, 1, 2, 3


class TddaError(RuntimeError):
    def __init__(self, status: int, where: str, message: str):
        super().__init__(f"{where}: {STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class CoreDesc(ctypes.Structure):
    _fields_ = [("Nx", ctypes.c_int), ("Ny", ctypes.c_int), ("Nz", ctypes.c_int), ("N", ctypes.c_int),
                ("R", ctypes.POINTER(ctypes.c_int)), ("d", ctypes.c_double), ("lam", ctypes.c_double),
                ("nback", ctypes.c_double), ("material", ctypes.POINTER(ctypes.c_double)),
                ("nmat", ctypes.c_int), ("method", ctypes.c_int), ("max_rhs", ctypes.c_int),
                ("device", ctypes.c_int)]


class XpassTune(ctypes.Structure):
    _fields_ = [("x_form", ctypes.c_int), ("x_tile", ctypes.c_int), ("ncand", ctypes.c_int),
                ("form", ctypes.c_int * 4), ("tile", ctypes.c_int * 4), ("ms", ctypes.c_double * 4)]


class BatchTune(ctypes.Structure):
    _fields_ = [("group", ctypes.c_int), ("ncand", ctypes.c_int), ("groups", ctypes.c_int * 4),
                ("ms", ctypes.c_double * 4)]


class SolveInfo(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("iterations", ctypes.c_int), ("error", ctypes.c_double),
                ("true_residual", ctypes.c_double), ("outer_iterations", ctypes.c_int),
                ("inner_iterations", ctypes.c_int)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class ServerDesc(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("hbm_budget_bytes", ctypes.c_double), ("workers", ctypes.c_int),
                ("precision", ctypes.c_int), ("max_it", ctypes.c_int), ("tol", ctypes.c_double),
                ("max_group", ctypes.c_int), ("dry_run", ctypes.c_int), ("dry_run_ms", ctypes.c_double)]


class RequestDesc(ctypes.Structure):
    _fields_ = [("Nx", ctypes.c_int), ("Ny", ctypes.c_int), ("Nz", ctypes.c_int), ("N", ctypes.c_int),
                ("R", ctypes.POINTER(ctypes.c_int)), ("d", ctypes.c_double), ("lam", ctypes.c_double),
                ("nback", ctypes.c_double), ("material", ctypes.POINTER(ctypes.c_double)), ("nmat", ctypes.c_int),
                ("diel_old", ctypes.POINTER(ctypes.c_double)), ("nrhs", ctypes.c_int),
                ("nK", ctypes.POINTER(ctypes.c_double)), ("nE0", ctypes.POINTER(ctypes.c_double)),
                ("E0", ctypes.POINTER(ctypes.c_double))]


class ServerCounters(ctypes.Structure):
    _fields_ = [("operators_built", ctypes.c_ulonglong), ("operator_hits", ctypes.c_ulonglong),
                ("operators_evicted", ctypes.c_ulonglong), ("shapes_built", ctypes.c_ulonglong),
                ("joined_running", ctypes.c_ulonglong), ("rounds", ctypes.c_ulonglong),
                ("max_slots_in_use", ctypes.c_int), ("max_lattices_in_use", ctypes.c_int),
                ("resident_operators", ctypes.c_int)]


class RequestInfo(ctypes.Structure):
    _fields_ = [("state", ctypes.c_int), ("status", ctypes.c_int), ("t_submit", ctypes.c_double),
                ("t_start", ctypes.c_double), ("t_done", ctypes.c_double), ("iterations", ctypes.c_int),
                ("error", ctypes.c_double), ("bytes", ctypes.c_double), ("group", ctypes.c_int)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


_LIB = None


def load() -> ctypes.CDLL:
    """Load libtdda.so; raise if it is missing (the product has no fallback)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build it with topo-dda-forwin64_gb300/build.py")
    L = ctypes.CDLL(LIB_PATH)
    vp, dp, ip, i, d = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int), \
        ctypes.c_int, ctypes.c_double
    sig = {
        "tdda_abi_version": (i, []),
        "tdda_last_error": (ctypes.c_char_p, []),
        "tdda_device_count": (i, []),
        "tdda_core_create": (i, [ctypes.POINTER(CoreDesc), ctypes.POINTER(vp)]),
        "tdda_core_destroy": (i, [vp]),
        "tdda_core_info": (i, [vp, dp, ip, dp]),
        "tdda_aproduct": (i, [vp, i, vp, vp, i]),
        "tdda_core_ldr_inter": (i, [vp, d, d, d, dp]),
        "tdda_model_create": (i, [vp, dp, d, dp, dp, ctypes.POINTER(vp)]),
        "tdda_model_destroy": (i, [vp]),
        "tdda_model_update_alpha": (i, [vp, dp]),
        "tdda_model_update_alpha_single": (i, [vp, i, d]),
        "tdda_model_change_E": (i, [vp, vp, i]),
        "tdda_model_reset_E": (i, [vp]),
        "tdda_model_initialize_P": (i, [vp, vp, i]),
        "tdda_model_aproduct_with_alb": (i, [vp, vp, vp, i]),
        "tdda_model_bicgstab": (i, [vp, i, d, ctypes.POINTER(SolveInfo)]),
        "tdda_model_solve_mixed": (i, [vp, i, d, ctypes.POINTER(SolveInfo)]),
        "tdda_model_update_E_in_structure": (i, [vp]),
        "tdda_model_get": (i, [vp, i, vp, i]),
        "tdda_model_iterations": (i, [vp]),
        "tdda_model_field_at": (i, [vp, i, vp, vp, i]),
        "tdda_core_create_periodic": (i, [ctypes.POINTER(CoreDesc), i, i, d, d, ctypes.POINTER(vp)]),
        "tdda_core_interaction": (i, [vp, d, d, d, dp]),
        "tdda_model_density_gradient": (i, [vp, i, vp, vp, i, vp, vp, vp]),
        "tdda_solve_batch": (i, [ctypes.POINTER(vp), i, i, i, d, ctypes.POINTER(SolveInfo)]),
        "tdda_solve_multi": (i, [ctypes.POINTER(vp), i, i, d, ctypes.POINTER(SolveInfo)]),
        "tdda_solve_multi_precision": (i, [ctypes.POINTER(vp), i, i, i, d, ctypes.POINTER(SolveInfo)]),
        "tdda_fft3d": (i, [vp, i, i, i, i]),
        "tdda_core_stream": (i, [vp, ctypes.POINTER(vp)]),
        "tdda_kernel_launches": (ctypes.c_ulonglong, []),
        "tdda_profile_aproduct": (i, [vp, i, i, i, dp]),
        "tdda_core_pass_count": (i, [vp, i]),
        "tdda_core_pass_name": (ctypes.c_char_p, [vp, i, i]),
        "tdda_core_set_xpass": (i, [vp, i, i]),
        "tdda_core_autotune": (i, [vp, i, i, ctypes.POINTER(XpassTune)]),
        "tdda_core_set_batch_group": (i, [vp, i]),
        "tdda_core_autotune_batch": (i, [vp, i, i, ctypes.POINTER(BatchTune)]),
        "tdda_aproduct_noalloc": (i, [vp, vp, vp]),
        "tdda_server_create": (i, [ctypes.POINTER(ServerDesc), ctypes.POINTER(vp)]),
        "tdda_server_submit": (i, [vp, ctypes.POINTER(RequestDesc), ctypes.POINTER(ctypes.c_ulonglong)]),
        "tdda_server_result": (i, [vp, ctypes.c_ulonglong, i, ctypes.POINTER(RequestInfo), vp]),
        "tdda_server_stats": (i, [vp, ip, ip, dp, dp]),
        "tdda_server_counters_get": (i, [vp, ctypes.POINTER(ServerCounters)]),
        "tdda_server_clock": (d, [vp]),
        "tdda_server_destroy": (i, [vp]),
        "tdda_request_bytes": (d, [i, i, i, i, i, i]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _LIB = L
    return L


def device_count() -> int:
    return load().tdda_device_count()


def kernel_launches() -> int:
    """Kernels libtdda has launched in this process."""
    return int(load().tdda_kernel_launches())


def _check(st: int, where: str, allowed=(OK,)):
    if st not in allowed:
        raise TddaError(st, where, load().tdda_last_error().decode())
    return st


def _c128(a, n=None) -> np.ndarray:
    a = np.ascontiguousarray(np.asarray(a, dtype=np.complex128).reshape(-1))
    if n is not None and a.size != n:
        raise ValueError(f"expected {n} complex entries, got {a.size}")
    return a


def _ptr(a: np.ndarray):
    return ctypes.c_void_p(a.ctypes.data)


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class AProductCore:
    """The interaction operator of one lattice at one wavelength (AProductCore.h:12-81)."""

    def __init__(self, Nx, Ny, Nz, R, d, lam, material, nback=1.0, method="LDR", max_rhs=1, device=0,
                 periodic=None):
        """periodic = (MAXm, MAXn, Lm, Ln): the periodic constructor (AProductCore.cpp:251-536)."""
        L = load()
        self.R = np.ascontiguousarray(np.asarray(R, dtype=np.int32).reshape(-1))
        self.N = self.R.size // 3
        self.Nx, self.Ny, self.Nz = int(Nx), int(Ny), int(Nz)
        self.d, self.lam, self.nback = float(d), float(lam), float(nback)
        mat = _c128(material)
        self._mat = mat
        desc = CoreDesc(self.Nx, self.Ny, self.Nz, self.N,
                        self.R.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), self.d, self.lam, self.nback,
                        _dptr(mat.view(np.float64)), mat.size, METHODS[method], int(max_rhs), int(device))
        h = ctypes.c_void_p()
        if periodic is None:
            _check(L.tdda_core_create(ctypes.byref(desc), ctypes.byref(h)), "tdda_core_create")
        else:
            mm, mn_, Lm, Ln = periodic
            _check(L.tdda_core_create_periodic(ctypes.byref(desc), int(mm), int(mn_), float(Lm), float(Ln),
                                               ctypes.byref(h)), "tdda_core_create_periodic")
        self.periodic = periodic
        self.h = h
        # handles of the live models on this core: a model must be destroyed before its core,
        # and the garbage collector may finalise a core and its models in any order
        self._models = set()
        self.max_rhs = int(max_rhs)
        K = ctypes.c_double()
        g = (ctypes.c_int * 3)()
        mn = np.zeros(mat.size, np.complex128)
        _check(L.tdda_core_info(h, ctypes.byref(K), g, _dptr(mn.view(np.float64))), "tdda_core_info")
        self.K = K.value
        self.grid = tuple(g)
        self.material = mn

    def get_N(self): return self.N
    def get_Nx(self): return self.Nx
    def get_Ny(self): return self.Ny
    def get_Nz(self): return self.Nz
    def get_R(self): return self.R
    def get_d(self): return self.d
    def get_lam(self): return self.lam
    def get_K(self): return self.K
    def get_material(self): return self.material
    def get_nback(self): return self.nback

    def Aproduct(self, b, precision: int = FP64) -> np.ndarray:
        """y = A_offdiag b (AProductCore.cpp:697-758); host arrays in and out."""
        b = _c128(b, 3 * self.N)
        y = np.empty_like(b)
        _check(load().tdda_aproduct(self.h, precision, _ptr(b), _ptr(y), MEM_HOST), "tdda_aproduct")
        return y

    def Aproduct_device(self, b_ptr: int, y_ptr: int, precision: int = FP64):
        _check(load().tdda_aproduct(self.h, precision, ctypes.c_void_p(b_ptr), ctypes.c_void_p(y_ptr),
                                    MEM_DEVICE), "tdda_aproduct")

    def stream(self) -> int:
        """The cudaStream_t of this core (for events recorded on it)."""
        p = ctypes.c_void_p()
        _check(load().tdda_core_stream(self.h, ctypes.byref(p)), "tdda_core_stream")
        return p.value or 0

    def pass_count(self, precision: int = FP32_REFINE) -> int:
        """Kernels of one A-product: 5, or 3 when the z and y passes are fused."""
        n = load().tdda_core_pass_count(self.h, int(precision))
        if n < 0:
            raise ValueError(f"pass_count: invalid precision {precision}")
        return n

    def pass_names(self, precision: int = FP32_REFINE) -> list:
        """Kernel of each of the five profile slots ("" where a fused kernel covers the slot)."""
        out = []
        for k in range(5):
            n = load().tdda_core_pass_name(self.h, int(precision), k)
            if n is None:
                raise ValueError(f"pass_names: invalid precision {precision}")
            out.append(n.decode())
        return out

    def set_xpass(self, form: int, tile: int = 0):
        """FP32 x-pass configuration: form 0 = register form (tile 8, 16, or 0 for the
        built-in choice), form 1 = shared-memory form (tile 0)."""
        _check(load().tdda_core_set_xpass(self.h, int(form), int(tile)), "tdda_core_set_xpass")

    def autotune(self, nrhs: int = 1, reps: int = 10) -> dict:
        """Time the FP32 x-pass candidates on this core's A-product and keep the fastest."""
        t = XpassTune()
        _check(load().tdda_core_autotune(self.h, int(nrhs), int(reps), ctypes.byref(t)), "tdda_core_autotune")
        return {"x_form": t.x_form, "x_tile": t.x_tile,
                "candidates": [{"form": t.form[k], "tile": t.tile[k], "ms": t.ms[k]} for k in range(t.ncand)]}

    def set_batch_group(self, group: int) -> None:
        """Right-hand sides per launch of the FP32 products of batched solves (0: all)."""
        _check(load().tdda_core_set_batch_group(self.h, int(group)), "tdda_core_set_batch_group")

    def autotune_batch(self, nrhs: int, reps: int = 5) -> dict:
        """Time the batch-schedule candidates on this core's FP32 A-product and keep the fastest."""
        t = BatchTune()
        _check(load().tdda_core_autotune_batch(self.h, int(nrhs), int(reps), ctypes.byref(t)),
               "tdda_core_autotune_batch")
        return {"group": t.group, "candidates": [{"group": t.groups[k], "ms": t.ms[k]} for k in range(t.ncand)]}

    def profile_aproduct(self, precision: int = FP32_REFINE, nrhs: int = 1, reps: int = 10) -> list:
        """Average ms of the five passes of one A-product (CUDA events on the core stream)."""
        out = (ctypes.c_double * 5)()
        _check(load().tdda_profile_aproduct(self.h, int(precision), int(nrhs), int(reps), out),
               "tdda_profile_aproduct")
        return list(out)

    def Aproduct_noalloc(self, b_ptr: int, y_ptr: int):
        """y = A_offdiag b on device memory (3N complex128 each) without any device
        allocation: the FFT work grid is the library's static scratch array."""
        _check(load().tdda_aproduct_noalloc(self.h, ctypes.c_void_p(b_ptr), ctypes.c_void_p(y_ptr)),
               "tdda_aproduct_noalloc")

    def LDR_inter(self, x, y, z) -> np.ndarray:
        out = np.zeros(6, np.complex128)
        _check(load().tdda_core_ldr_inter(self.h, x, y, z, _dptr(out.view(np.float64))), "tdda_core_ldr_inter")
        a = out
        return np.array([[a[0], a[1], a[2]], [a[1], a[3], a[4]], [a[2], a[4], a[5]]])

    def A_dic_generator(self, x, y, z) -> np.ndarray:
        """The core's interaction tensor, LDR or FCD (AProductCore.cpp:560-571), 3 x 3."""
        out = np.zeros(6, np.complex128)
        _check(load().tdda_core_interaction(self.h, x, y, z, _dptr(out.view(np.float64))), "tdda_core_interaction")
        a = out
        return np.array([[a[0], a[1], a[2]], [a[1], a[3], a[4]], [a[2], a[4], a[5]]])

    def close(self):
        if getattr(self, "h", None):
            for mh in list(getattr(self, "_models", ())):
                load().tdda_model_destroy(ctypes.c_void_p(mh))
            self._models = set()
            load().tdda_core_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DDAModel:
    """Incident field, polarisability and solve of one right-hand side (DDAModel.h:6-75)."""

    def __init__(self, core: AProductCore, n_K, E0, n_E0, diel_old):
        self.core = core
        self.n3 = 3 * core.N
        nK = np.ascontiguousarray(n_K, np.float64)
        nE = np.ascontiguousarray(n_E0, np.float64)
        diel = np.ascontiguousarray(diel_old, np.float64)
        if diel.size != self.n3:
            raise ValueError("diel_old must hold 3N densities")
        h = ctypes.c_void_p()
        _check(load().tdda_model_create(core.h, _dptr(nK), float(E0), _dptr(nE), _dptr(diel), ctypes.byref(h)),
               "tdda_model_create")
        self.h = h
        core._models.add(h.value)
        self.last_info = None

    def _get(self, field: int, out: np.ndarray = None) -> np.ndarray:
        if out is None:
            out = np.empty(self.n3, np.complex128)
        elif out.dtype != np.complex128 or out.size != self.n3 or not out.flags.c_contiguous:
            raise ValueError("out must be a contiguous complex128 array of 3N entries")
        _check(load().tdda_model_get(self.h, field, _ptr(out), MEM_HOST), "tdda_model_get")
        return out

    def get_P(self): return self._get(FIELD_P)
    def get_E(self): return self._get(FIELD_E)
    def get_al(self): return self._get(FIELD_AL)
    def get_diel(self): return self._get(FIELD_DIEL)
    def get_Einternal(self): return self._get(FIELD_EINTERNAL)
    def get_ITERATION(self) -> int: return load().tdda_model_iterations(self.h)

    def density_gradient(self, adjoints, coef, offsets, dipoles) -> np.ndarray:
        """Per design parameter, Re(sum lambda * dal/drho * P) over its dipoles, with
        lambda = sum_k coef[k] * P(adjoints[k]) (EvoDDAModel.cpp:610-638)."""
        adj = (ctypes.c_void_p * len(adjoints))(*[a.h for a in adjoints])
        cf = np.ascontiguousarray(coef, np.complex128)
        off = np.ascontiguousarray(offsets, np.int32)
        dip = np.ascontiguousarray(dipoles, np.int32)
        out = np.zeros(off.size - 1, np.float64)
        _check(load().tdda_model_density_gradient(self.h, len(adjoints), adj, _ptr(cf), off.size - 1, _ptr(off),
                                                  _ptr(dip), _ptr(out)), "tdda_model_density_gradient")
        return out

    def field_at(self, points) -> np.ndarray:
        """E at off-lattice points (npts x 3, nm) from the current P: npts x 3 complex
        (ObjDDAModel.cpp:20-96; DDAModel::solve_E with points d * RResult)."""
        pts = np.ascontiguousarray(points, np.float64).reshape(-1, 3)
        out = np.zeros((pts.shape[0], 3), np.complex128)
        _check(load().tdda_model_field_at(self.h, pts.shape[0], _ptr(pts), _ptr(out), MEM_HOST),
               "tdda_model_field_at")
        return out

    def UpdateAlpha(self, diel_old):
        diel = np.ascontiguousarray(diel_old, np.float64)
        _check(load().tdda_model_update_alpha(self.h, _dptr(diel)), "tdda_model_update_alpha")

    def UpdateAlphaSingle(self, idx: int, value: float):
        _check(load().tdda_model_update_alpha_single(self.h, int(idx), float(value)), "UpdateAlphaSingle")

    def change_E(self, E):
        E = _c128(E, self.n3)
        _check(load().tdda_model_change_E(self.h, _ptr(E), MEM_HOST), "tdda_model_change_E")

    def reset_E(self):
        _check(load().tdda_model_reset_E(self.h), "tdda_model_reset_E")

    def InitializeP(self, P=None):
        """P = the given host vector, or zero on the device (no transfer) when P is None."""
        if P is None:
            _check(load().tdda_model_initialize_P(self.h, None, MEM_HOST), "tdda_model_initialize_P")
            return
        P = _c128(P, self.n3)
        _check(load().tdda_model_initialize_P(self.h, _ptr(P), MEM_HOST), "tdda_model_initialize_P")

    def Aproductwithalb(self, b) -> np.ndarray:
        b = _c128(b, self.n3)
        y = np.empty_like(b)
        _check(load().tdda_model_aproduct_with_alb(self.h, _ptr(b), _ptr(y), MEM_HOST), "Aproductwithalb")
        return y

    def bicgstab(self, MAX_ITERATION: int, MAX_ERROR: float) -> dict:
        """FP64 BiCGSTAB (DDAModel.cpp:131-260).  Returns the solve info; a breakdown or a
        reached iteration limit is reported in info['status'], as the reference only prints."""
        info = SolveInfo()
        load().tdda_model_bicgstab(self.h, int(MAX_ITERATION), float(MAX_ERROR), ctypes.byref(info))
        _check(info.status, "bicgstab", allowed=(OK, NOT_CONVERGED, BREAKDOWN))
        self.last_info = info.as_dict()
        return self.last_info

    def solve_mixed(self, MAX_ITERATION: int, MAX_ERROR: float, jacobi: bool = False) -> dict:
        """FP32 BiCGSTAB with FP64 refinement to MAX_ERROR; jacobi: the inner solve
        right-preconditioned by diag(al) (TDDA_FP32_JACOBI)."""
        if jacobi:
            [info] = solve_batch([self], FP32_JACOBI, MAX_ITERATION, MAX_ERROR)
            return info
        info = SolveInfo()
        load().tdda_model_solve_mixed(self.h, int(MAX_ITERATION), float(MAX_ERROR), ctypes.byref(info))
        _check(info.status, "solve_mixed", allowed=(OK, NOT_CONVERGED, BREAKDOWN))
        self.last_info = info.as_dict()
        return self.last_info

    def update_E_in_structure(self):
        _check(load().tdda_model_update_E_in_structure(self.h), "update_E_in_structure")

    def close(self):
        """Destroys the model; a no-op when its core was closed first (which destroyed it)."""
        if getattr(self, "h", None):
            live = getattr(self.core, "_models", set())
            if self.h.value in live:
                live.discard(self.h.value)
                load().tdda_model_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def solve_batch(models, precision: int = FP64, max_it: int = 10000, tol: float = 1e-5) -> list:
    """Solve several models of one core in one batched pass per kernel."""
    n = len(models)
    arr = (ctypes.c_void_p * n)(*[m.h.value for m in models])
    infos = (SolveInfo * n)()
    st = load().tdda_solve_batch(arr, n, int(precision), int(max_it), float(tol), infos)
    # a right-hand side that stops without converging reports it in its own info
    _check(st, "tdda_solve_batch", allowed=(OK, NOT_CONVERGED, BREAKDOWN, ERR_NAN))
    out = [infos[k].as_dict() for k in range(n)]
    for m, o in zip(models, out):
        m.last_info = o
    return out


def solve_multi(models, max_it: int = 10000, tol: float = 1e-5, precision: int = FP32_REFINE) -> list:
    """FP32+refine solves (precision FP32_REFINE or FP32_JACOBI) of models on different cores
    that share one FFT grid shape, with the inner solves of all of them in one launch per pass
    (tdda_solve_multi_precision)."""
    n = len(models)
    arr = (ctypes.c_void_p * n)(*[m.h.value for m in models])
    infos = (SolveInfo * n)()
    st = load().tdda_solve_multi_precision(arr, n, int(precision), int(max_it), float(tol), infos)
    _check(st, "tdda_solve_multi", allowed=(OK, NOT_CONVERGED, BREAKDOWN, ERR_NAN))
    out = [infos[k].as_dict() for k in range(n)]
    for m, o in zip(models, out):
        m.last_info = o
    return out


def fft3d_device(ptr: int, n0: int, n1: int, n2: int, sign: int):
    """In-place complex128 3-D FFT of device memory at ptr (the engine's own FFT)."""
    _check(load().tdda_fft3d(ctypes.c_void_p(ptr), n0, n1, n2, sign), "tdda_fft3d")


@dataclass
class Solved:
    P: np.ndarray
    Einternal: np.ndarray
    info: dict


def solve_workload(w, precision: int = FP64, inc=None, tol=None, max_it=None) -> Solved:
    """One solve of a lattice.Workload through the reference-shaped API."""
    inc = inc or w.incidences[0]
    core = AProductCore(w.Nx, w.Ny, w.Nz, w.R, w.d, w.lam, w.material, w.nback)
    model = DDAModel(core, inc.nK, inc.E0, inc.nE0, w.diel_old)
    tol = w.tol if tol is None else tol
    max_it = w.max_it if max_it is None else max_it
    if precision == FP64:
        info = model.bicgstab(max_it, tol)
    elif precision == FP32_JACOBI:
        [info] = solve_batch([model], FP32_JACOBI, max_it, tol)
    else:
        info = model.solve_mixed(max_it, tol)
    model.update_E_in_structure()
    out = Solved(model.get_P(), model.get_Einternal(), info)
    model.close()
    core.close()
    return out


class Server:
    """Continuous-batching solve loop (tdda_server_*): submit structures, collect results."""

    def __init__(self, hbm_budget_bytes=150e9, workers=4, precision=FP32_REFINE, max_it=10000, tol=1e-5,
                 max_group=8, device=0, dry_run_ms=None):
        d = ServerDesc(int(device), float(hbm_budget_bytes), int(workers), int(precision), int(max_it), float(tol),
                       int(max_group), int(dry_run_ms is not None), float(dry_run_ms or 0.0))
        h = ctypes.c_void_p()
        _check(load().tdda_server_create(ctypes.byref(d), ctypes.byref(h)), "tdda_server_create")
        self.h = h
        self._keep = {}
        self._n = {}

    def submit(self, Nx, Ny, Nz, R, d, lam, material, diel_old, incidences, nback=1.0) -> int:
        """incidences: list of (nK, nE0, E0)."""
        R = np.ascontiguousarray(np.asarray(R, dtype=np.int32).reshape(-1))
        mat = _c128(material)
        diel = np.ascontiguousarray(diel_old, np.float64)
        nK = np.ascontiguousarray(np.array([np.asarray(i[0], np.float64) for i in incidences]).reshape(-1))
        nE = np.ascontiguousarray(np.array([np.asarray(i[1], np.float64) for i in incidences]).reshape(-1))
        E0 = np.ascontiguousarray(np.array([float(i[2]) for i in incidences]))
        req = RequestDesc(int(Nx), int(Ny), int(Nz), R.size // 3, R.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                          float(d), float(lam), float(nback), _dptr(mat.view(np.float64)), mat.size, _dptr(diel),
                          len(incidences), _dptr(nK), _dptr(nE), _dptr(E0))
        rid = ctypes.c_ulonglong()
        _check(load().tdda_server_submit(self.h, ctypes.byref(req), ctypes.byref(rid)), "tdda_server_submit")
        self._n[rid.value] = (R.size // 3, len(incidences))
        return rid.value

    def result(self, rid: int, wait: bool = True, with_P: bool = True):
        info = RequestInfo()
        N, nrhs = self._n[rid]
        P = np.zeros(3 * N * nrhs, np.complex128) if with_P else None
        _check(load().tdda_server_result(self.h, ctypes.c_ulonglong(rid), int(wait), ctypes.byref(info),
                                         _ptr(P) if with_P else None), "tdda_server_result")
        return info.as_dict(), (P.reshape(nrhs, 3 * N) if with_P else None)

    def stats(self) -> dict:
        q, r = ctypes.c_int(), ctypes.c_int()
        b, pk = ctypes.c_double(), ctypes.c_double()
        _check(load().tdda_server_stats(self.h, ctypes.byref(q), ctypes.byref(r), ctypes.byref(b), ctypes.byref(pk)),
               "tdda_server_stats")
        return {"queued": q.value, "running": r.value, "bytes": b.value, "peak_bytes": pk.value}

    def counters(self) -> dict:
        """Residency and continuous-batching counters (tdda_server_counters_get)."""
        c = ServerCounters()
        _check(load().tdda_server_counters_get(self.h, ctypes.byref(c)), "tdda_server_counters_get")
        return {f: getattr(c, f) for f, _ in ServerCounters._fields_}

    def clock(self) -> float:
        return load().tdda_server_clock(self.h)

    def close(self):
        if getattr(self, "h", None):
            load().tdda_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def request_bytes(Nx, Ny, Nz, N, nrhs, precision=FP32_REFINE) -> float:
    return float(load().tdda_request_bytes(Nx, Ny, Nz, N, nrhs, precision))
