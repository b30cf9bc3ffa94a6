"""The C-ABI library: it loads without a GPU and exports every symbol include/tdda.h declares.

CPU only -- no compute call is made here.
"""
import ctypes
import os
import re

import pytest

import tdda
from conftest import ROOT


def _declared():
    src = open(os.path.join(ROOT, "include", "tdda.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(tdda_[A-Za-z0-9_]+)\s*\(", src)))


def test_header_and_binding_agree():
    assert _declared() == sorted(tdda.EXPORTS)


def test_library_exports_every_declared_symbol():
    L = tdda.load()
    for name in _declared():
        assert hasattr(L, name), name


def test_abi_version_and_device_count_need_no_gpu():
    L = tdda.load()
    assert L.tdda_abi_version() == 1
    assert L.tdda_device_count() >= 0


def test_core_create_rejects_bad_arguments_before_touching_a_device():
    L = tdda.load()
    h = ctypes.c_void_p()
    assert L.tdda_core_create(None, ctypes.byref(h)) == tdda.ERR_INVALID_ARGUMENT
    desc = tdda.CoreDesc()
    desc.Nx = 0
    assert L.tdda_core_create(ctypes.byref(desc), ctypes.byref(h)) == tdda.ERR_INVALID_ARGUMENT
    assert b"invalid" in L.tdda_last_error()


def test_xpass_tuning_rejects_bad_arguments_before_touching_a_device():
    L = tdda.load()
    t = tdda.XpassTune()
    assert L.tdda_core_set_xpass(None, 0, 0) == tdda.ERR_INVALID_ARGUMENT
    assert L.tdda_core_autotune(None, 1, 1, ctypes.byref(t)) == tdda.ERR_INVALID_ARGUMENT
    assert b"invalid" in L.tdda_last_error()
    bt = tdda.BatchTune()
    assert L.tdda_core_set_batch_group(None, 0) == tdda.ERR_INVALID_ARGUMENT
    assert L.tdda_core_autotune_batch(None, 2, 1, ctypes.byref(bt)) == tdda.ERR_INVALID_ARGUMENT


def test_fcd_needs_the_spacing_inside_the_sici_tables():
    """FCD evaluates Si/Ci at (pi/d - K) r >= pi - K d, and the tables start at 0.1."""
    import numpy as np
    R = tdda.lattice.bulk(2, 2, 2)
    mat = np.array([1.0, 4.0 + 0.1j])
    with pytest.raises(tdda.TddaError) as e:
        tdda.AProductCore(2, 2, 2, R, 100.0, 200.0, mat, method="FCD")
    assert e.value.status == tdda.ERR_UNSUPPORTED
    assert b"FCD" in tdda.load().tdda_last_error()


def test_periodic_core_rejects_bad_images_before_touching_a_device():
    L = tdda.load()
    h = ctypes.c_void_p()
    desc = tdda.CoreDesc()
    assert L.tdda_core_create_periodic(ctypes.byref(desc), -1, 2, 10.0, 10.0, ctypes.byref(h)) == \
        tdda.ERR_INVALID_ARGUMENT
    assert L.tdda_core_create_periodic(ctypes.byref(desc), 2, 2, float("nan"), 10.0, ctypes.byref(h)) == \
        tdda.ERR_INVALID_ARGUMENT
    assert b"periodic" in L.tdda_last_error()
