"""The CPU FFT that times the reference's host path (oracle/_ref/ref_timer): Bluestein's
chirp-z transform for the prime lengths of the reference's 2N - 1 grids (127, 31, 191, 47,
19, ...), against numpy's FFT, both signs, cuFFT's conventions (forward -1, inverse +1,
unnormalised).  The checker's own oc_fft3d is unchanged and pinned by the golden tests."""
import ctypes
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import oracle as O  # noqa: E402


@pytest.mark.parametrize("shape", [(39, 39, 19), (127, 127, 31), (8, 6, 5), (17, 23, 7), (191, 13, 47)])
@pytest.mark.parametrize("sign", [-1, 1])
def test_bluestein_fft3d_matches_numpy(shape, sign):
    rng = np.random.Generator(np.random.PCG64(11))
    x = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    y = np.ascontiguousarray(x.copy())
    lib = O.lib()
    lib.oc_fft3d_fast.argtypes = [ctypes.c_int] * 3 + [ctypes.c_void_p, ctypes.c_int]
    assert lib.oc_fft3d_fast(*shape, y.ctypes.data_as(ctypes.c_void_p), sign) == 0
    ref = np.fft.fftn(x) if sign < 0 else np.fft.ifftn(x) * x.size
    assert np.max(np.abs(y - ref)) <= 1e-14 * np.max(np.abs(ref))
