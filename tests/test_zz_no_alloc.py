"""The allocation-free A-product entry point (tdda_aproduct_noalloc).

It serves callers that cannot allocate device memory when they run the product --
code under a pre-reserved memory budget, or a host framework that forbids
allocation after its setup -- by keeping the FFT work grid in a static device
array.  This file is collected last so that a run stopping at the first failure
has already run every other test.  Checked against the allocating entry point
(tdda_aproduct, the same passes on the core's own grid buffer), two calls in a
row, within the FP64 product tolerance of the other tests (1e-12 relative).
"""
import numpy as np
import pytest

import tdda
from conftest import rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if tdda.device_count() < 1:
        pytest.skip("no CUDA device")


@pytest.mark.parametrize("idx", [1, 2])
def test_noalloc_matches_allocating_product_twice(idx):
    torch = pytest.importorskip("torch")
    w = tdda.lattice.config(idx)
    core = tdda.AProductCore(w.Nx, w.Ny, w.Nz, w.R, w.d, w.lam, w.material)
    rng = np.random.Generator(np.random.PCG64(100 + idx))
    for call in range(2):
        b = rng.standard_normal(3 * w.N) + 1j * rng.standard_normal(3 * w.N)
        ref = core.Aproduct(b)
        bd = torch.from_numpy(b).to("cuda")
        yd = torch.full_like(bd, complex(np.nan, np.nan))
        torch.cuda.synchronize()
        core.Aproduct_noalloc(bd.data_ptr(), yd.data_ptr())
        y = yd.cpu().numpy()
        assert np.all(np.isfinite(y)), f"call {call}"
        assert rel(y, ref) <= 1e-12, f"call {call}"
    core.close()


def test_noalloc_smaller_grid_after_a_larger_one():
    """The static array keeps the last call's contents.  A product on the 64x64x16 grid
    fills it with values laid out for that grid's strides; the next product, on the
    20x20x10 grid and then on a sparse lattice, must read only entries it wrote itself."""
    torch = pytest.importorskip("torch")
    rng = np.random.Generator(np.random.PCG64(300))
    big = tdda.lattice.config(2)
    small = tdda.lattice.config(1)
    keep = rng.random(small.N) < 0.6
    Rs = small.R.reshape(-1, 3)[keep].ravel()
    cases = [(big.Nx, big.Ny, big.Nz, big.R, big.d, big.lam, big.material),
             (small.Nx, small.Ny, small.Nz, small.R, small.d, small.lam, small.material),
             (big.Nx, big.Ny, big.Nz, big.R, big.d, big.lam, big.material),
             (small.Nx, small.Ny, small.Nz, Rs, small.d, small.lam, small.material)]
    for k, (Nx, Ny, Nz, R, d, lam, mat) in enumerate(cases):
        core = tdda.AProductCore(Nx, Ny, Nz, R, d, lam, mat)
        n3 = R.size
        b = rng.standard_normal(n3) + 1j * rng.standard_normal(n3)
        ref = core.Aproduct(b)
        bd = torch.from_numpy(b).to("cuda")
        yd = torch.full_like(bd, complex(np.nan, np.nan))
        torch.cuda.synchronize()
        core.Aproduct_noalloc(bd.data_ptr(), yd.data_ptr())
        y = yd.cpu().numpy()
        assert np.all(np.isfinite(y)), f"case {k}"
        assert rel(y, ref) <= 1e-12, f"case {k}"
        core.close()


def test_noalloc_rejects_grids_beyond_its_static_size():
    torch = pytest.importorskip("torch")
    Nx, Ny, Nz = 128, 128, 32  # grid 3 x 128 x 256 x 64 entries > 4,194,304
    R = tdda.lattice.bulk(Nx, Ny, Nz)
    core = tdda.AProductCore(Nx, Ny, Nz, R, 10.0, 500.0, np.array([1.0, 2.25]))
    bd = torch.zeros(R.size, dtype=torch.complex128, device="cuda")
    yd = torch.zeros_like(bd)
    with pytest.raises(tdda.TddaError) as e:
        core.Aproduct_noalloc(bd.data_ptr(), yd.data_ptr())
    assert e.value.status == tdda.ERR_UNSUPPORTED and "static" in str(e.value)
    core.close()
