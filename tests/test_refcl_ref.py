"""The oracle pinned against the reference's own dense and CSR OpenCL kernels.

Fixtures ``refcl_*`` were made by running ``densecorrelator.cl`` and
``correlator.cl`` compiled as C (``oracle/opencl_wg_shim.h``,
``oracle/ref_wg_driver.c``) over the NDRanges of ``DenseCorrelator.correlate``
and ``SparseCorrelator.correlate`` (``tests/golden/make_wg_golden.py``).  Each
holds the reference's bin sums (exact integers), its float32 g2, and its
integer numerator (the kernel rerun with a normalisation of ones).  The
integer N and S must equal the oracle's bit for bit; the reference's float32
g2 (float32 denominator sums) agrees with the oracle's FP64 g2 to 2e-6.
"""
import numpy as np
import pytest

from conftest import golden
from oracle import g2_oracle as o

RTOL_REF = 2e-6


def _close(got, want, rtol=RTOL_REF):
    got = np.asarray(got, np.float64)
    want = np.asarray(want, np.float64)
    assert np.array_equal(np.isfinite(got), np.isfinite(want))
    ok = np.isfinite(want)
    assert np.all(np.abs(got[ok] - want[ok]) <= rtol * np.abs(want[ok]))


@pytest.mark.parametrize("name", ["refcl_dense_u8", "refcl_dense_wide"])
def test_dense_kernel_pins_oracle(name):
    z = golden(name)
    ex = o.g2_exact(z["frames"], z["qmask"])
    assert np.array_equal(z["numer_f"].astype(np.int64), ex["numerator"])
    assert np.array_equal(z["sums"].astype(np.int64), ex["sums"])
    _close(z["g2"], ex["g2"])
    _close(z["corr1d"], ex["denominator"])


@pytest.mark.parametrize("name", ["refcl_csr_u8", "refcl_csr_dense_rows"])
def test_csr_kernel_pins_oracle(name):
    z = golden(name)
    T, H, W = z["frames"].shape
    ex = o.csr_correlate_exact(z["data"], z["indices"], z["indptr"], z["offsets"], (H, W), T)
    assert np.array_equal(z["numer"], ex["numerator"][0])
    assert np.array_equal(z["sums"].astype(np.int64), ex["sums"][0])
    _close(z["g2"], ex["g2"][0])
