"""GPU parity of the sparse (CSR) correlator against the CPU oracle."""
import numpy as np
import pytest

from conftest import golden
from oracle import g2_oracle as o

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["dense_small_u8", "dense_bright_u8", "dense_u16"])
def test_csr_with_qmask(built_lib, cuda_device, name):
    from dynamix_gb300.correlator import SparseCorrelator
    z = golden(name)
    fr, qm = z["frames"], z["qmask"]
    T, H, W = fr.shape
    data, indices, indptr, offsets = o.frames_to_csr(fr)
    ref = o.csr_correlate_exact(data, indices, indptr, offsets, (H, W), T, qmask=qm)
    c = SparseCorrelator((H, W), T, qmask=qm)
    g = c.correlate(data, indices, indptr, offsets)
    assert np.array_equal(c.numerator, ref["numerator"])
    assert np.array_equal(c.sums, ref["sums"])
    assert np.array_equal(c.denominator, ref["denominator"])
    assert np.array_equal(g, ref["g2"].astype(np.float32), equal_nan=True)


def test_csr_single_q_matches_reference_normalisation(built_lib, cuda_device):
    """qmask=None: one q over all pixels, 1-D result, scale = H*W (intensity.py:108)."""
    from dynamix_gb300.correlator import SparseCorrelator
    z = golden("dense_edge")
    fr = z["frames"]
    T, H, W = fr.shape
    csr = o.frames_to_csr(fr, index_dtype=np.int64)
    c = SparseCorrelator((H, W), T)
    g = c.correlate(*csr)
    assert g.shape == (T,)
    ref = o.g2_exact(fr, None)
    assert np.array_equal(c.numerator, ref["numerator"])
    assert np.allclose(g, z["g2_all"][0], rtol=2e-6)


def test_csr_layout_errors(built_lib, cuda_device):
    from dynamix_gb300.correlator import SparseCorrelator
    z = golden("dense_small_u8")
    fr = z["frames"]
    T, H, W = fr.shape
    data, indices, indptr, offsets = o.frames_to_csr(fr)
    c = SparseCorrelator((H, W), T)
    with pytest.raises(AssertionError):
        c.correlate(data, indices, indptr[:-1], offsets)
    bad = indices.copy()
    bad[0] = W + 3
    with pytest.raises(ValueError):
        c.correlate(data, bad, indptr, offsets)
    with pytest.raises(ValueError):
        SparseCorrelator((H, W), T, bins=3)
