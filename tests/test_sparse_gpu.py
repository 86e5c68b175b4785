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


@pytest.mark.parametrize("name,index_dtype", [("dense_small_u8", np.uint32), ("dense_u16", np.int64),
                                              ("dense_128x128_u8", np.uint32)])
def test_csr_to_events_is_frames_compressor_layout(built_lib, cuda_device, name, index_dtype):
    """The device transposition yields exactly FramesCompressor's layout:
    pixel-major, frames ascending within a pixel (event.py:267-284)."""
    import torch
    from dynamix_gb300.engine_sparse import SparseEngine, csr_to_device
    z = golden(name)
    fr = z["frames"]
    T, H, W = fr.shape
    csr = o.frames_to_csr(fr, index_dtype=index_dtype)
    eng = SparseEngine((H, W), T, np.ones((H, W), np.int32), 1, [1.0])
    counts, ind, ip, off, ib, n, mx = csr_to_device(*csr, (H, W), T, eng.dev)
    times, data, evoff = eng.to_events(counts, ind, ip, off, ib, n)
    torch.cuda.synchronize()
    eng.check_error()
    d_ref, t_ref, o_ref = o.compress_all_stack(fr)
    assert np.array_equal(evoff.cpu().numpy().view(np.uint32), o_ref)
    assert np.array_equal(times[:n].cpu().numpy(), t_ref)
    assert np.array_equal(data[:n].cpu().numpy().astype(np.int64), d_ref.astype(np.int64))


def test_csr_duplicate_column_is_reported(built_lib, cuda_device):
    from dynamix_gb300.correlator import SparseCorrelator
    from dynamix_gb300.engine import DeviceError
    fr = np.zeros((3, 2, 8), np.uint8)
    fr[:, 0, 2] = 1
    fr[1, 1, 5] = 2
    data, indices, indptr, offsets = o.frames_to_csr(fr)
    indices = indices.copy()
    # frame 0, row 0 holds one element; make frame 1's row 0 name column 2 twice
    data2 = np.insert(data, 1, 1)
    indices2 = np.insert(indices, 1, 2)
    ip = indptr.reshape(3, 3).astype(np.int64)
    ip[1, 1:] += 1
    off = offsets.astype(np.int64)
    off[2:] += 1
    c = SparseCorrelator((2, 8), 3)
    with pytest.raises(DeviceError):
        c.correlate(data2, indices2.astype(np.uint32), ip.ravel().astype(np.uint32), off.astype(np.uint32))


def test_wide_rows_take_the_walk_kernels(built_lib, cuda_device):
    """Rows wider than the row-owned kernels take (29,000 px): global-atomic
    transposition, events unordered within a pixel, same exact sums."""
    from dynamix_gb300.correlator import SparseCorrelator
    rng = np.random.default_rng(8)
    T, H, W = 40, 2, 29010
    fr = (rng.random((T, H, W)) < 0.002).astype(np.uint8) * rng.integers(1, 5, (T, H, W)).astype(np.uint8)
    qm = np.zeros((H, W), np.int32)
    qm[:, :10000] = 1
    qm[:, 20000:] = 2
    csr = o.frames_to_csr(fr)
    c = SparseCorrelator((H, W), T, qmask=qm)
    g = c.correlate(*csr)
    assert c.engine.last["packed"] is False
    ref = o.g2_exact(fr, qm)
    assert np.array_equal(c.numerator, ref["numerator"])
    assert np.array_equal(c.sums, ref["sums"])
    assert np.array_equal(g, ref["g2"].astype(np.float32), equal_nan=True)


@pytest.mark.parametrize("name,index_dtype", [("dense_128x128_u8", np.int32), ("dense_u16", np.int64),
                                              ("synthetic", np.int32)])
def test_pinned_host_csr_pipeline(built_lib, cuda_device, name, index_dtype):
    # pinned host CSR tensors take the frame-group pipeline (count and stage of
    # a group while the next one is copied); equal to the oracle, and malformed
    # stacks still raise
    import torch
    from dynamix_gb300.correlator import SparseCorrelator
    if name == "synthetic":                        # 2600 frames: three frame groups of one sub-block
        from dynamix_gb300.speckle import annular_qmask, speckle_numpy
        fr = speckle_numpy(2600, (40, 56), 0.98, 0.2, seed=17)
        qm = annular_qmask((40, 56), 4, 2.0, 20.0)
    else:
        z = golden(name)
        fr, qm = z["frames"], z["qmask"]
    T, H, W = fr.shape
    data, indices, indptr, offsets = o.frames_to_csr(fr)
    ref = o.csr_correlate_exact(data, indices, indptr, offsets, (H, W), T, qmask=qm)
    pin = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a).astype(dt)).pin_memory()
    d = pin(data, data.dtype)
    ind, ip, off = (pin(a, index_dtype) for a in (indices, indptr, offsets))
    c = SparseCorrelator((H, W), T, qmask=qm)
    c.engine.HOST_SB_PER_CHUNK = 1                 # several frame groups even for short stacks
    assert c.engine.host_pipeline_ok(d, ind, ip, off)
    g = c.correlate(d, ind, ip, off)
    assert c.engine.last.get("host_sb_per_chunk") == 1
    assert np.array_equal(c.numerator, ref["numerator"])
    assert np.array_equal(c.sums, ref["sums"])
    assert np.array_equal(c.denominator, ref["denominator"])
    assert np.array_equal(g, ref["g2"].astype(np.float32), equal_nan=True)
    bad = ind.clone().pin_memory()
    bad[len(bad) // 3] = W + 5                     # a column outside the row
    with pytest.raises(ValueError):
        c.correlate(d, bad, ip, off)
    bad_off = off.clone().pin_memory()
    bad_off[3] = bad_off[4] + 1
    with pytest.raises(ValueError):
        c.correlate(d, ind, ip, bad_off)
    assert np.array_equal(c.correlate(d, ind, ip, off), g)


@pytest.mark.parametrize("name", ["refcl_csr_u8", "refcl_csr_dense_rows"])
def test_matches_reference_csr_kernel(built_lib, cuda_device, name):
    """N and S bit-exact against the reference's own correlator.cl (compute_sums +
    correlator_oneQ_Nt run as C by tests/golden/make_wg_golden.py); float32 g2
    within 2e-6 of the reference's float32 g2."""
    from dynamix_gb300.correlator import SparseCorrelator
    z = golden(name)
    T, H, W = z["frames"].shape
    c = SparseCorrelator((H, W), T)
    g = c.correlate(z["data"], z["indices"], z["indptr"], z["offsets"])
    assert np.array_equal(c.numerator[0], z["numer"])
    assert np.array_equal(c.sums[0], z["sums"].astype(np.int64))
    ref = z["g2"].astype(np.float64)
    assert np.all(np.abs(g.astype(np.float64) - ref) <= 2e-6 * np.abs(ref))
