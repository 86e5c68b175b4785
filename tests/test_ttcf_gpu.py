"""GPU two-time correlation (TTCF) against its restatement of the reference
(correlator/event_y.py:141-157)."""
import numpy as np
import pytest

from conftest import golden
from oracle import g2_oracle as o

pytestmark = pytest.mark.gpu


def _same(got, ref, rtol=2e-6):
    assert got.shape == ref.shape and got.dtype == np.float32
    nan = np.isnan(ref)
    assert np.array_equal(np.isnan(got), nan)
    inf = np.isinf(ref)
    assert np.array_equal(got[inf], ref[inf].astype(np.float32))
    ok = ~nan & ~inf
    assert np.all(np.abs(got[ok] - ref[ok]) <= rtol * np.abs(ref[ok]) + 1e-30)


@pytest.mark.parametrize("name,q", [("dense_small_u8", 1), ("dense_small_u8", 3), ("dense_128x128_u8", 2),
                                    ("dense_u16", 4)])
def test_ttcf_golden_frames(built_lib, cuda_device, name, q):
    from dynamix_gb300.correlator import MatMulCorrelator
    z = golden(name)
    fr, qm = z["frames"], z["qmask"]
    c = MatMulCorrelator(fr.shape[1:], fr.shape[0], qmask=qm)
    c.correlate(fr)
    _same(c.two_time(q), o.ttcf_exact(fr, qm, q))


def test_ttcf_zero_frames_not_mirrored(built_lib, cuda_device):
    # a bin with empty frames: the reference's diagonal k = -5 holds NaN, so it
    # does not mirror, and 0/0 gives NaN
    from dynamix_gb300.correlator import MatMulCorrelator
    rng = np.random.default_rng(5)
    T, H, W = 300, 24, 24
    fr = rng.poisson(0.05, (T, H, W)).astype(np.uint8)
    fr[::7] = 0
    qm = np.zeros((H, W), np.int32)
    qm[:12] = 1
    qm[12:] = 2
    c = MatMulCorrelator((H, W), T, qmask=qm)
    c.correlate(fr)
    for q in (1, 2):
        _same(c.two_time(q), o.ttcf_exact(fr, qm, q))


def test_ttcf_long_stack(built_lib, cuda_device):
    # several 128 x 256 tiles in both directions, T not a multiple of the tile
    from dynamix_gb300.correlator import MatMulCorrelator
    from dynamix_gb300.speckle import annular_qmask, speckle_numpy
    T, H, W = 1300, 48, 64
    fr = speckle_numpy(T, (H, W), 0.98, 0.5, seed=9)
    qm = annular_qmask((H, W), 3, 2.0, 24.0)
    c = MatMulCorrelator((H, W), T, qmask=qm)
    c.correlate(fr)
    _same(c.two_time(2), o.ttcf_exact(fr, qm, 2), rtol=5e-6)


def test_ttcf_rejects_bad_bin(built_lib, cuda_device):
    from dynamix_gb300.correlator import MatMulCorrelator
    z = golden("dense_small_u8")
    fr, qm = z["frames"], z["qmask"]
    c = MatMulCorrelator(fr.shape[1:], fr.shape[0], qmask=qm)
    c.correlate(fr)
    with pytest.raises(ValueError):
        c.two_time(int(qm.max()) + 1)


@pytest.mark.parametrize("name", ["eventy_ttcf_small", "eventy_ttcf_dark", "eventy_ttcf_tiles"])
def test_matches_reference_event_engine(built_lib, cuda_device, name):
    """The two-time matrix, g2 and deviation against the outputs of the
    reference's own nbecorrts_q (event_y.py:104-165, run by
    tests/golden/make_eventy_golden.py): the reference computes in float32,
    so the float32 results agree to 2e-6 relative (TTCF, g2) and the
    deviation to 1e-3 (float statistics on both sides); NaN positions equal."""
    from dynamix_gb300.correlator import MatMulCorrelator
    z = golden(name)
    fr, qm, q = z["frames"], z["qmask"], int(z["ttcf_par"])
    c = MatMulCorrelator(fr.shape[1:], fr.shape[0], qmask=qm)
    res, dev = c.correlate(fr, calc_std=True)
    _same(c.two_time(q), z["trc"].astype(np.float64))
    _same(res[:, 1:], z["res"].astype(np.float64))
    want = z["dev"].astype(np.float64)
    got = c.engine.dev_f64[: c.n_bins].cpu().numpy()[:, 1:]
    assert np.array_equal(np.isfinite(got), np.isfinite(want))
    ok = np.isfinite(want) & (np.abs(want) > 1e-6)
    assert np.all(np.abs(got[ok] - want[ok]) <= 1e-3 * np.abs(want[ok]))
