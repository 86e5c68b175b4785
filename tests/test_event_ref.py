"""The oracle pinned against the reference's own event kernels.

Fixtures ``event_ref_*.npz`` hold the outputs of ``evtcorrelator.cl``
(``event_correlator`` + ``normalize_correlation``), compiled as C and run on the
CPU by ``tests/golden/make_event_golden.py``.  The reference launches with
``image_height = shape[1]`` (``event.py:183``) and so ignores the rows
``y >= width`` of a tall image; the oracle reproduces its sums once those rows
are masked out.
"""
import numpy as np
import pytest

from conftest import golden
from oracle import g2_oracle as o

CASES = ["event_ref_u8", "event_ref_u16", "event_ref_tall_u8"]


def visible_qmask(z):
    qm = z["qmask"].copy()
    qm[qm.shape[1]:] = 0                     # rows the reference's launch reaches
    return qm


def full_scale(z):
    """The reference's scale factors: pixel counts of the whole q-mask."""
    return list(o.bins_from_qmask(z["qmask"], z["qmask"].shape)[3])


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference_event_kernel(name):
    z = golden(name)
    fr = z["frames"]
    T, H, W = fr.shape
    qm = visible_qmask(z)
    ref = o.event_correlate_exact(z["ev_times"], z["ev_data"], z["ev_offsets"], qm, (H, W), T,
                                  scale_factor=full_scale(z))
    assert np.array_equal(ref["numerator"], z["res_int"].astype(np.int64))
    assert np.array_equal(ref["sums"], z["sums"].astype(np.int64))
    g, rg = ref["g2"], z["g2"].astype(np.float64)
    ok = np.isfinite(g)
    assert np.array_equal(ok, np.isfinite(rg))
    # the reference's float32 denominator loop: relative error ~ T * 2^-24
    assert np.all(np.abs(rg[ok] - g[ok]) <= 1e-5 * np.abs(g[ok]))


@pytest.mark.parametrize("name", CASES)
def test_c_oracle_matches_reference_event_kernel(name):
    z = golden(name)
    T, H, W = z["frames"].shape
    N, S = o.event_pairsum_c(z["ev_times"], z["ev_data"], z["ev_offsets"], visible_qmask(z), (H, W), T,
                             n_threads=3)
    assert np.array_equal(N, z["res_int"].astype(np.int64))
    assert np.array_equal(S, z["sums"].astype(np.int64))


def test_tall_image_rows_dropped_by_reference():
    z = golden("event_ref_tall_u8")
    T, H, W = z["frames"].shape
    assert H > W
    full = o.g2_exact(z["frames"], z["qmask"])
    assert not np.array_equal(full["numerator"], z["res_int"].astype(np.int64))


@pytest.mark.parametrize("name", CASES)
def test_fixture_still_reproduced_by_reference_kernel(name):
    """Where the reference sources are present, rerun its kernels now."""
    from oracle import build_oracle
    if not build_oracle.build_ref():
        pytest.skip("reference sources not present")
    z = golden(name)
    T, H, W = z["frames"].shape
    r = o.reference_event_correlate(z["ev_times"], z["ev_data"], z["ev_offsets"], z["qmask"], (H, W), T,
                                    n_threads=2)
    for k in ("res_int", "sums", "g2"):
        assert np.array_equal(r[k], z[k]), k
