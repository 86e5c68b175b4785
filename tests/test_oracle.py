"""Pin the CPU oracle against golden vectors made by the reference itself.

The fixtures in tests/golden were produced by running the reference's
``MatMulCorrelator`` and ``FramesCompressor.compress_all_stack`` (script:
tests/golden/make_golden.py).  The float32 port must reproduce the reference
bit for bit; the exact int64/FP64 oracle must agree to float32 rounding.
"""
import numpy as np
import pytest

from conftest import golden
from oracle import g2_oracle as o

CASES = ["dense_small_u8", "dense_bright_u8", "dense_128x128_u8", "dense_u16"]


@pytest.mark.parametrize("name", CASES)
def test_port_matches_reference_bitwise(name):
    z = golden(name)
    res = o.matmul_correlator_port(z["frames"], z["qmask"])
    assert res.dtype == np.float32
    assert np.array_equal(res, z["g2_ref"], equal_nan=True)


@pytest.mark.parametrize("name", CASES)
def test_exact_oracle_matches_reference(name):
    z = golden(name)
    r = o.g2_exact(z["frames"], z["qmask"])
    ref = z["g2_ref"].astype(np.float64)
    # the reference keeps float32 sums; the exact oracle differs by rounding only
    rel = np.nanmax(np.abs(r["g2"] - ref) / np.abs(r["g2"]))
    assert rel < 2e-6
    # the reference test tolerance (test_dense.py:86): 5e-3 absolute
    assert np.nanmax(np.abs(r["g2"] - ref)) < 5e-3


@pytest.mark.parametrize("name", CASES[:2] + CASES[3:])
def test_std_matches_reference(name):
    z = golden(name)
    dev = o.dense_std_exact(z["frames"], z["qmask"])
    ref = z["g2_ref_std"].astype(np.float64)
    ok = np.isfinite(ref) & (np.abs(ref) > 1e-6)
    assert np.max(np.abs(dev[ok] - ref[ok]) / np.abs(ref[ok])) < 1e-3


@pytest.mark.parametrize("name", CASES)
def test_event_layout_matches_reference(name):
    z = golden(name)
    data, times, offsets = o.compress_all_stack(z["frames"])
    assert np.array_equal(data, z["ev_data"])
    assert np.array_equal(times, z["ev_times"])
    assert np.array_equal(offsets, z["ev_offsets"])
    assert offsets.dtype == np.uint32 and times.dtype == np.int32


@pytest.mark.parametrize("name", ["dense_small_u8", "dense_bright_u8", "dense_u16"])
def test_event_and_csr_restatements_equal_dense(name):
    z = golden(name)
    fr, qm = z["frames"], z["qmask"]
    T, H, W = fr.shape
    d = o.g2_exact(fr, qm)
    e = o.event_correlate_exact(z["ev_times"], z["ev_data"], z["ev_offsets"], qm, (H, W), T)
    for k in ("numerator", "sums", "denominator"):
        assert np.array_equal(d[k], e[k])
    c = o.frames_to_csr(fr)
    s = o.csr_correlate_exact(*c, (H, W), T, qmask=qm)
    for k in ("numerator", "sums", "denominator"):
        assert np.array_equal(d[k], s[k])


def test_edge_cases_match_reference():
    z = golden("dense_edge")
    fr = z["frames"]
    r_all = o.g2_exact(fr, None)
    assert r_all["g2"].shape == (1, fr.shape[0])
    assert np.nanmax(np.abs(r_all["g2"] - z["g2_all"]) / np.abs(r_all["g2"])) < 2e-6
    r_gap = o.g2_exact(fr, z["qmask_gap"])
    assert r_gap["g2"].shape == z["g2_gap"].shape
    assert np.all(np.isnan(r_gap["g2"][1])) and np.all(np.isnan(z["g2_gap"][1]))
    ok = ~np.isnan(z["g2_gap"])
    assert np.max(np.abs(r_gap["g2"][ok] - z["g2_gap"][ok]) / np.abs(r_gap["g2"][ok])) < 2e-6
