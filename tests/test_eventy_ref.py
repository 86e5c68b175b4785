"""The oracle pinned against the reference's legacy event engine and its
streaming compressor.

Fixtures ``eventy_ttcf_*`` hold the outputs of ``nbecorrts_q``
(``correlator/event_y.py:104-165``: event g2 ``res`` for lags 1..T-1, its
deviation ``dev`` and the two-time matrix ``trc`` of bin ``ttcf_par``);
``neiger_*`` hold the buffers of ``neigercompress`` (``io/readdata.py:441-457``)
called frame by frame (events in columns 1..cnt of ``evs``/``tms``, the sum
frame ``afr``, the mask after the stack, the per-frame trace).  Both were made
by running the reference's own functions (``tests/golden/make_eventy_golden.py``).
The reference computes in float32; the oracle in float64, so the float
results agree to float32 rounding (2e-6 relative) and the compression exactly.
"""
import numpy as np
import pytest

from conftest import golden
from oracle import g2_oracle as o

TTCF = ["eventy_ttcf_small", "eventy_ttcf_dark", "eventy_ttcf_tiles"]
HOT = ["neiger_thr40", "neiger_thr0", "neiger_nomask"]
RTOL = 2e-6


def close(got, ref, rtol=RTOL):
    ref = np.asarray(ref, dtype=np.float64)
    got = np.asarray(got, dtype=np.float64)
    assert got.shape == ref.shape
    assert np.array_equal(np.isnan(got), np.isnan(ref))
    assert np.array_equal(np.isinf(got), np.isinf(ref))
    ok = np.isfinite(ref)
    assert np.all(np.abs(got[ok] - ref[ok]) <= rtol * np.abs(ref[ok]) + 1e-30)


def reference_events(z):
    """Events of the reference's reader buffers in the FramesCompressor layout."""
    cnt = z["cnt"].astype(np.int64)
    parts = [(z["evs"][p, 1:c + 1], z["tms"][p, 1:c + 1]) for p, c in enumerate(cnt)]
    data = np.concatenate([d for d, _ in parts]).astype(np.int64)
    times = np.concatenate([t for _, t in parts]).astype(np.int64)
    offsets = np.concatenate([[0], np.cumsum(cnt)])
    return data, times, offsets


@pytest.mark.parametrize("name", TTCF)
def test_ttcf_oracle_matches_reference(name):
    z = golden(name)
    fr, qm, q = z["frames"], z["qmask"], int(z["ttcf_par"])
    close(o.ttcf_exact(fr, qm, q), z["trc"])


@pytest.mark.parametrize("name", TTCF)
def test_event_g2_and_deviation_match_reference(name):
    z = golden(name)
    fr, qm = z["frames"], z["qmask"]
    close(o.g2_exact(fr, qm)["g2"][:, 1:], z["res"])            # res[q-1, i-1] is lag i
    want = o.dense_std_exact(fr, qm)[:, 1:]
    dev = z["dev"].astype(np.float64)
    assert np.array_equal(np.isfinite(want), np.isfinite(dev))
    ok = np.isfinite(dev)
    assert np.all(np.abs(want[ok] - dev[ok]) <= RTOL * np.abs(dev[ok]) + 1e-12)


def test_dark_case_is_not_mirrored():
    z = golden("eventy_ttcf_dark")
    trc = z["trc"]
    assert np.isnan(np.diag(trc, -5)).any()                      # the rule of event_y.py:150-152 is off
    z = golden("eventy_ttcf_small")
    assert np.allclose(np.triu(z["trc"], 1), np.tril(z["trc"], -1).T)


@pytest.mark.parametrize("name", HOT)
def test_hot_pixel_compression_matches_reference(name):
    z = golden(name)
    fr = z["frames"]
    d, t, off, mask, sums = o.compress_hot_pixels(fr, int(z["threshold"]), z["mask0"].reshape(fr.shape[1:]))
    rd, rt, ro = reference_events(z)
    assert np.array_equal(off.astype(np.int64), ro)
    assert np.array_equal(d.astype(np.int64), rd)
    assert np.array_equal(t.astype(np.int64), rt)
    assert np.array_equal(mask, z["mask_after"].astype(bool))
    assert np.array_equal(sums, z["afr"].astype(np.int64))
    trace = np.bincount(t, weights=d.astype(np.float64), minlength=fr.shape[0])
    assert np.array_equal(trace.astype(np.int64), z["trace"].astype(np.int64))
