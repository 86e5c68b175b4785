"""Event layout builders (host side), checked against the reference's layout."""
import numpy as np
import pytest

from conftest import golden
from dynamix_gb300.correlator.event import FramesCompressor


@pytest.mark.parametrize("name", ["dense_small_u8", "dense_u16"])
def test_compress_all_stack_matches_reference(name):
    z = golden(name)
    d, t, o = FramesCompressor.compress_all_stack(z["frames"])
    assert np.array_equal(d, z["ev_data"]) and np.array_equal(t, z["ev_times"])
    assert np.array_equal(o, z["ev_offsets"]) and o.dtype == np.uint32 and t.dtype == np.int32


def test_progressive_compression_equals_whole_stack():
    # the reference's test_progressive_compression (dynamix/correlator/test/test_event.py:62-73)
    z = golden("dense_small_u8")
    fr = z["frames"]
    T = fr.shape[0]
    max_nnz = int((fr > 0).sum(axis=0).max())
    c = FramesCompressor(fr.shape[1:], T, max_nnz, dtype=fr.dtype)
    for f in fr:
        c.process_frame(f)
    d, t, o = c.get_compacted_events()
    rd, rt, ro = FramesCompressor.compress_all_stack(fr)
    assert np.array_equal(d, rd) and np.array_equal(t, rt) and np.array_equal(o, ro)


def test_progressive_compression_rejects_overflow():
    fr = np.ones((5, 2, 2), np.uint8)
    c = FramesCompressor((2, 2), 5, 3, dtype=np.uint8)
    for f in fr[:3]:
        c.process_frame(f)
    with pytest.raises(ValueError):
        c.process_frame(fr[3])
