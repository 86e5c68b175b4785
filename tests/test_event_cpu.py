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


@pytest.mark.parametrize("n_ctas", [1, 3, 152, 5000])
def test_cta_ranges_cover_each_pixel_once(n_ctas):
    from dynamix_gb300.engine_sparse import cta_ranges
    rng = np.random.default_rng(n_ctas)
    bins = np.sort(rng.integers(0, 9, 1234)).astype(np.int32)
    ro, rb, cro = cta_ranges(bins, n_ctas)
    assert ro[0] == 0 and ro[-1] == bins.size and np.all(np.diff(ro) > 0)
    assert cro[0] == 0 and cro[-1] == rb.size and np.all(np.diff(cro) >= 1)
    for r in range(rb.size):                         # every range holds one bin
        assert np.all(bins[ro[r]:ro[r + 1]] == rb[r])
    sizes = [ro[cro[c + 1]] - ro[cro[c]] for c in range(cro.size - 1)]
    assert max(sizes) - min(sizes) <= 1              # equal slices


def test_cta_ranges_empty():
    from dynamix_gb300.engine_sparse import cta_ranges
    ro, rb, cro = cta_ranges(np.zeros(0, np.int32), 152)
    assert ro.tolist() == [0] and rb.size == 0 and cro.tolist() == [0, 0]


@pytest.mark.parametrize("npix,chunks,taper", [(2162 * 2068, 8, 2), (1000, 8, 0), (10, 8, 2), (3, 8, 2)])
def test_host_chunk_bounds_cover_pixels(npix, chunks, taper):
    """Pixel chunks of the pinned-host event pipeline: they tile [0, npix),
    and the tapered tail never grows."""
    from dynamix_gb300.engine_sparse import EventEngine
    b = np.asarray(EventEngine.host_chunk_bounds(npix, chunks, taper))
    assert b[0] == 0 and b[-1] == npix and np.all(np.diff(b) >= 0)
    assert b.size - 1 <= chunks + taper
    if npix >= 64 * chunks:
        d = np.diff(b)
        assert np.all(d[chunks - 1:-1] <= d[chunks - 2:-2] + 1)
