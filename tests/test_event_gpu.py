"""GPU parity of the event-list correlator against the CPU oracle."""
import numpy as np
import pytest

from conftest import golden
from oracle import g2_oracle as o

pytestmark = pytest.mark.gpu


def check(c, ref, g):
    assert np.array_equal(c.sums, ref["sums"])
    assert np.array_equal(c.numerator, ref["numerator"])
    assert np.array_equal(c.denominator, ref["denominator"])
    assert np.array_equal(g, ref["g2"].astype(np.float32), equal_nan=True)


@pytest.mark.parametrize("name", ["dense_small_u8", "dense_bright_u8", "dense_128x128_u8", "dense_u16"])
def test_reference_event_layout(built_lib, cuda_device, name):
    from dynamix_gb300.correlator import EventCorrelator
    z = golden(name)
    fr, qm = z["frames"], z["qmask"]
    T = fr.shape[0]
    ref = o.g2_exact(fr, qm)
    c = EventCorrelator(fr.shape[1:], T, max_events_count=int(np.diff(z["ev_offsets"]).max()), qmask=qm)
    g = c.correlate(z["ev_times"], z["ev_data"], z["ev_offsets"])
    check(c, ref, g)
    # the reference's own float32 g2 agrees to float32 rounding
    rg = z["g2_ref"]
    ok = np.isfinite(rg)
    assert np.all(np.abs(g[ok] - rg[ok]) <= 2e-6 * np.abs(rg[ok]))


def test_shuffled_events_and_scale_factor(built_lib, cuda_device):
    from dynamix_gb300.correlator import EventCorrelator
    z = golden("dense_small_u8")
    fr, qm = z["frames"], z["qmask"]
    T = fr.shape[0]
    d, t, off = z["ev_data"].copy(), z["ev_times"].copy(), z["ev_offsets"]
    rng = np.random.default_rng(0)
    for p in range(off.size - 1):                       # order inside a pixel does not matter
        s, e = off[p], off[p + 1]
        perm = rng.permutation(e - s) + s
        d[s:e], t[s:e] = d[perm], t[perm]
    nb = int(qm.max())
    sf = np.linspace(10, 50, nb)
    c = EventCorrelator(fr.shape[1:], T, 64, qmask=qm, scale_factor=list(sf))
    g = c.correlate(t, d.astype(np.int32), off.astype(np.int64))
    ref = o.g2_exact(fr, qm, scale_factor=list(sf))
    check(c, ref, g)


def test_qmask_none_and_long_stack_global_path(built_lib, cuda_device):
    """T above the shared-memory capacity uses the global-atomic kernel."""
    from dynamix_gb300.correlator import EventCorrelator, FramesCompressor
    rng = np.random.default_rng(3)
    T, shape = 30000, (3, 4)
    fr = (rng.random((T,) + shape) < 0.01).astype(np.uint8) * rng.integers(1, 4, (T,) + shape).astype(np.uint8)
    d, t, off = FramesCompressor.compress_all_stack(fr)
    c = EventCorrelator(shape, T, int(np.diff(off).max()))
    g = c.correlate(t, d, off)
    ref = o.event_correlate_exact(t, d, off, None, shape, T)
    check(c, ref, g)


def test_large_counts_use_global_path(built_lib, cuda_device):
    from dynamix_gb300.correlator import EventCorrelator, FramesCompressor
    rng = np.random.default_rng(4)
    T, shape = 300, (6, 5)
    fr = np.where(rng.random((T,) + shape) < 0.05, rng.integers(40000, 65535, (T,) + shape), 0).astype(np.uint16)
    qm = np.ones(shape, np.int32)
    qm[:, 3:] = 2
    d, t, off = FramesCompressor.compress_all_stack(fr)
    c = EventCorrelator(shape, T, 64, qmask=qm)
    g = c.correlate(t, d, off)
    check(c, o.g2_exact(fr, qm), g)


def test_event_errors(built_lib, cuda_device):
    from dynamix_gb300.correlator import EventCorrelator
    z = golden("dense_small_u8")
    fr = z["frames"]
    c = EventCorrelator(fr.shape[1:], fr.shape[0], 4, total_events_count=10, allow_reallocate=False)
    with pytest.raises(ValueError):
        c.correlate(z["ev_times"], z["ev_data"], z["ev_offsets"])
    c = EventCorrelator(fr.shape[1:], fr.shape[0] - 10, 4)
    with pytest.raises(ValueError):                     # times beyond nframes
        c.correlate(z["ev_times"], z["ev_data"], z["ev_offsets"])
    with pytest.raises(AssertionError):
        c.correlate(z["ev_times"], z["ev_data"], z["ev_offsets"][:-1])


@pytest.mark.parametrize("bright", [False, True])
def test_many_pixels_bins_cut_across_ctas(built_lib, cuda_device, bright):
    """More binned pixels than CTAs, bins split between CTAs and CTAs holding
    several bins; bright counts take the global-atomic kernel."""
    from dynamix_gb300.correlator import EventCorrelator, FramesCompressor
    from dynamix_gb300.speckle import annular_qmask, speckle_numpy
    T, shape = 400, (40, 50)
    fr = speckle_numpy(T, shape, 0.95, 0.2, seed=11, dtype=np.uint16 if bright else np.uint8)
    if bright:
        fr = np.where(fr > 0, 46341 + fr.astype(np.int64) * 97 % 19000, 0).astype(np.uint16)   # max^2 >= 2^31
    qm = annular_qmask(shape, 7, 2, 30)
    d, t, off = FramesCompressor.compress_all_stack(fr)
    c = EventCorrelator(shape, T, int(np.diff(off).max()), qmask=qm)
    g = c.correlate(t, d, off)
    assert c.engine.last["kernel"] == ("global" if bright else "smem")
    check(c, o.g2_exact(fr, qm), g)


@pytest.mark.parametrize("name", ["event_ref_u8", "event_ref_u16", "event_ref_tall_u8"])
def test_against_reference_event_kernel(built_lib, cuda_device, name):
    """Bit-exact N and S against the reference's own event kernel (rows the
    reference reaches; it skips rows y >= width of a tall image)."""
    from dynamix_gb300.correlator import EventCorrelator
    z = golden(name)
    T, H, W = z["frames"].shape
    qm = z["qmask"].copy()
    qm[W:] = 0
    sf = list(o.bins_from_qmask(z["qmask"], (H, W))[3])       # scale of the whole q-mask, as the reference
    c = EventCorrelator((H, W), T, int(np.diff(z["ev_offsets"]).max()), qmask=qm, scale_factor=sf)
    g = c.correlate(z["ev_times"], z["ev_data"], z["ev_offsets"])
    assert np.array_equal(c.numerator, z["res_int"].astype(np.int64))
    assert np.array_equal(c.sums, z["sums"].astype(np.int64))
    rg = z["g2"]
    ok = np.isfinite(rg)
    assert np.array_equal(ok, np.isfinite(g))
    assert np.all(np.abs(g[ok] - rg[ok]) <= 1e-5 * np.abs(rg[ok]))


def test_pinned_host_events_pipeline(built_lib, cuda_device):
    # pinned host event arrays take the chunked copy/pair-sum pipeline; the
    # result equals the oracle, and bad inputs raise as on the other paths
    import torch
    from dynamix_gb300.correlator import EventCorrelator
    z = golden("dense_128x128_u8")
    fr, qm = z["frames"], z["qmask"]
    T = fr.shape[0]
    ref = o.g2_exact(fr, qm)
    t = torch.from_numpy(z["ev_times"]).pin_memory()
    d = torch.from_numpy(z["ev_data"]).pin_memory()
    off = torch.from_numpy(z["ev_offsets"].astype(np.int64)).pin_memory()
    c = EventCorrelator(fr.shape[1:], T, 1, qmask=qm)
    assert c.engine.host_pipeline_ok(t, d, off)
    g = c.correlate(t, d, off)
    check(c, ref, g)
    eng = c.engine
    assert eng.last.get("host_chunks") == len(eng.host_chunk_bounds(eng.npix, eng.HOST_CHUNKS, eng.HOST_TAPER)) - 1
    g2 = c.correlate(t, d, off)                      # a second call gives the same result
    assert np.array_equal(g, g2)
    bad_t = t.clone().pin_memory()
    bad_t[len(bad_t) // 2] = T                       # a frame outside [0, T)
    with pytest.raises(ValueError):
        c.correlate(bad_t, d, off)
    bad_off = off.clone().pin_memory()
    bad_off[5] = bad_off[6] + 1                      # decreasing offsets
    with pytest.raises(ValueError):
        c.correlate(t, d, bad_off)
    g3 = c.correlate(t, d, off)                      # and the correlator still works
    assert np.array_equal(g, g3)
