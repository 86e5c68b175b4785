"""GPU parity of frame compression (dense frames -> event lists) against the
reference's own layout (golden vectors) and the CPU restatements."""
import numpy as np
import pytest

from conftest import golden
from oracle import g2_oracle as o

pytestmark = pytest.mark.gpu


def _to_np(x):
    return x.cpu().numpy()


def _check_layout(got, ref):
    d, t, off = got
    rd, rt, ro = ref
    assert np.array_equal(_to_np(off).astype(np.int64), ro.astype(np.int64))
    assert np.array_equal(_to_np(t), rt)
    assert np.array_equal(_to_np(d).astype(np.int64), rd.astype(np.int64))


@pytest.mark.parametrize("name", ["dense_small_u8", "dense_bright_u8", "dense_128x128_u8", "dense_u16"])
def test_golden_layout(built_lib, cuda_device, name):
    import torch
    from dynamix_gb300.correlator import FramesCompressor
    z = golden(name)
    fr = torch.from_numpy(z["frames"]).to(cuda_device)
    d, t, off = FramesCompressor.compress_all_stack(fr)
    _check_layout((d, t, off), (z["ev_data"], z["ev_times"], z["ev_offsets"]))
    assert d.dtype == fr.dtype and t.dtype == torch.int32
    # numpy in, numpy out in the reference's dtypes
    nd, nt, no = FramesCompressor.compress_all_stack(z["frames"], device=cuda_device)
    assert no.dtype == np.uint32 and nt.dtype == np.int32 and nd.dtype == z["frames"].dtype
    assert np.array_equal(no, z["ev_offsets"]) and np.array_equal(nt, z["ev_times"])
    assert np.array_equal(nd, z["ev_data"])


@pytest.mark.parametrize("dtype,T,shape,density", [
    (np.uint8, 3000, (37, 53), 0.05),      # odd pixel count: scalar loads; T not a multiple of 1024
    (np.uint16, 2500, (64, 96), 0.3),      # vector loads; dense enough for in-place regions
    (np.int8, 1100, (40, 40), 0.1),        # negatives are not events
    (np.int16, 700, (33, 31), 0.2),
    (np.uint8, 1, (16, 16), 0.5),          # a single frame
])
def test_random_stacks(built_lib, cuda_device, dtype, T, shape, density):
    import torch
    from dynamix_gb300.compress import compress_all_stack_device
    rng = np.random.default_rng(T)
    info = np.iinfo(dtype)
    vals = rng.integers(max(info.min, -300), min(info.max, 3000) + 1, size=(T,) + shape)
    keep = rng.random((T,) + shape) < density
    fr = np.where(keep, vals, 0).astype(dtype)
    got = compress_all_stack_device(torch.from_numpy(fr).to(cuda_device))
    _check_layout(got, o.compress_all_stack(fr))


def test_empty_and_full(built_lib, cuda_device):
    import torch
    from dynamix_gb300.compress import compress_all_stack_device
    fr = np.zeros((1500, 8, 8), np.uint8)
    d, t, off = compress_all_stack_device(torch.from_numpy(fr).to(cuda_device))
    assert d.numel() == 0 and t.numel() == 0 and int(off.max()) == 0
    fr = np.full((2100, 8, 16), 7, np.uint8)          # every value an event: regions beyond the shared buffer
    got = compress_all_stack_device(torch.from_numpy(fr).to(cuda_device))
    _check_layout(got, o.compress_all_stack(fr))


def test_long_stack_split_output(built_lib, cuda_device):
    # frame numbers beyond 16 bits (only the split output holds them)
    import torch
    from dynamix_gb300.compress import StackCompressor
    rng = np.random.default_rng(7)
    T, shape = 70000, (4, 8)
    fr = (rng.random((T,) + shape) < 0.01).astype(np.uint8) * rng.integers(1, 5, (T,) + shape).astype(np.uint8)
    comp = StackCompressor(T, 32, device=cuda_device)
    got = comp.run(torch.from_numpy(fr.reshape(T, -1)).to(cuda_device))
    _check_layout(got, o.compress_all_stack(fr))
    with pytest.raises(ValueError):
        comp.emit(torch.from_numpy(fr.reshape(T, -1)).to(cuda_device), packed=True)


def test_packed_words(built_lib, cuda_device):
    import torch
    from dynamix_gb300.compress import StackCompressor
    z = golden("dense_u16")
    fr = z["frames"]
    T = fr.shape[0]
    comp = StackCompressor(T, fr[0].size, device=cuda_device)
    f = torch.from_numpy(fr.reshape(T, -1)).to(cuda_device)
    comp.count(f)
    words, off = comp.emit(f, packed=True)
    w = _to_np(words).view(np.uint32)
    assert np.array_equal(w >> 16, z["ev_times"]) and np.array_equal(w & 0xFFFF, z["ev_data"])
    assert np.array_equal(_to_np(off), z["ev_offsets"].astype(np.int64))


@pytest.mark.parametrize("threshold,with_mask", [(None, True), (40, False), (40, True), (0, False)])
def test_hot_pixel_threshold_and_mask(built_lib, cuda_device, threshold, with_mask):
    import torch
    from dynamix_gb300.compress import compress_all_stack_device
    rng = np.random.default_rng(11)
    T, shape = 2600, (24, 40)
    fr = (rng.poisson(0.3, (T,) + shape)).astype(np.uint8)
    hot = rng.random((T,) + shape) < 2e-4                 # rare bright values
    fr[hot] = 200
    mask0 = (rng.random(shape) < 0.05).astype(np.uint8) if with_mask else None
    rd, rt, ro, rmask, rsum = o.compress_hot_pixels(fr, threshold, mask0)
    m = torch.from_numpy(mask0.ravel().copy()).to(cuda_device) if with_mask else \
        torch.zeros(fr[0].size, dtype=torch.uint8, device=cuda_device)
    s = torch.zeros(fr[0].size, dtype=torch.int64, device=cuda_device)
    got = compress_all_stack_device(torch.from_numpy(fr).to(cuda_device), threshold=threshold, mask=m, sum_frame=s)
    _check_layout(got, (rd, rt, ro))
    assert np.array_equal(_to_np(m).astype(bool), rmask)
    assert np.array_equal(_to_np(s), rsum)


@pytest.mark.parametrize("dtype,density,threshold", [
    (np.uint8, 0.05, None),     # warp chunks of 32 frames assembled in shared memory
    (np.uint8, 0.05, 40),       # the same with the cut frame of the threshold
    (np.uint8, 0.6, None),      # chunks beyond the warp's shared slice: written word by word
    (np.uint16, 0.1, None),     # chunks of 16 frames
    (np.int16, 0.1, 40),
    (np.int8, 0.08, None),
])
def test_chunked_stage(built_lib, cuda_device, dtype, density, threshold):
    # CTA regions (1024 pixels x 1024 frames) far beyond the shared buffer; T leaves a
    # partial last sub-block with a tail shorter than one chunk
    import torch
    from dynamix_gb300.compress import compress_all_stack_device
    rng = np.random.default_rng(int(density * 1000) + (threshold or 0))
    T, shape = 2100, (32, 64)
    info = np.iinfo(dtype)
    vals = rng.integers(1, min(info.max, 60) + 1, size=(T,) + shape)
    fr = np.where(rng.random((T,) + shape) < density, vals, 0).astype(dtype)
    if info.min < 0:
        fr[rng.random((T,) + shape) < 0.05] = -3               # negatives are not events
    mask0 = (rng.random(shape) < 0.03).astype(np.uint8)
    rd, rt, ro, rmask, rsum = o.compress_hot_pixels(fr, threshold, mask0)
    m = torch.from_numpy(mask0.ravel().copy()).to(cuda_device)
    got = compress_all_stack_device(torch.from_numpy(fr).to(cuda_device), threshold=threshold, mask=m)
    _check_layout(got, (rd, rt, ro))
    assert np.array_equal(_to_np(m).astype(bool), rmask)


@pytest.mark.parametrize("threshold", [None, 30])
def test_streaming_equals_whole_stack(built_lib, cuda_device, threshold):
    # the reference's test_progressive_compression (correlator/test/test_event.py:62-73), on the GPU,
    # frames given one by one and in batches
    import torch
    from dynamix_gb300.correlator import FramesCompressor
    rng = np.random.default_rng(3)
    T, shape = 300, (20, 30)
    fr = rng.poisson(0.2, (T,) + shape).astype(np.uint16)
    fr[rng.random((T,) + shape) < 1e-3] = 90
    rd, rt, ro, rmask, rsum = o.compress_hot_pixels(fr, threshold)
    max_nnz = int(np.diff(ro.astype(np.int64)).max()) + 1
    c = FramesCompressor(shape, T, max_nnz, dtype=np.uint16, device=cuda_device, threshold=threshold)
    for f in fr[:10]:
        c.process_frame(f)
    c.process_frames(torch.from_numpy(fr[10:200]).to(cuda_device))
    c.process_frames(fr[200:])
    _check_layout(c.get_compacted_events(), (rd, rt, ro))
    assert np.array_equal(_to_np(c._device.mask).astype(bool), rmask)
    assert np.array_equal(_to_np(c._device.sum_frame), rsum)


def test_streaming_rejects_overflow(built_lib, cuda_device):
    from dynamix_gb300.correlator import FramesCompressor
    fr = np.ones((5, 2, 2), np.uint8)
    c = FramesCompressor((2, 2), 5, 3, dtype=np.uint8, device=cuda_device)
    c.process_frames(fr[:3])
    with pytest.raises(ValueError):
        c.process_frame(fr[3])


def test_compressed_stack_feeds_event_correlator(built_lib, cuda_device):
    import torch
    from dynamix_gb300.correlator import EventCorrelator, FramesCompressor
    z = golden("dense_small_u8")
    fr, qm = z["frames"], z["qmask"]
    T = fr.shape[0]
    d, t, off = FramesCompressor.compress_all_stack(torch.from_numpy(fr).to(cuda_device))
    c = EventCorrelator(fr.shape[1:], T, max_events_count=1, qmask=qm)
    g = c.correlate(t, d, off)
    ref = o.g2_exact(fr, qm)
    assert np.array_equal(c.numerator, ref["numerator"])
    assert np.array_equal(g, ref["g2"].astype(np.float32), equal_nan=True)


@pytest.mark.parametrize("name", ["neiger_thr40", "neiger_thr0", "neiger_nomask"])
def test_hot_pixel_matches_reference_reader(built_lib, cuda_device, name):
    """Threshold, sticky mask, sum frame and trace against the buffers of the
    reference's own neigercompress (io/readdata.py:441-457) called frame by
    frame (tests/golden/make_eventy_golden.py): bit-exact."""
    import torch
    from dynamix_gb300.compress import compress_all_stack_device
    z = golden(name)
    fr = z["frames"]
    cnt = z["cnt"].astype(np.int64)
    rd = np.concatenate([z["evs"][p, 1:c + 1] for p, c in enumerate(cnt)]).astype(np.int64)
    rt = np.concatenate([z["tms"][p, 1:c + 1] for p, c in enumerate(cnt)]).astype(np.int64)
    ro = np.concatenate([[0], np.cumsum(cnt)])
    m = torch.from_numpy(z["mask0"].astype(np.uint8).copy()).to(cuda_device)
    s = torch.zeros(fr[0].size, dtype=torch.int64, device=cuda_device)
    d, t, off = compress_all_stack_device(torch.from_numpy(fr).to(cuda_device), threshold=int(z["threshold"]),
                                          mask=m, sum_frame=s)
    assert np.array_equal(_to_np(off).astype(np.int64), ro)
    assert np.array_equal(_to_np(t).astype(np.int64), rt)
    assert np.array_equal(_to_np(d).astype(np.int64), rd)
    assert np.array_equal(_to_np(m).astype(bool), z["mask_after"].astype(bool))
    assert np.array_equal(_to_np(s), z["afr"].astype(np.int64))
    trace = np.bincount(_to_np(t).astype(np.int64), weights=_to_np(d).astype(np.float64), minlength=fr.shape[0])
    assert np.array_equal(trace.astype(np.int64), z["trace"].astype(np.int64))
