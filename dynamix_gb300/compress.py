"""Frame compression on the device: dense frames -> per-pixel event lists.

Device counterpart of dynamix's ``FramesCompressor`` (correlator/event.py:
207-321): ``compress_all_stack`` (event.py:267-284) for a whole (T, H, W)
stack and the streaming ``process_frame`` / ``get_compacted_events``
(event.py:286-321), with the hot-pixel threshold, sticky mask and sum frame of
the streaming reader (io/readdata.py:441-468, ``neigercompress``): a value
above the threshold masks its pixel from that frame on, a masked pixel gives
no events, and the sum frame adds every raw value.

Kernels (``csrc/g2_compress.cu``, gather in ``csrc/g2_csr.cu``): count per
(1024-frame sub-block, pixel), the sticky-mask pass, two scans, a stage pass
that writes each kept value as ``((t - sub-block start) << 16) | v`` in
(sub-block, pixel, frame) order, and the tiled gather into the per-pixel lists
(frame order within a pixel, the reference's layout).  Frames are uint8,
uint16, int8 or int16; only values > 0 are events.
"""
from __future__ import annotations

import numpy as np

from . import _lib
from .engine import DeviceError, _torch, ptr, require_cuda, stream_handle

SUBBLOCK = 1024
BLK_PX = 1024
TILE_P = 64
MAX_FRAMES_SPLIT = 400 * SUBBLOCK    # frame numbers written as int32 (split output)
MAX_FRAMES_PACKED = 65536            # frame numbers inside packed words


def _optr(t):
    """Device pointer of a tensor, or NULL for None."""
    return None if t is None else ptr(t)


def elem_kind(dtype):
    """Kind code of the C ABI for a torch dtype (1 u8, 2 u16, -1 i8, -2 i16)."""
    torch = _torch()
    kinds = {torch.uint8: 1, torch.uint16: 2, torch.int8: -1, torch.int16: -2}
    if dtype not in kinds:
        raise TypeError("frames must be uint8, uint16, int8 or int16, got %s" % dtype)
    return kinds[dtype]


def frames_on_device(frames, dev):
    """A contiguous (T, npix) device tensor holding the frames (numpy arrays
    are copied; CUDA tensors on ``dev`` are used in place)."""
    torch = _torch()
    if isinstance(frames, torch.Tensor):
        t = frames
    else:
        a = np.asarray(frames)
        if a.dtype not in (np.uint8, np.uint16, np.int8, np.int16):
            raise TypeError("frames must be uint8, uint16, int8 or int16, got %s" % a.dtype)
        t = torch.from_numpy(np.ascontiguousarray(a))
    if t.dim() < 2:
        raise ValueError("frames must have a frame axis and pixel axes")
    elem_kind(t.dtype)
    return t.to(dev).reshape(t.shape[0], -1).contiguous()


class StackCompressor:
    """``compress_all_stack`` on the device for stacks of ``nframes`` frames of
    ``npix`` pixels; the work buffers are kept for later calls.

    ``threshold`` (>= 0) and ``mask`` (device uint8 per pixel, updated in
    place) give the sticky hot-pixel mask; ``sum_frame`` (device int64 per
    pixel) gets every raw value added.
    """

    def __init__(self, nframes, npix, threshold=None, device=None):
        torch = _torch()
        self.lib = _lib.load()
        self.dev = require_cuda(device)
        self.T, self.npix = int(nframes), int(npix)
        if self.T <= 0 or self.npix <= 0:
            raise ValueError("nframes and npix must be positive")
        if self.T > MAX_FRAMES_SPLIT:
            raise ValueError("at most %d frames per stack" % MAX_FRAMES_SPLIT)
        self.threshold = -1 if threshold is None else int(threshold)
        if threshold is not None and not 0 <= self.threshold < 2 ** 31:
            raise ValueError("threshold must be a non-negative integer")
        self.n_sb = -(-self.T // SUBBLOCK)
        self.n_blk = -(-self.npix // BLK_PX)
        self.n_tiles = -(-self.npix // TILE_P)
        i16, i32, dev = torch.int16, torch.int32, self.dev
        self.sb_counts = torch.empty(self.n_sb * self.npix, dtype=i16, device=dev)
        thr = self.threshold >= 0
        self.sb_first = torch.empty(self.n_sb * self.npix, dtype=i16, device=dev) if thr else None
        self.sb_before = torch.empty(self.n_sb * self.npix, dtype=i16, device=dev) if thr else None
        nb = self.n_sb * self.n_blk
        self.blk_totals = torch.empty(nb, dtype=i32, device=dev)
        self.blk_base = torch.empty(nb + 1, dtype=i32, device=dev)
        self.blk_scratch = torch.empty(max(1, -(-nb // 8192)), dtype=i32, device=dev)
        self.counts = torch.empty(self.npix, dtype=i32, device=dev)
        self.ev_off = torch.empty(self.npix + 1, dtype=i32, device=dev)
        self.scan_scratch = torch.empty(max(1, -(-self.npix // 8192)), dtype=i32, device=dev)
        self.tile_pos = torch.empty(self.n_sb * self.n_tiles, dtype=i32, device=dev)
        self.t_cut = torch.empty(self.npix, dtype=i32, device=dev)
        self.err = torch.zeros(1, dtype=i32, device=dev)
        self.stage = None
        self.n_events = 0
        self.profile = False
        self.marks = []

    def _mark(self, name):
        if self.profile:
            torch = _torch()
            e = torch.cuda.Event(enable_timing=True)
            e.record(torch.cuda.current_stream(self.dev))
            self.marks.append((name, e))

    def stage_times(self, calls=1):
        """Milliseconds of each pass (CUDA events), averaged over the ``calls``
        profiled calls since the last reading."""
        torch = _torch()
        torch.cuda.synchronize(self.dev)
        out = {}
        for (_, a), (name, b) in zip(self.marks, self.marks[1:]):
            if name != "start":  # "start" closes the gap between two calls
                out[name] = out.get(name, 0.0) + a.elapsed_time(b) / calls
        self.marks = []
        return out

    def _stage_buffer(self, n):
        torch = _torch()
        if self.stage is None or self.stage.numel() < max(n, 1):
            self.stage = None
            self.stage = torch.empty(max(n, 1), dtype=torch.int32, device=self.dev)
        return self.stage

    def count(self, frames, mask=None, sum_frame=None):
        """Passes 1-3 on a (T, npix) device tensor; returns the event count
        (one device-to-host read)."""
        torch = _torch()
        f = frames
        if f.dim() != 2 or f.shape[0] != self.T or f.shape[1] != self.npix or not f.is_contiguous():
            raise ValueError("frames must be a contiguous (%d, %d) tensor" % (self.T, self.npix))
        if f.device != self.dev:
            raise ValueError("frames must be on %s" % self.dev)
        for name, t, dt in (("mask", mask, torch.uint8), ("sum_frame", sum_frame, torch.int64)):
            if t is not None and (t.device != self.dev or t.dtype != dt or t.numel() != self.npix
                                  or not t.is_contiguous()):
                raise ValueError("%s must be a contiguous %s tensor of %d elements on %s"
                                 % (name, dt, self.npix, self.dev))
        kind = elem_kind(f.dtype)
        st = stream_handle(self.dev)
        self.err.zero_()
        self._mark("start")
        self._cut = self.threshold >= 0 or mask is not None
        _lib.check(self.lib.g2_compress_count(ptr(f), kind, self.T, self.npix, self.threshold, ptr(self.sb_counts),
                                              _optr(self.sb_first), _optr(self.sb_before), ptr(self.blk_totals),
                                              _optr(sum_frame), st), "g2_compress_count")
        self._mark("count")
        _lib.check(self.lib.g2_compress_finish(ptr(self.sb_counts), _optr(self.sb_first), _optr(self.sb_before),
                                               self.T, self.npix, _optr(mask), ptr(self.blk_totals),
                                               ptr(self.counts), ptr(self.t_cut) if self._cut else None, st),
                   "g2_compress_finish")
        self._mark("finish")
        _lib.check(self.lib.g2_exclusive_scan_u32(ptr(self.counts), self.npix, ptr(self.ev_off),
                                                  ptr(self.scan_scratch), self.scan_scratch.numel(), st),
                   "g2_exclusive_scan_u32")
        nb = self.n_sb * self.n_blk
        _lib.check(self.lib.g2_exclusive_scan_u32(ptr(self.blk_totals), nb, ptr(self.blk_base),
                                                  ptr(self.blk_scratch), self.blk_scratch.numel(), st),
                   "g2_exclusive_scan_u32")
        self._mark("scans")
        self.n_events = int(self.ev_off[-1].to(torch.int64).item()) & 0xFFFFFFFF
        return self.n_events

    def emit(self, frames, packed=False):
        """Passes 4-5 after :meth:`count`: ``(data, times int32, offsets int64)``
        device tensors (data in the frames' dtype), or ``(words, offsets)``
        with ``packed`` (``(t << 16) | v`` as int32; at most 65,536 frames)."""
        torch = _torch()
        n = self.n_events
        st = stream_handle(self.dev)
        stage = self._stage_buffer(n)
        self._mark("host_read")  # from the scans to here: the event count read and the output allocation
        _lib.check(self.lib.g2_compress_stage(ptr(frames), elem_kind(frames.dtype), self.T, self.npix,
                                              ptr(self.sb_counts), ptr(self.t_cut) if self._cut else None,
                                              ptr(self.blk_base), ptr(self.tile_pos), ptr(stage), stage.numel(),
                                              ptr(self.err), st), "g2_compress_stage")
        self._mark("stage")
        if packed:
            if self.T > MAX_FRAMES_PACKED:
                raise ValueError("packed event words hold at most %d frames" % MAX_FRAMES_PACKED)
            words = torch.empty(max(n, 1), dtype=torch.int32, device=self.dev)
            _lib.check(self.lib.g2_events_gather_rel(ptr(stage), ptr(self.tile_pos), ptr(self.sb_counts), self.T,
                                                     self.npix, n, ptr(self.ev_off), 0, ptr(words), None, None,
                                                     ptr(self.err), st), "g2_events_gather_rel")
            self._mark("gather")
            self.check_error()
            return words[:n], self.offsets()
        edt = torch.uint16 if frames.element_size() == 2 else torch.uint8
        times = torch.empty(max(n, 1), dtype=torch.int32, device=self.dev)
        data = torch.empty(max(n, 1), dtype=edt, device=self.dev)
        _lib.check(self.lib.g2_events_gather_rel(ptr(stage), ptr(self.tile_pos), ptr(self.sb_counts), self.T,
                                                 self.npix, n, ptr(self.ev_off), frames.element_size(), None,
                                                 ptr(times), ptr(data), ptr(self.err), st), "g2_events_gather_rel")
        self._mark("gather")
        self.check_error()
        return data[:n].view(frames.dtype), times[:n], self.offsets()

    def offsets(self):
        """Event offsets (int64, npix + 1) of the last call."""
        torch = _torch()
        return self.ev_off.to(torch.int64) & 0xFFFFFFFF

    def run(self, frames, mask=None, sum_frame=None, packed=False):
        self.count(frames, mask, sum_frame)
        return self.emit(frames, packed)

    def check_error(self):
        e = int(self.err.item())
        if e:
            raise DeviceError("frame compression reported device error bits 0x%x" % e)


_stack_cache = {}


def compress_all_stack_device(frames, device=None, threshold=None, mask=None, sum_frame=None):
    """``compress_all_stack`` of a (T, H, W) stack on the device.  Returns
    ``(data, times int32, offsets)``: CUDA tensors for a CUDA input (offsets
    int64), numpy arrays in the reference's dtypes (offsets uint32) for a
    numpy input."""
    torch = _torch()
    on_gpu = isinstance(frames, torch.Tensor) and frames.is_cuda
    dev = frames.device if on_gpu else require_cuda(device)
    f = frames_on_device(frames, dev)
    key = (f.shape[0], f.shape[1], threshold, str(dev))
    comp = _stack_cache.get(key)
    if comp is None:
        if len(_stack_cache) > 8:
            _stack_cache.clear()
        comp = _stack_cache[key] = StackCompressor(f.shape[0], f.shape[1], threshold=threshold, device=dev)
    data, times, offsets = comp.run(f, mask=mask, sum_frame=sum_frame)
    if on_gpu:
        return data, times, offsets
    return data.cpu().numpy(), times.cpu().numpy(), offsets.cpu().numpy().astype(np.uint32)


class StreamCompressor:
    """Streaming compression on the device (``process_frame`` /
    ``get_compacted_events``): per pixel a row of ``max_nnz`` events and
    frame numbers; a batch of frames is appended per call."""

    def __init__(self, shape, nframes, max_nnz, dtype, threshold=None, device=None):
        torch = _torch()
        self.lib = _lib.load()
        self.dev = require_cuda(device)
        self.shape = tuple(int(s) for s in shape)
        self.npix = int(np.prod(self.shape))
        self.nframes = int(nframes)
        self.max_nnz = int(max_nnz)
        if self.max_nnz <= 0:
            raise ValueError("max_nnz must be positive")
        self.threshold = -1 if threshold is None else int(threshold)
        tdt = dtype if isinstance(dtype, torch.dtype) else {np.dtype(np.uint8): torch.uint8,
                                                             np.dtype(np.uint16): torch.uint16,
                                                             np.dtype(np.int8): torch.int8,
                                                             np.dtype(np.int16): torch.int16}.get(np.dtype(dtype))
        if tdt is None:
            raise TypeError("frames must be uint8, uint16, int8 or int16, got %s" % dtype)
        self.dtype = tdt
        elem_kind(tdt)
        self.events = torch.zeros((self.npix, self.max_nnz), dtype=tdt, device=self.dev)
        self.times = torch.zeros((self.npix, self.max_nnz), dtype=torch.int32, device=self.dev)
        self.events_counter = torch.zeros(self.npix, dtype=torch.int32, device=self.dev)
        self.mask = torch.zeros(self.npix, dtype=torch.uint8, device=self.dev)
        self.sum_frame = torch.zeros(self.npix, dtype=torch.int64, device=self.dev)
        self.err = torch.zeros(1, dtype=torch.int32, device=self.dev)
        self.scan_scratch = torch.empty(max(1, -(-self.npix // 8192)), dtype=torch.int32, device=self.dev)
        self.frames_counter = 0

    def process_frames(self, frames):
        """Append a batch of frames ((B, H, W) or one (H, W) frame)."""
        f = frames_on_device(frames if np.ndim(frames) == len(self.shape) + 1 else frames[None], self.dev)
        if f.shape[1] != self.npix:
            raise ValueError("frames must have %d pixels" % self.npix)
        if f.dtype != self.dtype:
            f = f.to(self.dtype)
        _lib.check(self.lib.g2_stream_compress(ptr(f), elem_kind(f.dtype), f.shape[0], self.frames_counter,
                                               self.npix, self.max_nnz, self.threshold, ptr(self.mask),
                                               ptr(self.sum_frame), ptr(self.events), ptr(self.times),
                                               ptr(self.events_counter), ptr(self.err), stream_handle(self.dev)),
                   "g2_stream_compress")
        self.frames_counter += f.shape[0]
        e = int(self.err.item())
        if e & _lib.DEVERR_RANGE:
            raise ValueError("a pixel has more than max_nnz=%d events" % self.max_nnz)
        if e:
            raise DeviceError("stream compression reported device error bits 0x%x" % e)

    def get_compacted_events(self):
        """``(events, times int32, offsets int64)`` device tensors of the
        frames processed so far."""
        torch = _torch()
        st = stream_handle(self.dev)
        off = torch.empty(self.npix + 1, dtype=torch.int32, device=self.dev)
        _lib.check(self.lib.g2_exclusive_scan_u32(ptr(self.events_counter), self.npix, ptr(off),
                                                  ptr(self.scan_scratch), self.scan_scratch.numel(), st),
                   "g2_exclusive_scan_u32")
        n = int(off[-1].to(torch.int64).item()) & 0xFFFFFFFF
        data = torch.empty(max(n, 1), dtype=self.dtype, device=self.dev)
        times = torch.empty(max(n, 1), dtype=torch.int32, device=self.dev)
        _lib.check(self.lib.g2_stream_compact(ptr(self.events), ptr(self.times), ptr(self.events_counter),
                                              self.events.element_size(), self.npix, self.max_nnz, ptr(off), n,
                                              ptr(data), ptr(times), ptr(self.err), st), "g2_stream_compact")
        e = int(self.err.item())
        if e:
            raise DeviceError("compaction reported device error bits 0x%x" % e)
        return data[:n], times[:n], off.to(torch.int64) & 0xFFFFFFFF
