"""Event-list correlator and the frame compressor that builds its input.

Drop-in counterparts of dynamix/correlator/event.py:

* :class:`EventCorrelator` (event.py:7-204): ``correlate(vol_times, vol_data,
  offsets)`` returns float32 ``(n_bins, nframes)``, g2 = scale * N / D with the
  scale factors of the base class (evtcorrelator.cl:58-77).  N and S are integer
  pair sums computed exactly on the GPU (G6); unlike the OpenCL kernel there is
  no per-pixel event limit and no 32-bit overflow.
* :class:`FramesCompressor` (event.py:207-321): the event layout -- per pixel
  (raster order) its non-zero counts and their frame indices, with uint32
  offsets of size H*W+1.
"""
from __future__ import annotations

import numpy as np

from ..engine_sparse import EventEngine
from .common import BaseCorrelator


class EventCorrelator(BaseCorrelator):

    def __init__(self, shape, nframes, max_events_count, total_events_count=None, allow_reallocate=True,
                 qmask=None, dtype="f", weights=None, scale_factor=None, extra_options={}, ctx=None,
                 devicetype="all", platformid=None, deviceid=None, block_size=None, memory=None, profile=False):
        super().__init__()
        self._set_parameters(shape, nframes, qmask, scale_factor, extra_options)
        self.dtype = dtype
        self._set_weights(weights)
        self.profile = profile
        self._set_events_size(max_events_count, total_events_count)
        self.allow_reallocate = allow_reallocate
        self.engine = EventEngine(self.shape, self.nframes, self.qmask, self.n_bins, self._scale_array(),
                                  device=self.extra_options.get("device"))

    def _set_events_size(self, max_events_count, total_events_count):
        self.max_events_count = max_events_count
        self.total_events_count = total_events_count or max_events_count * int(np.prod(self.shape))

    def _check_event_arrays(self, vol_times, vol_data, offsets):
        # event.py:104-115; len() also serves device tensors
        for arr in (vol_times, vol_data, offsets):
            assert np.ndim(arr) == 1
        assert len(vol_times) == len(vol_data)
        assert len(offsets) == int(np.prod(self.shape)) + 1
        numels = len(vol_data)
        if numels > self.total_events_count:
            if self.allow_reallocate:
                self.total_events_count = numels
            else:
                raise ValueError("Too many events and allow_reallocate was set to False")

    def correlate_device(self, vol_times, vol_data, offsets):
        """Run on the device and return the float32 g2 device tensor
        ``(n_bins, nframes)`` (no copy back).  CUDA tensors are used in place."""
        self._check_event_arrays(vol_times, vol_data, offsets)
        return self.engine.run(vol_times, vol_data, offsets)

    def correlate(self, vol_times, vol_data, offsets):
        self._check_event_arrays(vol_times, vol_data, offsets)
        out = self.engine.run(vol_times, vol_data, offsets)
        res = out.cpu().numpy()
        self.engine.check_error()
        return res

    @property
    def numerator(self):
        return self.engine.numer[: self.n_bins].cpu().numpy()

    @property
    def denominator(self):
        return self.engine.denom[: self.n_bins].cpu().numpy()

    @property
    def sums(self):
        return self.engine.sums[: self.n_bins].cpu().numpy()

    @property
    def g2_fp64(self):
        return self.engine.g2_f64[: self.n_bins].cpu().numpy()


class FramesCompressor(object):
    """Builds the event layout of :class:`EventCorrelator` from frames.

    For every pixel (raster order) the non-zero counts along time and their
    frame indices are compacted; ``offsets[k]:offsets[k+1]`` indexes pixel k.
    Same layout and dtypes as the reference (data in the frames' dtype, times
    int32, offsets uint32 of size H*W+1).
    """

    def __init__(self, shape, nframes, max_nnz, dtype=np.int8, device=None, threshold=None):
        self.shape = shape
        self.nframes = nframes
        self.dtype = dtype
        self.max_nnz = max_nnz
        self.npix = int(np.prod(self.shape))
        self.threshold = threshold
        self._device = None
        if device is not None:
            # the event rows live on the GPU; frames go through g2_stream_compress
            from ..compress import StreamCompressor
            self._device = StreamCompressor(shape, nframes, max_nnz, dtype, threshold=threshold, device=device)
            self.frames_counter = 0
            return
        self._init_events_datastructure()

    def _init_events_datastructure(self):
        self.events_counter = np.zeros(self.npix, dtype=np.int32)
        self.events = np.zeros((self.npix, self.max_nnz), dtype=self.dtype)
        self.times = np.zeros((self.npix, self.max_nnz), dtype=np.int32)
        self.mask = np.zeros(self.npix, dtype=bool)
        self.frames_counter = 0

    @staticmethod
    def compress_all_stack(frames, device=None, threshold=None, mask=None, sum_frame=None):
        """Event structure of a whole (T, H, W) stack: (data, times, offsets).

        A CUDA tensor, or any stack with ``device`` given, is compressed on
        the GPU (``dynamix_gb300.compress``; CUDA outputs for a CUDA input);
        ``threshold``, ``mask`` and ``sum_frame`` (device tensors) select the
        sticky hot-pixel mask and the sum frame there.  A numpy stack without
        ``device`` is compressed on the host as the reference does."""
        from ..engine import _torch
        torch = _torch()
        if device is not None or (isinstance(frames, torch.Tensor) and frames.is_cuda) \
                or threshold is not None or mask is not None or sum_frame is not None:
            from ..compress import compress_all_stack_device
            return compress_all_stack_device(frames, device=device, threshold=threshold, mask=mask,
                                             sum_frame=sum_frame)
        frames = np.asarray(frames)
        assert frames.ndim == 3
        ft = np.moveaxis(frames, 0, -1)
        nz = np.nonzero(ft > 0)
        data = ft[nz]
        times = nz[-1].astype(np.int32)
        counts = (frames > 0).sum(axis=0).ravel()
        offsets = np.zeros(counts.size + 1, dtype=np.uint32)
        offsets[1:] = np.cumsum(counts)
        return data, times, offsets

    def process_frame(self, frame):
        """Append one frame's non-zero counts to the per-pixel lists (on the
        GPU when the compressor was built with a device)."""
        if self._device is not None:
            self._device.process_frames(frame)
            self.frames_counter = self._device.frames_counter
            return
        f = np.asarray(frame).ravel()
        if self.threshold is not None:
            # sticky hot-pixel mask (io/readdata.py:452-458)
            self.mask |= f > self.threshold
            f = np.where(self.mask, 0, f)
        mask = f > 0
        idx = np.flatnonzero(mask)
        if idx.size and np.any(self.events_counter[idx] >= self.max_nnz):
            raise ValueError("a pixel has more than max_nnz=%d events" % self.max_nnz)
        self.events[idx, self.events_counter[idx]] = f[idx]
        self.times[idx, self.events_counter[idx]] = self.frames_counter
        self.events_counter[idx] += 1
        self.frames_counter += 1

    def process_frames(self, frames):
        """Append a batch of frames (B, H, W) -- one launch on the GPU."""
        if self._device is not None:
            self._device.process_frames(frames)
            self.frames_counter = self._device.frames_counter
            return
        for f in frames:
            self.process_frame(f)

    def get_compacted_events(self, wait_for_all_frames=True):
        """(events, times, offsets) of the frames processed so far (device
        tensors, offsets int64, when the compressor runs on the GPU)."""
        if self.frames_counter < self.nframes - 1 and wait_for_all_frames:
            raise RuntimeError("Not all frames were compressed yet (%d/%d)" % (self.frames_counter, self.nframes))
        if self._device is not None:
            return self._device.get_compacted_events()
        offsets = np.zeros(self.events_counter.size + 1, dtype=np.uint32)
        offsets[1:] = np.cumsum(self.events_counter)
        keep = np.arange(self.max_nnz)[None, :] < self.events_counter[:, None]
        return self.events[keep], self.times[keep], offsets
