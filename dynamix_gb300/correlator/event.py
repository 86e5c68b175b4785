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

    def __init__(self, shape, nframes, max_nnz, dtype=np.int8):
        self.shape = shape
        self.nframes = nframes
        self.dtype = dtype
        self.max_nnz = max_nnz
        self.npix = int(np.prod(self.shape))
        self._init_events_datastructure()

    def _init_events_datastructure(self):
        self.events_counter = np.zeros(self.npix, dtype=np.int32)
        self.events = np.zeros((self.npix, self.max_nnz), dtype=self.dtype)
        self.times = np.zeros((self.npix, self.max_nnz), dtype=np.int32)
        self.frames_counter = 0

    @staticmethod
    def compress_all_stack(frames):
        """Event structure of a whole (T, H, W) stack: (data, times, offsets)."""
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
        """Append one frame's non-zero counts to the per-pixel lists."""
        f = np.asarray(frame).ravel()
        mask = f > 0
        idx = np.flatnonzero(mask)
        if idx.size and np.any(self.events_counter[idx] >= self.max_nnz):
            raise ValueError("a pixel has more than max_nnz=%d events" % self.max_nnz)
        self.events[idx, self.events_counter[idx]] = f[idx]
        self.times[idx, self.events_counter[idx]] = self.frames_counter
        self.events_counter[idx] += 1
        self.frames_counter += 1

    def get_compacted_events(self, wait_for_all_frames=True):
        """(events, times, offsets) of the frames processed so far."""
        if self.frames_counter < self.nframes - 1 and wait_for_all_frames:
            raise RuntimeError("Not all frames were compressed yet (%d/%d)" % (self.frames_counter, self.nframes))
        offsets = np.zeros(self.events_counter.size + 1, dtype=np.uint32)
        offsets[1:] = np.cumsum(self.events_counter)
        keep = np.arange(self.max_nnz)[None, :] < self.events_counter[:, None]
        return self.events[keep], self.times[keep], offsets
