"""Dense-frame correlators on the GB300 tensor cores.

Drop-in counterparts of dynamix/correlator/dense.py and cuda.py:

* :class:`MatMulCorrelator` (dense.py:118-142) -- ``correlate(frames)`` returns
  float32 ``(n_bins, nframes)``; like the reference it normalises by the
  pixel count of each bin (``lenmatr``, dense.py:51, :62) and ignores
  ``scale_factor``.
* :class:`DenseCorrelator` (dense.py:145-272) -- same result, normalised by
  the bin scale factors (dense.py:215-221).
* :class:`CublasMatMulCorrelator` (cuda.py:19-125) -- the reference's GPU
  MatMul correlator; here the same engine as :class:`MatMulCorrelator`.
* :func:`py_dense_correlator` (dense.py:32-70) -- one bin.

All of them compute N and D exactly in int64 on the device (tensor-core Gram
with fused lag diagonals), so the float32 result agrees with an FP64
evaluation of the reference formula to float32 rounding.
"""
from __future__ import annotations

from collections import namedtuple

import numpy as np

from ..engine import DenseEngine, frames_to_device, require_cuda
from .common import BaseCorrelator

CorrelationResult = namedtuple("CorrelationResult", "res dev")


class _DenseBase(BaseCorrelator):
    _use_pixel_counts = True

    def _init_engine(self):
        opts = self.extra_options
        scale = self._pixel_counts() if self._use_pixel_counts else self._scale_array()
        self.engine = DenseEngine(self.shape, self.nframes, self.qmask, self.n_bins, scale,
                                  device=opts.get("device"), method=opts.get("method", "tc"),
                                  exact_limit=opts.get("exact_limit", 1 << 24), grid=opts.get("grid", 0),
                                  operand=opts.get("operand", "auto"), tile=opts.get("tile"))

    def correlate_device(self, frames):
        """Run on the device and return the float32 g2 device tensor (no copy back).

        ``frames``: (nframes, H, W) counts as a numpy array, a CPU tensor or a
        CUDA tensor (uint8 / uint16 tensors are used as they are).  A pinned
        uint8 CPU tensor is copied in chunks that overlap the packing and the
        Gram; it must stay alive until the result is read."""
        eng = self.engine
        if eng.pipelined_ok(frames) and not frames.is_cuda:
            return eng.run(frames)
        frames_dev = frames_to_device(frames, eng.dev)
        out = eng.run(frames_dev)
        return out

    def correlate(self, frames, calc_std=False):
        """g2 as float32 ``(n_bins, nframes)``; with ``calc_std`` a
        ``CorrelationResult(res, dev)`` whose ``dev`` is the deviation of
        dense.py:58-66 (float32, computed in float on the tensor cores and
        reduced in float64; NaN where the reference divides by zero)."""
        out = self.correlate_device(frames)
        res = out.cpu().numpy()
        self.engine.check_error()
        self.engine.check_denominator_range()
        if calc_std:
            dev = self.engine.deviation().cpu().numpy()
            self.engine.check_error()
            return CorrelationResult(res, dev)
        return res

    def two_time(self, q):
        """Two-time correlation of q bin ``q`` (1-based, the ``ttcf_par`` of
        event_y.py:104-161) for the last :meth:`correlate` call, float32
        ``(nframes, nframes)``: P G(t,t') / (S(t) S(t')) off the diagonal,
        the mean of the positive elements of the first upper diagonal on it
        (event_y.py:148-157).  Computed on the tensor cores from the last
        call's packed frames."""
        out = self.engine.two_time(int(q) - 1).cpu().numpy()
        return out

    # exact intermediate results of the last call (int64 / float64 numpy)
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


class MatMulCorrelator(_DenseBase):

    def __init__(self, shape, nframes, qmask=None, scale_factor=None, extra_options={}):
        super().__init__()
        self._set_parameters(shape, nframes, qmask, scale_factor, extra_options)
        self._init_engine()


class CublasMatMulCorrelator(MatMulCorrelator):
    """The reference's cuBLAS MatMul correlator (cuda.py:19-125); here the
    exact tensor-core engine.  ``cublas_handle`` in ``extra_options`` is ignored."""


class DenseCorrelator(_DenseBase):
    _use_pixel_counts = False

    def __init__(self, shape, nframes, qmask=None, dtype="f", weights=None, extra_options={}, ctx=None,
                 devicetype="all", platformid=None, deviceid=None, block_size=None, memory=None, profile=False):
        super().__init__()
        self._set_parameters(shape, nframes, qmask, None, extra_options)
        self.dtype = dtype
        self._set_weights(weights)
        self.profile = profile
        self._init_engine()


def py_dense_correlator(xpcs_data, mask, calc_std=False):
    """g2 of the pixels ``mask > 0`` of a (T, H, W) stack, float64 (T,), or
    ``CorrelationResult(res, dev)`` with ``calc_std``.

    Same contract as dense.py:32-70, evaluated on the GPU."""
    mask = np.asarray(mask)
    q = (mask > 0).astype(np.int32)
    T = np.shape(xpcs_data)[0]
    corr = MatMulCorrelator(q.shape, T, qmask=q)
    corr.correlate(xpcs_data)
    if calc_std:
        corr.engine.deviation()
        return CorrelationResult(corr.g2_fp64[0], corr.engine.dev_f64[0].cpu().numpy())
    return corr.g2_fp64[0]
