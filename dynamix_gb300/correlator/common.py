"""Parameter contract shared by all correlators.

Mirrors ``BaseCorrelator`` (dynamix/correlator/common.py:10-80) and the
constructor arguments of ``OpenclCorrelator`` (common.py:83-197): a scalar
``shape`` means square frames; ``qmask`` is cast to int32, its bins are
``1..qmask.max()`` (``qmask=None``: one bin holding every pixel); the scale
factor of a bin is its pixel count unless given (a scalar, a sequence with
one value per bin, or a dict ``bin -> value``); ``weights`` raise
``ValueError`` as in the reference; ``extra_options`` is kept as a dict.
OpenCL-only arguments (``ctx``, ``devicetype``, ``platformid``, ``deviceid``,
``block_size``, ``memory``) are accepted and ignored; ``profile=True`` records
CUDA-event timings in ``self.timings``.

Extra options understood here:
  ``device``       CUDA device (default: the current one)
  ``method``       ``"tc"`` (tensor-core Gram, default) or ``"plain"`` (CUDA-core comparator)
  ``exact_limit``  bound on every fp32 partial sum of the Gram (default 2^24)
  ``operand``      packed element type of the Gram: ``"auto"`` (default),
                   ``"e4m3"`` (counts <= 16), ``"fp16"`` (<= 2048) or ``"bytes"``
"""
from __future__ import annotations

import numpy as np


class BaseCorrelator(object):
    "Abstract base class for all correlators"

    def __init__(self):
        self.nframes = None
        self.shape = None
        self.bins = None
        self.n_bins = None
        self.output_shape = None
        self.weights = None
        self.scale_factors = None
        self.timings = {}

    def _set_parameters(self, shape, nframes, qmask, scale_factor, extra_options):
        self.nframes = int(nframes)
        self._set_shape(shape)
        self._set_qmask(qmask=qmask)
        self._set_scale_factor(scale_factor=scale_factor)
        self._configure_extra_options(extra_options)

    def _set_shape(self, shape):
        if np.isscalar(shape):
            self.shape = (int(shape), int(shape))
        else:
            assert len(shape) == 2
            self.shape = tuple(int(s) for s in shape)

    def _set_qmask(self, qmask=None):
        self.qmask = None
        if qmask is None:
            self.bins = np.array([1], dtype=np.int32)
            self.n_bins = 1
            self.qmask = np.ones(self.shape, dtype=np.int32)
        else:
            self.qmask = np.ascontiguousarray(qmask, dtype=np.int32)
            if self.qmask.shape != tuple(self.shape):
                raise ValueError("qmask shape %s does not match frame shape %s" % (self.qmask.shape, self.shape))
            self.n_bins = int(self.qmask.max()) if self.qmask.size else 0
            self.bins = np.arange(1, self.n_bins + 1, dtype=np.int32)
        self.output_shape = (self.n_bins, self.nframes)

    def _set_weights(self, weights=None):
        if weights is None:
            self.weights = None
            return
        weights = np.asarray(weights)
        assert weights.shape == tuple(self.shape)
        raise ValueError("Advanced weighting is not implemented yet")

    def _set_scale_factor(self, scale_factor=None):
        if self.n_bins == 0:
            s = scale_factor or np.prod(self.shape)
            self.scale_factors = {1: s}
            return
        if scale_factor is not None:
            if not np.iterable(scale_factor):
                scale_factor = [scale_factor]
            assert len(scale_factor) == self.n_bins
            if isinstance(scale_factor, dict):
                self.scale_factors = dict(scale_factor)
            else:
                self.scale_factors = {k: v for k, v in zip(self.bins, scale_factor)}
        else:
            self.scale_factors = {}
            for bin_val in self.bins:
                self.scale_factors[bin_val] = np.sum(self.qmask == bin_val)

    def _configure_extra_options(self, extra_options):
        self.extra_options = {}
        if extra_options is not None:
            self.extra_options.update(extra_options)

    # helpers for the GPU engines
    def _scale_array(self):
        if self.n_bins == 0:
            return np.zeros(0, dtype=np.float64)
        return np.array([float(self.scale_factors[b]) for b in self.bins], dtype=np.float64)

    def _pixel_counts(self):
        return np.array([float(np.sum(self.qmask == b)) for b in self.bins], dtype=np.float64)
