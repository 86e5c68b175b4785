"""Sparse (per-frame CSR) correlator.

Drop-in counterpart of dynamix/correlator/intensity.py:9-129
(``SparseCorrelator``): ``correlate(data, indices, indptr, offsets)`` with the
CSR layout of intensity.py:70-77 -- ``indptr`` of size (H+1)*nframes holding
each frame's row pointers relative to its first element, ``offsets`` of size
nframes+1.  With ``qmask=None`` (the reference's ``bins=0``) the correlation is
over all pixels and a 1-D ``(nframes,)`` float32 array is returned, normalised
by the pixel count (intensity.py:108); with a ``qmask`` the result is
``(n_bins, nframes)`` like the other correlators.  On the GPU the CSR stack is
transposed to per-pixel event lists and correlated with the exact integer
pair sums of the event correlator.
"""
from __future__ import annotations

import numpy as np

from ..engine_sparse import SparseEngine
from .common import BaseCorrelator


class SparseCorrelator(BaseCorrelator):

    def __init__(self, shape, nframes, dtype="f", bins=0, weights=None, extra_options={}, ctx=None,
                 devicetype="all", platformid=None, deviceid=None, block_size=None, memory=None, profile=False,
                 qmask=None, scale_factor=None):
        super().__init__()
        if qmask is None and bins not in (0, None):
            raise ValueError("bins > 0 needs a qmask")
        self._single_q = qmask is None
        self._set_parameters(shape, nframes, qmask, scale_factor, extra_options)
        self.dtype = dtype
        self._set_weights(weights)
        self.profile = profile
        self.engine = SparseEngine(self.shape, self.nframes, self.qmask, self.n_bins, self._scale_array(),
                                   device=self.extra_options.get("device"))

    def correlate_device(self, data, indices, indptr, offsets):
        """Run on the device and return the float32 g2 device tensor
        ``(n_bins, nframes)`` (no copy back).  Inputs may be numpy arrays or
        tensors; CUDA tensors are used in place."""
        return self.engine.run(data, indices, indptr, offsets)

    def correlate(self, data, indices, indptr, offsets, output=None):
        out = self.engine.run(data, indices, indptr, offsets)
        res = out.cpu().numpy()
        self.engine.check_error()
        if self._single_q:
            res = res.ravel()
        if output is not None:
            output[...] = res
            return output
        return res

    @property
    def numerator(self):
        return self.engine.events.numer[: self.n_bins].cpu().numpy()

    @property
    def denominator(self):
        return self.engine.events.denom[: self.n_bins].cpu().numpy()

    @property
    def sums(self):
        return self.engine.events.sums[: self.n_bins].cpu().numpy()

    @property
    def g2_fp64(self):
        return self.engine.events.g2_f64[: self.n_bins].cpu().numpy()
