"""CPU restatement of the dynamix g2 correlator arithmetic (test infrastructure).

Every correlator of the reference computes, per q-bin ``b`` with ``P_b`` pixels
and frames ``I(t, p)``, ``t = 0..T-1``:

* numerator   ``N_b(tau) = sum_t sum_{p in b} I(t, p) * I(t + tau, p)``
* bin sums    ``S_b(t)   = sum_{p in b} I(t, p)``
* denominator ``D_b(tau) = sum_t S_b(t) * S_b(t + tau)``
* ``g2_b(tau) = scale_b * N_b(tau) / D_b(tau)``, ``scale_b`` = ``P_b`` by default.

References (paths inside the dynamix project):

* ``dynamix/correlator/dense.py:32-70``   ``py_dense_correlator`` (Gram + diagonals)
* ``dynamix/correlator/dense.py:118-142``  ``MatMulCorrelator.correlate``
* ``dynamix/correlator/common.py:36-72``   bins / scale factors from the qmask
* ``dynamix/resources/opencl/densecorrelator.cl:6-176``  direct numerator, sums, 1-D correlation
* ``dynamix/resources/opencl/evtcorrelator.cl:3-77``     event pair sums + normalisation
* ``dynamix/resources/opencl/correlator.cl:19-217``      CSR sums + single-q correlation
* ``dynamix/correlator/event.py:267-321``  ``FramesCompressor`` event layout
* ``dynamix/correlator/intensity.py:70-77`` CSR layout (``indptr`` of size (H+1)*T)

``N``, ``S`` and ``D`` are computed exactly in int64 here; ``g2`` in float64.
The reference itself keeps float32 (MatMul) or 32-bit integers (OpenCL), so it
agrees with this restatement to float32 rounding; the tests pin that.
"""
from __future__ import annotations

import os

import numpy as np

__all__ = [
    "bins_from_qmask", "gather_bin", "g2_exact", "g2_from_nsd", "denominator_exact",
    "matmul_correlator_port", "py_dense_correlator_port", "compress_all_stack",
    "event_correlate_exact", "frames_to_csr", "csr_correlate_exact", "dense_std_exact",
]


def bins_from_qmask(qmask, shape, scale_factor=None):
    """Bins and scale factors exactly as ``BaseCorrelator`` derives them.

    Follows ``dynamix/correlator/common.py:36-46`` (qmask None -> one bin of all
    pixels; otherwise bins ``1..qmask.max()``) and ``common.py:56-72`` (scale
    factor = pixel count of the bin unless given).
    Returns ``(qmask_int32, n_bins, bins, scale_factors_float64_array, npix_per_bin)``.
    """
    if np.isscalar(shape):
        shape = (int(shape), int(shape))
    shape = tuple(int(s) for s in shape)
    if qmask is None:
        qm = np.ones(shape, dtype=np.int32)
        n_bins = 1
    else:
        qm = np.ascontiguousarray(qmask, dtype=np.int32)
        n_bins = int(qm.max()) if qm.size else 0
    bins = np.arange(1, n_bins + 1, dtype=np.int32)
    npix = np.array([int(np.sum(qm == b)) for b in bins], dtype=np.int64)
    if scale_factor is None:
        sf = npix.astype(np.float64)
    else:
        if isinstance(scale_factor, dict):
            sf = np.array([float(scale_factor[b]) for b in bins], dtype=np.float64)
        else:
            if not np.iterable(scale_factor):
                scale_factor = [scale_factor]
            assert len(scale_factor) == n_bins
            sf = np.asarray(scale_factor, dtype=np.float64)
    return qm, n_bins, bins, sf, npix


def gather_bin(frames, qmask, b):
    """``frames[:, qmask == b]`` as a (T, P_b) array (``dense.py:48-49``)."""
    T = frames.shape[0]
    flat = frames.reshape(T, -1)
    idx = np.flatnonzero(qmask.ravel() == b)
    return flat[:, idx]


def _numerator_bin(x):
    """Exact ``N(tau)`` for one bin from its (T, P) counts.

    The Gram ``X X^T`` is formed in float64 (BLAS); every entry is an integer
    bounded by ``P * max^2``, which is checked to be below 2^53 so the float64
    result is exact.  Diagonal sums are then taken in int64.  This is the
    integer statement of ``dense.py:54`` and ``dense.py:61-64``.
    """
    T, P = x.shape
    if P == 0:
        return np.zeros(T, dtype=np.int64)
    mx = int(x.max()) if x.size else 0
    if P * mx * mx >= 2 ** 53:
        raise OverflowError("Gram entries may exceed 2^53; oracle cannot be exact")
    xf = x.astype(np.float64)
    G = xf @ xf.T
    Gi = G.astype(np.int64)
    out = np.empty(T, dtype=np.int64)
    flat = Gi.ravel()
    for tau in range(T):
        out[tau] = flat[tau::T + 1][:T - tau].sum()
    return out


def denominator_exact(S):
    """``D(tau) = sum_t S(t) S(t+tau)`` in int64 (``densecorrelator.cl:156-176``,
    ``evtcorrelator.cl:70-73``; the reference accumulates it in float32)."""
    S = np.asarray(S, dtype=np.int64)
    T = S.shape[-1]
    D = np.zeros_like(S)
    for tau in range(T):
        D[..., tau] = np.einsum("...t,...t->...", S[..., :T - tau], S[..., tau:])
    return D


def g2_from_nsd(N, D, scale):
    """``g2 = scale * N / D`` in float64 (``dense.py:62-64``; ``evtcorrelator.cl:75``).

    ``0/0`` (an empty or dark bin) gives NaN as in the reference."""
    N = np.asarray(N, dtype=np.float64)
    D = np.asarray(D, dtype=np.float64)
    with np.errstate(divide="ignore", invalid="ignore"):
        return np.asarray(scale, dtype=np.float64)[:, None] * N / D


def g2_exact(frames, qmask=None, scale_factor=None):
    """Exact N, S, D (int64) and g2 (float64) for a dense stack (T, H, W).

    Returns a dict with keys ``numerator``, ``sums``, ``denominator`` (all
    ``(n_bins, T)`` int64), ``g2`` (float64) and ``scale``.
    """
    frames = np.asarray(frames)
    if frames.dtype.kind == "f":
        raise TypeError("the exact oracle needs integer counts")
    T = frames.shape[0]
    qm, n_bins, bins, sf, npix = bins_from_qmask(qmask, frames.shape[1:], scale_factor)
    N = np.zeros((n_bins, T), dtype=np.int64)
    S = np.zeros((n_bins, T), dtype=np.int64)
    for i, b in enumerate(bins):
        x = gather_bin(frames, qm, b).astype(np.int64)
        if np.any(x < 0):
            raise ValueError("counts must be non-negative")
        S[i] = x.sum(axis=1)
        N[i] = _numerator_bin(x)
    D = denominator_exact(S)
    return {"numerator": N, "sums": S, "denominator": D, "g2": g2_from_nsd(N, D, sf),
            "scale": sf, "npix": npix}


def dense_std_exact(frames, qmask=None):
    """``calc_std`` deviation of ``dense.py:58-66`` in float64.

    ``dev(tau) = std_t(ratio) / sqrt(T - tau)`` with
    ``ratio(t) = (G(t, t+tau) / P) / (mean(t) * mean(t+tau))``.
    """
    frames = np.asarray(frames)
    T = frames.shape[0]
    qm, n_bins, bins, _, _ = bins_from_qmask(qmask, frames.shape[1:])
    dev = np.zeros((n_bins, T), dtype=np.float64)
    for i, b in enumerate(bins):
        x = gather_bin(frames, qm, b).astype(np.float64)
        P = x.shape[1]
        G = x @ x.T
        m = x.mean(axis=1)
        with np.errstate(divide="ignore", invalid="ignore"):
            for tau in range(T):
                dn = np.diagonal(G, tau) / P
                dd = m[:T - tau] * m[tau:]
                dev[i, tau] = np.std(dn / dd) / np.sqrt(T - tau)
    return dev


def py_dense_correlator_port(xpcs_data, mask):
    """Faithful float32 restatement of ``py_dense_correlator`` (``dense.py:32-70``).

    The counts of the bin are gathered and cast to float32, the Gram is one
    float32 GEMM (numpy BLAS, all host threads), the mean outer product another,
    and the per-lag diagonal sums are taken as in the reference loop.  This is
    the CPU baseline that is timed; it is not used as the exactness checker.
    """
    ind = np.where(mask > 0)
    x = np.array(xpcs_data[:, ind[0], ind[1]], np.float32)
    mean = np.mean(x, axis=1)
    T, P = x.shape
    mean = mean.reshape(1, T)
    num = np.dot(x, x.T)
    den = np.dot(mean.T, mean)
    res = np.zeros(T)
    for i in range(T):
        res[i] = np.sum(np.diag(num, k=i) / P) / np.sum(np.diag(den, k=i))
    return res


def matmul_correlator_port(frames, qmask=None):
    """``MatMulCorrelator.correlate`` restated (``dense.py:118-142``): float32 (n_bins, T)."""
    T = frames.shape[0]
    qm, n_bins, bins, _, _ = bins_from_qmask(qmask, frames.shape[1:])
    res = np.zeros((n_bins, T), dtype=np.float32)
    with np.errstate(divide="ignore", invalid="ignore"):
        for i, b in enumerate(bins):
            res[i] = py_dense_correlator_port(frames, qm == b)
    return res


def compress_all_stack(frames):
    """Dense stack -> (data, times, offsets) event lists (``event.py:267-284``).

    Pixel-major, time-ascending within each pixel; values <= 0 are dropped;
    ``offsets`` is uint32 of size H*W+1, ``times`` int32."""
    assert frames.ndim == 3
    fT = np.moveaxis(frames, 0, -1)
    nz = np.nonzero(fT > 0)
    data = fT[nz]
    times = nz[-1].astype(np.int32)
    counts = (frames > 0).sum(axis=0).ravel()
    offsets = np.zeros(counts.size + 1, dtype=np.uint32)
    offsets[1:] = np.cumsum(counts)
    return data, times, offsets


def compress_hot_pixels(frames, threshold=None, mask=None):
    """Frame-by-frame compression with the sticky hot-pixel mask of the
    streaming reader (``io/readdata.py:452-466``, ``neigercompress``).

    Per frame ``i`` and pixel ``p``: the raw value is added to the sum frame; a
    value above ``threshold`` sets the pixel's mask; a masked pixel's value is
    zeroed; a value still > 0 is appended to the pixel's events with time
    ``i``.  Returns ``(data, times, offsets, mask_after, sum_frame)`` in the
    layout of :func:`compress_all_stack` (the mask and the sums per pixel)."""
    assert frames.ndim == 3
    T = frames.shape[0]
    f = frames.reshape(T, -1).astype(np.int64)
    m = np.zeros(f.shape[1], dtype=bool) if mask is None else np.asarray(mask).ravel().astype(bool).copy()
    kept = np.zeros_like(f)
    for i in range(T):
        fr = f[i].copy()
        if threshold is not None:
            m |= fr > threshold
        fr[m] = 0
        kept[i] = fr
    data, times, offsets = compress_all_stack(kept.reshape(frames.shape))
    return data.astype(frames.dtype), times, offsets, m, f.sum(axis=0)


def event_correlate_exact(vol_times, vol_data, offsets, qmask, shape, nframes, scale_factor=None):
    """Event-list correlation restated from ``evtcorrelator.cl:3-77``.

    For every pixel ``p`` with events ``(t_i, v_i)``: ``S[b][t_i] += v_i`` and,
    for every pair ``i <= j`` of its events, ``N[b][|t_j - t_i|] += v_i v_j``.
    Computed exactly in int64 (the reference uses 32-bit atomics).
    Returns the same dict as :func:`g2_exact`.
    """
    qm, n_bins, bins, sf, npix = bins_from_qmask(qmask, shape, scale_factor)
    T = int(nframes)
    N = np.zeros((n_bins, T), dtype=np.int64)
    S = np.zeros((n_bins, T), dtype=np.int64)
    offsets = np.asarray(offsets, dtype=np.int64)
    times = np.asarray(vol_times, dtype=np.int64)
    data = np.asarray(vol_data, dtype=np.int64)
    qflat = qm.ravel()
    counts = np.diff(offsets)
    pix_of_event = np.repeat(np.arange(qflat.size), counts)
    b_of_event = qflat[pix_of_event] - 1
    ok = b_of_event >= 0
    np.add.at(S, (b_of_event[ok], times[ok]), data[ok])
    # pairs, vectorised per pixel-size class
    for p in np.flatnonzero((counts > 0) & (qflat > 0)):
        b = qflat[p] - 1
        o0, o1 = offsets[p], offsets[p + 1]
        tt = times[o0:o1]
        vv = data[o0:o1]
        lag = np.abs(tt[None, :] - tt[:, None])
        prod = vv[None, :] * vv[:, None]
        iu = np.triu_indices(tt.size)
        np.add.at(N[b], lag[iu], prod[iu])
    D = denominator_exact(S)
    return {"numerator": N, "sums": S, "denominator": D, "g2": g2_from_nsd(N, D, sf),
            "scale": sf, "npix": npix}


def frames_to_csr(frames, index_dtype=np.uint32):
    """Dense stack -> the per-frame CSR layout of ``SparseCorrelator``.

    ``intensity.py:70-77`` / ``correlator.cl:110-217``: ``data`` (values),
    ``indices`` (column inside the row), ``indptr`` of size (H+1)*T holding each
    frame's row pointers *relative to that frame's first element*, and
    ``offsets`` of size T+1 (first element of each frame)."""
    T, H, W = frames.shape
    data, indices, indptr, offsets = [], [], np.zeros((T, H + 1), dtype=np.int64), np.zeros(T + 1, dtype=np.int64)
    for t in range(T):
        f = frames[t]
        r, c = np.nonzero(f > 0)
        data.append(f[r, c])
        indices.append(c)
        indptr[t, 1:] = np.cumsum(np.bincount(r, minlength=H))
        offsets[t + 1] = offsets[t] + r.size
    data = np.concatenate(data) if data else np.zeros(0, frames.dtype)
    indices = np.concatenate(indices).astype(index_dtype) if indices else np.zeros(0, index_dtype)
    return data.astype(frames.dtype), indices, indptr.ravel().astype(index_dtype), offsets.astype(index_dtype)


def csr_correlate_exact(data, indices, indptr, offsets, shape, nframes, qmask=None, scale_factor=None):
    """CSR correlation restated from ``correlator.cl:19-217``, extended to q-bins.

    Row-wise products of frame ``t`` and frame ``t + tau`` summed over matching
    columns give ``N``; per-frame sums give ``S``.  With ``qmask=None`` this is
    the reference's single-q case whose normalisation is ``prod(shape)``
    (``intensity.py:108``).  Exact int64.
    """
    H, W = (shape, shape) if np.isscalar(shape) else shape
    T = int(nframes)
    dense = np.zeros((T, H, W), dtype=np.int64)
    indptr = np.asarray(indptr, dtype=np.int64).reshape(T, H + 1)
    offsets = np.asarray(offsets, dtype=np.int64)
    indices = np.asarray(indices, dtype=np.int64)
    data = np.asarray(data, dtype=np.int64)
    for t in range(T):
        o = offsets[t]
        for r in range(H):
            s, e = indptr[t, r], indptr[t, r + 1]
            dense[t, r, indices[o + s:o + e]] = data[o + s:o + e]
    return g2_exact(dense, qmask, scale_factor)


def event_pairsum_c(vol_times, vol_data, offsets, qmask, shape, nframes, n_threads=None, pixels=None):
    """N and S (int64) of the event lists with the C restatement
    (``g2_oracle.c``), over all binned pixels or the listed ``pixels``.
    Same sums as :func:`event_correlate_exact`; threads give the same result."""
    from .build_oracle import load
    qm, n_bins, bins, sf, npix = bins_from_qmask(qmask, shape)
    qf = qm.ravel()
    pix = np.flatnonzero(qf > 0) if pixels is None else np.asarray(pixels, dtype=np.int64)
    pix = pix[qf[pix] > 0].astype(np.int32)
    b = (qf[pix] - 1).astype(np.int32)
    T = int(nframes)
    data = np.ascontiguousarray(vol_data)
    if data.dtype not in (np.uint8, np.uint16):
        data = data.astype(np.uint16 if data.size and data.max() > 255 else np.uint8)
    times = np.ascontiguousarray(vol_times, dtype=np.int32)
    offs = np.ascontiguousarray(offsets, dtype=np.uint32)
    N = np.zeros((n_bins, T), np.int64)
    S = np.zeros((n_bins, T), np.int64)
    ptr = lambda a: a.ctypes.data
    rc = load().g2o_event_pairsum(ptr(times), ptr(data), data.itemsize, ptr(offs), ptr(pix), ptr(b), pix.size, T,
                                  n_bins, ptr(N), ptr(S), int(n_threads or os.cpu_count() or 1))
    if rc:
        raise ValueError("g2o_event_pairsum failed with status %d" % rc)
    return N, S


def reference_event_correlate(vol_times, vol_data, offsets, qmask, shape, nframes, scale_factors=None,
                              n_threads=1):
    """Run the reference's own ``event_correlator`` and ``normalize_correlation``
    (``evtcorrelator.cl``, compiled as C into ``oracle/_ref``) with the launch
    arguments of ``EventCorrelator.correlate`` (``event.py:162-204``).
    Returns ``{"res_int": int32, "sums": uint32, "g2": float32}`` of shape
    (n_bins, nframes), or None when the reference sources are not present."""
    from .build_oracle import load_ref
    qm, n_bins, bins, sf, npix = bins_from_qmask(qmask, shape, scale_factors)
    data = np.ascontiguousarray(vol_data)
    tag = {1: "u8", 2: "u16"}.get(data.itemsize)
    if tag is None or data.dtype.kind not in "ui":
        raise TypeError("event data must be 8- or 16-bit integers")
    lib = load_ref(tag)
    if lib is None:
        return None
    offs = np.ascontiguousarray(offsets, dtype=np.uint32)
    if offs.size > 1 and int(np.diff(offs.astype(np.int64)).max()) > lib.g2r_max_evt_count():
        raise ValueError("a pixel has more events than the compiled MAX_EVT_COUNT")
    H, W = shape
    T = int(nframes)
    times = np.ascontiguousarray(vol_times, dtype=np.int32)
    qmi = np.ascontiguousarray(qm, dtype=np.int32)
    res_int = np.zeros((n_bins, T), np.int32)
    sums = np.zeros((n_bins, T), np.uint32)
    res = np.zeros((n_bins, T), np.float32)
    sfa = np.ascontiguousarray(sf, dtype=np.float32)
    ptr = lambda a: a.ctypes.data
    # event.py:185-190 launches over shape[::-1] = (W, H) and passes shape[1] as image_height
    rc = lib.g2r_event_correlate(ptr(times), ptr(data), ptr(offs), ptr(qmi), ptr(res_int), ptr(sums), ptr(res),
                                 ptr(sfa), W, H, W, T, n_bins, int(n_threads))
    if rc:
        raise ValueError("g2r_event_correlate failed with status %d" % rc)
    return {"res_int": res_int, "sums": sums, "g2": res}


def ttcf_exact(frames, qmask, q):
    """Two-time correlation of bin ``q`` (1-based) restated from
    ``correlator/event_y.py:141-157`` (with ``ncorrelatepm``, :72-98, for the
    pair sums): cc(t, t') = sum over the bin's pixels of I(t) I(t') for
    t' > t, s(t) the bin's frame sums, trc = (cc P / T) / (s s^T / T);
    mirrored (trc + trc^T) when its diagonal k = -5 sums below 1; the diagonal
    set to the mean of the positive elements of the first upper diagonal,
    except its last element.  float64."""
    T = frames.shape[0]
    x = frames.reshape(T, -1)[:, np.asarray(qmask).ravel() == q].astype(np.float64)
    P = x.shape[1]
    cc = np.triu(x @ x.T, 1)
    s = x.sum(axis=1).reshape(T, 1)
    with np.errstate(divide="ignore", invalid="ignore"):
        norm = (s @ s.T) / T
        trc = (cc * P / T) / norm
        if np.sum(np.diag(trc, k=-5)) < 1:
            trc = trc + trc.T
        tmp = np.diag(trc, k=1)
        tmp = np.mean(tmp[tmp > 0]) if np.any(tmp > 0) else np.nan
    for j in range(T - 1):
        trc[j, j] = tmp
    return trc
