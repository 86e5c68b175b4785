"""Synthetic XPCS speckle stacks and annular q-masks.

The reference's test datasets are external downloads; these seeded generators
stand in for them with the same shapes, dtypes and count statistics:

* field: per pixel, a complex Gaussian ``E(0) ~ CN(0, 1)`` evolving as the
  AR(1) process ``E(t) = rho * E(t-1) + sqrt(1 - rho^2) * CN(0, 1)``;
* counts: ``I(t, p) = Poisson(mu * |E(t, p)|^2)``, clipped to ``max_count``;
* q-mask: equal-width annuli ``b = 1..n_bins`` between ``r_min`` and ``r_max``
  around ``center``, 0 elsewhere.

``speckle_numpy`` (host, ``numpy.random.default_rng``) is used for the small
parity cases; ``speckle_torch`` (device, ``torch.Generator``) builds the large
benchmark stacks directly in HBM.  The two do not produce identical values.
"""
from __future__ import annotations

import math

import numpy as np


def annular_qmask(shape, n_bins, r_min, r_max, center=None):
    """Equal-width annuli ``[r_min + k w, r_min + (k+1) w)``, ``w = (r_max - r_min) / n_bins``."""
    H, W = shape
    if center is None:
        center = (H / 2.0, W / 2.0)
    cy, cx = center
    yy, xx = np.mgrid[0:H, 0:W]
    r = np.sqrt((yy - cy) ** 2 + (xx - cx) ** 2)
    width = (r_max - r_min) / float(n_bins)
    q = np.floor((r - r_min) / width).astype(np.int64) + 1
    q[(r < r_min) | (r >= r_max)] = 0
    q[q > n_bins] = 0
    return q.astype(np.int32)


def speckle_numpy(nframes, shape, rho, mu, seed=0, dtype=np.uint8, max_count=None):
    """Seeded AR(1) speckle stack on the host, shape (T, H, W)."""
    rng = np.random.default_rng(seed)
    H, W = shape
    if max_count is None:
        max_count = np.iinfo(dtype).max
    s = math.sqrt(max(0.0, 1.0 - rho * rho))
    inv = 1.0 / math.sqrt(2.0)
    E = (rng.standard_normal((H, W)) + 1j * rng.standard_normal((H, W))) * inv
    out = np.empty((nframes, H, W), dtype=dtype)
    for t in range(nframes):
        if t:
            E = rho * E + s * (rng.standard_normal((H, W)) + 1j * rng.standard_normal((H, W))) * inv
        lam = mu * (E.real ** 2 + E.imag ** 2)
        out[t] = np.minimum(rng.poisson(lam), max_count).astype(dtype)
    return out


def speckle_torch(nframes, shape, rho, mu, seed=0, dtype="uint8", max_count=None, device="cuda",
                  chunk=256):
    """Seeded AR(1) speckle stack generated on the device, shape (T, H, W).

    The AR(1) recursion runs frame by frame in float32 on the device; Poisson
    draws use ``torch.poisson`` with a seeded device generator.
    """
    import torch

    tdtype = {"uint8": torch.uint8, "uint16": torch.uint16, "int16": torch.int16}[str(np.dtype(dtype))]
    if max_count is None:
        max_count = int(np.iinfo(np.dtype(dtype)).max)
    g = torch.Generator(device=device)
    g.manual_seed(int(seed))
    H, W = shape
    s = math.sqrt(max(0.0, 1.0 - rho * rho))
    inv = 1.0 / math.sqrt(2.0)
    out = torch.empty((nframes, H, W), dtype=tdtype, device=device)
    re = torch.randn((H, W), generator=g, device=device) * inv
    im = torch.randn((H, W), generator=g, device=device) * inv
    buf = torch.empty((min(chunk, nframes), H, W), dtype=torch.float32, device=device)
    t = 0
    while t < nframes:
        n = min(chunk, nframes - t)
        for k in range(n):
            if t + k:
                re.mul_(rho).add_(torch.randn((H, W), generator=g, device=device), alpha=s * inv)
                im.mul_(rho).add_(torch.randn((H, W), generator=g, device=device), alpha=s * inv)
            torch.mul(re, re, out=buf[k]).addcmul_(im, im).mul_(mu)
        cnt = torch.poisson(buf[:n], generator=g).clamp_(max=max_count)
        if tdtype == torch.uint16:
            out[t:t + n] = cnt.to(torch.int32).to(torch.uint16)
        else:
            out[t:t + n] = cnt.to(tdtype)
        t += n
    return out


def speckle_csr_torch(nframes, shape, rho, mu, seed=0, device="cuda", chunk=64, max_count=255):
    """Seeded AR(1) speckle stack generated on the device and stored directly
    as per-frame CSR (the layout of dynamix's SparseCorrelator): returns
    ``(data uint8, indices int32, indptr int32 [(H+1)*T], offsets int64 [T+1])``
    device tensors.  Frames are built ``chunk`` at a time, so a sparse stack far
    larger than device memory as dense frames (e.g. 2162 x 2068 x 20000) fits."""
    import torch

    g = torch.Generator(device=device)
    g.manual_seed(int(seed))
    H, W = shape
    s = math.sqrt(max(0.0, 1.0 - rho * rho))
    inv = 1.0 / math.sqrt(2.0)
    re = torch.randn((H, W), generator=g, device=device) * inv
    im = torch.randn((H, W), generator=g, device=device) * inv
    buf = torch.empty((min(chunk, nframes), H, W), dtype=torch.float32, device=device)
    datas, cols, indptr_rows, counts = [], [], [], []
    t = 0
    while t < nframes:
        n = min(chunk, nframes - t)
        for k in range(n):
            if t + k:
                re.mul_(rho).add_(torch.randn((H, W), generator=g, device=device), alpha=s * inv)
                im.mul_(rho).add_(torch.randn((H, W), generator=g, device=device), alpha=s * inv)
            torch.mul(re, re, out=buf[k]).addcmul_(im, im).mul_(mu)
        cnt = torch.poisson(buf[:n], generator=g).clamp_(max=max_count).to(torch.uint8)
        nz = torch.nonzero(cnt)                                    # (frame, row, col), lexicographic
        datas.append(cnt[nz[:, 0], nz[:, 1], nz[:, 2]])
        cols.append(nz[:, 2].to(torch.int32))
        rows = torch.bincount(nz[:, 0] * H + nz[:, 1], minlength=n * H).view(n, H)
        ip = torch.zeros((n, H + 1), dtype=torch.int64, device=device)
        ip[:, 1:] = torch.cumsum(rows, dim=1)
        indptr_rows.append(ip.to(torch.int32))
        counts.append(ip[:, -1])
        t += n
    data = torch.cat(datas)
    indices = torch.cat(cols)
    indptr = torch.cat(indptr_rows).reshape(-1)
    per_frame = torch.cat(counts)
    offsets = torch.zeros(nframes + 1, dtype=torch.int64, device=device)
    offsets[1:] = torch.cumsum(per_frame, dim=0)
    return data, indices, indptr, offsets
