"""Host-side input preparation and g2 post-processing around the correlators.

Counterparts of dynamix's ``tools/tools.py`` helpers that sit either side of
the correlation:

* before it: the radial average of a 2-D pattern (``radi``, tools.py:14-50),
  the annular q mask from the scattering geometry (the mask-building part of
  ``make_q``, tools.py:175-296, without its file reading and writing) and the
  crop of frames to the q mask's bounding box (``reduce_matrix``,
  tools.py:482-503);
* after it: the linear-to-multi-tau rebinning of a correlation function
  (``cftomt``, tools.py:147-172) and the flat-field / smooth-intensity
  baseline correction with the multi-tau output table (``format_result``,
  tools.py:313-346).

They work on 2-D images or (T, 3) tables, so they run in numpy on the host, as
in the reference; the correlation itself runs on the GPU.
"""
from __future__ import annotations

import numpy as np


def radi(saxs, mask, cx, cy):
    """Radial average of a 2-D pattern about (cx, cy) (column, row).

    Pixels are binned by their distance rounded to the nearest integer
    (unmasked pixels only; ``mask`` > 0 is masked).  Returns ``(profile, r,
    smooth)``: the (n, 2) table of radius and mean intensity, the float32
    distance of every pixel (0 where masked), and the profile interpolated
    linearly back onto the image (0 where masked)."""
    saxs = np.asarray(saxs)
    mask = np.asarray(mask)
    rows, cols = np.indices(saxs.shape)
    r = np.float32(np.sqrt((cols - cx) ** 2 + (rows - cy) ** 2))
    ring = np.int16(r + 0.5)
    r[mask > 0] = 0
    live = mask < 1
    ring_live = ring[live]
    edges = np.arange(int(ring_live.min()), int(ring_live.max()) + 1, 1)
    total, edges = np.histogram(ring_live, weights=saxs[live], bins=edges)
    count, _ = np.histogram(ring_live, bins=edges)
    profile = np.zeros((len(edges) - 1, 2))
    profile[:, 0] = edges[:-1]
    profile[:, 1] = total / count
    # linear interpolation between the ring below and the ring above
    frac = r - np.array(r, np.uint16)
    below = np.array(r, np.uint16) - int(edges[0])
    below[mask > 0] = 0
    below[below > edges[-1]] = 0
    values = np.append(profile[:, 1], profile[-2:, 1])
    smooth = r * 0
    smooth[live] = values[below[live] + 1] * frac[live] + values[below[live]] * (1 - frac[live])
    return profile, r, smooth


def q_of_radius(radius_px, wavelength, distance, pix_size):
    """Scattering vector 4 pi / lambda sin(theta / 2) of a distance on the
    detector in pixels (the conversion of make_q, tools.py:264-265)."""
    return 4 * np.pi / wavelength * np.sin(np.arctan(pix_size * radius_px / distance) / 2.0)


def qmask_from_geometry(saxs, mask, cx, cy, wavelength, distance, pix_size, first_q, width_q, step_q, number_q):
    """The q mask of make_q (tools.py:241-296) for a 2-D pattern: ``number_q``
    rings centred on ``first_q + k step_q`` with ``width_q``, numbered 1.. (a
    pixel within half a width of several centres takes the last), 0 on masked
    pixels.  ``mask`` > 0 is masked (a beamstop mask already merged in).

    Returns ``(qmask uint16, profile, smooth, q_centres, q_intensity)``:
    ``profile`` is the radial average with its first column in q,
    ``smooth`` the radially smoothed pattern (0 where masked or NaN),
    ``q_intensity`` the profile intensity nearest each centre."""
    saxs = np.array(saxs)  # a copy in the pattern's own dtype (the sums follow it)
    mask = np.asarray(mask)
    saxs[mask > 0] = 0
    profile, r_px, smooth = radi(np.ma.array(saxs, mask=mask), mask, cx, cy)
    smooth[np.isnan(smooth)] = 0
    profile[:, 0] = q_of_radius(profile[:, 0], wavelength, distance, pix_size)
    r_q = q_of_radius(r_px, wavelength, distance, pix_size)
    centres = np.linspace(first_q, first_q + (number_q - 1) * step_q, number_q)
    qmask = np.zeros(mask.shape, dtype=np.asarray(mask).dtype)
    intensity = centres * 0
    for k, c in enumerate(centres):
        dist = np.abs(profile[:, 0] - c)
        intensity[k] = profile[dist == dist.min(), 1][0]
        qmask[np.abs(r_q - c) <= width_q / 2] = k + 1
    qmask[mask > 0] = 0
    return np.array(qmask, np.uint16), profile, smooth, centres, intensity


def reduce_matrix(data, qqmask, cdata, flatfield):
    """Crop frames (T, H, W) and the 2-D maps to the bounding box of the q
    mask's non-zero pixels, as reduce_matrix does (tools.py:482-503: the box
    ends one row and one column before the last non-zero pixel)."""
    rows, cols = np.nonzero(np.asarray(qqmask) > 0)
    r0, r1, c0, c1 = rows.min(), rows.max(), cols.min(), cols.max()
    return (data[:, r0:r1, c0:c1], qqmask[r0:r1, c0:c1], cdata[r0:r1, c0:c1], flatfield[r0:r1, c0:c1])


def cftomt(d, par=16):
    """Linear lag spacing -> multi-tau spacing (tools.py:147-172).

    ``d``: (n, >= 3) rows of (lag time, g2, error).  The first ``par`` rows are
    kept; then, level by level, neighbouring rows of the rest are averaged in
    pairs, every second of the first ``par`` averages is kept, and the
    averages from index ``par`` on (every second, the last one left out) form
    the next level.  Returns an (m, 3) array."""
    d = np.asarray(d)
    kept = [d[i, :3] for i in range(par)]
    level = d[par:, :3]
    while level.shape[0] >= par:
        pairs = (level[:-1, :] + level[1:, :]) / 2
        kept.extend(pairs[i] for i in range(0, par, 2))
        level = pairs[par:-1:2, :3]
    return np.array(kept)


def format_result(result, qqmask, flatfield, cdata, dt, ttcf_par, trc=None):
    """Baseline correction and multi-tau tables of a correlation result
    (tools.py:313-346).

    ``result`` has ``res`` and ``dev`` (n_q, n_lags) and optionally ``trc``
    (or pass ``trc``).  For bin q the correction is
    mean(c^2)/mean(c)^2 * mean(f^2)/mean(f)^2 over its pixels (c the smooth
    intensity ``cdata``, f the flat field); each row of res and dev is divided
    by it, with lag times (1..n) * dt, and rebinned by :func:`cftomt`.
    Returns ``(per_q_tables, save_table, trc)``: the list of (m, 3) tables, the
    tables side by side (lag column once), and the two-time matrix as given
    (uncorrected, as the reference returns it)."""
    res = np.asarray(result.res)
    dev = np.asarray(result.dev)
    if trc is None:
        trc = getattr(result, "trc", 0)
    qqmask = np.asarray(qqmask)
    n = res[0].size
    table = np.zeros((n, 3), np.float32)
    table[:, 0] = np.arange(1, n + 1, 1) * dt
    out = []
    save = None
    for q in range(1, int(qqmask.max()) + 1):
        f = flatfield[qqmask == q]
        c = cdata[qqmask == q]
        correction = (c ** 2).mean() / c.mean() ** 2 * ((f ** 2).mean() / f.mean() ** 2)
        table[:, 1] = res[q - 1, :] / correction
        table[:, 2] = dev[q - 1, :] / correction
        mt = cftomt(table)
        out.append(mt)
        save = mt if save is None else np.append(save, mt[:, 1:], axis=1)
    return out, save, trc
