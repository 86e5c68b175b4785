"""Generate golden vectors from the reference's legacy event engine and its
streaming compressor, run as the plain Python they are written in.

* ``nbecorrts_q`` (``dynamix/correlator/event_y.py:104-165``) with
  ``ncorrelatepm`` (``:72-98``): the event-correlation g2 ``res``, its
  deviation ``dev`` and the two-time correlation ``trc`` of one q bin
  (``ttcf_par``), including the mirror rule (``:148-152``) and the diagonal
  fill (``:153-156``).
* ``neigercompress`` (``dynamix/io/readdata.py:441-457``), called frame by
  frame as ``readdata.py:416-419`` does: the hot-pixel threshold, the sticky
  mask, the sum frame and the per-frame trace.

Both are numba functions; ``oracle/ref_import.py`` maps ``numba.jit`` to the
identity and ``prange`` to ``range``, so the reference's own bodies run
unchanged.  ``ncorrelatepm`` splits the frames among ``nproc`` workers by
``tstep = ceil(max(times) / nproc)`` and drops an event at ``t = max(times)``
when that is a multiple of ``nproc``; the script fixes ``nproc = 8`` and
checks that no case hits that edge.  Run where the dynamix sources are
available (first argument, ``$DYNAMIX_REFERENCE_ROOT``, or a ``reference``
checkout beside this repository)::

    python tests/golden/make_eventy_golden.py
"""
from __future__ import annotations

import contextlib
import io
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.abspath(os.path.join(HERE, "..", "..")))

from dynamix_gb300.speckle import annular_qmask, speckle_numpy  # noqa: E402
from oracle.ref_import import import_module  # noqa: E402

NPROC = 8

TTCF_CASES = [
    # name, T, shape, rho, mu, n_bins, ttcf_par (1-based), dark (frames zeroed in bin 2)
    ("eventy_ttcf_small", 200, (24, 20), 0.97, 0.6, 3, 2, None),
    ("eventy_ttcf_dark", 150, (20, 20), 0.95, 0.8, 3, 2, (40, 52)),
    ("eventy_ttcf_tiles", 300, (16, 24), 0.98, 0.4, 2, 1, None),
]

HOT_CASES = [
    # name, T, shape, mu, threshold, hot fraction, masked pixels at start
    ("neiger_thr40", 120, (20, 24), 0.8, 40, 3e-3, 5),
    ("neiger_thr0", 60, (12, 16), 0.3, 0, 0.0, 0),
    ("neiger_nomask", 80, (16, 16), 1.2, 250, 1e-3, 3),
]


def events_of(frames):
    """Pixel-major, time-ascending events of a stack (the layout the event
    engine reads): values, times, per-pixel counts over all pixels."""
    T = frames.shape[0]
    fT = frames.reshape(T, -1).T
    nz = np.nonzero(fT > 0)
    return fT[nz].astype(np.int64), nz[1].astype(np.int64), (fT > 0).sum(axis=1).astype(np.int64)


def make_ttcf(ey):
    ey.nproc = NPROC
    for name, T, shape, rho, mu, nb, q, dark in TTCF_CASES:
        frames = speckle_numpy(T, shape, rho, mu, seed=T + nb)
        qmask = annular_qmask(shape, nb, 0.0, min(shape) / 2.0)
        if dark is not None:
            frames[dark[0]:dark[1], qmask == 2] = 0
        evs, tms, cnt = events_of(frames)
        assert tms.max() % NPROC != 0, "a case at the tstep edge of ncorrelatepm"
        with contextlib.redirect_stdout(io.StringIO()):
            out = ey.nbecorrts_q(evs, tms, cnt, qmask.copy(), T, calc_std=True, ttcf_par=q)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), frames=frames, qmask=qmask, ttcf_par=q,
                            nproc=NPROC, res=out.res, dev=out.dev, trc=out.trc)
        print(name, frames.shape, "q", q, "trc nan", int(np.isnan(out.trc).sum()), "mirrored",
              bool(np.all(np.isfinite(np.diag(out.trc, -5))) and np.diag(out.trc, -5).sum() > 0))


def make_hot(rd):
    for name, T, shape, mu, thr, hot_frac, n_masked in HOT_CASES:
        rng = np.random.default_rng(T + thr)
        frames = rng.poisson(mu, (T,) + shape).astype(np.uint8)
        hot = rng.random((T,) + shape) < hot_frac
        frames[hot] = 200
        ll = shape[0] * shape[1]
        mask0 = np.zeros(ll, np.uint8)
        mask0[rng.choice(ll, n_masked, replace=False)] = 1
        # the reader's buffers (readdata.py:396-401); column 0 of evs/tms is never
        # written: the first event of a pixel goes to column cnt + 1 = 1
        lp = T + 2
        evs = np.zeros((ll, lp), np.uint8)
        tms = np.zeros((ll, lp), np.uint16)
        cnt = np.zeros(ll, np.uint16)
        afr = np.zeros(ll, np.uint32)
        m = mask0.copy()
        trace = np.zeros(T, np.uint32)
        tr = 0
        for i in range(T):
            fr = frames[i].ravel().astype(np.float32)           # the dropletized frame (float32)
            evs, tms, cnt, afr, m, tr = rd.neigercompress(evs, tms, cnt, afr, m, tr, fr, thr, i, ll, lp)
            trace[i] = tr
        np.savez_compressed(os.path.join(HERE, name + ".npz"), frames=frames, threshold=thr, mask0=mask0,
                            evs=evs, tms=tms, cnt=cnt, afr=afr, mask_after=m, trace=trace)
        print(name, frames.shape, "thr", thr, "masked after", int(m.sum()), "events", int(cnt.sum()))


def main(root=None):
    if root:
        os.environ["DYNAMIX_REFERENCE_ROOT"] = root
    ey = import_module("dynamix.correlator.event_y")      # reference code
    rd = import_module("dynamix.io.readdata")             # reference code
    make_ttcf(ey)
    make_hot(rd)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else None)
