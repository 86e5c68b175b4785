"""Autotuner of the dense step's launch shapes.

The tensor-core Gram's tile order and the chunked copy/pack/Gram pipeline have
free parameters that change speed but never results:

* ``super_rows`` -- side, in frames, of the square super-tiles the 128 x 256
  tiles are grouped in (concurrent CTAs share those frames in L2);
* ``pipe_chunks`` -- number of frame chunks the step is split into (more
  chunks overlap more of the copy and the packing with the Gram, fewer keep
  each grouped launch long);
* ``kslab`` -- cap on the K columns of one tile item (0: none); narrower
  slabs keep the rows the concurrent tiles read inside L2 at the price of
  more epilogues;
* ``tile`` -- the tensor-core block: ``"pair"`` (256 x 256 on CTA pairs,
  tcgen05 cta_group::2), ``"wide"`` (256 x 512 on CTA pairs, single-buffered
  accumulator: long K) or ``"single"`` (128 x 256 on one CTA);
* ``operand`` -- the packed operand kind tried first: ``"e4m3"`` (kind::f8f6f4,
  counts <= 16), ``"fp16"`` (kind::f16, counts <= 2048) or ``"bytes"``
  (kind::f16 on byte planes); a stack whose counts do not fit falls back to a
  wider kind, so a narrow choice only wins when the counts allow it.

:func:`tune_dense` times every candidate on the caller's own stack and keeps
the fastest for the key ``(nframes, pixels per bin)``; engines built later for
the same key pick it up (:func:`apply_cached`).  Choices are kept in memory
and, when ``path`` is given (or ``DYNAMIX_G2_TUNE_CACHE`` is set), in a JSON
file.  A candidate is ``(super_rows, pipe_chunks[, kslab[, tile[,
operand]]])``; missing trailing entries take the engine's current values.
"""
from __future__ import annotations

import json
import os
import threading

import numpy as np

DEFAULT_CANDIDATES = [(2048, pc, 0, tile, op) for tile in ("pair", "wide", "single") for pc in (6, 8, 12)
                      for op in ("e4m3", "fp16")]
FIELDS = ("super_rows", "pipe_chunks", "kslab", "tile", "operand")

_lock = threading.Lock()
_cache = {}
_loaded_from = set()


def key_of(T, qmask, n_bins):
    q = np.asarray(qmask).ravel()
    npix = np.bincount(q[q > 0], minlength=int(n_bins) + 1)[1:]
    return "T=%d;P=%s" % (int(T), ",".join(str(int(p)) for p in npix))


def _cache_path(path=None):
    return path or os.environ.get("DYNAMIX_G2_TUNE_CACHE")


def _load(path):
    if not path or path in _loaded_from or not os.path.exists(path):
        return
    with open(path) as f:
        data = json.load(f)
    _cache.update({k: tuple(v) for k, v in data.items()})
    _loaded_from.add(path)


def lookup(key, path=None):
    with _lock:
        _load(_cache_path(path))
        return _cache.get(key)


def store(key, value, path=None):
    with _lock:
        _cache[key] = tuple(value)
        p = _cache_path(path)
        if p:
            data = {}
            if os.path.exists(p):
                with open(p) as f:
                    data = json.load(f)
            data[key] = list(value)
            tmp = p + ".%d.tmp" % os.getpid()
            with open(tmp, "w") as f:
                json.dump(data, f, indent=1, sort_keys=True)
            os.replace(tmp, p)


def current(engine):
    """The engine's values of :data:`FIELDS`."""
    return (int(engine.super_rows), int(engine.pipe_chunks), int(getattr(engine, "kslab", 0)),
            getattr(engine, "tile", "single"), getattr(engine, "operand_hint", "auto"))


def complete(cand, engine):
    """A candidate with its missing trailing entries taken from the engine."""
    cand = tuple(cand)
    return cand + current(engine)[len(cand):]


def set_choice(engine, v):
    engine.super_rows, engine.pipe_chunks = int(v[0]), int(v[1])
    engine.kslab = int(v[2]) if len(v) > 2 else 0
    if len(v) > 3 and v[3] in ("pair", "wide", "single"):
        engine.tile = v[3]
    if len(v) > 4 and hasattr(engine, "set_operand_hint"):
        engine.set_operand_hint(v[4])


def apply_cached(engine, path=None):
    """Set an engine's launch shapes from an earlier tuning of its key."""
    with _lock:
        _load(_cache_path(path))
        if not _cache:
            return None                  # nothing tuned in this process: skip the key
    v = lookup(key_of(engine.T, engine.qmask, engine.n_bins), path)
    if v is not None:
        set_choice(engine, v)
    return v


def tune_dense(correlator, frames, candidates=None, repeats=3, path=None):
    """Time ``correlate_device(frames)`` for every candidate (CUDA events,
    after one warm-up call each), keep the fastest for this stack's key and
    return ``(best, {candidate: ms})`` with complete 5-entry candidates.
    ``frames`` must stay the same stack for all candidates."""
    import torch
    eng = correlator.engine
    start = current(eng)
    times = {}
    for cand in (candidates or DEFAULT_CANDIDATES):
        cand = tuple(cand) + start[len(cand):]     # missing entries: the engine's values at the start
        set_choice(eng, start)
        set_choice(eng, cand)
        correlator.correlate_device(frames)
        stream = torch.cuda.current_stream(eng.dev)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(repeats):
            correlator.correlate_device(frames)
        e1.record(stream)
        e1.synchronize()
        times[cand] = e0.elapsed_time(e1) / repeats
    eng.check_error()
    best = min(times, key=times.get)
    set_choice(eng, start)
    set_choice(eng, best)
    store(key_of(eng.T, eng.qmask, eng.n_bins), best, path)
    return best, times
