"""Autotuner bookkeeping (no GPU)."""
import json
import types

import numpy as np

from dynamix_gb300 import tune


def test_key_and_persistent_cache(tmp_path):
    qm = np.zeros((4, 5), np.int32)
    qm[0] = 1
    qm[1:3, :2] = 2
    k = tune.key_of(100, qm, 3)
    assert k == "T=100;P=5,4,0"
    path = str(tmp_path / "tune.json")
    tune.store(k, (4096, 12, 8192), path)
    assert json.load(open(path))[k] == [4096, 12, 8192]
    tune._cache.clear()
    tune._loaded_from.clear()
    assert tune.lookup(k, path) == (4096, 12, 8192)
    eng = types.SimpleNamespace(T=100, qmask=qm, n_bins=3, super_rows=2048, pipe_chunks=8, kslab=0)
    assert tune.apply_cached(eng, path) == (4096, 12, 8192)
    assert (eng.super_rows, eng.pipe_chunks, eng.kslab) == (4096, 12, 8192)
    other = types.SimpleNamespace(T=101, qmask=qm, n_bins=3, super_rows=2048, pipe_chunks=8)
    assert tune.apply_cached(other, path) is None and other.super_rows == 2048
