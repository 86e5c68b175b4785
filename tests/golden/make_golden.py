"""Generate golden vectors by running the reference dynamix code itself.

Run in a container where the dynamix sources are available (read-only is
fine); pass their location as the first argument::

    python tests/golden/make_golden.py /path/to/dynamix-checkout

The reference's ``MatMulCorrelator`` (``dynamix/correlator/dense.py:118-142``)
and ``FramesCompressor.compress_all_stack`` (``dynamix/correlator/event.py:267-284``)
are pure numpy, but their modules import pyopencl/silx at the top
(``dynamix/correlator/common.py:1-7``, ``dense.py:4-10``, ``event.py:3``).
Those imports are satisfied with inert stub modules; no stubbed object is ever
called on the path exercised here.  The outputs are saved as small ``.npz``
fixtures next to this script together with the inputs that produced them.
"""
from __future__ import annotations

import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.abspath(os.path.join(HERE, "..", "..")))

from dynamix_gb300.speckle import annular_qmask, speckle_numpy  # noqa: E402


def _install_stubs():
    def mod(name, **attrs):
        m = types.ModuleType(name)
        for k, v in attrs.items():
            setattr(m, k, v)
        sys.modules[name] = m
        return m

    class _Any:  # placeholder for classes that are only referenced, never used
        def __init__(self, *a, **k):
            raise RuntimeError("stub object used")

    mod("pyopencl", array=None)
    mod("pyopencl.array", Array=_Any, zeros=None, to_device=None)
    sys.modules["pyopencl"].array = sys.modules["pyopencl.array"]
    mod("pyopencl.tools", dtype_to_ctype=lambda d: "float")
    mod("silx")
    mod("silx.opencl")
    mod("silx.opencl.common", pyopencl=sys.modules["pyopencl"], ocl=None)
    mod("silx.opencl.processing", OpenclProcessing=_Any, KernelContainer=_Any)
    mod("silx.math")
    mod("silx.math.fft")
    mod("silx.math.fft.fftw", FFTW=_Any)


CASES = [
    # name, T, shape, rho, mu, dtype, n_bins, r_min, r_max, seed
    ("dense_small_u8", 200, (48, 40), 0.98, 0.5, np.uint8, 5, 2.0, 22.0, 11),
    ("dense_bright_u8", 120, (32, 32), 0.95, 20.0, np.uint8, 3, 0.0, 16.0, 12),
    ("dense_128x128_u8", 1000, (128, 128), 0.98, 0.05, np.uint8, 8, 0.0, 64.0, 0),
    ("dense_u16", 150, (40, 36), 0.99, 60.0, np.uint16, 4, 1.0, 20.0, 13),
]


def main(ref_root):
    _install_stubs()
    sys.path.insert(0, ref_root)
    from dynamix.correlator.dense import MatMulCorrelator  # reference code
    from dynamix.correlator.event import FramesCompressor  # reference code

    for name, T, shape, rho, mu, dt, nb, r0, r1, seed in CASES:
        frames = speckle_numpy(T, shape, rho, mu, seed=seed, dtype=dt,
                               max_count=4095 if dt == np.uint16 else None)
        center = (shape[0] / 2.0, shape[1] / 2.0)
        qmask = annular_qmask(shape, nb, r0, r1, center)
        corr = MatMulCorrelator(shape, T, qmask=qmask)
        g2 = corr.correlate(frames)
        res_std = corr.correlate(frames, calc_std=True)
        data, times, offsets = FramesCompressor.compress_all_stack(frames)
        np.savez_compressed(
            os.path.join(HERE, name + ".npz"), frames=frames, qmask=qmask, g2_ref=g2,
            g2_ref_std=res_std.dev, ev_data=data, ev_times=times, ev_offsets=offsets,
            meta=np.array([T, shape[0], shape[1], nb, seed]))
        print(name, frames.shape, frames.dtype, "max", frames.max(), "g2[0,:3]", g2[0, :3])

    # qmask=None (single bin of all pixels) and an empty middle bin
    frames = speckle_numpy(64, (24, 20), 0.9, 1.0, seed=14)
    g_all = MatMulCorrelator((24, 20), 64).correlate(frames)
    qm = np.zeros((24, 20), np.int32)
    qm[2:10, 3:9] = 1
    qm[12:20, 5:15] = 3  # bin 2 is empty -> NaN row in the reference
    with np.errstate(all="ignore"):
        g_gap = MatMulCorrelator((24, 20), 64, qmask=qm).correlate(frames)
    np.savez_compressed(os.path.join(HERE, "dense_edge.npz"), frames=frames, qmask_gap=qm,
                        g2_all=g_all, g2_gap=g_gap)
    print("edge", g_all.shape, g_gap.shape, np.isnan(g_gap[1]).all())


if __name__ == "__main__":
    from oracle.build_oracle import reference_root
    main(sys.argv[1] if len(sys.argv) > 1 else reference_root())
