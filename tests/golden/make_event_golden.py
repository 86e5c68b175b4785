"""Generate event-correlator golden vectors by running the reference's own
OpenCL kernels (``dynamix/resources/opencl/evtcorrelator.cl``) on the CPU.

The kernel file is compiled as C by ``oracle/build_oracle.py`` (``build_ref``:
gcc with ``oracle/opencl_shim.h``) and launched by ``oracle/ref_driver.c`` with
the arguments of ``EventCorrelator.correlate`` (``event.py:162-204``).  Run in
a container where the reference sources are available::

    python tests/golden/make_event_golden.py

Each fixture holds the event lists, the q-mask and the reference's outputs:
``res_int`` (int32 numerator), ``sums`` (uint32 frame sums) and ``g2``
(float32).  ``event_ref_tall_u8`` is an image taller than wide: the reference
passes ``shape[1]`` as ``image_height`` (``event.py:183``), so it drops the rows
``y >= width``; the fixture records that behaviour.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.abspath(os.path.join(HERE, "..", "..")))

from dynamix_gb300.speckle import annular_qmask, speckle_numpy  # noqa: E402
from oracle import g2_oracle as o  # noqa: E402

CASES = [
    # name, T, shape, rho, mu, dtype, max_count, n_bins, r_min, r_max, seed
    ("event_ref_u8", 300, (36, 52), 0.98, 0.8, np.uint8, 255, 6, 2.0, 25.0, 21),
    ("event_ref_u16", 200, (30, 30), 0.99, 40.0, np.uint16, 4095, 4, 0.0, 15.0, 22),
    ("event_ref_tall_u8", 100, (40, 24), 0.98, 0.8, np.uint8, 255, 3, 0.0, 20.0, 23),
]


def main():
    for name, T, shape, rho, mu, dtype, mx, nb, r0, r1, seed in CASES:
        fr = speckle_numpy(T, shape, rho, mu, seed=seed, dtype=dtype, max_count=mx)
        qm = annular_qmask(shape, nb, r0, r1)
        d, t, off = o.compress_all_stack(fr)
        r = o.reference_event_correlate(t, d, off, qm, shape, T)
        if r is None:
            raise SystemExit("reference sources not found")
        # the reference accumulates N in int32: refuse a fixture that wrapped
        visible = qm.copy()
        visible[shape[1]:] = 0
        exact = o.g2_exact(fr, visible)
        assert np.array_equal(r["res_int"].astype(np.int64), exact["numerator"]), name
        np.savez_compressed(os.path.join(HERE, name + ".npz"), frames=fr, qmask=qm, ev_data=d, ev_times=t,
                            ev_offsets=off, res_int=r["res_int"], sums=r["sums"], g2=r["g2"])
        print(name, "events", d.size, "bins", nb)


if __name__ == "__main__":
    main()
