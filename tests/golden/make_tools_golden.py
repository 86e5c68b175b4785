"""Golden vectors for the host-side tools (radial average, q mask from the
geometry, crop, multi-tau rebinning, baseline correction), made by running the
reference's own ``dynamix/tools/tools.py`` in this container.

That module imports plotting and detector-file readers at the top; they are
replaced by stub modules here (only ``readdata.readnpz`` and
``EdfMethods.loadedf`` are called, by ``make_q``, and they return the arrays
below).  ``make_q`` writes its results into a temporary directory, from which
they are read back; it runs with a numpy whose ``linspace`` arrays take a
one-element array as an element value (numpy 2.5 refuses that, older releases
did not, and make_q relies on it for a value it does not use).

Usage: python tests/golden/make_tools_golden.py /path/to/the/dynamix/checkout
Writes tests/golden/tools_ref.npz.
"""
import os
import sys
import tempfile
import types
from collections import namedtuple

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _stub(name, **attrs):
    m = types.ModuleType(name)
    m.__dict__.update(attrs)
    sys.modules[name] = m
    return m


class _LenientArray(np.ndarray):
    """An array that accepts a one-element array as one element's value, as
    numpy releases before 2.5 did (make_q assigns one that way, tools.py:287,
    to an intensity it does not use further)."""

    def __setitem__(self, key, value):
        if isinstance(value, np.ndarray) and value.size == 1:
            value = value.reshape(())
        super().__setitem__(key, value)


class _NumpyProxy(types.ModuleType):
    """numpy, except that linspace returns _LenientArray."""

    def __init__(self):
        super().__init__("numpy_proxy")

    def __getattr__(self, name):
        return getattr(np, name)

    @staticmethod
    def linspace(*a, **k):
        return np.linspace(*a, **k).view(_LenientArray)


def main(ref_root):
    rng = np.random.default_rng(21)
    H, W = 70, 90
    cy, cx = 31.3, 44.6
    rows, cols = np.indices((H, W))
    r = np.sqrt((cols - cx) ** 2 + (rows - cy) ** 2)
    saxs = (2000.0 / (1.0 + (r / 9.0) ** 2) + rng.random((H, W)) * 5).astype(np.float32)
    mask = np.zeros((H, W), np.uint8)
    mask[rng.random((H, W)) < 0.02] = 1            # dead pixels
    mask[28:35, 40:49] = 1                         # beamstop
    box = {"saxs": saxs, "mask": mask}

    _stub("pylab")
    _stub("dynamix.io.readdata", readnpz=lambda f: box["saxs"].copy())
    _stub("dynamix.io.EdfMethods", loadedf=lambda f: box["mask"].copy())
    _stub("dynamix.io.h5reader")
    _stub("dynamix.correlator.WXPCS", eigerpix=None)
    sys.path.insert(0, ref_root)
    import dynamix.io as dio  # reference package
    dio.readdata = sys.modules["dynamix.io.readdata"]
    dio.EdfMethods = sys.modules["dynamix.io.EdfMethods"]
    dio.h5reader = sys.modules["dynamix.io.h5reader"]
    from dynamix.tools import tools  # reference code

    out = {"saxs": saxs, "mask": mask, "cx": cx, "cy": cy}
    prof, rq, smooth = tools.radi(saxs, mask, cx, cy)
    out.update(radi_profile=prof, radi_r=rq, radi_smooth=smooth)

    geo = {"wavelength": 1.55, "distance": 5000.0, "pix_size": 0.075, "first_q": 0.004, "width_q": 0.0015,
           "step_q": 0.002, "number_q": 6}
    with tempfile.TemporaryDirectory() as tmp:
        savdir = tmp + os.sep
        config = {
            "sample_description": {"name": "s"},
            "data_location": {"data_dir": "", "sample_dir": "", "data_prefix": "", "data_sufix": "",
                              "first_file": "0", "last_file": "0", "dark_dir": "", "first_dark": "0",
                              "last_dark": "0", "result_dir": savdir},
            "exp_setup": {"geometry": "SAXS", "dbx": str(cx), "dby": str(cy), "lagtime": "0.01",
                          "wavelength": str(geo["wavelength"]), "detector_distance": str(geo["distance"]),
                          "firstq": str(geo["first_q"]), "widthq": str(geo["width_q"]),
                          "stepq": str(geo["step_q"]), "numberq": str(geo["number_q"]), "beamstop_mask": "none"},
            "correlator": {"method": "matmul", "low_threshold": "0", "bottom_ADU": "0", "top_ADU": "0",
                           "max_number": "0", "photon_ADU": "1", "ttcf": "0"},
            "detector": {"det_name": "custom", "pixels": str(geo["pix_size"]), "mask": "mask.edf",
                         "flatfield": "none"},
        }
        real_np = tools.np
        tools.np = _NumpyProxy()
        try:
            tools.make_q(config)
        finally:
            tools.np = real_np
        out["makeq_qmask"] = np.load(savdir + "s_qmask.npy")
        out["makeq_smooth"] = np.load(savdir + "s_gaus.npy")
        out["makeq_profile"] = np.loadtxt(savdir + "s_1D.dat")
    out.update({"geo_" + k: v for k, v in geo.items()})

    d = np.zeros((1500, 3))
    d[:, 0] = np.arange(1, 1501) * 0.01
    d[:, 1] = 1 + 0.3 * np.exp(-d[:, 0] / 2.0) + rng.normal(0, 0.01, 1500)
    d[:, 2] = rng.random(1500) * 0.01
    out["cf_in"] = d
    for par in (8, 16, 32):
        out["cftomt_%d" % par] = tools.cftomt(d, par)

    CR = namedtuple("CorrelationResult", "res dev trc")
    nq, nl = 3, 700
    res = (1 + 0.2 * rng.random((nq, nl))).astype(np.float32)
    dev = (0.01 * rng.random((nq, nl))).astype(np.float32)
    trc = rng.random((50, 50)).astype(np.float32)
    qq = np.zeros((H, W), np.int32)
    qq[rq < 10] = 1
    qq[(rq >= 10) & (rq < 20)] = 2
    qq[(rq >= 20) & (rq < 30)] = 3
    qq[mask > 0] = 0
    flat = (1 + 0.1 * rng.random((H, W))).astype(np.float32)
    cdata = (smooth + 1).astype(np.float32)
    per_q, save, trc_out = tools.format_result(CR(res, dev, trc), qq, flat, cdata, 0.01, 2)
    out.update(fr_res=res, fr_dev=dev, fr_trc=trc, fr_qq=qq, fr_flat=flat, fr_cdata=cdata, fr_save=save,
               fr_trc_out=trc_out)
    for i, t in enumerate(per_q):
        out["fr_q%d" % (i + 1)] = t

    data = rng.integers(0, 5, (4, H, W)).astype(np.uint8)
    rd, rq2, rc, rf = tools.reduce_matrix(data, qq, cdata, flat)
    out.update(rm_data=data, rm_out_data=rd, rm_out_qq=rq2, rm_out_cdata=rc, rm_out_flat=rf)
    np.savez_compressed(os.path.join(HERE, "tools_ref.npz"), **out)


if __name__ == "__main__":
    sys.path.insert(0, os.path.abspath(os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "..")))
    from oracle.build_oracle import reference_root
    main(sys.argv[1] if len(sys.argv) > 1 else reference_root())
