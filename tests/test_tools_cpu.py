"""Host-side tools against golden vectors made by the reference's own
tools.py (tests/golden/make_tools_golden.py)."""
from collections import namedtuple

import numpy as np
import pytest

from conftest import golden
from dynamix_gb300 import tools


@pytest.fixture(scope="module")
def z():
    return golden("tools_ref")


def test_radial_average(z):
    prof, r, smooth = tools.radi(z["saxs"], z["mask"], float(z["cx"]), float(z["cy"]))
    assert np.array_equal(prof, z["radi_profile"])
    assert np.array_equal(r, z["radi_r"])
    assert np.array_equal(smooth, z["radi_smooth"])


def test_qmask_from_geometry(z):
    geo = {k[4:]: float(z[k]) for k in z.files if k.startswith("geo_")}
    geo["number_q"] = int(geo["number_q"])
    qmask, prof, smooth, centres, inten = tools.qmask_from_geometry(z["saxs"], z["mask"], float(z["cx"]),
                                                                    float(z["cy"]), **geo)
    assert qmask.dtype == np.uint16 and np.array_equal(qmask, z["makeq_qmask"])
    assert np.array_equal(np.float32(smooth), z["makeq_smooth"])
    assert np.array_equal(prof, z["makeq_profile"])
    assert centres.size == geo["number_q"] and np.all(np.isfinite(inten))


@pytest.mark.parametrize("par", [8, 16, 32])
def test_multi_tau_rebinning(z, par):
    got = tools.cftomt(z["cf_in"], par)
    assert got.shape == z["cftomt_%d" % par].shape
    assert np.array_equal(got, z["cftomt_%d" % par])


def test_baseline_correction_and_tables(z):
    CR = namedtuple("CorrelationResult", "res dev trc")
    per_q, save, trc = tools.format_result(CR(z["fr_res"], z["fr_dev"], z["fr_trc"]), z["fr_qq"], z["fr_flat"],
                                           z["fr_cdata"], 0.01, 2)
    assert len(per_q) == 3
    for i, t in enumerate(per_q):
        assert np.array_equal(t, z["fr_q%d" % (i + 1)])
    assert np.array_equal(save, z["fr_save"])
    assert np.array_equal(trc, z["fr_trc_out"])
    # a result without a two-time matrix (our CorrelationResult) works too
    CR2 = namedtuple("CorrelationResult", "res dev")
    per_q2, save2, trc2 = tools.format_result(CR2(z["fr_res"], z["fr_dev"]), z["fr_qq"], z["fr_flat"],
                                              z["fr_cdata"], 0.01, 0)
    assert np.array_equal(save2, z["fr_save"]) and trc2 == 0


def test_reduce_matrix(z):
    d, q, c, f = tools.reduce_matrix(z["rm_data"], z["fr_qq"], z["fr_cdata"], z["fr_flat"])
    assert np.array_equal(d, z["rm_out_data"]) and np.array_equal(q, z["rm_out_qq"])
    assert np.array_equal(c, z["rm_out_cdata"]) and np.array_equal(f, z["rm_out_flat"])
