"""Exactness of the packed operand kinds on the GPU.

The tensor-core Gram accumulates integer products in fp32 (TMEM).  Its K
split keeps every partial sum below 2^24, which fp32 represents exactly --
provided the tensor core keeps full fp32 precision while accumulating.  These
tests check that on the device for both operand kinds (fp16, e4m3): a chunk
whose dot products reach a given magnitude with odd low bits, small terms
placed both before and after the large ones along K, must still be exact.
"""
import numpy as np
import pytest

from conftest import golden
from oracle import g2_oracle as o

pytestmark = pytest.mark.gpu


def _calibration_stack(k):
    """Frames (3, 1, P) whose Gram entries are about 2^k with odd low bits."""
    n = max(1, ((1 << k) - 64) // 225)   # pixels of value 15 (product 225)
    m = 63                               # pixels of value 1 (product 1)
    P = n + m
    fr = np.zeros((3, 1, P), dtype=np.uint8)
    fr[0, 0, :n] = 15                    # big terms first, small ones last
    fr[0, 0, n:] = 1
    fr[1, 0, :m] = 1                     # small terms first, big ones last
    fr[1, 0, m:] = 15
    rng = np.random.default_rng(k)
    fr[2, 0, :] = rng.integers(0, 16, P) | 1
    return fr


@pytest.mark.parametrize("operand", ["e4m3", "fp16"])
@pytest.mark.parametrize("k", [10, 12, 14, 15, 16, 18, 20, 22, 23, 24])
def test_fp32_accumulation_exact(built_lib, cuda_device, operand, k):
    from dynamix_gb300.correlator import MatMulCorrelator
    fr = _calibration_stack(k)
    qm = np.ones(fr.shape[1:], np.int32)
    ref = o.g2_exact(fr, qm)
    # lift the planner's bound so the whole K range is one chunk
    c = MatMulCorrelator(fr.shape[1:], 3, qmask=qm,
                         extra_options={"operand": operand, "exact_limit": 1 << 25})
    c.correlate(fr)
    assert c.engine.last["n_grams"] == 1
    x = fr.reshape(3, -1).astype(np.int64)
    gram = x @ x.T
    assert (1 << (k - 1)) < gram.max() <= (1 << 24)      # the largest entry sits just below 2^k
    assert np.array_equal(c.numerator, ref["numerator"])


@pytest.mark.parametrize("name", ["dense_small_u8", "dense_128x128_u8", "dense_edge"])
def test_e4m3_golden(built_lib, cuda_device, name):
    from dynamix_gb300.correlator import MatMulCorrelator
    z = golden(name)
    fr = z["frames"]
    qm = z["qmask"] if "qmask" in z else z["qmask_gap"]
    assert fr.max() <= 16
    ref = o.g2_exact(fr, qm)
    c = MatMulCorrelator(fr.shape[1:], fr.shape[0], qmask=qm)
    g = c.correlate(fr)
    assert c.engine.last["mode"] == "e4m3"
    assert np.array_equal(c.numerator, ref["numerator"])
    assert np.array_equal(c.denominator, ref["denominator"])
    assert np.array_equal(g, ref["g2"].astype(np.float32), equal_nan=True)


def test_e4m3_falls_back_when_counts_exceed_16(built_lib, cuda_device):
    from dynamix_gb300.correlator import MatMulCorrelator
    z = golden("dense_bright_u8")
    fr, qm = z["frames"], z["qmask"]
    assert fr.max() > 16
    ref = o.g2_exact(fr, qm)
    c = MatMulCorrelator(fr.shape[1:], fr.shape[0], qmask=qm)
    for _ in range(2):
        g = c.correlate(fr)
        assert c.engine.last["mode"] == "fp16"
        assert np.array_equal(c.numerator, ref["numerator"])
        assert np.array_equal(g, ref["g2"].astype(np.float32), equal_nan=True)
    # a dim stack afterwards goes back to e4m3
    d = golden("dense_small_u8")
    c2 = MatMulCorrelator(d["frames"].shape[1:], d["frames"].shape[0], qmask=d["qmask"])
    c2.engine._u8_hint = 0
    c2.correlate(d["frames"])
    assert c2.engine.last["mode"] == "fp16"
    c2.correlate(d["frames"])
    assert c2.engine.last["mode"] == "e4m3"
    assert np.array_equal(c2.numerator, o.g2_exact(d["frames"], d["qmask"])["numerator"])


def test_forced_operand_rejects_out_of_range(built_lib, cuda_device):
    from dynamix_gb300.correlator import MatMulCorrelator
    from dynamix_gb300.engine import DeviceError
    z = golden("dense_bright_u8")
    fr, qm = z["frames"], z["qmask"]
    c = MatMulCorrelator(fr.shape[1:], fr.shape[0], qmask=qm, extra_options={"operand": "e4m3"})
    with pytest.raises(DeviceError):
        c.correlate(fr)
