"""GPU parity of the dense correlators against the CPU oracle.

N, S and D must match the oracle bit for bit (int64); g2 (float64) within
1e-12 relative of the oracle's FP64 value -- tighter than the 1e-6 bound the
tensor-core path promises -- and the float32 result within 2e-6 relative of
the reference's own MatMulCorrelator output (golden vectors).
"""
import numpy as np
import pytest

from conftest import golden
from oracle import g2_oracle as o

pytestmark = pytest.mark.gpu

G2_RTOL_FP64 = 1e-12   # exact N and D, one float64 division
G2_RTOL_REF = 2e-6     # reference float32 sums vs exact


def run(frames, qmask, method="tc", cls="MatMulCorrelator", shape=None, **opts):
    from dynamix_gb300 import correlator
    T = frames.shape[0]
    shape = shape or frames.shape[1:]
    c = getattr(correlator, cls)(shape, T, qmask=qmask, extra_options=dict(method=method, **opts))
    g = c.correlate(frames)
    return c, g


def assert_exact(c, ref, g32=None):
    assert np.array_equal(c.sums, ref["sums"])
    assert np.array_equal(c.numerator, ref["numerator"])
    assert np.array_equal(c.denominator, ref["denominator"])
    g = c.g2_fp64
    both_nan = np.isnan(g) & np.isnan(ref["g2"])
    assert np.array_equal(np.isnan(g), np.isnan(ref["g2"]))
    ok = ~both_nan
    if ok.any():
        assert np.all(np.abs(g[ok] - ref["g2"][ok]) <= G2_RTOL_FP64 * np.abs(ref["g2"][ok]))
    if g32 is not None:
        assert g32.dtype == np.float32
        assert np.array_equal(g32, ref["g2"].astype(np.float32), equal_nan=True)


@pytest.mark.parametrize("method", ["tc", "plain"])
@pytest.mark.parametrize("name", ["dense_small_u8", "dense_bright_u8", "dense_128x128_u8", "dense_u16"])
def test_golden_cases(built_lib, cuda_device, name, method):
    z = golden(name)
    ref = o.g2_exact(z["frames"], z["qmask"])
    c, g = run(z["frames"], z["qmask"], method)
    assert_exact(c, ref, g)
    rg = z["g2_ref"]
    ok = np.isfinite(rg)
    assert np.all(np.abs(g[ok] - rg[ok]) <= G2_RTOL_REF * np.abs(rg[ok]))


@pytest.mark.parametrize("method", ["tc", "plain"])
def test_qmask_none_and_empty_bin(built_lib, cuda_device, method):
    z = golden("dense_edge")
    fr = z["frames"]
    c, g = run(fr, None, method)
    assert g.shape == (1, fr.shape[0])
    assert_exact(c, o.g2_exact(fr, None), g)
    c, g = run(fr, z["qmask_gap"], method)
    assert np.all(np.isnan(g[1]))
    assert_exact(c, o.g2_exact(fr, z["qmask_gap"]), g)
    assert np.allclose(g, z["g2_gap"], rtol=G2_RTOL_REF, equal_nan=True)


@pytest.mark.parametrize("T", [1, 2, 127, 128, 129, 255, 256, 257, 383])
def test_ragged_frame_counts(built_lib, cuda_device, T):
    from dynamix_gb300.speckle import annular_qmask, speckle_numpy
    fr = speckle_numpy(T, (20, 26), 0.95, 1.5, seed=T)
    qm = annular_qmask((20, 26), 3, 1.0, 12.0)
    ref = o.g2_exact(fr, qm)
    for method in ("tc", "plain"):
        c, g = run(fr, qm, method)
        assert_exact(c, ref, g)


def test_single_pixel_bins_and_dark_frames(built_lib, cuda_device):
    T, shape = 150, (9, 11)
    rng = np.random.default_rng(7)
    fr = rng.poisson(0.7, size=(T,) + shape).astype(np.uint8)
    fr[40:60] = 0                                 # dark frames
    qm = np.zeros(shape, np.int32)
    qm[0, 0] = 1                                  # one-pixel bin
    qm[4, 3] = 2
    qm[5:9, 5:11] = 3
    qm[8, 0] = 5                                  # bin 4 empty
    ref = o.g2_exact(fr, qm)
    for method in ("tc", "plain"):
        c, g = run(fr, qm, method)
        assert_exact(c, ref, g)


def test_saturated_u8_forces_k_split(built_lib, cuda_device):
    # every count 255: each 64-pixel segment carries 64*255^2 of the 2^24 budget
    T, shape = 300, (40, 60)
    rng = np.random.default_rng(1)
    fr = np.where(rng.random((T,) + shape) < 0.9, 255, rng.integers(0, 255, (T,) + shape)).astype(np.uint8)
    qm = np.ones(shape, np.int32)
    qm[:, :7] = 2
    ref = o.g2_exact(fr, qm)
    for method in ("tc", "plain"):
        c, g = run(fr, qm, method)
        assert c.engine.last["n_grams"] > 2
        assert_exact(c, ref, g)


def test_exact_limit_adversarial(built_lib, cuda_device):
    """Sums close to 2^24 in fp32 accumulation stay exact.

    With 255-valued counts on 258 pixels a frame's self product is
    258 * 65025 = 16,776,450 (2^24 - 766); odd counts make every partial sum
    odd-valued at some point, so a truncating accumulator would show."""
    T, shape = 64, (1, 258)
    rng = np.random.default_rng(2)
    fr = np.full((T,) + shape, 255, dtype=np.uint8)
    fr[::3, 0, ::7] = rng.integers(1, 255, fr[::3, 0, ::7].shape, dtype=np.uint8) | 1
    qm = np.ones(shape, np.int32)
    ref = o.g2_exact(fr, qm)
    c, g = run(fr, qm, "tc")
    assert_exact(c, ref, g)


@pytest.mark.parametrize("method", ["tc", "plain"])
def test_u16_byte_split(built_lib, cuda_device, method):
    from dynamix_gb300.speckle import annular_qmask, speckle_numpy
    T, shape = 200, (24, 30)
    fr = speckle_numpy(T, shape, 0.99, 900.0, seed=9, dtype=np.uint16, max_count=65535)
    assert fr.max() > 2048
    qm = annular_qmask(shape, 3, 0.0, 15.0)
    ref = o.g2_exact(fr, qm)
    c, g = run(fr, qm, method)
    assert c.engine.last["split"] == 1
    assert_exact(c, ref, g)


def test_dense_correlator_scale_factor_and_dtypes(built_lib, cuda_device):
    z = golden("dense_small_u8")
    fr, qm = z["frames"], z["qmask"]
    nb = int(qm.max())
    sf = np.arange(1, nb + 1) * 10.0
    from dynamix_gb300.correlator import DenseCorrelator
    c = DenseCorrelator(fr.shape[1:], fr.shape[0], qmask=qm)
    g = c.correlate(fr.astype(np.int16))               # other integer dtypes are accepted
    assert_exact(c, o.g2_exact(fr, qm), g)
    c.scale_factors = {b: s for b, s in zip(c.bins, sf)}
    c2 = DenseCorrelator(fr.shape[1:], fr.shape[0], qmask=qm)
    c2._set_scale_factor(list(sf))
    c2._init_engine()
    g2 = c2.correlate(fr)
    assert np.allclose(g2, o.g2_exact(fr, qm, scale_factor=list(sf))["g2"], rtol=1e-6)
    with pytest.raises(ValueError):
        c.correlate(-fr.astype(np.int16) - 1)
    with pytest.raises(ValueError):
        DenseCorrelator(fr.shape[1:], fr.shape[0], qmask=qm, weights=np.ones(fr.shape[1:]))


def test_device_tensor_input_and_repeat(built_lib, cuda_device):
    import torch
    z = golden("dense_small_u8")
    fr, qm = z["frames"], z["qmask"]
    ref = o.g2_exact(fr, qm)
    from dynamix_gb300.correlator import MatMulCorrelator
    c = MatMulCorrelator(fr.shape[1:], fr.shape[0], qmask=qm)
    d = torch.from_numpy(fr).to(cuda_device)
    for _ in range(3):                                 # buffers reused across calls
        g = c.correlate(d)
        assert_exact(c, ref, g)


def test_tc_equals_plain_at_medium_size(built_lib, cuda_device):
    """tensor-core and plain kernels agree bit for bit on a larger stack."""
    import torch
    from dynamix_gb300.correlator import MatMulCorrelator
    from dynamix_gb300.speckle import annular_qmask, speckle_torch
    T, shape = 2000, (128, 160)
    fr = speckle_torch(T, shape, 0.99, 0.3, seed=4, device=cuda_device)
    qm = annular_qmask(shape, 6, 5.0, 70.0)
    a = MatMulCorrelator(shape, T, qmask=qm, extra_options={"method": "tc"})
    b = MatMulCorrelator(shape, T, qmask=qm, extra_options={"method": "plain"})
    ga, gb = a.correlate(fr), b.correlate(fr)
    assert np.array_equal(a.numerator, b.numerator)
    assert np.array_equal(a.denominator, b.denominator)
    assert np.array_equal(ga, gb, equal_nan=True)
    # size-independent checks against torch reductions of the same stack
    f = fr.to(torch.int64).reshape(T, -1)
    qt = torch.as_tensor(qm.ravel(), device=cuda_device)
    for bi in range(6):
        x = f[:, qt == bi + 1]
        assert int((x * x).sum()) == int(a.numerator[bi, 0])
        assert np.array_equal(x.sum(dim=1).cpu().numpy(), a.sums[bi])
        assert int((x[1:] * x[:-1]).sum()) == int(a.numerator[bi, 1])


def test_unaligned_device_view(built_lib, cuda_device):
    """A device view that starts off a 16-byte boundary is handled (copied)."""
    import torch
    from dynamix_gb300.correlator import MatMulCorrelator
    z = golden("dense_small_u8")
    fr, qm = z["frames"], z["qmask"]
    T = fr.shape[0]
    big = torch.zeros(fr.size + 1, dtype=torch.uint8, device=cuda_device)
    big[1:] = torch.from_numpy(fr.ravel()).to(cuda_device)
    view = big[1:].view(fr.shape)
    assert view.data_ptr() % 16 != 0
    c = MatMulCorrelator(fr.shape[1:], T, qmask=qm)
    g = c.correlate(view)
    assert_exact(c, o.g2_exact(fr, qm), g)


@pytest.mark.parametrize("T", [300, 1000, 2100])
def test_chunked_pipeline_matches_single_pass(built_lib, cuda_device, T):
    """Copy/pack/Gram overlapped chunk by chunk (pinned host input or device
    input) gives the same exact sums as the one-pass pipeline and the oracle."""
    import torch
    from dynamix_gb300.correlator import MatMulCorrelator
    from dynamix_gb300.speckle import annular_qmask, speckle_numpy
    shape = (40, 52)
    fr = speckle_numpy(T, shape, 0.99, 0.4, seed=T, dtype=np.uint8, max_count=16)
    qm = annular_qmask(shape, 5, 2.0, 26.0)
    ref = o.g2_exact(fr, qm)
    a = MatMulCorrelator(shape, T, qmask=qm)
    host = torch.from_numpy(fr).pin_memory()
    g = a.correlate(host)
    assert a.engine.last.get("pipeline_chunks", 0) >= (2 if T >= 512 else 1)
    assert_exact(a, ref, g)
    g = a.correlate(host.to(cuda_device))
    assert_exact(a, ref, g)
    b = MatMulCorrelator(shape, T, qmask=qm)
    b.engine.pipeline = False
    gb = b.correlate(fr)
    assert "pipeline_chunks" not in b.engine.last
    assert np.array_equal(a.numerator, b.numerator) and np.array_equal(a.sums, b.sums)
    assert np.array_equal(g, gb, equal_nan=True)


@pytest.mark.parametrize("top", [None, 16, 17])
def test_host_frames_cropped_to_qmask_columns(built_lib, cuda_device, top):
    """u8 frames in pinned host memory cross the link cropped to the q-mask's
    column window; the results equal the oracle's, also when a count of 16
    needs the exact maximum of the cropped frames and when a count of 17 moves
    the stack to fp16 operands (rerun from the whole host frames)."""
    import torch
    from dynamix_gb300.correlator import MatMulCorrelator
    from dynamix_gb300.speckle import annular_qmask, speckle_numpy
    T, shape = 700, (48, 400)
    fr = speckle_numpy(T, shape, 0.99, 0.4, seed=5, dtype=np.uint8, max_count=15)
    qm = annular_qmask(shape, 6, 3.0, 30.0, center=(24, 200))    # binned columns 171..229
    fr[T // 3, 5, 2] = 200                                      # unbinned, outside the window
    if top is not None:
        fr[T // 2, 24, 210] = top                               # binned
        fr[T // 2, 24, 211] = 1
    ref = o.g2_exact(fr, qm)
    c = MatMulCorrelator(shape, T, qmask=qm)
    eng = c.engine
    c0, wc = eng.crop
    assert c0 % 16 == 0 and wc % 16 == 0 and c0 <= 171 and c0 + wc > 229 and wc < shape[1]
    host = torch.from_numpy(fr).pin_memory()
    g = c.correlate(host)
    assert_exact(c, ref, g)
    if top == 17:
        assert eng.last["mode"] == "fp16"
    else:
        assert eng.last["mode"] == "e4m3" and eng.last["crop"] == [c0, wc]
        assert eng.last["h2d_bytes"] == T * shape[0] * wc
    g = c.correlate(host)                 # after a rerun on fp16 the next call starts there
    assert_exact(c, ref, g)
    g = c.correlate(host.to(cuda_device))  # device input: whole frames
    assert_exact(c, ref, g)


@pytest.mark.parametrize("name", ["dense_small_u8", "dense_bright_u8", "dense_128x128_u8", "dense_u16"])
def test_calc_std(built_lib, cuda_device, name):
    """calc_std (dense.py:58-66): against the float64 oracle to 1e-4 relative
    (float products and ratios on the tensor cores, float64 reduction) and
    against the reference's own float32 result to 1e-3; NaN exactly where the
    reference divides by zero."""
    from dynamix_gb300.correlator import MatMulCorrelator, py_dense_correlator
    z = golden(name)
    fr, qm = z["frames"], z["qmask"]
    c = MatMulCorrelator(fr.shape[1:], fr.shape[0], qmask=qm)
    res, dev = c.correlate(fr, calc_std=True)
    ref = o.g2_exact(fr, qm)
    assert np.array_equal(c.numerator, ref["numerator"])
    assert np.array_equal(res, ref["g2"].astype(np.float32), equal_nan=True)
    want = o.dense_std_exact(fr, qm)
    got = c.engine.dev_f64[: c.n_bins].cpu().numpy()
    assert np.array_equal(np.isfinite(got), np.isfinite(want))
    ok = np.isfinite(want)
    assert np.all(np.abs(got[ok] - want[ok]) <= 1e-4 * np.abs(want[ok]) + 1e-9)
    assert np.allclose(dev, got.astype(np.float32), rtol=1e-6, equal_nan=True)
    rs = z["g2_ref_std"].astype(np.float64)
    okr = np.isfinite(rs) & (np.abs(rs) > 1e-6)
    assert np.max(np.abs(got[okr] - rs[okr]) / np.abs(rs[okr])) < 1e-3
    # one bin through py_dense_correlator
    r1, d1 = py_dense_correlator(fr, qm == 1, calc_std=True)
    assert np.allclose(d1, got[0], rtol=1e-9, equal_nan=True)


@pytest.mark.parametrize("case", ["golden_u16_forced_planes", "bright_u16"])
def test_calc_std_byte_planes(built_lib, cuda_device, case):
    """calc_std on byte-plane operands (counts above 2048, or the planes
    forced): each bin's Gram is assembled from its four plane combinations in
    float32 and the deviation reduced in float64 -- within 1e-4 relative of the
    float64 oracle, within 1e-3 of the reference's own float32 result where
    the golden vectors have it, NaN exactly where the reference divides by
    zero."""
    from dynamix_gb300.correlator import MatMulCorrelator
    from dynamix_gb300.speckle import annular_qmask, speckle_numpy
    if case == "golden_u16_forced_planes":
        z = golden("dense_u16")
        fr, qm, rs = z["frames"], z["qmask"], z["g2_ref_std"].astype(np.float64)
        opts = {"operand": "bytes"}
    else:
        fr = speckle_numpy(300, (24, 30), 0.99, 900.0, seed=19, dtype=np.uint16, max_count=4095)
        assert fr.max() > 2048
        qm = annular_qmask((24, 30), 3, 0.0, 15.0)
        rs, opts = None, {}
        fr[100:110] = 0                                # dark frames: zero denominators (NaN deviations)
    c = MatMulCorrelator(fr.shape[1:], fr.shape[0], qmask=qm, extra_options=opts)
    res, dev = c.correlate(fr, calc_std=True)
    assert c.engine.last["split"] == 1
    assert np.array_equal(c.numerator, o.g2_exact(fr, qm)["numerator"])
    want = o.dense_std_exact(fr, qm)
    got = c.engine.dev_f64[: c.n_bins].cpu().numpy()
    assert np.array_equal(np.isfinite(got), np.isfinite(want))
    ok = np.isfinite(want)
    assert np.all(np.abs(got[ok] - want[ok]) <= 1e-4 * np.abs(want[ok]) + 1e-9)
    assert np.allclose(dev, got.astype(np.float32), rtol=1e-6, equal_nan=True)
    if rs is not None:
        okr = np.isfinite(rs) & (np.abs(rs) > 1e-6)
        assert np.max(np.abs(got[okr] - rs[okr]) / np.abs(rs[okr])) < 1e-3


def test_autotuner_keeps_results_exact(built_lib, cuda_device):
    import torch
    from dynamix_gb300 import tune
    from dynamix_gb300.correlator import MatMulCorrelator
    from dynamix_gb300.speckle import annular_qmask, speckle_numpy
    T, shape = 1200, (40, 52)
    fr = speckle_numpy(T, shape, 0.99, 0.4, seed=5, dtype=np.uint8, max_count=16)
    qm = annular_qmask(shape, 4, 2.0, 26.0)
    c = MatMulCorrelator(shape, T, qmask=qm)
    d = torch.from_numpy(fr).to(cuda_device)
    cands = [(1024, 2), (2048, 4, 256, "single"), (4096, 8, 512, "pair", "fp16"), (2048, 6, 0, "pair", "e4m3")]
    best, times = tune.tune_dense(c, d, candidates=cands, repeats=1)
    assert best in times and len(times) == 4 and all(len(k) == 5 for k in times)
    assert tune.current(c.engine)[:4] == best[:4]
    g = c.correlate(d)
    assert_exact(c, o.g2_exact(fr, qm), g)
    for cand in times:                                   # every candidate gives the same exact sums
        tune.set_choice(c.engine, cand)
        assert_exact(c, o.g2_exact(fr, qm), c.correlate(d))
        assert c.engine.last["tile"] == cand[3]
    c2 = MatMulCorrelator(shape, T, qmask=qm)            # same key: the choice is reused
    assert tune.current(c2.engine)[:4] == best[:4]


@pytest.mark.parametrize("bright", [False, True])
def test_64_narrow_bins(built_lib, cuda_device, bright):
    """More than 32 bins inside one 2048-pixel pack chunk (fp16 / byte planes
    carry per-chunk bin slots for S)."""
    from dynamix_gb300.correlator import MatMulCorrelator
    from dynamix_gb300.speckle import annular_qmask, speckle_numpy
    T, shape = 150, (256, 256)
    fr = speckle_numpy(T, shape, 0.95, 3.0, seed=9, dtype=np.uint16)
    if bright:
        fr = (fr.astype(np.int64) * 700).astype(np.uint16)        # byte planes
    qm = annular_qmask(shape, 64, 0.0, 102.4)
    c = MatMulCorrelator(shape, T, qmask=qm)
    g = c.correlate(fr)
    assert c.engine.last["mode"] == ("bytes" if bright else "fp16")
    assert_exact(c, o.g2_exact(fr, qm), g)


# ---- the u8 __dp4a plain comparator -----------------------------------------
@pytest.mark.parametrize("name", ["dense_small_u8", "dense_bright_u8", "dense_128x128_u8"])
def test_dp4a_golden_cases(built_lib, cuda_device, name):
    z = golden(name)
    ref = o.g2_exact(z["frames"], z["qmask"])
    c, g = run(z["frames"], z["qmask"], "dp4a")
    assert c.engine.last["mode"] == "u8"
    assert_exact(c, ref, g)


def test_dp4a_edges_and_ragged(built_lib, cuda_device):
    z = golden("dense_edge")
    fr = z["frames"]
    for qm in (None, z["qmask_gap"]):
        c, g = run(fr, qm, "dp4a")
        assert_exact(c, o.g2_exact(fr, qm), g)
    from dynamix_gb300.speckle import annular_qmask, speckle_numpy
    for T in (1, 127, 129, 257):
        fr = speckle_numpy(T, (20, 26), 0.95, 3.0, seed=T)
        qm = annular_qmask((20, 26), 3, 1.0, 12.0)
        c, g = run(fr, qm, "dp4a")
        assert_exact(c, o.g2_exact(fr, qm), g)


def test_dp4a_saturated_wide_bin(built_lib, cuda_device):
    """Counts of 255 over a 70,000-pixel bin: one Gram entry is 70,000 * 255^2
    > 2^32, so the K split at 65,536 columns is what keeps the uint32
    accumulators exact."""
    T, shape = 40, (1, 70000)
    rng = np.random.default_rng(3)
    fr = np.where(rng.random((T,) + shape) < 0.95, 255, rng.integers(0, 255, (T,) + shape)).astype(np.uint8)
    qm = np.ones(shape, np.int32)
    qm[0, :100] = 2
    ref = o.g2_exact(fr, qm)
    c, g = run(fr, qm, "dp4a")
    assert c.engine.last["n_grams"] >= 3
    assert_exact(c, ref, g)


def test_dp4a_rejects_u16(built_lib, cuda_device):
    fr = np.full((8, 4, 4), 300, dtype=np.uint16)
    with pytest.raises(ValueError):
        run(fr, None, "dp4a")


@pytest.mark.parametrize("tile", ["pair", "single"])
@pytest.mark.parametrize("name", ["refcl_dense_u8", "refcl_dense_wide"])
def test_matches_reference_dense_kernel(built_lib, cuda_device, name, tile):
    """N and S bit-exact against the reference's own densecorrelator.cl
    (correlator_multiQ_dense + compute_sums_dense, run as C by
    tests/golden/make_wg_golden.py); DenseCorrelator's float32 g2 within 2e-6
    of the reference kernel's float32 g2."""
    z = golden(name)
    fr, qm = z["frames"], z["qmask"]
    c, g = run(fr, qm, "tc", cls="DenseCorrelator", tile=tile)
    assert np.array_equal(c.numerator, z["numer_f"].astype(np.int64))
    assert np.array_equal(c.sums, z["sums"].astype(np.int64))
    ref = z["g2"].astype(np.float64)
    ok = np.isfinite(ref)
    assert np.array_equal(np.isfinite(g), ok)
    assert np.all(np.abs(g[ok] - ref[ok]) <= 2e-6 * np.abs(ref[ok]))


@pytest.mark.parametrize("operand", ["fp16", "bytes"])
def test_k_split_reuse_across_stacks(built_lib, cuda_device, operand):
    """One correlator, several fp16 / byte-plane stacks: a stack whose energy
    bounds lie within those planned for before reuses the K split without a
    host round trip; a brighter one is detected on the device and run again
    through the planned path.  Every result is exact."""
    from dynamix_gb300.correlator import MatMulCorrelator
    from dynamix_gb300.speckle import annular_qmask, speckle_numpy
    T, shape = 400, (24, 40)
    qm = annular_qmask(shape, 4, 1.0, 20.0)
    mus = {"fp16": (20.0, 60.0, 5.0, 20.0), "bytes": (700.0, 2000.0, 300.0, 700.0)}[operand]
    c = MatMulCorrelator(shape, T, qmask=qm, extra_options={"operand": operand})
    plans = []
    for i, mu in enumerate(mus):
        fr = speckle_numpy(T, shape, 0.97, mu, seed=40 + i, dtype=np.uint16, max_count=65535)
        g = c.correlate(fr)
        assert c.engine.last["mode"] == operand
        assert_exact(c, o.g2_exact(fr, qm), g)
        plans.append(c.engine.last["plan"])
    assert plans[0] == "planned" and plans[1] == "planned"   # the first stack, then a brighter one
    assert plans[2] == "reused" and plans[3] == "reused"     # dimmer, and the first again


@pytest.mark.parametrize("dtype", [np.uint8, np.uint16])
def test_fp16_pipeline_with_reused_split(built_lib, cuda_device, dtype):
    """Stacks on fp16 operands reuse a K split once one covers them: from
    pinned host memory through the chunked copy / pack / Gram pipeline,
    device-resident ones unchunked; a brighter stack falls back to the
    planned path; every result equals the oracle."""
    import torch
    from dynamix_gb300.correlator import MatMulCorrelator
    from dynamix_gb300.speckle import annular_qmask, speckle_numpy
    T, shape = 1100, (30, 50)
    qm = annular_qmask(shape, 5, 2.0, 25.0)
    c = MatMulCorrelator(shape, T, qmask=qm, extra_options={"operand": "fp16"})
    seen = []
    for i, (mu, where) in enumerate(((20.0, "device"), (12.0, "device"), (12.0, "host"), (60.0, "host"),
                                     (25.0, "device"))):
        fr = speckle_numpy(T, shape, 0.98, mu, seed=70 + i, dtype=dtype, max_count=255 if dtype == np.uint8 else 2000)
        inp = torch.from_numpy(fr)
        inp = inp.to(cuda_device) if where == "device" else inp.pin_memory()
        g = c.correlate(inp)
        assert c.engine.last["mode"] == "fp16"
        assert_exact(c, o.g2_exact(fr, qm), g)
        seen.append((c.engine.last.get("plan"), "pipeline_chunks" in c.engine.last))
    assert seen[0] == ("planned", False)
    assert seen[1] == ("reused", False)                   # device-resident: unchunked, split reused
    assert seen[2] == ("reused", True)                    # pinned host: the chunked pipeline
    assert seen[3] == ("planned", False)                  # brighter: detected, run again on a fresh plan
    assert seen[4] == ("reused", False)
