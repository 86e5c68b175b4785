"""GPU parity of the CTA-pair tensor-core Grams (g2_gram_tc_pair, 256 x 256
blocks, and g2_gram_tc_wide, 256 x 512 blocks, on tcgen05 cta_group::2)
against the CPU oracle: N, S and D bit-exact (int64), g2 within 1e-12 relative
of the oracle's FP64 value -- the same bar as the single-CTA kernel."""
import numpy as np
import pytest

from conftest import golden
from oracle import g2_oracle as o
from test_dense_gpu import assert_exact, run

pytestmark = pytest.mark.gpu


TILES = ["pair", "wide"]


@pytest.mark.parametrize("tile", TILES)
@pytest.mark.parametrize("name", ["dense_small_u8", "dense_bright_u8", "dense_128x128_u8", "dense_u16"])
def test_pair_golden_cases(built_lib, cuda_device, name, tile):
    z = golden(name)
    ref = o.g2_exact(z["frames"], z["qmask"])
    c, g = run(z["frames"], z["qmask"], "tc", tile=tile)
    assert c.engine.last["tile"] == tile
    assert_exact(c, ref, g)


@pytest.mark.parametrize("tile", TILES)
@pytest.mark.parametrize("operand", ["e4m3", "fp16", "bytes"])
def test_pair_operands(built_lib, cuda_device, operand, tile):
    from dynamix_gb300.speckle import annular_qmask, speckle_numpy
    T, shape = 300, (24, 40)
    dt = np.uint16 if operand == "bytes" else np.uint8
    mu = 900.0 if operand == "bytes" else (0.8 if operand == "e4m3" else 20.0)
    fr = speckle_numpy(T, shape, 0.97, mu, seed=31, dtype=dt, max_count=65535 if dt == np.uint16 else None)
    qm = annular_qmask(shape, 4, 1.0, 20.0)
    c, g = run(fr, qm, "tc", tile=tile, operand=operand)
    assert c.engine.last["mode"] == operand
    assert_exact(c, o.g2_exact(fr, qm), g)


@pytest.mark.parametrize("tile", TILES)
@pytest.mark.parametrize("T", [1, 2, 31, 32, 33, 200, 255, 256, 257, 300, 511, 512, 513, 700, 767, 768, 769, 1100])
def test_pair_ragged_frame_counts(built_lib, cuda_device, T, tile):
    from dynamix_gb300.speckle import annular_qmask, speckle_numpy
    fr = speckle_numpy(T, (20, 26), 0.95, 1.5, seed=T + 1)
    qm = annular_qmask((20, 26), 3, 1.0, 12.0)
    c, g = run(fr, qm, "tc", tile=tile)
    assert_exact(c, o.g2_exact(fr, qm), g)


@pytest.mark.parametrize("tile", TILES)
def test_pair_edges(built_lib, cuda_device, tile):
    z = golden("dense_edge")
    fr = z["frames"]
    for qm in (None, z["qmask_gap"]):
        c, g = run(fr, qm, "tc", tile=tile)
        assert_exact(c, o.g2_exact(fr, qm), g)


@pytest.mark.parametrize("tile", TILES)
def test_pair_saturated_k_split(built_lib, cuda_device, tile):
    T, shape = 300, (40, 60)
    rng = np.random.default_rng(1)
    fr = np.where(rng.random((T,) + shape) < 0.9, 255, rng.integers(0, 255, (T,) + shape)).astype(np.uint8)
    qm = np.ones(shape, np.int32)
    qm[:, :7] = 2
    c, g = run(fr, qm, "tc", tile=tile)
    assert c.engine.last["n_grams"] > 2
    assert_exact(c, o.g2_exact(fr, qm), g)


@pytest.mark.parametrize("tile", TILES)
@pytest.mark.parametrize("T", [1000, 2100])
def test_pair_pipeline_host_and_device(built_lib, cuda_device, T, tile):
    """The chunked copy/pack/Gram pipeline with pair blocks, from pinned host
    memory and from the device, equals the single-pass result and the oracle."""
    import torch
    from dynamix_gb300.correlator import MatMulCorrelator
    from dynamix_gb300.speckle import annular_qmask, speckle_numpy
    shape = (30, 50)
    fr = speckle_numpy(T, shape, 0.98, 0.3, seed=T)
    qm = annular_qmask(shape, 5, 2.0, 25.0)
    ref = o.g2_exact(fr, qm)
    c = MatMulCorrelator(shape, T, qmask=qm, extra_options={"tile": tile})
    host = torch.from_numpy(fr).pin_memory()
    g = c.correlate(host)
    assert c.engine.last.get("pipeline_chunks", 1) > 1
    assert_exact(c, ref, g)
    g2 = c.correlate(torch.from_numpy(fr).to(cuda_device))
    assert_exact(c, ref, g2)


def test_pair_equals_single_at_medium_size(built_lib, cuda_device):
    import torch
    from dynamix_gb300.correlator import MatMulCorrelator
    from dynamix_gb300.speckle import annular_qmask, speckle_torch
    T, shape = 3000, (64, 128)
    fr = speckle_torch(T, shape, 0.99, 0.2, seed=3, device=cuda_device)
    qm = annular_qmask(shape, 6, 4.0, 60.0)
    out = {}
    for tile in ("single", "pair", "wide"):
        c = MatMulCorrelator(shape, T, qmask=qm, extra_options={"tile": tile})
        c.correlate(fr)
        out[tile] = (c.numerator, c.sums, c.denominator)
    for t in ("pair", "wide"):
        for a, b in zip(out["single"], out[t]):
            assert np.array_equal(a, b)
    torch.cuda.synchronize()
