"""GPU tests of the u8 e4m3 pack by work units (g2_pack_e4m3_units): the
packed matrix is byte-identical to the per-word kernel's (g2_pack_e4m3), and
its range check -- an OR of the moved bytes, resolved by the exact binned
maximum when a count of 16 or more may be present -- keeps the results
exact."""
import ctypes

import numpy as np
import pytest

from oracle import g2_oracle as o
from test_dense_gpu import assert_exact, run

pytestmark = pytest.mark.gpu

MASKS = [
    ((514, 1030), 16, 20.0, 400.0, (257, 515)),
    ((256, 256), 12, 8.0, 128.0, (128, 128)),
    ((61, 77), 5, 0.0, 30.0, (30, 38)),       # npix not a multiple of 16: every frame start unaligned
    ((1062, 1028), 64, 0.0, 411.0, (531, 514)),
]


def _packed(lib, torch, dev, frames, L, units):
    T = frames.shape[0]
    npix = frames[0].numel()
    out = torch.zeros(T * L.packed_cols, dtype=torch.uint8, device=dev)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    st = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    if units:
        rc = lib.g2_pack_e4m3_units(p(frames), T, npix, p(L.d_unit_block_off), p(L.d_units), L.n_chunks, p(out),
                                    L.packed_cols, p(err), st)
    else:
        rc = lib.g2_pack_e4m3(p(frames), 1, T, npix, p(L.d_chunk_word_off), p(L.d_word_dst), p(L.d_word_src),
                              L.n_chunks, p(out), L.packed_cols, p(err), st)
    assert rc == 0
    torch.cuda.synchronize(dev)
    return out.cpu().numpy(), int(err.item())


@pytest.mark.parametrize("mask", MASKS, ids=lambda m: "%dx%d" % m[0])
def test_units_pack_equals_word_pack(built_lib, cuda_device, mask):
    import torch
    from dynamix_gb300 import _lib
    from dynamix_gb300.engine import device_layout
    from dynamix_gb300.plan import MODE_E4M3
    from dynamix_gb300.speckle import annular_qmask
    shape, nb, r0, r1, c = mask
    qm = annular_qmask(shape, nb, r0, r1, center=c)
    L = device_layout(qm, nb, MODE_E4M3, cuda_device)
    rng = np.random.default_rng(nb)
    # 603 frames of the 514 x 1030 stack: each CTA moves many steps (the
    # offsets it advances per step) and the last step is ragged
    for T in (1, 5, 37) + ((603,) if shape == (514, 1030) else ()):
        fr = torch.from_numpy(rng.integers(0, 16, (T,) + shape).astype(np.uint8)).to(cuda_device)
        a, ea = _packed(built_lib, torch, cuda_device, fr, L, units=True)
        b, eb = _packed(built_lib, torch, cuda_device, fr, L, units=False)
        assert np.array_equal(a, b)
        assert ea == 0 and eb == 0                     # counts <= 15: the OR stays <= 15
    # counts up to 255: the same bytes move; the OR flags the stack for an exact check
    fr = torch.from_numpy(rng.integers(0, 256, (9,) + shape).astype(np.uint8)).to(cuda_device)
    a, ea = _packed(built_lib, torch, cuda_device, fr, L, units=True)
    b, eb = _packed(built_lib, torch, cuda_device, fr, L, units=False)
    assert np.array_equal(a, b)
    assert ea == _lib.DEVERR_RANGE_CHECK and eb == _lib.DEVERR_RANGE


@pytest.mark.parametrize("kind", ["interleaved", "empty_chunks"])
def test_units_pack_unusual_chunks(built_lib, cuda_device, kind):
    # interleaved: two bins alternating pixel by pixel, so every destination
    # word is a gather and a 2048-pixel chunk holds 16 blocks of units (more
    # than one per mover warp); empty_chunks: the first 5,000 pixels unbinned,
    # so whole chunks move nothing
    import torch
    from dynamix_gb300.engine import device_layout
    from dynamix_gb300.plan import MODE_E4M3
    shape = (64, 130)
    qm = np.zeros(shape, np.int32)
    if kind == "interleaved":
        qm.ravel()[:] = 1 + np.arange(qm.size) % 2
        nb = 2
    else:
        qm.ravel()[5000:] = 1 + (np.arange(qm.size - 5000) // 700) % 3
        nb = 3
    L = device_layout(qm, nb, MODE_E4M3, cuda_device)
    blocks = np.diff(L.unit_block_off)
    assert blocks.max() > 15 if kind == "interleaved" else (blocks == 0).any()
    rng = np.random.default_rng(7)
    for T in (1, 6, 41):
        fr = torch.from_numpy(rng.integers(0, 16, (T,) + shape).astype(np.uint8)).to(cuda_device)
        a, ea = _packed(built_lib, torch, cuda_device, fr, L, units=True)
        b, eb = _packed(built_lib, torch, cuda_device, fr, L, units=False)
        assert np.array_equal(a, b)
        assert ea == 0 and eb == 0


@pytest.mark.parametrize("pipelined", [True, False])
@pytest.mark.parametrize("top", [16, 17])
def test_range_check_resolution(built_lib, cuda_device, top, pipelined):
    """A count of 16 makes the OR ambiguous: the exact maximum (16) keeps the
    e4m3 operand; a 17 moves the stack to fp16.  Exact either way."""
    import torch
    from dynamix_gb300.correlator import MatMulCorrelator
    from dynamix_gb300.speckle import annular_qmask, speckle_numpy
    T, shape = 700, (32, 48)
    fr = np.minimum(speckle_numpy(T, shape, 0.97, 1.0, seed=top), 15).astype(np.uint8)
    fr[T // 2, 10, 20] = top
    fr[T // 3, 12, 22] = 1
    qm = annular_qmask(shape, 4, 2.0, 23.0)
    c = MatMulCorrelator(shape, T, qmask=qm)
    c.engine.pipeline = pipelined
    g = c.correlate(torch.from_numpy(fr).to(cuda_device))
    assert c.engine.last["mode"] == ("e4m3" if top == 16 else "fp16")
    assert_exact(c, o.g2_exact(fr, qm), g)


def test_dp4a_with_units_pack(built_lib, cuda_device):
    from dynamix_gb300.speckle import annular_qmask, speckle_numpy
    fr = speckle_numpy(300, (40, 44), 0.97, 30.0, seed=3)
    assert fr.max() > 16
    qm = annular_qmask((40, 44), 4, 2.0, 20.0)
    c, g = run(fr, qm, "dp4a")
    assert_exact(c, o.g2_exact(fr, qm), g)
