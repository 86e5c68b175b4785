"""Host logic of the dense pipeline, checked on the CPU.

A numpy emulation of the pack kernel and of the per-item semantics of the
Gram kernels (what each g2_gram_item adds to N) must reproduce the oracle's
numerator exactly; this pins the layout, the K split and the upper-triangle
item enumeration independently of the GPU.
"""
import numpy as np
import pytest

from conftest import golden
from dynamix_gb300 import plan
from dynamix_gb300._lib import BK, PACK_CHUNK, PACK_MAX_SLOTS, PLAIN_BM, PLAIN_BN, TC_BM, TC_BN  # noqa: F401
from dynamix_gb300.speckle import annular_qmask, speckle_numpy
from oracle import g2_oracle as o


def emulate_pack(frames, L):
    """What g2_pack_frames writes, from the layout's chunk tables; the packed
    matrix is cross-checked against the per-bin column map, and the segment
    energy bound is built from per-piece maxima exactly as the kernel does."""
    T = frames.shape[0]
    flat = frames.reshape(T, -1).astype(np.int64)
    packed = np.zeros((T, L.packed_cols), dtype=np.int64)
    chunk = np.repeat(np.arange(L.n_chunks), np.diff(L.chunk_entry_off))
    meta = L.entry_meta.astype(np.int64)
    pix = chunk * PACK_CHUNK + (meta & 2047)
    slot = (meta >> 11) & 127
    piece = L.chunk_piece_off[chunk] + (meta >> 18)
    b = L.chunk_slot_bin[chunk * PACK_MAX_SLOTS + slot]
    # the slot's bin is the bin whose columns hold the entry
    assert np.all((b >= 0) & (L.plane0[b] <= L.entry_dst) & (L.entry_dst < L.plane0[b] + L.kpad[b]))
    v = flat[:, pix]
    energy = np.zeros((L.n_planes, T, max(L.n_pieces, 1)), dtype=np.int64)
    if L.split:
        packed[:, L.entry_dst] = v >> 8
        packed[:, L.entry_dst + L.bin_kpad[b]] = v & 255
        np.add.at(energy[0].T, piece, ((v >> 8) ** 2).T)
        np.add.at(energy[1].T, piece, ((v & 255) ** 2).T)
    else:
        packed[:, L.entry_dst] = v
        np.add.at(energy[0].T, piece, (v ** 2).T)
    # the same matrix from the column map (bins contiguous, raster order)
    ref = np.zeros_like(packed)
    cs = L.col_src.reshape(-1, BK)
    for s in range(L.n_segs):
        src = cs[s]
        vv = np.where(src >= 0, flat[:, np.maximum(src, 0)], 0)
        if L.split:
            ref[:, L.seg_dst0[s]:L.seg_dst0[s] + BK] = vv >> 8
            ref[:, L.seg_dst1[s]:L.seg_dst1[s] + BK] = vv & 255
        else:
            ref[:, L.seg_dst0[s]:L.seg_dst0[s] + BK] = vv
    assert np.array_equal(packed, ref)
    piece_max = energy.max(axis=1)[:, : L.n_pieces].ravel()
    emax = L.segment_emax(piece_max)
    true = (packed.reshape(T, -1, BK) ** 2).sum(axis=2).max(axis=0)
    assert np.all(emax >= true)
    return packed, emax


def run_items(packed, items, n_rows, T, bm, bn, ones=None):
    """What the Gram kernels add for each item: lag sums over t <= t' < T and,
    when the packed matrix carries the row of ones (``ones``), the bin sums
    from that row's column.  Returns N (and S when ``ones`` is given)."""
    N = np.zeros(n_rows * T, dtype=np.int64)
    S = np.zeros(n_rows * T, dtype=np.int64)
    rows = [packed] + ([ones[None, :].astype(np.int64)] if ones is not None else [])
    P = np.concatenate(rows + [np.zeros((bn + bm, packed.shape[1]), dtype=np.int64)])
    for it in items:
        i0, j0, a0, b0, kl = int(it["i0"]), int(it["j0"]), int(it["a_k0"]), int(it["b_k0"]), int(it["k_len"])
        G = P[i0:i0 + bm, a0:a0 + kl] @ P[j0:j0 + bn, b0:b0 + kl].T
        assert G.max(initial=0) <= plan.EXACT_LIMIT
        r, c = np.meshgrid(np.arange(bm), np.arange(bn), indexing="ij")
        t, tp = i0 + r, j0 + c
        tau = tp - t
        ok = (tau >= 0) & (t < T) & (tp < T)
        np.add.at(N, int(it["out_off"]) + tau[ok], G[ok] << int(it["shift"]))
        if it["s_off"] >= 0:
            sel = (tp == T) & (t < T)
            np.add.at(S, int(it["s_off"]) + t[sel], G[sel])
    if ones is None:
        return N.reshape(n_rows, T)
    return N.reshape(n_rows, T), S.reshape(n_rows, T)


@pytest.mark.parametrize("mode", [0, 1, 2])
@pytest.mark.parametrize("kind", ["tc", "plain"])
@pytest.mark.parametrize("name", ["dense_small_u8", "dense_u16"])
def test_item_semantics_reproduce_oracle(name, kind, mode):
    z = golden(name)
    fr, qm = z["frames"], z["qmask"]
    T = fr.shape[0]
    nb = int(qm.max())
    L = plan.PackLayout(qm, nb, mode)
    if mode == 0 and fr.max() > plan.FP16_MAX_EXACT:
        pytest.skip("counts do not fit fp16")
    if mode == 2 and fr.max() > plan.E4M3_MAX_EXACT:
        pytest.skip("counts do not fit e4m3")
    packed, emax = emulate_pack(fr, L)
    if mode == plan.MODE_E4M3:
        emax = plan.e4m3_segment_bound(L)
    grams = plan.chunk_grams(L, emax)
    bm, bn = (TC_BM, TC_BN) if kind == "tc" else (PLAIN_BM, PLAIN_BN)
    ref = o.g2_exact(fr, qm)
    if L.ones_row and kind == "tc":
        items = plan.gram_items(T, grams, kind=kind, s_base=0)
        N, S = run_items(packed, items, nb, T, bm, bn, ones=L.ones_row_values())
        assert np.array_equal(S, ref["sums"])
    else:
        items = plan.gram_items(T, grams, kind=kind)
        N = run_items(packed, items, nb, T, bm, bn)
    assert np.array_equal(N, ref["numerator"])


def test_k_split_honours_bound_with_bright_counts():
    # all counts 255: a 64-column segment has energy 64*255^2 = 4.16e6, so a
    # Gram over 1000 columns must be split to keep sums <= 2^24
    T, shape = 40, (20, 50)
    fr = np.full((T,) + shape, 255, dtype=np.uint8)
    qm = np.ones(shape, dtype=np.int32)
    L = plan.PackLayout(qm, 1, 0)
    packed, emax = emulate_pack(fr, L)
    grams = plan.chunk_grams(L, emax)
    assert len(grams) > 1
    for (_, a, b, k0, kl, _) in grams:
        assert (packed[:, a + k0:a + k0 + kl] ** 2).sum(axis=1).max() <= plan.EXACT_LIMIT
    items = plan.gram_items(T, grams, kind="tc")
    N = run_items(packed, items, 1, T, TC_BM, TC_BN)
    assert np.array_equal(N, o.g2_exact(fr, qm)["numerator"])


def test_supertile_order_keeps_rows_local():
    # consecutive windows of 152 items touch far fewer rows than the whole stack
    i0, j0 = plan._tiles(10000, TC_BM, TC_BN)
    rows = []
    for w in range(0, i0.size - 152, 152):
        r = set()
        for a, b in zip(i0[w:w + 152], j0[w:w + 152]):
            r.update(range(a, a + TC_BM))
            r.update(range(b, b + TC_BN))
        rows.append(len(r))
    assert np.mean(rows) < 6000


def test_tiles_cover_upper_triangle_once():
    for T in (1, 5, 127, 128, 129, 255, 256, 257, 300, 1000):
        for bm, bn in ((TC_BM, TC_BN), (PLAIN_BM, PLAIN_BN)):
            i0, j0 = plan._tiles(T, bm, bn)
            cover = np.zeros((T + bn, T + bn), dtype=np.int32)
            for a, b in zip(i0, j0):
                cover[a:a + bm, b:b + bn] += 1
            up = np.triu(np.ones((T, T), dtype=bool))
            assert np.all(cover[:T, :T][up] == 1)


def test_layout_groups_bins_in_raster_order():
    qm = annular_qmask((30, 34), 3, 2.0, 15.0)
    L = plan.PackLayout(qm, 3, 0)
    for b in range(3):
        pix = L.col_src[L.src_off[b]:L.src_off[b] + L.npix[b]]
        assert np.array_equal(pix, np.flatnonzero(qm.ravel() == b + 1))
        assert np.all(L.col_src[L.src_off[b] + L.npix[b]:L.src_off[b] + L.kpad[b]] == -1)
    assert L.packed_cols % plan.PAD == 0 and np.all(L.kpad % plan.PAD == 0)


def test_gram_macs_matches_config():
    # 514 x 1030, 16 annuli r in [20, 400) around (257, 515): 1.898e13 MACs at T = 10000
    qm = annular_qmask((514, 1030), 16, 20.0, 400.0, center=(257, 515))
    npix = np.bincount(qm.ravel(), minlength=17)[1:]
    assert npix.sum() == 379563
    assert abs(plan.gram_macs(10000, npix) - 1.898e13) / 1.898e13 < 1e-3


def test_speckle_generator_statistics():
    fr = speckle_numpy(200, (32, 32), 0.9, 2.0, seed=3)
    m = fr.mean()
    assert 1.7 < m < 2.3
    # speckle contrast: var/mean^2 ~ 1 + 1/mean for Poisson-exponential counts
    c = fr.var() / m ** 2
    assert 1.0 < c < 2.2


def test_e4m3_word_tables_decode_to_entries():
    qm = annular_qmask((70, 90), 5, 3.0, 40.0)
    L = plan.PackLayout(qm, 5, plan.MODE_E4M3)
    chunk_e = np.repeat(np.arange(L.n_chunks), np.diff(L.chunk_entry_off))
    want = set(zip((chunk_e * PACK_CHUNK + (L.entry_meta.astype(np.int64) & 2047)).tolist(),
                   L.entry_dst.tolist()))
    got = set()
    chunk_w = np.repeat(np.arange(L.n_chunks), np.diff(L.chunk_word_off))
    x = L.word_src[:, 0].astype(np.int64)
    y = L.word_src[:, 1].astype(np.int64)
    srcs = np.stack([x & 0xFFF, (x >> 12) & 0xFFF, (x >> 24) | ((y & 0xF) << 8), (y >> 4) & 0xFFF], axis=1)
    live = L.word_dst >= 0
    assert live.all() and np.all(L.word_dst % 4 == 0)
    for w in np.flatnonzero(live):
        for i in range(4):
            if srcs[w, i] != 0xFFF:
                got.add((int(chunk_w[w] * PACK_CHUNK + srcs[w, i]), int(L.word_dst[w] + i)))
        # the slot names the bin whose columns hold the word
        b = L.chunk_slot_bin[chunk_w[w] * PACK_MAX_SLOTS + ((y[w] >> 16) & 127)]
        assert L.plane0[b] <= L.word_dst[w] < L.plane0[b] + L.kpad[b]
    assert got == want


@pytest.mark.parametrize("mode", [plan.MODE_FP16, plan.MODE_BYTES, plan.MODE_E4M3])
def test_many_narrow_bins_share_a_chunk(mode):
    """64 annuli on a 256-wide frame: a 2048-pixel chunk holds more than 32
    bins (the serving mix has up to 64 bins on 256 x 256 frames)."""
    qm = annular_qmask((256, 256), 64, 0.0, 102.4)
    L = plan.PackLayout(qm, 64, mode)
    chunk = np.repeat(np.arange(L.n_chunks), np.diff(L.chunk_entry_off))
    slots = (L.entry_meta.astype(np.int64) >> 11) & 127
    per_chunk = max(np.unique(slots[chunk == c]).size for c in range(L.n_chunks) if np.any(chunk == c))
    assert per_chunk > 32
    fr = speckle_numpy(3, (256, 256), 0.9, 3.0, seed=2, dtype=np.uint16 if mode == plan.MODE_BYTES else np.uint8)
    if mode == plan.MODE_BYTES:
        fr = fr * 300
    if mode != plan.MODE_E4M3:
        emulate_pack(fr, L)


def test_kslab_caps_item_k_and_keeps_the_sums():
    """A K-slab cap splits every Gram into pieces of at most that many columns
    whose item sums still reproduce the oracle."""
    z = golden("dense_small_u8")
    fr, qm = z["frames"], z["qmask"]
    T = fr.shape[0]
    nb = int(qm.max())
    L = plan.PackLayout(qm, nb, plan.MODE_FP16)
    packed, emax = emulate_pack(fr, L)
    grams = plan.chunk_grams(L, emax, kslab=128)
    assert all(g[4] <= 128 for g in grams)
    assert len(grams) > len(plan.chunk_grams(L, emax))
    items = plan.gram_items(T, grams, kind="tc")
    N = run_items(packed, items, nb, T, TC_BM, TC_BN)
    assert np.array_equal(N, o.g2_exact(fr, qm)["numerator"])


@pytest.mark.parametrize("T,n,growth", [(10000, 8, 1.5), (10000, 8, 0.0), (1000, 3, 1.5), (300, 1, 1.5),
                                        (2100, 8, 2.0), (257, 2, 1.5)])
def test_pipeline_chunk_bounds(T, n, growth):
    """Frame chunks of the e4m3 pipeline: cut at multiples of 128 frames,
    strictly increasing, covering [0, T); with growth > 0 they do not shrink
    (apart from rounding and the last one)."""
    from dynamix_gb300.engine import DenseEngine
    b = DenseEngine.pipe_bounds(T, n, growth)
    assert b[0] == 0 and b[-1] == T and np.all(np.diff(b) > 0)
    assert np.all(b[1:-1] % 128 == 0) and b.size - 1 <= n
    if growth > 0 and b.size > 3:
        d = np.diff(b)[:-1]
        assert np.all(d[1:] >= d[:-1] - 128)


@pytest.mark.parametrize("n,workers", [(2520, 76), (301, 76), (77, 76), (1000, 1), (5, 8), (0, 4)])
def test_native_lpt_schedule_matches_python(built_lib, n, workers):
    """g2_balance_lpt (the library's host scheduler) places every item in the
    same slot as the Python schedule, each worker's items in index order."""
    rng = np.random.default_rng(n)
    cost = np.round(rng.random(n) * 8, 1) + 0.5      # many equal costs: ties must break alike
    a, na = plan.lpt_slots(cost, workers)
    b, nb = plan.lpt_slots_py(cost, workers)
    assert na == nb and np.array_equal(a, b)
    assert np.unique(a).size == n and (n == 0 or a.max() < na)
    w = a % workers
    for k in range(workers):
        assert np.all(np.diff(a[w == k]) > 0)          # index order within a worker


def test_native_lpt_rejects_bad_arguments(built_lib):
    import ctypes as C
    slots = np.empty(3, dtype=np.int64)
    n_slots = C.c_int64(0)
    bad = np.array([1.0, np.nan, 2.0])
    assert built_lib.g2_balance_lpt(bad.ctypes.data_as(C.c_void_p), 3, 2, slots.ctypes.data_as(C.c_void_p),
                                    C.byref(n_slots)) != 0
    ok = np.array([1.0, 2.0, 3.0])
    assert built_lib.g2_balance_lpt(ok.ctypes.data_as(C.c_void_p), 3, 0, slots.ctypes.data_as(C.c_void_p),
                                    C.byref(n_slots)) != 0


@pytest.mark.parametrize("T,n", [(10000, 8), (2100, 8), (1000, 3), (300, 1), (5000, 4)])
def test_pipeline_chunk_bounds_tapered(T, n):
    """Host-input pipelines cut the last chunk into halving pieces: the
    untapered bounds stay, the pieces are multiples of 128 frames (the last
    one ends at T) and no piece grows towards the end."""
    from dynamix_gb300.engine import DenseEngine
    plain = DenseEngine.pipe_bounds(T, n, 0.0)
    b = DenseEngine.pipe_bounds(T, n, 0.0, taper=3)
    assert b[0] == 0 and b[-1] == T and np.all(np.diff(b) > 0)
    assert set(plain[:-1].tolist()) <= set(b.tolist())
    assert np.all(b[1:-1] % 128 == 0) and b.size - plain.size <= 3
    tail = np.diff(b[plain.size - 2:])
    assert np.all(tail[1:-1] <= tail[:-2])


def test_column_window_and_cropped_layout():
    # host frames are copied cropped to the q-mask's column window: the window
    # is 16-byte aligned, and the cropped frame's layout packs the same pixels
    # into the same columns
    from dynamix_gb300.plan import MODE_E4M3, MODE_FP16, PackLayout, column_window
    from dynamix_gb300.speckle import annular_qmask
    q = annular_qmask((514, 1030), 16, 20.0, 400.0, center=(257, 515))
    assert column_window(q, 16, 0.1) == (112, 816)
    assert column_window(annular_qmask((256, 256), 12, 8.0, 128.0, center=(128, 128)), 12, 0.1) is None
    assert column_window(np.zeros((4, 64), np.int32), 1, 0.1) is None
    z = np.zeros((4, 400), np.int32)
    z[:, 395] = 1
    z[:, 3] = 2                                   # above n_bins: not binned
    assert column_window(z, 1, 0.1) == (384, 16)
    assert column_window(z[:, 210:], 1, 0.1) is None   # 176 of 190 columns skipped: under the 192-byte gap
    z[0, 3] = 1
    assert column_window(z, 1, 0.1) is None       # columns 0..395 of 400
    for qm, nb in ((q, 16), (annular_qmask((61, 300), 5, 0.0, 30.0, center=(30, 140)), 5)):
        c0, wc = column_window(qm, nb, 0.1)
        W = qm.shape[1]
        for mode in (MODE_E4M3, MODE_FP16):
            full = PackLayout(qm, nb, mode)
            crop = PackLayout(np.ascontiguousarray(qm[:, c0:c0 + wc]), nb, mode)
            assert crop.packed_cols == full.packed_cols
            cs = crop.col_src.astype(np.int64)
            mapped = np.where(cs >= 0, cs // wc * W + c0 + cs % wc, -1)
            assert np.array_equal(mapped, full.col_src)
