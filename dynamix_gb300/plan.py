"""Host-side planning of the dense g2 pipeline.

* :class:`PackLayout` -- where each q-bin's pixels go in the packed operand
  matrix ``[T][packed_cols]``.  Bins are contiguous and padded to a multiple
  of 128 columns.  Packing modes: 0 = fp16 counts (<= 2048), 1 = fp16 high-byte
  and low-byte planes side by side (any uint16), 2 = e4m3 counts (<= 16, one
  byte per element).
* :func:`k_chunks` -- the K split of one Gram so that every fp32 partial sum
  is an integer below ``limit`` (2^24 by default): by Cauchy-Schwarz,
  ``|sum_k a(t,k) b(t',k)| <= sqrt(max_t sum a^2 * max_t' sum b^2)``, and the
  pack kernel reports ``max_t sum`` of squares per 64-column segment.
* :func:`gram_items` -- the upper-triangle item list (g2_gram_item records) for
  one job, LPT-ordered (longest K first) and, within a Gram, grouped in square
  super-tiles so that the CTAs running at the same time share operand rows in L2.

The per-bin arithmetic it plans is that of ``py_dense_correlator``
(dynamix/correlator/dense.py:48-64) with bins from ``BaseCorrelator._set_qmask``
(dynamix/correlator/common.py:36-46).
"""
from __future__ import annotations

import numpy as np

from ._lib import (BK, ITEM_DTYPE, ITEM_EMPTY, KIND_E4M3, KIND_FP16, PACK_CHUNK, PACK_MAX_PIECES, PACK_MAX_SLOTS,
                   PACK_WORDS_PER_CHUNK, PAD, PLAIN_BM, PLAIN_BN, TC_BM, TC_BN)

EXACT_LIMIT = 1 << 24   # fp32 represents every integer up to 2^24 exactly
FP16_MAX_EXACT = 2048   # fp16 represents every integer up to 2^11 exactly
E4M3_MAX_EXACT = 16     # e4m3 represents every integer up to 2^4 exactly
SUPER_ROWS = 2048       # frames per side of a super-tile

MODE_FP16, MODE_BYTES, MODE_E4M3 = 0, 1, 2
UNIT_NONE, UNIT_VEC, UNIT_WORD, UNIT_GATHER, UNIT_BYTE = 0, 1, 2, 3, 4   # classes of the e4m3 pack's units

# (rows, columns) of one Gram item per kernel: the single-CTA tensor-core
# block (g2_gram_tc), the CTA-pair blocks (g2_gram_tc_pair: 256 rows over two
# SMs; g2_gram_tc_wide: 256 x 512), and the CUDA-core comparators' blocks
PAIR_BM, PAIR_BN = 256, 256
TILE_SHAPES = {"tc": (TC_BM, TC_BN), "pair": (PAIR_BM, PAIR_BN), "wide": (PAIR_BM, 2 * PAIR_BN),
               "plain": (PLAIN_BM, PLAIN_BN), "dp4a": (PLAIN_BM, PLAIN_BN)}


def _roundup(x, m):
    return (x + m - 1) // m * m


class PackLayout:
    """Packed-column layout of the bins of one q-mask for one packing mode."""

    def __init__(self, qmask, n_bins, mode):
        qflat = np.ascontiguousarray(qmask, dtype=np.int32).ravel()
        qflat = np.where(qflat >= 1, qflat, 0)               # bins are 1..n_bins, the rest unused
        self.npix_total = qflat.size
        self.n_bins = int(n_bins)
        self.mode = int(mode)
        self.split = self.mode == MODE_BYTES
        self.kind = KIND_E4M3 if self.mode == MODE_E4M3 else KIND_FP16
        self.elem_bytes = 1 if self.mode == MODE_E4M3 else 2
        order = np.argsort(qflat, kind="stable")            # raster order within each bin
        counts = np.bincount(qflat, minlength=self.n_bins + 1)[: self.n_bins + 1]
        starts = np.concatenate([[0], np.cumsum(counts)])
        self.npix = counts[1:].astype(np.int64)               # P_b, b = 1..n_bins
        self.kpad = _roundup(self.npix, PAD)
        nseg_b = self.kpad // BK
        self.n_segs = int(nseg_b.sum())
        col_src = np.full(int(self.kpad.sum()), -1, dtype=np.int32)
        self.src_off = np.concatenate([[0], np.cumsum(self.kpad)])[:-1]
        for b in range(self.n_bins):
            pix = order[starts[b + 1]:starts[b + 2]]
            col_src[self.src_off[b]:self.src_off[b] + pix.size] = pix
        self.col_src = col_src
        self.seg_bin = np.repeat(np.arange(self.n_bins, dtype=np.int32), nseg_b)
        seg_local = np.arange(self.n_segs, dtype=np.int64) - np.repeat(self.src_off // BK, nseg_b)
        width = self.kpad * (2 if self.split else 1)
        self.bin_off = np.concatenate([[0], np.cumsum(width)])[:-1].astype(np.int64)
        self.packed_cols = int(max(PAD, width.sum()))
        # plane offsets (first packed column) per bin
        self.plane0 = self.bin_off.copy()                       # counts, or high bytes
        self.plane1 = self.bin_off + self.kpad if self.split else None  # low bytes
        self.seg_dst0 = (np.repeat(self.plane0, nseg_b) + seg_local * BK).astype(np.int32)
        if self.split:
            self.seg_dst1 = (np.repeat(self.plane1, nseg_b) + seg_local * BK).astype(np.int32)
        else:
            self.seg_dst1 = np.zeros(self.n_segs, dtype=np.int32)
        if self.packed_cols >= 2 ** 31:
            raise ValueError("too many binned pixels for one job")
        self._build_chunks(qflat, order, starts)

    def _build_chunks(self, qflat, order, starts):
        """Tables of the pack kernel: binned pixels per 2048-pixel chunk, their
        packed column, local bin slot and local piece (64-column output
        segment within the chunk)."""
        n = self.npix_total
        self.n_chunks = -(-n // PACK_CHUNK)
        pix = np.flatnonzero(qflat > 0).astype(np.int64)            # pixel order
        b = qflat[pix].astype(np.int64) - 1
        rank = np.empty(n, dtype=np.int64)                             # rank of a pixel inside its bin
        for bb in range(self.n_bins):
            seg = order[starts[bb + 1]:starts[bb + 2]]
            rank[seg] = np.arange(seg.size)
        dst = self.plane0[b] + rank[pix]
        chunk = pix // PACK_CHUNK
        self.chunk_entry_off = np.searchsorted(chunk, np.arange(self.n_chunks + 1)).astype(np.int32)
        # bin slots within a chunk
        key = chunk * (self.n_bins + 1) + b
        ukey = np.unique(key)
        ukey_chunk = ukey // (self.n_bins + 1)
        first_of_chunk = np.searchsorted(ukey_chunk, ukey_chunk)
        slot_of_key = np.arange(ukey.size) - first_of_chunk
        if slot_of_key.size and slot_of_key.max() >= PACK_MAX_SLOTS:
            raise ValueError("more than %d bins in one %d-pixel chunk" % (PACK_MAX_SLOTS, PACK_CHUNK))
        slot = slot_of_key[np.searchsorted(ukey, key)]
        self.chunk_slot_bin = np.full(self.n_chunks * PACK_MAX_SLOTS, -1, dtype=np.int32)
        self.chunk_slot_bin[ukey_chunk * PACK_MAX_SLOTS + slot_of_key] = (ukey % (self.n_bins + 1)).astype(np.int32)
        # pieces: (output segment, chunk)
        seg = dst // BK
        nseg = self.packed_cols // BK
        pkey = chunk * nseg + seg
        upkey = np.unique(pkey)
        up_chunk = upkey // nseg
        self.chunk_piece_off = np.searchsorted(up_chunk, np.arange(self.n_chunks + 1)).astype(np.int32)
        piece = np.searchsorted(upkey, pkey) - self.chunk_piece_off[chunk]
        if piece.size and piece.max() >= PACK_MAX_PIECES:
            raise ValueError("more than %d pieces in one chunk" % PACK_MAX_PIECES)
        self.n_pieces = int(upkey.size)
        self.piece_seg = (upkey % nseg).astype(np.int64)
        if self.split:
            piece_bin = np.empty(self.n_pieces, dtype=np.int64)          # bin of each piece
            piece_bin[np.searchsorted(upkey, pkey)] = b
            self.piece_seg1 = self.piece_seg + self.kpad[piece_bin] // BK
        self.entry_dst = dst.astype(np.int32)
        src_off = pix - chunk * PACK_CHUNK
        self.entry_meta = (src_off | (slot << 11) | (piece << 18)).astype(np.uint32)
        self.bin_kpad = self.kpad.astype(np.int32)
        self.n_planes = 2 if self.split else 1
        # words of the byte-permutation pack (e4m3): 4 aligned packed columns of
        # one bin (bins are 128-column aligned) with their 4 chunk-local sources
        if self.mode == MODE_E4M3:
            nq = self.packed_cols // 4
            wkey = chunk * nq + dst // 4
            uw, widx = np.unique(wkey, return_inverse=True)
            srcs = np.full((uw.size, 4), 0xFFF, dtype=np.int64)
            srcs[widx, dst % 4] = src_off
            wslot = np.zeros(uw.size, dtype=np.int64)
            wslot[widx] = slot
            wchunk = uw // nq
            self.chunk_word_off = np.searchsorted(wchunk, np.arange(self.n_chunks + 1)).astype(np.int32)
            if uw.size and np.diff(self.chunk_word_off).max() > PACK_WORDS_PER_CHUNK:
                raise ValueError("more than %d packed words in one chunk" % PACK_WORDS_PER_CHUNK)
            self.word_dst = ((uw % nq) * 4).astype(np.int32)
            ws = np.empty((uw.size, 2), dtype=np.uint32)
            ws[:, 0] = (srcs[:, 0] | (srcs[:, 1] << 12) | ((srcs[:, 2] & 0xFF) << 24)).astype(np.uint32)
            ws[:, 1] = ((srcs[:, 2] >> 8) | (srcs[:, 3] << 4) | (wslot << 16)).astype(np.uint32)
            self.word_src = ws
            self._build_units(dst, pix, chunk)

    def _build_units(self, dst, pix, chunk):
        """Work units of the u8 e4m3 pack (``g2_pack_e4m3_units``), per chunk
        in blocks of 32 of one class (a warp runs a block without diverging):
        UNIT_VEC 16 destination bytes from 16 consecutive source bytes (one
        16-byte store), UNIT_WORD 4 from 4 consecutive, UNIT_GATHER 4 from 4
        arbitrary source bytes of the chunk, UNIT_BYTE one byte (destination
        words shared with another chunk or with bin padding).  A unit is four
        uint32: destination (in units of its size), source offset(s) in the
        chunk, class."""
        n = self.packed_cols
        dchunk = np.full(n, -1, dtype=np.int64)
        dsrc = np.full(n, -1, dtype=np.int64)
        dchunk[dst] = chunk
        dsrc[dst] = pix - chunk * PACK_CHUNK
        nv, nw = n // 16, n // 4
        vc, vs = dchunk.reshape(nv, 16), dsrc.reshape(nv, 16)
        vec = (vc[:, 0] >= 0) & (vc == vc[:, :1]).all(1) & (np.diff(vs, axis=1) == 1).all(1)
        wc, ws = dchunk.reshape(nw, 4), dsrc.reshape(nw, 4)
        owned = (wc[:, 0] >= 0) & (wc == wc[:, :1]).all(1) & ~np.repeat(vec, 4)
        run = owned & (np.diff(ws, axis=1) == 1).all(1)
        gat = owned & ~run
        byte = (dchunk >= 0) & ~np.repeat(vec, 16) & ~np.repeat(owned, 4)
        classes = []
        iv = np.flatnonzero(vec)
        classes.append((vc[iv, 0], np.stack([iv, vs[iv, 0], np.zeros_like(iv), np.full_like(iv, UNIT_VEC)], 1)))
        iw = np.flatnonzero(run)
        classes.append((wc[iw, 0], np.stack([iw, ws[iw, 0], np.zeros_like(iw), np.full_like(iw, UNIT_WORD)], 1)))
        ig = np.flatnonzero(gat)
        g = ws[ig]
        classes.append((wc[ig, 0], np.stack([ig, g[:, 0] | (g[:, 1] << 16), g[:, 2] | (g[:, 3] << 16),
                                             np.full_like(ig, UNIT_GATHER)], 1)))
        ib = np.flatnonzero(byte)
        classes.append((dchunk[ib], np.stack([ib, dsrc[ib], np.zeros_like(ib), np.full_like(ib, UNIT_BYTE)], 1)))
        # blocks: per chunk, per class, groups of 32 units (the last one padded with UNIT_NONE)
        blocks_per_chunk = np.zeros(self.n_chunks, dtype=np.int64)
        per_class = []
        for ch, u in classes:
            order = np.argsort(ch, kind="stable")
            ch, u = ch[order], u[order]
            cnt = np.bincount(ch, minlength=self.n_chunks)
            nb = -(-cnt // 32)
            blocks_per_chunk += nb
            per_class.append((ch, u, cnt, nb))
        off = np.concatenate([[0], np.cumsum(blocks_per_chunk)])
        units = np.zeros((int(off[-1]) * 32, 4), dtype=np.uint32)
        units[:, 3] = UNIT_NONE
        nxt = off[:-1].copy()                      # next free block of each chunk
        for ch, u, cnt, nb in per_class:
            first = np.concatenate([[0], np.cumsum(cnt)])[:-1]
            rank = np.arange(ch.size) - first[ch]  # position of a unit inside its chunk's class list
            slot = (nxt[ch] * 32 + rank).astype(np.int64)
            units[slot] = u.astype(np.uint32)
            nxt += nb
        self.unit_block_off = off.astype(np.int32)
        self.units = units.reshape(-1)

    def segment_emax(self, piece_emax):
        """Per 64-column output segment, the sum over its pieces of the pieces'
        energy bounds (each bounds its piece's sum of squares in every frame):
        an upper bound of the segment's energy in every frame (indexed by
        packed column // 64)."""
        pe = np.asarray(piece_emax, dtype=np.float64)
        nseg = self.packed_cols // BK
        out = np.bincount(self.piece_seg, weights=pe[: self.n_pieces], minlength=nseg)
        if self.split:
            out += np.bincount(self.piece_seg1, weights=pe[self.n_pieces: 2 * self.n_pieces], minlength=nseg)
        return out

    @property
    def packed_bytes_per_frame(self):
        return self.packed_cols * self.elem_bytes

    @property
    def ones_row(self):
        """e4m3 jobs carry a row of ones after the last frame: the Gram turns
        it into the bin sums (G(t, ones) = S(t))."""
        return self.mode == MODE_E4M3

    def ones_row_values(self):
        """Row of ones: 1 in every binned column, 0 in the bin padding."""
        row = np.zeros(self.packed_cols, dtype=np.uint8 if self.elem_bytes == 1 else np.uint16)
        for b in range(self.n_bins):
            row[self.plane0[b]:self.plane0[b] + self.npix[b]] = 1
        return row

    def grams(self):
        """The Grams to run per bin: (bin, a_plane_off, b_plane_off, kpad, shift)."""
        out = []
        for b in range(self.n_bins):
            if self.kpad[b] == 0:
                continue
            kp = int(self.kpad[b])
            if not self.split:
                out.append((b, int(self.plane0[b]), int(self.plane0[b]), kp, 0))
            else:
                h, lo = int(self.plane0[b]), int(self.plane1[b])
                out.append((b, h, h, kp, 16))    # high x high, weight 2^16
                out.append((b, h, lo, kp, 8))    # high x low,  weight 2^8
                out.append((b, lo, h, kp, 8))    # low  x high, weight 2^8
                out.append((b, lo, lo, kp, 0))   # low  x low
        return out


def k_chunks(emax_a, emax_b, limit=EXACT_LIMIT):
    """Split a Gram's units into chunks with exact fp32 sums.

    ``emax_a[u]`` / ``emax_b[u]``: bound on the sum of squares of the A / B
    packed values of unit ``u`` over every frame.  A chunk ``[u0, u1)`` is valid
    when ``sum(emax_a) * sum(emax_b) <= limit^2`` (hence every partial sum of
    the dot products is <= limit).  A unit that alone exceeds the bound is
    infeasible (OverflowError).  Returns a list of ``(u0, u1)``.
    """
    ea = np.asarray(emax_a, dtype=np.float64)
    eb = np.asarray(emax_b, dtype=np.float64)
    n = ea.size
    lim2 = float(limit) * float(limit)
    if n and np.any(ea * eb > lim2):
        raise OverflowError("a packed unit exceeds the exact fp32 bound")
    if n and ea.sum() * eb.sum() <= lim2:
        return [(0, n)]
    # greedy: each chunk takes units while the product of its sums fits (the
    # sums are integers below 2^53, so prefix-sum differences are exact)
    sa = np.concatenate(([0.0], np.cumsum(ea)))
    sb = np.concatenate(([0.0], np.cumsum(eb)))
    chunks = []
    u0 = 0
    while u0 < n:
        over = np.flatnonzero((sa[u0 + 1:] - sa[u0]) * (sb[u0 + 1:] - sb[u0]) > lim2)
        u1 = n if over.size == 0 else u0 + int(over[0])
        chunks.append((u0, u1))
        u0 = u1
    return chunks


_TILE_CACHE = {}


def _tiles(T, bm, bn, super_rows=SUPER_ROWS, extra_col=False):
    """(i0, j0) of every bm x bn block holding some t' >= t (t, t' < T); with
    ``extra_col`` the columns run to T inclusive (the row of ones).

    Ordered by square super-tiles of ``super_rows`` frames per side (upper
    triangle, row-major), then row-major inside a super-tile."""
    key = (T, bm, bn, super_rows, extra_col)
    if key not in _TILE_CACHE:
        ni = -(-T // bm)
        nj = -(-(T + (1 if extra_col else 0)) // bn)
        ii, jj = np.meshgrid(np.arange(ni), np.arange(nj), indexing="ij")
        i0 = (ii * bm).ravel()
        j0 = (jj * bn).ravel()
        keep = j0 + bn - 1 >= i0
        i0, j0 = i0[keep], j0[keep]
        order = np.lexsort((j0, i0, j0 // super_rows, i0 // super_rows))
        _TILE_CACHE[key] = (i0[order].astype(np.int32), j0[order].astype(np.int32))
    return _TILE_CACHE[key]


def gram_items(T, chunked_grams, job=0, out_base=0, kind="tc", s_base=None, super_rows=SUPER_ROWS):
    """Build the item list of one job.

    ``chunked_grams``: iterable of ``(bin, a_off, b_off, k0, k_len, shift)`` with
    columns relative to the job's packed matrix.  ``kind`` selects the block
    shape (:data:`TILE_SHAPES`: single-CTA tensor-core 128x256, CTA-pair
    256x256, CUDA-core 128x128).  Items are sorted by k_len
    (descending, stable) so that the persistent kernel's static round-robin
    schedule starts with the longest items.  ``s_base`` (tensor-core items of a
    job whose packed matrix carries the row of ones): element offset of the
    job's bin sums; the blocks then also cover that row and add S_b(t) at
    ``s_base + b * T + t``.
    """
    bm, bn = TILE_SHAPES[kind]
    i0, j0 = _tiles(int(T), bm, bn, super_rows=int(super_rows), extra_col=s_base is not None)
    parts = []
    for (b, a_off, b_off, k0, klen, shift) in chunked_grams:
        it = np.empty(i0.size, dtype=ITEM_DTYPE)
        it["job"] = job
        it["i0"] = i0
        it["j0"] = j0
        it["a_k0"] = a_off + k0
        it["b_k0"] = b_off + k0
        it["k_len"] = klen
        it["shift"] = shift
        it["nframes"] = T
        it["out_off"] = out_base + b * T
        it["s_off"] = -1 if s_base is None else s_base + b * T
        parts.append(it)
    if not parts:
        return np.empty(0, dtype=ITEM_DTYPE)
    items = np.concatenate(parts)
    order = np.argsort(-items["k_len"].astype(np.int64), kind="stable")
    return items[order]


ITEM_OVERHEAD_STAGES = 4   # fixed cost of an item (descriptor, epilogue hand-off), in full-width stages


def item_costs(items, stage_elems, kind, ones=True):
    """Relative tensor-core time of each item: its K stages times the share
    of a full-width MMA its columns take, plus a fixed per-item cost.  Pair
    items use n = min(256, frames (+ row of ones) left from j0, rounded up to
    32) columns (g2_gram_tc_pair), wide items two such halves, the left one
    skipped below the diagonal, and an epilogue that is not overlapped
    (g2_gram_tc_wide); single-CTA items always 256."""
    bn = TILE_SHAPES[kind][1]
    stages = items["k_len"].astype(np.float64) / float(stage_elems)
    if kind in ("pair", "wide"):
        live = items["nframes"].astype(np.int64) - items["j0"].astype(np.int64)
        if ones:
            live = live + (items["s_off"] >= 0)
        r = (live + 31) // 32 * 32
        if kind == "pair":
            n = np.clip(r, 32, bn)
        else:
            n0 = np.where(items["j0"].astype(np.int64) + PAIR_BN <= items["i0"], 0, np.clip(r, 32, PAIR_BN))
            n1 = np.clip(r - PAIR_BN, 0, PAIR_BN)
            n = n0 + n1
            return stages * (n / float(bn)) + ITEM_OVERHEAD_STAGES + n / 64.0
        stages = stages * (n / float(bn))
    return stages + ITEM_OVERHEAD_STAGES


def balance_items(items, workers, stage_elems, kind, ones=True):
    """Static longest-first list schedule of one launch's items over
    ``workers`` persistent workers (CTAs, or CTA pairs for "pair" items):
    each item, largest cost first, goes to the least-loaded worker, and the
    list is laid out so that worker w reads slots w, w + workers, ... (the
    kernels' pattern), unused slots holding ``job = G2_ITEM_EMPTY``.  Items
    keep their relative order within a worker (bins and super-tiles stay
    together in time)."""
    n = items.size
    if workers <= 1 or n <= workers:
        return items
    cost = np.ascontiguousarray(item_costs(items, stage_elems, kind, ones), dtype=np.float64)
    slots, n_slots = lpt_slots(cost, workers)
    out = np.zeros(n_slots, dtype=ITEM_DTYPE)
    out["job"] = ITEM_EMPTY
    out[slots] = items
    return out


def lpt_slots(cost, workers):
    """Slot of every item in the longest-first schedule of
    :func:`balance_items`, and the slot count: the library's
    ``g2_balance_lpt`` (microseconds for ten thousand items), or the same
    schedule in Python where the library is not built (planning on a host
    without the toolkit)."""
    import ctypes as C
    n = int(cost.size)
    try:
        from . import _lib
        lib = _lib.load()
    except ImportError:
        lib = None
    if lib is not None:
        slots = np.empty(n, dtype=np.int64)
        n_slots = C.c_int64(0)
        _lib.check(lib.g2_balance_lpt(cost.ctypes.data_as(C.c_void_p), n, int(workers),
                                      slots.ctypes.data_as(C.c_void_p), C.byref(n_slots)), "g2_balance_lpt")
        return slots, int(n_slots.value)
    return lpt_slots_py(cost, workers)


def lpt_slots_py(cost, workers):
    """:func:`lpt_slots` in Python (a heap of worker loads)."""
    import heapq
    order = np.argsort(-cost, kind="stable")
    heap = [(0.0, w) for w in range(workers)]
    owner = np.empty(cost.size, dtype=np.int64)
    for i in order:
        load, w = heapq.heappop(heap)
        owner[i] = w
        heapq.heappush(heap, (load + float(cost[i]), w))
    slots = np.empty(cost.size, dtype=np.int64)
    nxt = np.zeros(workers, dtype=np.int64)
    for i in range(cost.size):
        w = owner[i]
        slots[i] = w + nxt[w] * workers
        nxt[w] += 1
    return slots, int(nxt.max()) * workers


def chunk_grams(layout, seg_emax, limit=EXACT_LIMIT, kslab=0):
    """Apply :func:`k_chunks` to every Gram of a layout, in units of PAD columns.

    ``seg_emax`` is indexed by packed column // 64.  ``kslab`` > 0 also caps
    every chunk at that many columns (rounded down to PAD): the tiles that run
    at the same time then share a narrower slab of K in L2.  Returns the list
    of ``(bin, a_off, b_off, k0, k_len, shift)``."""
    per = PAD // BK
    cap = max(1, int(kslab) // PAD) if kslab else 0
    out = []
    for (b, a_off, b_off, kp, shift) in layout.grams():
        nseg = kp // BK
        ea = np.asarray(seg_emax[a_off // BK: a_off // BK + nseg], dtype=np.float64).reshape(-1, per).sum(1)
        eb = np.asarray(seg_emax[b_off // BK: b_off // BK + nseg], dtype=np.float64).reshape(-1, per).sum(1)
        for (u0, u1) in k_chunks(ea, eb, limit):
            step = cap if cap else u1 - u0
            for v0 in range(u0, u1, step):
                v1 = min(u1, v0 + step)
                out.append((b, a_off, b_off, v0 * PAD, (v1 - v0) * PAD, shift))
    return out


def column_window(qmask2d, n_bins, min_saving, min_gap=192):
    """(first column, width) of the smallest column window holding every
    binned pixel of a (H, W) q-mask, widened to 16-byte multiples of a u8 row
    (16-byte aligned host reads), or None when nothing is binned or the window
    leaves less than ``min_saving`` of the row, or less than ``min_gap``
    bytes, out.  (Row-by-row host-to-device copies whose rows skip only a
    short gap ran far below the link rate: 27-81 GB/s at 928 to 1024 of 1030
    bytes and at 2048 of 2068, against 198-206 GB/s for windows of at most
    896 of 1030 and 1856 of 2068.)"""
    q = np.asarray(qmask2d)
    W = q.shape[1]
    cols = np.flatnonzero(((q >= 1) & (q <= n_bins)).any(axis=0))
    if cols.size == 0:
        return None
    c0 = int(cols[0]) // 16 * 16
    c1 = min(W, -(-(int(cols[-1]) + 1) // 16) * 16)
    if c1 - c0 > (1.0 - float(min_saving)) * W or W - (c1 - c0) < int(min_gap):
        return None
    return c0, c1 - c0


def e4m3_segment_bound(layout):
    """Energy bound per 64-column segment for e4m3 operands without looking at
    the data: every count is <= 16, so a segment's sum of squares is <= 64 * 256
    (a Gram chunk of up to 65,536 columns stays below 2^24)."""
    return np.full(layout.packed_cols // BK, BK * E4M3_MAX_EXACT ** 2, dtype=np.float64)


def gram_macs(T, npix):
    """Algorithmic multiply-accumulates of the upper-triangle Grams (incl. diagonal)."""
    return int(np.sum(np.asarray(npix, dtype=np.int64))) * T * (T + 1) // 2


def std_items(T, layout, npix, job=0):
    """Items of the calc_std pass (``g2_gram_std``): for every bin one Gram
    over its whole K (the deviation is a float statistic, so K is not split),
    tiles of the upper triangle, ``shift`` = the bin's pixel count and
    ``out_off`` = ``s_off`` = bin * T.  Needs a layout without byte planes."""
    if layout.split:
        raise ValueError("calc_std needs counts <= 2048 (no byte planes)")
    i0, j0 = _tiles(int(T), TC_BM, TC_BN)
    parts = []
    for b in range(layout.n_bins):
        kp = int(layout.kpad[b])
        if kp == 0 or int(npix[b]) == 0:
            continue
        it = np.empty(i0.size, dtype=ITEM_DTYPE)
        it["job"] = job
        it["i0"] = i0
        it["j0"] = j0
        it["a_k0"] = int(layout.plane0[b])
        it["b_k0"] = int(layout.plane0[b])
        it["k_len"] = kp
        it["shift"] = int(npix[b])
        it["nframes"] = T
        it["out_off"] = b * T
        it["s_off"] = b * T
        parts.append(it)
    if not parts:
        return np.empty(0, dtype=ITEM_DTYPE)
    items = np.concatenate(parts)
    return items[np.argsort(-items["k_len"].astype(np.int64), kind="stable")]
