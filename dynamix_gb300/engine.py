"""Device pipelines behind the correlator classes.

PyTorch only owns device memory and the CUDA stream; all arithmetic runs in
the hand-written sm_103a kernels of ``libdynamix_g2.so`` (C ABI in
``include/dynamix_g2.h``).  There is no CPU path: constructing an engine
without a CUDA device or without the built library raises.

Dense pipeline (one job = one frame stack, all its q-bins):

    G1 pack + bin sums   -> packed fp16 operand [T][cols], S (int64), segment energies
       (host: K split from the segment energies, item list; cached)
    G2 tensor-core Gram  -> N (int64), or G5 plain direct kernel (comparator)
    G3 denominator       -> D (int64)
    G4 finalize          -> g2 (float32 and float64)
"""
from __future__ import annotations

import collections
import ctypes as C
import hashlib
import threading

import numpy as np

from . import _lib
from .plan import (E4M3_MAX_EXACT, EXACT_LIMIT, FP16_MAX_EXACT, MODE_BYTES, MODE_E4M3, MODE_FP16, TILE_SHAPES,
                   PackLayout, balance_items, chunk_grams, column_window, e4m3_segment_bound, gram_items)


def _torch():
    import torch
    return torch


def require_cuda(device=None):
    torch = _torch()
    if not torch.cuda.is_available():
        raise RuntimeError("dynamix_gb300 needs a CUDA device (sm_103); none is available")
    dev = torch.device(device if device is not None else "cuda")
    if dev.type != "cuda":
        raise ValueError("device must be a CUDA device")
    if dev.index is None:
        dev = torch.device("cuda", torch.cuda.current_device())
    return dev


def ptr(t):
    return C.c_void_p(t.data_ptr())


def stream_handle(dev):
    return C.c_void_p(_torch().cuda.current_stream(dev).cuda_stream)


class DeviceError(RuntimeError):
    pass


def frames_to_device(frames, dev):
    """Validate a (T, H, W) stack of non-negative integer counts and return a
    contiguous uint8 / uint16 device tensor.

    numpy arrays and CPU tensors are copied (asynchronously when pinned);
    device tensors of a supported dtype are used in place."""
    torch = _torch()
    if isinstance(frames, torch.Tensor):
        t = frames
        if t.dtype in (torch.uint8, torch.uint16):
            t = t.to(dev, non_blocking=True).contiguous()
            if t.data_ptr() % 16:
                t = t.clone()          # the pack kernel reads 16-byte aligned words
            return t
        frames = t.cpu().numpy()
    a = np.asarray(frames)
    if a.dtype == np.uint8 or a.dtype == np.uint16:
        host = torch.from_numpy(np.ascontiguousarray(a))
        return host.to(dev, non_blocking=False)
    if a.dtype.kind not in "iuf":
        raise TypeError("frames must hold integer photon counts")
    if a.size:
        if a.dtype.kind == "f" and not np.all(np.isfinite(a) & (a == np.round(a))):
            raise TypeError("float frames must hold integer counts")
        lo, hi = a.min(), a.max()
        if lo < 0:
            raise ValueError("counts must be non-negative")
        if hi > 65535:
            raise ValueError("counts above 65535 are not supported")
    tgt = np.uint8 if (a.size == 0 or a.max() <= 255) else np.uint16
    return torch.from_numpy(np.ascontiguousarray(a.astype(tgt))).to(dev)


_WORKERS = {}
_LAYOUTS = collections.OrderedDict()
_LAYOUTS_LOCK = threading.Lock()
_LAYOUTS_MAX = 48


def qmask_digest(qmask):
    q = np.ascontiguousarray(qmask, dtype=np.int32)
    return "%s:%s" % (q.shape, hashlib.blake2b(q.tobytes(), digest_size=16).hexdigest())


def device_layout(qmask, n_bins, mode, dev, digest=None):
    """The packing layout of a q-mask with its read-only tables on ``dev``,
    shared process-wide (least recently used of 48 kept): building one costs
    host time proportional to the frame size.  ``digest``: the q-mask's
    :func:`qmask_digest` when the caller has it."""
    torch = _torch()
    q = np.ascontiguousarray(qmask, dtype=np.int32)
    key = (str(dev), digest or qmask_digest(q), int(n_bins), int(mode))
    with _LAYOUTS_LOCK:
        L = _LAYOUTS.get(key)
        if L is not None:
            _LAYOUTS.move_to_end(key)
            return L
    L = PackLayout(q, n_bins, mode)
    d = lambda a: torch.as_tensor(a, device=dev)
    L.d_col_src = d(L.col_src)
    L.d_chunk_entry_off = d(L.chunk_entry_off)
    L.d_entry_dst = d(L.entry_dst)
    L.d_entry_meta = d(L.entry_meta.view(np.int32))
    L.d_chunk_slot_bin = d(L.chunk_slot_bin)
    L.d_chunk_piece_off = d(L.chunk_piece_off)
    L.d_bin_kpad = d(L.bin_kpad)
    if mode == MODE_E4M3:
        L.d_chunk_word_off = d(L.chunk_word_off)
        L.d_word_dst = d(L.word_dst)
        L.d_word_src = d(L.word_src.view(np.int32))
        L.d_unit_block_off = d(L.unit_block_off)
        L.d_units = d(L.units.view(np.int32))
    with _LAYOUTS_LOCK:
        _LAYOUTS[key] = L
        while len(_LAYOUTS) > _LAYOUTS_MAX:
            _LAYOUTS.popitem(last=False)
    return L


class DenseEngine:
    """Exact g2 of a dense (T, H, W) stack for the bins of one q-mask.

    ``operand`` selects the packed element type of the tensor-core Gram:
    ``"auto"`` (e4m3 when every binned count is <= 16, else fp16 counts when
    <= 2048, else fp16 byte planes), or one of ``"e4m3"``, ``"fp16"``,
    ``"bytes"``.  The plain comparator always uses fp16.

    ``tile`` selects the tensor-core kernel: ``"pair"`` (256 x 256 blocks on
    CTA pairs, g2_gram_tc_pair), ``"wide"`` (256 x 512 blocks on CTA pairs,
    g2_gram_tc_wide: fewer bytes per MMA, epilogue not overlapped) or
    ``"single"`` (128 x 256 blocks, one CTA each, g2_gram_tc)."""

    MODES = {"fp16": MODE_FP16, "bytes": MODE_BYTES, "e4m3": MODE_E4M3}

    def __init__(self, shape, nframes, qmask, n_bins, scale, device=None, method="tc",
                 exact_limit=EXACT_LIMIT, grid=0, operand="auto", numer=None, sums=None, layouts=None,
                 qmask_digest=None, tile=None):
        torch = _torch()
        self.lib = _lib.load()
        self.dev = require_cuda(device)
        self.shape = tuple(int(s) for s in shape)
        self.T = int(nframes)
        self.npix = self.shape[0] * self.shape[1]
        self.qmask = np.ascontiguousarray(qmask, dtype=np.int32)
        self.n_bins = int(n_bins)
        self.crop = self._column_window()
        if method not in ("tc", "plain", "dp4a"):
            raise ValueError("method must be 'tc', 'plain' or 'dp4a'")
        if operand != "auto" and operand not in self.MODES:
            raise ValueError("operand must be 'auto', 'e4m3', 'fp16' or 'bytes'")
        if method == "plain" and operand == "e4m3":
            raise ValueError("the plain kernel reads fp16 operands")
        if method == "dp4a" and operand not in ("auto", "e4m3"):
            raise ValueError("the dp4a kernel reads the raw u8 counts (the e4m3 packing)")
        self.method = method
        self.operand = operand
        tile = self.TILE if tile is None else tile
        if tile not in ("pair", "single", "wide"):
            raise ValueError("tile must be 'pair', 'wide' or 'single'")
        self.tile = tile
        self.exact_limit = int(exact_limit)
        self.grid = int(grid)
        self.scale = torch.as_tensor(np.asarray(scale, dtype=np.float64), device=self.dev)
        rows = max(self.n_bins, 1)
        z = lambda dt: torch.zeros((rows, self.T), dtype=dt, device=self.dev)
        # N and S may be views into a caller's arena (grouped launches address
        # several jobs' sums through one base pointer)
        self.sums = z(torch.int64) if sums is None else sums
        self.numer = z(torch.int64) if numer is None else numer
        self.denom = z(torch.int64)
        self.g2_f32 = z(torch.float32)
        self.g2_f64 = z(torch.float64)
        self.err = torch.zeros(1, dtype=torch.int32, device=self.dev)
        self.maxval = torch.zeros(1, dtype=torch.int32, device=self.dev)
        self._layouts = {} if layouts is None else layouts   # may be shared by engines of one q-mask
        self._qdigest = qmask_digest
        self._items_cache = {}
        self.packed = None
        self.last = {}
        self._u8_hint = MODE_E4M3 if method == "tc" else MODE_FP16
        self._u16_hint = MODE_E4M3 if method == "tc" else MODE_FP16
        self.operand_hint = "auto"
        self._packed_mode = None
        self.pipeline = True      # chunked copy/pack/Gram overlap where it applies
        self.pipe_chunks = self.PIPE_CHUNKS
        self.pipe_chunks_host = self.PIPE_CHUNKS_HOST
        self.pipe_growth = self.PIPE_GROWTH
        self.pipe_gram_streams = self.PIPE_GRAM_STREAMS
        self.super_rows = self.SUPER_ROWS
        self.kslab = self.KSLAB
        from .tune import apply_cached
        apply_cached(self)        # launch shapes an earlier tuning run chose for this (T, pixels per bin)
        self.profile = False      # record CUDA events around every stage
        self.stage_ms = {}
        self._events = []

    def set_operand_hint(self, operand):
        """The packed operand kind the next call tries first (tensor-core
        path, ``operand="auto"``): "e4m3", "fp16", "bytes" or "auto" (the
        narrowest)."""
        if operand not in ("auto", "e4m3", "fp16", "bytes"):
            raise ValueError("operand hint must be 'auto', 'e4m3', 'fp16' or 'bytes'")
        self.operand_hint = operand
        if self.method != "tc" or self.operand != "auto":
            return
        mode = MODE_E4M3 if operand == "auto" else self.MODES[operand]
        self._u8_hint = mode if mode != MODE_BYTES else MODE_FP16
        self._u16_hint = mode

    def _mark(self, name):
        if self.profile:
            torch = _torch()
            ev = torch.cuda.Event(enable_timing=True)
            ev.record(torch.cuda.current_stream(self.dev))
            self._events.append((name, ev))

    def take_events(self):
        """Hand over the stage events of the last run (no synchronisation)."""
        ev, self._events = self._events, []
        return ev

    def _tmark(self, name, stream):
        """A CUDA event on ``stream`` for the pipeline timeline (profile mode)."""
        if self.profile:
            torch = _torch()
            ev = torch.cuda.Event(enable_timing=True)
            ev.record(stream)
            self._timeline.append((name, ev))

    def take_timeline(self):
        """Milliseconds from the start of the last pipelined run (profile mode)
        to each recorded point: ``pack<c>``/``pack<c>_end`` on the pack stream,
        ``gram<c>``/``gram<c>_end`` on the chunk's Gram stream (the first when
        the launch may begin), ``normalise``, ``end``.  Synchronises."""
        tl, self._timeline = getattr(self, "_timeline", []), []
        if not tl:
            return {}
        tl[-1][1].synchronize()
        t0 = tl[0][1]
        return {name: t0.elapsed_time(ev) for name, ev in tl}

    @staticmethod
    def stage_times(events):
        """Milliseconds per stage from a list of (name, event); synchronises."""
        out = {}
        if len(events) >= 2:
            events[-1][1].synchronize()
            for (n0, e0), (_, e1) in zip(events[:-1], events[1:]):
                out[n0] = out.get(n0, 0.0) + e0.elapsed_time(e1)
        return out

    # -- layout / buffers ------------------------------------------------
    # Frames copied in from host memory cross the host link cropped to the
    # q-mask's bounding columns (widened to 16-byte multiples) when that saves
    # at least CROP_MIN_SAVING of the bytes (see plan.column_window): the
    # packed operand is the same (the binned pixels keep their raster order),
    # and the link (about 200 GB/s) sets the pace of such a call.  Measured on
    # the 514 x 1030 detector with annuli r 20-400: columns 112..927, 0.79 of
    # the bytes, one 2-D copy per frame chunk at 198-200 GB/s of copied bytes
    # against 211 GB/s for whole frames: 27.5 -> 24.2 ms per call.
    CROP_MIN_SAVING = 0.15

    def _column_window(self):
        """(first column, width) of the cropped host copies of u8 frames, or
        None when the q-mask's binned columns span nearly the whole frame."""
        return column_window(self.qmask.reshape(self.shape), self.n_bins, self.CROP_MIN_SAVING)

    def _crop_layout(self, mode):
        """The packing layout of the cropped frames (:meth:`_column_window`)."""
        key = ("crop", mode)
        if key not in self._layouts:
            c0, wc = self.crop
            q = np.ascontiguousarray(self.qmask.reshape(self.shape)[:, c0:c0 + wc])
            self._layouts[key] = device_layout(q, self.n_bins, mode, self.dev)
        return self._layouts[key]

    def _layout(self, mode):
        if mode not in self._layouts:
            if getattr(self, "_qdigest", None) is None:
                self._qdigest = qmask_digest(self.qmask)
            self._layouts[mode] = device_layout(self.qmask, self.n_bins, mode, self.dev, self._qdigest)
        return self._layouts[mode]

    def _piece_emax(self, L):
        """This engine's buffer of per-piece energy maxima for layout L (the
        layout itself may be shared by other engines)."""
        torch = _torch()
        bufs = self.__dict__.setdefault("_emax_bufs", {})
        n = max(1, L.n_pieces * 2)  # two planes (g2_pack_frames)
        if L.mode not in bufs or bufs[L.mode].numel() < n:
            bufs[L.mode] = torch.zeros(n, dtype=torch.int32, device=self.dev)
        return bufs[L.mode]

    def ones(self, L):
        """Whether the packed operand of layout L carries the row of ones after
        the frames, from which the tensor-core Gram takes the bin sums: e4m3
        operands always, fp16 operands on the tensor-core path (the fp16 bit
        pattern 1 is 2^-24, the scale of the counts; the pack then skips its
        sum reduction).  Byte planes and the plain kernel get the sums from
        the pack."""
        return bool(L.ones_row or (L.mode == MODE_FP16 and self.method == "tc"))

    def _packed_buffer(self, L):
        """The packed operand buffer, [T (+1)][packed_cols]; zeroed whenever its
        layout changes, since the pack kernels write only the binned columns
        (padding stays 0).  Layouts with :meth:`ones` get the row of ones after
        the frames."""
        torch = _torch()
        ones = self.ones(L)
        rows = self.T + (1 if ones else 0)
        nbytes = rows * L.packed_bytes_per_frame
        fresh = False
        if self.packed is None or self.packed.numel() < nbytes:
            self.packed = None
            self.packed = torch.zeros(nbytes, dtype=torch.uint8, device=self.dev)
            fresh = True
        elif self._packed_mode != L.mode:
            self.packed.zero_()
            fresh = True
        if fresh:
            self._packed_mode = L.mode
            if ones:
                row = torch.from_numpy(L.ones_row_values().view(np.uint8)).to(self.dev)
                off = self.T * L.packed_bytes_per_frame
                self.packed[off:off + row.numel()].copy_(row)
        return self.packed

    # -- stages ----------------------------------------------------------
    def _binned_max(self, frames_dev, cropped=False):
        L0 = self._crop_layout(MODE_FP16) if cropped else self._layout(MODE_FP16)
        npix = self.shape[0] * self.crop[1] if cropped else self.npix
        self.maxval.zero_()
        _lib.check(self.lib.g2_binned_max(ptr(frames_dev), frames_dev.element_size(), self.T, npix,
                                          ptr(L0.d_col_src), L0.col_src.size, ptr(self.maxval),
                                          stream_handle(self.dev)), "g2_binned_max")
        return int(self.maxval.item())

    def choose_mode(self, frames_dev):
        if self.operand != "auto":
            return self.MODES[self.operand]
        # start from the narrowest operand the last stack of this width needed;
        # the pack kernels flag counts that do not fit and the step reruns wider
        return self._u8_hint if frames_dev.element_size() == 1 else self._u16_hint

    def pack_fp16_frames(self, frames_ptr, elem_bytes, nframes, L, packed_ptr, emax, stream):
        """One launch of the fp16 pack (with the row of ones: no bin sums)
        over ``nframes`` frames at ``frames_ptr`` into the packed rows at
        ``packed_ptr``; the energy maxima are combined into ``emax``."""
        _lib.check(self.lib.g2_pack_frames(
            C.c_void_p(frames_ptr), elem_bytes, nframes, self.npix, ptr(L.d_chunk_entry_off), ptr(L.d_entry_dst),
            ptr(L.d_entry_meta), ptr(L.d_chunk_slot_bin), ptr(L.d_chunk_piece_off), ptr(L.d_bin_kpad), L.n_chunks,
            MODE_FP16, C.c_void_p(packed_ptr), L.packed_cols, None, self.n_bins, ptr(emax), L.n_pieces,
            ptr(self.err), stream if isinstance(stream, C.c_void_p) else C.c_void_p(stream)), "g2_pack_frames")

    def pack(self, frames_dev, mode):
        L = self._layout(mode)
        packed = self._packed_buffer(L)
        self.sums.zero_()
        emax = self._piece_emax(L)
        emax.zero_()
        self.err.zero_()
        st = stream_handle(self.dev)
        if mode == MODE_E4M3:
            self.pack_e4m3(frames_dev.data_ptr(), frames_dev.element_size(), self.T, L, packed.data_ptr(), st)
            return L
        _lib.check(self.lib.g2_pack_frames(
            ptr(frames_dev), frames_dev.element_size(), self.T, self.npix, ptr(L.d_chunk_entry_off),
            ptr(L.d_entry_dst), ptr(L.d_entry_meta), ptr(L.d_chunk_slot_bin), ptr(L.d_chunk_piece_off),
            ptr(L.d_bin_kpad), L.n_chunks, mode, ptr(packed), L.packed_cols, None if self.ones(L) else ptr(self.sums),
            self.n_bins, ptr(emax), L.n_pieces, ptr(self.err), st), "g2_pack_frames")
        return L

    @property
    def item_kind(self):
        """The planner's block kind of this engine's numerator kernel."""
        if self.method == "tc":
            return {"pair": "pair", "wide": "wide"}.get(self.tile, "tc")
        return self.method

    def workers(self):
        """Persistent workers of a tensor-core Gram launch (CTAs, or CTA pairs
        for the pair tile), as the kernel will use them."""
        pair = {"pair": 1, "wide": 2}.get(self.tile, 0)
        if self.grid > 0:
            return (self.grid + 1) // 2 if pair else self.grid
        key = (str(self.dev), pair)
        if key not in _WORKERS:
            n = C.c_int32(0)
            _lib.check(self.lib.g2_gram_workers(pair, C.byref(n)), "g2_gram_workers")
            _WORKERS[key] = int(n.value)
        return _WORKERS[key]

    def balanced(self, items, L):
        """``items`` laid out for the kernel's workers, longest-first balanced
        (tensor-core launches only)."""
        if self.method != "tc" or items.size == 0:
            return items
        return balance_items(items, self.workers(), 128 if L.kind == _lib.KIND_E4M3 else 64, self.item_kind,
                             ones=self.ones(L))

    pack_units = True         # u8 e4m3 packing by work units (g2_pack_e4m3_units)

    def pack_e4m3(self, frames_ptr, elem_bytes, nframes, L, packed_ptr, stream, npix=None):
        """One launch of the e4m3 pack over ``nframes`` frames of ``npix``
        pixels (default: the engine's frame) at ``frames_ptr`` into the packed
        rows at ``packed_ptr``."""
        st = stream if isinstance(stream, C.c_void_p) else C.c_void_p(stream)
        npix = self.npix if npix is None else int(npix)
        if elem_bytes == 1 and self.pack_units:
            _lib.check(self.lib.g2_pack_e4m3_units(
                C.c_void_p(frames_ptr), nframes, npix, ptr(L.d_unit_block_off), ptr(L.d_units), L.n_chunks,
                C.c_void_p(packed_ptr), L.packed_cols, ptr(self.err), st), "g2_pack_e4m3_units")
        else:
            _lib.check(self.lib.g2_pack_e4m3(
                C.c_void_p(frames_ptr), elem_bytes, nframes, npix, ptr(L.d_chunk_word_off), ptr(L.d_word_dst),
                ptr(L.d_word_src), L.n_chunks, C.c_void_p(packed_ptr), L.packed_cols, ptr(self.err), st),
                "g2_pack_e4m3")

    def resolve_range_check(self, code, frames_dev, cropped=False):
        """An e4m3 pack that could not tell whether every count fits sets
        DEVERR_RANGE_CHECK: the exact binned maximum of ``frames_dev`` (frames
        cropped to :meth:`_column_window` with ``cropped``) decides
        (DEVERR_RANGE when a count exceeds 16).  Returns the resolved code."""
        if not code & _lib.DEVERR_RANGE_CHECK:
            return code
        code &= ~_lib.DEVERR_RANGE_CHECK
        if self._binned_max(frames_dev, cropped) > E4M3_MAX_EXACT:
            code |= _lib.DEVERR_RANGE
        self.err.fill_(code)
        return code

    def items_for(self, L, grams):
        key = (L.mode, self.item_kind, tuple(grams), self.super_rows, self.grid)
        if key not in self._items_cache:
            torch = _torch()
            items = gram_items(self.T, grams, job=0, out_base=0, kind=self.item_kind,
                               s_base=0 if (self.ones(L) and self.method in ("tc", "dp4a")) else None,
                               super_rows=self.super_rows)
            items = self.balanced(items, L)
            dev_items = torch.from_numpy(items.view(np.uint8).copy()).to(self.dev)
            if len(self._items_cache) > 8:
                self._items_cache.clear()
            self._items_cache[key] = (items, dev_items, len(grams))
        return self._items_cache[key]

    def numerator(self, L, items_dev, n_items):
        self.numer.zero_()
        jobs = _lib.jobs_array([(self.packed.data_ptr(), self.T, L.packed_cols, L.kind, self.ones(L))])
        st = stream_handle(self.dev)
        if self.method == "tc":
            self.gram_launch(jobs, items_dev.data_ptr(), n_items, st)
        elif self.method == "dp4a":
            _lib.check(self.lib.g2_plain_dp4a(jobs, 1, ptr(items_dev), n_items, ptr(self.numer),
                                              self.numer.numel(), ptr(self.sums), self.sums.numel(), ptr(self.err),
                                              st), "g2_plain_dp4a")
        else:
            _lib.check(self.lib.g2_plain_direct(jobs, 1, ptr(items_dev), n_items, ptr(self.numer),
                                                self.numer.numel(), ptr(self.err), st), "g2_plain_direct")

    def gram_launch(self, jobs, items_ptr, n_items, stream):
        """One launch of the tensor-core Gram kernel this engine's tile selects."""
        fn, name = {"pair": (self.lib.g2_gram_tc_pair, "g2_gram_tc_pair"),
                    "wide": (self.lib.g2_gram_tc_wide, "g2_gram_tc_wide")}.get(
                        self.tile, (self.lib.g2_gram_tc, "g2_gram_tc"))
        _lib.check(fn(jobs, 1, C.c_void_p(items_ptr), n_items, ptr(self.numer), self.numer.numel(), ptr(self.sums),
                      self.sums.numel(), ptr(self.err), self.grid,
                      stream if isinstance(stream, C.c_void_p) else C.c_void_p(stream)), name)

    def normalise(self):
        st = stream_handle(self.dev)
        if self.n_bins == 0:
            return
        _lib.check(self.lib.g2_denominator(ptr(self.sums), self.n_bins, self.T, ptr(self.denom), st),
                   "g2_denominator")
        _lib.check(self.lib.g2_finalize(ptr(self.numer), ptr(self.denom), ptr(self.scale), self.n_bins, self.T,
                                        ptr(self.g2_f32), ptr(self.g2_f64), st), "g2_finalize")

    def check_error(self):
        code = int(self.err.item())
        if code:
            raise DeviceError(_lib.device_error_message(code))

    def _pack_and_plan(self, frames_dev, mode):
        """Pack, read the segment energies and the error word (one sync), plan
        the K split; fall back to a wider packing when the counts do not fit."""
        while True:
            L = self.pack(frames_dev, mode)
            if mode == MODE_E4M3:
                seg_emax = e4m3_segment_bound(L)          # counts <= 16 bound every sum
            else:
                pe = self._piece_emax(L).cpu().numpy().view(np.uint32)
                seg_emax = L.segment_emax(pe)
            code = int(self.err.item())
            if mode == MODE_E4M3:
                code = self.resolve_range_check(code, frames_dev)
            wide = frames_dev.element_size() == 2
            if code & _lib.DEVERR_RANGE and mode == MODE_E4M3 and self.operand == "auto":
                mode = MODE_FP16
                if wide:
                    self._u16_hint = MODE_FP16
                else:
                    self._u8_hint = MODE_FP16
                continue
            if code & _lib.DEVERR_RANGE and mode == MODE_FP16 and self.operand == "auto":
                mode = MODE_BYTES
                if wide:
                    self._u16_hint = MODE_BYTES
                continue
            if code:
                raise DeviceError(_lib.device_error_message(code))
            try:
                grams = chunk_grams(L, seg_emax, self.exact_limit, self.kslab)
            except OverflowError:
                if mode != MODE_BYTES and self.operand == "auto":
                    mode = MODE_BYTES
                    continue
                raise
            if (mode == MODE_FP16 and self.method == "tc" and self.operand == "auto" and L.n_pieces
                    and int(pe[L.n_pieces: 2 * L.n_pieces].max()) <= 16 * 16):
                # every count <= 16 (the chunks' largest squares): the next call can use e4m3
                if frames_dev.element_size() == 1:
                    self._u8_hint = MODE_E4M3
                else:
                    self._u16_hint = MODE_E4M3
            return L, grams

    # -- chunked pipeline (e4m3) ---------------------------------------------
    TILE = "pair"
    PIPE_CHUNKS = 8
    SUPER_ROWS = 2048
    KSLAB = 0                 # no cap on the K columns of one tile item
    # chunk c of the frames weighs (c + 1) ** PIPE_GROWTH; growing chunks
    # start the tensor cores earlier but cut the Gram into more uneven
    # launches, and measured slower on the dense 514x1030x10k stack (1.0:
    # +0.05 ms, 1.5: +0.2 ms, 2.0: +0.3 ms per step), so chunks are equal
    PIPE_GROWTH = 0.0
    PIPE_GRAM_STREAMS = 2     # consecutive chunks' Gram launches alternate streams (-0.11 ms per step)
    # the first two chunks' Gram tiles share one launch (the first chunk's
    # alone leave most SMs idle: 11.81 -> 11.72 ms per step; three: 11.92)
    PIPE_MERGE_FIRST = 2
    # Frames copied from the host: the copies set the pace, and the Gram tiles
    # of the last chunk (a column strip of the whole triangle) can only run
    # after the last copy.  The last chunk is therefore cut into pieces of
    # 1/2, 1/4, ... of it (PIPE_TAPER_HOST halvings), so that the work left
    # after the last copy is a thin strip (pinned 514x1030x10k u8 stack:
    # 28.8 ms per call untapered, 27.6-28.2 ms with 2 to 4 cuts).
    PIPE_TAPER_HOST = 2
    # Frames from host memory: twice as many chunks, so that the first chunk's
    # copy (before any packing) and the work left after the last copy are
    # shorter (pinned 514x1030x10k u8 stack, cropped copies of 21.1 ms: 24.1 ms
    # per call with 8 chunks, 23.3 with 16 or 24, 24.5 with 6; 256x256x5k u16
    # on fp16 operands: 4.04 -> 3.98 ms)
    PIPE_CHUNKS_HOST = 16

    @staticmethod
    def pipe_bounds(T, n, growth, taper=0):
        """Frame bounds of ``n`` pipeline chunks (multiples of 128 frames, the
        last ending at T); chunk c's length grows as (c + 1) ** growth; with
        ``taper`` > 0 the last chunk is cut into pieces of half, a quarter,
        ... of it (``taper`` cuts, pieces of at least 128 frames)."""
        w = np.arange(1, n + 1, dtype=np.float64) ** float(growth)
        cum = np.cumsum(w)[:-1] / w.sum() * T
        b = [0]
        for x in cum:
            v = int(round(x / 128.0)) * 128
            if b[-1] < v < T:
                b.append(v)
        rest = int(T) - b[-1]
        for _ in range(int(taper)):
            v = b[-1] + int(round(rest / 2.0 / 128.0)) * 128
            if not b[-1] < v < T or T - v < 128:
                break
            b.append(v)
            rest = int(T) - v
        b.append(int(T))
        return np.array(b, dtype=np.int64)

    def _pipe_plan(self, L, taper=0, grams=None, chunks=None):
        """Items of the Gram grouped by the frame chunk whose packing makes
        them ready (a tile needs frames up to its last column), LPT order
        inside a group; cached per layout and K split (``grams``; default the
        e4m3 split, which needs no energies).  ``chunks``: the number of frame
        chunks (default ``pipe_chunks``)."""
        chunks = self.pipe_chunks if chunks is None else int(chunks)
        key = ("pipe", L.mode, self.T, self.exact_limit, self.grid, chunks, self.super_rows, self.kslab,
               self.item_kind, self.pipe_growth, int(taper), None if grams is None else tuple(grams))
        if key not in self._items_cache:
            torch = _torch()
            if grams is None:
                grams = chunk_grams(L, e4m3_segment_bound(L), self.exact_limit, self.kslab)
            items = gram_items(self.T, grams, job=0, out_base=0, kind=self.item_kind,
                               s_base=0 if self.ones(L) else None, super_rows=self.super_rows)
            T = self.T
            n = max(1, min(chunks, T // 256))
            bounds = self.pipe_bounds(T, n, self.pipe_growth, taper)
            need = np.minimum(items["j0"].astype(np.int64) + TILE_SHAPES[self.item_kind][1], T)
            grp = np.searchsorted(bounds[1:], need, side="left")
            # each chunk's launch balanced over the kernel's workers
            parts = [self.balanced(items[grp == g], L) for g in range(bounds.size - 1)]
            starts = np.concatenate([[0], np.cumsum([p.size for p in parts])]).astype(np.int64)
            items = np.concatenate(parts) if parts else items[:0]
            dev_items = torch.from_numpy(items.view(np.uint8).copy()).to(self.dev)
            if len(self._items_cache) > 8:
                self._items_cache.clear()
            self._items_cache[key] = (items, dev_items, bounds, starts, len(grams))
        return self._items_cache[key]

    def _streams(self):
        """(copy, pack, second Gram) side streams of the pipeline."""
        if getattr(self, "_side_streams", None) is None:
            torch = _torch()
            self._side_streams = tuple(torch.cuda.Stream(self.dev) for _ in range(3))
        return self._side_streams

    def _frames_buffer(self, shape, dtype):
        torch = _torch()
        buf = getattr(self, "_frames_buf", None)
        if buf is None or buf.dtype != dtype or tuple(buf.shape) != tuple(shape):
            self._frames_buf = None
            self._frames_buf = torch.empty(tuple(shape), dtype=dtype, device=self.dev)
        return self._frames_buf

    def pipelined_ok(self, frames):
        """The chunked pipeline applies on the tensor-core path to u8 stacks
        while their counts are known (or expected) to be <= 16 (e4m3), and to
        u8 / u16 stacks in pinned host memory on fp16 operands once a K split
        can be reused (see :meth:`_speculative_ok`): fp16 packs keep no
        per-frame state except energy maxima, which chunks combine."""
        return self._pipeline_mode(frames) is not None

    def _pipeline_mode(self, frames):
        torch = _torch()
        if not (self.method == "tc" and self.pipeline and isinstance(frames, torch.Tensor) and self.n_bins > 0
                and frames.dtype in (torch.uint8, torch.uint16)
                and (frames.is_cuda or (frames.is_pinned() and frames.is_contiguous()))):
            return None
        if (frames.dtype == torch.uint8 and self.operand in ("auto", "e4m3")
                and (self.operand == "e4m3" or self._u8_hint == MODE_E4M3)):
            return MODE_E4M3
        # fp16 from pinned host memory only: there the copies set the pace and
        # hide the pack and most of the Gram (256x256x5k u16: 4.99 -> 3.94 ms per
        # call); a device-resident stack runs faster unchunked (1.80 against
        # 2.00 ms: the chunk launches of so short a Gram cost more than the
        # 0.47 ms pack they would hide)
        mode = self.choose_mode(frames)
        if mode == MODE_FP16 and not frames.is_cuda and self._speculative_ok(mode):
            return MODE_FP16
        return None

    def run_pipelined(self, frames):
        """G1 + G2 chunk by chunk of frames: copy (host input) -> pack -> the
        Gram tiles that chunk completes, on three streams, so copies, packing
        and tensor-core work overlap; then G3 + G4.  One synchronisation at the
        end reads the error word; counts above 16 rerun on fp16 operands."""
        torch = _torch()
        mode = self._pipeline_mode(frames)
        L = self._layout(mode)
        packed = self._packed_buffer(L)
        host = not frames.is_cuda
        if mode == MODE_E4M3:
            grams, bound = None, None
        else:                                 # fp16: the reused K split and the bounds it covers
            _, bound, grams = self._plans[mode]
        items, dev_items, bounds, starts, n_grams = self._pipe_plan(
            L, self.PIPE_TAPER_HOST if host else 0, grams,
            self.pipe_chunks_host if host else self.pipe_chunks)
        # u8 frames from host memory come in cropped to the q-mask's columns
        # (the pack then reads the cropped frames with the cropped layout)
        crop = host and mode == MODE_E4M3 and frames.element_size() == 1 and self.crop is not None
        Lp = self._crop_layout(mode) if crop else L
        if Lp.packed_cols != L.packed_cols:
            raise RuntimeError("cropped packing layout differs from the frame's")
        npix_in = self.shape[0] * self.crop[1] if crop else self.npix
        if crop:
            frames_dev = self._frames_buffer((self.T, self.shape[0], self.crop[1]), frames.dtype)
        else:
            frames_dev = self._frames_buffer(frames.shape, frames.dtype) if host else frames
        if not host and frames_dev.data_ptr() % 16:
            frames_dev = frames_dev.clone()
        cur = torch.cuda.current_stream(self.dev)
        copy_s, pack_s, gram_s = self._streams()
        # consecutive chunks' Gram launches alternate between the caller's
        # stream and a second one, so a launch's CTAs take the SMs that the
        # previous launch's last items leave (sums are atomic adds: exact in
        # any order)
        gram_streams = (cur, gram_s) if self.pipe_gram_streams > 1 else (cur,)
        self._events = []
        self._mark("pipeline")
        self.numer.zero_()
        self.sums.zero_()
        self.err.zero_()
        emax = None
        if mode != MODE_E4M3:
            emax = self._piece_emax(L)
            emax.zero_()                      # chunks combine their energy maxima (atomicMax)
        start = torch.cuda.Event()
        start.record(cur)                     # the previous call's work and the zeroing are done first
        copy_s.wait_event(start)
        pack_s.wait_event(start)
        gram_s.wait_event(start)
        self._timeline = []
        self._tmark("start", cur)
        npix, pc = npix_in, L.packed_cols
        eb = frames_dev.element_size()
        row_bytes = L.packed_bytes_per_frame
        jobs = _lib.jobs_array([(packed.data_ptr(), self.T, pc, L.kind, self.ones(L))])
        item_bytes = _lib.ITEM_DTYPE.itemsize
        for c in range(bounds.size - 1):
            t0, t1 = int(bounds[c]), int(bounds[c + 1])
            if host:
                with torch.cuda.stream(copy_s):
                    if crop:
                        _lib.check(self.lib.g2_copy_cols_h2d(
                            C.c_void_p(frames_dev.data_ptr() + t0 * npix), C.c_void_p(frames.data_ptr() + t0 * self.npix),
                            self.shape[1], self.crop[0], self.crop[1], (t1 - t0) * self.shape[0],
                            C.c_void_p(copy_s.cuda_stream)), "g2_copy_cols_h2d")
                    else:
                        frames_dev[t0:t1].copy_(frames[t0:t1], non_blocking=True)
                    e = torch.cuda.Event()
                    e.record(copy_s)
                pack_s.wait_event(e)
            self._tmark("pack%d" % c, pack_s)
            if mode == MODE_E4M3:
                self.pack_e4m3(frames_dev.data_ptr() + t0 * npix, 1, t1 - t0, Lp, packed.data_ptr() + t0 * pc,
                               pack_s.cuda_stream, npix=npix)
            else:
                self.pack_fp16_frames(frames_dev.data_ptr() + t0 * npix * eb, eb, t1 - t0, L,
                                      packed.data_ptr() + t0 * row_bytes, emax, pack_s.cuda_stream)
            self._tmark("pack%d_end" % c, pack_s)
            e = torch.cuda.Event()
            e.record(pack_s)
            # the first PIPE_MERGE_FIRST chunks' tiles go in one launch (the
            # first chunk alone completes too few tiles to fill the GPU)
            merge = max(1, min(int(self.PIPE_MERGE_FIRST), bounds.size - 1))
            if c < merge - 1:
                continue
            k0, k1 = int(starts[0 if c == merge - 1 else c]), int(starts[c + 1])
            if k1 > k0:
                gs = gram_streams[c % len(gram_streams)]
                gs.wait_event(e)
                self._tmark("gram%d" % c, gs)
                self.gram_launch(jobs, dev_items.data_ptr() + k0 * item_bytes, k1 - k0, gs.cuda_stream)
                self._tmark("gram%d_end" % c, gs)
        if len(gram_streams) > 1:
            done = torch.cuda.Event()
            done.record(gram_s)
            cur.wait_event(done)
        self._mark("normalise")
        self._tmark("normalise", cur)
        self.normalise()
        self._mark("end")
        self._tmark("end", cur)
        if host:
            self._frames_host_ref = frames            # alive until the copies are done
        if mode != MODE_E4M3:
            # one synchronisation: the error word and whether the stack's
            # energy bounds exceed those the reused split covers
            m = L.n_pieces
            above = ((emax[:m].to(torch.int64) & 0xFFFFFFFF) > bound).any().to(torch.int32)
            code, over = (int(x) for x in torch.stack([self.err[0], above]).cpu())
            if code or over:                          # out of range, or a brighter stack: planned path
                return self.run(frames_dev, pipelined=False, reuse_split=False)
            self.last = {"mode": "fp16", "split": int(L.split), "n_items": int(items.size), "n_grams": n_grams,
                         "packed_cols": L.packed_cols, "pipeline_chunks": int(bounds.size - 1), "tile": self.tile,
                         "plan": "reused", "h2d_bytes": int(self.T * npix * eb) if host else 0, "crop": None}
            return self.g2_f32[: self.n_bins]
        code = self.resolve_range_check(int(self.err.item()), frames_dev, cropped=crop)
        if code & _lib.DEVERR_RANGE and self.operand == "auto":
            self._u8_hint = MODE_FP16                 # counts above 16: rerun on fp16 operands
            return self.run(frames if crop else frames_dev, pipelined=False)
        self.last = {"mode": "e4m3", "split": int(L.split), "n_items": int(items.size), "n_grams": n_grams,
                     "packed_cols": L.packed_cols, "pipeline_chunks": int(bounds.size - 1), "tile": self.tile,
                     "h2d_bytes": int(self.T * npix * eb) if host else 0, "crop": list(self.crop) if crop else None}
        return self.g2_f32[: self.n_bins]

    # -- whole pipeline ----------------------------------------------------
    def run(self, frames_dev, pipelined=True, reuse_split=True):
        """Run G1..G4 on a device stack; returns the float32 g2 device tensor.

        Pipelined stacks (see :meth:`pipelined_ok`) and stacks whose K split
        can be reused synchronise once, at the end; otherwise once after G1
        to read the segment energies (K split).  ``reuse_split=False`` plans
        the split from this stack's energies."""
        if tuple(frames_dev.shape) != (self.T,) + self.shape:
            raise ValueError("frames should have shape %s, got %s" % ((self.T,) + self.shape,
                                                                    tuple(frames_dev.shape)))
        if self.n_bins == 0:
            return self.g2_f32[:0]
        if pipelined and self.pipelined_ok(frames_dev):
            return self.run_pipelined(frames_dev)
        if not frames_dev.is_cuda:
            frames_dev = frames_to_device(frames_dev, self.dev)
        self._events = []
        self._mark("split")
        if self.method == "dp4a":
            return self._run_dp4a(frames_dev)
        mode = self.choose_mode(frames_dev)
        self._mark("pack")
        if reuse_split and self._speculative_ok(mode):
            g2 = self._run_speculative(frames_dev, mode)
            if g2 is not None:
                return g2
            self._events = []
            self._mark("pack")
        L, grams = self._pack_and_plan(frames_dev, mode)
        grams = self._remember_plan(L, grams)
        items, items_dev, n_chunks = self.items_for(L, grams)
        self._mark("gram_" + self.method)
        self.numerator(L, items_dev, items.size)
        self._mark("normalise")
        self.normalise()
        self._mark("end")
        self.last = {"mode": ["fp16", "bytes", "e4m3"][L.mode], "split": int(L.split), "n_items": int(items.size),
                     "n_grams": n_chunks, "packed_cols": L.packed_cols,
                     "tile": self.tile if self.method == "tc" else self.method, "plan": "planned"}
        return self.g2_f32[: self.n_bins]

    # -- reuse of the K split (fp16 operands and byte planes) -----------------
    # The K split of fp16 / byte-plane operands depends on the stack's energy
    # bounds, which the pack writes to the device; planning it on the host
    # costs a synchronisation with the GPU idle in between.  A split planned
    # from bounds B stays exact for every stack whose bounds are <= B piece
    # by piece (the Cauchy-Schwarz bound only grows with them).  So the engine
    # keeps B = the piecewise maximum of the bounds it has planned for (per
    # layout), and the next stack runs pack -> device check of its bounds
    # against B -> Gram with B's split -> normalisation without a
    # synchronisation; the check is read with the error word at the end, and
    # a stack above B is run again through the planned path (its Gram
    # results discarded), after which B covers it.
    SPECULATE_PLAN = True

    def _speculative_ok(self, mode):
        return (self.SPECULATE_PLAN and self.method == "tc" and mode != MODE_E4M3
                and mode in getattr(self, "_plans", {}))

    def _remember_plan(self, L, grams):
        """After a planned run on fp16 / byte-plane operands: widen the
        envelope B of layout L with this stack's bounds and return the split
        planned from B (valid for this stack too)."""
        if not (self.SPECULATE_PLAN and self.method == "tc") or L.mode == MODE_E4M3:
            return grams
        torch = _torch()
        m = L.n_pieces * (2 if L.split else 1)
        pe = self._piece_emax(L)[:m]
        plans = self.__dict__.setdefault("_plans", {})
        old = plans.get(L.mode)
        pe = pe.to(torch.int64) & 0xFFFFFFFF          # the pack's uint32 bounds
        bound = pe if old is None or old[0] is not L else torch.maximum(old[1], pe)
        host = np.zeros(2 * L.n_pieces, dtype=np.uint32)
        host[:m] = bound.cpu().numpy().astype(np.uint32)
        try:
            env = chunk_grams(L, L.segment_emax(host), self.exact_limit, self.kslab)
        except OverflowError:
            plans.pop(L.mode, None)
            return grams
        plans[L.mode] = (L, bound, env)
        return env

    def _run_speculative(self, frames_dev, mode):
        """Pack, check against the envelope, Gram with the envelope's split,
        normalise; one synchronisation.  None when the stack needs the
        planned path (bounds above the envelope, or counts outside the
        operand's range)."""
        torch = _torch()
        L0, bound, grams = self._plans[mode]
        L = self.pack(frames_dev, mode)
        if L is not L0:
            return None
        m = L.n_pieces * (2 if L.split else 1)
        above = ((self._piece_emax(L)[:m].to(torch.int64) & 0xFFFFFFFF) > bound).any().to(torch.int32)
        items, items_dev, n_chunks = self.items_for(L, grams)
        self._mark("gram_" + self.method)
        self.numerator(L, items_dev, items.size)
        self._mark("normalise")
        self.normalise()
        self._mark("end")
        code, over = (int(x) for x in torch.stack([self.err[0], above]).cpu())
        if code or over:
            return None
        self.last = {"mode": ["fp16", "bytes", "e4m3"][L.mode], "split": int(L.split), "n_items": int(items.size),
                     "n_grams": n_chunks, "packed_cols": L.packed_cols, "tile": self.tile, "plan": "reused"}
        return self.g2_f32[: self.n_bins]

    def _run_dp4a(self, frames_dev):
        """The u8 plain comparator: the e4m3 pack (a byte permutation, so the
        packed matrix holds the raw u8 counts whatever their range), then the
        __dp4a direct kernel over 128 x 128 blocks of at most 65,536 columns
        (exact uint32 entries for any u8 counts), bin sums from the row of
        ones, G3, G4."""
        if frames_dev.element_size() != 1:
            raise ValueError("the dp4a kernel reads u8 counts")
        self._mark("pack")
        L = self.pack(frames_dev, MODE_E4M3)
        code = int(self.err.item()) & ~(_lib.DEVERR_RANGE | _lib.DEVERR_RANGE_CHECK)   # counts > 16 are fine here
        if code:
            raise DeviceError(_lib.device_error_message(code))
        self.err.zero_()
        grams = chunk_grams(L, e4m3_segment_bound(L), self.exact_limit, self.kslab)
        items, items_dev, n_chunks = self.items_for(L, grams)
        self._mark("gram_dp4a")
        self.numerator(L, items_dev, items.size)
        self._mark("normalise")
        self.normalise()
        self._mark("end")
        self.last = {"mode": "u8", "split": 0, "n_items": int(items.size), "n_grams": n_chunks,
                     "packed_cols": L.packed_cols}
        return self.g2_f32[: self.n_bins]

    def deviation(self):
        """calc_std of the last run (dense.py:58-66): float32 device tensor
        ``(n_bins, T)``; float64 in ``self.dev_f64``.  One more tensor-core pass
        over the packed operand of the last run (u8/u16 counts <= 2048)."""
        torch = _torch()
        if self.method != "tc":
            raise NotImplementedError("calc_std runs on the tensor-core path")
        L = self._layouts.get(self._packed_mode)
        if L is None or self.packed is None:
            raise RuntimeError("deviation() needs a preceding run()")
        if L.split:
            return self._deviation_planes(L)
        key = ("std", L.mode, self.T)
        if key not in self._items_cache:
            from .plan import std_items
            npix = np.bincount(self.qmask.ravel()[self.qmask.ravel() > 0], minlength=self.n_bins + 1)[1:]
            items = std_items(self.T, L, npix)
            self._items_cache[key] = (items, torch.from_numpy(items.view(np.uint8).copy()).to(self.dev))
        items, dev_items = self._items_cache[key]
        rows = max(self.n_bins, 1)
        if getattr(self, "_std_bufs", None) is None:
            z = lambda dt: torch.zeros((rows, self.T), dtype=dt, device=self.dev)
            self._std_bufs = (z(torch.float64), z(torch.float64), z(torch.int32), z(torch.float32), z(torch.float64))
        sd, sd2, zeros, d32, d64 = self._std_bufs
        sd.zero_()
        sd2.zero_()
        zeros.zero_()
        st = stream_handle(self.dev)
        jobs = _lib.jobs_array([(self.packed.data_ptr(), self.T, L.packed_cols, L.kind, self.ones(L))])
        if items.size:
            _lib.check(self.lib.g2_gram_std(jobs, 1, ptr(dev_items), items.size, ptr(self.sums), self.sums.numel(),
                                            ptr(self.g2_f32), ptr(sd), ptr(sd2), ptr(zeros), sd.numel(),
                                            ptr(self.err), self.grid, st), "g2_gram_std")
        _lib.check(self.lib.g2_std_finalize(ptr(sd), ptr(sd2), ptr(zeros), self.n_bins, self.T, ptr(d32), ptr(d64),
                                            st), "g2_std_finalize")
        self.dev_f64 = d64
        return d32[: self.n_bins]

    def _deviation_planes(self, L):
        """calc_std of a byte-plane stack (counts above 2048): the per-pair
        ratio needs the four plane Grams of a pair together, so each bin's
        Gram G = 2^16 G_hh + 2^8 (G_hl + G_lh) + G_ll is assembled in a T x T
        float32 matrix (one tensor-core pass per plane combination, whole K)
        and each lag's deviation statistics are reduced from it."""
        torch = _torch()
        from .plan import _tiles
        T = self.T
        rows = max(self.n_bins, 1)
        z = lambda dt: torch.zeros((rows, T), dtype=dt, device=self.dev)
        sd, sd2, zeros, d32, d64 = z(torch.float64), z(torch.float64), z(torch.int32), z(torch.float32), \
            z(torch.float64)
        mat = getattr(self, "_gram_matrix", None)
        if mat is None or mat.numel() < T * T:
            self._gram_matrix = None
            mat = self._gram_matrix = torch.empty((T, T), dtype=torch.float32, device=self.dev)
        npix = np.bincount(self.qmask.ravel()[self.qmask.ravel() > 0], minlength=self.n_bins + 1)[1:]
        i0, j0 = _tiles(T, TILE_SHAPES["tc"][0], TILE_SHAPES["tc"][1])
        st = stream_handle(self.dev)
        jobs = _lib.jobs_array([(self.packed.data_ptr(), T, L.packed_cols, L.kind, 0)])
        by_bin = {}
        for (b, a_off, b_off, kp, shift) in L.grams():
            by_bin.setdefault(b, []).append((a_off, b_off, kp, shift))
        for b, combos in by_bin.items():
            if int(npix[b]) == 0:
                continue
            for n, (a_off, b_off, kp, shift) in enumerate(combos):
                it = np.zeros(i0.size, dtype=_lib.ITEM_DTYPE)
                it["i0"], it["j0"] = i0, j0
                it["a_k0"], it["b_k0"], it["k_len"], it["shift"] = a_off, b_off, kp, shift
                it["nframes"], it["out_off"], it["s_off"] = T, 0, -1
                dev_items = torch.from_numpy(it.view(np.uint8).copy()).to(self.dev)
                _lib.check(self.lib.g2_gram_matrix(jobs, 1, ptr(dev_items), it.size, ptr(mat), T, T, 1 if n else 0,
                                                   ptr(self.err), self.grid, st), "g2_gram_matrix")
            S = self.sums[b * T:(b + 1) * T] if self.sums.dim() == 1 else self.sums[b]
            _lib.check(self.lib.g2_matrix_deviation(ptr(mat), T, T, ptr(S), float(npix[b]), ptr(self.g2_f32[b]),
                                                    ptr(sd[b]), ptr(sd2[b]), ptr(zeros[b]), st),
                       "g2_matrix_deviation")
        _lib.check(self.lib.g2_std_finalize(ptr(sd), ptr(sd2), ptr(zeros), self.n_bins, T, ptr(d32), ptr(d64), st),
                   "g2_std_finalize")
        self.dev_f64 = d64
        return d32[: self.n_bins]

    def two_time(self, b):
        """Two-time correlation of bin ``b`` (0-based) for the last run: the
        TTCF of event_y.py:141-157, float32 device tensor ``(T, T)``:
        P G(t,t') / (S(t) S(t')) off the diagonal (mirrored when the
        reference mirrors it), the mean of the first upper diagonal's
        positive elements on the diagonal.  One more tensor-core pass over the
        bin's part of the last run's packed operand."""
        torch = _torch()
        if self.method != "tc":
            raise NotImplementedError("the two-time correlation runs on the tensor-core path")
        L = self._layouts.get(self._packed_mode)
        if L is None or self.packed is None:
            raise RuntimeError("two_time() needs a preceding run()")
        if L.split:
            raise NotImplementedError("the two-time correlation needs counts <= 2048 (no byte planes)")
        if not 0 <= b < self.n_bins:
            raise ValueError("bin %d outside [0, %d)" % (b, self.n_bins))
        key = ("std", L.mode, self.T)
        if key not in self._items_cache:
            from .plan import std_items
            npix = np.bincount(self.qmask.ravel()[self.qmask.ravel() > 0], minlength=self.n_bins + 1)[1:]
            items = std_items(self.T, L, npix)
            self._items_cache[key] = (items, torch.from_numpy(items.view(np.uint8).copy()).to(self.dev))
        items = self._items_cache[key][0]
        mine = items[items["out_off"] == b * self.T]
        if mine.size == 0:
            raise ValueError("bin %d has no pixels" % (b + 1))
        items_dev = torch.from_numpy(mine.view(np.uint8).copy()).to(self.dev)
        S = self.sums[b * self.T:(b + 1) * self.T] if self.sums.dim() == 1 else self.sums[b]
        s_h = S.cpu().numpy().astype(np.float64)
        # the reference mirrors when its diagonal k = -5 (0 or NaN = 0/0) sums below 1
        mirror = 1 if self.T <= 5 or not np.any(s_h[:-5] * s_h[5:] == 0) else 0
        out = torch.empty((self.T, self.T), dtype=torch.float32, device=self.dev)
        st = stream_handle(self.dev)
        jobs = _lib.jobs_array([(self.packed.data_ptr(), self.T, L.packed_cols, L.kind, self.ones(L))])
        _lib.check(self.lib.g2_gram_ttcf(jobs, 1, ptr(items_dev), mine.size, ptr(self.sums), self.sums.numel(),
                                         ptr(out), self.T, self.T, mirror, ptr(self.err), self.grid, st),
                   "g2_gram_ttcf")
        _lib.check(self.lib.g2_ttcf_finish(ptr(out), self.T, self.T, ptr(S), mirror, st), "g2_ttcf_finish")
        self.check_error()
        return out

    def check_denominator_range(self):
        """Raise if int64 D could have overflowed (checked from S on the host)."""
        S = self.sums[: self.n_bins].cpu().numpy()
        if S.size and float(S.max()) ** 2 * self.T >= 2.0 ** 63:
            raise OverflowError("denominator exceeds int64 for these counts")
