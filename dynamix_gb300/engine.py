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

import ctypes as C

import numpy as np

from . import _lib
from .plan import (E4M3_MAX_EXACT, EXACT_LIMIT, FP16_MAX_EXACT, MODE_BYTES, MODE_E4M3, MODE_FP16, PackLayout,
                   chunk_grams, e4m3_segment_bound, gram_items)


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


class DenseEngine:
    """Exact g2 of a dense (T, H, W) stack for the bins of one q-mask.

    ``operand`` selects the packed element type of the tensor-core Gram:
    ``"auto"`` (e4m3 when every binned count is <= 16, else fp16 counts when
    <= 2048, else fp16 byte planes), or one of ``"e4m3"``, ``"fp16"``,
    ``"bytes"``.  The plain comparator always uses fp16."""

    MODES = {"fp16": MODE_FP16, "bytes": MODE_BYTES, "e4m3": MODE_E4M3}

    def __init__(self, shape, nframes, qmask, n_bins, scale, device=None, method="tc",
                 exact_limit=EXACT_LIMIT, grid=0, operand="auto"):
        torch = _torch()
        self.lib = _lib.load()
        self.dev = require_cuda(device)
        self.shape = tuple(int(s) for s in shape)
        self.T = int(nframes)
        self.npix = self.shape[0] * self.shape[1]
        self.qmask = np.ascontiguousarray(qmask, dtype=np.int32)
        self.n_bins = int(n_bins)
        if method not in ("tc", "plain"):
            raise ValueError("method must be 'tc' or 'plain'")
        if operand != "auto" and operand not in self.MODES:
            raise ValueError("operand must be 'auto', 'e4m3', 'fp16' or 'bytes'")
        if method == "plain" and operand == "e4m3":
            raise ValueError("the plain kernel reads fp16 operands")
        self.method = method
        self.operand = operand
        self.exact_limit = int(exact_limit)
        self.grid = int(grid)
        self.scale = torch.as_tensor(np.asarray(scale, dtype=np.float64), device=self.dev)
        rows = max(self.n_bins, 1)
        z = lambda dt: torch.zeros((rows, self.T), dtype=dt, device=self.dev)
        self.sums = z(torch.int64)
        self.numer = z(torch.int64)
        self.denom = z(torch.int64)
        self.g2_f32 = z(torch.float32)
        self.g2_f64 = z(torch.float64)
        self.err = torch.zeros(1, dtype=torch.int32, device=self.dev)
        self.maxval = torch.zeros(1, dtype=torch.int32, device=self.dev)
        self._layouts = {}
        self._items_cache = {}
        self.packed = None
        self.last = {}
        self._u8_hint = MODE_E4M3 if method == "tc" else MODE_FP16
        self._packed_mode = None
        self.profile = False      # record CUDA events around every stage
        self.stage_ms = {}
        self._events = []

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
    def _layout(self, mode):
        if mode not in self._layouts:
            torch = _torch()
            L = PackLayout(self.qmask, self.n_bins, mode)
            d = lambda a: torch.as_tensor(a, device=self.dev)
            L.d_col_src = d(L.col_src)
            L.d_chunk_entry_off = d(L.chunk_entry_off)
            L.d_entry_dst = d(L.entry_dst)
            L.d_entry_meta = d(L.entry_meta.view(np.int32))
            L.d_chunk_slot_bin = d(L.chunk_slot_bin)
            L.d_chunk_piece_off = d(L.chunk_piece_off)
            L.d_bin_kpad = d(L.bin_kpad)
            L.d_piece_emax = torch.zeros(max(1, L.n_pieces * L.n_planes), dtype=torch.int32, device=self.dev)
            if mode == MODE_E4M3:
                L.d_chunk_word_off = d(L.chunk_word_off)
                L.d_word_dst = d(L.word_dst)
                L.d_word_src = d(L.word_src.view(np.int32))
            self._layouts[mode] = L
        return self._layouts[mode]

    def _packed_buffer(self, L):
        """The packed operand buffer, [T (+1)][packed_cols]; zeroed whenever its
        layout changes, since the pack kernels write only the binned columns
        (padding stays 0).  e4m3 layouts get the row of ones after the frames."""
        torch = _torch()
        rows = self.T + (1 if L.ones_row else 0)
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
            if L.ones_row:
                row = torch.from_numpy(L.ones_row_values().view(np.uint8)).to(self.dev)
                off = self.T * L.packed_bytes_per_frame
                self.packed[off:off + row.numel()].copy_(row)
        return self.packed

    # -- stages ----------------------------------------------------------
    def _binned_max(self, frames_dev):
        L0 = self._layout(MODE_FP16)
        self.maxval.zero_()
        _lib.check(self.lib.g2_binned_max(ptr(frames_dev), frames_dev.element_size(), self.T, self.npix,
                                          ptr(L0.d_col_src), L0.col_src.size, ptr(self.maxval),
                                          stream_handle(self.dev)), "g2_binned_max")
        return int(self.maxval.item())

    def choose_mode(self, frames_dev):
        if self.operand != "auto":
            return self.MODES[self.operand]
        if frames_dev.element_size() == 1:
            return self._u8_hint
        m = self._binned_max(frames_dev)
        if m <= E4M3_MAX_EXACT and self.method == "tc":
            return MODE_E4M3
        return MODE_FP16 if m <= FP16_MAX_EXACT else MODE_BYTES

    def pack(self, frames_dev, mode):
        L = self._layout(mode)
        packed = self._packed_buffer(L)
        self.sums.zero_()
        L.d_piece_emax.zero_()
        self.err.zero_()
        st = stream_handle(self.dev)
        if mode == MODE_E4M3:
            _lib.check(self.lib.g2_pack_e4m3(
                ptr(frames_dev), frames_dev.element_size(), self.T, self.npix, ptr(L.d_chunk_word_off),
                ptr(L.d_word_dst), ptr(L.d_word_src), L.n_chunks, ptr(packed), L.packed_cols, ptr(self.err), st),
                "g2_pack_e4m3")
            return L
        _lib.check(self.lib.g2_pack_frames(
            ptr(frames_dev), frames_dev.element_size(), self.T, self.npix, ptr(L.d_chunk_entry_off),
            ptr(L.d_entry_dst), ptr(L.d_entry_meta), ptr(L.d_chunk_slot_bin), ptr(L.d_chunk_piece_off),
            ptr(L.d_bin_kpad), L.n_chunks, mode, ptr(packed), L.packed_cols, ptr(self.sums), self.n_bins,
            ptr(L.d_piece_emax), L.n_pieces, ptr(self.err), st), "g2_pack_frames")
        return L

    def items_for(self, L, grams):
        key = (L.mode, self.method, tuple(grams))
        if key not in self._items_cache:
            torch = _torch()
            items = gram_items(self.T, grams, job=0, out_base=0, kind=self.method,
                               s_base=0 if (L.ones_row and self.method == "tc") else None)
            dev_items = torch.from_numpy(items.view(np.uint8).copy()).to(self.dev)
            if len(self._items_cache) > 8:
                self._items_cache.clear()
            self._items_cache[key] = (items, dev_items, len(grams))
        return self._items_cache[key]

    def numerator(self, L, items_dev, n_items):
        self.numer.zero_()
        jobs = _lib.jobs_array([(self.packed.data_ptr(), self.T, L.packed_cols, L.kind, L.ones_row)])
        st = stream_handle(self.dev)
        if self.method == "tc":
            _lib.check(self.lib.g2_gram_tc(jobs, 1, ptr(items_dev), n_items, ptr(self.numer), self.numer.numel(),
                                           ptr(self.sums), self.sums.numel(), ptr(self.err), self.grid, st),
                       "g2_gram_tc")
        else:
            _lib.check(self.lib.g2_plain_direct(jobs, 1, ptr(items_dev), n_items, ptr(self.numer),
                                                self.numer.numel(), ptr(self.err), st), "g2_plain_direct")

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
                seg_emax = L.segment_emax(L.d_piece_emax.cpu().numpy().view(np.uint32))
            code = int(self.err.item())
            if code & _lib.DEVERR_RANGE and mode == MODE_E4M3 and self.operand == "auto":
                mode = MODE_FP16
                self._u8_hint = MODE_FP16
                continue
            if code & _lib.DEVERR_RANGE and mode == MODE_FP16 and self.operand == "auto":
                mode = MODE_BYTES
                continue
            if code:
                raise DeviceError(_lib.device_error_message(code))
            try:
                grams = chunk_grams(L, seg_emax, self.exact_limit)
            except OverflowError:
                if mode != MODE_BYTES and self.operand == "auto":
                    mode = MODE_BYTES
                    continue
                raise
            if (mode == MODE_FP16 and frames_dev.element_size() == 1 and self.method == "tc"
                    and self.operand == "auto" and seg_emax.size and int(seg_emax.max()) < 17 * 17):
                self._u8_hint = MODE_E4M3        # every count <= 16: the next call can use e4m3
            return L, grams

    # -- whole pipeline ----------------------------------------------------
    def run(self, frames_dev):
        """Run G1..G4 on a device stack; returns the float32 g2 device tensor.

        Synchronises once after G1 to read the segment energies (K split)."""
        if tuple(frames_dev.shape) != (self.T,) + self.shape:
            raise ValueError("frames should have shape %s, got %s" % ((self.T,) + self.shape,
                                                                    tuple(frames_dev.shape)))
        if self.n_bins == 0:
            return self.g2_f32[:0]
        self._events = []
        self._mark("split")
        mode = self.choose_mode(frames_dev)
        self._mark("pack")
        L, grams = self._pack_and_plan(frames_dev, mode)
        items, items_dev, n_chunks = self.items_for(L, grams)
        self._mark("gram_" + self.method)
        self.numerator(L, items_dev, items.size)
        self._mark("normalise")
        self.normalise()
        self._mark("end")
        self.last = {"mode": ["fp16", "bytes", "e4m3"][L.mode], "split": int(L.split), "n_items": int(items.size),
                     "n_grams": n_chunks, "packed_cols": L.packed_cols}
        return self.g2_f32[: self.n_bins]

    def check_denominator_range(self):
        """Raise if int64 D could have overflowed (checked from S on the host)."""
        S = self.sums[: self.n_bins].cpu().numpy()
        if S.size and float(S.max()) ** 2 * self.T >= 2.0 ** 63:
            raise OverflowError("denominator exceeds int64 for these counts")


def _events_to_device(vol_times, vol_data, offsets, npix, dev):
    """Validate the event arrays (layout of dynamix's FramesCompressor) and
    move them to the device: times int32, counts uint8/uint16, offsets uint32.
    Returns (times, counts, offsets, host offsets int64, max count, (min t, max t))."""
    torch = _torch()

    def host(a):
        return a.cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)

    offs64 = host(offsets).astype(np.int64)
    if offs64.ndim != 1 or offs64.size != npix + 1:
        raise ValueError("offsets should have size %d, got %s" % (npix + 1, offs64.shape))
    if offs64[0] != 0 or np.any(np.diff(offs64) < 0):
        raise ValueError("offsets must start at 0 and be non-decreasing")
    n_ev = int(offs64[-1])
    if n_ev >= 2 ** 32:
        raise ValueError("too many events for uint32 offsets")
    if np.ndim(vol_times) != 1 or np.ndim(vol_data) != 1 or len(vol_times) != len(vol_data):
        raise ValueError("vol_times and vol_data must be 1-D arrays of the same size")
    if len(vol_times) < n_ev:
        raise ValueError("offsets reference %d events but only %d are given" % (n_ev, len(vol_times)))

    def to_dev(a):
        if isinstance(a, torch.Tensor):
            t = a[:n_ev]
            if t.dtype == torch.uint16:
                t = t.to(torch.int32)
            return t.to(dev)
        a = np.ascontiguousarray(np.asarray(a)[:n_ev])
        if a.dtype == np.uint16 or a.dtype == np.uint32:
            a = a.astype(np.int64)
        return torch.from_numpy(a).to(dev)

    times = to_dev(vol_times)
    if times.dtype.is_floating_point:
        raise TypeError("event times must be integers")
    times = times.to(torch.int32).contiguous()
    counts = to_dev(vol_data)
    if counts.dtype.is_floating_point:
        if n_ev and not bool(torch.all(counts == torch.round(counts))):
            raise TypeError("event counts must be integers")
    counts = counts.to(torch.int32) if counts.dtype != torch.int64 else counts
    mx = int(counts.max().item()) if n_ev else 0
    mn = int(counts.min().item()) if n_ev else 0
    if mn < 0:
        raise ValueError("counts must be non-negative")
    if mx > 65535:
        raise ValueError("counts above 65535 are not supported")
    counts = counts.to(torch.uint8) if mx <= 255 else counts.to(torch.int32).to(torch.uint16)
    tmin = int(times.min().item()) if n_ev else 0
    tmax = int(times.max().item()) if n_ev else 0
    offs_d = torch.from_numpy(offs64.astype(np.uint32).view(np.int32)).to(dev)
    return times, counts.contiguous(), offs_d, offs64, mx, (tmin, tmax)


class EventEngine:
    """Exact g2 from per-pixel event lists (G6 pair sums, then G3, G4)."""

    def __init__(self, shape, nframes, qmask, n_bins, scale, device=None, ranges_per_sm=4):
        torch = _torch()
        self.lib = _lib.load()
        self.dev = require_cuda(device)
        self.shape = tuple(int(s) for s in shape)
        self.npix = self.shape[0] * self.shape[1]
        self.T = int(nframes)
        if self.T >= 2 ** 31:
            raise ValueError("too many frames")
        self.n_bins = int(n_bins)
        q = np.ascontiguousarray(qmask, dtype=np.int32).ravel()
        self.qflat = np.where(q >= 1, q, 0)
        order = np.argsort(self.qflat, kind="stable")
        counts = np.bincount(self.qflat, minlength=self.n_bins + 1)[: self.n_bins + 1]
        starts = np.concatenate([[0], np.cumsum(counts)])
        self.binned = order[starts[1]:]                         # binned pixels, bin by bin
        self.binned_bin = self.qflat[self.binned] - 1
        self.ranges_per_sm = int(ranges_per_sm)
        self.scale = torch.as_tensor(np.asarray(scale, dtype=np.float64), device=self.dev)
        rows = max(self.n_bins, 1)
        z = lambda dt: torch.zeros((rows, self.T), dtype=dt, device=self.dev)
        self.sums, self.numer, self.denom = z(torch.int64), z(torch.int64), z(torch.int64)
        self.g2_f32, self.g2_f64 = z(torch.float32), z(torch.float64)
        self.err = torch.zeros(1, dtype=torch.int32, device=self.dev)
        self.last = {}

    def plan_ranges(self, offs64):
        """Cut the binned pixels with events into ranges of one bin each, of
        about equal pair counts (the work of a CTA)."""
        n = np.diff(offs64)[self.binned]
        keep = n > 0
        pix = self.binned[keep]
        pb = self.binned_bin[keep]
        pairs = n[keep] * (n[keep] + 1) // 2
        total = int(pairs.sum())
        sms = _torch().cuda.get_device_properties(self.dev).multi_processor_count
        target = max(1, total // max(1, sms * self.ranges_per_sm))
        cum = np.cumsum(pairs)
        # range id = (bin, cumulative pairs // target), cut at bin changes
        key = pb.astype(np.int64) * (total // target + 2) + (cum - pairs) // target
        starts = np.flatnonzero(np.concatenate([[True], key[1:] != key[:-1]])) if pix.size else np.zeros(0, np.int64)
        range_off = np.concatenate([starts, [pix.size]]).astype(np.int32)
        range_bin = pb[starts].astype(np.int32) if pix.size else np.zeros(0, np.int32)
        return pix.astype(np.int32), range_off, range_bin, total

    def run(self, vol_times, vol_data, offsets):
        times_d, data_d, offs_d, offs64, mx, (tmin, tmax) = _events_to_device(vol_times, vol_data, offsets,
                                                                           self.npix, self.dev)
        if offs64[-1] and (tmin < 0 or tmax >= self.T):
            raise ValueError("event times must lie in [0, nframes)")
        return self.run_device(times_d, data_d, offs_d, offs64, mx)

    def run_device(self, times_d, data_d, offs_d, offs64, mx):
        """G6 + G3 + G4 on device-resident events (times int32, counts
        uint8/uint16, offsets uint32 on the device; offsets also on the host)."""
        torch = _torch()
        pix, range_off, range_bin, total = self.plan_ranges(offs64)
        self.numer.zero_()
        self.sums.zero_()
        self.err.zero_()
        st = stream_handle(self.dev)
        if range_bin.size and self.n_bins:
            d = lambda a: torch.from_numpy(a).to(self.dev)
            pix_d, ro_d, rb_d = d(pix), d(range_off), d(range_bin)
            _lib.check(self.lib.g2_event_pairsum(
                ptr(times_d), ptr(data_d), data_d.element_size(), int(offs64[-1]), ptr(offs_d), self.npix,
                ptr(pix_d), ptr(ro_d), ptr(rb_d), int(range_bin.size), self.T, self.n_bins, mx, ptr(self.numer),
                ptr(self.sums), ptr(self.err), st), "g2_event_pairsum")
        if self.n_bins:
            _lib.check(self.lib.g2_denominator(ptr(self.sums), self.n_bins, self.T, ptr(self.denom), st),
                       "g2_denominator")
            _lib.check(self.lib.g2_finalize(ptr(self.numer), ptr(self.denom), ptr(self.scale), self.n_bins,
                                            self.T, ptr(self.g2_f32), ptr(self.g2_f64), st), "g2_finalize")
        self.last = {"n_events": int(offs64[-1]), "pairs": total, "n_ranges": int(range_bin.size),
                     "max_count": mx}
        return self.g2_f32[: self.n_bins]

    def check_error(self):
        code = int(self.err.item())
        if code:
            raise DeviceError(_lib.device_error_message(code))


def _csr_to_device(data, indices, indptr, offsets, shape, nframes, dev):
    """Validate a CSR stack (layout of dynamix's SparseCorrelator) and move it
    to the device with one index type (uint32 when every index fits, else int64)."""
    torch = _torch()
    H, W = shape

    def host(a):
        return a.cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)

    data, indices, indptr, offsets = (host(a).ravel() for a in (data, indices, indptr, offsets))
    assert data.size == indices.size
    assert indptr.size == (H + 1) * nframes
    assert offsets.size == nframes + 1
    n = int(data.size)
    if data.dtype.kind == "f":
        if n and not np.all(data == np.round(data)):
            raise TypeError("counts must be integers")
    if n and data.min() < 0:
        raise ValueError("counts must be non-negative")
    mx = int(data.max()) if n else 0
    if mx > 65535:
        raise ValueError("counts above 65535 are not supported")
    big = max(int(offsets.max()) if offsets.size else 0, int(indptr.max()) if indptr.size else 0, n) >= 2 ** 32
    idt = np.int64 if big else np.uint32
    if n and (indices.min() < 0 or indices.max() >= W):
        raise ValueError("column indices must lie in [0, width)")
    d = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a.astype(dt, copy=False)).view(
        np.int64 if dt == np.int64 else np.int32)).to(dev)
    data_d = torch.from_numpy(np.ascontiguousarray(data.astype(np.uint8 if mx <= 255 else np.uint16))).to(dev)
    return (data_d, d(indices, idt), d(indptr, idt), d(offsets, idt), 8 if big else 4, n, mx)


class SparseEngine:
    """Exact g2 from per-frame CSR: transpose to event lists (G7), then G6-G4."""

    def __init__(self, shape, nframes, qmask, n_bins, scale, device=None):
        torch = _torch()
        self.events = EventEngine(shape, nframes, qmask, n_bins, scale, device=device)
        self.lib = self.events.lib
        self.dev = self.events.dev
        self.shape, self.T, self.npix = self.events.shape, self.events.T, self.events.npix
        self.counts = torch.zeros(self.npix, dtype=torch.int32, device=self.dev)
        self.ev_off = torch.zeros(self.npix + 1, dtype=torch.int32, device=self.dev)
        n_tiles = -(-self.npix // 8192)
        self.scan_scratch = torch.zeros(max(1, n_tiles), dtype=torch.int32, device=self.dev)
        self.last = {}

    def to_events(self, data_d, indices_d, indptr_d, offsets_d, ib, n, mx):
        """CSR on the device -> (times, counts, offsets) event lists on the device."""
        torch = _torch()
        st = stream_handle(self.dev)
        err = self.events.err
        err.zero_()
        self.counts.zero_()
        H, W = self.shape
        _lib.check(self.lib.g2_csr_count(ptr(indices_d), ptr(indptr_d), ptr(offsets_d), ib, n, self.T, H, W,
                                         ptr(self.counts), ptr(err), st), "g2_csr_count")
        _lib.check(self.lib.g2_exclusive_scan_u32(ptr(self.counts), self.npix, ptr(self.ev_off),
                                                  ptr(self.scan_scratch), self.scan_scratch.numel(), st),
                   "g2_exclusive_scan_u32")
        times_d = torch.empty(max(1, n), dtype=torch.int32, device=self.dev)
        evdata_d = torch.empty(max(1, n), dtype=data_d.dtype, device=self.dev)
        self.counts.zero_()                              # reused as the scatter cursor
        _lib.check(self.lib.g2_csr_scatter(ptr(data_d), data_d.element_size(), ptr(indices_d), ptr(indptr_d),
                                           ptr(offsets_d), ib, n, self.T, H, W, ptr(self.ev_off), ptr(self.counts),
                                           ptr(times_d), ptr(evdata_d), ptr(err), st), "g2_csr_scatter")
        offs64 = self.ev_off.cpu().numpy().view(np.uint32).astype(np.int64)
        code = int(err.item())
        if code:
            raise DeviceError(_lib.device_error_message(code))
        if offs64[-1] != n:
            raise DeviceError("CSR transposition lost elements")
        return times_d, evdata_d, self.ev_off, offs64

    def run(self, data, indices, indptr, offsets):
        data_d, indices_d, indptr_d, offsets_d, ib, n, mx = _csr_to_device(data, indices, indptr, offsets,
                                                                          self.shape, self.T, self.dev)
        times_d, evdata_d, offs_d, offs64 = self.to_events(data_d, indices_d, indptr_d, offsets_d, ib, n, mx)
        out = self.events.run_device(times_d, evdata_d, offs_d, offs64, mx)
        self.last = dict(self.events.last, n_elements=n)
        return out

    def check_error(self):
        self.events.check_error()
