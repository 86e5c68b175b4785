"""Device pipelines of the event-list and sparse (CSR) correlators.

Event lists (G6): per pixel, its events (frame, count) in the layout of
dynamix's FramesCompressor.  The binned pixels are listed bin by bin once per
q-mask and that list is cut into one contiguous slice per CTA (split at bin
boundaries), so a call needs no host-side planning: the pair-sum kernel adds
N and S, then G3 (denominator) and G4 (g2) follow.

CSR (G7): per-frame CSR in the layout of dynamix's SparseCorrelator, transposed
on the device (count, scan, scatter) into event lists, then the same G6-G4.

Inputs that already live on the GPU are validated there (no host round trip);
numpy inputs are validated on the host before the copy.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .engine import DeviceError, _torch, ptr, require_cuda, stream_handle

# shared memory of the shared-counter pair kernel besides its 2 x T counters:
# 24 warps x 2 half-warp pixels x 2 staging buffers x 128 events x 4 bytes
# (g2_event.cu, ev::SMEM_FIXED)
PAIRS_SMEM_FIXED = 24 * 2 * 2 * 128 * 4


def _is_cuda(a):
    torch = _torch()
    return isinstance(a, torch.Tensor) and a.is_cuda


def _int_counts_to_device(counts, n, dev):
    """Validated non-negative integer counts -> device uint8 (max <= 255) or
    uint16 tensor; returns (tensor, max)."""
    torch = _torch()
    if isinstance(counts, torch.Tensor):
        c = counts[:n]
        if c.dtype == torch.uint16:
            c = c.to(torch.int32)
        c = c.to(dev)
    else:
        a = np.ascontiguousarray(np.asarray(counts)[:n])
        if a.dtype.kind not in "iuf":
            raise TypeError("counts must be integers")
        if a.dtype == np.uint16 or a.dtype == np.uint32:
            a = a.astype(np.int64)
        c = torch.from_numpy(a).to(dev)
    if c.dtype.is_floating_point:
        if n and not bool(torch.all(c == torch.round(c))):
            raise TypeError("counts must be integers")
        c = c.to(torch.int32)
    if n == 0:
        return torch.zeros(1, dtype=torch.uint8, device=dev), 0
    if c.dtype == torch.uint8:
        return c.contiguous(), int(c.max().item())
    lo, hi = torch.aminmax(c)
    if int(lo.item()) < 0:
        raise ValueError("counts must be non-negative")
    mx = int(hi.item())
    if mx > 65535:
        raise ValueError("counts above 65535 are not supported")
    out = c.to(torch.uint8) if mx <= 255 else c.to(torch.int32).to(torch.uint16)
    return out.contiguous(), mx


def events_to_device(vol_times, vol_data, offsets, npix, nframes, dev):
    """Validate event arrays and move them to the device.

    Returns ``(times int32, counts uint8/uint16, offsets uint32 (as int32),
    n_events, max_count)``.  Raises ValueError for a bad layout or times
    outside [0, nframes)."""
    torch = _torch()
    if np.ndim(vol_times) != 1 or np.ndim(vol_data) != 1 or np.ndim(offsets) != 1:
        raise ValueError("event arrays must be 1-D")
    if len(vol_times) != len(vol_data):
        raise ValueError("vol_times and vol_data must have the same size")
    if len(offsets) != npix + 1:
        raise ValueError("offsets should have size %d, got %d" % (npix + 1, len(offsets)))
    if _is_cuda(offsets):
        o = offsets.to(dev).to(torch.int64)
        if int(o[0].item()) != 0 or not bool(torch.all(o[1:] >= o[:-1])):
            raise ValueError("offsets must start at 0 and be non-decreasing")
        n_ev = int(o[-1].item())
    else:
        o = np.asarray(offsets).astype(np.int64)
        if o[0] != 0 or np.any(np.diff(o) < 0):
            raise ValueError("offsets must start at 0 and be non-decreasing")
        n_ev = int(o[-1])
    if n_ev >= 2 ** 32:
        raise ValueError("too many events for uint32 offsets")
    if len(vol_times) < n_ev:
        raise ValueError("offsets reference %d events but only %d are given" % (n_ev, len(vol_times)))
    if isinstance(o, np.ndarray):
        offs_d = torch.from_numpy(o.astype(np.uint32).view(np.int32)).to(dev)
    else:
        offs_d = o.to(torch.int32)                     # values < 2^31 here; uint32 bit pattern otherwise
    if isinstance(vol_times, torch.Tensor):
        times = vol_times[:n_ev].to(dev)
    else:
        times = torch.from_numpy(np.ascontiguousarray(np.asarray(vol_times)[:n_ev])).to(dev)
    if times.dtype.is_floating_point:
        raise TypeError("event times must be integers")
    times = times.to(torch.int32).contiguous()
    if n_ev:
        tmin, tmax = (int(x.item()) for x in torch.aminmax(times))
        if tmin < 0 or tmax >= nframes:
            raise ValueError("event times must lie in [0, nframes)")
    counts, mx = _int_counts_to_device(vol_data, n_ev, dev)
    return times, counts, offs_d, n_ev, mx


def csr_to_device(data, indices, indptr, offsets, shape, nframes, dev):
    """Validate a CSR stack and move it to the device with one index type
    (uint32 when every index fits, else int64).  Returns
    ``(data, indices, indptr, offsets, index_bytes, n_elements, max_count)``."""
    torch = _torch()
    H, W = shape
    for a in (data, indices, indptr, offsets):
        assert np.ndim(a) == 1
    assert len(data) == len(indices)
    assert len(indptr) == (H + 1) * nframes
    assert len(offsets) == nframes + 1
    n = int(len(data))

    def dev_int(a):
        if isinstance(a, torch.Tensor):
            t = a.to(dev)
            return t.to(torch.int64) if t.dtype in (torch.uint16, torch.uint32) else t
        a = np.asarray(a)
        if a.dtype == np.uint32 or a.dtype == np.uint64:
            a = a.astype(np.int64)
        return torch.from_numpy(np.ascontiguousarray(a)).to(dev)

    ind, ip, off = dev_int(indices), dev_int(indptr), dev_int(offsets)
    big = max(int(off[-1].item()), int(ip.max().item()) if ip.numel() else 0, n) >= 2 ** 31
    if n:
        lo, hi = torch.aminmax(ind)
        if int(lo.item()) < 0 or int(hi.item()) >= W:
            raise ValueError("column indices must lie in [0, width)")
    it = torch.int64 if big else torch.int32
    ind, ip, off = (x.to(it).contiguous() for x in (ind, ip, off))
    counts, mx = _int_counts_to_device(data, n, dev)
    return counts, ind, ip, off, 8 if big else 4, n, mx


def cta_ranges(binned_bin, n_ctas):
    """Static work split of the pair-sum kernel.

    ``binned_bin`` is the bin of every binned pixel, the pixels listed bin by
    bin.  The list is cut into ``n_ctas`` (at most one per pixel) contiguous
    slices of equal size, and each slice at the bin changes inside it, giving
    ranges of pixels of one bin.  Returns int32 ``(range_off [n_ranges + 1],
    range_bin [n_ranges], cta_range_off [n_ctas + 1])``: CTA c handles ranges
    ``cta_range_off[c] .. cta_range_off[c+1]``, range r the pixels
    ``range_off[r] .. range_off[r+1]`` of the list."""
    binned_bin = np.asarray(binned_bin, dtype=np.int32)
    n = binned_bin.size
    n_ctas = max(1, min(int(n_ctas), n))
    bounds = (np.arange(n_ctas + 1, dtype=np.int64) * n) // n_ctas
    cuts = set(bounds.tolist())
    if n:
        cuts.update((np.flatnonzero(np.diff(binned_bin)) + 1).tolist())
    starts = np.array(sorted(c for c in cuts if c < n), dtype=np.int64)
    range_off = np.concatenate([starts, [n]]).astype(np.int32)
    range_bin = binned_bin[starts].astype(np.int32) if n else np.zeros(0, np.int32)
    cta_range_off = np.searchsorted(starts, bounds).astype(np.int32)
    return range_off, range_bin, cta_range_off


class EventEngine:
    """Exact g2 from per-pixel event lists (G6 pair sums, then G3, G4)."""

    SMEM_CTAS_PER_SM = 1   # the shared-memory kernel holds 2 x T counters per CTA
    GLOBAL_CTAS_PER_SM = 8

    def __init__(self, shape, nframes, qmask, n_bins, scale, device=None):
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
        q = np.where(q >= 1, q, 0)
        order = np.argsort(q, kind="stable")
        counts = np.bincount(q, minlength=self.n_bins + 1)[: self.n_bins + 1]
        self.binned = order[counts[0]:].astype(np.int32)          # binned pixels, bin by bin
        self.binned_bin = (q[self.binned] - 1).astype(np.int32)
        sms = torch.cuda.get_device_properties(self.dev).multi_processor_count
        self.pix_list = torch.from_numpy(self.binned).to(self.dev)
        self.plans = {k: self._plan(sms * n) for k, n in
                      (("smem", self.SMEM_CTAS_PER_SM), ("global", self.GLOBAL_CTAS_PER_SM))}
        self.scale = torch.as_tensor(np.asarray(scale, dtype=np.float64), device=self.dev)
        rows = max(self.n_bins, 1)
        z = lambda dt: torch.zeros((rows, self.T), dtype=dt, device=self.dev)
        self.sums, self.numer, self.denom = z(torch.int64), z(torch.int64), z(torch.int64)
        self.g2_f32, self.g2_f64 = z(torch.float32), z(torch.float64)
        self.err = torch.zeros(1, dtype=torch.int32, device=self.dev)
        self.last = {}
        self.profile = False
        self._events = []

    def _mark(self, name):
        """With ``profile`` set, record a CUDA event named ``name`` on the stream."""
        if self.profile:
            torch = _torch()
            e = torch.cuda.Event(enable_timing=True)
            e.record(torch.cuda.current_stream(self.dev))
            self._events.append((name, e))

    def take_events(self):
        ev, self._events = self._events, []
        return ev

    @staticmethod
    def stage_times(events):
        """{stage: ms} from consecutive marks (stage = the name of its end mark)."""
        out = {}
        for (_, a), (name, b) in zip(events, events[1:]):
            out[name] = out.get(name, 0.0) + a.elapsed_time(b)
        return out

    def _plan(self, n_ctas):
        torch = _torch()
        range_off, range_bin, cta_range_off = cta_ranges(self.binned_bin, n_ctas)
        d = lambda a: torch.from_numpy(a).to(self.dev)
        return d(range_off), d(range_bin), d(cta_range_off), int(range_bin.size), int(cta_range_off.size - 1)

    def run(self, vol_times, vol_data, offsets):
        if self.host_pipeline_ok(vol_times, vol_data, offsets):
            return self.run_host_pipelined(vol_times, vol_data, offsets)
        times, counts, offs, n_ev, mx = events_to_device(vol_times, vol_data, offsets, self.npix, self.T,
                                                         self.dev)
        return self.run_device(times, counts, offs, n_ev, mx)

    HOST_CHUNKS = 8
    # the last pixel chunk is cut into halving pieces (HOST_TAPER cuts): the
    # pair sums left after the last copy cover a thin slice of the pixels
    HOST_TAPER = 2

    @staticmethod
    def host_chunk_bounds(npix, chunks, taper):
        """Pixel bounds of the host pipeline's chunks: ``chunks`` equal ones,
        the last cut ``taper`` times in half."""
        b = [npix * c // chunks for c in range(chunks)]
        for _ in range(int(taper)):
            mid = (b[-1] + npix) // 2
            if not b[-1] < mid < npix:
                break
            b.append(mid)
        b.append(npix)
        return b

    def host_pipeline_ok(self, vol_times, vol_data, offsets):
        """Pinned host tensors (times int32, counts uint8/uint16, offsets
        int32/int64 of npix + 1) go through the chunked host pipeline."""
        torch = _torch()
        ts = (vol_times, vol_data, offsets)
        if not all(isinstance(x, torch.Tensor) and not x.is_cuda and x.is_pinned() and x.is_contiguous()
                   and x.dim() == 1 for x in ts):
            return False
        return (vol_times.dtype == torch.int32 and vol_data.dtype in (torch.uint8, torch.uint16)
                and offsets.dtype in (torch.int32, torch.int64) and offsets.numel() == self.npix + 1
                and vol_times.numel() == vol_data.numel() and self.n_bins > 0)

    def _chunk_plans(self):
        """Per pixel chunk (raster order, :meth:`host_chunk_bounds`): its
        binned pixels bin by bin and their CTA ranges, for both pair kernels."""
        plans = getattr(self, "_host_plans", None)
        if plans is None:
            torch = _torch()
            sms = torch.cuda.get_device_properties(self.dev).multi_processor_count
            bounds = self.host_chunk_bounds(self.npix, self.HOST_CHUNKS, self.HOST_TAPER)
            plans = []
            for c in range(len(bounds) - 1):
                keep = (self.binned >= bounds[c]) & (self.binned < bounds[c + 1])
                pix, bins = self.binned[keep], self.binned_bin[keep]
                d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(self.dev)
                per = {}
                for k, n in (("smem", self.SMEM_CTAS_PER_SM), ("global", self.GLOBAL_CTAS_PER_SM)):
                    ro, rb, cro = cta_ranges(bins, sms * n)
                    per[k] = (d(ro), d(rb), d(cro), int(rb.size), int(cro.size - 1))
                plans.append((bounds[c], bounds[c + 1], d(pix.astype(np.int32)), per))
            self._host_plans = plans
        return plans

    def run_host_pipelined(self, vol_times, vol_data, offsets):
        """Events in pinned host memory: the offsets first, then every pixel
        chunk's counts and frame times back to back on the copy stream.  As
        soon as a chunk's counts have arrived its largest count is taken on
        the device and read by the host (it picks the chunk's pair kernel and
        whether its counters need drain checks), and the chunk's pair sums
        run while later chunks are still being copied.  Offsets that do not
        start at 0 or decrease are found on the device and raise ValueError
        after the call (the pair kernels bound every access), as do frame
        times outside [0, nframes)."""
        torch = _torch()
        cur = torch.cuda.current_stream(self.dev)
        copy_s = getattr(self, "_copy_stream", None)
        if copy_s is None:
            copy_s = self._copy_stream = torch.cuda.Stream(self.dev)
        max_s = getattr(self, "_max_stream", None)
        if max_s is None:
            max_s = self._max_stream = torch.cuda.Stream(self.dev)
        host_off = offsets                                 # pinned host offsets: chunk bounds, n_ev
        n_ev = int(host_off[-1])
        if host_off.dtype == torch.int32:
            n_ev &= 0xFFFFFFFF                             # uint32 offsets held in int32
        if n_ev >= 2 ** 32:
            raise ValueError("too many events for uint32 offsets")
        if vol_times.numel() < n_ev:
            raise ValueError("offsets reference %d events but only %d are given" % (n_ev, vol_times.numel()))
        offs64 = offsets.to(self.dev, non_blocking=True).to(torch.int64)
        if offsets.dtype == torch.int32:
            offs64 = offs64 & 0xFFFFFFFF                   # uint32 offsets held in int32
        self._offsets_bad = ((offs64[0] != 0) | (offs64[1:] < offs64[:-1]).any()).to(torch.int32)
        offs = offs64.to(torch.int32)                      # uint32 bit pattern (n_ev < 2^32)
        times = getattr(self, "_times_buf", None)
        if times is None or times.numel() < max(n_ev, 1):
            self._times_buf = None
            times = self._times_buf = torch.empty(max(n_ev, 1), dtype=torch.int32, device=self.dev)
        counts = getattr(self, "_counts_buf", None)
        if counts is None or counts.numel() < max(n_ev, 1) or counts.dtype != vol_data.dtype:
            self._counts_buf = None
            counts = self._counts_buf = torch.empty(max(n_ev, 1), dtype=vol_data.dtype, device=self.dev)
        self.numer.zero_()
        self.sums.zero_()
        self.err.zero_()
        st = stream_handle(self.dev)
        start = torch.cuda.Event()
        start.record(cur)
        copy_s.wait_event(start)
        max_s.wait_event(start)
        plans = self._chunk_plans()
        mx_host = torch.zeros(len(plans), dtype=torch.int32, pin_memory=True)
        spans, ready, mx_ready = [], [], []
        for c, (p0, p1, pix, per) in enumerate(plans):    # every copy first, so the link never waits
            e0 = min(int(host_off[p0]) & 0xFFFFFFFF, n_ev)   # malformed offsets: kept in range here,
            e1 = min(int(host_off[p1]) & 0xFFFFFFFF, n_ev)   # reported after the call
            spans.append((e0, e1))
            if e1 <= e0:
                ready.append(None)
                mx_ready.append(None)
                continue
            with torch.cuda.stream(copy_s):
                counts[e0:e1].copy_(vol_data[e0:e1], non_blocking=True)
                times[e0:e1].copy_(vol_times[e0:e1], non_blocking=True)
                done = torch.cuda.Event()
                done.record(copy_s)
            ready.append(done)
            with torch.cuda.stream(max_s):
                max_s.wait_event(done)
                part = counts[e0:e1]
                m = torch.amax(part if part.dtype == torch.uint8 else part.to(torch.int32)).to(torch.int32)
                mx_host[c].copy_(m, non_blocking=True)
                got = torch.cuda.Event()
                got.record(max_s)
            mx_ready.append(got)
        self._mark("start_pairs")
        mx_all, kinds = 0, set()
        for c, (p0, p1, pix, per) in enumerate(plans):
            e0, e1 = spans[c]
            if ready[c] is None:
                continue
            mx_ready[c].synchronize()                      # this chunk's counts are in: its largest
            mx = int(mx_host[c])
            mx_all = max(mx_all, mx)
            use_smem = self.T * 8 + PAIRS_SMEM_FIXED + 192 <= 227 * 1024 and self.T <= 65535 and mx * mx < 2 ** 31
            kind = "smem" if use_smem else "global"
            kinds.add(kind)
            ro, rb, cro, n_ranges, n_ctas = per[kind]
            cur.wait_event(ready[c])
            if n_ranges:
                _lib.check(self.lib.g2_event_pairsum(
                    ptr(times), ptr(counts), counts.element_size(), n_ev, ptr(offs), self.npix, ptr(pix),
                    ptr(ro), ptr(rb), n_ranges, ptr(cro), n_ctas, self.T, self.n_bins, mx, ptr(self.numer),
                    ptr(self.sums), ptr(self.err), st), "g2_event_pairsum")
        self._mark("pairsum")
        _lib.check(self.lib.g2_denominator(ptr(self.sums), self.n_bins, self.T, ptr(self.denom), st),
                   "g2_denominator")
        _lib.check(self.lib.g2_finalize(ptr(self.numer), ptr(self.denom), ptr(self.scale), self.n_bins,
                                        self.T, ptr(self.g2_f32), ptr(self.g2_f64), st), "g2_finalize")
        self._mark("normalize")
        self._host_refs = (vol_times, vol_data, offsets)  # alive until the copies have run
        self._times_checked = True
        self.last = {"n_events": n_ev, "max_count": mx_all,
                     "kernel": "smem" if kinds <= {"smem"} else ("global" if kinds == {"global"} else "mixed"),
                     "host_chunks": len(plans)}
        return self.g2_f32[: self.n_bins]

    def run_device(self, times, counts, offs, n_ev, mx, reset_error=True):
        """G6 + G3 + G4 on validated device events: ``times`` int32 with
        ``counts``, or packed words ``(t << 16) | v`` with ``counts=None``
        (``reset_error=False`` keeps the flags an earlier stage of the same
        call has set)."""
        self.numer.zero_()
        self.sums.zero_()
        if reset_error:
            self.err.zero_()
        st = stream_handle(self.dev)
        # the C side makes the same choice (shared counters for 2 x T frames,
        # times below 2^16, products below 2^31)
        use_smem = self.T * 8 + PAIRS_SMEM_FIXED + 192 <= 227 * 1024 and self.T <= 65535 and mx * mx < 2 ** 31
        ro, rb, cro, n_ranges, n_ctas = self.plans["smem" if use_smem else "global"]
        self._mark("start_pairs")
        if n_ranges and self.n_bins and n_ev and counts is None:     # packed words (t << 16) | v
            _lib.check(self.lib.g2_event_pairsum_packed(
                ptr(times), n_ev, ptr(offs), self.npix, ptr(self.pix_list), ptr(ro), ptr(rb), n_ranges, ptr(cro),
                n_ctas, self.T, self.n_bins, mx, ptr(self.numer), ptr(self.sums), ptr(self.err), st),
                "g2_event_pairsum_packed")
        elif n_ranges and self.n_bins and n_ev:
            _lib.check(self.lib.g2_event_pairsum(
                ptr(times), ptr(counts), counts.element_size(), n_ev, ptr(offs), self.npix, ptr(self.pix_list),
                ptr(ro), ptr(rb), n_ranges, ptr(cro), n_ctas, self.T, self.n_bins, mx, ptr(self.numer),
                ptr(self.sums), ptr(self.err), st), "g2_event_pairsum")
        self._mark("pairsum")
        if self.n_bins:
            _lib.check(self.lib.g2_denominator(ptr(self.sums), self.n_bins, self.T, ptr(self.denom), st),
                       "g2_denominator")
            _lib.check(self.lib.g2_finalize(ptr(self.numer), ptr(self.denom), ptr(self.scale), self.n_bins,
                                            self.T, ptr(self.g2_f32), ptr(self.g2_f64), st), "g2_finalize")
        self._mark("normalize")
        self.last = {"n_events": n_ev, "max_count": mx, "kernel": "smem" if use_smem else "global",
                     "n_ranges": n_ranges, "n_ctas": n_ctas}
        return self.g2_f32[: self.n_bins]

    def check_error(self):
        code = int(self.err.item())
        times_checked, csr_checked = getattr(self, "_times_checked", False), getattr(self, "_csr_checked", False)
        self._times_checked = self._csr_checked = False
        offsets_bad, self._offsets_bad = getattr(self, "_offsets_bad", None), None
        if offsets_bad is not None and int(offsets_bad.item()):
            raise ValueError("offsets must start at 0 and be non-decreasing")
        if code == _lib.DEVERR_BOUNDS and times_checked:
            raise ValueError("event times must lie in [0, nframes)")
        if code == _lib.DEVERR_BOUNDS and csr_checked:
            raise ValueError("malformed CSR stack: row pointers, or column indices outside [0, width) or not "
                             "increasing within a row")
        if code:
            raise DeviceError(_lib.device_error_message(code))


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
        self.scan_scratch = torch.zeros(max(1, -(-self.npix // 8192)), dtype=torch.int32, device=self.dev)
        self._ev_cap = 0
        self.last = {}

    ROW_MAX_W = 29000

    def packed_for(self, n):
        """Events travel as packed words (t << 16) | v: frames < 2^16, rows the
        row-owned kernels take (at most 29,000 pixels wide, 65,535 rows),
        fewer than 2^32 elements."""
        return self.T <= 65535 and self.shape[1] <= self.ROW_MAX_W and self.shape[0] <= 65535 and n < 2 ** 32

    def _counts_and_offsets(self, indices, indptr, offsets, ib, n):
        st = stream_handle(self.dev)
        H, W = self.shape
        self.counts.zero_()
        _lib.check(self.lib.g2_csr_count(ptr(indices), ptr(indptr), ptr(offsets), ib, n, self.T, H, W,
                                         ptr(self.counts), ptr(self.events.err), st), "g2_csr_count")
        _lib.check(self.lib.g2_exclusive_scan_u32(ptr(self.counts), self.npix, ptr(self.ev_off),
                                                  ptr(self.scan_scratch), self.scan_scratch.numel(), st),
                   "g2_exclusive_scan_u32")

    def _buffer(self, name, n, dtype):
        torch = _torch()
        buf = getattr(self, name, None)
        if buf is None or buf.numel() < max(n, 1) or buf.dtype != dtype:
            setattr(self, name, None)
            buf = torch.empty(max(n, 1), dtype=dtype, device=self.dev)
            setattr(self, name, buf)
        return buf

    SUBBLOCK = 1024
    TILE_P = 64

    def to_words(self, data, indices, indptr, offsets, ib, n, sort=False):
        """CSR on the device -> packed event words and event offsets (uint32
        as int32) on the device; requires :meth:`packed_for`.  Counts per
        (1024-frame sub-block, pixel) and per (sub-block, row), their scans,
        the stage pass (runs grouped by sub-block, row and pixel) and the
        gather pass (64-pixel tiles; each pixel's runs in sub-block order, in
        frame order inside each run with ``sort``, so the whole list is in
        frame order)."""
        torch = _torch()
        H, W = self.shape
        st = stream_handle(self.dev)
        self.events._mark("start_transpose")
        n_sb = -(-self.T // self.SUBBLOCK)
        n_rows = n_sb * H
        sbc = self._buffer("sb_counts", n_sb * self.npix, torch.int16)
        rb = self._buffer("row_bounds", (H + 1) * self.T, torch.int32)
        rt = self._buffer("row_totals", n_rows, torch.int32)
        base = self._buffer("row_base", n_rows + 1, torch.int32)
        rscr = self._buffer("row_scan_scratch", -(-n_rows // 8192), torch.int32)
        self.counts.zero_()
        _lib.check(self.lib.g2_csr_count_blocked(ptr(indices), ptr(indptr), ptr(offsets), ib, n, self.T, H, W,
                                                 ptr(rb), ptr(self.counts), ptr(sbc), ptr(rt),
                                                 ptr(self.events.err), st), "g2_csr_count_blocked")
        _lib.check(self.lib.g2_exclusive_scan_u32(ptr(self.counts), self.npix, ptr(self.ev_off),
                                                  ptr(self.scan_scratch), self.scan_scratch.numel(), st),
                   "g2_exclusive_scan_u32")
        _lib.check(self.lib.g2_exclusive_scan_u32(ptr(rt), n_rows, ptr(base), ptr(rscr), rscr.numel(), st),
                   "g2_exclusive_scan_u32")
        stage = self._buffer("stage_words", n, torch.int32)
        tpos = self._buffer("tile_pos", n_sb * -(-self.npix // self.TILE_P), torch.int32)
        _lib.check(self.lib.g2_csr_stage_blocked(ptr(data), data.element_size(), ptr(indices), ptr(rb), ib, n,
                                                 self.T, H, W, ptr(sbc), ptr(base), ptr(tpos), ptr(stage),
                                                 ptr(self.events.err), st), "g2_csr_stage_blocked")
        words = self._buffer("ev_words", n, torch.int32)
        _lib.check(self.lib.g2_csr_gather_blocked(ptr(stage), ptr(tpos), ptr(sbc), self.T, self.npix, n,
                                                  ptr(self.ev_off), 1 if sort else 0, ptr(words),
                                                  ptr(self.events.err), st), "g2_csr_gather_blocked")
        self.events._mark("transpose")
        return words, self.ev_off

    def to_events(self, data, indices, indptr, offsets, ib, n):
        """CSR on the device -> (times int32, counts, offsets) event lists on
        the device, in the FramesCompressor layout (frames ascending within a
        pixel when :meth:`packed_for` holds, else in an unspecified order)."""
        torch = _torch()
        self.events.err.zero_()
        times = self._buffer("ev_times", n, torch.int32)
        evdata = self._buffer("ev_data", n, data.dtype)
        if self.packed_for(n):
            words, off = self.to_words(data, indices, indptr, offsets, ib, n, sort=True)
            _lib.check(self.lib.g2_events_unpack(ptr(words), n, data.element_size(), ptr(times), ptr(evdata),
                                                 stream_handle(self.dev)), "g2_events_unpack")
            return times, evdata, off
        H, W = self.shape
        self.events._mark("start_transpose")
        self._counts_and_offsets(indices, indptr, offsets, ib, n)
        self.counts.zero_()                              # reused as the scatter cursor
        _lib.check(self.lib.g2_csr_scatter(ptr(data), data.element_size(), ptr(indices), ptr(indptr), ptr(offsets),
                                           ib, n, self.T, H, W, ptr(self.ev_off), ptr(self.counts),
                                           ptr(times), ptr(evdata), ptr(self.events.err), stream_handle(self.dev)),
                   "g2_csr_scatter")
        self.events._mark("transpose")
        return times, evdata, self.ev_off

    HOST_SB_PER_CHUNK = 4   # 1024-frame sub-blocks per copied frame group

    def host_pipeline_ok(self, data, indices, indptr, offsets):
        """Pinned host tensors (counts uint8/uint16; indices, row pointers and
        frame offsets all int32 or all int64) of a stack the packed
        transposition takes go through the frame-group pipeline."""
        torch = _torch()
        ts = (data, indices, indptr, offsets)
        if not all(isinstance(x, torch.Tensor) and not x.is_cuda and x.is_pinned() and x.is_contiguous()
                   and x.dim() == 1 for x in ts):
            return False
        H, W = self.shape
        return (data.dtype in (torch.uint8, torch.uint16) and indices.dtype in (torch.int32, torch.int64)
                and indptr.dtype == indices.dtype and offsets.dtype == indices.dtype
                and data.numel() == indices.numel() and indptr.numel() == (H + 1) * self.T
                and offsets.numel() == self.T + 1 and self.packed_for(data.numel()) and self.events.n_bins > 0)

    def _dev_buffer(self, name, like, n):
        torch = _torch()
        buf = getattr(self, name, None)
        if buf is None or buf.numel() < max(n, 1) or buf.dtype != like:
            setattr(self, name, None)
            buf = torch.empty(max(n, 1), dtype=like, device=self.dev)
            setattr(self, name, buf)
        return buf

    def run_host_pipelined(self, data, indices, indptr, offsets):
        """A CSR stack in pinned host memory, frame group by frame group: the
        copy of group g + 1 runs while group g is counted and staged (the
        staging bases continue across groups through a running carry); the
        gather, the pair sums and the normalisation follow.  Frame offsets are
        checked on the host; malformed rows or columns found by the kernels
        raise ValueError after the call."""
        torch = _torch()
        H, W = self.shape
        T, npix = self.T, self.npix
        n = int(data.numel())
        off_h = offsets.to(torch.int64)
        if int(off_h[0]) != 0 or bool(torch.any(off_h[1:] < off_h[:-1])) or int(off_h[-1]) > n:
            raise ValueError("frame offsets must start at 0, never decrease and stay within the elements")
        ib = indices.element_size()
        eb = data.element_size()
        cur = torch.cuda.current_stream(self.dev)
        copy_s = getattr(self, "_copy_stream", None)
        if copy_s is None:
            copy_s = self._copy_stream = torch.cuda.Stream(self.dev)
        d_data = self._dev_buffer("_h_data", data.dtype, n)
        d_ind = self._dev_buffer("_h_ind", indices.dtype, n)
        d_ip = self._dev_buffer("_h_ip", indptr.dtype, indptr.numel())
        d_off = self._dev_buffer("_h_off", offsets.dtype, offsets.numel())
        n_sb = -(-T // self.SUBBLOCK)
        n_tiles = -(-npix // self.TILE_P)
        G = self.HOST_SB_PER_CHUNK
        sbc = self._buffer("sb_counts", n_sb * npix, torch.int16)
        rt = self._buffer("row_totals", n_sb * H + 1, torch.int32)
        base = self._buffer("row_base", n_sb * H + 1, torch.int32)
        rscr = self._buffer("row_scan_scratch", -(-(G * H) // 8192) + 1, torch.int32)
        carry = self._buffer("row_carry", 1, torch.int32)
        rb = self._buffer("row_bounds_group", (H + 1) * min(T, G * self.SUBBLOCK), torch.int32)
        tpos = self._buffer("tile_pos", n_sb * n_tiles, torch.int32)
        stage = self._buffer("stage_words", n, torch.int32)
        err = self.events.err
        self.counts.zero_()
        carry.zero_()
        err.zero_()
        st = stream_handle(self.dev)
        start = torch.cuda.Event()
        start.record(cur)
        copy_s.wait_event(start)
        with torch.cuda.stream(copy_s):
            d_off.copy_(offsets, non_blocking=True)
        self.events._mark("start_transpose")
        addr = lambda t, k: C.c_void_p(t.data_ptr() + k * t.element_size())
        for sb0 in range(0, n_sb, G):
            f0, f1 = sb0 * self.SUBBLOCK, min(T, (sb0 + G) * self.SUBBLOCK)
            e0, e1 = int(off_h[f0]), int(off_h[f1])
            with torch.cuda.stream(copy_s):
                if e1 > e0:
                    d_ind[e0:e1].copy_(indices[e0:e1], non_blocking=True)
                    d_data[e0:e1].copy_(data[e0:e1], non_blocking=True)
                d_ip[f0 * (H + 1):f1 * (H + 1)].copy_(indptr[f0 * (H + 1):f1 * (H + 1)], non_blocking=True)
                done = torch.cuda.Event()
                done.record(copy_s)
            cur.wait_event(done)
            k = -(-(f1 - f0) // self.SUBBLOCK)
            _lib.check(self.lib.g2_csr_count_blocked(ptr(d_ind), addr(d_ip, f0 * (H + 1)), addr(d_off, f0), ib, n,
                                                     f1 - f0, H, W, ptr(rb), ptr(self.counts),
                                                     addr(sbc, sb0 * npix), addr(rt, sb0 * H), ptr(err), st),
                       "g2_csr_count_blocked")
            _lib.check(self.lib.g2_exclusive_scan_u32(addr(rt, sb0 * H), k * H, addr(base, sb0 * H), ptr(rscr),
                                                      rscr.numel(), st), "g2_exclusive_scan_u32")
            _lib.check(self.lib.g2_add_carry_u32(addr(base, sb0 * H), k * H, ptr(carry), st), "g2_add_carry_u32")
            _lib.check(self.lib.g2_csr_stage_frames(ptr(d_data), eb, ptr(d_ind), ptr(rb), ib, n, f0, f1 - f0,
                                                    e1 - e0, H, W, addr(sbc, sb0 * npix), addr(base, sb0 * H),
                                                    addr(tpos, sb0 * n_tiles), ptr(stage), ptr(err), st),
                       "g2_csr_stage_frames")
        _lib.check(self.lib.g2_exclusive_scan_u32(ptr(self.counts), npix, ptr(self.ev_off), ptr(self.scan_scratch),
                                                  self.scan_scratch.numel(), st), "g2_exclusive_scan_u32")
        words = self._buffer("ev_words", n, torch.int32)
        _lib.check(self.lib.g2_csr_gather_blocked(ptr(stage), ptr(tpos), ptr(sbc), T, npix, n, ptr(self.ev_off), 0,
                                                  ptr(words), ptr(err), st), "g2_csr_gather_blocked")
        self.events._mark("transpose")
        mx = int(d_data[:n].to(torch.int32).max().item()) if n else 0
        self._host_refs = (data, indices, indptr, offsets)
        out = self.events.run_device(words, None, self.ev_off, n, mx, reset_error=False)
        self.events._csr_checked = True
        self.last = dict(self.events.last, n_elements=n, packed=True, host_sb_per_chunk=G)
        return out

    def run(self, data, indices, indptr, offsets):
        if self.host_pipeline_ok(data, indices, indptr, offsets):
            return self.run_host_pipelined(data, indices, indptr, offsets)
        counts, ind, ip, off, ib, n, mx = csr_to_device(data, indices, indptr, offsets, self.shape, self.T,
                                                        self.dev)
        packed = self.packed_for(n)
        if packed:
            self.events.err.zero_()
            words, evoff = self.to_words(counts, ind, ip, off, ib, n)
            out = self.events.run_device(words, None, evoff, n, mx, reset_error=False)
        else:
            times, evdata, evoff = self.to_events(counts, ind, ip, off, ib, n)
            out = self.events.run_device(times, evdata, evoff, n, mx, reset_error=False)
        self.last = dict(self.events.last, n_elements=n, packed=packed)
        return out

    def check_error(self):
        self.events.check_error()
