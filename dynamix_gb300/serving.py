"""Continuous-batching g2 service on one GPU.

Correlation jobs (a dense ``(T, H, W)`` stack and its q-mask, any frame shape
and length) arrive while others run.  The server

* admits a job when one of its ``max_active`` slots and enough of its HBM
  budget are free (the budget covers the job's frames while they are on the
  device and its packed operand; the frames are released as soon as they are
  packed);
* copies the frames in (when they come from host memory) and packs them on a
  side stream, while the tensor cores work on the jobs admitted earlier;
* runs the Gram work of all active jobs as a sequence of grouped persistent
  launches (``g2_gram_tc_pair`` takes up to ``G2_MAX_JOBS`` jobs per launch): each
  launch takes a slice of the active jobs' tiles -- oldest job first while
  few jobs are in the server, so that below saturation each finishes about
  as soon as it would alone; shortest remaining first, with a share for
  every job, once the backlog grows, so a short job that arrives behind long
  ones finishes in a few launches instead of waiting for them;
* finishes a job whose last tiles were launched (denominator and g2 on the
  compute stream, results copied to pinned host memory) and hands the result
  to the caller.

N and S of all active jobs live in two int64 arenas, so that one launch
addresses every job's sums through one base pointer.  Results are exact
(integer N, S, D) and therefore identical whether a job runs alone or in a
mix.

There is no reference counterpart: dynamix correlates one stack per call
(``correlator/dense.py:118-142``).  Each job computes exactly what
``MatMulCorrelator.correlate`` computes (g2 normalised by the bin's pixel
count unless a scale factor is given).
"""
from __future__ import annotations

import collections
import itertools
import threading
import time

import numpy as np

from . import _lib
from .engine import (DenseEngine, DeviceError, _torch, device_layout, frames_to_device, ptr, require_cuda,
                     stream_handle)
from .plan import MODE_BYTES, MODE_E4M3, MODE_FP16, TILE_SHAPES, gram_items



class ArenaFull(Exception):
    pass


class Arena:
    """First-fit allocator of element ranges in a fixed device array."""

    def __init__(self, n):
        self.n = int(n)
        self.free = [(0, self.n)]          # sorted (start, length)

    def alloc(self, k):
        k = int(k)
        for i, (s, ln) in enumerate(self.free):
            if ln >= k:
                if ln == k:
                    self.free.pop(i)
                else:
                    self.free[i] = (s + k, ln - k)
                return s
        raise ArenaFull(k)

    def release(self, s, k):
        self.free.append((int(s), int(k)))
        self.free.sort()
        merged = []
        for s0, l0 in self.free:
            if merged and merged[-1][0] + merged[-1][1] == s0:
                merged[-1] = (merged[-1][0], merged[-1][1] + l0)
            else:
                merged.append((s0, l0))
        self.free = merged

    @property
    def used(self):
        return self.n - sum(ln for _, ln in self.free)


def plan_slice(remaining, item_ops, next_items, slice_ops, policy="srpt", age=None):
    """Items each active job contributes to one grouped launch.

    ``remaining[j]``: int ops job j still needs; ``item_ops[j]``: ops of each of
    its items (launch order); ``next_items[j]``: its first item not launched.

    ``policy="srpt"``: jobs are served shortest remaining first; a job gets
    what is left of ``slice_ops`` but at least ``slice_ops / (2 n)`` and at
    least one item, so every job advances in every launch.
    ``policy="fifo"``: jobs are served oldest first (ascending ``age``, e.g.
    submission times); the oldest takes up to the whole slice and what it
    leaves goes to the next, so a launch holds more than one job only where a
    job ends inside the slice (at least one item of the oldest job), and jobs
    finish in age order.

    Returns ``(job, n_items, ops)`` in service order, jobs with nothing left
    omitted."""
    n = len(remaining)
    if n == 0:
        return []
    if policy == "fifo":
        key = (lambda j: (age[j], j)) if age is not None else (lambda j: j)
        floor = 0.0
    elif policy == "srpt":
        key = lambda j: (remaining[j], j)   # noqa: E731
        floor = float(slice_ops) / (2 * n)
    else:
        raise ValueError("unknown slice policy %r" % (policy,))
    left = float(slice_ops)
    out = []
    for j in sorted(range(n), key=key):
        k0 = int(next_items[j])
        ops = np.asarray(item_ops[j], dtype=np.float64)[k0:]
        if ops.size == 0:
            continue
        cum = np.cumsum(ops)
        k = int(np.searchsorted(cum, max(left, floor), side="right"))
        if policy == "fifo" and out:
            if k == 0:                      # the rest of the slice holds no item of the next job
                break
        else:
            k = min(max(1, k), ops.size)    # the first job (fifo) and every job (srpt) advance
        out.append((j, k, float(cum[k - 1])))
        left -= float(cum[k - 1])
        if policy == "fifo" and k < ops.size:
            break                           # the next job waits for this one's remaining items
    return out


def slice_policy(n_backlog, fifo_max):
    """The slice policy for ``n_backlog`` jobs in the server (queued, packing
    or running): oldest first while the backlog is short -- below saturation
    every job then finishes about as soon as it would alone, and the longest
    job is not pushed back again and again by shorter arrivals -- and
    shortest remaining first once it grows past ``fifo_max``, when short jobs
    would otherwise wait behind long ones."""
    return "fifo" if n_backlog <= fifo_max else "srpt"


def admit_order(needs, used, budget, free_slots):
    """Indices of queued jobs (in arrival order, ``needs`` = their bytes) that
    can start now: first fit in arrival order under ``budget`` with ``used``
    bytes held and ``free_slots`` slots; a job larger than the whole budget is
    reported separately.  Returns ``(admit, too_large)``."""
    admit, too_large = [], []
    for i, need in enumerate(needs):
        if need > budget:
            too_large.append(i)
            continue
        if len(admit) >= free_slots:
            break
        if used + need <= budget:
            admit.append(i)
            used += need
    return admit, too_large


class Request:
    """Handle of a submitted job.  ``wait()`` blocks until the result is there;
    ``g2`` (float32 ``(n_bins, T)``), ``numerator``, ``sums``, ``denominator``
    (int64) are host arrays afterwards; ``latency`` is seconds from submission
    to result."""

    _ids = itertools.count()

    def __init__(self, frames, qmask, scale_factor):
        self.id = next(self._ids)
        self.frames = frames
        self.qmask = qmask
        self.scale_factor = scale_factor
        self.t_submit = time.perf_counter()
        self.t_admit = None
        self.t_done = None
        self.error = None
        self.g2 = self.numerator = self.sums = self.denominator = None
        self.info = {}
        self._done = threading.Event()

    @property
    def latency(self):
        return None if self.t_done is None else self.t_done - self.t_submit

    def done(self):
        return self._done.is_set()

    def wait(self, timeout=None):
        if not self._done.wait(timeout):
            raise TimeoutError("job %d not finished" % self.id)
        if self.error is not None:
            raise self.error
        return self.g2


class _Job:
    """Server-side state of one request."""

    def __init__(self, req, shape, T, qmask, n_bins, scale, elem_bytes, from_host):
        self.req = req
        self.shape = shape
        self.T = T
        self.qmask = qmask
        self.n_bins = n_bins
        self.scale = scale
        self.elem_bytes = elem_bytes
        self.from_host = from_host
        self.engine = None
        self.layout = None
        self.items = None          # numpy ITEM_DTYPE, job field rewritten per launch
        self.item_ops = None       # int ops of each item
        self.next_item = 0
        self.remaining_ops = 0
        self.arena_off = None
        self.staging_off = None    # 256-byte units into the staging arena (pinned host frames)
        self.reserved = 0          # bytes of the HBM budget held
        self.frames_dev = None
        self.mode = None
        self.pack_event = None
        self.host_err = None
        self.host_emax = None
        self.host_out = None
        self.done_event = None

    @property
    def rows(self):
        return max(self.n_bins, 1)


class G2Server:
    """See the module docstring.  ``hbm_budget``: bytes of device memory the
    server may hold for admitted jobs (frames in flight + packed operands);
    ``arena_elems``: int64 elements of each of the N and S arenas (the sum of
    ``n_bins * T`` over the active jobs must fit); ``slice_ops``: tensor-core
    int ops per grouped launch; ``policy``: ``"auto"`` (oldest first while at
    most ``fifo_max`` jobs are queued, packing or running, shortest remaining
    first beyond; :func:`slice_policy`), ``"fifo"`` or ``"srpt"``;
    ``staging_bytes``: device bytes of the staging arena that frames copied
    from page-locked host memory land in until they are packed (allocated at
    the first such job; a job larger than it gets its own buffer)."""

    def __init__(self, hbm_budget=150e9, max_active=_lib.MAX_JOBS, arena_elems=1 << 25, slice_ops=2e13,
                 device=None, method="tc", policy="auto", fifo_max=4, staging_bytes=48e9):
        torch = _torch()
        self.lib = _lib.load()
        self.dev = require_cuda(device)
        self.budget = int(hbm_budget)
        self.max_active = min(int(max_active), _lib.MAX_JOBS)
        self.slice_ops = float(slice_ops)
        self.method = method
        # tensor-core launches run 256 x 256 blocks on CTA pairs (g2_gram_tc_pair)
        self.kind = "pair" if method == "tc" else method
        bm, bn = TILE_SHAPES[self.kind]
        self.ops_per_col = 2.0 * bm * bn           # int ops of one block per unit of k_len
        if policy not in ("auto", "fifo", "srpt"):
            raise ValueError("unknown slice policy %r" % (policy,))
        self.policy = policy
        self.fifo_max = int(fifo_max)
        self.arena = Arena(arena_elems)
        # frames copied in from page-locked host memory live in one staging
        # arena (first-fit ranges, 256-byte aligned) until packed, so that jobs
        # of every size reuse the same device memory instead of allocating and
        # freeing tens of GB each
        self.staging_bytes = int(staging_bytes) // 256 * 256
        self.staging = None
        self.staging_arena = Arena(self.staging_bytes // 256)
        self.numer_arena = torch.zeros(int(arena_elems), dtype=torch.int64, device=self.dev)
        self.sums_arena = torch.zeros(int(arena_elems), dtype=torch.int64, device=self.dev)
        self.err = torch.zeros(1, dtype=torch.int32, device=self.dev)
        self.compute = torch.cuda.Stream(self.dev)
        self.side = torch.cuda.Stream(self.dev)
        self.queue = collections.deque()
        self.active = []
        self.finishing = []
        self._inflight = []        # (event, pinned items, device items, jobs) per grouped launch
        self.used = 0
        self.lock = threading.Lock()
        self._params_cache = {}    # (shape, qmask digest, scale) -> (qmask, n_bins, scale, digest)
        self._digest_cache = {}    # (id(qmask), H, W) -> (qmask, digest)
        self.packing = []          # jobs whose copy-in / packing is in flight
        self.stats = {"launches": 0, "items": 0, "admitted": 0, "finished": 0, "max_active": 0,
                      "max_used_bytes": 0, "fifo_launches": 0, "srpt_launches": 0}
        self._thread = None
        self._stop = False

    # -- client side -----------------------------------------------------
    def submit(self, frames, qmask=None, scale_factor=None):
        """Queue a job; ``frames`` (T, H, W) u8/u16 as a CUDA tensor (used in
        place), a CPU tensor (pinned memory gives an asynchronous copy) or a
        numpy array.  Returns a :class:`Request`."""
        req = Request(frames, qmask, scale_factor)
        with self.lock:
            self.queue.append(req)
        return req

    def start(self):
        """Serve from a background thread until :meth:`stop`."""
        self._stop = False
        self._thread = threading.Thread(target=self._loop, daemon=True)
        self._thread.start()

    def stop(self):
        self._stop = True
        if self._thread is not None:
            self._thread.join()
            self._thread = None

    def _loop(self):
        torch = _torch()
        torch.cuda.set_device(self.dev)
        while not self._stop:
            if not self.step():
                time.sleep(0.0002)

    def idle(self):
        with self.lock:
            return not (self.queue or self.packing or self.active or self.finishing or self._inflight)

    def run_until_idle(self):
        while not self.idle():
            if not self.step():
                time.sleep(0.0002)

    # -- scheduling --------------------------------------------------------
    def step(self):
        """One scheduling round: launch the next grouped Gram slice, start the
        copy-in and packing of newly admitted jobs (asynchronous, side stream),
        promote jobs whose packing finished, hand over finished results.
        Returns True when it did any work."""
        launched = self._launch_slice()
        admitted = self._admit()
        packed = self._poll_packs()
        reaped = self._reap()
        return launched or admitted or packed or reaped

    def _params(self, req):
        """(shape, T, qmask int32, n_bins, scale) of a request, cached per q-mask."""
        import hashlib

        from .correlator.common import BaseCorrelator
        fr = req.frames
        if fr is None or len(getattr(fr, "shape", ())) != 3:
            raise ValueError("frames must be a (T, H, W) stack")
        T, H, W = (int(x) for x in fr.shape)
        qm = None if req.qmask is None else np.ascontiguousarray(req.qmask, dtype=np.int32)
        # the same q-mask object is usually submitted again: hash it once
        ident = (id(req.qmask), H, W)
        cached = self._digest_cache.get(ident)
        if cached is not None and cached[0] is req.qmask:
            digest = cached[1]
        else:
            digest = hashlib.blake2b(qm.tobytes() if qm is not None else b"all", digest_size=16).hexdigest()
            if len(self._digest_cache) > 256:
                self._digest_cache.clear()
            self._digest_cache[ident] = (req.qmask, digest)
        sf = req.scale_factor
        key = (H, W, digest, None if sf is None else repr(sf))
        if key not in self._params_cache:
            bc = BaseCorrelator()
            if qm is None:
                bc._set_parameters((H, W), T, None, sf, {})
            else:
                if qm.shape != (H, W):
                    raise ValueError("qmask shape %s does not match frame shape %s" % (qm.shape, (H, W)))
                bc._set_shape((H, W))
                bc.nframes = T
                bc.qmask = qm
                bc.n_bins = int(qm.max()) if qm.size else 0
                bc.bins = np.arange(1, bc.n_bins + 1, dtype=np.int32)
                if sf is None:
                    cnt = np.bincount(qm.ravel()[qm.ravel() > 0], minlength=bc.n_bins + 1)
                    bc.scale_factors = {b: int(cnt[b]) for b in bc.bins}
                else:
                    bc._set_scale_factor(sf)
            if len(self._params_cache) > 64:
                self._params_cache.clear()
            self._params_cache[key] = (bc.qmask, bc.n_bins, bc._scale_array(), "%s:%s" % ((H, W), digest))
        qmask, n_bins, scale, qd = self._params_cache[key]
        return (H, W), T, qmask, n_bins, scale, qd

    def _estimate(self, job):
        """Bytes of the budget a job needs at its peak: frames copied to the
        device plus the widest packed operand its counts may need."""
        cols = (device_layout(job.qmask, job.n_bins, MODE_FP16, self.dev, job.qdigest).packed_cols
                if job.n_bins else 0)
        frames = job.T * job.shape[0] * job.shape[1] * job.elem_bytes if job.from_host else 0
        return frames + (job.T + 1) * cols * (2 if job.elem_bytes == 1 else 4)

    def _make_job(self, req):
        """Server-side job of a request (built once, kept on the request)."""
        torch = _torch()
        if getattr(req, "_job", None) is None:
            shape, T, qmask, n_bins, scale, qd = self._params(req)
            fr = req.frames
            from_host = not (isinstance(fr, torch.Tensor) and fr.is_cuda)
            dt = fr.dtype if isinstance(fr, torch.Tensor) else np.asarray(fr).dtype
            elem = 1 if dt in (torch.uint8, np.uint8) else 2     # other integer types become u8 or u16
            job = _Job(req, shape, T, qmask, n_bins, scale, elem, from_host)
            job.qdigest = qd if req.qmask is not None else None
            req._job = (job, self._estimate(job))
        return req._job

    def _admit(self):
        with self.lock:
            pending = list(self.queue)
        free = self.max_active - len(self.active) - len(self.finishing) - len(self.packing)
        if not pending or free <= 0:
            return False
        cands = []
        for req in pending:
            try:
                cands.append((req,) + self._make_job(req))
            except Exception as e:                 # malformed request: fail it, keep serving
                self._dequeue(req)
                self._fail(req, e)
        admit, too_large = admit_order([c[2] for c in cands], self.used, self.budget, free)
        for i in too_large:
            req, job, need = cands[i]
            self._dequeue(req)
            self._fail(req, MemoryError("job needs %.1f GB, the budget is %.1f GB" % (need / 1e9,
                                                                                      self.budget / 1e9)))
        admitted = False
        for i in admit:
            req, job, need = cands[i]
            try:
                job.arena_off = self.arena.alloc(job.rows * job.T)
            except ArenaFull:
                continue                           # stays queued until sums space frees up
            if self._stageable(req):
                units = -(-self._frame_bytes(job) // 256)
                if units <= self.staging_arena.n:
                    try:
                        job.staging_off = self.staging_arena.alloc(units)
                    except ArenaFull:              # stays queued until staging space frees up
                        self.arena.release(job.arena_off, job.rows * job.T)
                        job.arena_off = None
                        continue
            self._dequeue(req)
            job.reserved = need
            self.used += need
            try:
                self._start(job)
            except Exception as e:
                self._release(job)
                self._fail(req, e)
                continue
            admitted = True
        return admitted

    @staticmethod
    def _stageable(req):
        """Frames in page-locked host memory, copied asynchronously."""
        torch = _torch()
        fr = req.frames
        return (isinstance(fr, torch.Tensor) and not fr.is_cuda and fr.dtype in (torch.uint8, torch.uint16)
                and fr.is_pinned() and fr.is_contiguous())

    @staticmethod
    def _frame_bytes(job):
        return job.T * job.shape[0] * job.shape[1] * job.elem_bytes

    def _staged_frames(self, job, fr):
        """The device tensor a pinned host stack is copied into: its range of
        the staging arena, or a buffer of its own."""
        torch = _torch()
        if job.staging_off is None:
            return torch.empty(fr.shape, dtype=fr.dtype, device=self.dev)
        if self.staging is None:
            self.staging = torch.empty(self.staging_bytes, dtype=torch.uint8, device=self.dev)
        off = job.staging_off * 256
        raw = self.staging[off:off + self._frame_bytes(job)]
        return raw.view(fr.dtype).view(fr.shape)

    def _release_staging(self, job):
        if job.staging_off is not None:
            self.staging_arena.release(job.staging_off, -(-self._frame_bytes(job) // 256))
            job.staging_off = None

    def _dequeue(self, req):
        with self.lock:
            if req in self.queue:
                self.queue.remove(req)

    def _start(self, job):
        """Queue the frames' copy-in and the packing on the side stream; the
        error word (and, for fp16 operands, the segment energies) follow to
        pinned host memory, and :meth:`_poll_packs` plans the job's tiles once
        they have arrived -- the host never waits for the GPU here."""
        torch = _torch()
        req = job.req
        req.t_admit = time.perf_counter()
        off, n = job.arena_off, job.rows * job.T
        numer = self.numer_arena[off:off + n].view(job.rows, job.T)
        sums = self.sums_arena[off:off + n].view(job.rows, job.T)
        with torch.cuda.stream(self.side):
            numer.zero_()                           # the pack zeroes the sums
            fr = req.frames
            if self._stageable(req):
                frames_dev = self._staged_frames(job, fr)
                frames_dev.copy_(fr, non_blocking=True)         # asynchronous on the side stream
            else:
                frames_dev = frames_to_device(fr, self.dev)      # validates, converts, or uses in place
            job.frames_dev = frames_dev
            job.engine = DenseEngine(job.shape, job.T, job.qmask, job.n_bins, job.scale, device=self.dev,
                                     method=self.method, numer=numer, sums=sums, qmask_digest=job.qdigest)
            # the pack's error word is read after the frames are released: the
            # kernel that checks every count exactly is the one that fits
            job.engine.pack_units = False
        req.frames = None                           # the server keeps no reference to the input
        if job.n_bins == 0:
            self._promote(job, np.empty(0, dtype=_lib.ITEM_DTYPE))
            return
        job.mode = job.engine.choose_mode(frames_dev)
        self._launch_pack(job)
        self.packing.append(job)

    def _launch_pack(self, job):
        torch = _torch()
        eng = job.engine
        with torch.cuda.stream(self.side):
            L = eng.pack(job.frames_dev, job.mode)
            job.layout = L
            job.host_err = torch.empty(1, dtype=torch.int32, pin_memory=True)
            job.host_err.copy_(eng.err, non_blocking=True)
            job.host_emax = None
            if job.mode != MODE_E4M3:
                emax = eng._piece_emax(L)
                job.host_emax = torch.empty(emax.numel(), dtype=torch.int32, pin_memory=True)
                job.host_emax.copy_(emax, non_blocking=True)
            job.pack_event = torch.cuda.Event()
            job.pack_event.record(self.side)

    def _poll_packs(self):
        """Plan the tiles of every job whose packing has finished (a count
        that does not fit the operand repacks wider)."""
        from .plan import chunk_grams, e4m3_segment_bound
        done = [j for j in self.packing if j.pack_event.query()]
        for job in done:
            self.packing.remove(job)
            eng, L = job.engine, job.layout
            try:
                code = int(job.host_err[0])
                wider = {MODE_E4M3: MODE_FP16, MODE_FP16: MODE_BYTES}.get(job.mode)
                if code & _lib.DEVERR_RANGE and wider is not None:
                    job.mode = wider
                    self._launch_pack(job)
                    self.packing.append(job)
                    continue
                if code:
                    raise DeviceError(_lib.device_error_message(code))
                if job.mode == MODE_E4M3:
                    seg_emax = e4m3_segment_bound(L)
                else:
                    seg_emax = L.segment_emax(job.host_emax.numpy().view(np.uint32))
                try:
                    grams = chunk_grams(L, seg_emax, eng.exact_limit)
                except OverflowError:
                    if job.mode == MODE_BYTES:
                        raise
                    job.mode = MODE_BYTES
                    self._launch_pack(job)
                    self.packing.append(job)
                    continue
                off = job.arena_off
                items = gram_items(job.T, grams, job=0, out_base=off, kind=self.kind,
                                   s_base=off if (eng.ones(L) and self.method == "tc") else None)
            except Exception as e:
                self._release(job)
                self._fail(job.req, e)
                continue
            self.compute.wait_event(job.pack_event)
            self._promote(job, items)
        return bool(done)

    def _promote(self, job, items):
        """A packed job joins the grouped launches."""
        eng = job.engine
        job.frames_dev = None                      # packed: the frames are no longer needed
        self._release_staging(job)                 # the pack that read them has completed
        if eng.packed is not None:
            eng.packed.record_stream(self.compute)
        packed_bytes = 0 if eng.packed is None else eng.packed.numel()
        self.used -= job.reserved
        job.reserved = packed_bytes
        self.used += packed_bytes
        job.items = items
        job.item_ops = items["k_len"].astype(np.float64) * self.ops_per_col
        job.remaining_ops = float(job.item_ops.sum())
        job.next_item = 0
        job.req.info.update(mode=None if job.layout is None else ["fp16", "bytes", "e4m3"][job.layout.mode],
                            n_items=int(items.size), packed_bytes=int(packed_bytes))
        self.active.append(job)
        if items.size == 0:
            self._finish(job)                       # no binned pixel: nothing to correlate
        self.stats["admitted"] += 1
        self.stats["max_active"] = max(self.stats["max_active"], len(self.active))
        self.stats["max_used_bytes"] = max(self.stats["max_used_bytes"], self.used)

    def _launch_slice(self):
        """One grouped persistent launch over a slice of every active job's
        tiles (shortest remaining job first; each job gets at least
        1 / (2 n_active) of the slice so none starves)."""
        torch = _torch()
        self._retire_launches()
        if not self.active or len(self._inflight) >= 2:
            return False
        act = self.active
        policy = self.policy
        if policy == "auto":
            with self.lock:
                queued = len(self.queue)
            policy = slice_policy(queued + len(self.packing) + len(act), self.fifo_max)
        plan = plan_slice([j.remaining_ops for j in act], [j.item_ops for j in act], [j.next_item for j in act],
                          self.slice_ops, policy=policy, age=[(j.req.t_submit, j.req.id) for j in act])
        parts, jobs, taken = [], [], []
        for idx, k, ops in plan:
            job = act[idx]
            it = job.items[job.next_item:job.next_item + k].copy()
            it["job"] = len(jobs)
            parts.append(it)
            L = job.layout
            jobs.append((job.engine.packed.data_ptr(), job.T, L.packed_cols, L.kind, job.engine.ones(L)))
            taken.append((job, k, ops))
        if not parts:
            return False
        items = np.concatenate(parts)
        items = items[np.argsort(-items["k_len"].astype(np.int64), kind="stable")]
        host = torch.from_numpy(items.view(np.uint8).copy()).pin_memory()
        with torch.cuda.stream(self.compute):
            dev_items = torch.empty(host.numel(), dtype=torch.uint8, device=self.dev)
            dev_items.copy_(host, non_blocking=True)
            jarr = _lib.jobs_array(jobs)
            st = stream_handle(self.dev)
            if self.method == "tc":
                _lib.check(self.lib.g2_gram_tc_pair(jarr, len(jobs), ptr(dev_items), items.size,
                                                    ptr(self.numer_arena), self.numer_arena.numel(),
                                                    ptr(self.sums_arena), self.sums_arena.numel(), ptr(self.err), 0,
                                                    st), "g2_gram_tc_pair")
            else:                                   # the CUDA-core comparator, same items and sums
                _lib.check(self.lib.g2_plain_direct(jarr, len(jobs), ptr(dev_items), items.size,
                                                    ptr(self.numer_arena), self.numer_arena.numel(), ptr(self.err),
                                                    st), "g2_plain_direct")
            ev = torch.cuda.Event()
            ev.record(self.compute)
        members = []
        for job, k, ops in taken:
            job.next_item += k
            job.remaining_ops -= ops
            members.append(job)
        self._inflight.append((ev, host, dev_items, members))
        self.stats["launches"] += 1
        self.stats[policy + "_launches"] += 1
        self.stats["items"] += int(items.size)
        for job in [j for j in self.active if j.next_item >= j.items.size]:
            self._finish(job)
        return True

    def _retire_launches(self):
        """Drop launches that completed; a raised device error flag fails the
        jobs of that launch."""
        keep = []
        for rec in self._inflight:
            ev, host, dev_items, members = rec
            if ev.query():
                code = int(self.err.item())
                if code:
                    self.err.zero_()
                    for job in members:
                        job.req.info["device_error"] = code
            else:
                keep.append(rec)
        self._inflight = keep

    def _finish(self, job):
        """Denominator, g2 and the copies to pinned host memory, queued on the
        compute stream after the job's last tiles."""
        torch = _torch()
        self.active.remove(job)
        eng = job.engine
        with torch.cuda.stream(self.compute):
            if job.n_bins:
                eng.normalise()
            rows = job.rows
            out = {k: torch.empty((rows, job.T), dtype=dt, pin_memory=True) for k, dt in
                   (("g2", torch.float32), ("numerator", torch.int64), ("sums", torch.int64),
                    ("denominator", torch.int64))}
            for k, src in (("g2", eng.g2_f32), ("numerator", eng.numer), ("sums", eng.sums),
                           ("denominator", eng.denom)):
                out[k].copy_(src, non_blocking=True)
            job.done_event = torch.cuda.Event()
            job.done_event.record(self.compute)
        job.host_out = out
        eng.packed = None                        # freed once the compute stream is past it
        self.used -= job.reserved
        job.reserved = 0
        self.finishing.append(job)

    def _reap(self):
        done = [j for j in self.finishing if j.done_event.query()]
        for job in done:
            self.finishing.remove(job)
            req = job.req
            out = job.host_out
            nb = job.n_bins
            req.g2 = out["g2"].numpy()[:nb]
            req.numerator = out["numerator"].numpy()[:nb]
            req.sums = out["sums"].numpy()[:nb]
            req.denominator = out["denominator"].numpy()[:nb]
            code = req.info.get("device_error", 0) | int(job.engine.err.item())
            if code:
                req.error = DeviceError(_lib.device_error_message(code))
            elif nb and req.sums.size and float(req.sums.max()) ** 2 * job.T >= 2.0 ** 63:
                req.error = OverflowError("denominator exceeds int64 for these counts")
            self._release(job)
            req.t_done = time.perf_counter()
            self.stats["finished"] += 1
            req._done.set()
        return bool(done)

    def _release(self, job):
        job.frames_dev = None
        self._release_staging(job)
        if job.arena_off is not None:
            self.arena.release(job.arena_off, job.rows * job.T)
            job.arena_off = None
        self.used -= job.reserved
        job.reserved = 0
        job.engine = None

    def _fail(self, req, err):
        req.error = err
        req.t_done = time.perf_counter()
        req._done.set()
