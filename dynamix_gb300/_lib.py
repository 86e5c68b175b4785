"""ctypes binding of the C ABI in ``include/dynamix_g2.h``.

The library is built in-tree (``python -m dynamix_gb300.build``) at
``dynamix_gb300/_lib/libdynamix_g2.so``.  There is no fallback: if the library
is missing, every correlator raises at construction.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libdynamix_g2.so")

G2_OK = 0
STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA runtime error", 3: "unsupported device or feature",
          4: "size exceeds a kernel limit"}
DEVERR_TIMEOUT, DEVERR_BOUNDS, DEVERR_RANGE, DEVERR_RANGE_CHECK = 1, 2, 4, 8

BK = 64          # source segment width (pixels)
PAD = 128        # packed bins and packed_cols are multiples of this
PACK_CHUNK, PACK_MAX_SLOTS, PACK_MAX_PIECES, PACK_WORDS_PER_CHUNK = 2048, 128, 512, 768
TC_BM, TC_BN = 128, 256
PLAIN_BM, PLAIN_BN = 128, 128
MAX_JOBS = 32
ITEM_EMPTY = -1
KIND_FP16, KIND_E4M3 = 0, 1

# numpy mirror of g2_gram_item (48 bytes, 8-byte aligned)
ITEM_DTYPE = np.dtype([("job", "<i4"), ("i0", "<i4"), ("j0", "<i4"), ("a_k0", "<i4"), ("b_k0", "<i4"),
                       ("k_len", "<i4"), ("shift", "<i4"), ("nframes", "<i4"), ("out_off", "<i8"),
                       ("s_off", "<i8")])
assert ITEM_DTYPE.itemsize == 48


class Job(C.Structure):
    _fields_ = [("packed_dev", C.c_void_p), ("nframes", C.c_int64), ("packed_cols", C.c_int64),
                ("elem_kind", C.c_int32), ("ones_row", C.c_int32)]


_p = C.c_void_p
_i32 = C.c_int32
_i64 = C.c_int64

# name -> (restype, argtypes); every symbol declared in include/dynamix_g2.h
SIGNATURES = {
    "g2_abi_version": (C.c_int, []),
    "g2_status_string": (C.c_char_p, [C.c_int]),
    "g2_device_info": (C.c_int, [C.c_int, _p, _p, _p]),
    "g2_balance_lpt": (C.c_int, [_p, _i64, _i32, _p, _p]),
    "g2_copy_cols_h2d": (C.c_int, [_p, _p, _i64, _i64, _i64, _i64, _p]),
    "g2_pack_frames": (C.c_int, [_p, _i32, _i64, _i64, _p, _p, _p, _p, _p, _p, _i64, _i32, _p, _i64, _p, _i32, _p,
                                 _i64, _p, _p]),
    "g2_pack_e4m3": (C.c_int, [_p, _i32, _i64, _i64, _p, _p, _p, _i64, _p, _i64, _p, _p]),
    "g2_binned_max": (C.c_int, [_p, _i32, _i64, _i64, _p, _i64, _p, _p]),
    "g2_pack_e4m3_units": (C.c_int, [_p, _i64, _i64, _p, _p, _i64, _p, _i64, _p, _p]),
    "g2_gram_tc": (C.c_int, [_p, _i32, _p, _i64, _p, _i64, _p, _i64, _p, _i32, _p]),
    "g2_gram_tc_pair": (C.c_int, [_p, _i32, _p, _i64, _p, _i64, _p, _i64, _p, _i32, _p]),
    "g2_gram_tc_wide": (C.c_int, [_p, _i32, _p, _i64, _p, _i64, _p, _i64, _p, _i32, _p]),
    "g2_gram_workers": (C.c_int, [_i32, _p]),
    "g2_plain_direct": (C.c_int, [_p, _i32, _p, _i64, _p, _i64, _p, _p]),
    "g2_plain_dp4a": (C.c_int, [_p, _i32, _p, _i64, _p, _i64, _p, _i64, _p, _p]),
    "g2_tc_rate_probe": (C.c_int, [_i32, _i64, _i32, _p, _p]),
    "g2_gram_std": (C.c_int, [_p, _i32, _p, _i64, _p, _i64, _p, _p, _p, _p, _i64, _p, _i32, _p]),
    "g2_std_finalize": (C.c_int, [_p, _p, _p, _i32, _i64, _p, _p, _p]),
    "g2_gram_matrix": (C.c_int, [_p, _i32, _p, _i64, _p, _i64, _i64, _i32, _p, _i32, _p]),
    "g2_matrix_deviation": (C.c_int, [_p, _i64, _i64, _p, C.c_double, _p, _p, _p, _p, _p]),
    "g2_gram_ttcf": (C.c_int, [_p, _i32, _p, _i64, _p, _i64, _p, _i64, _i64, _i32, _p, _i32, _p]),
    "g2_ttcf_finish": (C.c_int, [_p, _i64, _i64, _p, _i32, _p]),
    "g2_event_pairsum": (C.c_int, [_p, _p, _i32, _i64, _p, _i64, _p, _p, _p, _i32, _p, _i32, _i32, _i32, _i32, _p,
                                   _p, _p, _p]),
    "g2_event_pairsum_packed": (C.c_int, [_p, _i64, _p, _i64, _p, _p, _p, _i32, _p, _i32, _i32, _i32, _i32, _p,
                                          _p, _p, _p]),
    "g2_csr_count": (C.c_int, [_p, _p, _p, _i32, _i64, _i32, _i32, _i32, _p, _p, _p]),
    "g2_exclusive_scan_u32": (C.c_int, [_p, _i64, _p, _p, _i64, _p]),
    "g2_csr_scatter": (C.c_int, [_p, _i32, _p, _p, _p, _i32, _i64, _i32, _i32, _i32, _p, _p, _p, _p, _p, _p]),
    "g2_csr_count_blocked": (C.c_int, [_p, _p, _p, _i32, _i64, _i32, _i32, _i32, _p, _p, _p, _p, _p, _p]),
    "g2_csr_stage_blocked": (C.c_int, [_p, _i32, _p, _p, _i32, _i64, _i32, _i32, _i32, _p, _p, _p, _p, _p, _p]),
    "g2_csr_gather_blocked": (C.c_int, [_p, _p, _p, _i32, _i64, _i64, _p, _i32, _p, _p, _p]),
    "g2_csr_stage_frames": (C.c_int, [_p, _i32, _p, _p, _i32, _i64, _i32, _i32, _i64, _i32, _i32, _p, _p, _p, _p,
                                      _p, _p]),
    "g2_add_carry_u32": (C.c_int, [_p, _i64, _p, _p]),
    "g2_events_unpack": (C.c_int, [_p, _i64, _i32, _p, _p, _p]),
    "g2_compress_count": (C.c_int, [_p, _i32, _i32, _i64, _i32, _p, _p, _p, _p, _p, _p]),
    "g2_compress_finish": (C.c_int, [_p, _p, _p, _i32, _i64, _p, _p, _p, _p, _p]),
    "g2_compress_stage": (C.c_int, [_p, _i32, _i32, _i64, _p, _p, _p, _p, _p, _i64, _p, _p]),
    "g2_events_gather_rel": (C.c_int, [_p, _p, _p, _i32, _i64, _i64, _p, _i32, _p, _p, _p, _p, _p]),
    "g2_stream_compress": (C.c_int, [_p, _i32, _i32, _i64, _i64, _i32, _i32, _p, _p, _p, _p, _p, _p, _p]),
    "g2_stream_compact": (C.c_int, [_p, _p, _p, _i32, _i64, _i32, _p, _i64, _p, _p, _p, _p]),
    "g2_denominator": (C.c_int, [_p, _i32, _i64, _p, _p]),
    "g2_finalize": (C.c_int, [_p, _p, _p, _i32, _i64, _p, _p, _p]),
    "g2_normalize_static": (C.c_int, [_p, _p, _p, _i32, _i64, _p, _p, _p]),
}
STATIC_DENOM_MAX = 1 << 19

_lock = threading.Lock()
_lib = None


class G2Error(RuntimeError):
    pass


def load(path=None):
    """Load (once) and return the ctypes library; raise if it is not built."""
    global _lib
    with _lock:
        if _lib is not None and path is None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise ImportError("dynamix_gb300 CUDA library not built (%s); run `python -m dynamix_gb300.build` "
                              "or __graft_entry__.build()" % p)
        lib = C.CDLL(p)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        if path is None:
            _lib = lib
        return lib


def check(status, what):
    if status != G2_OK:
        raise G2Error("%s failed: %s (status %d)" % (what, STATUS.get(status, "unknown"), status))


def jobs_array(jobs):
    """[(packed_ptr, nframes, packed_cols, elem_kind, ones_row), ...] -> ctypes array of Job."""
    if not 1 <= len(jobs) <= MAX_JOBS:
        raise ValueError("between 1 and %d jobs per launch" % MAX_JOBS)
    arr = (Job * len(jobs))()
    for i, (ptr, T, cols, kind, ones) in enumerate(jobs):
        arr[i].packed_dev = ptr
        arr[i].nframes = T
        arr[i].packed_cols = cols
        arr[i].elem_kind = kind
        arr[i].ones_row = int(bool(ones))
    return arr


def device_error_message(code):
    msgs = []
    if code & DEVERR_TIMEOUT:
        msgs.append("a bounded device wait timed out")
    if code & DEVERR_BOUNDS:
        msgs.append("an out-of-range index was skipped")
    if code & DEVERR_RANGE:
        msgs.append("a count does not fit the packing")
    if code & DEVERR_RANGE_CHECK:
        msgs.append("a count may not fit the packing (unchecked)")
    return "; ".join(msgs) or "device error %d" % code
