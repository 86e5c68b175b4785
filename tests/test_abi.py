"""The C-ABI library loads without a GPU and exports every declared symbol."""
import ctypes
import os
import re

import numpy as np

from conftest import ROOT


def header_functions():
    src = open(os.path.join(ROOT, "include", "dynamix_g2.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\*?\s*(g2_[a-z0-9_]+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = header_functions()
    for n in ("g2_pack_frames", "g2_gram_tc", "g2_plain_direct", "g2_denominator", "g2_finalize"):
        assert n in names


def test_library_exports_every_declared_symbol(built_lib):
    lib = ctypes.CDLL(built_lib._name)
    missing = [n for n in header_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_every_declared_symbol(built_lib):
    from dynamix_gb300 import _lib
    assert sorted(_lib.SIGNATURES) == header_functions()


def test_host_utilities_without_gpu(built_lib):
    assert built_lib.g2_abi_version() == 1
    assert built_lib.g2_status_string(0) == b"ok"
    assert built_lib.g2_status_string(1) == b"invalid argument"


def test_argument_errors_are_caught_on_host(built_lib):
    # null pointers / bad sizes are rejected before any CUDA call
    assert built_lib.g2_denominator(None, 1, 10, None, None) == 1
    assert built_lib.g2_finalize(None, None, None, 1, 10, None, None, None) == 1
    assert built_lib.g2_gram_tc(None, 0, None, 0, None, 0, None, 0, None, 0, None) == 1
    assert built_lib.g2_pack_frames(None, 1, 1, 1, None, None, None, None, None, None, 1, 0, None, 128, None, 1,
                                    None, 0, None, None) == 1
    assert built_lib.g2_normalize_static(None, None, None, 1, 10, None, None, None) == 1
    assert built_lib.g2_compress_count(None, 1, 10, 16, -1, None, None, None, None, None, None) == 1
    assert built_lib.g2_compress_count(1, 3, 10, 16, -1, 1, None, None, 1, None, None) == 1   # bad kind
    assert built_lib.g2_compress_count(1, 1, 10, 16, 5, 1, None, None, 1, None, None) == 1    # threshold, no outputs
    assert built_lib.g2_compress_stage(None, 1, 10, 16, None, None, None, None, None, 0, None, None) == 1
    assert built_lib.g2_events_gather_rel(1, 1, 1, 10, 16, 0, 1, 1, 1, 1, 1, 1, None) == 1  # both output forms
    assert built_lib.g2_stream_compress(1, 1, 1, 0, 16, 0, -1, None, None, 1, 1, 1, 1, None) == 1  # max_nnz 0
    assert built_lib.g2_stream_compact(None, None, None, 1, 16, 4, None, 0, None, None, None, None) == 1


def test_item_layout_matches_c_struct():
    from dynamix_gb300 import _lib
    assert _lib.ITEM_DTYPE.itemsize == 48
    assert ctypes.sizeof(_lib.Job) == 32
    assert list(_lib.ITEM_DTYPE.names) == ["job", "i0", "j0", "a_k0", "b_k0", "k_len", "shift", "nframes",
                                           "out_off", "s_off"]
    assert np.dtype(_lib.ITEM_DTYPE).fields["out_off"][1] == 32
