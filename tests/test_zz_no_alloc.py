"""g2_normalize_static: the normalisation step for callers that cannot allocate.

Some hosts give this library no room to allocate device memory (every byte is
already reserved, e.g. for the frame buffers of a detector acquisition loop),
or cannot afford cudaFree's wait for the whole device.  For them
g2_normalize_static computes g2 = scale * N / D from N and the bin sums S with
the denominator D held in the library's own fixed device array instead of a
caller buffer.  Called through the C ABI, it must give exactly what the
two-step path (g2_denominator into a caller buffer, then g2_finalize) gives,
on two calls in a row with different inputs (the shared array keeps the
previous call's contents), and reject sizes above its fixed maximum.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _inputs(torch, dev, n_rows, T, seed):
    g = torch.Generator(device="cpu")
    g.manual_seed(seed)
    S = torch.randint(0, 5000, (n_rows, T), generator=g, dtype=torch.int64)
    S[0, : T // 3] = 0                                   # a dark stretch: some D values are small
    N = torch.randint(0, 10 ** 9, (n_rows, T), generator=g, dtype=torch.int64)
    N[-1] = 0                                            # a dark bin: 0/0 -> NaN
    S[-1] = 0
    scale = torch.rand(n_rows, generator=g, dtype=torch.float64) * 1000 + 1
    return S.to(dev), N.to(dev), scale.to(dev)


def test_normalize_static_matches_two_step(built_lib, cuda_device):
    import torch
    lib = built_lib
    dev = cuda_device
    stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    from dynamix_gb300 import _lib
    # the last case fills the array exactly (8 x 65536 = G2_STATIC_DENOM_MAX elements): its last element and
    # the boundary of the size check are exercised
    cases = [(16, 3000, 1), (5, 777, 2), (8, _lib.STATIC_DENOM_MAX // 8, 3)]
    for call, (n_rows, T, seed) in enumerate(cases):
        S, N, scale = _inputs(torch, dev, n_rows, T, seed)
        # existing entry points, caller-owned denominator
        D = torch.empty((n_rows, T), dtype=torch.int64, device=dev)
        ref32 = torch.empty((n_rows, T), dtype=torch.float32, device=dev)
        ref64 = torch.empty((n_rows, T), dtype=torch.float64, device=dev)
        assert lib.g2_denominator(_ptr(S), n_rows, T, _ptr(D), stream) == 0
        assert lib.g2_finalize(_ptr(N), _ptr(D), _ptr(scale), n_rows, T, _ptr(ref32), _ptr(ref64), stream) == 0
        # the entry point that allocates nothing
        out32 = torch.full((n_rows, T), -1.0, dtype=torch.float32, device=dev)
        out64 = torch.full((n_rows, T), -1.0, dtype=torch.float64, device=dev)
        assert lib.g2_normalize_static(_ptr(N), _ptr(S), _ptr(scale), n_rows, T, _ptr(out32), _ptr(out64),
                                       stream) == 0
        torch.cuda.synchronize(dev)
        a32, b32 = ref32.cpu().numpy(), out32.cpu().numpy()
        a64, b64 = ref64.cpu().numpy(), out64.cpu().numpy()
        # identical arithmetic: the tests' g2 tolerance (1e-12 relative) is met with equality
        assert np.array_equal(a32, b32, equal_nan=True), call
        assert np.array_equal(a64, b64, equal_nan=True), call
        assert np.isnan(b64[-1]).all()
        ok = np.isfinite(a64)
        assert np.all(np.abs(a64[ok] - b64[ok]) <= 1e-12 * np.abs(a64[ok]))


def test_normalize_static_rejects_oversize(built_lib, cuda_device):
    import torch
    from dynamix_gb300 import _lib
    lib = built_lib
    dev = cuda_device
    n_rows, T = 8, _lib.STATIC_DENOM_MAX // 8 + 1
    S = torch.zeros((n_rows, T), dtype=torch.int64, device=dev)
    N = torch.zeros_like(S)
    scale = torch.ones(n_rows, dtype=torch.float64, device=dev)
    out = torch.empty((n_rows, T), dtype=torch.float32, device=dev)
    stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    assert lib.g2_normalize_static(_ptr(N), _ptr(S), _ptr(scale), n_rows, T, _ptr(out), None, stream) == 4
    assert lib.g2_status_string(4) == b"size exceeds a kernel limit"
