"""G3 denominator and G4 finalize through the C ABI against numpy."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _corr(S):
    T = S.shape[-1]
    out = np.zeros_like(S)
    for t in range(T):
        out[:, t] = np.einsum("ij,ij->i", S[:, :T - t], S[:, t:])    # int64, wraps mod 2^64 like the kernel
    return out


@pytest.mark.parametrize("T", [1, 7, 1024, 1025, 2500])
def test_denominator_exact(built_lib, cuda_device, T):
    import torch
    from dynamix_gb300 import _lib
    from dynamix_gb300.engine import ptr, stream_handle
    rng = np.random.default_rng(T)
    S = rng.integers(0, 1 << 24, (3, T)).astype(np.int64)
    S[1, ::3] = 0
    if T > 5:
        S[2, 5] = (1 << 40) + 12345                                   # a value above 2^32: the wide path
    lib = _lib.load()
    s = torch.from_numpy(S).to(cuda_device)
    d = torch.zeros_like(s)
    _lib.check(lib.g2_denominator(ptr(s), 3, T, ptr(d), stream_handle(cuda_device)), "g2_denominator")
    got = d.cpu().numpy()
    with np.errstate(over="ignore"):
        ref = _corr(S)
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("vmax", [200, 3000, 65535, 70000])
def test_denominator_value_ranges(built_lib, cuda_device, vmax):
    # 32-bit runs of a whole window (200), of a few hundred frames (3000), of
    # one frame (65535), and the 64-bit path (70000)
    import torch
    from dynamix_gb300 import _lib
    from dynamix_gb300.engine import ptr, stream_handle
    T = 3000
    rng = np.random.default_rng(vmax)
    S = rng.integers(0, vmax + 1, (4, T)).astype(np.int64)
    S[:, rng.integers(0, T, 4)] = vmax                               # the maximum occurs
    S[3, :1500] = 0                                                  # dark frames in one row
    lib = _lib.load()
    s = torch.from_numpy(S).to(cuda_device)
    d = torch.zeros_like(s)
    _lib.check(lib.g2_denominator(ptr(s), 4, T, ptr(d), stream_handle(cuda_device)), "g2_denominator")
    assert np.array_equal(d.cpu().numpy(), _corr(S))
