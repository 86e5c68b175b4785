"""Parity at the full benchmark sizes, through checks whose cost does not grow
with the number of lags: the oracle cannot run these sizes in a test, so every
result is compared exactly (int64) with what plain torch reductions of the same
stack on the device give, and with the independent plain kernel where there is
one.

* dense 514 x 1030 x 10,000 u8, 16 annuli r 20-400 px (the benchmark stack):
  N of every lag against the plain (non-tensor-core) kernel; S of every frame
  and D of every lag against torch; N at sampled lags against torch;
* dense 256 x 256 x 5,000 u16 <= 4095, 12 annuli r 8-128 px: the same;
* CSR / event lists 2162 x 2068 x 20,000 u8, mean 0.005, 32 annuli r 20-1000 px:
  the CSR and event correlators give the same N, S, D; S and D against torch
  sums of the CSR elements; N(0) and N at sampled lags against a torch search
  for each event's partner at t + lag in the sorted event lists;
* frame compression of the benchmark stack: the event lists scattered back
  give the stack (encode -> decode round trip), frames strictly ascending
  within every pixel.

g2 is checked against P N / D in float64 within 1e-12 relative (one rounding
of each of two operations).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

G2_RTOL = 1e-12


def _i32(x):
    """int32 copy of a uint8 / uint16 tensor (uint16 through an int16 view)."""
    import torch
    if x.dtype == torch.uint16:
        return x.view(torch.int16).to(torch.int32) & 0xFFFF
    return x.to(torch.int32)


def _bins(qmask, dev):
    import torch
    return torch.as_tensor(np.ascontiguousarray(qmask).ravel().astype(np.int64), device=dev)


def _dense_sums(f, qt, n_bins, chunk=256):
    """S_b(t) of a (T, npix) stack, int64 (n_bins, T)."""
    import torch
    T = f.shape[0]
    out = torch.zeros((T, n_bins + 1), dtype=torch.int64, device=f.device)
    for t0 in range(0, T, chunk):
        t1 = min(T, t0 + chunk)
        out[t0:t1].index_add_(1, qt, _i32(f[t0:t1]).to(torch.int64))
    return out[:, 1:].T.contiguous()


def _dense_lag(f, qt, n_bins, lag, chunk=512):
    """N_b(lag) = sum_t sum_{p in b} f[t, p] f[t + lag, p], int64 (n_bins,)."""
    import torch
    T, npix = f.shape
    per_px = torch.zeros(npix, dtype=torch.int64, device=f.device)
    for t0 in range(0, T - lag, chunk):
        t1 = min(T - lag, t0 + chunk)
        a = _i32(f[t0:t1])
        b = _i32(f[t0 + lag:t1 + lag])
        per_px += (a * b).sum(0, dtype=torch.int64)
    out = torch.zeros(n_bins + 1, dtype=torch.int64, device=f.device)
    out.index_add_(0, qt, per_px)
    return out[1:]


def _lags_from_sums(S):
    """D_b(lag) = sum_t S_b(t) S_b(t + lag) for every lag, int64 (n_bins, T)."""
    import torch
    T = S.shape[1]
    D = torch.empty_like(S)
    for lag in range(T):
        D[:, lag] = (S[:, :T - lag] * S[:, lag:]).sum(1)
    return D


def _check_g2(c, n_pix):
    N, D, g = c.numerator, c.denominator, c.g2_fp64
    with np.errstate(divide="ignore", invalid="ignore"):
        ref = n_pix[:, None] * N.astype(np.float64) / D.astype(np.float64)
    assert np.array_equal(np.isnan(g), np.isnan(ref))
    ok = ~np.isnan(ref)
    assert np.all(np.abs(g[ok] - ref[ok]) <= G2_RTOL * np.abs(ref[ok]))


def _dense_case(dev, T, shape, rho, mu, seed, dtype, max_count, qmask, lags):
    import torch
    from dynamix_gb300.correlator import MatMulCorrelator
    from dynamix_gb300.speckle import speckle_torch
    n_bins = int(qmask.max())
    frames = speckle_torch(T, shape, rho, mu, seed=seed, dtype=dtype, max_count=max_count, device=dev)
    tc = MatMulCorrelator(shape, T, qmask=qmask, extra_options={"method": "tc"})
    g_tc = tc.correlate(frames)
    pl = MatMulCorrelator(shape, T, qmask=qmask, extra_options={"method": "plain"})
    g_pl = pl.correlate(frames)
    # the two kernels: every lag of every bin
    assert np.array_equal(tc.numerator, pl.numerator)
    assert np.array_equal(tc.denominator, pl.denominator)
    assert np.array_equal(g_tc, g_pl, equal_nan=True)
    # S and D against torch
    f = frames.reshape(T, -1)
    qt = _bins(qmask, dev)
    S = _dense_sums(f, qt, n_bins)
    assert np.array_equal(tc.sums, S.cpu().numpy())
    assert np.array_equal(tc.denominator, _lags_from_sums(S).cpu().numpy())
    # N at sampled lags against torch
    for lag in lags:
        assert np.array_equal(tc.numerator[:, lag], _dense_lag(f, qt, n_bins, lag).cpu().numpy()), lag
    n_pix = np.array([(qmask == b).sum() for b in range(1, n_bins + 1)], dtype=np.float64)
    _check_g2(tc, n_pix)
    assert np.array_equal(g_tc, tc.g2_fp64.astype(np.float32), equal_nan=True)
    del frames, f
    torch.cuda.empty_cache()


def test_dense_514x1030_u8_T10000(built_lib, cuda_device):
    from dynamix_gb300.speckle import annular_qmask
    shape = (514, 1030)
    qm = annular_qmask(shape, 16, 20.0, 400.0, center=(257, 515))
    _dense_case(cuda_device, 10000, shape, 0.99, 0.1, 1, "uint8", None, qm,
                lags=[0, 1, 2, 3, 31, 257, 1000, 4999, 9000, 9999])


def test_dense_256x256_u16_T5000(built_lib, cuda_device):
    from dynamix_gb300.speckle import annular_qmask
    shape = (256, 256)
    qm = annular_qmask(shape, 12, 8.0, 128.0, center=(128, 128))
    _dense_case(cuda_device, 5000, shape, 0.995, 50.0, 3, "uint16", 4095, qm,
                lags=[0, 1, 2, 7, 100, 2500, 4999])


def test_sparse_and_events_2162x2068_T20000(built_lib, cuda_device):
    import torch
    from dynamix_gb300.correlator import EventCorrelator, SparseCorrelator
    from dynamix_gb300.speckle import annular_qmask, speckle_csr_torch
    dev = cuda_device
    T, (H, W) = 20000, (2162, 2068)
    qm = annular_qmask((H, W), 32, 20.0, 1000.0, center=(1081, 1034))
    n_bins = 32
    data, indices, indptr, offsets = speckle_csr_torch(T, (H, W), 0.99, 0.005, seed=4, device=dev)
    offsets = offsets.to(torch.int32)
    n_elem = int(data.numel())
    sc = SparseCorrelator((H, W), T, qmask=qm)
    sc.correlate_device(data, indices, indptr, offsets)
    sc.engine.check_error()
    ev_t, ev_d, ev_o = (x.clone() for x in sc.engine.to_events(data, indices, indptr, offsets, 4, n_elem))
    ec = EventCorrelator((H, W), T, 1, qmask=qm)
    ec.correlate_device(ev_t, ev_d, ev_o)
    ec.engine.check_error()
    # the CSR and the event paths
    assert np.array_equal(sc.numerator, ec.numerator)
    assert np.array_equal(sc.sums, ec.sums)
    assert np.array_equal(sc.denominator, ec.denominator)

    # S from the CSR elements: frame and row of each element from the offsets and row pointers
    qt = _bins(qm, dev)
    per_frame = (offsets[1:].to(torch.int64) - offsets[:-1].to(torch.int64))
    t_of = torch.repeat_interleave(torch.arange(T, device=dev), per_frame)
    ip = indptr.view(T, H + 1).to(torch.int64)
    r_of = torch.repeat_interleave(torch.arange(T * H, device=dev), (ip[:, 1:] - ip[:, :-1]).reshape(-1)) % H
    pix = r_of * W + indices.to(torch.int64)
    del r_of
    b_of = qt[pix]
    v = data.to(torch.int64)
    S = torch.zeros((n_bins + 1) * T, dtype=torch.int64, device=dev)
    S.index_add_(0, b_of * T + t_of, v)
    S = S.view(n_bins + 1, T)[1:]
    assert np.array_equal(sc.sums, S.cpu().numpy())
    assert np.array_equal(sc.denominator, _lags_from_sums(S).cpu().numpy())
    N0 = torch.zeros(n_bins + 1, dtype=torch.int64, device=dev)
    N0.index_add_(0, b_of, v * v)
    assert np.array_equal(sc.numerator[:, 0], N0[1:].cpu().numpy())
    del t_of, pix, b_of, v, data, indices, indptr

    # N at sampled lags: for each event, its partner at t + lag in the same pixel
    n_ev = int(ev_t.numel())
    eo = ev_o.to(torch.int64)
    p_of = torch.repeat_interleave(torch.arange(H * W, device=dev), eo[1:] - eo[:-1])
    t64 = ev_t.to(torch.int64)
    key = p_of * T + t64
    assert bool((key[1:] > key[:-1]).all())             # pixel-major, frames ascending
    eb = qt[p_of]
    ev = ev_d.to(torch.int64)
    del p_of
    for lag in [1, 2, 5, 64, 1000, 12345, 19999]:
        idx = torch.searchsorted(key, key + lag)
        idx.clamp_(max=n_ev - 1)
        hit = (key[idx] == key + lag) & (t64 + lag < T)
        prod = torch.where(hit, ev * ev[idx], torch.zeros_like(ev))
        N = torch.zeros(n_bins + 1, dtype=torch.int64, device=dev)
        N.index_add_(0, eb, prod)
        assert np.array_equal(sc.numerator[:, lag], N[1:].cpu().numpy()), lag
        del idx, hit, prod
    n_pix = np.array([(qm == b).sum() for b in range(1, n_bins + 1)], dtype=np.float64)
    _check_g2(ec, n_pix)
    torch.cuda.empty_cache()


def test_compress_514x1030_u8_T10000_round_trip(built_lib, cuda_device):
    import torch
    from dynamix_gb300.compress import compress_all_stack_device
    from dynamix_gb300.speckle import speckle_torch
    T, shape = 10000, (514, 1030)
    frames = speckle_torch(T, shape, 0.99, 0.1, seed=1, device=cuda_device)
    d, t, off = compress_all_stack_device(frames)
    f = frames.reshape(T, -1)
    npix = f.shape[1]
    counts = (f > 0).sum(0, dtype=torch.int64)
    assert int(off[0]) == 0 and torch.equal(off[1:] - off[:-1], counts)
    p_of = torch.repeat_interleave(torch.arange(npix, device=cuda_device), counts)
    t64 = t.to(torch.int64)
    same = p_of[1:] == p_of[:-1]
    assert bool((t64[1:] > t64[:-1])[same].all())         # frames strictly ascending within a pixel
    back = torch.zeros_like(f)
    back[t64, p_of] = d
    assert torch.equal(back, f)                            # encode -> decode gives the stack
    del frames, f, back
    torch.cuda.empty_cache()
