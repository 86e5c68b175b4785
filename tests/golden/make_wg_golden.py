"""Generate golden vectors by running the reference's own dense and CSR
OpenCL kernels on the CPU.

``densecorrelator.cl`` (``correlator_multiQ_dense``, ``compute_sums_dense``,
``correlate_1D``) and ``correlator.cl`` (``compute_sums``,
``correlator_oneQ_Nt``) use work-group barriers and local memory; they are
compiled as C with ``oracle/opencl_wg_shim.h`` by
``oracle/build_oracle.py`` (``build_ref_wg``) and launched by
``oracle/ref_wg_driver.c`` over the NDRanges, with the compile options and
arguments of ``DenseCorrelator.correlate`` (``dense.py:170-272``) and
``SparseCorrelator.correlate`` (``intensity.py:59-129``).

Besides the reference's own float32 g2, each fixture pins the integer
numerator: the dense kernel is run a second time with a normalisation of
ones (its output is then float(N), exact below 2^24), the CSR kernel with
frame sums of ones (its output is then N / (T - tau), from which N is
recovered exactly below 2^23).  The cases respect the kernels' own limits:
W <= 1024 and counts <= 127 for the dense kernel (it reads signed ``char``),
rows of at most 64 elements for the CSR kernel (one 64-wide work-group per
row) and products below 256 (it multiplies in the data type).  Run where the
dynamix sources are available::

    python tests/golden/make_wg_golden.py
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.abspath(os.path.join(HERE, "..", "..")))

from dynamix_gb300.speckle import annular_qmask, speckle_numpy  # noqa: E402
from oracle import build_oracle  # noqa: E402
from oracle import g2_oracle as o  # noqa: E402

DENSE_CASES = [
    # name, T, shape, rho, mu, n_bins, seed
    ("refcl_dense_u8", 120, (20, 48), 0.97, 1.5, 4, 21),
    ("refcl_dense_wide", 80, (6, 300), 0.95, 3.0, 3, 22),
]
CSR_CASES = [
    # name, T, shape, rho, mu, seed
    ("refcl_csr_u8", 64, (24, 40), 0.97, 0.4, 23),
    ("refcl_csr_dense_rows", 48, (10, 64), 0.9, 1.0, 24),
]


def nextpow2(n):
    return 1 << int(np.ceil(np.log2(n)))


def p(a):
    return ctypes.c_void_p(a.ctypes.data)


def run_dense(name, T, shape, rho, mu, nb, seed):
    H, W = shape
    frames = speckle_numpy(T, shape, rho, mu, seed=seed)
    assert frames.max() <= 127 and W <= 1024
    qmask = annular_qmask(shape, nb, 0.0, max(shape) / 2.0, center=(H / 2.0, W / 2.0)).astype(np.int32)
    n_bins = int(qmask.max())
    wg0 = min(1024, nextpow2(W))
    lib = build_oracle.load_ref_wg("dense", {
        "IMAGE_WIDTH": W, "NUM_BINS": n_bins, "DTYPE": "unsigned char", "DTYPE_SUMS": "unsigned int",
        "N_FRAMES": T, "USE_SHARED": 0, "SUM_WG_SIZE": wg0})
    fr = np.ascontiguousarray(frames)
    qm = np.ascontiguousarray(qmask)
    sums = np.zeros((n_bins, T), np.uint32)
    assert lib.g2w_dense_sums(p(fr), p(qm), p(sums), H, T) == 0
    corr1d = np.zeros((n_bins, T), np.float32)
    assert lib.g2w_dense_corr1d(p(sums), p(corr1d), T, n_bins) == 0
    # _normalize_sums (dense.py:204-211): divide by the bins' scale factors
    # (their pixel counts by default, common.py:56-72)
    npix = np.bincount(qm.ravel(), minlength=n_bins + 1)[1:].astype(np.float32)
    sums_f = corr1d.copy()
    for i in range(n_bins):
        sums_f[i] /= np.array([npix[i]], dtype=np.float32)[0]
    out = np.zeros((n_bins, T), np.float32)
    frames_c = fr.view(np.int8)
    assert lib.g2w_dense_numerator(p(frames_c), p(qm), p(sums_f), p(out), H, T, wg0) == 0
    ones = np.ones((n_bins, T), np.float32)
    numer_f = np.zeros((n_bins, T), np.float32)
    assert lib.g2w_dense_numerator(p(frames_c), p(qm), p(ones), p(numer_f), H, T, wg0) == 0
    exact = o.g2_exact(frames, qmask)
    assert exact["numerator"].max() < 2 ** 24
    np.savez_compressed(os.path.join(HERE, name + ".npz"), frames=frames, qmask=qmask, sums=sums, corr1d=corr1d,
                        g2=out, numer_f=numer_f)
    print(name, frames.shape, "N exact:", np.array_equal(numer_f.astype(np.int64), exact["numerator"]),
          "S exact:", np.array_equal(sums.astype(np.int64), exact["sums"]))


def run_csr(name, T, shape, rho, mu, seed):
    H, W = shape
    frames = speckle_numpy(T, shape, rho, mu, seed=seed)
    frames = np.minimum(frames, 15).astype(np.uint8)           # products < 256 (uchar arithmetic)
    data, indices, indptr, offsets = o.frames_to_csr(frames)
    data = np.ascontiguousarray(data.astype(np.uint8))
    indices = np.ascontiguousarray(indices.astype(np.int32))
    indptr = np.ascontiguousarray(indptr.astype(np.int32))
    offsets = np.ascontiguousarray(offsets.astype(np.int32))
    assert np.diff(indptr.reshape(T, H + 1), axis=1).max() <= 64
    lib = build_oracle.load_ref_wg("csr", {"IMAGE_WIDTH": W, "DTYPE": "unsigned char", "IDX_DTYPE": "int",
                                           "SUM_WG_SIZE": 1024})
    sums = np.zeros(T, np.float32)
    assert lib.g2w_csr_sums(p(data), p(offsets), p(sums), T) == 0
    # intensity.py:110: d_sums *= 1 / sqrt(prod(shape)) (float32 array op)
    scaled = (sums * np.float32(1.0 / np.sqrt(H * W))).astype(np.float32)
    norm_mask = np.ones(H * W, np.float32)
    g2 = np.zeros(T, np.float32)
    assert lib.g2w_csr_correlate(p(data), p(indices), p(indptr), p(offsets), p(norm_mask), p(scaled), p(g2), H,
                                 T) == 0
    ones = np.ones(T, np.float32)
    n_over = np.zeros(T, np.float32)
    assert lib.g2w_csr_correlate(p(data), p(indices), p(indptr), p(offsets), p(norm_mask), p(ones), p(n_over), H,
                                 T) == 0
    n_rec = np.rint(n_over.astype(np.float64) * (T - np.arange(T))).astype(np.int64)
    exact = o.g2_exact(frames, None)
    assert exact["numerator"].max() < 2 ** 23
    np.savez_compressed(os.path.join(HERE, name + ".npz"), frames=frames, data=data, indices=indices, indptr=indptr,
                        offsets=offsets, sums=sums, g2=g2, numer=n_rec)
    print(name, frames.shape, "N exact:", np.array_equal(n_rec, exact["numerator"][0]),
          "S exact:", np.array_equal(sums.astype(np.int64), exact["sums"][0]))


def main(root=None):
    if root:
        os.environ["DYNAMIX_REFERENCE_ROOT"] = root
    if build_oracle.build_ref_wg("dense", {"IMAGE_WIDTH": 8, "NUM_BINS": 1, "DTYPE": "unsigned char",
                                           "DTYPE_SUMS": "unsigned int", "N_FRAMES": 2, "USE_SHARED": 0,
                                           "SUM_WG_SIZE": 8}) is None:
        raise SystemExit("the reference sources are not available")
    for case in DENSE_CASES:
        run_dense(*case)
    for case in CSR_CASES:
        run_csr(*case)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else None)
