"""The g2 service on the GPU: every job of a mix equals the oracle and equals
the same job run alone (exact integers, so bit for bit)."""
import numpy as np
import pytest

from oracle import g2_oracle as o

pytestmark = pytest.mark.gpu


def _mix():
    from dynamix_gb300.speckle import annular_qmask, speckle_numpy
    jobs = []
    spec = [  # T, shape, rho, mu, dtype, n_bins, seed
        (300, (24, 40), 0.98, 0.5, np.uint8, 5, 1),
        (129, (33, 17), 0.95, 3.0, np.uint8, 3, 2),      # counts above 16: fp16 operands
        (520, (20, 20), 0.99, 0.2, np.uint8, 4, 3),
        (200, (16, 30), 0.99, 40.0, np.uint16, 2, 4),
        (64, (40, 40), 0.9, 1.0, np.uint8, 6, 5),
    ]
    for T, shape, rho, mu, dt, nb, seed in spec:
        fr = speckle_numpy(T, shape, rho, mu, seed=seed, dtype=dt)
        qm = annular_qmask(shape, nb, 0.0, min(shape) / 2.0)
        jobs.append((fr, qm))
    return jobs


def _check(req, fr, qm):
    ref = o.g2_exact(fr, qm)
    assert np.array_equal(req.numerator, ref["numerator"])
    assert np.array_equal(req.sums, ref["sums"])
    assert np.array_equal(req.denominator, ref["denominator"])
    assert np.array_equal(req.g2, ref["g2"].astype(np.float32), equal_nan=True)


def test_mix_matches_oracle_and_alone(built_lib, cuda_device):
    import torch
    from dynamix_gb300.serving import G2Server
    jobs = _mix()
    # tiny slices: every job spans several grouped launches shared with the others
    srv = G2Server(hbm_budget=2e9, slice_ops=2e8)
    reqs = []
    for i, (fr, qm) in enumerate(jobs):
        if i % 3 == 0:
            inp = torch.from_numpy(fr).pin_memory()         # pinned host: asynchronous copy
        elif i % 3 == 1:
            inp = torch.from_numpy(fr).cuda()               # device-resident, used in place
        else:
            inp = fr                                         # numpy
        reqs.append(srv.submit(inp, qm))
    srv.run_until_idle()
    assert srv.stats["launches"] >= 3          # jobs span several grouped launches
    assert srv.stats["max_active"] >= 2
    for r, (fr, qm) in zip(reqs, jobs):
        r.wait()
        _check(r, fr, qm)
    # each job alone on a fresh server gives the same arrays
    for r, (fr, qm) in zip(reqs, jobs):
        solo = G2Server(hbm_budget=2e9, arena_elems=1 << 20)
        q = solo.submit(fr, qm)
        solo.run_until_idle()
        q.wait()
        for k in ("g2", "numerator", "sums", "denominator"):
            assert np.array_equal(getattr(q, k), getattr(r, k), equal_nan=True), k


@pytest.mark.parametrize("policy", ["fifo", "srpt"])
def test_mix_each_policy(built_lib, cuda_device, policy):
    """Oldest-first and shortest-first slices give the same exact results."""
    from dynamix_gb300.serving import G2Server
    jobs = _mix()
    srv = G2Server(hbm_budget=2e9, slice_ops=2e8, policy=policy)
    reqs = [srv.submit(fr, qm) for fr, qm in jobs]
    srv.run_until_idle()
    assert srv.stats[policy + "_launches"] == srv.stats["launches"] >= 3
    for r, (fr, qm) in zip(reqs, jobs):
        r.wait()
        _check(r, fr, qm)


def test_background_thread_and_budget(built_lib, cuda_device):
    from dynamix_gb300.serving import G2Server
    jobs = _mix()[:3]
    need = max(fr.nbytes * 3 for fr, _ in jobs)
    srv = G2Server(hbm_budget=need, slice_ops=1e9)     # room for about one job at a time
    srv.start()
    try:
        reqs = [srv.submit(fr, qm) for fr, qm in jobs]
        for r, (fr, qm) in zip(reqs, jobs):
            r.wait(timeout=120)
            _check(r, fr, qm)
            assert r.latency is not None and r.latency > 0
    finally:
        srv.stop()
    assert srv.used == 0 and srv.arena.used == 0


def test_errors_do_not_stop_the_server(built_lib, cuda_device):
    from dynamix_gb300.serving import G2Server
    fr, qm = _mix()[0]
    srv = G2Server(hbm_budget=1e6)
    big = srv.submit(np.zeros((2000, 64, 64), np.uint8), None)        # larger than the budget
    bad = srv.submit(np.zeros((10, 4), np.uint8), None)              # not a stack
    neg = srv.submit(-np.ones((5, 4, 4), np.int16), None)           # 16-bit but negative counts
    ok = srv.submit(fr[:50], qm)
    srv.run_until_idle()
    with pytest.raises(MemoryError):
        big.wait()
    with pytest.raises(ValueError):
        bad.wait()
    with pytest.raises(ValueError):
        neg.wait()
    ok.wait()
    _check(ok, fr[:50], qm)


def test_staging_arena_limits(built_lib, cuda_device):
    """Pinned host frames go through the staging arena: a job larger than the
    whole arena gets a buffer of its own, jobs that do not fit beside each
    other wait for space; the results stay exact and the arena drains."""
    import torch
    from dynamix_gb300.serving import G2Server
    jobs = _mix()
    sizes = [fr.nbytes for fr, _ in jobs]
    srv = G2Server(hbm_budget=2e9, slice_ops=2e8, staging_bytes=max(sizes) * 1.5)
    reqs = [srv.submit(torch.from_numpy(fr).pin_memory(), qm) for fr, qm in jobs]
    big = np.concatenate([jobs[0][0]] * 2)                     # twice the first job's frames
    reqs.append(srv.submit(torch.from_numpy(big).pin_memory(), jobs[0][1]))
    srv.run_until_idle()
    for r, (fr, qm) in zip(reqs, jobs + [(big, jobs[0][1])]):
        r.wait()
        _check(r, fr, qm)
    assert srv.staging_arena.used == 0 and srv.arena.used == 0 and srv.used == 0
