"""Continuous-batching correlation service (cellspe_service_*).

Jobs of uneven shape are submitted together; the service admits them by
device footprint and runs them concurrently.  Each result must be identical
to the same job run alone through cellspe_fx_correlate.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _jobs():
    import synth

    rng = np.random.default_rng(5)
    shapes = [(4, 512, 32), (8, 1024, 16), (24, 2048, 8), (6, 8192, 8), (16, 2048, 24), (4, 32768, 8),
              (12, 1024, 40), (24, 512, 64)]
    jobs = []
    for n, (S, N, K) in enumerate(shapes):
        rho = float(rng.uniform(0.01, 0.2))
        raw = synth.stations_offset_binary(S, N * K, rho=rho, seed=100 + n)
        mode = n % 2   # alternate FP32 and tensor-core jobs
        jobs.append((S, N, K, mode, raw))
    return jobs


@pytest.mark.parametrize("priority_samples", [0, -1, 1 << 17], ids=["default", "one-priority", "split"])
def test_service_mix_equals_solo(cg, priority_samples):
    """Identical results whichever stream priority a job runs at (default: all
    these jobs are small; split: one on the high-priority stream, the rest not;
    one-priority: no high-priority stream)."""
    jobs = _jobs()
    solo = []
    for S, N, K, mode, raw in jobs:
        vis = np.zeros((N // 2, S * (S + 1) // 2), np.complex64)
        cg.fx_correlate(cg.fx_params(S, N, K, raw.shape[1], x_mode=mode), raw, vis)
        solo.append(vis)
    svc = cg.Service(max_streams=4, priority_samples=priority_samples)
    try:
        outs, ids = [], []
        for S, N, K, mode, raw in jobs:
            vis = np.full((N // 2, S * (S + 1) // 2), np.nan, np.complex64)
            outs.append(vis)
            ids.append(svc.submit(cg.fx_params(S, N, K, raw.shape[1], x_mode=mode), raw, vis))
        lat = [svc.wait(i) for i in ids]
        st = svc.stats()
    finally:
        svc.close()
    for a, b in zip(outs, solo):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert st["completed"] == len(jobs) and st["failed"] == 0
    assert 0 < st["p50_ms"] <= st["p99_ms"] and all(x > 0 for x in lat)


def test_service_large_jobs_one_at_a_time(cg):
    """Jobs of at least large_samples samples never overlap each other; smaller
    jobs are admitted past a large job that waits.  Results are unchanged."""
    jobs = _jobs()
    solo = []
    for S, N, K, mode, raw in jobs:
        vis = np.zeros((N // 2, S * (S + 1) // 2), np.complex64)
        cg.fx_correlate(cg.fx_params(S, N, K, raw.shape[1], x_mode=mode), raw, vis)
        solo.append(vis)
    for large, max_run in ((1, 1), (1 << 19, None)):
        svc = cg.Service(max_streams=4, large_samples=large)
        try:
            outs, ids = [], []
            for S, N, K, mode, raw in jobs:
                vis = np.full((N // 2, S * (S + 1) // 2), np.nan, np.complex64)
                outs.append(vis)
                ids.append(svc.submit(cg.fx_params(S, N, K, raw.shape[1], x_mode=mode), raw, vis))
            for i in ids:
                svc.wait(i)
            st = svc.stats()
        finally:
            svc.close()
        for a, b in zip(outs, solo):
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
        assert st["completed"] == len(jobs) and st["failed"] == 0
        if max_run is not None:
            assert st["max_running"] == max_run


def test_service_admission_by_footprint(cg):
    import synth

    S, N, K = 8, 2048, 16
    raw = synth.stations_offset_binary(S, N * K, rho=0.1, seed=3)
    p = cg.fx_params(S, N, K, raw.shape[1])
    need = cg.lib().cellspe_fx_workspace_bytes(ctypes_byref(p))
    # budget for one job at a time: jobs still all complete, one after another
    svc = cg.Service(hbm_budget_bytes=int(need * 1.5), max_streams=4)
    try:
        outs = [np.zeros((N // 2, S * (S + 1) // 2), np.complex64) for _ in range(4)]
        ids = [svc.submit(cg.fx_params(S, N, K, raw.shape[1]), raw, o) for o in outs]
        for i in ids:
            svc.wait(i)
        st = svc.stats()
        assert st["completed"] == 4 and st["max_running"] == 1
        big = cg.fx_params(S, N, 4 * K, raw.shape[1] * 4)
        with pytest.raises(cg.CellspeError) as e:
            svc.submit(big, np.zeros((S, raw.shape[1] * 4), np.uint8), np.zeros((N // 2, 36), np.complex64))
        assert e.value.code == cg.ERR_NOMEM
    finally:
        svc.close()
    assert all(np.array_equal(outs[0], o) for o in outs[1:])


def ctypes_byref(x):
    import ctypes

    return ctypes.byref(x)


def test_service_failed_job_reports_worker_error(cg):
    """A job that the worker rejects (here N = 3000, not a power of two) fails
    alone: wait() raises with the worker's message, the next job still runs."""
    import synth

    S, N, K = 4, 2048, 8
    raw = synth.stations_offset_binary(S, N * K, rho=0.1, seed=8)
    svc = cg.Service()
    try:
        bad = svc.submit(cg.fx_params(S, 3000, 4, raw.shape[1]), raw, np.zeros((1500, 10), np.complex64))
        out = np.zeros((N // 2, S * (S + 1) // 2), np.complex64)
        good = svc.submit(cg.fx_params(S, N, K, raw.shape[1]), raw, out)
        with pytest.raises(cg.CellspeError) as e:
            svc.wait(bad)
        assert e.value.code == cg.ERR_ARG and "power of two" in str(e.value)
        svc.wait(good)
        st = svc.stats()
    finally:
        svc.close()
    ref = np.zeros_like(out)
    cg.fx_correlate(cg.fx_params(S, N, K, raw.shape[1]), raw, ref)
    assert np.array_equal(out, ref) and st["failed"] == 1 and st["completed"] == 1


@pytest.mark.parametrize("N,K", [(2048, 64), (1024, 32), (8192, 8)])
def test_service_batches_small_jobs_bit_identical(cg, N, K):
    """batch_inputs > 0: queued small device-buffer jobs of one shape run as one
    stacked job (one F-stage and one X-stage launch) and each job's triangle is
    gathered into its own buffer, channel- or baseline-major.  One worker and a
    large job submitted first let the small ones queue up; every small job's
    visibilities must equal its solo run bit for bit, and the service must have
    formed at least one batch."""
    import torch

    import synth

    sizes = [4, 8, 2, 16, 5, 12, 3, 8, 7]
    small = []
    for n, S in enumerate(sizes):
        raw = synth.device_stations(S, N * K, 0.1, seed=300 + n)
        order = cg.VIS_BASELINE_MAJOR if n % 3 == 2 else cg.VIS_CHANNEL_MAJOR
        small.append((S, raw, order))
    big_raw = synth.device_stations(200, 2048 * 1024, 0.02, seed=299)
    solo = []
    for S, raw, order in small:
        C, P = N // 2, S * (S + 1) // 2
        v = torch.empty((P, C) if order == cg.VIS_BASELINE_MAJOR else (C, P), dtype=torch.complex64, device="cuda")
        cg.fx_correlate(cg.fx_params(S, N, K, raw.shape[1], x_mode=cg.X_TC_FP16, vis_order=order), raw, v)
        solo.append(v)
    torch.cuda.synchronize()
    svc = cg.Service(max_streams=1, batch_inputs=64)
    try:
        big = torch.empty((1024, 200 * 201 // 2), dtype=torch.complex64, device="cuda")
        ids = [svc.submit(cg.fx_params(200, 2048, 1024, big_raw.shape[1], x_mode=cg.X_TC_FP16), big_raw, big)]
        outs = []
        for S, raw, order in small:
            v = torch.full_like(solo[len(outs)], float("nan"))
            outs.append(v)
            ids.append(svc.submit(cg.fx_params(S, N, K, raw.shape[1], x_mode=cg.X_TC_FP16, vis_order=order), raw, v))
        for i in ids:
            svc.wait(i)
        st = svc.stats()
    finally:
        svc.close()
    torch.cuda.synchronize()
    for a, b in zip(outs, solo):
        assert torch.equal(a.view(torch.float32), b.view(torch.float32))
    assert st["failed"] == 0 and st["completed"] == len(ids)
    assert st["batched_jobs"] >= 2 and st["batched_launches"] >= 1


def test_service_concurrent_small_and_large_x_tiles(cg):
    """Two workers launch the tensor-core X stage with its single-tile form
    (S <= 128, smaller shared memory) and its tiled form (S > 128) at the same
    time: the kernel's shared-memory limit is only ever raised, so neither
    launch can find it lowered by the other (which failed with 'too many
    resources requested for launch' before)."""
    import torch

    import synth

    N, K = 512, 64
    raws = {S: synth.device_stations(S, N * K, 0.05, seed=S) for S in (24, 200)}
    svc = cg.Service(max_streams=2, batch_inputs=-1)
    try:
        ids, outs = [], []
        for n in range(24):
            S = 24 if n % 2 else 200
            v = torch.empty((N // 2, S * (S + 1) // 2), dtype=torch.complex64, device="cuda")
            outs.append(v)
            ids.append(svc.submit(cg.fx_params(S, N, K, raws[S].shape[1], x_mode=cg.X_TC_FP16), raws[S], v))
        for i in ids:
            svc.wait(i)
        st = svc.stats()
    finally:
        svc.close()
    assert st["failed"] == 0 and st["completed"] == 24
    for a, b in zip(outs[2:], outs):
        assert torch.equal(a, b)
