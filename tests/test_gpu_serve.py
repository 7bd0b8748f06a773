"""The continuous-batching serve loop (ufoir_serve_*), through the C ABI.

Each job runs the kernels of the plain per-job call, so its result must be
the same, bit for bit, whether it runs alone or in a mix with other jobs in
flight. Failure handling is exercised on the host: invalid parameters, a job
larger than the budget, cancellation, a wait that times out, and injected
allocation failures; none of these faults the GPU.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _jobs(ufoir, oracle):
    rng = np.random.default_rng(7)
    specs = [(ufoir.METHOD_SIRT, 48, 40, dict(num_iterations=4, relaxation_factor=0.25)),
             (ufoir.METHOD_SART, 33, 30, dict(num_iterations=2, relaxation_factor=0.3)),
             (ufoir.METHOD_ASDPOCS, 40, 36, dict(asdpocs=dict(num_iterations=2, norm_mode=ufoir.NORM_COMPAT,
                                                                df_minimizer=dict(num_iterations=2)))),
             (ufoir.METHOD_SIRT, 96, 120, dict(num_iterations=3)),
             (ufoir.METHOD_SART, 64, 45, dict(num_iterations=1)),
             (ufoir.METHOD_SIRT, 20, 18, dict(num_iterations=6, relaxation_factor=0.5)),
             (ufoir.METHOD_ASDPOCS, 24, 20, dict(asdpocs=dict(num_iterations=3, norm_mode=ufoir.NORM_FP64,
                                                                df_minimizer=dict(num_iterations=1))))]
    jobs = []
    for method, n, na, kw in specs:
        step = float(np.float32(np.pi / na))
        vol = rng.random((n, n), dtype=np.float32)
        sino = oracle.forward(oracle.projector(n, na, np.float32(step)), vol)
        jobs.append((ufoir.job_desc(method, n, na, step, **dict(kw)), sino, kw))
    return jobs


def _solo(ufoir, ctx, desc, sino, kw):
    p = ufoir.ParallelProjector(ctx, step=desc.step, axis_position=desc.axis_position, is_forward=0)
    if desc.method == ufoir.METHOD_SIRT:
        out = ufoir.sirt(p, sino, **kw)
    elif desc.method == ufoir.METHOD_SART:
        out = ufoir.sart(p, sino, **kw)
    else:
        out = ufoir.asdpocs(p, sino, **kw["asdpocs"])
    p.close()
    return out


@pytest.mark.parametrize("policy", ["continuous", "continuous_unbatched", "one_at_a_time", "sjf_one_at_a_time"])
def test_results_in_the_mix_equal_results_alone(ufoir_lib, gpu_ctx, oracle, policy):
    ufoir = ufoir_lib
    jobs = _jobs(ufoir, oracle)
    pol = {"continuous": ufoir.SERVE_CONTINUOUS, "continuous_unbatched": ufoir.SERVE_CONTINUOUS,
           "one_at_a_time": ufoir.SERVE_ONE_AT_A_TIME, "sjf_one_at_a_time": ufoir.SERVE_SJF_ONE_AT_A_TIME}[policy]
    with ufoir.Server(gpu_ctx, policy=pol, max_active_jobs=8, batch_sirt=policy == "continuous") as srv:
        handles = [srv.submit(d, s) for d, s, _ in jobs]
        for jid, _ in handles:
            assert srv.wait(jid, 120000) == ufoir.OK
            assert srv.poll(jid) == ufoir.JOB_DONE
        st = srv.stats()
    assert st["completed"] == len(jobs) and st["failed"] == 0
    assert st["p99_latency_ms"] >= st["p50_latency_ms"] > 0
    if policy == "continuous":
        assert st["peak_active_jobs"] >= 2
        assert st["batched_iterations"] > 0       # the SIRT jobs advanced in the mixed batch
    elif policy == "continuous_unbatched":
        assert st["peak_active_jobs"] >= 2 and st["batched_iterations"] == 0
    else:
        assert st["peak_active_jobs"] == 1 and st["batched_iterations"] == 0
    for (d, s, kw), (_, out) in zip(jobs, handles):
        alone = _solo(ufoir, gpu_ctx, d, s, kw)
        assert np.array_equal(out, alone), (d.method, d.n_dets, float(np.abs(out - alone).max()))


def test_served_sirt_matches_oracle(ufoir_lib, gpu_ctx, oracle):
    n, na = 40, 30
    step = np.float32(np.pi / na)
    rng = np.random.default_rng(3)
    sino = oracle.forward(oracle.projector(n, na, step), rng.random((n, n), dtype=np.float32))
    with ufoir_lib.Server(gpu_ctx) as srv:
        jid, out = srv.submit(ufoir_lib.job_desc(ufoir_lib.METHOD_SIRT, n, na, float(step), num_iterations=5), sino)
        assert srv.wait(jid, 60000) == ufoir_lib.OK
    want = oracle.sirt(oracle.projector(n, na, step), sino, 5, 0.25)
    assert np.array_equal(out, want)


def test_budget_admission_and_rejection(ufoir_lib, gpu_ctx, oracle):
    ufoir = ufoir_lib
    jobs = _jobs(ufoir, oracle)[:4]
    # a budget that fits roughly one job at a time still completes everything
    with ufoir.Server(gpu_ctx, hbm_budget=1_200_000) as srv:
        handles = [srv.submit(d, s) for d, s, _ in jobs]
        assert srv.drain(120000) == ufoir.OK
        st = srv.stats()
        assert st["peak_hbm_bytes"] <= 1_200_000
        with pytest.raises(ufoir.UfoirError) as e:     # larger than the whole budget
            srv.submit(ufoir.job_desc(ufoir.METHOD_SIRT, 1448, 1200, 0.0026, num_iterations=1),
                       np.zeros((1200, 1448), np.float32))
        assert e.value.status == ufoir.ERR_BUDGET
    for (d, s, kw), (_, out) in zip(jobs, handles):
        assert np.array_equal(out, _solo(ufoir, gpu_ctx, d, s, kw))


def test_invalid_jobs_are_refused(ufoir_lib, gpu_ctx):
    ufoir = ufoir_lib
    sino = np.zeros((10, 16), np.float32)
    with ufoir.Server(gpu_ctx) as srv:
        for bad in [ufoir.job_desc(7, 16, 10, 0.1),
                    ufoir.job_desc(ufoir.METHOD_SIRT, 16, 10, 0.1, relaxation_factor=2.0),
                    ufoir.job_desc(ufoir.METHOD_SART, 16, 10, -1.0),
                    ufoir.job_desc(ufoir.METHOD_ASDPOCS, 16, 10, 0.1, asdpocs=dict(ng=5000))]:
            with pytest.raises(ufoir.UfoirError) as e:
                srv.submit(bad, sino)
            assert e.value.status == ufoir.ERR_INVALID
        assert srv.wait(12345, 0) == ufoir.ERR_NOT_FOUND


def test_cancel_and_timeout(ufoir_lib, gpu_ctx):
    ufoir = ufoir_lib
    n, na = 724, 900
    big = ufoir.job_desc(ufoir.METHOD_SART, n, na, float(np.float32(np.pi / na)), num_iterations=20)
    sino = np.ones((na, n), np.float32)
    small = ufoir.job_desc(ufoir.METHOD_SIRT, 32, 20, 0.15, num_iterations=2)
    with ufoir.Server(gpu_ctx, max_active_jobs=1) as srv:
        j1, _ = srv.submit(big, sino)
        j2, _ = srv.submit(small, np.ones((20, 32), np.float32))
        assert srv.cancel(j2) == ufoir.OK
        assert srv.poll(j2) == ufoir.JOB_CANCELLED
        assert srv.wait(j2, 0) == ufoir.ERR_CANCELLED
        assert srv.wait(j1, 1) == ufoir.ERR_TIMEOUT          # still running
        assert srv.cancel(j1) == ufoir.ERR_STATE              # running jobs are not cancelled
        assert srv.wait(j1, 300000) == ufoir.OK
        st = srv.stats()
    assert st["cancelled"] == 1 and st["completed"] == 1


def test_injected_allocation_failures_do_not_stop_the_server(ufoir_lib, gpu_ctx, oracle):
    ufoir = ufoir_lib
    jobs = _jobs(ufoir, oracle)[:6]
    with ufoir.Server(gpu_ctx, fail_allocation_every=2) as srv:
        handles = [srv.submit(d, s) for d, s, _ in jobs]
        status = [srv.wait(jid, 120000) for jid, _ in handles]
        st = srv.stats()
    assert status.count(ufoir.ERR_NOMEM) == 3 and status.count(ufoir.OK) == 3
    assert st["failed"] == 3 and st["completed"] == 3
    for (d, s, kw), (jid, out), rc in zip(jobs, handles, status):
        if rc == ufoir.OK:
            assert np.array_equal(out, _solo(ufoir, gpu_ctx, d, s, kw))


def _job_bytes(ufoir, ctx, desc, sino):
    """Device bytes the server reserves for a job (its peak alone)."""
    with ufoir.Server(ctx, policy=ufoir.SERVE_ONE_AT_A_TIME) as srv:
        jid, _ = srv.submit(desc, sino)
        assert srv.wait(jid, 120000) == ufoir.OK
        return srv.stats()["peak_hbm_bytes"]


@pytest.mark.parametrize("admit_age_ms", [60000, 1])
def test_admission_passes_a_job_that_does_not_fit_until_it_is_old(ufoir_lib, gpu_ctx, admit_age_ms):
    # X runs; Y (X's shape) does not fit beside it; Z (small) does. Z may pass
    # Y while Y is younger than admit_age_ms; once Y is older, nothing passes it.
    ufoir = ufoir_lib
    big_n, big_na = 1448, 1200
    big = ufoir.job_desc(ufoir.METHOD_SIRT, big_n, big_na, float(np.float32(np.pi / big_na)), num_iterations=200)
    small = ufoir.job_desc(ufoir.METHOD_SIRT, 64, 30, float(np.float32(np.pi / 30)), num_iterations=2)
    big_sino = np.zeros((big_na, big_n), np.float32)
    small_sino = np.ones((30, 64), np.float32)
    bx = _job_bytes(ufoir, gpu_ctx, big, big_sino)
    bz = _job_bytes(ufoir, gpu_ctx, small, small_sino)
    budget = bx + bz + (bx // 4)       # X and Z fit together, X and Y do not
    import time
    with ufoir.Server(gpu_ctx, hbm_budget=budget, admit_age_ms=admit_age_ms) as srv:
        x, _ = srv.submit(big, big_sino)
        y, _ = srv.submit(big, big_sino)
        time.sleep(0.05)
        z, _ = srv.submit(small, small_sino)
        assert srv.wait(z, 120000) == ufoir.OK
        y_state = srv.poll(y)
        for jid in (x, y):
            assert srv.wait(jid, 120000) == ufoir.OK
        st = srv.stats()
    assert st["completed"] == 3 and st["peak_hbm_bytes"] <= budget
    if admit_age_ms > 1000:
        assert y_state == ufoir.JOB_QUEUED       # Z passed Y while X was running
    else:
        assert y_state != ufoir.JOB_QUEUED       # Y was too old to be passed: Z came after it
