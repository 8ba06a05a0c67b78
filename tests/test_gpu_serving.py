"""Serving loop on the GPU: every solve of a batched mix gives the same
result as the same request served alone and as the single-mesh LSRK loop,
the FP64 path matches the oracle, and admission respects the memory budget."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def small_mix(seed=0, n=14):
    from advection_miniapp_gb300.serving import request_mix
    return request_mix(n, seed=seed, sizes=(2, 3, 4), degrees=(1, 2, 3, 4, 5, 6), t_range=(0.02, 0.12))


def test_mix_equals_alone_and_single_mesh(cuda, adv_lib):
    from advection_miniapp_gb300.serving import STATE_DONE, Server, run_mix
    reqs = small_mix()
    # several degrees and both precisions share the device; step counts are
    # not multiples of the tick length
    assert len({(r.degree, r.precision) for r in reqs}) >= 4
    results, summary, mixed = run_mix(reqs, rate_clock=False, steps_per_tick=4, keep_solutions=True)
    assert all(results[r.index]["state"] == STATE_DONE for r in reqs)
    for r in reqs:
        with Server(keep_solutions=True, steps_per_tick=3) as srv:
            rid = srv.submit(r)
            srv.drain()
            alone = srv.solution(rid, r.n_dofs)
            res = srv.result(rid)
        np.testing.assert_array_equal(alone, mixed[r.index])
        assert res["rel_l2_error"] == results[r.index]["rel_l2_error"]
        # the single-mesh operator with the same step
        op = adv_lib.AdvectionOperation(r.config())
        u, rr, k = (op.initialize_dof_vector() for _ in range(3))
        op.project_initial(u)
        op.lsrk_steps(adv_lib.LSRK_5_4, 0.0, res["dt"], res["steps"], u, rr, k)
        np.testing.assert_array_equal(u.cpu().numpy(), alone)
        err, nrm = op.l2_error(u, r.t_end)
        assert abs(err / nrm - res["rel_l2_error"]) <= 1e-12 * max(1.0, err / nrm)
        assert np.isfinite(res["rel_l2_error"])


def test_fp64_request_matches_oracle(cuda, oracle_mod):
    from advection_miniapp_gb300.serving import Request, Server
    r = Request(0, 3, 3, (0.6, -0.48, 0.64), (0.25, 0.5, 0.125), 0.05, 0)
    with Server(keep_solutions=True) as srv:
        rid = srv.submit(r)
        srv.drain()
        u = srv.solution(rid, r.n_dofs)
        res = srv.result(rid)
    o = oracle_mod.Oracle(degree=3, n_cells=(3, 3, 3), velocity=r.velocity, ic_params=r.phase)
    ou, orr, ok = o.project(0.0), o.zeros(), o.zeros()
    for s in range(res["steps"]):
        o.lsrk_step(s * res["dt"], res["dt"], ou, orr, ok)
    assert np.abs(u - ou).max() <= 1e-12 * np.abs(ou).max()
    err, nrm = o.l2_error(ou, r.t_end)
    assert abs(res["rel_l2_error"] - err / nrm) <= 1e-10 * err / nrm


def test_budget_limits_concurrency(cuda, adv_lib):
    from advection_miniapp_gb300.serving import Server
    reqs = small_mix(seed=5, n=10)
    biggest = max(r.device_bytes() for r in reqs)
    budget = 2 * biggest
    with Server(memory_budget_bytes=budget, steps_per_tick=2, keep_solutions=True) as srv:
        ids = [srv.submit(r) for r in reqs]
        peak_bytes, peak_running, done = 0, 0, 0
        while done < len(reqs):
            done += srv.poll()
            st = srv.stats()
            peak_bytes = max(peak_bytes, st["device_bytes"])
            peak_running = max(peak_running, st["running"])
        assert peak_bytes <= budget
        assert srv.stats()["device_bytes"] == 0
        assert 1 <= peak_running < len(reqs)
        limited = [srv.solution(i, r.n_dofs) for i, r in zip(ids, reqs)]
    with Server(keep_solutions=True, max_active=3) as srv:
        ids = [srv.submit(r) for r in reqs]
        srv.drain()
        assert srv.stats()["completed"] == len(reqs)
        capped = [srv.solution(i, r.n_dofs) for i, r in zip(ids, reqs)]
    for a, b in zip(limited, capped):
        np.testing.assert_array_equal(a, b)


def test_rejected_requests(cuda, adv_lib):
    from advection_miniapp_gb300.serving import Request, Server
    r = Request(0, 4, 3, (1.0, 0.0, 0.0), (0.0, 0.0, 0.0), 0.1, 0)
    with Server(memory_budget_bytes=r.device_bytes() - 1) as srv:
        with pytest.raises(adv_lib.AdvError):
            srv.submit(r)
    with Server() as srv:
        cfg = r.config()
        cfg.periodic = 0
        with pytest.raises(adv_lib.AdvError):
            srv.submit_config(cfg, 0.1)
        cfg = r.config()
        cfg.mesh_type = adv_lib.MESH_DEFORMED
        with pytest.raises(adv_lib.AdvError):
            srv.submit_config(cfg, 0.1)
        with pytest.raises(adv_lib.AdvError):
            srv.submit_config(r.config(), -1.0)
        assert srv.stats()["submitted"] == 0


def test_request_that_cannot_be_allocated_fails_alone(cuda, adv_lib):
    """A request within the budget whose buffers exceed the device memory by
    far (1024^3 cells of degree 6: 2.9 TB per vector against 288 GB of HBM)
    fails at admission with state 3; the other requests are served as usual."""
    from advection_miniapp_gb300.serving import STATE_DONE, STATE_FAILED, Request, Server
    small = Request(0, 3, 2, (1.0, 0.0, 0.0), (0.0, 0.0, 0.0), 0.05, 0)
    huge = Request(1, 1024, 6, (1.0, 0.0, 0.0), (0.0, 0.0, 0.0), 0.001, 0)
    with Server(memory_budget_bytes=10 ** 14) as srv:
        ids = [srv.submit(small), srv.submit(huge), srv.submit(small)]
        srv.drain()
        states = [srv.result(i)["state"] for i in ids]
        assert states == [STATE_DONE, STATE_FAILED, STATE_DONE]
        assert srv.stats()["device_bytes"] == 0 and srv.stats()["completed"] == 3


def test_shortest_first_policy_same_results(cuda, adv_lib):
    """Admission order changes latency, not results: shortest-first with a
    small concurrency cap gives the FIFO results bit for bit, and finishes
    the smallest request before the largest."""
    from advection_miniapp_gb300.serving import run_mix
    reqs = small_mix(seed=9, n=12)
    res_f, _, sol_f = run_mix(reqs, rate_clock=False, keep_solutions=True)
    res_s, _, sol_s = run_mix(reqs, rate_clock=False, keep_solutions=True, policy="shortest", max_active=2)
    for r in reqs:
        np.testing.assert_array_equal(sol_f[r.index], sol_s[r.index])
    work = {r.index: r.work() for r in reqs}
    small, big = min(work, key=work.get), max(work, key=work.get)
    assert res_s[small]["latency_s"] < res_s[big]["latency_s"]


def test_cancel_queued_and_running_requests(cuda, adv_lib):
    """Cancelling frees the request's memory and lets the others finish with
    the results they have alone."""
    from advection_miniapp_gb300.serving import (STATE_CANCELLED, STATE_DONE, STATE_RUNNING, Request, Server)
    long_run = Request(0, 4, 3, (1.0, 0.0, 0.0), (0.0, 0.0, 0.0), 5.0, 0)   # about 700 steps
    short = Request(1, 3, 2, (0.0, 1.0, 0.0), (0.0, 0.0, 0.0), 0.05, 1)
    with Server(keep_solutions=True, max_active=1, steps_per_tick=2) as srv:
        a = srv.submit(long_run)
        b = srv.submit(short)
        c = srv.submit(short)
        srv.poll()                                   # admits a only (max_active 1)
        assert srv.result(a)["state"] == STATE_RUNNING
        srv.cancel(b)                                # queued: leaves at once
        assert srv.result(b)["state"] == STATE_CANCELLED
        srv.cancel(a)                                # running: leaves after its tick
        srv.drain()
        assert srv.result(a)["state"] == STATE_CANCELLED
        assert srv.result(c)["state"] == STATE_DONE
        st = srv.stats()
        assert st["device_bytes"] == 0 and st["completed"] == 3 and st["running"] == 0
        with pytest.raises(adv_lib.AdvError):
            srv.cancel(c)
        sol = srv.solution(c, short.n_dofs)
    with Server(keep_solutions=True) as srv:
        rid = srv.submit(short)
        srv.drain()
        np.testing.assert_array_equal(srv.solution(rid, short.n_dofs), sol)


def test_call_timing(cuda, adv_lib):
    """adv_set_timing / adv_timing: the device time of the timed calls
    (outermost only), like the reference's computing_times."""
    op = adv_lib.AdvectionOperation(degree=3, n_cells=(6, 6, 6), mesh_type=1, deformation=0.05)
    u, r, k = (op.initialize_dof_vector() for _ in range(3))
    op.project_initial(u)
    assert op.timing() == (0.0, 0)
    op.set_timing(True)
    op.lsrk_steps(adv_lib.LSRK_5_4, 0.0, 1e-3, 4, u, r, k)
    d = op.initialize_dof_vector()
    op.apply(u, d, 0.0)
    sec, calls = op.timing()
    assert calls == 2 and sec > 0.0
    op.set_timing(False)
    op.apply(u, d, 0.0)
    assert op.timing()[1] == 2
