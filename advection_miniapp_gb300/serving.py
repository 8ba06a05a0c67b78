"""Serving loop: many independent advection solves on one GPU.

`Server` wraps the adv_server_* C ABI: requests (periodic affine n^3 meshes,
constant velocity, degree 1..6, FP64 or FP32 operator) are admitted FIFO under
a device-memory budget, batched per (degree, precision) into graph-captured
multi-solve stage launches, and retired with their relative L2 error against
the exactly translated initial data.  The reference runs one solve per program
(advection_solver.cc:1323-1372); this loop has no counterpart there.

`request_mix` draws the request stream of the serving workload (every request
from its own seed): n uniform in {4,6,8,12,16,24,32}, degree uniform in
{2..6}, velocity with uniform components in [-1, 1] normalised to length 1,
the sine-product + Gaussian initial data shifted by a uniform phase in
[0,1)^3, end time uniform in [0.1, 1], LSRK(5,4) at Courant number 0.5, a
precision tag FP64 or FP32-operator, Poisson arrivals at a given rate.

    python -m advection_miniapp_gb300.serving --requests 256 --rate 200 --budget-gb 150
"""
import argparse
import ctypes
import json
import time
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import IC_SINE_GAUSS, MESH_CARTESIAN, PRECISION_FP32_OPERATOR, PRECISION_FP64

SIZES = (4, 6, 8, 12, 16, 24, 32)
DEGREES = (2, 3, 4, 5, 6)
STATE_QUEUED, STATE_RUNNING, STATE_DONE, STATE_FAILED, STATE_CANCELLED = 0, 1, 2, 3, 4
POLICIES = {"fifo": 0, "shortest": 1}


@dataclass
class Request:
    index: int
    n: int
    degree: int
    velocity: tuple
    phase: tuple
    t_end: float
    precision: int
    arrival: float = 0.0
    courant: float = 0.5

    @property
    def n_dofs(self):
        return self.n ** 3 * (self.degree + 1) ** 3

    def steps(self):
        """Step count of the time-step rule (advection_solver.cc:1155-1167)."""
        dt = self.courant * (1.0 / self.n) / np.linalg.norm(self.velocity) / self.degree ** 1.5
        return max(1, int(np.ceil(self.t_end / dt - 1e-12)))

    def device_bytes(self):
        """Device memory the server reserves for the solve: u, r, k and, for
        the FP64 operator (collocation form), two face-trace buffers of
        6 (k+1)^2 values per cell."""
        b = 3 * 8 * self.n_dofs
        if self.precision == PRECISION_FP64:
            b += 2 * 6 * 8 * self.n_dofs // (self.degree + 1)
        return b

    def work(self):
        """DoF-stages of the solve (5 stages per step)."""
        return self.n_dofs * 5 * self.steps()

    def config(self):
        from . import make_config
        return make_config(degree=self.degree, n_cells=(self.n,) * 3, mesh_type=MESH_CARTESIAN, periodic=1,
                           velocity=self.velocity, flux_alpha=1.0, initial_condition=IC_SINE_GAUSS,
                           ic_params=tuple(self.phase) + (0.0,) * 5, precision=self.precision)


def request_mix(n_requests, seed=0, rate=None, sizes=SIZES, degrees=DEGREES, t_range=(0.1, 1.0),
                precisions=(PRECISION_FP64, PRECISION_FP32_OPERATOR)):
    """Seeded request stream; request i depends only on (seed, i).  With a
    rate (requests/s) the arrivals are a Poisson process starting at 0."""
    arrivals = np.zeros(n_requests)
    if rate:
        arrivals = np.cumsum(np.random.default_rng([seed, 1 << 30]).exponential(1.0 / rate, n_requests))
        arrivals -= arrivals[0]
    out = []
    for i in range(n_requests):
        g = np.random.default_rng([seed, i])
        n = int(g.choice(sizes))
        k = int(g.choice(degrees))
        v = g.uniform(-1.0, 1.0, 3)
        while np.linalg.norm(v) < 1e-3:
            v = g.uniform(-1.0, 1.0, 3)
        v = v / np.linalg.norm(v)
        phase = g.uniform(0.0, 1.0, 3)
        t_end = float(g.uniform(*t_range))
        prec = int(precisions[int(g.integers(len(precisions)))])
        out.append(Request(i, n, k, tuple(float(x) for x in v), tuple(float(x) for x in phase), t_end, prec,
                           float(arrivals[i])))
    return out


class Server:
    """Python face of adv_server (not thread-safe, like the C object)."""

    def __init__(self, memory_budget_bytes=150 * 10 ** 9, steps_per_tick=8, max_active=4096, keep_solutions=False,
                 policy="fifo"):
        import torch
        torch.cuda.init()
        self._lib = _lib.load()
        self._s = ctypes.c_void_p()
        _lib.check(self._lib.adv_server_create(int(memory_budget_bytes), steps_per_tick, max_active,
                                               1 if keep_solutions else 0, ctypes.byref(self._s)),
                   "adv_server_create")
        _lib.check(self._lib.adv_server_set_policy(self._s, POLICIES[policy]), "adv_server_set_policy")

    def close(self):
        if getattr(self, "_s", None):
            self._lib.adv_server_destroy(self._s)
            self._s = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def submit_config(self, config, t_end, courant=0.5):
        rid = ctypes.c_int64()
        _lib.check(self._lib.adv_server_submit(self._s, ctypes.byref(config), float(t_end), float(courant),
                                               ctypes.byref(rid)), "adv_server_submit")
        return rid.value

    def submit(self, req):
        return self.submit_config(req.config(), req.t_end, req.courant)

    def poll(self):
        n = ctypes.c_int()
        _lib.check(self._lib.adv_server_poll(self._s, ctypes.byref(n)), "adv_server_poll")
        return n.value

    def cancel(self, rid):
        """Queued: leaves at once; running: at the end of its group's tick."""
        _lib.check(self._lib.adv_server_cancel(self._s, rid), "adv_server_cancel")

    def drain(self):
        _lib.check(self._lib.adv_server_drain(self._s), "adv_server_drain")

    def result(self, rid):
        st, steps = ctypes.c_int(), ctypes.c_int()
        err, lat, dt = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        _lib.check(self._lib.adv_server_result(self._s, rid, ctypes.byref(st), ctypes.byref(err), ctypes.byref(lat),
                                               ctypes.byref(steps), ctypes.byref(dt)), "adv_server_result")
        return {"state": st.value, "rel_l2_error": err.value, "latency_s": lat.value, "steps": steps.value,
                "dt": dt.value}

    def solution(self, rid, n_dofs):
        out = np.empty(n_dofs)
        _lib.check(self._lib.adv_server_solution(self._s, rid, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                                 n_dofs), "adv_server_solution")
        return out

    def stats(self):
        a = (ctypes.c_int64 * 8)()
        _lib.check(self._lib.adv_server_stats(self._s, a), "adv_server_stats")
        keys = ("submitted", "queued", "running", "completed", "device_bytes", "budget", "ticks", "launches")
        return dict(zip(keys, list(a)))


def run_mix(requests, rate_clock=True, memory_budget_bytes=150 * 10 ** 9, steps_per_tick=8, max_active=4096,
            keep_solutions=False, policy="fifo"):
    """Drive a server with the request stream: each request is submitted
    when the wall clock passes its arrival time (all at once without
    rate_clock).  Returns (results, summary, server solutions or None)."""
    import torch
    order = sorted(requests, key=lambda r: r.arrival)
    with Server(memory_budget_bytes, steps_per_tick, max_active, keep_solutions, policy) as srv:
        ids = {}
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        nxt = 0
        done = 0
        while done < len(order):
            now = time.perf_counter() - t0
            while nxt < len(order) and (not rate_clock or order[nxt].arrival <= now):
                ids[order[nxt].index] = srv.submit(order[nxt])
                nxt += 1
            done += srv.poll()
            if done < len(order) and nxt < len(order) and rate_clock:
                wait = order[nxt].arrival - (time.perf_counter() - t0)
                if wait > 0 and srv.stats()["running"] == 0:
                    time.sleep(min(wait, 0.01))
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        results = {i: srv.result(rid) for i, rid in ids.items()}
        sols = None
        if keep_solutions:
            sols = {r.index: srv.solution(ids[r.index], r.n_dofs) for r in requests}
        stats = srv.stats()
    lat = np.array([results[r.index]["latency_s"] for r in requests])
    work = sum(r.work() for r in requests)
    failed = sum(results[r.index]["state"] == STATE_FAILED for r in requests)
    summary = {"requests": len(requests), "failed": int(failed), "wall_s": wall,
               "throughput_req_s": len(requests) / wall,
               "p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
               "gdof_stages_per_s": work / wall / 1e9, "ticks": stats["ticks"], "launches": stats["launches"],
               "max_rel_l2_error": max(results[r.index]["rel_l2_error"] for r in requests),
               "rel_l2_error": error_summary(requests, results)}
    return results, summary, sols


def error_summary(requests, results):
    """Relative L2 errors of the solves (each against its exactly translated
    initial data): percentiles per precision tag and the whole list in
    request order."""
    out = {}
    for name, tag in (("fp64", PRECISION_FP64), ("fp32_operator", PRECISION_FP32_OPERATOR)):
        e = np.array([results[r.index]["rel_l2_error"] for r in requests if r.precision == tag])
        if len(e):
            out[name] = {"count": int(len(e)), "p50": float(np.percentile(e, 50)),
                         "p99": float(np.percentile(e, 99)), "max": float(e.max())}
    out["per_request"] = [float(results[r.index]["rel_l2_error"]) for r in sorted(requests, key=lambda q: q.index)]
    return out


def run_one_at_a_time(requests, rate_clock=True):
    """Baseline: a single worker serving the requests one after another in
    arrival order, each through its own AdvectionOperation and the fused LSRK
    step loop; a request waits for its arrival time (with rate_clock) and for
    the requests before it.  Latency = completion - arrival, as for the
    server.  Returns (results, summary)."""
    import torch

    from . import AdvectionOperation, LSRK_5_4
    results = {}
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for r in sorted(requests, key=lambda q: q.arrival):
        arrival = r.arrival if rate_clock else 0.0
        wait = arrival - (time.perf_counter() - t0)
        if wait > 0:
            time.sleep(wait)
        op = AdvectionOperation(r.config())
        steps = r.steps()
        dt = r.t_end / steps
        u, rr, k = (op.initialize_dof_vector() for _ in range(3))
        op.project_initial(u)
        op.lsrk_steps(LSRK_5_4, 0.0, dt, steps, u, rr, k)
        err, nrm = op.l2_error(u, r.t_end)
        results[r.index] = {"rel_l2_error": err / nrm, "latency_s": time.perf_counter() - t0 - arrival,
                            "steps": steps, "dt": dt}
        op.close()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    work = sum(r.work() for r in requests)
    lat = np.array([results[r.index]["latency_s"] for r in requests])
    summary = {"requests": len(requests), "wall_s": wall, "throughput_req_s": len(requests) / wall,
               "p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
               "gdof_stages_per_s": work / wall / 1e9, "rel_l2_error": error_summary(requests, results)}
    return results, summary


def launch_overhead(cases=((4, 2), (8, 4), (16, 4))):
    """Per-launch cost of small solves: one FP64 request of n^3 cells of
    degree k through the single-mesh step loop (stream launches, timed with
    CUDA events and on the host clock) and through the server (graph-captured
    ticks of 8 or 32 steps, alone or 16 copies batched in one group), as host
    wall time per kernel launch of the tick graphs."""
    import torch

    from . import AdvectionOperation, LSRK_5_4
    out = {}
    for n, k in cases:
        r = Request(0, n, k, (0.6, -0.48, 0.64), (0.1, 0.2, 0.3), 4.0 if n == 4 else 1.0, PRECISION_FP64)
        steps = r.steps()
        dt = r.t_end / steps
        op = AdvectionOperation(r.config())
        u, rr, kk = (op.initialize_dof_vector() for _ in range(3))
        op.project_initial(u)
        op.lsrk_steps(LSRK_5_4, 0.0, dt, 10, u, rr, kk)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        n0 = op.launch_count()
        t0 = time.perf_counter()
        e0.record()
        op.lsrk_steps(LSRK_5_4, 0.0, dt, steps, u, rr, kk)
        e1.record()
        e1.synchronize()
        wall = time.perf_counter() - t0
        nl = op.launch_count() - n0
        res = {"steps": steps, "n_dofs": r.n_dofs, "stream_launches": nl,
               "stream_us_per_launch_device": e0.elapsed_time(e1) * 1e3 / nl,
               "stream_us_per_launch_wall": wall * 1e6 / nl}
        op.close()
        for spt in (8, 32):
            for copies in (1, 16):
                with Server(steps_per_tick=spt) as srv:
                    torch.cuda.synchronize()
                    t0 = time.perf_counter()
                    for _ in range(copies):
                        srv.submit(r)
                    srv.drain()
                    torch.cuda.synchronize()
                    wall = time.perf_counter() - t0
                    st = srv.stats()
                res[f"server_spt{spt}_x{copies}"] = {"wall_s": wall, "ticks": st["ticks"], "launches": st["launches"],
                                                     "us_per_graph_node": wall * 1e6 / st["launches"]}
        out[f"{n}^3 k{k}"] = res
    return out


def main(argv=None):
    p = argparse.ArgumentParser(description="serving-loop measurement on one GPU")
    p.add_argument("--requests", type=int, default=256)
    p.add_argument("--rate", type=float, default=200.0, help="Poisson arrival rate (requests/s); 0: all at once")
    p.add_argument("--seed", type=int, default=0)
    p.add_argument("--budget-gb", type=float, default=150.0)
    p.add_argument("--steps-per-tick", type=int, default=8)
    p.add_argument("--max-active", type=int, default=4096, help="solves on the device at once")
    p.add_argument("--policy", choices=sorted(POLICIES), default="fifo", help="admission order")
    p.add_argument("--t-max", type=float, default=1.0, help="upper end of the end-time range [0.1, t_max]")
    p.add_argument("--baseline", action="store_true", help="also run the requests one at a time")
    p.add_argument("--overhead", action="store_true",
                   help="only measure the per-launch cost of small solves (stream launches vs tick graphs)")
    args = p.parse_args(argv)
    if args.overhead:
        print(json.dumps(launch_overhead()))
        return
    reqs = request_mix(args.requests, args.seed, args.rate or None, t_range=(0.1, args.t_max))
    _, summary, _ = run_mix(reqs, rate_clock=bool(args.rate), memory_budget_bytes=int(args.budget_gb * 1e9),
                            steps_per_tick=args.steps_per_tick, max_active=args.max_active, policy=args.policy)
    out = {"rate_req_s": args.rate, "seed": args.seed, "t_range": [0.1, args.t_max], "policy": args.policy,
           "max_active": args.max_active, "serving": summary}
    if args.baseline:
        _, base = run_one_at_a_time(reqs, rate_clock=bool(args.rate))
        out["one_at_a_time"] = base
    print(json.dumps(out))


if __name__ == "__main__":
    main()
