"""Benchmark: GDoF/s per LSRK stage of the matrix-free DG advection operator.

Workload (the plain method at GPU scale): 64^3 cells of
the sine-deformed unit cube (amplitude 0.08), FE_DGQ degree 4 (125 DoFs per
cell, 32,768,000 DoFs), velocity (1, 0.15, -0.05), periodic, upwind flux,
LSRK(5,4), Courant 0.5 / k^1.5, seeded analytic initial data.  One "step" is
one LSRK(5,4) time step = 5 fused stage launches over the whole mesh.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Our arm prints one JSON line: `value` is the FP64 operator's whole-job
GDoF/s per stage with all data resident in HBM (three 262 MB vectors plus the
geometry, larger than the 129 MB L2, so no flush is needed); `fp32_operator`
holds the FP32-operator path (FP64 vectors) with its L2 error next to the FP64
one; `e2e` repeats the FP64 measurement through the C ABI's host-buffer entry
point (adv_lsrk_steps_host), which copies the solution from pinned host memory
to the device and back around every step; `roofline` and `cpu_baseline`
explain the numbers; `serving` gives the p50/p99 solve latency of the
serving loop at a sustained arrival rate (256 requests of the serving mix,
FIFO admission) beside one-at-a-time solving; `advection_diffusion` and
`implicit` measure the two other GPU workloads (32^3 cells of degree 5 with
SIPG and the rotating field; BDF2 with FGMRES on 32^3 deformed cells).  With
--gpus N > 1 (torchrun) every rank solves its own replica (the path has no
data exchange between independent solves): weak scaling.

The reference arm (--impl reference) times the CPU oracle, the FP64 C++
restatement of the reference's algorithm (the deal.II reference cannot be
built here), with all host threads on the same workload.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = "deformed-k4-64"
WORKLOAD_DESC = ("64^3 sine-deformed cells (amplitude 0.08), degree 4, 32,768,000 DoFs, "
                 "velocity (1, 0.15, -0.05), periodic, upwind, LSRK(5,4), Courant 0.5/k^1.5")

METRIC = "GDoF/s per LSRK stage, FP64 vs FP32-op at equal L2 error; p50/p99 solve latency"
STAGES = 5


def config_dict():
    c = dict(CONFIG)
    c["workload"] = f"{WORKLOAD}: {WORKLOAD_DESC}"
    return c


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=100)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-serving", action="store_true")
    p.add_argument("--no-workloads", action="store_true",
                   help="skip the advection-diffusion and implicit workloads")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# --------------------------------------------------------------------------
# algorithmic work model of the fused stage kernel (per cell, n = k + 1)
# --------------------------------------------------------------------------
def _sweep_cost(n, anti):
    """(instructions, flops) of one 1D sweep over a pencil of n values as the
    kernel executes it: the full n x n product for n < 5, else the even-odd
    form (sums/differences of mirrored entries, two half-size products,
    recombination)."""
    if n < 5:
        return n * n, 2 * n * n - n
    h, odd = n // 2, n % 2
    inst = 2 * h + h * (h + odd + h + 2) + odd * (h + (0 if anti else 1))
    flops = 2 * h + h * (4 * h + 2 * odd) + odd * (2 * h - 1 + (0 if anti else 2))
    return inst, flops


def fp_work_per_cell(n, curved=True, stage=True, collocation=False, traces=False, upwind=False):
    """(FP instructions, flops with FMA = 2) of one fused stage per cell,
    phase by phase as in the kernels.  Nodal form (stage_kernel.cuh):
    interpolation sweeps of the own cell (3 x n^2 pencils) and of the six
    neighbour layers (2 x 6n rows), three direction passes per pencil (two
    face traces, flux, volume term with the weighted derivative, two lifts),
    1/det J, three inverse-mass sweeps and the two-FMA update per DoF.
    Collocation form (stage_gauss.cuh): no interpolation or inverse-mass
    sweeps; the neighbours' face values are n-term contractions at the 6 n^2
    face points.  With face traces the stage reads its own and the
    neighbours' face values and instead contracts the 3 n^2 pencils of its
    output (2n FMAs each) for the next stage.  Upwind traces (the upwind
    flux, where each face point reads only its upwind cell's trace): one
    n-term contraction per pencil and direction instead of two (the rare
    point that needs both is not counted), and one product per face flux
    instead of a product and an FMA."""
    si, sf = _sweep_cost(n, anti=False)
    di, df = _sweep_cost(n, anti=True)
    p = n * n
    if collocation and traces:
        nt = 1 if upwind else 2
        inst = 3 * p * nt * n
        flops = 3 * p * nt * (2 * n - 1)
    elif collocation:
        inst = 6 * p * n
        flops = 6 * p * (2 * n - 1)
    else:
        inst = 3 * p * si + 12 * n * si
        flops = 3 * p * sf + 12 * n * sf
    own_i, own_f = (0, 0) if traces else (2 * n, 2 * (2 * n - 1))
    # per pencil and direction: 4 for the two face fluxes and 2 for their
    # sum and difference, n products vt U, the lifted even-odd sweep, n lift
    # FMAs and n additions into the accumulated Z (not in the first direction)
    flux_i, flux_f = (2, 2) if upwind else (4, 6)
    pass_i = own_i + flux_i + 2 + n + di + 2 * n
    if curved and n >= 5:
        # FP64 on field geometry: the even and odd parts of vt U take one
        # product and two FMAs per mirrored pair instead of two products and
        # two additions (same flops)
        pass_i -= n // 2
    pass_f = own_f + flux_f + 2 + n + df + 4 * n
    inst += 3 * p * pass_i - p * n
    flops += 3 * p * pass_f - p * n
    if curved:
        inst += n ** 3
        flops += n ** 3
    if not collocation:
        inst += 3 * p * si
        flops += 3 * p * sf
    upd = 2 if stage else 1
    inst += upd * n ** 3
    flops += 2 * upd * n ** 3
    return inst, flops


# DRAM bytes (read + write) per DoF of one stage launch of the dominant
# kernels, from ncu captures of the 40^3 curved degree-4 case (8,000,000 DoFs,
# vectors and geometry larger than L2; profiles/ has the commands), scaled to
# the workload by the DoF count
NCU_TRAFFIC_PER_DOF = {"fp64": (531.901184e6 + 145.704960e6) / 8.0e6, "fp32": (297.173248e6 + 95.730432e6) / 8.0e6,
                       # FP32 increment stage (stage_gauss_kernel<5, float, ..., INC>), the block's
                       # dominant kernel: 19 of the 21 launches of a 4-step block
                       "fp32_increment": (309.134336e6 + 67.868928e6) / 8.0e6}

# the bench workload's config dict, identical in both arms
CONFIG = {"workload": None, "l2": "inputs larger than L2 (three 262 MB FP64 vectors + geometry per stage)"}


def increment_bytes_per_dof_step(n, interval=4, stages=STAGES):
    """Algorithmic DRAM bytes per DoF and step of the FP32 increment form in
    collocation (anchor every `interval` steps): the FP64 anchor reads u_a and
    writes K0 (FP64), K0 and G (binary32) with FP64 geometry; the first FP32
    stage reads G and K0 (binary32) and writes e (FP64) and G; the others read
    G, e, K0 and write e, G; the block's last stage reads G, e, K0 (FP64) and
    u_a and writes u; every FP32 stage reads the binary32 geometry."""
    q = interval * stages
    vec = (8 + 8 + 4 + 4) + (4 + 4 + 8 + 4) + (q - 3) * (4 + 8 + 4 + 8 + 4) + (4 + 8 + 8 + 8 + 8)
    geo = geometry_bytes_per_dof(n, 8) + (q - 1) * geometry_bytes_per_dof(n, 4)
    return (vec + geo) / interval


def traffic(per_dof, n_dofs):
    """DRAM bytes of one stage launch of the workload from the ncu figure per DoF."""
    return None if per_dof is None else round(per_dof * n_dofs)


def bytes_per_dof_step():
    """FP64 vector bytes of one LSRK(5,4) step per DoF: stage 0 reads u and
    writes u', r (24 B); stages 1-3 read r, u and write u, r (32 B); the last
    stage reads r, u and writes u (24 B)."""
    return 24 + 3 * 32 + 24


def geometry_bytes_per_dof(n, word):
    # per Gauss point 4 values (det J J^{-1} a, 1/det J); per face point 2 values, 3 faces per cell
    return 4 * word + 3 * 2 * word / n


# --------------------------------------------------------------------------
# clocks during the timed region
# --------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            # the timed region starts once the sampler is running
            t0 = time.time()
            while not self.lines and time.time() - t0 < 3.0 and self.proc.poll() is None:
                time.sleep(0.01)
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.thread.join(timeout=2)

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


# --------------------------------------------------------------------------
# reference arm and CPU baseline: the oracle on the host cores
# --------------------------------------------------------------------------
def oracle_run(steps, warmup, time_budget=None):
    from oracle import oracle as O
    O.build()
    threads = O.max_threads()
    o = O.Oracle(degree=4, n_cells=(64, 64, 64), mesh_type=1, deformation=0.08)
    dt = o.time_step(0.5)
    u = o.project(0.0)
    r, k = o.zeros(), o.zeros()
    t = 0.0
    for _ in range(warmup):
        o.lsrk_step(t, dt, u, r, k)
        t += dt
    done = 0
    t0 = time.perf_counter()
    while done < steps:
        o.lsrk_step(t, dt, u, r, k)
        t += dt
        done += 1
        if time_budget is not None and time.perf_counter() - t0 > time_budget:
            break
    el = time.perf_counter() - t0
    return dict(gdofs=o.n_dofs * STAGES * done / el / 1e9, seconds=el, steps=done, threads=threads,
                n_dofs=o.n_dofs)


def reference_arm(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    res = oracle_run(args.steps, args.warmup, time_budget=120.0)
    sample = (f"{res['steps']} full LSRK(5,4) steps of the {WORKLOAD} workload after {args.warmup} warm-up "
              f"steps, {res['seconds']:.1f} s")
    line = {
        "impl": "reference", "metric": METRIC, "value": round(res["gdofs"], 5), "unit": "GDoF/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": res["seconds"] / res["steps"] * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded analytic initial data)",
        "config": config_dict(), "arm": "CPU oracle (C++ FP64 restatement, OpenMP)",
        "cpu_baseline": {"value": round(res["gdofs"], 5), "unit": "GDoF/s", "cores": res["threads"],
                         "kind": "port", "sample": sample},
        "e2e": {"value": round(res["gdofs"], 5), "unit": "GDoF/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------
# our arm
# --------------------------------------------------------------------------
def time_steps(torch, op, adv, u, r, k, dt, steps, warmup, stream):
    """Seconds of `steps` fused steps after `warmup` untimed ones, and the
    kernel launches inside the timed region."""
    with torch.cuda.stream(stream):
        op.lsrk_steps(adv.LSRK_5_4, 0.0, dt, warmup, u, r, k, stream=stream)
        stream.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        n0 = op.launch_count()
        e0.record(stream)
        op.lsrk_steps(adv.LSRK_5_4, warmup * dt, dt, steps, u, r, k, stream=stream)
        e1.record(stream)
        e1.synchronize()
        n1 = op.launch_count()
    return e0.elapsed_time(e1) / 1e3, n1 - n0


def run_precision(torch, adv, precision, args, stream, sampler_index):
    op = adv.AdvectionOperation(adv.workload_config(WORKLOAD, precision=precision))
    dt = op.time_step(0.5)
    u = op.initialize_dof_vector()
    op.project_initial(u)
    r, k = op.initialize_dof_vector(), op.initialize_dof_vector()
    torch.cuda.synchronize()
    with ClockSampler(sampler_index) as clk:
        sec, launches = time_steps(torch, op, adv, u, r, k, dt, args.steps, args.warmup, stream)
    err, nrm = op.l2_error(u, (args.warmup + args.steps) * dt)
    return dict(op=op, u=u, r=r, k=k, dt=dt, seconds=sec, launches=launches, rel_l2=err / nrm,
                clocks=clk.summary())


def e2e_fp64(torch, adv, args, stream):
    """FP64 through the C ABI with the solution in pinned host memory: every
    step is one adv_lsrk_steps_host call, which copies the solution in, runs
    the step and copies it back (the copies in chunks of z layers, overlapped
    with the first and the last stage)."""
    op = adv.AdvectionOperation(adv.workload_config(WORKLOAD))
    dt = op.time_step(0.5)
    u = op.initialize_dof_vector()
    op.project_initial(u)
    host = torch.empty(op.n_dofs, dtype=torch.float64, pin_memory=True)
    host.copy_(u.cpu())
    r, k = op.initialize_dof_vector(), op.initialize_dof_vector()
    nb = op.n_dofs * 8

    def step(t):
        op.lsrk_steps_host(adv.LSRK_5_4, t, dt, 1, host, u, r, k, stream=stream)

    with torch.cuda.stream(stream):
        for s in range(args.warmup):
            step(s * dt)
        stream.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for s in range(args.steps):
            step((args.warmup + s) * dt)
        e1.record(stream)
        e1.synchronize()
    sec = e0.elapsed_time(e1) / 1e3
    return dict(value=op.n_dofs * STAGES * args.steps / sec / 1e9, h2d=nb, d2h=nb)


def l2_distance(torch, op, a, b):
    """Relative L2 distance ||a - b|| / ||b|| of two solutions as finite-element
    functions (norms through the mass matrix)."""
    d = a - b
    md = op.initialize_dof_vector()
    op.apply_mass(d, md)
    mb = op.initialize_dof_vector()
    op.apply_mass(b, mb)
    return float(torch.dot(d, md).sqrt() / torch.dot(b, mb).sqrt())


def advection_diffusion_run(torch, adv, stream, sampler_index, t_end=0.5):
    """The advection-diffusion workload (32^3 affine cells of degree 5,
    7,077,888 DoFs, rotating field times cos(pi t / 0.5), SIPG with
    diffusivity 1e-3 and penalty (k+1)^2/h, Dirichlet-zero data, Gaussian blob
    of width 0.1 at (0.3, 0.5, 0.5)): LSRK(5,4) to t = 0.5 with the FP64
    operator and with the FP32 operator (FP64 vectors), timed with CUDA
    events, and the L2 distance between the two final solutions."""
    out, sols = {}, {}
    for name, precision in (("fp64", adv.PRECISION_FP64), ("fp32_operator", adv.PRECISION_FP32_OPERATOR)):
        op = adv.AdvectionOperation(adv.workload_config("advection-diffusion-k5-32", precision=precision))
        dt = op.time_step(0.5)
        steps = max(1, int(-(-t_end // dt)))
        dt = t_end / steps
        u = op.initialize_dof_vector()
        op.project_initial(u)
        r, k = op.initialize_dof_vector(), op.initialize_dof_vector()
        torch.cuda.synchronize()
        with ClockSampler(sampler_index) as clk, torch.cuda.stream(stream):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            n0 = op.launch_count()
            e0.record(stream)
            op.lsrk_steps(adv.LSRK_5_4, 0.0, dt, steps, u, r, k, stream=stream)
            e1.record(stream)
            e1.synchronize()
            launches = op.launch_count() - n0
        sec = e0.elapsed_time(e1) / 1e3
        out[name] = {"value": round(op.n_dofs * STAGES * steps / sec / 1e9, 4), "unit": "GDoF/s",
                     "ms_per_step": round(sec / steps * 1e3, 4), "steps": steps, "kernel_launches": launches,
                     "clocks": clk.summary()}
        sols[name] = (op, u)
        del r, k
    op64, u64 = sols["fp64"]
    out["fp32_speedup_vs_fp64"] = round(out["fp32_operator"]["value"] / out["fp64"]["value"], 3)
    out["l2_distance_fp32_vs_fp64"] = l2_distance(torch, op64, sols["fp32_operator"][1], u64)
    out["n_dofs"] = op64.n_dofs
    out["t_end"] = t_end
    out["workload"] = ("advection-diffusion-k5-32: 32^3 affine cells, degree 5, 7,077,888 DoFs, rotating field "
                       "x cos(pi t / 0.5), SIPG nu = 1e-3, penalty (k+1)^2/h, Dirichlet-zero data, Gaussian blob "
                       "(width 0.1 at (0.3, 0.5, 0.5)), LSRK(5,4) to t = 0.5")
    del sols
    torch.cuda.empty_cache()
    return out


def implicit_run(torch, adv, stream, sampler_index, steps=50):
    """The implicit workload (32^3 deformed cells of degree 4, 4,096,000
    DoFs, the 8^3 workload's velocity and initial data): BDF2 at Courant
    number 8 with FGMRES(30) to a relative tolerance of 1e-10, the block-Jacobi
    FDM preconditioner in FP32 and, for the reference run, in FP64; iterations
    per step, time per step (CUDA events) and the L2 distance between the two
    solutions (advection_solver_implicit.cc:1865-1870 prints the iterations)."""
    op = adv.AdvectionOperation(adv.workload_config("deformed-k4-32"))
    dt = op.time_step(8.0)
    out, sols = {}, {}
    for name, precision in (("fp32_precond", adv.PRECISION_FP32_OPERATOR), ("fp64_precond", adv.PRECISION_FP64)):
        s = adv.ImplicitSolver(op, restart=30, precond_precision=precision)
        u_nm1, u_n, u_new = (op.initialize_dof_vector() for _ in range(3))
        op.project_initial(u_n)
        its = []
        torch.cuda.synchronize()
        with ClockSampler(sampler_index) as clk, torch.cuda.stream(stream):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            n0 = op.launch_count()
            e0.record(stream)
            for step in range(steps):
                its.append(s.bdf2_step((step + 1) * dt, dt, step == 0, u_n, u_nm1, u_new, rel_tol=1e-10,
                                       stream=stream))
                u_nm1, u_n, u_new = u_n, u_new, u_nm1
            e1.record(stream)
            e1.synchronize()
            launches = op.launch_count() - n0
        sec = e0.elapsed_time(e1) / 1e3
        err, nrm = op.l2_error(u_n, steps * dt)
        out[name] = {"iterations_per_step": round(sum(its) / steps, 3), "ms_per_step": round(sec / steps * 1e3, 3),
                     "rel_l2_error_vs_exact": err / nrm, "kernel_launches": launches, "clocks": clk.summary()}
        sols[name] = u_n
        s.close()
    out["l2_distance_fp32_vs_fp64_precond"] = l2_distance(torch, op, sols["fp32_precond"], sols["fp64_precond"])
    out.update(steps=steps, dt=dt, courant=8.0, n_dofs=op.n_dofs,
               workload="deformed-k4-32: 32^3 sine-deformed cells, degree 4, 4,096,000 DoFs, BDF2 (BDF1 first "
                        "step) at Courant 8, FGMRES(30) rel. tol. 1e-10, block-Jacobi FDM preconditioner")
    del sols, op
    torch.cuda.empty_cache()
    return out


# Poisson arrival rate at which the serving loop is measured: the highest
# rate of a sweep (512 requests of the mix at 2, 4, ..., 12 requests/s, FIFO)
# whose p99 latency stayed within the bound below; the GPU serves about
# 9.5-9.8 requests/s of this mix
SUSTAINED_RATE = 8.0
P99_BOUND_S = 10.0


def serving_run(n_requests=256, rate=SUSTAINED_RATE):
    """p50/p99 solve latency (arrival to completion) of the serving loop at a
    sustained Poisson arrival rate: the seeded request mix of the serving
    workload (meshes of 4^3 to 32^3 cells, degrees 2-6, end times 0.1-1,
    FP64 or FP32 operator), FIFO admission under the 150 GB budget, beside
    the same requests solved one at a time in arrival order at the same
    rate.  Each solve's relative L2 error against its exact solution is
    reported (percentiles per precision, and the list)."""
    from advection_miniapp_gb300 import serving as srv_mod
    reqs = srv_mod.request_mix(n_requests, 0, rate)
    _, srv, _ = srv_mod.run_mix(reqs, rate_clock=True, policy="fifo")
    _, base = srv_mod.run_one_at_a_time(reqs, rate_clock=True)
    keep = ("p50_latency_s", "p99_latency_s", "throughput_req_s", "gdof_stages_per_s", "wall_s")
    server = {k: round(srv[k], 4) for k in keep}
    server.update(failed=srv["failed"], ticks=srv["ticks"], kernel_launches=srv["launches"],
                  rel_l2_error=srv["rel_l2_error"])
    one = {k: round(base[k], 4) for k in keep}
    one["rel_l2_error"] = {k: v for k, v in base["rel_l2_error"].items() if k != "per_request"}
    return {"sustained_rate_req_s": rate, "p99_bound_s": P99_BOUND_S,
            "p99_within_bound": bool(srv["p99_latency_s"] <= P99_BOUND_S),
            "requests": n_requests, "admission": "FIFO under a 150 GB device-memory budget",
            "latency": "arrival to completion", "server": server, "one_at_a_time": one}


def ours(args):
    import torch
    import torch.distributed as dist

    import advection_miniapp_gb300 as adv
    from advection_miniapp_gb300 import build as b

    rank, world, local = dist_env()
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    if rank == 0:
        b.build()
    if world > 1:
        dist.barrier()
    dev_index = int(os.environ.get("CUDA_VISIBLE_DEVICES", str(local)).split(",")[local]) \
        if os.environ.get("CUDA_VISIBLE_DEVICES") else local
    stream = torch.cuda.Stream()

    fp64_peak = adv.measure_fma_peak(adv.PRECISION_FP64, stream=stream)
    # FP64 instructions in the kernels' mix of FMA, MUL and ADD (issue-slot
    # equivalent TFLOP/s, as the kernel's `achieved`)
    fp64_mix_peak = adv.measure_fma_peak(2, stream=stream)
    fp32_peak = adv.measure_fma_peak(adv.PRECISION_FP32_OPERATOR, stream=stream)

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    barrier()
    r64 = run_precision(torch, adv, adv.PRECISION_FP64, args, stream, dev_index)
    n_dofs, n_cells = r64["op"].n_dofs, r64["op"].n_cells
    del r64["op"], r64["u"], r64["r"], r64["k"]
    torch.cuda.empty_cache()
    barrier()
    r32 = run_precision(torch, adv, adv.PRECISION_FP32_OPERATOR, args, stream, dev_index)
    del r32["op"], r32["u"], r32["r"], r32["k"]
    torch.cuda.empty_cache()
    barrier()
    rinc = run_precision(torch, adv, adv.PRECISION_FP32_INCREMENT, args, stream, dev_index)
    del rinc["op"], rinc["u"], rinc["r"], rinc["k"]
    torch.cuda.empty_cache()
    barrier()

    def max_over_ranks(x):
        if world == 1:
            return x
        t = torch.tensor([x], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return t.item()

    sec64, sec32 = max_over_ranks(r64["seconds"]), max_over_ranks(r32["seconds"])
    secinc = max_over_ranks(rinc["seconds"])
    units = n_dofs * STAGES * args.steps * world
    v64, v32, vinc = units / sec64 / 1e9, units / sec32 / 1e9, units / secinc / 1e9

    e2e = None
    if not args.no_e2e:
        e = e2e_fp64(torch, adv, args, stream)
        e2e = {"value": round(e["value"] * world, 4), "unit": "GDoF/s", "h2d_bytes_per_step": e["h2d"],
               "d2h_bytes_per_step": e["d2h"]}
    barrier()

    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return

    n = 5
    # stage launch durations: the timed region over its stage launches (the
    # FP64 run adds two basis changes per lsrk_steps call, under 1 % of it)
    launch64 = r64["seconds"] / (STAGES * args.steps)
    launch32 = r32["seconds"] / (STAGES * args.steps)
    # average over the 5 launches of a step: 4 stages with 2 update FMAs per DoF, the last with 1;
    # FP64 runs the collocation form, FP32 the nodal form (the library's default choice)
    # (the workload's upwind flux with a constant velocity: upwind traces)
    inst = (4 * fp_work_per_cell(n, collocation=True, traces=True, upwind=True)[0]
            + fp_work_per_cell(n, stage=False, collocation=True, traces=True, upwind=True)[0]) / STAGES
    flops = (4 * fp_work_per_cell(n, collocation=True, traces=True, upwind=True)[1]
             + fp_work_per_cell(n, stage=False, collocation=True, traces=True, upwind=True)[1]) / STAGES
    flops32 = (4 * fp_work_per_cell(n)[1] + fp_work_per_cell(n, stage=False)[1]) / STAGES
    vec_bytes_launch = bytes_per_dof_step() / STAGES * n_dofs
    # FP64 instructions of any kind (FMA, add, mul) take one issue slot of the
    # FP64 pipe; expressed as FMA-equivalent TFLOP/s (2 flops per slot) they
    # compare with the measured FMA peak
    achieved64 = 2 * inst * n_cells / launch64 / 1e12
    algorithmic64 = flops * n_cells / launch64 / 1e12
    achieved32_hbm = vec_bytes_launch / launch32 / 1e9
    geo32 = geometry_bytes_per_dof(n, 4) * n_dofs / launch32 / 1e9
    geo64 = geometry_bytes_per_dof(n, 8) * n_dofs / launch64 / 1e9
    hbm_peak = 6780.7
    peaks_file = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_file):
        hbm_peak = json.load(open(peaks_file)).get("hbm_gbs", hbm_peak)
    inc_gbs = increment_bytes_per_dof_step(n) * n_dofs / (secinc / args.steps) / 1e9

    serving = None
    if not args.no_serving and world == 1:
        serving = serving_run()
    adv_diff = implicit = None
    if not args.no_workloads:
        adv_diff = advection_diffusion_run(torch, adv, stream, dev_index)
        implicit = implicit_run(torch, adv, stream, dev_index)

    cpu = None
    if not args.no_cpu_baseline:
        res = oracle_run(steps=10, warmup=0, time_budget=20.0)
        cpu = {"value": round(res["gdofs"], 5), "unit": "GDoF/s", "cores": res["threads"], "kind": "port",
               "sample": f"{res['steps']} LSRK(5,4) steps of the full {WORKLOAD} workload on the host cores "
                         f"({res['seconds']:.1f} s) by the FP64 C++ oracle"}

    line = {
        "metric": METRIC,
        "value": round(v64, 4),
        "unit": "GDoF/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(sec64 / args.steps * 1e3, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded analytic initial data on the deformed mesh; no dataset)",
        "config": config_dict(), "precision": "FP64 operator, FP64 vectors",
        "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
        "rel_l2_error": r64["rel_l2"],
        "roofline": {"bound": "fp64", "achieved": round(achieved64, 4), "peak": round(fp64_peak, 4),
                     "unit": "TFLOP/s", "frac": round(achieved64 / fp64_peak, 4),
                     "traffic": traffic(NCU_TRAFFIC_PER_DOF["fp64"], n_dofs),
                     "form": "collocation with upwind face traces (Gauss-point values inside lsrk_steps)",
                     "peak_source": "FP64 FMA microbenchmark (adv_measure_fma_peak) on this GPU",
                     "achieved_definition": "2 x FP64 instructions per second (each FP64 add/mul/FMA takes one "
                                            "FMA issue slot); algorithmic_tflops counts FMA = 2, add/mul = 1",
                     "algorithmic_tflops": round(algorithmic64, 4),
                     "flops_per_cell": flops, "fp64_inst_per_cell": inst,
                     "fp64_inst_frac": round(inst * n_cells / launch64 / (fp64_peak * 1e12 / 2), 4),
                     "fp64_mix_peak": round(fp64_mix_peak, 4),
                     "frac_of_mix_peak": round(achieved64 / fp64_mix_peak, 4),
                     "mix_peak_source": "adv_measure_fma_peak(2): 7 FMA, 4 MUL, 3 ADD chains per iteration",
                     "hbm_achieved_gbs": round(vec_bytes_launch / launch64 / 1e9 + geo64, 2),
                     "hbm_frac_of_measured": round((vec_bytes_launch / launch64 / 1e9 + geo64) / hbm_peak, 4),
                     "launch_ms": round(launch64 * 1e3, 4)},
        "fp32_operator": {
            "value": round(v32, 4), "unit": "GDoF/s", "speedup_vs_fp64": round(v32 / v64, 3),
            "rel_l2_error": r32["rel_l2"], "fp64_rel_l2_error": r64["rel_l2"],
            "l2_error_ratio": round(r32["rel_l2"] / r64["rel_l2"], 6),
            "ms_per_step": round(sec32 / args.steps * 1e3, 4),
            "roofline": {"bound": "hbm", "achieved": round(achieved32_hbm, 2), "peak": hbm_peak, "unit": "GB/s",
                         "frac": round(achieved32_hbm / hbm_peak, 4),
                         "traffic": traffic(NCU_TRAFFIC_PER_DOF["fp32"], n_dofs), "form": "nodal",
                         "geometry_gbs": round(geo32, 2),
                         "frac_with_geometry": round((achieved32_hbm + geo32) / hbm_peak, 4),
                         "fp32_flops_tflops": round(flops32 * n_cells / launch32 / 1e12, 3),
                         "fp32_peak_tflops": round(fp32_peak, 3), "launch_ms": round(launch32 * 1e3, 4)},
            "clocks": r32["clocks"]},
        "fp32_increment": {
            "value": round(vinc, 4), "unit": "GDoF/s", "speedup_vs_fp64": round(vinc / v64, 3),
            "rel_l2_error": rinc["rel_l2"], "l2_error_ratio": round(rinc["rel_l2"] / r64["rel_l2"], 6),
            "ms_per_step": round(secinc / args.steps * 1e3, 4),
            "form": "per 4 steps (anchor_interval 4) one FP64 operator evaluation K0 = L(u_a) at the block's "
                    "start u_a and 19 FP32 operator evaluations on the increments r - u_a (u - u_a - C K0 kept in "
                    "FP64, the operator input in binary32); collocation basis",
            "roofline": {"bound": "hbm", "achieved": round(inc_gbs, 2), "peak": hbm_peak, "unit": "GB/s",
                         "frac": round(inc_gbs / hbm_peak, 4),
                         "traffic": traffic(NCU_TRAFFIC_PER_DOF["fp32_increment"], n_dofs),
                         "traffic_definition": "DRAM bytes of one FP32 increment stage launch (the block's "
                                               "dominant kernel), ncu at 40^3 scaled by the DoFs",
                         "bytes_per_dof_step": round(increment_bytes_per_dof_step(n), 2),
                         "definition": "algorithmic vector and geometry bytes of a 4-step block (one FP64 anchor "
                                       "and 19 FP32 stages) over the block's time"},
            "clocks": rinc["clocks"]},
        "e2e": e2e,
        "serving": serving,
        "advection_diffusion": adv_diff,
        "implicit": implicit,
        "gpu_launches": r64["launches"] + r32["launches"] + rinc["launches"],
        "clocks": r64["clocks"],
        "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        reference_arm(args)
    else:
        ours(args)


if __name__ == "__main__":
    main()
