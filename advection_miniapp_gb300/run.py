"""Command-line driver: the counterpart of the reference's AdvectionProblem::run
and main() (advection_solver.cc:1246-1318, 1323-1372).

    python -m advection_miniapp_gb300.run --mesh deformed --cells 64 --degree 4 \
        --steps 100 --precision fp64 [--output-every 20]

Builds the operator (reinit), sets the time step by the reference's rule
(Courant number / k^1.5, advection_solver.cc:1155-1167), projects the initial
data, runs the low-storage Runge-Kutta loop and prints the relative L2 error,
mass, energy and H1 seminorm at the output steps, then the time per step and
per element like the reference's summary (advection_solver.cc:1302-1311).
"""
import argparse
import json
import math
import time

import torch

from . import (FORM_AUTO, FORM_COLLOCATION, FORM_COLLOCATION_NO_TRACES, FORM_NODAL, AdvectionOperation, IC_BLOB, IC_SINE_GAUSS, IC_WAVE, LSRK_3_3, LSRK_5_4, LSRK_7_4, LSRK_9_5,
               LowStorageRungeKuttaIntegrator, MESH_CARTESIAN, MESH_DEFORMED, PRECISION_FP32_INCREMENT,
               PRECISION_FP32_OPERATOR,
               PRECISION_FP64, VELOCITY_ROTATING, make_config, workload_config)

SCHEMES = {"3_3": LSRK_3_3, "5_4": LSRK_5_4, "7_4": LSRK_7_4, "9_5": LSRK_9_5}
ICS = {"sine-gauss": IC_SINE_GAUSS, "blob": IC_BLOB, "wave": IC_WAVE}


def parse(argv=None):
    p = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    p.add_argument("--workload", default=None,
                   help="a named workload (workload_config) instead of the mesh/degree/velocity options")
    p.add_argument("--t-end", type=float, default=None,
                   help="run to this time (steps = ceil(t_end / dt), dt rounded to t_end / steps)")
    p.add_argument("--mesh", choices=["cartesian", "deformed"], default="cartesian")
    p.add_argument("--cells", type=int, default=8, help="cells per direction")
    p.add_argument("--degree", type=int, default=3)
    p.add_argument("--deformation", type=float, default=0.08)
    p.add_argument("--velocity", type=float, nargs=3, default=(1.0, 0.15, -0.05))
    p.add_argument("--initial-condition", choices=sorted(ICS), default="sine-gauss")
    p.add_argument("--courant", type=float, default=0.5)
    p.add_argument("--steps", type=int, default=200)
    p.add_argument("--scheme", choices=sorted(SCHEMES), default="5_4")
    p.add_argument("--precision", choices=["fp64", "fp32", "fp32-increment"], default="fp64",
                   help="FP64 operator, FP32 operator, or FP32 operator on the stage increments with one FP64 "
                        "evaluation per anchor interval")
    p.add_argument("--anchor-interval", type=int, default=0,
                   help="fp32-increment: steps per FP64 anchor evaluation (0: the library default, 4)")
    p.add_argument("--form", choices=["auto", "nodal", "collocation", "collocation-no-traces"], default="auto",
                   help="basis of the stages inside the fused step loop (fused_form)")
    p.add_argument("--flux-alpha", type=float, default=1.0)
    p.add_argument("--skew", type=float, default=0.0)
    p.add_argument("--output-every", type=int, default=0, help="0: only at the start and the end")
    p.add_argument("--json", action="store_true", help="print one JSON summary line")
    p.add_argument("--vtu", default=None, metavar="PREFIX",
                   help="write PREFIX_NNN.vtu (solution and analytic solution) at every output step")
    p.add_argument("--save-state", default=None, metavar="PATH", help="write the final state for a restart")
    p.add_argument("--compare-fp64", action="store_true",
                   help="FP32 operator: rerun with the FP64 operator and report both errors and the difference")
    p.add_argument("--implicit", action="store_true",
                   help="BDF2 steps with FGMRES and the block-Jacobi FDM preconditioner instead of LSRK")
    p.add_argument("--restart", type=int, default=30, help="FGMRES restart length (implicit)")
    p.add_argument("--tolerance", type=float, default=1e-10, help="FGMRES relative tolerance (implicit)")
    p.add_argument("--precond-precision", choices=["fp64", "fp32"], default="fp32",
                   help="precision of the FDM preconditioner (implicit)")
    p.add_argument("--compare-fp64-precond", action="store_true",
                   help="implicit: rerun with the FP64 preconditioner and report the difference")
    return p.parse_args(argv)


def run_implicit(args, op):
    """BDF2 + FGMRES: the implicit workload (advection_solver_implicit.cc:1788-1886 with BDF2)."""
    import time as _time

    from . import ImplicitSolver, PRECISION_FP32_OPERATOR, PRECISION_FP64

    dt = op.time_step(args.courant)

    def solve(precond):
        s = ImplicitSolver(op, restart=args.restart, precond_precision=precond)
        u_nm1, u_n, u_new = (op.initialize_dof_vector() for _ in range(3))
        op.project_initial(u_n)
        its = []
        torch.cuda.synchronize()
        t0 = _time.perf_counter()
        for step in range(args.steps):
            its.append(s.bdf2_step((step + 1) * dt, dt, step == 0, u_n, u_nm1, u_new, rel_tol=args.tolerance))
            u_nm1, u_n, u_new = u_n, u_new, u_nm1
        torch.cuda.synchronize()
        return u_n, its, _time.perf_counter() - t0

    prec = PRECISION_FP32_OPERATOR if args.precond_precision == "fp32" else PRECISION_FP64
    u, its, wall = solve(prec)
    err, nrm = op.l2_error(u, args.steps * dt)
    out = {"n_dofs": op.n_dofs, "steps": args.steps, "dt": dt, "t_end": args.steps * dt, "courant": args.courant,
           "precond_precision": args.precond_precision, "iterations_per_step": sum(its) / len(its),
           "iterations": its, "rel_l2_error": err / nrm, "s_per_step": wall / args.steps}
    if args.compare_fp64_precond:
        u64, its64, _ = solve(PRECISION_FP64)
        e64, n64 = op.l2_error(u64, args.steps * dt)
        d = (u - u64)
        out["fp64_precond"] = {"iterations_per_step": sum(its64) / len(its64), "rel_l2_error": e64 / n64,
                               "max_rel_difference": float(d.abs().max() / u64.abs().max())}
    return out


def main(argv=None):
    args = parse(argv)
    precision = {"fp64": PRECISION_FP64, "fp32": PRECISION_FP32_OPERATOR,
                 "fp32-increment": PRECISION_FP32_INCREMENT}[args.precision]
    if args.workload:
        cfg = workload_config(args.workload, precision=precision)
    else:
        cfg = make_config(degree=args.degree, n_cells=(args.cells,) * 3,
                          mesh_type=MESH_DEFORMED if args.mesh == "deformed" else MESH_CARTESIAN,
                          deformation=args.deformation if args.mesh == "deformed" else 0.0,
                          velocity=tuple(args.velocity), initial_condition=ICS[args.initial_condition],
                          flux_alpha=args.flux_alpha, factor_skew=args.skew, precision=precision)
    cfg.anchor_interval = args.anchor_interval
    cfg.fused_form = {"auto": FORM_AUTO, "nodal": FORM_NODAL, "collocation": FORM_COLLOCATION,
                      "collocation-no-traces": FORM_COLLOCATION_NO_TRACES}[args.form]
    op = AdvectionOperation(cfg)
    if args.implicit:
        res = run_implicit(args, op)
        if args.json:
            print(json.dumps(res))
        else:
            for k, v in res.items():
                print(f"   {k}: {v}")
        return
    integ = LowStorageRungeKuttaIntegrator(SCHEMES[args.scheme])
    dt = op.time_step(args.courant)
    if args.t_end is not None:
        # rounding of setup_dofs (advection_solver.cc:1161-1167)
        args.steps = max(1, math.ceil(args.t_end / dt - 1e-12))
        dt = args.t_end / args.steps
    if not args.json:
        print(f"   Number of elements:            {op.n_cells}")
        print(f"   Polynomial degree:             {op.degree}")
        print(f"   Number of degrees of freedom:  {op.n_dofs}")
        print(f"   Time step size: {dt:.6g}")
    u = op.initialize_dof_vector()
    op.project_initial(u)
    r, k = op.initialize_dof_vector(), op.initialize_dof_vector()
    u_start = u.clone() if cfg.velocity_type == VELOCITY_ROTATING else None

    n_out = [0]

    def output(step, t):
        err, nrm = op.l2_error(u, t)
        me = op.compute_mass_and_energy(u)
        if args.vtu:
            op.write_vtu(u, t, f"{args.vtu}_{n_out[0]:03d}.vtu")
            n_out[0] += 1
        if not args.json:
            print(f"   Time {t:8.3g}  error {err / nrm:10.5g}  mass {me[0]:16.10g}  energy {me[1]:16.10g}"
                  f"  H1-semi {me[2]:9.4g}")
        return err / nrm, me

    output(0, 0.0)
    t = 0.0
    wall = 0.0
    step = 0
    chunk = args.output_every if args.output_every > 0 else args.steps
    while step < args.steps:
        n = min(chunk, args.steps - step)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        if n == 1:
            integ.perform_time_step(op, t, dt, u, r, k)
        else:
            op.lsrk_steps(integ.scheme, t, dt, n, u, r, k)
        torch.cuda.synchronize()
        wall += time.perf_counter() - t0
        step += n
        t = step * dt
        if args.output_every > 0 or step == args.steps:
            rel, me = output(step, t)
    if args.save_state:
        op.save_state(u, t, args.save_state)
    per_step = wall / max(args.steps, 1)
    stage_rate = op.n_dofs * integ.n_stages() * args.steps / wall / 1e9 if wall > 0 else 0.0
    res = {"workload": args.workload, "precision": args.precision, "n_dofs": op.n_dofs, "steps": args.steps,
           "dt": dt, "t_end": t, "rel_l2_error": rel, "mass_energy": list(me), "s_per_step": per_step,
           "gdofs_per_stage": stage_rate}
    if u_start is not None:
        # return to the start of the time-periodic rotating flow
        # (advection_solver_variable.cc:1249-1252): small when t_end is a
        # multiple of the period and there is no diffusion
        ret = float((u - u_start).abs().max() / u_start.abs().max())
        res["return_to_start_max_rel"] = ret
        if not args.json:
            print(f"   Return to start: ||u(T) - u(0)||_inf / ||u(0)||_inf = {ret:.4e}")
    if args.compare_fp64 and precision != PRECISION_FP64:
        cfg.precision = PRECISION_FP64
        op64 = AdvectionOperation(cfg)
        u64, r64, k64 = (op64.initialize_dof_vector() for _ in range(3))
        op64.project_initial(u64)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        op64.lsrk_steps(integ.scheme, 0.0, dt, args.steps, u64, r64, k64)
        torch.cuda.synchronize()
        wall64 = time.perf_counter() - t0
        e64, n64 = op64.l2_error(u64, t)
        res["fp64"] = {"rel_l2_error": e64 / n64, "gdofs_per_stage": op.n_dofs * integ.n_stages() * args.steps
                       / wall64 / 1e9, "max_rel_difference": float((u - u64).abs().max() / u64.abs().max()),
                       "error_ratio_fp32_over_fp64": rel / (e64 / n64)}
    if args.json:
        print(json.dumps(res))
    else:
        print(f"\n   Performed {args.steps} time steps.")
        print(f"   Average wall clock time per time step: {per_step:.4g}s, time per element: "
              f"{per_step / op.n_cells:.4g}s")
        print(f"   Throughput: {stage_rate:.4g} GDoF/s per Runge-Kutta stage")


if __name__ == "__main__":
    main()
