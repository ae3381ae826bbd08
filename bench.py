"""Benchmark of the GB300 solve backend on the 3-D neo-Hooke cube (64^3 Q1 bricks).

Workload: 64^3 Q1 bricks (274,625 nodes, 823,875 DOFs), E = 1, nu = 0.3, x = 0 clamped,
u_x prescribed on x = 1.  One step = one load-step solve (load step 1 of 10, u_x = 0.03)
to a float64 Newton residual of 1e-10 times the first one, i.e. one ``solver.solver``
call, started from the linear lifting u_x = 0.03 x of the prescribed values (from u = 0 the
first element layer is stretched threefold at h = 1/64 and undamped Newton, the
reference's algorithm, diverges).  Metric: time to the 1e-10 relative residual (s, lower is
better) of the mixed-precision path (float32 tangent and Jacobi-PCG inside the float64
Newton/refinement loop); the plain float64 Jacobi-PCG path is timed beside it.  The
64^3 problem (~0.3 GB of float32 matrix, 0.6 GB float64) exceeds the 129 MB L2, so no
flush is needed between steps.

--impl reference times the CPU oracle (float64 NumPy/SciPy/torch.func restatement of the
reference path) on a bounded sample of the same workload and scales it to one load step.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")


def _peaks():
    try:
        with open(PEAKS) as fh:
            p = json.load(fh)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self):
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), f"agx_clocks_{os.getpid()}.csv")

    def __enter__(self):
        os.makedirs(os.path.dirname(self.path), exist_ok=True)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", "0"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        try:
            rows = [l.split(",") for l in open(self.path).read().strip().splitlines() if l.strip()]
            sm = [float(r[1]) for r in rows]
            mx = max(float(r[2]) for r in rows)
            names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
            reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if "Active" in v and "Not" not in v})
            return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": reasons, "samples": len(rows)}
        except Exception as e:  # noqa: BLE001
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "error": str(e)}


def _solve_once(w, static, newton_rtol, x0=None, profile_ctx=None):
    from autopdex_gb300 import solver
    st = dict(w.settings)
    st = w.steps[0](st)
    sol, info = solver.solver(w.dofs if x0 is None else x0, st, static, newton_tol=0.0, newton_rtol=newton_rtol,
                              maxiter=30)
    return sol, info


def gpu_arm(args):
    import torch
    import ctypes as C
    from autopdex_gb300 import configs, solver, _native as N
    from autopdex_gb300._problem import get_problem

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    n = args.size
    w = configs.neo_hooke_cube(n=n, n_steps=10)
    mixed = dict(w.static_settings, precision="mixed", solver="pcg")
    plain = dict(w.static_settings, precision="float64", solver="pcg")
    rtol = 1e-10
    kw = dict(krylov_tol=args.krylov_tol)

    # device-resident inputs: dofs and prescribed values already on the GPU
    st = w.steps[0](dict(w.settings))
    prob = get_problem(w.dofs, st, mixed)
    dev = prob.device
    x0_host = np.zeros((w.n_dofs // 3, 3))
    x0_host[:, 0] = w.raw["stretch"] / w.raw["n_steps"] * w.raw["coords"][:, 0]
    x0_host = x0_host.reshape(-1)
    g_dev = torch.as_tensor(np.asarray(st["dirichlet conditions"], dtype=np.float64).reshape(-1), device=dev)
    st_dev = dict(st)
    st_dev["dirichlet conditions"] = g_dev.reshape(-1, 3)
    x0_dev = torch.as_tensor(x0_host.reshape(-1, 3), device=dev)

    def run_dev(static, **over):
        k = dict(kw, **over)
        return solver.solver(x0_dev, st_dev, static, newton_tol=0.0, newton_rtol=rtol, maxiter=30, **k)

    for _ in range(args.warmup):
        run_dev(mixed)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    lib = N.load()
    l0 = C.c_int64()
    prob._call("agx_launch_count", C.byref(l0))
    prob._call("agx_profile", 1)
    stream = torch.cuda.current_stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    infos = []
    with Clocks() as clk:
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps):
            sol, info = run_dev(mixed)
            infos.append((info, solver.last_info.krylov_iterations))
        e1.record(stream)
        torch.cuda.synchronize()
    if dist:
        dist.barrier()
    t_ms = e0.elapsed_time(e1)
    ms = (C.c_double * N.AGX_PROF_CATEGORIES)()
    cnt = (C.c_int64 * N.AGX_PROF_CATEGORIES)()
    prob._call("agx_profile_read", ms, cnt)
    prob._call("agx_profile", 0)
    l1 = C.c_int64()
    prob._call("agx_launch_count", C.byref(l1))
    if dist:
        from autopdex_gb300 import replicas
        t_ms = replicas.max_over_ranks(t_ms, device=dev)
    per_step_s = t_ms / 1e3 / args.steps

    # verify the solution of the last timed step: float64 residual ratio
    res0 = solver.last_info.res0
    res_end = solver.last_info.res_norm

    # plain float64 Jacobi-PCG on the same step, beside the headline: (a) with the same inner
    # tolerance schedule as the mixed path, (b) with inner solves to 1e-11 (direct-solve accuracy)
    def timed(static, **over):
        run_dev(static, **over)
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        _, inf = run_dev(static, **over)
        b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / 1e3, inf, solver.last_info.krylov_iterations
    if args.only_mixed:
        plain_s, info_p, plain_kry = float("nan"), (0, 0.0, False), 0
        tight_s, info_t, tight_kry = float("nan"), (0, 0.0, False), 0
    else:
        plain_s, info_p, plain_kry = timed(plain)
        tight_s, info_t, tight_kry = timed(plain, krylov_tol=1e-11)

    # end to end through the public API with host buffers (H2D of the inputs, D2H of the result)
    def run_host():
        s = dict(st)
        return solver.solver(x0_host.reshape(-1, 3), s, mixed, newton_tol=0.0, newton_rtol=rtol, maxiter=30, **kw)
    if not args.only_mixed:
        run_host()
    torch.cuda.synchronize()
    k_e2e = 0 if args.only_mixed else max(1, min(args.steps, 3))
    t0 = time.perf_counter()
    for _ in range(k_e2e):
        out_host, _ = run_host()
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t0) / max(1, k_e2e)

    # roofline of the dominant kernel (largest category)
    cats = {"tangent_assembly": N.AGX_PROF_TANGENT, "residual_assembly": N.AGX_PROF_RESIDUAL,
            "spmv": N.AGX_PROF_SPMV, "krylov_vector": N.AGX_PROF_VECTOR}
    shares = {k: ms[v] for k, v in cats.items()}
    launches = {k: int(cnt[v]) for k, v in cats.items()}
    b = 3
    nnzb = prob.nnzb
    n_nodes = w.n_dofs // 3
    # fused product: matrix planes + columns + rowptr; reads z and p_old, writes p_new and q
    spmv_bytes = nnzb * (b * b * 4 + 4) + (n_nodes + 1) * 4 + 4 * w.n_dofs * 4
    spmv_avg_ms = ms[N.AGX_PROF_SPMV] / max(1, cnt[N.AGX_PROF_SPMV])
    peak, peak_kind = _peaks()
    achieved = spmv_bytes / (spmv_avg_ms * 1e-3) / 1e9
    traffic = None
    tr_path = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tr_path):
        try:
            traffic = json.load(open(tr_path)).get("spmv_f32_bsr3_64cube_bytes_per_launch")
        except Exception:
            traffic = None
    # element tangent pass: algorithmic bytes (coords, dofs, conn, scatter map, float32 values)
    n_e = n ** 3
    asm_bytes = n_nodes * 3 * 8 + w.n_dofs * 8 + n_e * 8 * 4 + n_e * 64 * 4 + nnzb * 9 * 4
    asm_avg_ms = ms[N.AGX_PROF_TANGENT] / max(1, cnt[N.AGX_PROF_TANGENT])
    # The 3-D neo-Hooke tangent is bound by arithmetic, not bytes: an analytic count of the
    # float32 kernel's flops, per lane (8 per element) and Gauss point (8): Jacobian by group
    # sums, its inverse and the gradients ~100, shape functions ~15, F, F^-1 and F^-T g ~110,
    # the 8 rows of 3 x 3 tangent entries ~83 each -> ~890; against the measured FP32 rate.
    asm_flops = n_e * 8 * 8 * (100 + 15 + 110 + 8 * 83)
    fp32_peak_tflops = 69.8  # FMA-chain probe on this GPU (2 flops per FMA)

    line = {
        "metric": "time_to_1e-10_relative_fp64_residual (64^3 neo-Hooke cube, load step 1 of 10)",
        "value": per_step_s,
        "unit": "s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": per_step_s * 1e3,
        "higher_is_better": False,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 tangent/SpMV + f64 residual",
        "data": "synthetic (structured meshes of the workloads; no dataset)",
        "config": {"workload": f"neo_hooke_cube_{n}^3_hex8_load_step_1", "n_dofs": w.n_dofs, "nnz": nnzb * 9,
                   "newton_rtol": rtol, "krylov": "jacobi-pcg f32 (rtol %.0e)" % args.krylov_tol,
                   "l2": "working set > 129 MB L2 (no flush needed)", "parallelism": "replicas" if world > 1 else "1 gpu",
                   "krylov_chunks": "CUDA graphs of 32 iterations", "spmv_lanes_per_row": "autotuned"},
        "plain_fp64_pcg_s": plain_s,
        "speedup_mixed_vs_plain_fp64": plain_s / per_step_s,
        "plain_fp64_pcg_tight_s": tight_s,
        "newton_iterations": int(infos[-1][0][0]),
        "newton_iterations_plain_fp64": int(info_p[0]),
        "newton_iterations_plain_fp64_tight": int(info_t[0]),
        "krylov_iterations_mixed": int(infos[-1][1]),
        "krylov_iterations_plain_fp64": int(plain_kry),
        "krylov_iterations_plain_fp64_tight": int(tight_kry),
        "converged": bool(not infos[-1][0][2]) and (res_end <= rtol * res0 * 1.0000001),
        "final_residual_ratio": res_end / res0 if res0 else None,
        "kernel_ms_per_step": {k: v / args.steps for k, v in shares.items()},
        "kernel_launches_per_step": {k: v / args.steps for k, v in launches.items()},
        "roofline": {"bound": "hbm", "kernel": f"spmv_dot_kernel<float,3,{getattr(prob, 'spmv_tpr', 8)}> "
                                                "(BSR 3x3 SpMV, direction update, dot)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind, "traffic": traffic, "algorithmic_bytes": spmv_bytes,
                     "avg_launch_ms": spmv_avg_ms},
        "assembly": {"kernel": "element_kernel<HEX8,NEO_HOOKE,float> (tangent pass)",
                     "algorithmic_bytes": asm_bytes, "avg_launch_ms": asm_avg_ms,
                     "achieved_gbs": asm_bytes / (asm_avg_ms * 1e-3) / 1e9 if asm_avg_ms else None,
                     "flops_estimate": asm_flops,
                     "achieved_tflops": asm_flops / (asm_avg_ms * 1e-3) / 1e12 if asm_avg_ms else None,
                     "fp32_peak_tflops": fp32_peak_tflops,
                     "frac_fp32_peak": asm_flops / (asm_avg_ms * 1e-3) / 1e12 / fp32_peak_tflops if asm_avg_ms else None},
        "e2e": {"value": e2e_s, "unit": "s", "h2d_bytes_per_step": 2 * w.n_dofs * 8,
                "d2h_bytes_per_step": w.n_dofs * 8},
        "gpu_launches": int(l1.value - l0.value),
        "clocks": clk.summary(),
    }
    if rank == 0 and not args.only_mixed:
        try:
            line["assembly_hbm"] = assembly_roofline()
            line["assembly_hbm_2048"] = assembly_roofline(n=2048)  # values (151 MB) larger than L2
        except Exception as e:  # noqa: BLE001 -- reported, the headline stands
            line["assembly_hbm"] = {"error": str(e)[:200]}
    if rank == 0 and not args.only_mixed and not args.no_learned:
        try:
            line["heat_learned"] = heat_learned(n=args.learned_n)
        except Exception as e:  # noqa: BLE001 -- reported, the headline stands
            line["heat_learned"] = {"error": str(e)[:200]}
    if rank == 0 and args.more_workloads:
        try:
            line["other_workloads"] = other_workloads()
        except Exception as e:  # noqa: BLE001 -- reported, the headline stands
            line["other_workloads"] = {"error": str(e)[:300]}
    if rank == 0 and not args.no_cpu_baseline and not args.only_mixed:
        try:
            line["cpu_baseline"] = cpu_baseline(n, int(info_t[0]), int(tight_kry), budget_s=args.cpu_budget)
        except Exception as e:  # noqa: BLE001 -- reported, the headline stands
            line["cpu_baseline"] = {"error": str(e)[:300]}
    if dist:
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(line))


TRAIN_N = 256  # resolution the shipped network was trained on (heat_unet_n256.npz)


def heat_learned(n=1024, seed=10000, rtol=1e-10):
    """Heat conduction with k = exp(GRF) on n x n Q1 quads: time to a 1e-10 relative float64 residual for
    plain float64 Jacobi-PCG, mixed Jacobi-PCG and the learned preconditioner in mixed FCG."""
    import torch
    from autopdex_gb300 import configs, learned, solver
    path = os.path.join(learned.WEIGHTS_DIR, "heat_unet_n256.npz")
    if not os.path.exists(path):
        return {"skipped": "no trained weights"}
    net = learned.UNet.load(path)
    out = {"workload": f"heat_grf_{n}x{n}_q1 (seed {seed})", "weights": os.path.basename(path),
           "network_grid": f"{n // max(1, n // TRAIN_N) + 1}^2 nodes (coarsening {max(1, n // TRAIN_N)})"}
    variants = [("plain_fp64_pcg", dict(precision="float64", solver="pcg"), dict(krylov_tol=1e-11)),
                ("mixed_pcg", dict(precision="mixed", solver="pcg"), dict(krylov_tol=1e-5)),
                ("learned_mixed_fcg", dict(precision="mixed", solver="fcg", **{"type of preconditioner": "learned"}),
                 dict(krylov_tol=1e-4))]
    factor = max(1, n // TRAIN_N)
    for name, st, kw in variants:
        w = configs.heat_grf(n=n, seed=seed)
        static = dict(w.static_settings, **st)
        if name.startswith("learned"):
            solver.set_learned_preconditioner(None, learned.GridPreconditioner(net, n, n, w.settings["conductivity"],
                                                                                  factor=factor))
        solver.solver(w.dofs, w.settings, static, newton_tol=0.0, newton_rtol=rtol, maxiter=30,
                      krylov_maxiter=400000, **kw)  # warm-up (context, graphs)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sol, info = solver.solver(w.dofs, w.settings, static, newton_tol=0.0, newton_rtol=rtol, maxiter=30,
                                  krylov_maxiter=400000, **kw)
        torch.cuda.synchronize()
        li = solver.last_info
        out[name] = {"s": time.perf_counter() - t0, "newton": int(info[0]), "krylov": int(li.krylov_iterations),
                     "residual_ratio": li.res_norm / li.res0 if li.res0 else None, "diverged": bool(info[2])}
    out["speedup_learned_vs_plain_fp64"] = out["plain_fp64_pcg"]["s"] / out["learned_mixed_fcg"]["s"]
    return out


def assembly_roofline(n=1024, reps=20):
    """Float32 tangent assembly of the 1024^2 random-conductivity heat mesh (an HBM-bound
    assembly: a scalar potential on Q1 quads), timed with CUDA events per agx_assemble call.

    Algorithmic bytes: coordinates + DOFs + connectivity +
    values written once (n_nodes dim 8 + n_dofs 8 + n_e nen 4 + nnz 4); the row kernel of
    structured grids moves coordinates, conductivities, row pointers and values."""
    import ctypes as C
    import torch
    from autopdex_gb300 import configs, _native as N
    from autopdex_gb300._problem import get_problem
    w = configs.heat_grf(n=n, seed=0)
    prob = get_problem(w.dofs, w.settings, w.static_settings)
    prob.update_models(w.settings)
    x = torch.zeros(prob.n_dofs, dtype=torch.float64, device=prob.device)
    for _ in range(3):
        prob._call("agx_assemble", C.c_void_p(x.data_ptr()), None, N.AGX_F32)
    # The mesh's arrays and values (about 60 MB) fit in the 129 MB L2: every timed call
    # follows a write of a 256 MB buffer, so that its inputs come from HBM.
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=prob.device)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
    for a, b in ev:  # per call, the library's own timing off
        flush.fill_(1)
        a.record()
        prob._call("agx_assemble", C.c_void_p(x.data_ptr()), None, N.AGX_F32)
        b.record()
    torch.cuda.synchronize()
    call_ms = sum(a.elapsed_time(b) for a, b in ev)
    prob._call("agx_profile", 1)
    for _ in range(reps):  # per kernel: the library's events around each row-kernel launch
        flush.fill_(1)
        prob._call("agx_assemble", C.c_void_p(x.data_ptr()), None, N.AGX_F32)
    torch.cuda.synchronize()
    ms = (C.c_double * N.AGX_PROF_CATEGORIES)()
    cnt = (C.c_int64 * N.AGX_PROF_CATEGORIES)()
    prob._call("agx_profile_read", ms, cnt)
    prob._call("agx_profile", 0)
    del flush
    n_e = n * n
    nbytes = prob.n_nodes * 2 * 8 + prob.n_dofs * 8 + n_e * 4 * 4 + prob.nnzb * 4
    call_s = call_ms / 1e3 / reps
    kern_s = ms[N.AGX_PROF_TANGENT] / 1e3 / max(1, cnt[N.AGX_PROF_TANGENT])
    peak, kind = _peaks()
    return {"workload": f"heat_grf_{n}x{n}_q1 float32 tangent", "kernel": "grid_tangent_kernel<HEAT_POTENTIAL,float>",
            "algorithmic_bytes": nbytes, "call_us": call_s * 1e6, "kernel_us": kern_s * 1e6,
            "achieved_gbs_call": nbytes / call_s / 1e9, "achieved_gbs_kernel": nbytes / kern_s / 1e9,
            "peak_gbs": peak, "frac_call": nbytes / call_s / 1e9 / peak, "frac_kernel": nbytes / kern_s / 1e9 / peak,
            "peak_source": kind, "l2": "256 MB buffer written before every timed call"}


def _timed_solve(w, static, step=None, x0=None, rtol=1e-10, **kw):
    """One solver.solver call (warm context: a first call builds it), CUDA-synchronised wall
    time, with the Newton and Krylov counts and the final float64 residual ratio."""
    import torch
    from autopdex_gb300 import solver
    st = dict(w.settings)
    if step is not None:
        st = step(st)
    dofs = w.dofs if x0 is None else x0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sol, info = solver.solver(dofs, st, static, newton_tol=0.0, newton_rtol=rtol, maxiter=30, **kw)
    torch.cuda.synchronize()
    li = solver.last_info
    return sol, {"s": time.perf_counter() - t0, "newton": int(info[0]), "krylov": int(li.krylov_iterations),
                 "residual_ratio": li.res_norm / li.res0 if li.res0 else None, "diverged": bool(info[2])}


def other_workloads(cook_n=128, cook_rtol=1e-6, heat3d_n=128, heat3d_steps=2):
    """The 200^2 Poisson, Cook membrane and 3-D backward-Euler heat workloads beside the headline:
    plain float64 against mixed precision where the
    method allows it (BiCGStab, for the non-symmetric backward-Euler tangent, runs in float64).

    Cook's membrane (nu = 0.4999) is run at cook_n^2 to a relative Newton residual of cook_rtol:
    with Jacobi-PCG the float64 Newton residual of this nearly incompressible problem stalls
    near 4.5e-7 of the first one already at 128^2 (measured: 31 Newton iterations and 1.8 M CG
    iterations without getting below it), so 1e-10 is out of reach for the plain method."""
    from autopdex_gb300 import configs
    out = {}
    # 200^2 Poisson, one Newton step with the direct-solver name ('lapack')
    w = configs.poisson(n=200, solver="lapack")
    _timed_solve(w, w.static_settings)
    _, out["poisson_200_fp64_direct"] = _timed_solve(w, w.static_settings)
    # Cook membrane, load step 1 of 20
    res = {}
    for name, prec, ktol in (("plain_fp64_pcg", "float64", 1e-8), ("mixed_pcg", "mixed", 1e-5)):
        w = configs.cook_membrane(n=cook_n, precision=prec)
        _timed_solve(w, w.static_settings, step=w.steps[0], rtol=cook_rtol, krylov_tol=ktol, krylov_maxiter=400000)
        _, res[name] = _timed_solve(w, w.static_settings, step=w.steps[0], rtol=cook_rtol, krylov_tol=ktol,
                                    krylov_maxiter=400000)
    res["speedup_mixed_vs_plain_fp64"] = res["plain_fp64_pcg"]["s"] / res["mixed_pcg"]["s"]
    out[f"cook_{cook_n}_load_step_1_rtol_{cook_rtol:g}"] = res
    # 3-D nonlinear backward-Euler heat, the first time steps: float64 BiCGStab (the tangent has
    # a small non-symmetric k'(T) part) against mixed Jacobi-PCG (float32 CG on the
    # mass-dominated tangent inside the float64 Newton loop, which the float64 residual judges)
    import numpy as np
    res = {}
    for name, sol_name, prec, ktol in (("plain_fp64_bicgstab", "bicgstab", "float64", 1e-11),
                                       ("mixed_pcg", "pcg", "mixed", 1e-5)):
        w = configs.heat_transient(n=heat3d_n, solver=sol_name, precision=prec)
        T = np.asarray(w.raw["T0"], dtype=np.float64)
        steps = []
        for k in range(heat3d_steps + 1):
            w.settings["dofs n"] = {"T": T.copy()}
            sol, r = _timed_solve(w, w.static_settings, x0={"T": T.copy()}, krylov_tol=ktol)
            T = np.asarray(sol["T"])
            if k:
                steps.append(r)  # the first call builds the context and is not counted
        res[name] = {"s_per_step": sum(r["s"] for r in steps) / len(steps), "per_step": steps,
                     "sum_T_squared": float(np.sum(T * T))}
    res["speedup_mixed_vs_plain_fp64"] = res["plain_fp64_bicgstab"]["s_per_step"] / res["mixed_pcg"]["s_per_step"]
    out[f"heat_be_{heat3d_n}^3_steps_1_to_{heat3d_steps}"] = res
    return out


def cpu_baseline(n, newton_iters, cg_iters, budget_s=20.0):
    """CPU oracle on a bounded sample of the workload, scaled to one load step.

    The oracle's C restatement (oracle/c/orc.c: closed-form float64 neo-Hooke brick and
    Jacobi-PCG on CSR, OpenMP over all host cores) on the 32^3 cube: (a) residual and tangent
    cost per element; (b) COO -> CSR with Dirichlet rows and columns deleted, as
    scipy_assembling does (solver.py:1180-1222, SciPy, single-threaded as there), per stored
    entry; (c) Jacobi-PCG cost per iteration per stored entry -- the reference's 'cg' +
    'jacobi' algorithm on the assembled matrix.  Scaled with the Newton and CG iteration
    counts of the float64 GPU path on the full problem:
    t = newton_iters (2 n_e t_res + n_e t_tan + nnz t_csr) + cg_iters nnz t_iter."""
    import scipy.sparse as sps
    from autopdex_gb300 import configs
    from oracle import corc

    threads = corc.threads()
    ns = 32
    w = configs.neo_hooke_cube(n=ns, n_steps=10)
    coords, conn = w.raw["coords"], w.raw["conns"][0]
    n_e = conn.shape[0]
    u = np.random.default_rng(0).uniform(-1e-3, 1e-3, coords.shape)
    corc.neo_hooke_hex8(conn[:256], coords, u, w.raw["E"], w.raw["nu"])  # threads up, library loaded
    t0 = time.perf_counter()
    corc.neo_hooke_hex8(conn, coords, u, w.raw["E"], w.raw["nu"], tangent=False)
    t_res = (time.perf_counter() - t0) / n_e
    t0 = time.perf_counter()
    _, K_e = corc.neo_hooke_hex8(conn, coords, u, w.raw["E"], w.raw["nu"])
    t_tan = (time.perf_counter() - t0) / n_e
    edofs = (conn[:, :, None] * 3 + np.arange(3)).reshape(n_e, 24)
    free = ~np.asarray(w.raw["dirichlet"], dtype=bool)
    t0 = time.perf_counter()
    A = sps.coo_matrix((K_e.ravel(), (np.repeat(edofs, 24, axis=1).ravel(), np.tile(edofs, (1, 24)).ravel())),
                       shape=(free.size, free.size)).tocsr()
    A = A[free][:, free].tocsr()
    t_csr = (time.perf_counter() - t0) / A.nnz
    del K_e
    b = np.random.default_rng(1).standard_normal(A.shape[0])
    corc.pcg_csr(A, b, 3)
    iters = 100
    t0 = time.perf_counter()
    corc.pcg_csr(A, b, iters)
    t_iter = (time.perf_counter() - t0) / iters / A.nnz
    nnz = 243 * (n + 1) ** 3  # stored entries of the full problem: 27 node blocks of 3 x 3 per node (upper bound)
    n_e_full = n ** 3
    est = newton_iters * (2 * n_e_full * t_res + n_e_full * t_tan + nnz * t_csr) + cg_iters * nnz * t_iter
    return {"value": est, "unit": "s", "cores": threads, "kind": "port",
            "sample": (f"oracle C restatement on the {ns}^3 cube ({threads} threads): residual {t_res * 1e6:.2f} and "
                       f"tangent {t_tan * 1e6:.2f} us per element, COO->CSR with Dirichlet deletion (SciPy) "
                       f"{t_csr * 1e9:.1f} ns and Jacobi-PCG {t_iter * 1e9:.2f} ns per stored entry and iteration; "
                       f"scaled to {n}^3 with the float64 GPU path's {newton_iters} Newton and {cg_iters} CG "
                       f"iterations")}


def reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    n = args.size
    # iteration counts of the float64 path on the 64^3 load step, measured on the GPU arm
    newton_iters, cg_iters = args.ref_newton_iters, args.ref_cg_iters
    vals = []
    for _ in range(args.warmup):
        cpu_baseline(n, newton_iters, cg_iters)
    t0 = time.perf_counter()
    last = None
    for _ in range(args.steps):
        last = cpu_baseline(n, newton_iters, cg_iters)
        vals.append(last["value"])
    wall = time.perf_counter() - t0
    v = float(np.median(vals))
    line = {"impl": "reference",
            "metric": "time_to_1e-10_relative_fp64_residual (64^3 neo-Hooke cube, load step 1 of 10)",
            "value": v, "unit": "s", "n_gpus": int(os.environ.get("WORLD_SIZE", "1")), "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": wall / args.steps * 1e3, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"neo_hooke_cube_{n}^3_hex8_load_step_1"},
            "cpu_baseline": {"value": v, "unit": "s", "cores": last["cores"], "kind": last["kind"],
                             "sample": last["sample"]},
            "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--size", type=int, default=64)
    ap.add_argument("--krylov-tol", type=float, default=1e-4)
    ap.add_argument("--cpu-budget", type=float, default=20.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--only-mixed", action="store_true", help="time the mixed path only (profiling runs)")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-preconditioner heat section")
    ap.add_argument("--learned-n", type=int, default=1024)
    ap.add_argument("--more-workloads", action="store_true", help="also time the Poisson, Cook and 3-D transient heat workloads")
    ap.add_argument("--ref-newton-iters", type=int, default=4)
    ap.add_argument("--ref-cg-iters", type=int, default=3000)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "gb300" else args.warmup
    if args.impl == "reference":
        reference_arm(args)
    else:
        gpu_arm(args)


if __name__ == "__main__":
    main()
