"""Benchmark of the GB300 solve backend on the workloads of AutoPDEx's Newton solve path.

Headline (``value``): time to a 1e-10 relative float64 residual of the learned + mixed-precision
solve of the 1024^2 random-conductivity heat problem -- flexible CG in float32 with the U-Net
two-level preconditioner inside the float64 Newton / refinement loop -- through
``solver.solver`` with device-resident inputs; the plain float64 Jacobi-PCG solve of the same
problem is timed beside it (the metric compares the two).  One step = one solve from zero.
The problem's matrix and vectors exceed the 129 MB L2 only in part (88 MB of float32 values),
so a 256 MB buffer is written before every timed step.

``e2e``: the same solve through solver.solver with host NumPy inputs and outputs (the host to
device copies of the DOFs and prescribed values and the device to host copy of the solution
inside the timed region).

Sub-records (``configs``), each with its error against the float64 oracle:
  poisson_200       200^2 Q1 Poisson, one Newton step with the direct (banded Cholesky) solve
  neo_hooke_64cube  64^3 neo-Hooke cube, all 10 load steps, mixed precision and plain float64
  cook_512          512^2 Cook membrane (nu = 0.4999), load steps of the 20, float64 direct and
                    plain float64 Jacobi-PCG
  heat_1024         the headline problem: plain float64, mixed and learned + mixed
  heat_be_128cube   128^3 backward-Euler heat, time steps with mixed Jacobi-PCG and float64
                    BiCGStab
``roofline``: the dominant kernel of the headline solve (per-category CUDA-event times from a
separate profiled pass; the timed region runs with CUDA graphs and no instrumentation).
``assembly_hbm``: the float32 tangent assembly of the 1024^2 and 2048^2 heat meshes.
``cpu_baseline``: the oracle's C restatement (C elements, SciPy COO -> CSR with Dirichlet
deletion as scipy_assembling does, OpenMP Jacobi-PCG to the same 1e-10) on the full 1024^2
problem, timed on the host's cores.

``--impl reference`` times that CPU path (the reference itself is JAX code and no JAX exists
offline) on the headline's workload, one full solve per step.
``--case conv|assembly|solve`` runs one small case for ncu captures (no JSON line).
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
RTOL = 1e-10
TRAIN_N = 256  # resolution the shipped heat network was trained on (heat_unet_n256.npz)

# DRAM traffic per launch of the dominant kernels (dram__bytes_read.sum + dram__bytes_write.sum,
# one ncu capture each; the commands are in the named profile summaries)
NCU_TRAFFIC = {}


def _peaks():
    try:
        with open(PEAKS) as fh:
            p = json.load(fh)
        return float(p["hbm_gbs"]), float(p.get("bf16_tflops", 1941.6)), "measured"
    except Exception:
        return 6800.0, 1900.0, "fallback"


class Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self):
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), f"agx_clocks_{os.getpid()}.csv")

    def __enter__(self):
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


# ---- helpers -------------------------------------------------------------------------------
def _sync():
    import torch
    torch.cuda.synchronize()


def _events():
    import torch
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def _flat(d):
    a = next(iter(d.values())) if isinstance(d, dict) else d
    if hasattr(a, "detach"):
        a = a.detach().cpu().numpy()
    return np.asarray(a, dtype=np.float64).reshape(-1)


def _info():
    from autopdex_gb300 import solver
    li = solver.last_info
    return {"newton": int(li.iterations), "krylov": int(li.krylov_iterations), "res0": float(li.res0),
            "res": float(li.res_norm), "residual_ratio": (li.res_norm / li.res0) if li.res0 else 0.0,
            "diverged": bool(li.diverged)}


def _timed(fn):
    """CUDA-event time (s) of fn() on torch's current stream (the library's stream)."""
    a, b = _events()
    _sync()
    a.record()
    out = fn()
    b.record()
    _sync()
    return a.elapsed_time(b) / 1e3, out


def _profile(prob, fn):
    """Per-category kernel times (ms) and launch counts of fn() with the library's events on
    (CUDA graphs are not used while profiling)."""
    import ctypes as C
    from autopdex_gb300 import _native as N
    prob._call("agx_profile", 1)
    try:
        fn()
        _sync()
        ms = (C.c_double * N.AGX_PROF_CATEGORIES)()
        cnt = (C.c_int64 * N.AGX_PROF_CATEGORIES)()
        prob._call("agx_profile_read", ms, cnt)
    finally:
        prob._call("agx_profile", 0)
    names = {N.AGX_PROF_TANGENT: "tangent_assembly", N.AGX_PROF_RESIDUAL: "residual_assembly",
             N.AGX_PROF_SPMV: "krylov_product", N.AGX_PROF_VECTOR: "krylov_vector",
             N.AGX_PROF_PRECOND: "network", N.AGX_PROF_FACTOR: "factorization", N.AGX_PROF_SMOOTH: "smoothing_product"}
    return {v: float(ms[k]) for k, v in names.items()}, {v: int(cnt[k]) for k, v in names.items()}


def _launches(prob):
    import ctypes as C
    v = C.c_int64()
    prob._call("agx_launch_count", C.byref(v))
    return int(v.value)


def _flush_buffer():
    import torch
    return torch.empty(256 << 20, dtype=torch.uint8, device="cuda")


# ---- the headline: 1024^2 heat, learned + mixed against plain float64 -------------------------
def _heat_variants():
    return [("plain_fp64_pcg", dict(precision="float64", solver="pcg"), dict(krylov_tol=1e-11)),
            ("mixed_pcg", dict(precision="mixed", solver="pcg"), dict(krylov_tol=1e-5)),
            ("learned_mixed_fcg", dict(precision="mixed", solver="fcg", **{"type of preconditioner": "learned"}),
             dict(krylov_tol=1e-3))]


BF16_SMOOTHING = False  # --bf16-smoothing: the two-level products on a bf16 copy of the values


def _heat_learned_setup(w, n):
    from autopdex_gb300 import learned, solver
    net = learned.UNet.load(os.path.join(learned.WEIGHTS_DIR, "heat_unet_n256.npz"))
    factor = max(1, n // TRAIN_N)
    pc = learned.GridPreconditioner(net, n, n, w.settings["conductivity"], factor=factor,
                                    bf16_smoothing=BF16_SMOOTHING)
    solver.set_learned_preconditioner(None, pc)
    return net, pc, factor


def headline(args, rank):
    import torch
    from autopdex_gb300 import configs, learned, solver
    from autopdex_gb300._problem import get_problem
    n = args.size
    w = configs.heat_grf(n=n, seed=10000)
    net, pc, factor = _heat_learned_setup(w, n)
    name, st, kw = _heat_variants()[2]
    static = dict(w.static_settings, **st)
    kw = dict(kw, newton_tol=0.0, newton_rtol=RTOL, maxiter=30, krylov_maxiter=400000)
    dev = torch.device("cuda", torch.cuda.current_device())
    x0 = torch.zeros(w.n_dofs, dtype=torch.float64, device=dev)
    st_dev = dict(w.settings)
    st_dev["dirichlet conditions"] = {"T": torch.zeros(w.n_dofs, dtype=torch.float64, device=dev)}
    dofs_dev = {"T": x0}

    def run():
        return solver.solver(dofs_dev, st_dev, static, **kw)
    for _ in range(args.warmup):
        run()
    prob = get_problem(dofs_dev, st_dev, static)
    flush = _flush_buffer()
    _sync()
    if args.dist:
        args.dist.barrier()
    l0 = _launches(prob) + net.launches
    stream = torch.cuda.current_stream()
    ev = [_events() for _ in range(args.steps)]
    infos = []
    with Clocks() as clk:
        _sync()
        for a, b in ev:
            flush.fill_(1)  # inputs from HBM: the 256 MB write evicts the problem from L2
            a.record(stream)
            sol, info = run()
            b.record(stream)
            infos.append(_info())
        _sync()
    l1 = _launches(prob) + net.launches  # the library's kernels and the network's (conv, pool, transfers)
    if args.dist:
        args.dist.barrier()
    t_ms = sum(a.elapsed_time(b) for a, b in ev)
    if args.dist:
        from autopdex_gb300 import replicas
        t_ms = replicas.max_over_ranks(t_ms, device=dev)
    per_step = t_ms / 1e3 / args.steps
    out = {"s": per_step, "info": infos[-1], "launches_per_step": (l1 - l0) / args.steps, "clocks": clk.summary(),
           "prob": prob, "solution": sol, "w": w, "net": net, "factor": factor, "static": static, "kw": kw,
           "conv_variants": {k: (v[0] if k != "us_per_pass" else [round(t, 1) for t in v])
                             for k, v in pc.loaders.items()},
           "run": run}
    # the comparison of the metric: plain float64 Jacobi-PCG (and mixed Jacobi-PCG) on the same problem
    cmp = {}
    for vname, vst, vkw in _heat_variants()[:2]:
        vstatic = dict(w.static_settings, **vst)
        vkw = dict(vkw, newton_tol=0.0, newton_rtol=RTOL, maxiter=30, krylov_maxiter=400000)
        solver.solver(w.dofs, w.settings, vstatic, **vkw)
        flush.fill_(1)
        s, _ = _timed(lambda: solver.solver(w.dofs, w.settings, vstatic, **vkw))
        cmp[vname] = dict(s=s, **_info())
    cmp["learned_mixed_fcg"] = dict(s=per_step, **infos[-1])
    cmp["speedup_learned_mixed_vs_plain_fp64"] = cmp["plain_fp64_pcg"]["s"] / per_step
    out["comparison"] = cmp
    del flush
    return out


def headline_e2e(h, steps):
    """The headline solve through solver.solver with host arrays: H2D of the DOFs and the
    prescribed values, D2H of the solution, inside the timed region."""
    from autopdex_gb300 import solver
    w = h["w"]
    static, kw = h["static"], h["kw"]
    dofs = {"T": np.zeros(w.n_dofs)}
    solver.solver(dofs, w.settings, static, **kw)
    t0 = time.perf_counter()
    k = max(1, min(steps, 3))
    for _ in range(k):
        sol, _ = solver.solver(dofs, w.settings, static, **kw)
        assert isinstance(sol["T"], np.ndarray)
    _sync()
    s = (time.perf_counter() - t0) / k
    return {"value": s, "unit": "s", "h2d_bytes_per_step": 2 * w.n_dofs * 8, "d2h_bytes_per_step": w.n_dofs * 8}


def _network_flops(hp, wp):
    """Tensor-core FLOPs of one U-Net forward pass on an hp x wp padded grid."""
    from autopdex_gb300 import learned
    level = {"e0": 0, "e1": 1, "e2": 2, "b3": 3, "d2": 2, "d1": 1, "d0": 0, "ou": 0}
    tot = 0
    for name, c1, c2, co, relu in learned.LAYERS:
        lv = level[name[:2]]
        h, w_ = hp // learned.POOL ** lv, wp // learned.POOL ** lv
        tot += 2 * 9 * (c1 + c2) * co * h * w_
    return tot


def network_application_ms(pc, n_dofs, reps=30):
    """GPU time of one application of the learned preconditioner's network (restriction, U-Net,
    prolongation), captured in a CUDA graph and replayed the way FCG's graphs run it, timed with
    CUDA events on the replay stream.  (The profiled pass launches the callback from Python, so
    its per-application time is mostly host launch overhead.)"""
    import torch
    dev = pc.net.device
    r = torch.randn(n_dofs, dtype=torch.float32, device=dev)
    z = torch.empty_like(r)
    # outside a solve: the network must not skip on the last solve's converged flag
    skip, pc.skip_flag = pc.skip_flag, None
    try:
        return _network_application_ms(pc, r, z, n_dofs, reps)
    finally:
        pc.skip_flag = skip


def _network_application_ms(pc, r, z, n_dofs, reps):
    import torch
    dev = pc.net.device
    s = torch.cuda.Stream(device=dev)
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        rc = pc.apply_ptr(r.data_ptr(), z.data_ptr(), n_dofs, s.cuda_stream)
        assert rc == 0, rc
    s.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        pc.apply_ptr(r.data_ptr(), z.data_ptr(), n_dofs, s.cuda_stream)
    a, b = _events()
    with torch.cuda.stream(s):
        g.replay()
        a.record(s)
        for _ in range(reps):
            g.replay()
        b.record(s)
    s.synchronize()
    pc.net.check()
    return a.elapsed_time(b) / reps


def headline_roofline(h):
    """Per-category shares of the headline solve and the roofline of its dominant kernel.

    Kernel times per category come from the library's CUDA events in a profiled pass (graphs
    off); the network's per-application time from graph replays (network_application_ms), since
    the profiled pass launches it from Python.  The dominant kernel is the category with the
    largest GPU time per solve."""
    from autopdex_gb300 import learned
    prob = h["prob"]
    ms, cnt = _profile(prob, h["run"])
    net_app_ms = network_application_ms(prob.learned, prob.n_dofs) if prob.learned is not None else 0.0
    ms["network_profiled_with_host_launches"] = ms["network"]
    ms["network"] = net_app_ms * cnt["network"]
    tot = sum(v for k, v in ms.items() if k != "network_profiled_with_host_launches")
    shares = {k: (v / tot if tot else 0.0) for k, v in ms.items() if k != "network_profiled_with_host_launches"}
    hbm, bf16, kind = _peaks()
    n_nodes, n, ndof = prob.n_nodes, prob.n_dofs, prob.ndof
    nnzb = prob.nnzb
    s = 4  # float32 products
    # algorithmic bytes per launch: values and columns of every stored block, row pointers, and
    # the vectors (fused Krylov product: z, p_old read, p_new, q written; plain product: x, y);
    # the structured grid's product (code 512) reads no row pointers or column indices
    tpr = getattr(prob, "spmv_tpr", 0)
    grid = tpr in (512, 1024, 2048)
    matrix = nnzb * ndof * ndof * s if grid else nnzb * (ndof * ndof * s + 4) + 4 * (n_nodes + 1)
    fused = matrix + 4 * n * s
    # the two-level products carry their element-wise work: per application 2 (nu - 1) sweep
    # products (x gathered; rc, z read and written; D^-1 read; the new increment written: 7
    # vectors), one residual product (x; rc read and written: 3) and one step product (y, rc
    # read, K y written: 3); nu = 3 smoothing steps on either side
    nu = 3
    plain = matrix + n * s * (2 * (nu - 1) * 7 + 3 + 3) / (2 * (nu - 1) + 2)
    hc = h["w"].raw["n"] // h["factor"] + 1
    flops = _network_flops(learned.padded(hc), learned.padded(hc))
    var = ("grid, 2 rows per lane" if tpr == 1024 else "grid") if grid else f"bsr, {tpr} lanes per row"
    cand = {"smoothing_product": ("hbm", plain, f"tl_spmv<1,{var}> (two-level smoothing, residual and step products "
                                                "with their element-wise work fused)"),
            "krylov_product": ("hbm", fused, f"spmv_dot_kernel<float,1,{var}> (FCG product with direction update "
                                             "and dot)"),
            "network": ("tensor", flops, "U-Net forward: 15 conv3x3_tc (tcgen05, BF16), pooling, upsampling and "
                                         "grid transfers, replayed from a CUDA graph")}
    dom = max(cand, key=lambda k: ms.get(k, 0.0))

    def entry(k):
        b_, wk, kn = cand[k]
        a_ms = ms[k] / max(1, cnt[k])
        if b_ == "hbm":
            ach = wk / (a_ms * 1e-3) / 1e9
            return {"bound": "hbm", "kernel": kn, "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                    "peak_source": kind, "algorithmic_bytes": wk, "avg_launch_ms": a_ms, "launches": cnt[k],
                    "traffic": NCU_TRAFFIC.get(kn)}
        ach = wk / (a_ms * 1e-3) / 1e12
        return {"bound": "tensor", "kernel": kn, "achieved": ach, "peak": bf16, "unit": "TFLOP/s", "frac": ach / bf16,
                "peak_source": kind, "flops_per_application": wk, "avg_application_ms": a_ms, "applications": cnt[k],
                "traffic": NCU_TRAFFIC.get(kn)}
    roof = entry(dom)
    roof["other_kernels"] = {k: entry(k) for k in cand if k != dom and cnt.get(k)}
    return roof, {"ms": ms, "launches": cnt, "shares": shares}


# ---- oracle errors and the CPU path (the checker; oracle/ is used only here) ------------------
def _oracle_residual(w, u, settings=None, accurate=False):
    """Float64 residual of workload w at DOFs u by the oracle's C restatement."""
    from oracle import corc
    r = w.raw
    st = settings if settings is not None else w.settings
    kind, coords = r["kind"], r["coords"]
    n = coords.shape[0]
    if kind == "poisson":
        Re, _ = corc.q1_elements("poisson", r["conns"][0], coords, u, [20.0, 10.0, 1.0, 0.5], tangent=False)
        return corc.scatter(r["conns"][0], 1, Re, n)
    if kind == "heat":
        Re, _ = corc.q1_elements("heat", r["conns"][0], coords, u, [1.0], elem_field=r["k"], tangent=False)
        return corc.scatter(r["conns"][0], 1, Re, n)
    if kind == "neo_hooke_3d":
        Re, _ = corc.q1_elements("neo_hooke", r["conns"][0], coords, u, [r["E"], r["nu"]], accurate=accurate,
                                 tangent=False)
        return corc.scatter(r["conns"][0], 3, Re, 3 * n)
    if kind == "cook":
        Re, _ = corc.q1_elements("neo_hooke", r["conns"][0], coords, u, [r["E"], r["nu"]], accurate=accurate,
                                 tangent=False)
        R = corc.scatter(r["conns"][0], 2, Re, 2 * n)
        Rl = corc.neumann_lines(r["conns"][1], coords, (0.0, float(st["load multiplier"])))
        return R + corc.scatter(r["conns"][1], 2, Rl, 2 * n)
    if kind == "heat_be":
        Tn = _flat(st["dofs n"])
        Re, _ = corc.q1_elements("heat_be", r["conns"][0], coords, u, [1.0, 0.5, 1.0, float(st["time increment"])],
                                 node_field=Tn, tangent=False)
        return corc.scatter(r["conns"][0], 1, Re, n)
    raise ValueError(kind)


def oracle_errors(w, u_gpu, res0, settings=None, u_oracle=None, scale=1.0, seed=0):
    """Errors against the float64 oracle: residual parity at a random non-converged state
    (||R_gpu - R_oracle|| / ||R_oracle||), the true float64 residual of the GPU solution
    evaluated by the oracle relative to the load step's first residual, and, when the oracle
    solved too, ||u_gpu - u_oracle||_inf."""
    from autopdex_gb300 import assembler
    st = settings if settings is not None else w.settings
    free = ~np.asarray(w.raw["dirichlet"], dtype=bool).reshape(-1)
    rng = np.random.default_rng(seed)
    ur = rng.uniform(-scale, scale, w.n_dofs)
    shape = np.shape(next(iter(w.dofs.values()))) if isinstance(w.dofs, dict) else np.shape(w.dofs)
    ur_d = {next(iter(w.dofs)): ur.reshape(shape)} if isinstance(w.dofs, dict) else ur.reshape(shape)
    R_gpu = _flat(assembler.assemble_residual(ur_d, st, w.static_settings))
    acc = w.raw["kind"] in ("cook", "neo_hooke_3d")
    R_or = _oracle_residual(w, ur, st, accurate=acc)
    out = {"residual_parity": float(np.linalg.norm(R_gpu - R_or) / np.linalg.norm(R_or)),
           "residual_parity_state": f"uniform random DOFs in [-{scale:g}, {scale:g}]"}
    R_true = _oracle_residual(w, _flat(u_gpu), st, accurate=acc)
    out["true_residual_ratio"] = float(np.linalg.norm(R_true[free]) / res0) if res0 else None
    if acc:
        R_ref = _oracle_residual(w, _flat(u_gpu), st, accurate=False)
        out["true_residual_ratio_reference_evaluation"] = float(np.linalg.norm(R_ref[free]) / res0) if res0 else None
    if u_oracle is not None:
        out["max_abs_u_minus_oracle"] = float(np.abs(_flat(u_gpu) - _flat(u_oracle)).max())
        out["max_abs_u_oracle"] = float(np.abs(_flat(u_oracle)).max())
    return out


def cpu_solve(w, rtol=RTOL, direct=False, maxiter=2000000):
    """The CPU path of one linear(ized) solve from zero: C elements, SciPy COO -> CSR with the
    Dirichlet rows and columns deleted (scipy_assembling, solver.py:1180-1222), then spsolve
    (direct, solver.py:1520) or the C Jacobi-PCG to rtol; returns the solution and timings."""
    import scipy.sparse as sps
    import scipy.sparse.linalg as spla
    from oracle import corc
    r = w.raw
    coords, conn = r["coords"], r["conns"][0]
    n = coords.shape[0]
    free = ~np.asarray(r["dirichlet"], dtype=bool)
    u0 = np.zeros(n)
    t0 = time.perf_counter()
    if r["kind"] == "heat":
        Re, Ke = corc.q1_elements("heat", conn, coords, u0, [1.0], elem_field=r["k"])
    else:
        Re, Ke = corc.q1_elements("poisson", conn, coords, u0, [20.0, 10.0, 1.0, 0.5])
    R = corc.scatter(conn, 1, Re, n)
    t1 = time.perf_counter()
    m = conn.shape[1]
    A = sps.coo_matrix((Ke.ravel(), (np.repeat(conn, m, axis=1).ravel(), np.tile(conn, (1, m)).ravel())),
                       shape=(n, n)).tocsr()
    A = A[:, free][free].tocsr()
    del Ke
    t2 = time.perf_counter()
    b = -R[free]
    if direct:
        x = spla.spsolve(A.tocsc(), b)
        its = 0
    else:
        x, rr, its = corc.pcg_csr_tol(A, b, rtol, maxiter)
    t3 = time.perf_counter()
    u = np.zeros(n)
    u[free] = x
    rel = float(np.linalg.norm(A @ x - b) / np.linalg.norm(b))
    return u, {"s": t3 - t0, "elements_s": t1 - t0, "coo_to_csr_s": t2 - t1, "solve_s": t3 - t2, "iterations": its,
               "relative_residual": rel, "threads": corc.threads()}


# ---- sub-records -------------------------------------------------------------------------------
def rec_poisson(n=200, cpu=True):
    from autopdex_gb300 import configs, solver
    w = configs.poisson(n=n, solver="lapack")
    kw = dict(newton_tol=1e-10)
    solver.solver(w.dofs, w.settings, w.static_settings, **kw)
    s, (sol, info) = _timed(lambda: solver.solver(w.dofs, w.settings, w.static_settings, **kw))
    out = {"workload": f"poisson_{n}x{n}_q1 (one Newton step, direct solve)", "gpu_direct": dict(s=s, **_info())}
    wp = configs.poisson(n=n, solver="pcg")
    solver.solver(wp.dofs, wp.settings, wp.static_settings, newton_tol=1e-10, krylov_tol=1e-13)
    s2, _ = _timed(lambda: solver.solver(wp.dofs, wp.settings, wp.static_settings, newton_tol=1e-10,
                                          krylov_tol=1e-13))
    out["gpu_plain_fp64_pcg_1e-13"] = dict(s=s2, **_info())
    res0 = out["gpu_direct"]["res0"]
    u_or = None
    if cpu:
        u_or, c = cpu_solve(w, direct=True)
        out["cpu_baseline"] = dict(c, kind="port", sample="full problem: C elements, SciPy COO->CSR with Dirichlet "
                                   "deletion, SciPy spsolve (single-threaded SuperLU)")
    out["oracle_error"] = oracle_errors(w, sol, res0, u_oracle=u_or)
    return out


def rec_neo_hooke_cube(n=64, steps=10):
    import torch
    from autopdex_gb300 import configs, solver
    out = {"workload": f"neo_hooke_cube_{n}^3_hex8, load steps 1..{steps} of 10 (u_x = 0.03 k on x = 1), Newton to "
                       f"1e-10 of each step's first residual"}
    for name, prec, ktol in (("mixed_pcg", "mixed", 1e-4), ("plain_fp64_pcg", "float64", 1e-4)):
        w = configs.neo_hooke_cube(n=n, n_steps=10, precision=prec)
        dev = torch.device("cuda", torch.cuda.current_device())
        # start of load step 1 from the linear lifting of the prescribed values (from u = 0 the
        # first element layer is stretched threefold at h = 1/64 and undamped Newton diverges)
        x0 = np.zeros((w.n_dofs // 3, 3))
        x0[:, 0] = w.raw["stretch"] / w.raw["n_steps"] * w.raw["coords"][:, 0]
        kw = dict(newton_tol=0.0, newton_rtol=RTOL, maxiter=30, krylov_tol=ktol)
        per = []

        lift = torch.as_tensor(x0, device=dev)

        def all_steps(nsteps=steps):
            x = torch.zeros_like(lift)
            settings = dict(w.settings)
            for k in range(nsteps):
                # each step starts from the previous solution plus the linear lifting of the
                # prescribed increment (u_x += 0.03 x), consistent with the new boundary values
                x = x + lift
                settings = w.steps[k](settings)
                settings["dirichlet conditions"] = torch.as_tensor(np.asarray(settings["dirichlet conditions"]),
                                                                   device=dev)
                x, _ = solver.solver(x, settings, w.static_settings, **kw)
                per.append(_info())
            return x, settings
        # warm-up on the timed path itself (context, autotuning, graphs and everything else a
        # first pass sets up: a one-step warm-up left about 1 s of it in the timed mixed run):
        # all steps for the mixed solve, the first for the plain one
        all_steps(steps if prec == "mixed" else 1)
        per.clear()
        s, (x, settings) = _timed(all_steps)
        out[name] = {"s": s, "newton": sum(p["newton"] for p in per), "krylov": sum(p["krylov"] for p in per),
                     "max_residual_ratio": max(p["residual_ratio"] for p in per),
                     "diverged": any(p["diverged"] for p in per)}
        if name == "mixed_pcg":
            st_np = dict(settings)
            st_np["dirichlet conditions"] = np.asarray(settings["dirichlet conditions"].cpu())
            out["oracle_error"] = oracle_errors(w, x, per[-1]["res0"], settings=st_np, scale=0.003)
    out["speedup_mixed_vs_plain_fp64"] = out["plain_fp64_pcg"]["s"] / out["mixed_pcg"]["s"]
    return out


def rec_cook(n=512, steps=1, plain_limit_s=120.0, with_learned=False):
    """Cook's membrane: float64 Newton with the direct (banded Cholesky) solve, with plain
    float64 Jacobi-PCG, and, when trained weights exist, with the learned preconditioner in
    float64 flexible CG (the float32 / bf16 two-level preconditioner inside float64 vectors)."""
    from autopdex_gb300 import configs, learned, solver
    out = {"workload": f"cook_membrane_{n}x{n}_q1 (nu = 0.4999), load steps 1..{steps} of 20"}
    # the float64 residual of this nearly incompressible membrane stalls near 4e-8 of a load
    # step's first residual at 512^2 (rounding of the displacements, amplified by lam / mu =
    # 5000, not the solver: the direct solve stalls there too), so the Newton tolerance is 1e-7
    rt = 1e-7
    out["newton_rtol"] = rt
    variants = [("direct_fp64", dict(solver="lapack"), 1e-13), ("plain_fp64_pcg", dict(solver="pcg"), 1e-4)]
    wpath = os.path.join(learned.WEIGHTS_DIR, "membrane_unet_n256.npz")
    if with_learned and os.path.exists(wpath):
        variants.append(("learned_fp64_fcg", dict(solver="fcg", **{"type of preconditioner": "learned"}), 1e-4))
    for name, st, ktol in variants:
        w = configs.cook_membrane(n=n)
        static = dict(w.static_settings, precision="float64", **st)
        kw = dict(newton_tol=0.0, newton_rtol=rt, maxiter=12, krylov_tol=ktol, krylov_maxiter=200000)
        if name.startswith("learned"):
            net = learned.UNet.load(wpath)
            factor = n // 128
            coarse = configs.cook_membrane(n=n // factor)
            solver.set_learned_preconditioner(None, learned.GridPreconditioner(
                net, n, n, factor=factor, nd=2, aux=learned.node_features(coarse.raw["coords"])))
            out["network"] = {"weights": os.path.basename(wpath), "grid": f"{n // factor + 1}^2 (coarsening {factor})"}
        x = w.dofs
        settings = dict(w.settings)
        per = []
        t0 = time.perf_counter()
        for k in range(steps):
            settings = w.steps[k](settings)
            s, (x, info) = _timed(lambda: solver.solver(x, settings, static, **kw))
            per.append(dict(s=s, **_info()))
            if time.perf_counter() - t0 > plain_limit_s:
                break
        out[name] = {"s": sum(p["s"] for p in per), "steps_run": len(per), "per_step": per}
        if name == "direct_fp64":
            out["oracle_error"] = oracle_errors(w, x, per[-1]["res0"], settings=settings, scale=1e-5)
    if "learned_fp64_fcg" in out and out["learned_fp64_fcg"]["steps_run"] == out["plain_fp64_pcg"]["steps_run"]:
        out["speedup_learned_vs_plain_fp64"] = out["plain_fp64_pcg"]["s"] / out["learned_fp64_fcg"]["s"]
    return out


def rec_heat(h):
    """The headline problem's record: the three variants and the oracle's errors."""
    w = h["w"]
    out = {"workload": f"heat_grf_{w.raw['n']}x{w.raw['n']}_q1 (seed 10000), time to {RTOL:g}",
           "network_grid": f"{w.raw['n'] // h['factor'] + 1}^2 nodes (coarsening {h['factor']})"}
    out.update(h["comparison"])
    return out


def rec_heat_be(n=128, steps=100, plain_steps=3):
    """The 128^3 backward-Euler heat workload: all 100 time steps with mixed Jacobi-PCG and with
    the learned (3-D network) + mixed flexible CG, the first plain_steps with float64 BiCGStab;
    Newton to a 1e-10 float64 residual ratio in every step; and the float32 tangent assembly's
    roofline."""
    import torch
    from autopdex_gb300 import configs, learned, solver
    out = {"workload": f"heat_be_{n}^3_hex8 (k = 1 + 0.5 T^2, dt = 1e-3), time steps 1..{steps} of 100"}
    variants = [("mixed_pcg", dict(solver="pcg", precision="mixed"), 1e-5, steps),
                ("plain_fp64_bicgstab", dict(solver="bicgstab", precision="float64"), 1e-11, plain_steps)]
    wpath = os.path.join(learned.WEIGHTS_DIR, f"brick_unet_n{n}.npz")
    if os.path.exists(wpath):
        # inner tolerance 1e-4 (measured over 5 steps with Chebyshev smoothing: 1e-3 / 1e-4 / 1e-5
        # -> 20 / 16 / 16 Newton steps, 35.5 / 29.4 / 32.2 ms per time step; over 10 steps with the
        # damped Jacobi sweeps: 3e-5 / 1e-4 / 3e-4 / 1e-3 -> 20.6 / 19.8 / 20.0 / 19.7 ms)
        variants.insert(1, ("learned_mixed_fcg", dict(solver="fcg", precision="mixed",
                                                      **{"type of preconditioner": "learned"}), 1e-4, steps))
    for name, st, ktol, nsteps in variants:
        w = configs.heat_transient(n=n)
        static = dict(w.static_settings, **st)
        pc = None
        if name.startswith("learned"):
            net = learned.UNet3D.load(wpath)
            pc = learned.BrickPreconditioner(net, n, factor=4)
            solver.set_learned_preconditioner(None, pc)
            out["network"] = {"weights": os.path.basename(wpath), "grid": f"{pc.nc}^3 nodes (coarsening 4), "
                              f"image {pc.npad}^3"}
        dev = torch.device("cuda", torch.cuda.current_device())
        T0 = torch.as_tensor(w.raw["T0"], device=dev)
        kw = dict(newton_tol=0.0, newton_rtol=RTOL, maxiter=30, krylov_tol=ktol)
        settings = dict(w.settings)
        settings["dofs n"] = {"T": T0.clone()}
        settings["dirichlet conditions"] = {"T": torch.zeros_like(T0)}
        per = []
        first = {}
        start, mid = _events()

        def run(count=nsteps):
            T = T0.clone()
            for k in range(count):
                settings["dofs n"] = {"T": T}
                Tn, _ = solver.solver({"T": T}, settings, static, **kw)
                per.append(_info())
                if k == 0:
                    first["T1"] = Tn["T"].clone()
                if k == plain_steps - 1:
                    mid.record()
                T = Tn["T"]
            return T
        # warm-up on the timed path itself (context, tuning, graphs and whatever else a first pass
        # sets up): all steps for the fast solves, one for plain float64
        run(nsteps if nsteps > plain_steps else 1)
        per.clear()
        first.clear()
        start.record()
        s, T = _timed(run)
        if pc is not None:
            solver.set_learned_preconditioner(None, None)
        out[name] = {"s_per_step": s / nsteps, "steps": nsteps,
                     f"s_per_step_first_{plain_steps}": start.elapsed_time(mid) / 1e3 / plain_steps,
                     "newton": sum(p["newton"] for p in per), "krylov": sum(p["krylov"] for p in per),
                     "max_residual_ratio": max(p["residual_ratio"] for p in per),
                     "sum_T_squared": float((T * T).sum())}
        if name == "mixed_pcg":
            st0 = dict(w.settings)
            st0["dofs n"] = {"T": w.raw["T0"]}
            out["oracle_error_first_step"] = oracle_errors(w, first["T1"], per[0]["res0"], settings=st0, scale=1.0)
    # over the same time steps (the first plain_steps: the later ones need fewer iterations)
    key = f"s_per_step_first_{plain_steps}"
    base = out["plain_fp64_bicgstab"][key]
    out["speedup_mixed_vs_plain_fp64"] = base / out["mixed_pcg"][key]
    if "learned_mixed_fcg" in out:
        out["speedup_learned_vs_plain_fp64"] = base / out["learned_mixed_fcg"][key]
    try:
        out["assembly_hbm"] = assembly_roofline(workload="heat_be", n=n)
    except Exception as e:  # noqa: BLE001 -- the record keeps the solve numbers
        out["assembly_hbm"] = {"error": str(e)[:200]}
    return out


def assembly_roofline(n=1024, reps=20, workload="heat_grf"):
    """Float32 tangent assembly, timed with CUDA events per agx_assemble call after a 256 MB
    buffer write (inputs from HBM): of the n^2 random-conductivity heat mesh (``heat_grf``,
    the structured-grid kernel) or of the n^3 backward-Euler brick mesh (``heat_be``, the
    element kernel with its scatter into the tangent's slots).  Algorithmic bytes: coordinates
    + DOFs (+ the previous time step's DOFs) + connectivity + values written once (n_nodes dim 8
    + n_dofs 8 (x 2) + n_e nen 4 + nnz 4)."""
    import ctypes as C
    import torch
    from autopdex_gb300 import configs, _native as N
    from autopdex_gb300._problem import get_problem
    if workload == "heat_be":
        w = configs.heat_transient(n=n)
        dim, nen, n_e, kernel = 3, 8, n ** 3, "element_kernel<HEAT_BE, float> (scatter into the slot map)"
    else:
        w = configs.heat_grf(n=n, seed=0)
        dim, nen, n_e, kernel = 2, 4, n * n, "grid_tangent_kernel<HEAT_POTENTIAL,float>"
    prob = get_problem(w.dofs, w.settings, w.static_settings)
    prob.update_models(w.settings)
    if workload == "heat_be":
        x = torch.as_tensor(w.raw["T0"], dtype=torch.float64, device=prob.device)
    else:
        x = torch.zeros(prob.n_dofs, dtype=torch.float64, device=prob.device)
    for _ in range(3):
        prob._call("agx_assemble", C.c_void_p(x.data_ptr()), None, N.AGX_F32)
    flush = _flush_buffer()
    ev = [_events() for _ in range(reps)]
    for a, b in ev:
        flush.fill_(1)
        a.record()
        prob._call("agx_assemble", C.c_void_p(x.data_ptr()), None, N.AGX_F32)
        b.record()
    _sync()
    call_ms = sum(a.elapsed_time(b) for a, b in ev)

    def kern():
        for _ in range(reps):
            flush.fill_(1)
            prob._call("agx_assemble", C.c_void_p(x.data_ptr()), None, N.AGX_F32)
    ms, cnt = _profile(prob, kern)
    del flush
    nbytes = prob.n_nodes * dim * 8 + prob.n_dofs * 8 * (2 if workload == "heat_be" else 1) + n_e * nen * 4 + \
        prob.nnzb * prob.ndof * prob.ndof * 4
    call_s = call_ms / 1e3 / reps
    kern_s = ms["tangent_assembly"] / 1e3 / max(1, cnt["tangent_assembly"])
    peak, _, kind = _peaks()
    name = f"heat_be_{n}^3_hex8" if workload == "heat_be" else f"heat_grf_{n}x{n}_q1"
    return {"workload": f"{name} float32 tangent", "kernel": kernel,
            "algorithmic_bytes": nbytes, "call_us": call_s * 1e6, "kernel_us": kern_s * 1e6,
            "achieved_gbs_call": nbytes / call_s / 1e9, "achieved_gbs_kernel": nbytes / kern_s / 1e9,
            "peak_gbs": peak, "frac_call": nbytes / call_s / 1e9 / peak, "frac_kernel": nbytes / kern_s / 1e9 / peak,
            "peak_source": kind, "l2": "256 MB buffer written before every timed call"}


def cpu_baseline_headline(h, budget_s=120.0):
    """The CPU path on the full headline problem (one solve to 1e-10 with Jacobi-PCG), and the
    headline's errors against it."""
    w = h["w"]
    u_or, c = cpu_solve(w, rtol=RTOL)
    err = oracle_errors(w, h["solution"], h["info"]["res0"], u_oracle=u_or)
    base = {"value": c["s"], "unit": "s", "cores": c["threads"], "kind": "port",
            "sample": (f"the full {w.raw['n']}^2 problem: C elements ({c['elements_s']:.2f} s), SciPy COO->CSR with "
                       f"Dirichlet deletion ({c['coo_to_csr_s']:.2f} s), C OpenMP Jacobi-PCG to {RTOL:g} "
                       f"({c['iterations']} iterations, {c['solve_s']:.2f} s)"),
            "relative_residual": c["relative_residual"]}
    return base, err


# ---- arms ----------------------------------------------------------------------------------------
def gpu_arm(args):
    import torch
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    args.dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        args.dist = dist
    h = headline(args, rank)
    n = args.size
    line = {
        "metric": f"time_to_{RTOL:g}_relative_fp64_residual (learned+mixed vs plain FP64 Jacobi-PCG; "
                  f"{n}^2 random-conductivity heat, the learned-preconditioner workload)",
        "value": h["s"], "unit": "s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": h["s"] * 1e3, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 FCG + bf16 network + f64 residual/refinement",
        "data": "synthetic (seeded Gaussian random field conductivity; no dataset)",
        "config": {"workload": f"heat_grf_{n}x{n}_q1_seed10000", "n_dofs": h["w"].n_dofs, "newton_rtol": RTOL,
                   "krylov": "flexible CG (float32) with the U-Net two-level preconditioner, inner rtol 1e-3",
                   "network_grid": f"{n // h['factor'] + 1}^2 (coarsening {h['factor']})",
                   "l2": "256 MB buffer written before every timed step", "krylov_chunks": "CUDA graphs",
                   "conv_variants": h["conv_variants"],
                   "parallelism": "replicas" if world > 1 else "1 gpu"},
        "newton_iterations": h["info"]["newton"], "krylov_iterations": h["info"]["krylov"],
        "final_residual_ratio": h["info"]["residual_ratio"],
        "converged": (not h["info"]["diverged"]) and h["info"]["residual_ratio"] <= RTOL * 1.0000001,
        "plain_fp64_pcg_s": h["comparison"]["plain_fp64_pcg"]["s"],
        "speedup_learned_mixed_vs_plain_fp64": h["comparison"]["speedup_learned_mixed_vs_plain_fp64"],
        "gpu_launches": int(round(h["launches_per_step"] * args.steps)),
        "clocks": h["clocks"],
    }
    try:
        line["e2e"] = headline_e2e(h, args.steps)
    except Exception as e:  # noqa: BLE001 -- reported, the headline stands
        line["e2e"] = {"error": str(e)[:200]}
    try:
        line["roofline"], line["kernel_ms_per_step"] = headline_roofline(h)
    except Exception as e:  # noqa: BLE001
        line["roofline"] = {"error": str(e)[:200]}
    configs_out = {}
    if rank == 0 and not args.only_headline:
        configs_out["heat_1024"] = rec_heat(h)
        for key, fn in (("poisson_200", lambda: rec_poisson(cpu=not args.no_cpu_baseline)),
                        ("neo_hooke_64cube", rec_neo_hooke_cube),
                        ("cook_512", lambda: rec_cook(steps=args.cook_steps)),
                        ("heat_be_128cube", rec_heat_be)):
            try:
                configs_out[key] = fn()
            except Exception as e:  # noqa: BLE001 -- reported, the headline stands
                configs_out[key] = {"error": str(e)[:300]}
        try:
            line["assembly_hbm"] = assembly_roofline()
            line["assembly_hbm_2048"] = assembly_roofline(n=2048)  # values (151 MB) larger than L2
        except Exception as e:  # noqa: BLE001
            line["assembly_hbm"] = {"error": str(e)[:200]}
    if rank == 0 and not args.no_cpu_baseline:
        try:
            line["cpu_baseline"], err = cpu_baseline_headline(h)
            if "heat_1024" in configs_out:
                configs_out["heat_1024"]["oracle_error"] = err
            line["oracle_error"] = err
        except Exception as e:  # noqa: BLE001
            line["cpu_baseline"] = {"error": str(e)[:300]}
    if configs_out:
        line["configs"] = configs_out
    if args.dist:
        args.dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(line, default=float))


def reference_arm(args):
    """The CPU path of the headline workload (one full solve to 1e-10 per step) on all host
    cores: the oracle's C restatement, since the reference is JAX code and no JAX exists."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from autopdex_gb300 import configs
    n = args.size
    w = configs.heat_grf(n=n, seed=10000)
    for _ in range(args.warmup):
        cpu_solve(w)
    vals, last = [], None
    t0 = time.perf_counter()
    for _ in range(args.steps):
        _, last = cpu_solve(w)
        vals.append(last["s"])
    wall = time.perf_counter() - t0
    v = float(np.median(vals))
    sample = (f"full {n}^2 problem per step: C elements, SciPy COO->CSR with Dirichlet deletion, C OpenMP "
              f"Jacobi-PCG to {RTOL:g} ({last['iterations']} iterations)")
    line = {"impl": "reference",
            "metric": f"time_to_{RTOL:g}_relative_fp64_residual (learned+mixed vs plain FP64 Jacobi-PCG; "
                      f"{n}^2 random-conductivity heat, the learned-preconditioner workload)",
            "value": v, "unit": "s", "n_gpus": int(os.environ.get("WORLD_SIZE", "1")), "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": wall / args.steps * 1e3, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"heat_grf_{n}x{n}_q1_seed10000"},
            "cpu_baseline": {"value": v, "unit": "s", "cores": last["threads"], "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# ---- small cases for ncu captures (no JSON line) ----------------------------------------------
def case(args):
    import ctypes as C
    import torch
    from autopdex_gb300 import configs, learned, solver, _native as N
    from autopdex_gb300._problem import get_problem
    if args.case == "conv":
        net = learned.UNet(seed=0)
        if args.halo_loader >= 0:
            assert net.lib.agx_nn_set_halo_loader(args.halo_loader) == 0
        _, c1, c2, co, relu = next(l for l in learned.LAYERS if l[0] == args.layer)
        g = torch.Generator(device="cuda").manual_seed(0)
        x1 = torch.randn(1, args.size, args.size, c1, device="cuda", generator=g).to(torch.bfloat16)
        x2 = torch.randn(1, args.size, args.size, c2, device="cuda", generator=g).to(torch.bfloat16) if c2 else None
        net._conv(args.layer, x1, x2, 1, (args.size, args.size))  # warm-up (attributes, first launch)
        _sync()
        a, b = _events()
        a.record()
        for _ in range(args.reps):
            net._conv(args.layer, x1, x2, 1, (args.size, args.size))
        b.record()
        _sync()
        net.check()
        print(f"conv {args.layer} on {args.size}^2: {args.reps} launches after one warm-up launch, "
              f"{a.elapsed_time(b) * 1e3 / max(1, args.reps):.2f} us per launch (CUDA events, back to back)")
        return
    make = {"heat": lambda: configs.heat_grf(n=args.size, seed=10000, precision=args.precision, solver=args.solver),
            "poisson": lambda: configs.poisson(n=args.size, precision=args.precision, solver=args.solver),
            "neo_hooke": lambda: configs.neo_hooke_cube(n=args.size, precision=args.precision, solver=args.solver),
            "cook": lambda: configs.cook_membrane(n=args.size, precision=args.precision, solver=args.solver),
            "heat_be": lambda: configs.heat_transient(n=args.size, precision=args.precision, solver=args.solver)}
    w = make[args.workload]()
    if args.case == "assembly":
        prob = get_problem(w.dofs, w.settings, w.static_settings)
        prob.update_models(w.settings)
        x = torch.zeros(prob.n_dofs, dtype=torch.float64, device=prob.device)
        dt = N.AGX_F32 if args.precision == "mixed" else N.AGX_F64
        for _ in range(args.reps):
            prob._call("agx_assemble", C.c_void_p(x.data_ptr()), None, dt)
        _sync()
        print(f"assembly {w.name}: {args.reps} calls")
        return
    static = dict(w.static_settings)
    if args.learned and args.workload == "heat_be":  # the 3-D network on the brick grid coarsened by 4
        net3 = learned.UNet3D.load(os.path.join(learned.WEIGHTS_DIR, f"brick_unet_n{args.size}.npz"))
        solver.set_learned_preconditioner(None, learned.BrickPreconditioner(net3, args.size, factor=4))
        static["type of preconditioner"] = "learned"
    elif args.learned:
        _heat_learned_setup(w, args.size)
        static["type of preconditioner"] = "learned"
    settings = w.steps[0](dict(w.settings)) if w.steps else w.settings
    kw = dict(newton_tol=0.0, newton_rtol=RTOL if args.workload != "cook" else 1e-7, maxiter=30,
              krylov_tol=args.krylov_tol, krylov_maxiter=400000)
    x0 = w.dofs
    if args.workload == "neo_hooke":  # load step 1 from the linear lifting of the prescribed u_x
        x0 = np.zeros((w.n_dofs // 3, 3))
        x0[:, 0] = w.raw["stretch"] / w.raw["n_steps"] * w.raw["coords"][:, 0]
    solver.solver(x0, settings, static, **kw)  # context, autotuning, graphs
    if args.tpr:  # a product variant instead of the autotuner's pick (lanes per row, +256: four blocks per trip)
        prob = get_problem(x0, settings, static)
        dt = N.AGX_F32 if args.precision == "mixed" else N.AGX_F64
        prob._call("agx_set_tuning", dt, int(args.tpr))
    for _ in range(args.reps):
        solver.solver(x0, settings, static, **kw)
    _sync()
    print(f"solve {w.name}: {args.reps} solves after a warm-up solve, last {json.dumps(_info())}")
    if args.profile:  # one more solve with the library's per-category CUDA events (graphs off)
        prob = get_problem(x0, settings, static)
        ms, cnt = _profile(prob, lambda: solver.solver(x0, settings, static, **kw))
        print("profile (ms, launches): " + json.dumps({k: [round(v, 3), cnt[k]] for k, v in ms.items() if cnt[k]}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--size", type=int, default=1024)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--only-headline", action="store_true", help="time the headline only (profiling runs)")
    ap.add_argument("--cook-steps", type=int, default=1)
    ap.add_argument("--case", choices=["conv", "assembly", "solve"], help="one small case for ncu captures")
    ap.add_argument("--workload", default="heat", choices=["heat", "poisson", "neo_hooke", "cook", "heat_be"])
    ap.add_argument("--profile", action="store_true", help="solve case: per-category kernel times of one more solve")
    ap.add_argument("--precision", default="mixed")
    ap.add_argument("--solver", default="pcg")
    ap.add_argument("--learned", action="store_true")
    ap.add_argument("--krylov-tol", type=float, default=1e-4)
    ap.add_argument("--layer", default="e0b")
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--tpr", type=int, default=0, help="solve case: SpMV variant code instead of the autotuner's")
    ap.add_argument("--bf16-smoothing", action="store_true",
                    help="the learned preconditioner's smoothing products on a bf16 copy of the tangent values")
    ap.add_argument("--halo-loader", type=int, default=-1, help="conv case: agx_nn_set_halo_loader mode")
    args = ap.parse_args()
    global BF16_SMOOTHING
    BF16_SMOOTHING = args.bf16_smoothing
    if args.case:
        case(args)
        return
    if args.impl == "reference":
        reference_arm(args)
        return
    args.warmup = max(args.warmup, 3)
    gpu_arm(args)


if __name__ == "__main__":
    main()
