"""Diagnostics run on the GPU (not part of the solve path).

    python -m autopdex_gb300.diag                    # memory / FP64 / FP32 / atomic throughput probe
    python -m autopdex_gb300.diag conv --size 1088 --layer e0b --reps 3
        # one U-Net convolution layer of the learned preconditioner on a size x size image,
        # launched `reps` times (a small, self-contained case for ncu captures of conv3x3_tc)
    python -m autopdex_gb300.diag assembly --workload heat --size 1024 --reps 20
        # tangent / residual assembly passes of one workload, timed with CUDA events
    python -m autopdex_gb300.diag solve --workload heat --size 1024 --precision float64 --krylov-tol 1e-11
        # one solver.solver call (after a warm-up call) with per-category kernel times
"""
import argparse
import os
import subprocess
import sys

from autopdex_gb300 import build as B

HERE = os.path.dirname(os.path.abspath(__file__))


def probe():
    src = os.path.join(HERE, "throughput_probe.cu")
    exe = os.path.join(B.LIBDIR, "throughput_probe")
    os.makedirs(B.LIBDIR, exist_ok=True)
    subprocess.run([B._nvcc()] + B.ARCH + ["-O3", "-o", exe, src], check=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    sys.stdout.write(r.stdout)
    sys.exit(r.returncode)


def conv(size, layer, reps):
    import torch
    from autopdex_gb300 import learned
    net = learned.UNet(seed=0)
    _, c1, c2, co, relu = next(l for l in learned.LAYERS if l[0] == layer)
    g = torch.Generator(device="cuda").manual_seed(0)
    x1 = torch.randn(1, size, size, c1, device="cuda", generator=g).to(torch.bfloat16)
    x2 = torch.randn(1, size, size, c2, device="cuda", generator=g).to(torch.bfloat16) if c2 else None
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    start.record()
    for _ in range(reps):
        net._conv(layer, x1, x2, 1, size, size)
    end.record()
    torch.cuda.synchronize()
    net.check()
    flops = 2 * 9 * (c1 + c2) * co * size * size
    ms = start.elapsed_time(end) / reps
    print(f"conv {layer} {c1}+{c2}->{co} on {size}x{size}: {ms * 1e3:.1f} us per launch "
          f"({flops / ms / 1e9:.1f} TFLOP/s, launch overhead included)")


def assembly(workload, size, reps):
    import ctypes as C
    import json
    import torch
    from autopdex_gb300 import configs, _native as N
    from autopdex_gb300._problem import get_problem
    if workload == "heat":
        w = configs.heat_grf(n=size, seed=0)
    elif workload == "poisson":
        w = configs.poisson(n=size)
    else:
        w = configs.neo_hooke_cube(n=size)
    prob = get_problem(w.dofs, w.settings, w.static_settings)
    prob.update_models(w.settings)
    x = torch.zeros(prob.n_dofs, dtype=torch.float64, device=prob.device)
    R = torch.empty_like(x)
    out = {"workload": w.name, "n_dofs": prob.n_dofs, "nnzb": prob.nnzb}
    for name, res, dt in (("tangent_f32", None, N.AGX_F32), ("tangent_f64", None, N.AGX_F64),
                          ("residual_f64", R, -1)):
        rp = C.c_void_p(res.data_ptr()) if res is not None else None
        for _ in range(3):
            prob._call("agx_assemble", C.c_void_p(x.data_ptr()), rp, dt)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(reps):  # per call, the library's own timing off
            prob._call("agx_assemble", C.c_void_p(x.data_ptr()), rp, dt)
        b.record()
        torch.cuda.synchronize()
        prob._call("agx_profile", 1)
        for _ in range(reps):  # per kernel pass, with the library's events
            prob._call("agx_assemble", C.c_void_p(x.data_ptr()), rp, dt)
        torch.cuda.synchronize()
        ms = (C.c_double * N.AGX_PROF_CATEGORIES)()
        cnt = (C.c_int64 * N.AGX_PROF_CATEGORIES)()
        prob._call("agx_profile_read", ms, cnt)
        prob._call("agx_profile", 0)
        cat = N.AGX_PROF_TANGENT if dt >= 0 else N.AGX_PROF_RESIDUAL
        out[name] = {"call_us": a.elapsed_time(b) / reps * 1e3,
                     "kernel_us": ms[cat] / max(1, cnt[cat]) * 1e3}
    print(json.dumps(out))


def solve(workload, size, precision, krylov_tol):
    import ctypes as C
    import json
    import time
    import torch
    from autopdex_gb300 import configs, solver, _native as N
    from autopdex_gb300._problem import get_problem
    w = configs.heat_grf(n=size, seed=10000, precision=precision) if workload == "heat" else \
        configs.poisson(n=size, precision=precision)
    kw = dict(newton_tol=0.0, newton_rtol=1e-10, maxiter=30, krylov_tol=krylov_tol, krylov_maxiter=400000)
    solver.solver(w.dofs, w.settings, w.static_settings, **kw)
    prob = get_problem(w.dofs, w.settings, w.static_settings)
    prob._call("agx_profile", 1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    _, info = solver.solver(w.dofs, w.settings, w.static_settings, **kw)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    ms = (C.c_double * N.AGX_PROF_CATEGORIES)()
    cnt = (C.c_int64 * N.AGX_PROF_CATEGORIES)()
    prob._call("agx_profile_read", ms, cnt)
    prob._call("agx_profile", 0)
    names = ["tangent", "residual", "spmv", "vector", "precond"]
    print(json.dumps({"workload": w.name, "precision": precision, "s (profiled, no graphs)": dt,
                      "newton": int(info[0]), "krylov": int(solver.last_info.krylov_iterations),
                      "ms": {n: ms[i] for i, n in enumerate(names)},
                      "launches": {n: int(cnt[i]) for i, n in enumerate(names)}}))


def main():
    if len(sys.argv) < 2 or sys.argv[1] == "probe":
        probe()
        return
    ap = argparse.ArgumentParser()
    ap.add_argument("what", choices=["conv", "assembly", "solve"])
    ap.add_argument("--precision", default="float64")
    ap.add_argument("--krylov-tol", type=float, default=1e-11)
    ap.add_argument("--size", type=int, default=1088)
    ap.add_argument("--layer", default="e0b")
    ap.add_argument("--workload", default="heat", choices=["heat", "poisson", "neo_hooke"])
    ap.add_argument("--reps", type=int, default=3)
    a = ap.parse_args()
    if a.what == "conv":
        conv(a.size, a.layer, a.reps)
    elif a.what == "assembly":
        assembly(a.workload, a.size, a.reps)
    else:
        solve(a.workload, a.size, a.precision, a.krylov_tol)


if __name__ == "__main__":
    main()
