"""Benchmark: ILU(0)-PCG solves/s on the 128^3 anisotropic 7-point system to a 1e-10 relative
residual, mixed precision (FP32 PCG with FP64 refinement by reliable updates) against plain FP64,
plus SpMV GB/s against the measured HBM copy bandwidth.  The restarted refinement (a new FP32
PCG per FP64 sweep) is timed beside it.

One step = one complete solve from x0 = 0 (ILU setup excluded, timed separately).
    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
Under torchrun with N > 1 each rank solves its own replica (the path does not shard);
value = solves of all ranks / max wall time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "PCG solves/s (128³ Poisson, 1e-10 rel res) mixed vs FP64; SpMV GB/s vs HBM peak"
GRID = int(os.environ.get("HGB_BENCH_GRID", "128"))
COEF = (1.0, 1.0, 0.01)
RTOL = 1e-10
IR_INNER_RTOL = 1e-5     # first refinement sweep; later sweeps stop at what the target needs
RU_DELTA = 0.01          # reliable update when ||r|| has dropped 100x since the last one
SEED = 2


def workload():
    from hala_gb300 import problems as P
    p, i, v = P.aniso3d(GRID, coef=COEF)
    n = len(p) - 1
    xt = np.random.default_rng(SEED).standard_normal(n)
    b = P.csr_matvec(p, i, v, xt)
    return p, i, v, xt, b


def spmv_bytes(n, nnz, vbytes, xbytes):
    # vals + indx per entry, pntr, x read once, y written once (the algorithmic minimum)
    return (vbytes + 4) * nnz + 4 * (n + 1) + 2 * xbytes * n


def ilu_apply_bytes(n, nnz, vbytes, xbytes):
    # both triangles' values and columns once, row pointers twice, diag/perm per solve,
    # input, intermediate (write + read) and output vectors
    return (vbytes + 4) * nnz + 8 * (n + 1) + 16 * n + 4 * xbytes * n


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.dev = device_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_sample(p, i, v, b, full_iters, target_s=12.0):
    """FP64 ILU(0)-PCG of the oracle (the reference's algorithm, serial) on the host cores:
    a bounded sample of iterations, extrapolated to one full solve."""
    from oracle import oracle as O
    tol = RTOL * float(np.linalg.norm(b))
    f, d, _ = O.ilu_factor(p, i, v)
    t0 = time.perf_counter()
    O.cg(p, i, v, b, tol=tol, max_iter=4, diag=d, ilu=f)
    per_it = (time.perf_counter() - t0) / 4
    m = int(max(8, min(400, target_s / max(per_it, 1e-6))))
    t0 = time.perf_counter()
    _, it, _ = O.cg(p, i, v, b, tol=tol, max_iter=m, diag=d, ilu=f)
    dt = time.perf_counter() - t0
    per_it = dt / max(it - 1, 1)
    return {"value": 1.0 / (per_it * full_iters), "unit": "solves/s", "cores": 1, "kind": "port",
            "sample": f"{it - 1} FP64 ILU(0)-PCG iterations of the 128^3 solve ({dt:.1f} s), extrapolated "
                      f"to the {full_iters} iterations of a full solve; ILU factor excluded"}


def run_reference(args, rank, world):
    """Reference arm: the reference's CPU algorithm for the path (the oracle port: the reference's
    own sources are not on this machine), FP64 ILU(0)-PCG, timed on the host cores."""
    if rank != 0:
        return
    from oracle import oracle as O
    p, i, v, xt, b = workload()
    n = len(p) - 1
    tol = RTOL * float(np.linalg.norm(b))
    f, d, _ = O.ilu_factor(p, i, v)
    # warm-up: one full solve gives the iteration count of the workload
    t0 = time.perf_counter()
    x, full_iters, _ = O.cg(p, i, v, b, tol=tol, diag=d, ilu=f) if args.warmup > 0 else (None, 0, 0)
    t_full = time.perf_counter() - t0
    if not full_iters:
        full_iters = 300
    per_step_iters = 10
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        _, it, _ = O.cg(p, i, v, b, tol=tol, max_iter=per_step_iters + 1, diag=d, ilu=f)
        times.append((time.perf_counter() - t0) / (it - 1))
    per_it = statistics.median(times)
    val = 1.0 / (per_it * full_iters)
    sample = (f"{args.steps} steps of {per_step_iters} FP64 ILU(0)-PCG iterations (serial, as the reference's "
              f"sparse path), extrapolated to the {full_iters}-iteration full solve (one full solve in "
              f"warm-up took {t_full:.1f} s)")
    print(json.dumps({
        "metric": METRIC, "value": val, "unit": "solves/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": per_it * full_iters * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
        "config": {"workload": f"ILU(0)-PCG 3D 7-point anisotropic {GRID}^3 (1,1,0.01), rel res 1e-10",
                   "n": n, "nnz": int(len(i))},
        "cpu_baseline": {"value": val, "unit": "solves/s", "cores": 1, "kind": "port", "sample": sample},
        "e2e": {"value": val, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def max_over_ranks(times_ms, device):
    """Replicas: each rank times its own solves; the job's time is the slowest rank's (barrier on
    both sides of the timed region), so value = solves of all ranks / that time."""
    import torch
    import torch.distributed as dist
    t = torch.tensor(times_ms, dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()


def aggregate_rate(world, ms_per_solve):
    """Whole-job solves/s of `world` replicas whose slowest rank took ms_per_solve per solve."""
    return world * 1e3 / ms_per_solve


def flush_l2(buf):
    buf.add_(1.0)   # writes 256 MB > the 129 MB L2


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--grid", type=int, default=None, help="grid edge (default 128: the headline workload)")
    ap.add_argument("--kernels-only", action="store_true",
                    help="only the SpMV and ILU-apply launches (for profiling captures)")
    args = ap.parse_args()
    if args.grid:
        global GRID
        GRID = args.grid

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return

    import torch
    import torch.distributed as dist
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    from hala_gb300 import build as hb
    hb.build()
    from hala_gb300 import engine as E

    p, i, v, xt, b = workload()
    n, nnz = len(p) - 1, len(i)
    tol = RTOL * float(np.linalg.norm(b))
    eng = E.gpu_engine(local)
    gp, gi, gv = (torch.from_numpy(a).to(dev) for a in (p, i, v))
    gb = torch.from_numpy(b).to(dev)
    gv32 = gv.float()
    A64 = E.make_sparse_matrix(eng, n, gp, gi, gv)
    A32 = E.make_sparse_matrix(eng, n, gp, gi, gv32)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    M64 = E.make_ilu(eng, gp, gi, gv)
    torch.cuda.synchronize()
    setup64 = time.perf_counter() - t0
    t0 = time.perf_counter()
    M32 = E.make_ilu(eng, gp, gi, gv, store=torch.float32)
    torch.cuda.synchronize()
    setup32 = time.perf_counter() - t0
    flush = torch.empty(32 * 1024 * 1024, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    if args.kernels_only:
        y64 = torch.empty(n, dtype=torch.float64, device=dev)
        y32 = torch.empty(n, dtype=torch.float32, device=dev)
        xs32 = gb.float()
        Ab = E.make_sparse_matrix(eng, n, gp, gi, gv.to(torch.bfloat16))
        for _ in range(3):
            flush_l2(flush)
            A64.gemv("N", 1.0, gb, 0.0, y64)
            flush_l2(flush)
            A32.gemv("N", 1.0, xs32, 0.0, y32)
            flush_l2(flush)
            Ab.gemv("N", 1.0, xs32, 0.0, y32)
            flush_l2(flush)
            M64.apply(gb, y64)
            flush_l2(flush)
            M32.apply(xs32, y32)
        torch.cuda.synchronize()
        print(json.dumps({"kernels_only": True, "n": n, "nnz": nnz}))
        return

    def timed(fn, steps, warm):
        for _ in range(warm):
            flush_l2(flush)
            fn()
        ms, infos = [], []
        for _ in range(steps):
            flush_l2(flush)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            infos.append(fn())
            e1.record(stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        return ms, infos

    x = torch.zeros(n, dtype=torch.float64, device=dev)

    def solve64():
        x.zero_()
        return E.solve_cg_info(eng, A64, M64, gb, x, tol)

    def solve_mixed():
        x.zero_()
        return E.solve_ru_pcg(eng, A64, A32, M32, gb, x, tol, delta=RU_DELTA)

    def solve_ir():
        x.zero_()
        return E.solve_ir_pcg(eng, A64, A32, M32, gb, x, tol, inner_rtol=IR_INNER_RTOL)

    clocks = ClockSampler(torch.cuda.current_device())
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    ms64, inf64 = timed(solve64, args.steps, args.warmup)
    x64 = x.clone()
    msmx, infmx = timed(solve_mixed, args.steps, args.warmup)
    xmx = x.clone()
    msir, infir = timed(solve_ir, args.steps, args.warmup)
    torch.cuda.synchronize()

    # ---- kernel timing for the roofline (same stream, CUDA events, L2 flushed per launch)
    def kernel_ms(fn, reps=10):
        out = []
        for _ in range(reps):
            flush_l2(flush)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            e1.synchronize()
            out.append(e0.elapsed_time(e1))
        return statistics.median(out)

    y64 = torch.empty(n, dtype=torch.float64, device=dev)
    y32 = torch.empty(n, dtype=torch.float32, device=dev)
    xs32 = gb.float()
    gvb = gv.to(torch.bfloat16)
    Ab = E.make_sparse_matrix(eng, n, gp, gi, gvb)
    # SpMV: 20 launches back to back per timing (the FP64 and FP32 matrices, 217 / 142 MB, exceed the
    # 129 MB L2, so each launch streams from HBM; a single launch would also time the launch gap).
    # The BF16 matrix (112 MB) fits in L2: one launch after a flush.
    def spmv_ms(fn, batch=20, reps=5):
        out = []
        for _ in range(reps):
            flush_l2(flush)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(batch):
                fn()
            e1.record(stream)
            e1.synchronize()
            out.append(e0.elapsed_time(e1) / batch)
        return statistics.median(out)

    t_spmv64 = spmv_ms(lambda: A64.gemv("N", 1.0, gb, 0.0, y64))
    t_spmv32 = spmv_ms(lambda: A32.gemv("N", 1.0, xs32, 0.0, y32))
    t_spmvbf = kernel_ms(lambda: Ab.gemv("N", 1.0, xs32, 0.0, y32))
    t_ilu64 = kernel_ms(lambda: M64.apply(gb, y64))
    t_ilu32 = kernel_ms(lambda: M32.apply(xs32, y32))
    clk = clocks.stop()

    # ---- end to end through the host-buffer entry points (pinned host memory)
    pin = lambda a: torch.from_numpy(a).pin_memory().numpy()  # noqa: E731
    hp, hi, hv, hb_ = pin(p), pin(i), pin(v), pin(b)
    hx = torch.zeros(n, dtype=torch.float64).pin_memory().numpy()
    e2e_ms = []
    for k in range(args.warmup + args.steps):
        hx[:] = 0.0
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        E.solve_ru_pcg_mixed(eng, tol, hp, hi, hv, M32, hb_, hx, delta=RU_DELTA)
        if k >= args.warmup:
            e2e_ms.append((time.perf_counter() - t0) * 1e3)
    h2d = 4 * (n + 1) + 4 * nnz + 8 * nnz + 8 * n + 8 * n
    d2h = 8 * n
    e2e_err = float(np.linalg.norm(b - __import__("hala_gb300.problems", fromlist=["x"]).csr_matvec(p, i, v, hx))
                    / np.linalg.norm(b))

    # ---- aggregate (replicas): solves of all ranks / max time
    t_mx = statistics.mean(msmx)
    t_64 = statistics.mean(ms64)
    t_e2e = statistics.mean(e2e_ms)
    t_ir = statistics.mean(msir)
    if world > 1:
        t_mx, t_64, t_e2e, t_ir = max_over_ranks([t_mx, t_64, t_e2e, t_ir], dev)
    if rank != 0:
        dist.destroy_process_group()
        return

    peak, peak_src = peaks()
    vb64 = spmv_bytes(n, nnz, 8, 8)
    ib64 = ilu_apply_bytes(n, nnz, 8, 8)
    ib32 = ilu_apply_bytes(n, nnz, 4, 4) + 8 * n    # + FP64 pivots
    xs = x64.cpu().numpy()
    xm = xmx.cpu().numpy()
    from hala_gb300 import problems as P
    res64 = float(np.linalg.norm(b - P.csr_matvec(p, i, v, xs)) / np.linalg.norm(b))
    resmx = float(np.linalg.norm(b - P.csr_matvec(p, i, v, xm)) / np.linalg.norm(b))
    it64 = inf64[-1].iterations
    launches = (sum(int(q.kernel_launches) for q in inf64) + sum(int(q.kernel_launches) for q in infmx)
                + sum(int(q.kernel_launches) for q in infir))
    launches += 2 * 20 * 5 + 10 + 4 * 10   # kernel timing: 2 x 100 SpMV, 10 BF16 SpMV, 2 x 10 ILU applies (2 launches each)
    # dominant kernel of the headline (mixed) solve: the FP32-store triangular sweeps (ILU apply)
    ach_ilu = ib32 / (t_ilu32 * 1e-3) / 1e9
    prof = {}
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            prof = json.load(f)
    except Exception:
        pass
    roof = {"bound": "hbm", "kernel": "bsolve_kernel x2 (ILU(0) apply of the FP32 store: forward + backward "
                                      "sweep; latency-bound wavefront, see ilu_apply)",
            "achieved": ach_ilu, "peak": peak, "unit": "GB/s", "frac": ach_ilu / peak,
            "traffic": prof.get("ilu_apply_f32_bytes"), "peak_source": peak_src,
            "algorithmic_bytes": ib32, "ms_per_launch": t_ilu32 / 2, "ms_per_apply": t_ilu32}
    spmv = {"kernel": "spmv_warp_kernel", "f64": {"ms": t_spmv64, "gbs": vb64 / (t_spmv64 * 1e-3) / 1e9,
                                               "frac": vb64 / (t_spmv64 * 1e-3) / 1e9 / peak, "bytes": vb64,
                                               "traffic": prof.get("spmv_f64_bytes")},
            "f32": {"ms": t_spmv32, "gbs": spmv_bytes(n, nnz, 4, 4) / (t_spmv32 * 1e-3) / 1e9,
                    "frac": spmv_bytes(n, nnz, 4, 4) / (t_spmv32 * 1e-3) / 1e9 / peak,
                    "bytes": spmv_bytes(n, nnz, 4, 4), "traffic": prof.get("spmv_f32_bytes")},
            "bf16f32": {"ms": t_spmvbf, "gbs": spmv_bytes(n, nnz, 2, 4) / (t_spmvbf * 1e-3) / 1e9,
                        "bytes": spmv_bytes(n, nnz, 2, 4)},
            "peak": peak, "unit": "GB/s",
            "timing": "f64/f32: 20 launches back to back (matrix > L2), median of 5; bf16: one launch after an L2 flush"}
    cpu = None
    if not args.no_cpu_baseline and world == 1:
        try:
            cpu = cpu_sample(p, i, v, b, it64)
        except Exception as e:  # report, do not hide
            cpu = {"value": None, "error": str(e)}
    out = {
        "metric": METRIC, "value": aggregate_rate(world, t_mx), "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_mx, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 inner / f64 refinement", "data": "synthetic",
        "config": {"workload": f"ILU(0)-PCG, 3D 7-point anisotropic {GRID}^3 coef (1,1,0.01), b = A x_true "
                               f"(x_true ~ N(0,1), seed {SEED}), x0 = 0, ||b-Ax|| < 1e-10 ||b||",
                   "n": n, "nnz": nnz, "form": "mixed: FP32 values/vectors/ILU (FP64 pivots) PCG, FP64 "
                                               f"refinement by reliable updates (delta {RU_DELTA})",
                   "l2": "flushed between timed solves (256 MB write); matrix 217 MB > 129 MB L2",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "fp64": {"solves_per_s": aggregate_rate(world, t_64), "ms_per_solve": t_64, "iterations": it64,
                 "rel_residual": res64, "setup_ms": setup64 * 1e3},
        "mixed": {"solves_per_s": aggregate_rate(world, t_mx), "ms_per_solve": t_mx, "inner_iterations": infmx[-1].iterations,
                  "reliable_updates": infmx[-1].outer, "rel_residual": resmx,
                  "err_vs_fp64": float(np.linalg.norm(xm - xs) / np.linalg.norm(xs)),
                  "err_vs_xtrue": float(np.linalg.norm(xm - xt) / np.linalg.norm(xt)), "setup_ms": setup32 * 1e3},
        "mixed_over_fp64": t_64 / t_mx,
        "mixed_restarted_ir": {"solves_per_s": aggregate_rate(world, t_ir),
                               "ms_per_solve": t_ir, "inner_iterations": infir[-1].iterations,
                               "sweeps": infir[-1].outer, "inner_rtol": IR_INNER_RTOL},
        "roofline": roof, "spmv": spmv,
        "ilu_apply": {"f64": {"ms": t_ilu64, "gbs": ib64 / (t_ilu64 * 1e-3) / 1e9, "bytes": ib64,
                              "traffic": prof.get("ilu_apply_f64_bytes")},
                      "f32": {"ms": t_ilu32, "gbs": ib32 / (t_ilu32 * 1e-3) / 1e9, "bytes": ib32,
                              "traffic": prof.get("ilu_apply_f32_bytes")}},
        "e2e": {"value": aggregate_rate(world, t_e2e), "unit": "solves/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "entry": "hgb_mixed_ru_pcg_solve (host pntr/indx/vals/b/x)",
                "rel_residual": e2e_err},
        "gpu_launches": launches,
        "cpu_baseline": cpu,
        "clocks": clk,
    }
    print(json.dumps(out), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
