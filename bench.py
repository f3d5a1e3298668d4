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
WORKLOAD = ("ILU(0)-PCG, 3D 7-point anisotropic {grid}^3 coef (1,1,0.01), b = A x_true (x_true ~ N(0,1), "
            "seed 2), x0 = 0, ||b-Ax|| < 1e-10 ||b||")


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


def cpu_sample(p, i, v, b):
    """FP64 ILU(0)-PCG of the oracle (the reference's algorithm, serial) on the host cores: one
    complete solve to the 1e-10 relative residual from x0 = 0 (ILU factor excluded)."""
    from oracle import oracle as O
    tol = RTOL * float(np.linalg.norm(b))
    f, d, _ = O.ilu_factor(p, i, v)
    t0 = time.perf_counter()
    _, it, _ = O.cg(p, i, v, b, tol=tol, diag=d, ilu=f)
    dt = time.perf_counter() - t0
    return {"value": 1.0 / dt, "unit": "solves/s", "cores": 1, "kind": "port",
            "sample": f"one complete FP64 ILU(0)-PCG solve of the {GRID}^3 system ({it} iterations, {dt:.1f} s), "
                      "serial as the reference's sparse path; ILU factor excluded"}


def run_reference(args, rank, world):
    """Reference arm: the reference's CPU algorithm for the path (the oracle port: the reference's
    own sources are not on this machine), FP64 ILU(0)-PCG, timed on the host cores.  Every step is
    one complete solve to the 1e-10 relative residual from x0 = 0; the ILU factor is computed once,
    outside the timed steps (the reference's own factorisation is O(n^2): about 37 min here)."""
    if rank != 0:
        return
    from oracle import oracle as O
    p, i, v, xt, b = workload()
    n = len(p) - 1
    tol = RTOL * float(np.linalg.norm(b))
    f, d, _ = O.ilu_factor(p, i, v)
    for _ in range(args.warmup):
        O.cg(p, i, v, b, tol=tol, diag=d, ilu=f)
    times, its = [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        x, it, _ = O.cg(p, i, v, b, tol=tol, diag=d, ilu=f)
        times.append(time.perf_counter() - t0)
        its.append(it)
    per = statistics.mean(times)
    val = 1.0 / per
    res = float(np.linalg.norm(b - __import__("hala_gb300.problems", fromlist=["x"]).csr_matvec(p, i, v, x))
                / np.linalg.norm(b))
    sample = (f"{args.steps} complete FP64 ILU(0)-PCG solves ({its[-1]} iterations each, rel. residual "
              f"{res:.2e}) after {args.warmup} untimed ones; serial, as the reference's sparse path")
    print(json.dumps({
        "metric": METRIC, "value": val, "unit": "solves/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": per * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
        "config": {"workload": WORKLOAD.format(grid=GRID), "n": n, "nnz": int(len(i))},
        "cpu_baseline": {"value": val, "unit": "solves/s", "cores": 1, "kind": "port", "sample": sample},
        "e2e": {"value": val, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def _events_ms(stream, fn, steps, warm, flush=None):
    """Median CUDA-event time of fn on stream (after warm untimed calls); returns (ms, last result)."""
    import torch
    for _ in range(warm):
        if flush is not None:
            flush_l2(flush)
        fn()
    out, res = [], None
    for _ in range(steps):
        if flush is not None:
            flush_l2(flush)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        res = fn()
        e1.record(stream)
        e1.synchronize()
        out.append(e0.elapsed_time(e1))
    return statistics.median(out), res


def other_workloads(E, eng, dev, stream, flush, peak, steps=3, warm=2):
    """The path's other workloads, timed on the device (CUDA events, setup excluded): CG on the 256^2
    Poisson system, ILU(0)-GMRES(30) on the 96^3 convection-diffusion operator (FP64 and mixed),
    the 4,096 independent systems in one persistent launch, and the 512^2 differentiable solve
    (forward and adjoint).  Each entry reports its time, iterations and residual."""
    import torch
    from hala_gb300 import problems as P
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)   # noqa: E731
    out = {}
    launches = 0

    # 256^2 2D Poisson, unpreconditioned CG to 1e-10 (5 MB of matrix: L2-resident, not flushed)
    p, i, v = P.poisson2d(256)
    n = len(p) - 1
    b = P.csr_matvec(p, i, v, np.random.default_rng(1).uniform(-1, 1, n))
    tol = 1e-10 * float(np.linalg.norm(b))
    A = E.make_sparse_matrix(eng, n, T(p), T(i), T(v))
    gb, x = T(b), torch.zeros(n, dtype=torch.float64, device=dev)

    def cg():
        x.zero_()
        return E.solve_cg_info(eng, A, None, gb, x, tol)
    ms, info = _events_ms(stream, cg, steps, warm)
    launches += (steps + warm) * int(info.kernel_launches)
    res = float(np.linalg.norm(b - P.csr_matvec(p, i, v, x.cpu().numpy())) / np.linalg.norm(b))
    out["cg_poisson256"] = {"ms_per_solve": ms, "iterations": info.iterations, "rel_residual": res,
                            "us_per_iteration": 1e3 * ms / max(info.iterations, 1), "n": n, "nnz": len(i),
                            "l2": "not flushed (5 MB system)"}

    # 96^3 convection-diffusion, ILU(0)-GMRES(30): FP64 to 1e-9 of ||P^-1 b|| (the reference's test on
    # the preconditioned residual), and mixed FP32-inner GMRES with FP64 refinement to a 1e-9 true residual
    p, i, v = P.convdiff3d(96)
    n = len(p) - 1
    b = np.random.default_rng(3).uniform(-1, 1, n)
    gp, gi, gv, gb = T(p), T(i), T(v), T(b)
    A64 = E.make_sparse_matrix(eng, n, gp, gi, gv)
    M64 = E.make_ilu(eng, gp, gi, gv)
    pb = torch.empty(n, dtype=torch.float64, device=dev)
    M64.apply(gb, pb)
    ptol = 1e-9 * float(torch.linalg.vector_norm(pb))
    x = torch.zeros(n, dtype=torch.float64, device=dev)

    def gm64():
        x.zero_()
        return E.solve_gmres(eng, E.stop_criteria(ptol), 30, gp, gi, gv, gb, x, ilu=M64, matrix=A64)
    ms64, apps = _events_ms(stream, gm64, steps, warm, flush)
    r64 = float(np.linalg.norm(b - P.csr_matvec(p, i, v, x.cpu().numpy())) / np.linalg.norm(b))
    A32 = E.make_sparse_matrix(eng, n, gp, gi, gv.float())
    M32 = E.make_ilu(eng, gp, gi, gv, store=torch.float32)
    ttol = 1e-9 * float(np.linalg.norm(b))

    def gmmx():
        x.zero_()
        return E.solve_ir_gmres(eng, A64, A32, M32, 30, gb, x, ttol, inner_rtol=1e-4)
    msmx, infmx = _events_ms(stream, gmmx, steps, warm, flush)
    launches += (steps + warm) * int(infmx.kernel_launches)
    rmx = float(np.linalg.norm(b - P.csr_matvec(p, i, v, x.cpu().numpy())) / np.linalg.norm(b))
    out["gmres30_convdiff96"] = {
        "n": n, "nnz": len(i),
        "fp64": {"ms_per_solve": ms64, "applications": apps, "true_rel_residual": r64,
                 "stop": "preconditioned residual < 1e-9 ||P^-1 b||"},
        "mixed": {"ms_per_solve": msmx, "inner_iterations": infmx.iterations, "sweeps": infmx.outer,
                  "true_rel_residual": rmx, "stop": "||b - Ax|| < 1e-9 ||b||"}}
    del A64, M64, A32, M32

    # 4,096 independent Erdos-Renyi Laplacians (n_i log-uniform in [64, 4096]), FP32 CG with FP64
    # refinement to 1e-8 per system, one persistent launch replayed from a CUDA graph
    S = 4096
    sp_, p, i, v = P.er_laplacian_batch(S, 64, 4096, seed=4)
    nt = len(p) - 1
    b = np.random.default_rng(5).uniform(-1, 1, nt)
    B = E.gpu_batch(eng, T(sp_), T(p), T(i), T(v))
    gb = T(b)
    x = torch.zeros(nt, dtype=torch.float64, device=dev)
    iters = torch.zeros(S, dtype=torch.int32, device=dev)
    rel = torch.zeros(S, dtype=torch.float64, device=dev)

    # launch shape: timed on this batch before the measurement (setup, not in the timed region)
    shape = B.autotune(gb, x, 1e-8)

    def batch():
        x.zero_()
        return B.solve(gb, x, rtol=1e-8, iters=iters, relres=rel)
    msb, _ = _events_ms(stream, batch, steps, warm, flush)
    launches += 2 * (steps + warm)
    it = iters.cpu().numpy().astype(np.int64)
    ni = np.diff(sp_).astype(np.int64)
    nnz_i = (p[sp_[1:]] - p[sp_[:-1]]).astype(np.int64)
    # algorithmic bytes: every inner iteration streams its system's matrix (FP32 values, int32
    # columns and row pointers) and touches x and b once per system in FP64
    mat_bytes = float(np.sum(it * (8 * nnz_i + 4 * (ni + 1)))) + float(np.sum(16 * ni))
    gbs = mat_bytes / (msb * 1e-3) / 1e9
    out["batch_4096"] = {"ms_per_batch": msb, "systems_per_s": S * 1e3 / msb, "rows": nt, "nnz": len(i),
                         "launch_shape": {"block_threads": shape[0], "warp_max_n": shape[1]},
                         "max_rel_residual": float(rel.max()), "iterations_total": int(it.sum()),
                         "roofline": {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s",
                                      "frac": gbs / peak, "algorithmic_bytes": mat_bytes,
                                      "bytes": "sum over systems of inner iterations x (8 nnz_i + 4 (n_i + 1)) + 16 n_i"}}
    del B

    # 512^2 variable-coefficient diffusion: forward mixed ILU(0)-PCG (FP32 PCG, FP64 reliable updates)
    # to 3e-11 and the adjoint solve A^T lam = 2 (u - u_target) with dL/dA on the pattern
    nn = 512
    k1, k2 = np.exp(P.grf2d(nn, 16.0, 1.0, seed=1)), np.exp(P.grf2d(nn, 16.0, 1.0, seed=2))
    p, i, v = P.vardiff2d(nn, k1)
    v2 = P.vardiff2d(nn, k2)[2]
    n = len(p) - 1
    gp, gi = T(p), T(i)
    f = torch.ones(n, dtype=torch.float64, device=dev)
    tol = 3e-11 * float(torch.linalg.vector_norm(f))

    def ops(vals):
        gv = T(vals)
        return (E.make_sparse_matrix(eng, n, gp, gi, gv), E.make_sparse_matrix(eng, n, gp, gi, gv.float()),
                E.make_ilu(eng, gp, gi, gv, store=torch.float32), gv)
    A64, A32, M32, gv = ops(v)
    ut = torch.zeros(n, dtype=torch.float64, device=dev)
    t2 = ops(v2)
    E.solve_ru_pcg(eng, t2[0], t2[1], t2[2], f, ut, tol, delta=0.01, max_iter=20000)
    del t2
    u = torch.zeros(n, dtype=torch.float64, device=dev)
    lam = torch.zeros(n, dtype=torch.float64, device=dev)
    gvals = torch.empty_like(gv)
    fw = {}

    def forward_adjoint():
        u.zero_()
        lam.zero_()
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record(stream)
        fi = E.solve_ru_pcg(eng, A64, A32, M32, f, u, tol, delta=0.01, max_iter=20000)
        e1.record(stream)
        g = 2.0 * (u - ut)
        ai = E.solve_ru_pcg_op(eng, A64, A32, M32, "T", g, lam, 3e-11 * float(torch.linalg.vector_norm(g)),
                               delta=0.01, max_iter=20000)
        E.pattern_grad(A64, -1.0, lam, u, gvals)
        e2.record(stream)
        e2.synchronize()
        fw.setdefault("fwd", []).append(e0.elapsed_time(e1))
        fw.setdefault("adj", []).append(e1.elapsed_time(e2))
        return fi, ai
    msfa, (fi, ai) = _events_ms(stream, forward_adjoint, 2, 1)
    launches += 3 * (int(fi.kernel_launches) + int(ai.kernel_launches))
    # the same forward solve in plain FP64 (ILU(0)-PCG, FP64 factor), for the mixed-vs-FP64 comparison
    M64 = E.make_ilu(eng, gp, gi, gv)

    def forward64():
        u.zero_()
        return E.solve_cg_info(eng, A64, M64, f, u, tol, max_iter=20000)
    ms64f, fi64 = _events_ms(stream, forward64, 2, 1)
    launches += 3 * int(fi64.kernel_launches)
    del M64
    res = float(np.linalg.norm(1.0 - P.csr_matvec(p, i, v, u.cpu().numpy())) / np.sqrt(n))
    out["adjoint_vardiff512"] = {"ms_forward_fp64_pcg": ms64f, "forward_fp64_iterations": fi64.iterations,
                                 "ms_forward_plus_adjoint": msfa, "ms_forward": statistics.median(fw["fwd"][1:]),
                                 "ms_adjoint": statistics.median(fw["adj"][1:]), "forward_iterations": fi.iterations,
                                 "adjoint_iterations": ai.iterations, "forward_rel_residual": res, "n": n,
                                 "loss": float(torch.sum((u - ut) ** 2))}

    # 128^3 SpMM over 4 right-hand sides (sparse_gemm): one pass over the matrix against the four
    # single-column products; algorithmic bytes = the matrix once + the columns of X and Y
    p, i, v = P.aniso3d(GRID, coef=COEF)
    n, k = len(p) - 1, 4
    gp, gi, gv = T(p), T(i), T(v)
    mm = {"nrhs": k, "n": n, "nnz": len(i), "l2": "flushed before each product"}
    for name, vdt in (("f64", torch.float64), ("f32", torch.float32)):
        A = E.make_sparse_matrix(eng, n, gp, gi, gv.to(vdt))
        X = torch.randn(n * k, dtype=vdt, device=dev)
        Y = torch.empty_like(X)
        t1, _ = _events_ms(stream, lambda: A.gemm(k, 1.0, X, 0.0, Y), 5, 2, flush)

        def cols():
            for c in range(k):
                A.gemv("N", 1.0, X[c * n:(c + 1) * n], 0.0, Y[c * n:(c + 1) * n])
        t2, _ = _events_ms(stream, cols, 5, 2, flush)
        launches += 7 * (1 + k)
        vb = 8 if vdt == torch.float64 else 4
        byts = (vb + 4) * len(i) + 4 * (n + 1) + 2 * k * vb * n
        mm[name] = {"ms_one_pass": t1, "ms_column_by_column": t2, "gbs": byts / (t1 * 1e-3) / 1e9,
                    "frac": byts / (t1 * 1e-3) / 1e9 / peak, "algorithmic_bytes": byts}
        del A
    out["spmm_aniso128_4rhs"] = mm
    return out, launches


LIBRARY_EXE = os.path.join(ROOT, "baseline", "cusparse", "_build", "cusparse_pcg")


def library_baseline(p, i, v, b, tmpdir, gmres=False):
    """The reference's GPU path (cuSPARSE SpMV / csrilu02 / SpSV and cuBLAS BLAS-1 in host pointer
    mode, the loop of solve_cg_core, or with gmres=True the GMRES(30) of solve_gmres with its
    per-iteration host read-back) restated in baseline/cusparse and built by the package build, run
    on the given system outside this arm's timed region.  Returns its JSON line, or why it did not run."""
    exe = LIBRARY_EXE
    if not os.path.exists(exe):
        return {"unavailable": "baseline/cusparse was not built (nvcc or cuSPARSE missing at build time)"}
    n = len(p) - 1
    np.array([n], np.int32).tofile(os.path.join(tmpdir, "n.i32"))
    p.astype(np.int32).tofile(os.path.join(tmpdir, "pntr.i32"))
    i.astype(np.int32).tofile(os.path.join(tmpdir, "indx.i32"))
    v.astype(np.float64).tofile(os.path.join(tmpdir, "vals.f64"))
    b.astype(np.float64).tofile(os.path.join(tmpdir, "b.f64"))
    r = subprocess.run([exe, tmpdir] + (["gmres"] if gmres else []), capture_output=True, text=True, timeout=600)
    if r.returncode != 0:
        return {"unavailable": f"cusparse_pcg exited {r.returncode}: {r.stderr.strip()[-300:]}"}
    return json.loads(r.stdout.strip().splitlines()[-1])


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
                    help="only the SpMV, ILU-apply and SpMM launches (for profiling captures)")
    ap.add_argument("--no-other-workloads", action="store_true",
                    help="skip the other workloads and the library baseline (reported beside the headline)")
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
    M16 = E.make_ilu(eng, gp, gi, gv, store=torch.bfloat16)
    torch.cuda.synchronize()
    setup16 = time.perf_counter() - t0
    M32 = E.make_ilu(eng, gp, gi, gv, store=torch.float32)
    flush = torch.empty(32 * 1024 * 1024, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    if args.kernels_only:
        y64 = torch.empty(n, dtype=torch.float64, device=dev)
        y32 = torch.empty(n, dtype=torch.float32, device=dev)
        xs32 = gb.float()
        Ab = E.make_sparse_matrix(eng, n, gp, gi, gv.to(torch.bfloat16))
        X4 = torch.randn(4 * n, dtype=torch.float64, device=dev)
        Y4 = torch.empty_like(X4)
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
            flush_l2(flush)
            M16.apply(xs32, y32)
            flush_l2(flush)
            A64.gemm(4, 1.0, X4, 0.0, Y4)   # one-pass SpMM over 4 columns
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

    # the headline mixed form: FP32 operator and vectors, the ILU(0) factor stored in BF16 (FP64
    # pivots), FP64 reliable updates; the same with an FP32-stored factor beside it
    def solve_mixed():
        x.zero_()
        return E.solve_ru_pcg(eng, A64, A32, M16, gb, x, tol, delta=RU_DELTA)

    def solve_ir():
        x.zero_()
        return E.solve_ir_pcg(eng, A64, A32, M32, gb, x, tol, inner_rtol=IR_INNER_RTOL)

    def solve_mixed_f32_store():
        x.zero_()
        return E.solve_ru_pcg(eng, A64, A32, M32, gb, x, tol, delta=RU_DELTA)

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
    msbs, infbs = timed(solve_mixed_f32_store, args.steps, args.warmup)
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
    # two copies of the BF16 matrix (2 x 112 MB > the 129 MB L2), alternated launch by launch
    gvb = gv.to(torch.bfloat16)
    gp2, gi2, gvb2 = gp.clone(), gi.clone(), gvb.clone()
    Ab = [E.make_sparse_matrix(eng, n, gp, gi, gvb), E.make_sparse_matrix(eng, n, gp2, gi2, gvb2)]
    # SpMV: 20 launches back to back per timing (the FP64 and FP32 matrices, 217 / 142 MB, exceed the
    # 129 MB L2, so each launch streams from HBM; a single launch would also time the launch gap).
    def spmv_ms(fn, batch=20, reps=5):
        out = []
        for _ in range(reps):
            flush_l2(flush)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for k in range(batch):
                fn(k)
            e1.record(stream)
            e1.synchronize()
            out.append(e0.elapsed_time(e1) / batch)
        return statistics.median(out)

    t_spmv64 = spmv_ms(lambda k: A64.gemv("N", 1.0, gb, 0.0, y64))
    t_spmv32 = spmv_ms(lambda k: A32.gemv("N", 1.0, xs32, 0.0, y32))
    t_spmvbf = spmv_ms(lambda k: Ab[k & 1].gemv("N", 1.0, xs32, 0.0, y32))
    eng.set_spmv_mode("exact")      # the reference's rounding: separately rounded multiply and add
    t_spmv64x = spmv_ms(lambda k: A64.gemv("N", 1.0, gb, 0.0, y64))
    t_spmv32x = spmv_ms(lambda k: A32.gemv("N", 1.0, xs32, 0.0, y32))
    eng.set_spmv_mode("fused")
    t_ilu64 = kernel_ms(lambda: M64.apply(gb, y64))
    t_ilu32 = kernel_ms(lambda: M32.apply(xs32, y32))
    t_ilu16 = kernel_ms(lambda: M16.apply(xs32, y32))
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
        E.solve_ru_pcg_mixed(eng, tol, hp, hi, hv, M16, hb_, hx, delta=RU_DELTA)
        if k >= args.warmup:
            e2e_ms.append((time.perf_counter() - t0) * 1e3)
    h2d = 4 * (n + 1) + 4 * nnz + 8 * nnz + 8 * n + 8 * n
    d2h = 8 * n
    # the same from host buffers with the ILU(0) setup inside the step: make_ilu(mixed_engine, ...)
    # (host pattern and values; the copies overlap the host planning of the triangular schedules)
    # then the solve
    setup_ms, e2es_ms = [], []
    for k in range(args.warmup + args.steps):
        hx[:] = 0.0
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        Mh = E.make_ilu_host(eng, hp, hi, hv, store=torch.bfloat16)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        E.solve_ru_pcg_mixed(eng, tol, hp, hi, hv, Mh, hb_, hx, delta=RU_DELTA)
        if k >= args.warmup:
            setup_ms.append((t1 - t0) * 1e3)
            e2es_ms.append((time.perf_counter() - t0) * 1e3)
        del Mh
    e2e_err = float(np.linalg.norm(b - __import__("hala_gb300.problems", fromlist=["x"]).csr_matvec(p, i, v, hx))
                    / np.linalg.norm(b))

    # ---- the path's other workloads and the library baseline (outside the timed headline region)
    others, other_launches, lib = None, 0, None
    if not args.no_other_workloads:
        others, other_launches = other_workloads(E, eng, dev, stream, flush, peaks()[0])
        if rank == 0:
            import tempfile
            from hala_gb300 import problems as P
            lib = {}
            pc, ic, vc = P.convdiff3d(96)
            bc = np.random.default_rng(3).uniform(-1, 1, len(pc) - 1)
            for key, args_ in (("pcg_aniso128", (p, i, v, b, False)), ("gmres30_convdiff96", (pc, ic, vc, bc, True))):
                with tempfile.TemporaryDirectory() as tdir:
                    try:
                        lib[key] = library_baseline(*args_[:4], tdir, gmres=args_[4])
                    except Exception as e:  # report, do not hide
                        lib[key] = {"unavailable": f"library baseline failed: {e}"}

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
    ib16 = ilu_apply_bytes(n, nnz, 2, 4) + 8 * n
    xs = x64.cpu().numpy()
    xm = xmx.cpu().numpy()
    from hala_gb300 import problems as P
    res64 = float(np.linalg.norm(b - P.csr_matvec(p, i, v, xs)) / np.linalg.norm(b))
    resmx = float(np.linalg.norm(b - P.csr_matvec(p, i, v, xm)) / np.linalg.norm(b))
    it64 = inf64[-1].iterations
    launches = (sum(int(q.kernel_launches) for q in inf64) + sum(int(q.kernel_launches) for q in infmx)
                + sum(int(q.kernel_launches) for q in infir) + sum(int(q.kernel_launches) for q in infbs))
    launches += 5 * 20 * 5 + 6 * 10   # kernel timing: 5 x 100 SpMV, 3 x 10 ILU applies (2 launches each)
    # dominant kernel of the headline (mixed) solve: the BF16-store triangular sweeps (ILU apply)
    ach_ilu = ib16 / (t_ilu16 * 1e-3) / 1e9
    prof = {}
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            prof = json.load(f)
    except Exception:
        pass
    roof = {"bound": "hbm", "kernel": "bsolve_kernel x2 (ILU(0) apply of the BF16 store: forward + backward "
                                      "sweep; latency-bound wavefront, see ilu_apply)",
            "achieved": ach_ilu, "peak": peak, "unit": "GB/s", "frac": ach_ilu / peak,
            "traffic": prof.get("ilu_apply_bf16_bytes"), "peak_source": peak_src,
            "algorithmic_bytes": ib16, "ms_per_launch": t_ilu16 / 2, "ms_per_apply": t_ilu16}
    spmv = {"kernel": "spmv_warp_kernel", "f64": {"ms": t_spmv64, "gbs": vb64 / (t_spmv64 * 1e-3) / 1e9,
                                               "frac": vb64 / (t_spmv64 * 1e-3) / 1e9 / peak, "bytes": vb64,
                                               "traffic": prof.get("spmv_f64_bytes")},
            "f32": {"ms": t_spmv32, "gbs": spmv_bytes(n, nnz, 4, 4) / (t_spmv32 * 1e-3) / 1e9,
                    "frac": spmv_bytes(n, nnz, 4, 4) / (t_spmv32 * 1e-3) / 1e9 / peak,
                    "bytes": spmv_bytes(n, nnz, 4, 4), "traffic": prof.get("spmv_f32_bytes")},
            "bf16f32": {"ms": t_spmvbf, "gbs": spmv_bytes(n, nnz, 2, 4) / (t_spmvbf * 1e-3) / 1e9,
                        "frac": spmv_bytes(n, nnz, 2, 4) / (t_spmvbf * 1e-3) / 1e9 / peak,
                        "bytes": spmv_bytes(n, nnz, 2, 4), "traffic": prof.get("spmv_bf16_bytes")},
            "f64_exact": {"ms": t_spmv64x, "gbs": vb64 / (t_spmv64x * 1e-3) / 1e9,
                          "frac": vb64 / (t_spmv64x * 1e-3) / 1e9 / peak},
            "f32_exact": {"ms": t_spmv32x, "gbs": spmv_bytes(n, nnz, 4, 4) / (t_spmv32x * 1e-3) / 1e9,
                          "frac": spmv_bytes(n, nnz, 4, 4) / (t_spmv32x * 1e-3) / 1e9 / peak},
            "peak": peak, "unit": "GB/s",
            "mode": "f64/f32/bf16: fused multiply-add (the default, used by the solves); *_exact: separately "
                    "rounded multiply and add (bit-identical to the reference's CPU product)",
            "timing": "20 launches back to back, median of 5; f64/f32 matrices (217 / 142 MB) exceed the 129 MB L2, "
                      "bf16 alternates two copies of its 112 MB matrix"}
    cpu = None
    if not args.no_cpu_baseline and world == 1:
        try:
            cpu = cpu_sample(p, i, v, b)
        except Exception as e:  # report, do not hide
            cpu = {"value": None, "error": str(e)}
    out = {
        "metric": METRIC, "value": aggregate_rate(world, t_mx), "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_mx, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 inner (bf16 ILU factor) / f64 refinement",
        "data": "synthetic",
        "config": {"workload": WORKLOAD.format(grid=GRID),
                   "n": n, "nnz": nnz, "form": "mixed: PCG with FP32 matrix values and vectors and the "
                                               "ILU(0) factor stored in BF16 (FP64 pivots), FP64 refinement "
                                               f"by reliable updates (delta {RU_DELTA})",
                   "l2": "flushed between timed solves (256 MB write); matrix 217 MB > 129 MB L2",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "fp64": {"solves_per_s": aggregate_rate(world, t_64), "ms_per_solve": t_64, "iterations": it64,
                 "rel_residual": res64, "setup_ms": setup64 * 1e3},
        "mixed": {"solves_per_s": aggregate_rate(world, t_mx), "ms_per_solve": t_mx, "inner_iterations": infmx[-1].iterations,
                  "reliable_updates": infmx[-1].outer, "rel_residual": resmx,
                  "err_vs_fp64": float(np.linalg.norm(xm - xs) / np.linalg.norm(xs)),
                  "err_vs_xtrue": float(np.linalg.norm(xm - xt) / np.linalg.norm(xt)), "setup_ms": setup16 * 1e3},
        "mixed_over_fp64": t_64 / t_mx,
        "mixed_f32_store": {"solves_per_s": 1e3 / statistics.mean(msbs), "ms_per_solve": statistics.mean(msbs),
                            "inner_iterations": infbs[-1].iterations, "reliable_updates": infbs[-1].outer,
                            "form": "as mixed, the ILU(0) factor stored in FP32 (FP64 pivots)"},
        "mixed_restarted_ir": {"solves_per_s": aggregate_rate(world, t_ir),
                               "ms_per_solve": t_ir, "inner_iterations": infir[-1].iterations,
                               "sweeps": infir[-1].outer, "inner_rtol": IR_INNER_RTOL},
        "roofline": roof, "spmv": spmv,
        "ilu_apply": {"f64": {"ms": t_ilu64, "gbs": ib64 / (t_ilu64 * 1e-3) / 1e9, "bytes": ib64,
                              "traffic": prof.get("ilu_apply_f64_bytes")},
                      "f32": {"ms": t_ilu32, "gbs": ib32 / (t_ilu32 * 1e-3) / 1e9, "bytes": ib32,
                              "traffic": prof.get("ilu_apply_f32_bytes")},
                      "bf16": {"ms": t_ilu16, "gbs": ib16 / (t_ilu16 * 1e-3) / 1e9, "bytes": ib16,
                               "traffic": prof.get("ilu_apply_bf16_bytes")}},
        "e2e": {"value": aggregate_rate(world, t_e2e), "unit": "solves/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "entry": "hgb_mixed_ru_pcg_solve (host pntr/indx/vals/b/x)",
                "rel_residual": e2e_err,
                "with_setup": {"solves_per_s": 1e3 / statistics.mean(e2es_ms), "ms_per_step": statistics.mean(e2es_ms),
                               "ilu_setup_ms": statistics.mean(setup_ms),
                               "entries": "hgb_ilu0_create_host (BF16 store) + hgb_mixed_ru_pcg_solve, host buffers"}},
        "gpu_launches": launches,
        "other_workloads": others,
        "gpu_launches_other_workloads": other_launches,
        "library_baseline": lib,
        "cpu_baseline": cpu,
        "clocks": clk,
    }
    print(json.dumps(out), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
