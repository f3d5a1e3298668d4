"""Builds and runs the cuSPARSE/cuBLAS restatement of the reference's GPU path and prints its JSON
line: ILU(0)-PCG on the 128^3 anisotropic workload of bench.py (same matrix and right-hand side), or
with --gmres ILU(0)-GMRES(30) on the 96^3 convection-diffusion operator (b ~ U[-1,1], seed 3).
    python baseline/cusparse/run.py [--grid G] [--gmres]"""
import argparse
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--grid", type=int, default=None)
    ap.add_argument("--gmres", action="store_true")
    args = ap.parse_args()
    if args.gmres:
        from hala_gb300 import problems as P
        p, i, v = P.convdiff3d(args.grid or 96)
        b = np.random.default_rng(3).uniform(-1, 1, len(p) - 1)
    else:
        import bench
        bench.GRID = args.grid or 128
        p, i, v, xt, b = bench.workload()
    exe = os.path.join(tempfile.gettempdir(), "hgb_cusparse_pcg")
    subprocess.run(["nvcc", "-O3", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a", "-Xcompiler",
                    "-Wno-deprecated-declarations", os.path.join(HERE, "cusparse_pcg.cu"),
                    "-o", exe, "-lcusparse", "-lcublas"], check=True)
    with tempfile.TemporaryDirectory() as d:
        np.array([len(p) - 1], np.int32).tofile(os.path.join(d, "n.i32"))
        p.astype(np.int32).tofile(os.path.join(d, "pntr.i32"))
        i.astype(np.int32).tofile(os.path.join(d, "indx.i32"))
        v.astype(np.float64).tofile(os.path.join(d, "vals.f64"))
        b.astype(np.float64).tofile(os.path.join(d, "b.f64"))
        r = subprocess.run([exe, d] + (["gmres"] if args.gmres else []), capture_output=True, text=True)
        sys.stdout.write(r.stdout)
        sys.stderr.write(r.stderr)
        sys.exit(r.returncode)


if __name__ == "__main__":
    main()
