"""Builds and runs the cuSPARSE/cuBLAS restatement of the reference's GPU ILU(0)-PCG path on the
128^3 anisotropic workload of bench.py (same matrix and right-hand side) and prints its JSON line.
    python baseline/cusparse/run.py [--grid G]"""
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
    ap.add_argument("--grid", type=int, default=128)
    args = ap.parse_args()
    import bench
    bench.GRID = args.grid
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
        r = subprocess.run([exe, d], capture_output=True, text=True)
        sys.stdout.write(r.stdout)
        sys.stderr.write(r.stderr)
        sys.exit(r.returncode)


if __name__ == "__main__":
    main()
