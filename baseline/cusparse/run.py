"""Runs the cuSPARSE/cuBLAS restatement of the reference's GPU path (built by the package build into
baseline/cusparse/_build) and prints its JSON line: ILU(0)-PCG on the 128^3 anisotropic workload of
bench.py (same matrix and right-hand side), or with --gmres ILU(0)-GMRES(30) on the 96^3
convection-diffusion operator (b ~ U[-1,1], seed 3).  bench.py reports both beside its own line.
    python baseline/cusparse/run.py [--grid G] [--gmres]"""
import argparse
import json
import os
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
    import bench
    if args.gmres:
        from hala_gb300 import problems as P
        p, i, v = P.convdiff3d(args.grid or 96)
        b = np.random.default_rng(3).uniform(-1, 1, len(p) - 1)
    else:
        bench.GRID = args.grid or 128
        p, i, v, xt, b = bench.workload()
    with tempfile.TemporaryDirectory() as d:
        print(json.dumps(bench.library_baseline(p, i, v, b, d, gmres=args.gmres)))


if __name__ == "__main__":
    main()
