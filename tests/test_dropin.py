"""The drop-in: the reference's own solver templates (hex/solvers/*.hpp, unmodified, with its common/
blas/ sparse/ wax/ layers) compile and link over include/hala_gb/gpu/hala_gpu.hpp in place of the
reference's gpu/ directory, instantiating solve_cg_ilu, solve_cg, solve_gmres_ilu and
solve_batch_cg_ilu on hala::gpu_engine and hala::mixed_engine with every product, ILU, triangular
solve and vector operation resolved to libhgb.  Needs the reference's headers (directory
HALA_REFERENCE, default /root/reference); skipped where they are absent, which includes every GPU
machine (tests/cpp/dropin_solvers.cpp also runs the reference's solver cases when executed on one)."""
import os
import subprocess

import pytest

from hala_gb300 import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("HALA_REFERENCE", "/root/reference")
SRC = os.path.join(ROOT, "tests", "cpp", "dropin_solvers.cpp")
OUT = os.path.join(ROOT, "hala_gb300", "_lib")


def reference_includes(ref):
    dirs = ["common", "blas", "sparse", "lapack", "hex/solvers", "hex/vex", "wax", "hex/cholmod"]
    # the backend directory replaces the reference's gpu/ (which is not on the path)
    return (["-I" + os.path.join(ROOT, "oracle", "ref")] + ["-I" + os.path.join(ref, d) for d in dirs]
            + ["-I" + os.path.join(ROOT, "include", "hala_gb", "gpu"), "-I" + os.path.join(ROOT, "include"),
               "-I/usr/local/cuda/include"])


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "hex", "solvers")), reason="reference headers not present")
def test_reference_solver_templates_build_over_the_backend():
    build.build()
    obj = os.path.join(OUT, "dropin_solvers.o")
    shim = os.path.join(OUT, "blas_shim.o")
    exe = os.path.join(OUT, "dropin_solvers")
    cmd = ["g++", "-std=c++17", "-O1", "-DHALA_ENABLE_GPU", "-DHALA_ENABLE_CUDA", "-Wall", "-Wno-unused-variable",
           *reference_includes(REF), "-c", SRC, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    # host-side Givens rotations and the cpu_engine comparison use Fortran BLAS: the oracle's shim
    r = subprocess.run(["gcc", "-std=c11", "-O2", "-c", os.path.join(ROOT, "oracle", "ref", "blas_shim.c"), "-o", shim],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run(["g++", "-o", exe, obj, shim, "-L" + OUT, "-lhgb", "-L/usr/local/cuda/lib64", "-lcudart",
                        "-Wl,-rpath," + OUT], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    # every libhgb entry the templates resolved to is an hgb_* symbol of the library
    nm = subprocess.run(["nm", "-u", exe], capture_output=True, text=True).stdout
    used = sorted({ln.split()[-1] for ln in nm.splitlines() if ln.split()[-1].startswith("hgb_")})
    for must in ("hgb_csr_gemv", "hgb_ilu0_create", "hgb_ilu0_apply", "hgb_dot_f64", "hgb_nrm2_f64", "hgb_axpy_f64",
                 "hgb_gemv_f64", "hgb_dgmm_f64", "hgb_csr_gemm", "hgb_ilu0_apply_nrhs"):
        assert must in used, (must, used)
    # and nothing of cuSPARSE or cuBLAS
    assert "cusparse" not in nm and "cublas" not in nm
