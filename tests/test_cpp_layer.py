"""The C++ host layer (include/hala_gb/hala_gb.hpp) compiles against the C ABI; on a GPU the
reference's own test cases, written against it, pass."""
import os
import subprocess

import pytest

from hala_gb300 import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "hala_gb_cases.cpp")
EXE = os.path.join(ROOT, "hala_gb300", "_lib", "hala_gb_cases")


def compile_cases():
    build.build()
    cmd = ["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"), "-I/usr/local/cuda/include", SRC,
           "-o", EXE, "-L" + os.path.dirname(build.LIB), "-lhgb", "-L/usr/local/cuda/lib64", "-lcudart",
           "-Wl,-rpath," + os.path.dirname(build.LIB), "-Wl,-rpath,/usr/local/cuda/lib64"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_cpp_layer_compiles():
    compile_cases()


@pytest.mark.gpu
def test_cpp_layer_reference_cases():
    compile_cases()
    r = subprocess.run([EXE], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ALL PASS" in r.stdout
