"""Builds tests/cpp/test_adaptor.cpp against the MGmol-shaped C++ surface
(mgmol_gb300/cpp/mgmol_adaptor.h) and runs it on the GPU."""
import os
import subprocess

import pytest

from mgmol_gb300 import capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA = "/usr/local/cuda"


def build_adaptor_test():
    capi.load()
    out = os.path.join(ROOT, "mgmol_gb300", "_build", "test_adaptor")
    os.makedirs(os.path.dirname(out), exist_ok=True)
    libdir = os.path.join(ROOT, "mgmol_gb300")
    cmd = ["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "mgmol_gb300", "cpp"),
           "-I", os.path.join(CUDA, "include"), os.path.join(ROOT, "tests", "cpp", "test_adaptor.cpp"),
           "-o", out, "-L", libdir, "-lmgx", f"-Wl,-rpath,{libdir}", "-L", os.path.join(CUDA, "lib64"),
           "-lcudart", f"-Wl,-rpath,{os.path.join(CUDA, 'lib64')}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return out


def test_adaptor_compiles():
    assert os.path.exists(build_adaptor_test())


@pytest.mark.gpu
def test_reference_unit_tests_through_the_adaptor():
    exe = build_adaptor_test()
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.count("ok ") == 8
