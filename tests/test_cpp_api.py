"""The C++ mirror of MAST's API (mast-multiphysics_gb300/mast_api/mast_api.hpp),
exercised by C++ tests written like MAST's own (tests/cpp/test_mast_api.cpp):
[cpu] cases run anywhere, [gpu] cases drive the CUDA path through the mirror."""
import os
import subprocess

import pytest

import mastgpu as M
import oracle as O

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
OUT = os.path.join(REPO, "tests", "cpp", "_build")


def build_cpp_tests():
    M.build()
    O.build()
    os.makedirs(OUT, exist_ok=True)
    exe = os.path.join(OUT, "test_mast_api")
    lib_dir = os.path.dirname(M.LIB_PATH)
    oracle_dir = os.path.dirname(O.LIB_PATH)
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Wno-unused-function",
           "-I", os.path.join(REPO, "include"),
           "-I", os.path.join(REPO, "mast-multiphysics_gb300", "mast_api"),
           "-I", os.path.join(REPO, "oracle"),
           os.path.join(REPO, "tests", "cpp", "test_mast_api.cpp"), "-o", exe,
           "-L", lib_dir, "-L", oracle_dir, "-lmastgpu", "-lmastoracle",
           "-Wl,-rpath," + lib_dir, "-Wl,-rpath," + oracle_dir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def run(tag):
    exe = build_cpp_tests()
    r = subprocess.run([exe, tag], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert " 0 failed" in r.stdout
    return r.stdout


def test_cpp_mirror_cpu_cases():
    out = run("[cpu]")
    assert "9 test cases" in out


@pytest.mark.gpu
def test_cpp_mirror_gpu_cases():
    out = run("[gpu]")
    assert "6 test cases" in out
