"""The C++ facade with the reference's interface (include/ie_solver_gb300.hpp),
driven by tests/cpp/facade_test.cpp the way the reference's own test drives
its solver (ie_solver_test.cpp:29-96): backward error <= 50 tol against the
dense operator assembled through the facade's Kernel, U and Psi.

On CPU the program runs its host-only checks (tree construction and mirror,
ie_Mat arithmetic, RS_ERR_NO_DEVICE from a factorization without a GPU).
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_DIR = os.path.join(ROOT, "ie-solver_gb300", "lib")


def _build(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    if not os.path.exists(os.path.join(LIB_DIR, "librskel.so")):
        pytest.fail("librskel.so is missing: run __graft_entry__.build()")
    exe = str(tmp_path / "facade_test")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "facade_test.cpp"), "-L", LIB_DIR, "-lrskel",
           f"-Wl,-rpath,{LIB_DIR}", "-o", exe]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    return exe


def test_facade_host_checks(tmp_path):
    exe = _build(tmp_path)
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    res = subprocess.run([exe, "--host"], capture_output=True, text=True, env=env, timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr


@pytest.mark.gpu
def test_facade_solves_like_the_reference_test(tmp_path):
    exe = _build(tmp_path)
    res = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    print(res.stdout)
    assert res.returncode == 0, res.stdout + res.stderr
    assert "all passed" in res.stdout
