"""The C++ host mirror of the reference's solver plugin surface (solver,
solver_registry, microenvironment) and the gb300_solver plugin, exercised by a C++
test program that reads like the reference's gtests (tests/cpp/test_host_mirror.cpp).
The registry and mesh tests need no GPU; the plugin tests run on the GPU."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BUILD = os.path.join(ROOT, "tests", "_build")
EXE = os.path.join(BUILD, "test_host_mirror")


@pytest.fixture(scope="module")
def host_test_exe(pcg):
    from physicore_gb300 import _build
    host_lib = _build.build_host()
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(ROOT, "tests", "cpp", "test_host_mirror.cpp")
    pkg = os.path.dirname(host_lib)
    subprocess.run([_build.cxx(), "-std=c++20", "-O2", "-Wall", "-Wextra", src, "-I", os.path.join(ROOT, "include"),
                    "-L", pkg, "-lphysicore_gb300_host", "-lphysicore_gb300", f"-Wl,-rpath,{pkg}", "-o", EXE],
                   check=True)
    return EXE


def _run(exe, *args):
    r = subprocess.run([exe, *args], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


def test_registry_and_mesh(host_test_exe):
    out = _run(host_test_exe, "--cpu")
    assert "3 tests, 0 failures" in out


@pytest.mark.gpu
def test_gb300_solver_plugin(host_test_exe):
    out = _run(host_test_exe)
    assert "7 tests, 0 failures" in out, out
