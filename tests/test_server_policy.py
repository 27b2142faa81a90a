"""The serving policy (admission by free memory, continuous batching, refusals,
allocation failures, malformed requests, cancellation, step faults) against a fake
backend, compiled and run on the CPU (tests/cpp/test_server_policy.cpp)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_server_policy_with_fake_backend(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "test_server_policy")
    subprocess.run([cxx, "-std=c++20", "-O1", "-Wall", "-Wextra", "-Werror",
                    os.path.join(ROOT, "tests", "cpp", "test_server_policy.cpp"), "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "10 tests, 0 failures" in r.stdout
