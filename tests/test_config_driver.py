"""Settings reader, microenvironment builder and VTK image serializer of the host
mirror (tests/cpp/test_config.cpp), with the written images read back here.  No
GPU: the serializer writes through a CPU test solver whose densities are
s*1000 + x + 10*y + 100*z + 0.25*steps."""
import os
import subprocess

import numpy as np
import pytest

from vti import read_pvd, read_vti

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BUILD = os.path.join(ROOT, "tests", "_build")


@pytest.fixture(scope="module")
def config_run(pcg, tmp_path_factory):
    from physicore_gb300 import _build
    host_lib = _build.build_host()
    os.makedirs(BUILD, exist_ok=True)
    exe = os.path.join(BUILD, "test_config")
    pkg = os.path.dirname(host_lib)
    subprocess.run([_build.cxx(), "-std=c++20", "-O2", "-Wall", "-Wextra",
                    os.path.join(ROOT, "tests", "cpp", "test_config.cpp"), "-I", os.path.join(ROOT, "include"),
                    "-L", pkg, "-lphysicore_gb300_host", "-lphysicore_gb300", f"-Wl,-rpath,{pkg}", "-o", exe],
                   check=True)
    scratch = str(tmp_path_factory.mktemp("config"))
    r = subprocess.run([exe, scratch], capture_output=True, text=True, timeout=300)
    return r, scratch


def test_config_reader_and_builder(config_run):
    r, _ = config_run
    assert r.returncode == 0 and "8 tests, 0 failures" in r.stdout, r.stdout + r.stderr


@pytest.mark.parametrize("dims", [3, 2])
def test_vti_images(config_run, dims):
    _, scratch = config_run
    out = os.path.join(scratch, f"out{dims}")
    # mesh [-40,60) x [20,80) x [-60,0) with voxels 20 x 20 x 30
    n = (5, 3, 2 if dims == 3 else 1)
    entries = read_pvd(os.path.join(out, "microenvironment.pvd"))
    assert [t for t, _ in entries] == [0.0, 0.125]
    assert [f for _, f in entries] == [os.path.join("vtk_microenvironment", f"microenvironment_{i:06d}.vti")
                                       for i in range(2)]
    z, y, x = np.meshgrid(np.arange(n[2]), np.arange(n[1]), np.arange(n[0]), indexing="ij")
    for k, steps in enumerate((0, 2)):
        img = read_vti(os.path.join(out, entries[k][1]))
        if dims == 3:
            assert img["extent"] == [-2, 3, 1, 4, -2, 0] and img["spacing"] == [20.0, 20.0, 30.0]
        else:
            assert img["extent"] == [-2, 3, 1, 4, 0, 0] and img["spacing"] == [20.0, 20.0, 0.0]
        assert list(img["arrays"]) == ["first", "second one", "third"]
        for s, name in enumerate(img["arrays"]):
            want = s * 1000.0 + x + 10.0 * y + 100.0 * z + 0.25 * steps
            assert np.array_equal(img["arrays"][name], want), (name, steps)
