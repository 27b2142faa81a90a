"""Agents moved on the device (pcg_get_agents_device): positions and activity
written straight into the context's device arrays by other GPU work, followed by
pcg_recompute_positional_data, give the same ballots (bit-exact counts and
conflict flag) and fields as the oracle given the same moves on the host."""
import ctypes
import ctypes.util
import os

import numpy as np
import pytest

from physicore_gb300 import workloads as W
from test_gpu_golden import rel_err

pytestmark = pytest.mark.gpu


def _cudart():
    names = [ctypes.util.find_library("cudart"), "libcudart.so", "/usr/local/cuda/lib64/libcudart.so"]
    for n in names:
        if n and (os.path.exists(n) or not n.startswith("/")):
            try:
                return ctypes.CDLL(n)
            except OSError:
                continue
    pytest.fail("no CUDA runtime library to copy device memory with")


def _device_copy(rt, dst, src, nbytes):
    rt.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
    assert rt.cudaMemcpy(ctypes.c_void_p(dst), ctypes.c_void_p(src), ctypes.c_size_t(nbytes), 3) == 0  # D2D
    assert rt.cudaDeviceSynchronize() == 0


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("seed", [0, 2, 5, 7, 9])
def test_agents_moved_on_the_device(pcg, oracle_mod, seed, precision):
    import torch
    p = W.random_small(seed)
    if p.get("agents") is None or not len(p["agents"]["volumes"]):
        pytest.skip("problem without agents")
    g = W.apply(pcg.Solver(precision), p)
    o = W.apply(oracle_mod.OracleSolver(threads=2), p)
    g.solve(2)
    o.solve(2)
    a = p["agents"]
    A = len(a["volumes"])
    rng = np.random.default_rng(100 + seed)
    pos = np.ascontiguousarray(a["positions"][rng.permutation(A)])
    act = a["is_active"].copy()
    act[rng.integers(0, A, max(1, A // 5))] ^= 1
    # the moves come from device memory, as a GPU mechanics module would write them
    src_pos = torch.from_numpy(pos).cuda()
    src_act = torch.from_numpy(act).cuda()
    torch.cuda.synchronize()
    g.synchronize()
    d_pos, d_act = g.agents_device()
    rt = _cudart()
    _device_copy(rt, d_pos, src_pos.data_ptr(), pos.nbytes)
    _device_copy(rt, d_act, src_act.data_ptr(), act.nbytes)
    g.recompute_positional_data()
    o.update_agents(pos, act)
    o.recompute_positional_data()
    g.solve(3)
    o.solve(3)
    assert np.array_equal(g.get_counts(), o.get_counts())
    assert g.get_conflict() == o.get_conflict()
    tol = 1e-12 if precision == 1 else 1e-5
    assert rel_err(g.get_field(), o.get_field()) <= tol


def test_agents_device_without_agents(pcg):
    p = dict(W.random_small(11))
    p["agents"] = None
    g = W.apply(pcg.Solver(0), p)
    with pytest.raises(pcg.PcgError):
        g.agents_device()
