"""Parity at the benchmark configurations, at full size, against the FP64 oracle.

plain_100 (100^3 voxels, 1 substrate, FP64 field, all six faces Dirichlet 1.0,
1,000 interior agents, 100 steps): the reference's own CPU-runnable case, stepped
on the GPU in FP64 and held to 1e-12 relative.

large_320 (320^3 voxels x 8 substrates, FP32 field U[0,1], x-face Dirichlet plus
10,000 interior voxels, 1,000,000 agents): the headline workload, stepped 100
times in FP32 and held to 1e-5 relative.

Errors are stated both ways, per substrate, worst substrate reported:
  max_rel = max |gpu - oracle| / max |oracle|
  l2_rel  = ||gpu - oracle||_2 / ||oracle||_2
Ballot counts and the conflict flag are integers and must be identical.  The step
order is the reference's (openmp_solver.cpp:23-40): every solve call runs
diffusion, Dirichlet, bulk and cells; the first call rebuilds the ballots.
"""
import os

import numpy as np
import pytest

from physicore_gb300 import workloads as W

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-12
FP32_RTOL = 1e-5


def errors(got, ref):
    S = ref.shape[-1]
    g = got.reshape(-1, S)
    r = ref.reshape(-1, S)
    d = np.abs(g - r)
    max_rel = d.max(axis=0) / np.abs(r).max(axis=0)
    l2_rel = np.sqrt((d ** 2).sum(axis=0)) / np.sqrt((r ** 2).sum(axis=0))
    return float(max_rel.max()), float(l2_rel.max())


def threads():
    return max(2, min(72, os.cpu_count() or 2))


def test_plain_100_fp64_100_steps(pcg, oracle_mod):
    p = W.plain_100()
    g = W.apply(pcg.Solver(pcg.FP64), p)
    o = W.apply(oracle_mod.OracleSolver(threads=threads()), p)
    for chunk in (1, 49, 50):  # 100 steps in three solve calls; only the first rebuilds the ballots
        g.solve(chunk)
        o.solve(chunk)
    max_rel, l2_rel = errors(g.get_field(), o.get_field())
    print(f"plain_100 FP64 after 100 steps: max_rel {max_rel:.3e}, l2_rel {l2_rel:.3e}")
    assert max_rel <= FP64_RTOL and l2_rel <= FP64_RTOL
    assert np.array_equal(g.get_counts(), o.get_counts())
    assert g.get_conflict() == o.get_conflict()
    ig, io = g.get_internalized(), o.get_internalized()
    ie = float((np.abs(ig - io) / np.abs(io).max(axis=0)).max())
    assert ie <= FP64_RTOL, f"internalized relative error {ie:.3e}"


def test_large_320_fp32_100_steps(pcg, oracle_mod):
    p = W.large()
    g = W.apply(pcg.Solver(pcg.FP32), p)
    o = W.apply(oracle_mod.OracleSolver(threads=threads()), p)
    del p
    g.solve(1)
    o.solve(1)
    e1 = errors(g.get_field(), o.get_field())
    assert np.array_equal(g.get_counts(), o.get_counts())
    assert g.get_conflict() == o.get_conflict()
    g.solve(99)
    o.solve(99)
    max_rel, l2_rel = errors(g.get_field(), o.get_field())
    print(f"large_320 FP32: after 1 step max_rel {e1[0]:.3e} l2_rel {e1[1]:.3e}; "
          f"after 100 steps max_rel {max_rel:.3e}, l2_rel {l2_rel:.3e}")
    assert max_rel <= FP32_RTOL, f"max_rel {max_rel:.3e} after 100 steps"
    assert l2_rel <= FP32_RTOL, f"l2_rel {l2_rel:.3e} after 100 steps"
