"""Dense-agent stress on the ballots and atomics (the 200^3 x 4 FP32 workload with
4,000,000 agents in a Gaussian cluster of sigma 200 um at the domain centre, up to
about a hundred agents per voxel), against the oracle at full size.

Per-voxel agent counts and the conflict flag must be bit-exact; fields within
1e-5 relative per substrate of the FP64 oracle; internalized amounts within the
FP32 bound of test_gpu_parity.check.  The agents move before the third call (a
permutation of the positions) and the ballots are rebuilt.
"""
import os

import numpy as np
import pytest

from physicore_gb300 import workloads as W
from test_gpu_parity import check, max_denominator, run_both

pytestmark = pytest.mark.gpu


def test_dense_cluster_full_size(pcg, oracle_mod):
    p = W.dense()
    snaps = run_both(pcg, oracle_mod, p, pcg.FP32, threads=max(2, min(16, os.cpu_count() or 2)))
    counts = snaps[0]["counts"][1]
    assert counts.max() >= 50, "the cluster should pile tens of agents into its central voxels"
    assert snaps[0]["conflict"][1]
    check(snaps, 1e-5, p["name"], voxel_volume=float(np.prod(p["voxel"])), den_max=max_denominator(p))
