"""Agent-to-voxel placement at voxel boundaries: agents sit on every boundary of a
mesh and 1..16 ulps either side of it (and outside the mesh's upper faces
rounded back in), so the GPU's fast FP32 estimate must defer to the FP64 division
wherever the two could differ.  Per-voxel counts and the conflict flag must equal
the oracle's (cartesian_mesh::voxel_position, mesh.cpp:37-61) bit for bit, and
the fields must meet the usual tolerance, in both builds.
"""
import numpy as np
import pytest

from physicore_gb300 import workloads as W
from test_gpu_golden import rel_err

pytestmark = pytest.mark.gpu


def boundary_problem(seed):
    rng = np.random.default_rng(seed)
    S, voxel, n, bbmin = 3, (25, 20, 10), (37, 30, 20), (-100, 40, 7)
    bbmax = tuple(bbmin[d] + voxel[d] * n[d] for d in range(3))
    A = 20000
    pos = np.empty((A, 3))
    for d in range(3):
        k = rng.integers(0, n[d] + 1, A)  # a boundary index (n: the upper face)
        x = bbmin[d] + voxel[d] * k.astype(np.float64)
        ulps = rng.integers(-16, 17, A)
        for u in range(1, 17):
            x = np.where(ulps >= u, np.nextafter(x, np.inf), x)
            x = np.where(ulps <= -u, np.nextafter(x, -np.inf), x)
        lo, hi = float(bbmin[d]), np.nextafter(float(bbmax[d]), -np.inf)
        pos[:, d] = np.clip(x, lo, hi)
    ag = W.agents_block(rng, A, S, pos, net_export_hi=0.5)
    return dict(name=f"boundary_{seed}", dims=3, bbmin=bbmin, bbmax=bbmax, voxel=voxel, dt=0.01,
                D=np.array([1e3, 50.0, 2e4]), decay=np.array([0.1, 0.5, 1e-3]), initial=np.zeros(S),
                field=rng.random((n[2], n[1], n[0], S)), field_layout="interleaved", boundary=[], interior=None,
                bulk=None, agents=ag, compute_internalized=True)


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("seed", [0, 1])
def test_boundary_agents_counts_bit_exact(pcg, oracle_mod, precision, seed):
    p = boundary_problem(seed)
    g = W.apply(pcg.Solver(precision), p)
    o = W.apply(oracle_mod.OracleSolver(threads=4), p)
    g.solve(2)
    o.solve(2)
    assert np.array_equal(g.get_counts(), o.get_counts())
    assert g.get_conflict() == o.get_conflict()
    assert rel_err(g.get_field(), o.get_field()) <= (1e-12 if precision == 1 else 1e-5)
