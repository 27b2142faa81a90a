"""Host-side checks of the workload generator and of oracle invariants (CPU only)."""
import numpy as np
import pytest

from physicore_gb300 import workloads as W


def voxel_histogram(p):
    a = p["agents"]
    dims = p["dims"]
    grid = [-(-(p["bbmax"][d] - p["bbmin"][d]) // p["voxel"][d]) if d < dims else 1 for d in range(3)]
    idx = np.zeros((len(a["volumes"]), 3), dtype=np.int64)
    for d in range(dims):
        # cartesian_mesh::voxel_position: truncation of an FP64 quotient (mesh.cpp:49-56)
        idx[:, d] = ((a["positions"][:, d] - float(p["bbmin"][d])) / float(p["voxel"][d])).astype(np.int64)
    act = a["is_active"].astype(bool)
    lin = idx[act, 0] + grid[0] * (idx[act, 1] + grid[1] * idx[act, 2])
    return np.bincount(lin, minlength=grid[0] * grid[1] * grid[2]).reshape(grid[2], grid[1], grid[0])


def test_generator_is_deterministic():
    a, b = W.random_small(11), W.random_small(11)
    assert np.array_equal(a["field"], b["field"])
    assert np.array_equal(a["agents"]["positions"], b["agents"]["positions"])


@pytest.mark.parametrize("seed", range(12))
def test_oracle_runs_random_problems(oracle_mod, seed):
    p = W.random_small(seed)
    o = W.apply(oracle_mod.OracleSolver(threads=2), p)
    o.solve(2)
    f = o.get_field()
    assert np.isfinite(f).all()
    if o.A:
        assert np.array_equal(o.get_counts(), voxel_histogram(p))
        assert o.get_conflict() == bool((voxel_histogram(p) > 1).any())


def test_oracle_mass_identity(oracle_mod):
    rng = np.random.default_rng(2)
    S = 2
    decay = np.array([0.3, 0.01])
    p = dict(name="m", dims=2, bbmin=(0, 0, 0), bbmax=(70, 50, 0), voxel=(10, 10, 10), dt=0.1,
             D=np.array([50.0, 5e3]), decay=decay, initial=np.zeros(S), field=rng.random((1, 5, 7, S)),
             field_layout="interleaved", boundary=[], interior=None, bulk=None, agents=None,
             compute_internalized=False)
    o = W.apply(oracle_mod.OracleSolver(), p)
    m0 = o.mass()
    o.solve(3)
    assert np.allclose(o.mass(), m0 * (1 / (1 + decay * 0.1 / 2)) ** 6, rtol=1e-13, atol=0)


def test_workload_shapes():
    p = W.plain_100(n=10, agents=50)
    assert p["agents"]["positions"].shape == (50, 3)
    assert (p["agents"]["positions"] >= 20).all() and (p["agents"]["positions"] < 180).all()
    q = W.large(n=16, S=3, agents=100, interior=20)
    assert q["field"].shape == (3, 16, 16, 16) and q["field"].dtype == np.float32
    assert q["interior"][0].shape[1] == 3


@pytest.mark.parametrize("seed", range(12))
def test_oracle_sweep_mass_identity_mixed_problems(oracle_mod, seed):
    """The premise of the per-step mass check: whatever Dirichlet, bulk and agents
    did before, the sweeps of one step divide every substrate's total by the
    product over the axes of the matrix column sums, 1 + decay*dt/dims, plus
    r = dt*D/h^2 on an axis of length 1 (its diagonal loses r once, not twice)."""
    p = W.random_small(seed)
    o = W.apply(oracle_mod.OracleSolver(threads=2), p)
    o.solve(2)
    before = o.mass()
    o.run_phases(oracle_mod.PHASE_DIFFUSION, False)
    after = o.mass()
    decay, D = np.asarray(p["decay"], float), np.asarray(p["D"], float)
    f = np.ones_like(decay)
    for a in range(p["dims"]):
        r = D * p["dt"] / float(p["voxel"][a]) ** 2 if o.grid[a] == 1 else 0.0
        f = f * (1.0 + decay * p["dt"] / p["dims"] + r)
    assert np.allclose(after * f, before, rtol=1e-12, atol=1e-300)
