"""The fused x + y sweep of 3-D meshes (pcg_set_sweep_fusion): one launch walks
z-slabs, each slab's y tiles waiting for its x tiles.  Each line's arithmetic is
the unfused sweeps', so fields must be bit-identical to the two-launch path for
every slab size (one plane per slab up to the whole mesh) and lag, in both
builds, with and without the mass check, and within tolerance of the oracle.
"""
import numpy as np
import pytest

from physicore_gb300 import workloads as W
from test_gpu_golden import rel_err

pytestmark = pytest.mark.gpu


def problems(agents=False):
    """3-D random problems with 3-9 substrates.  Without agents by default: sums
    over agents sharing a voxel are floating-point atomics in any order, so two
    runs with colliding agents are not bit-identical whatever the sweeps do."""
    out, seed = [], 500
    while len(out) < 8:
        p = W.random_small(seed, max_side=40, max_S=9)
        seed += 1
        if p["dims"] == 3 and len(p["D"]) >= 3 and min(W_grid(p)) > 1:
            if not agents:
                p["agents"] = None
            out.append(p)
    return out


def W_grid(p):
    return [-(-(p["bbmax"][a] - p["bbmin"][a]) // p["voxel"][a]) for a in range(3)]


@pytest.mark.parametrize("precision", [0, 1])
def test_fused_sweeps_bit_identical_to_two_launches(pcg, oracle_mod, precision):
    for p in problems():
        ref = W.apply(pcg.Solver(precision), p)
        ref.set_sweep_fusion(False)
        ref.solve(3)
        f_ref = ref.get_field()
        plane = W_grid(p)[0] * len(p["D"]) * W_grid(p)[1] * (8 if precision else 4)
        for slab_bytes, lag in [(1, 1), (plane * 3, 1), (plane * 2, 2), (plane * 5, 3), (1 << 40, 2)]:
            g = W.apply(pcg.Solver(precision), p)
            g.set_sweep_fusion(True, slab_bytes, lag)
            g.solve(3)
            assert np.array_equal(g.get_field(), f_ref), (p["name"], slab_bytes, lag)
        o = W.apply(oracle_mod.OracleSolver(threads=2), p)
        o.solve(3)
        assert rel_err(f_ref, o.get_field()) <= (1e-12 if precision == 1 else 1e-5), p["name"]


@pytest.mark.parametrize("precision", [0, 1])
def test_fused_sweeps_with_agents_match_oracle(pcg, oracle_mod, precision):
    for p in problems(agents=True)[:4]:
        g = W.apply(pcg.Solver(precision), p)
        g.set_sweep_fusion(True, 1, 1)
        o = W.apply(oracle_mod.OracleSolver(threads=2), p)
        g.solve(3)
        o.solve(3)
        assert rel_err(g.get_field(), o.get_field()) <= (1e-12 if precision == 1 else 1e-5), p["name"]
        if g.A:
            assert np.array_equal(g.get_counts(), o.get_counts())


def test_fused_sweeps_with_mass_check(pcg):
    for p in problems()[:4]:
        a = W.apply(pcg.Solver(0), p)
        b = W.apply(pcg.Solver(0), p)
        b.set_sweep_fusion(False)
        for s in (a, b):
            s.set_mass_check(True)
            s.solve(4)
        ca, cb = a.get_mass_check(), b.get_mass_check()
        assert np.array_equal(a.get_field(), b.get_field())
        assert np.allclose(ca["before"], cb["before"], rtol=1e-12, atol=0)
        assert np.allclose(ca["after"], cb["after"], rtol=1e-12, atol=0)
        assert np.all(ca["worst"] <= 1e-5)


def test_fused_sweeps_large_lines(pcg, oracle_mod):
    """Lines longer than one TMA box (y of 300 points) and many slabs."""
    rng = np.random.default_rng(9)
    S, n = 4, (48, 300, 37)
    p = dict(name="fused_long", dims=3, bbmin=(0, 0, 0), bbmax=tuple(v * 20 for v in n), voxel=(20, 20, 20),
             dt=0.01, D=np.geomspace(10.0, 1e5, S), decay=np.geomspace(1e-4, 1.0, S), initial=np.zeros(S),
             field=rng.random((n[2], n[1], n[0], S)), field_layout="interleaved",
             boundary=[(0, 0, rng.random(S), np.ones(S, np.uint8)), (2, 1, rng.random(S), np.ones(S, np.uint8))],
             interior=None, bulk=None, agents=None, compute_internalized=False)
    ref = W.apply(pcg.Solver(0), p)
    ref.set_sweep_fusion(False)
    ref.solve(2)
    g = W.apply(pcg.Solver(0), p)
    g.set_sweep_fusion(True, 48 * S * 300 * 4 * 2, 2)
    g.solve(2)
    assert np.array_equal(g.get_field(), ref.get_field())
    o = W.apply(oracle_mod.OracleSolver(threads=4), p)
    o.solve(2)
    assert rel_err(g.get_field(), o.get_field()) <= 1e-5
