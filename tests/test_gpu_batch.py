"""Batched stepping of many domains (pcg_batch_*) against the oracle and against
the same contexts stepped one at a time.

A batch runs every phase of a step as one launch over all its domains, with each
domain's own arithmetic, so every batched domain must meet the parity bar of the
single-domain tests against the FP64 oracle (1e-12 relative in the FP64 build,
1e-5 in the FP32 build, counts and conflict flags identical), and must agree with
pcg_solve on an identical context to the same tolerances.  Covered: dims 1-3,
n = 1 axes, 1-9 substrates, faces, interior nodes, uniform and per-voxel bulk,
colliding and inactive agents, recompute after agent moves, both x mappings and
several y/z chunk sizes, graph replay versus direct launches, descriptor rebuild
after a setter, the autotuner leaving the fields untouched, and an agent outside
its mesh reported as a device fault.
"""
import numpy as np
import pytest

from physicore_gb300 import workloads as W
from test_gpu_golden import rel_err
from test_gpu_parity import check, max_denominator

pytestmark = pytest.mark.gpu

SEEDS = list(range(24))
FP32_RTOL, FP64_RTOL = 1e-5, 1e-12


def _problems(seeds=SEEDS):
    return [W.random_small(s) for s in seeds]


def _snap(s):
    out = dict(field=s.get_field())
    if s.A:
        out.update(internalized=s.get_internalized(), counts=s.get_counts(), conflict=s.get_conflict())
    return out


def _move_agents(problems, solvers_sets, seed=7):
    """Agents permute positions and one toggles activity, in every solver set alike."""
    rng = np.random.default_rng(seed)
    for p, group in zip(problems, zip(*solvers_sets)):
        A = group[0].A
        if not A:
            continue
        a = p["agents"]
        pos = a["positions"][rng.permutation(A)]
        act = a["is_active"].copy()
        act[rng.integers(0, A)] ^= 1
        for s in group:
            s.update_agents(positions=pos, is_active=act)
            s.recompute_positional_data()


def _run(pcg, oracle_mod, problems, precision, configure=None, graph=True, steps=(1, 2, 1)):
    batched = [W.apply(pcg.Solver(precision), p) for p in problems]
    single = [W.apply(pcg.Solver(precision), p) for p in problems]
    oracle = [W.apply(oracle_mod.OracleSolver(threads=2), p) for p in problems]
    b = pcg.Batch(batched)
    b.set_graph(graph)
    if configure:
        configure(b)
    history = []
    for k, n in enumerate(steps):
        if k == 2:
            _move_agents(problems, [batched, single, oracle])
        b.solve(n)
        b.synchronize()
        for s in single + oracle:
            s.solve(n)
        history.append([(_snap(g), _snap(s), _snap(o)) for g, s, o in zip(batched, single, oracle)])
    b.close()
    return history


def _verify(problems, history, precision):
    rtol = FP64_RTOL if precision == 1 else FP32_RTOL
    for k, step in enumerate(history):
        for p, (g, s, o) in zip(problems, step):
            name = f"{p['name']} call {k}"
            vv = None if precision == 1 else float(np.prod(p["voxel"]))
            dm = max_denominator(p)
            check([{key: (g[key], o[key]) for key in g}], rtol, name + " vs oracle", voxel_volume=vv, den_max=dm)
            check([{key: (g[key], s[key]) for key in g}], rtol, name + " vs single", voxel_volume=vv, den_max=dm)


@pytest.mark.parametrize("precision", [0, 1], ids=["fp32", "fp64"])
def test_batch_matches_oracle_and_single(pcg, oracle_mod, precision):
    problems = _problems()
    _verify(problems, _run(pcg, oracle_mod, problems, precision), precision)


@pytest.mark.parametrize("mapping,rows", [(1, 0), (1, 2), (0, 1), (0, 32)], ids=["sub", "sub2", "row1", "row32"])
def test_batch_x_mappings(pcg, oracle_mod, mapping, rows):
    problems = _problems(range(8))
    hist = _run(pcg, oracle_mod, problems, 1, configure=lambda b: b.force_config(0, mapping, rows))
    _verify(problems, hist, 1)


@pytest.mark.parametrize("chunk", [8, 16, 24, 256])
def test_batch_yz_chunks(pcg, oracle_mod, chunk):
    problems = _problems(range(8, 16))

    def cfg(b):
        b.force_config(1, 0, chunk)
        b.force_config(2, 0, chunk)
    _verify(problems, _run(pcg, oracle_mod, problems, 1, configure=cfg), 1)


@pytest.mark.parametrize("graph", [True, False], ids=["graph", "direct"])
def test_batch_step_budgets(pcg, oracle_mod, graph):
    """Domains take part in only the first budgets[d] steps of a call: each matches
    the oracle after exactly that many steps (0: untouched)."""
    problems = _problems(range(10))
    budgets = [0, 1, 5, 2, 7, 7, 3, 0, 6, 4]
    batched = [W.apply(pcg.Solver(1), p) for p in problems]
    b = pcg.Batch(batched)
    b.set_graph(graph)
    b.solve(7, budgets=budgets)
    b.synchronize()
    for p, g, n in zip(problems, batched, budgets):
        o = W.apply(oracle_mod.OracleSolver(threads=2), p)
        if n:
            o.solve(n)
        e = rel_err(g.get_field(), o.get_field())
        assert e <= FP64_RTOL, f"{p['name']} budget {n}: {e:.3e}"
        if g.A and n:
            assert np.array_equal(g.get_counts(), o.get_counts()), p["name"]


@pytest.mark.parametrize("precision", [0, 1], ids=["fp32", "fp64"])
def test_batch_and_single_steps_interleave(pcg, oracle_mod, precision):
    """The same contexts stepped in a batch, then alone, then in the batch again,
    without a recompute request in between: the two kinds of step keep different
    ballot lists, so each rebuilds the ballot left by the other, and every stage
    matches the oracle, internalized amounts included."""
    problems = [p for p in _problems(range(40)) if p["agents"] is not None and p["compute_internalized"]
                and len(p["agents"]["volumes"]) > 4][:6]
    assert len(problems) >= 4
    ctx = [W.apply(pcg.Solver(precision), p) for p in problems]
    oracle = [W.apply(oracle_mod.OracleSolver(threads=2), p) for p in problems]
    rtol = FP64_RTOL if precision == 1 else FP32_RTOL
    b = pcg.Batch(ctx)
    for stage, alone in (("batch", False), ("single", True), ("batch again", False), ("single again", True)):
        if alone:
            for s in ctx:
                s.solve(2)
        else:
            b.solve(2)
            b.synchronize()
        for o in oracle:
            o.solve(2)
        for p, g, o in zip(problems, ctx, oracle):
            gs, os_ = _snap(g), _snap(o)
            vv = None if precision == 1 else float(np.prod(p["voxel"]))
            check([{key: (gs[key], os_[key]) for key in gs}], rtol, f"{p['name']} after {stage}", voxel_volume=vv,
                  den_max=max_denominator(p))
    b.close()


def test_batch_direct_launches(pcg, oracle_mod):
    problems = _problems(range(16, 24))
    _verify(problems, _run(pcg, oracle_mod, problems, 0, graph=False), 0)


def test_batch_picks_up_setters(pcg, oracle_mod):
    """A Dirichlet face added after the batch was built reaches the next batched step."""
    problems = _problems(range(4))
    batched = [W.apply(pcg.Solver(1), p) for p in problems]
    oracle = [W.apply(oracle_mod.OracleSolver(threads=2), p) for p in problems]
    b = pcg.Batch(batched)
    b.solve(2)
    for s in oracle:
        s.solve(2)
    S0 = batched[0].S
    for s in (batched[0], oracle[0]):
        s.set_dirichlet_boundary(0, 1, np.full(S0, 0.25), np.ones(S0, dtype=np.uint8))
    b.solve(3)
    b.synchronize()
    for s in oracle:
        s.solve(3)
    for g, o, p in zip(batched, oracle, problems):
        assert rel_err(g.get_field(), o.get_field()) <= FP64_RTOL, p["name"]


def test_batch_autotune_keeps_state(pcg, oracle_mod):
    problems = [W.random_small(s, max_side=40) for s in range(6)]
    batched = [W.apply(pcg.Solver(0), p) for p in problems]
    before = [s.get_field(dtype=np.float32) for s in batched]
    b = pcg.Batch(batched)
    b.autotune()
    b.synchronize()
    for s, f in zip(batched, before):
        assert np.array_equal(s.get_field(dtype=np.float32), f)
    d = b.describe()
    assert d["domains"] == len(problems)
    for bucket in d["buckets"]:
        assert bucket["tried"] and bucket["us"] > 0
    oracle = [W.apply(oracle_mod.OracleSolver(threads=2), p) for p in problems]
    b.solve(3)
    b.synchronize()
    for s in oracle:
        s.solve(3)
    for g, o, p in zip(batched, oracle, problems):
        assert rel_err(g.get_field(), o.get_field()) <= FP32_RTOL, p["name"]


def test_batch_counts_launches(pcg):
    problems = _problems(range(6))
    batched = [W.apply(pcg.Solver(0), p) for p in problems]
    b = pcg.Batch(batched)
    b.reset_kernel_stats()
    b.solve(4)
    b.synchronize()
    n = b.launch_count()
    # one launch per phase per step, whatever the number of domains
    assert 0 < n <= 4 * 14
    stats = b.kernel_stats()
    assert stats["sweep_x"]["launches"] == 4


def test_batch_agent_outside_is_reported(pcg):
    p = W.random_small(3)
    p["agents"] = W.agents_block(np.random.default_rng(0), 4, W.random_small(3)["D"].size,
                                 np.full((4, p["dims"]), 1e9))
    s = W.apply(pcg.Solver(0), p)
    ok = W.apply(pcg.Solver(0), W.random_small(5))
    b = pcg.Batch([ok, s])
    b.solve(1)
    with pytest.raises(pcg.PcgError) as ei:
        b.synchronize()
    assert ei.value.code == 4 and "outside" in str(ei.value)


def test_batch_rejects_mixed_precision(pcg):
    a = W.apply(pcg.Solver(0), W.random_small(1))
    c = W.apply(pcg.Solver(1), W.random_small(2))
    with pytest.raises(pcg.PcgError) as ei:
        pcg.Batch([a, c])
    assert ei.value.code == 1
