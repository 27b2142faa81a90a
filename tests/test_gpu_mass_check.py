"""The per-step FP64 mass check (pcg_set_mass_check / pcg_get_mass_check): on
random problems with Dirichlet faces and nodes, bulk and agents, every checked
step's sweeps keep the identity after * f = before (f: the product of the sweep
matrices' column sums; worst residual <= 1e-12 in the FP64 build, <= 1e-5 in
FP32), the last step's
totals equal the oracle's before and after its diffusion phase, and the field
is the same with the check on as with it off (to the parity tolerance)."""
import numpy as np
import pytest

from physicore_gb300 import workloads as W
from test_gpu_golden import rel_err

pytestmark = pytest.mark.gpu

STEPS = 5


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("seed", range(12))
def test_mass_check_matches_oracle(pcg, oracle_mod, seed, precision):
    p = W.random_small(seed)
    g = W.apply(pcg.Solver(precision), p)
    g.set_mass_check(True)
    g.solve(STEPS)
    chk = g.get_mass_check()
    tol = 1e-12 if precision == 1 else 1e-5
    assert chk["steps"] == STEPS
    assert np.all(chk["worst"] <= tol), chk["worst"]

    o = W.apply(oracle_mod.OracleSolver(threads=2), p)
    o.solve(STEPS - 1)
    before = o.mass()
    o.run_phases(oracle_mod.PHASE_DIFFUSION, False)
    after = o.mass()
    scale = np.maximum(np.abs(before), 1e-300)
    assert np.all(np.abs(chk["before"] - before) <= tol * scale), (chk["before"], before)
    assert np.all(np.abs(chk["after"] - after) <= tol * scale), (chk["after"], after)

    # the field of an unchecked run (faces then come from their own kernel); not
    # bit-equal in general: sums over agents sharing a voxel are atomic, in any order
    h = W.apply(pcg.Solver(precision), p)
    h.solve(STEPS)
    assert rel_err(g.get_field(), h.get_field()) <= tol


def test_mass_check_reset_and_off(pcg):
    p = W.random_small(3)
    g = W.apply(pcg.Solver(0), p)
    g.set_mass_check(True)
    g.solve(2)
    assert g.get_mass_check()["steps"] == 2
    g.set_mass_check(False)
    g.solve(3)
    assert g.get_mass_check()["steps"] == 2
    g.set_mass_check(True)
    assert g.get_mass_check()["steps"] == 0 and np.all(g.get_mass_check()["worst"] == 0)
    g.solve(1)
    assert g.get_mass_check()["steps"] == 1


def test_mass_check_never_enabled(pcg):
    g = W.apply(pcg.Solver(0), W.random_small(4))
    with pytest.raises(pcg.PcgError):
        g.get_mass_check()


@pytest.mark.parametrize("precision", [0, 1])
def test_mass_check_many_substrates(pcg, oracle_mod, precision):
    """40 substrates: the x sweep takes its row-per-thread path for any S (totals
    added per row) and the y/z sweeps add per tile (40 does not divide 32)."""
    rng = np.random.default_rng(77)
    S, n = 40, (7, 6, 5)
    p = dict(name="many_substrates", dims=3, bbmin=(0, 0, 0), bbmax=tuple(v * 20 for v in n), voxel=(20, 20, 20),
             dt=0.01, D=np.geomspace(10.0, 1e5, S), decay=np.geomspace(1e-4, 1.0, S), initial=np.zeros(S),
             field=rng.random((n[2], n[1], n[0], S)), field_layout="interleaved",
             boundary=[(0, 0, rng.random(S), np.ones(S, np.uint8))], interior=None, bulk=None, agents=None,
             compute_internalized=False)
    g = W.apply(pcg.Solver(precision), p)
    g.set_mass_check(True)
    g.solve(STEPS)
    chk = g.get_mass_check()
    tol = 1e-12 if precision == 1 else 1e-5
    assert chk["steps"] == STEPS and np.all(chk["worst"] <= tol), chk["worst"]
    o = W.apply(oracle_mod.OracleSolver(threads=2), p)
    o.solve(STEPS - 1)
    before = o.mass()
    o.run_phases(oracle_mod.PHASE_DIFFUSION, False)
    after = o.mass()
    assert np.all(np.abs(chk["before"] - before) <= tol * np.abs(before))
    assert np.all(np.abs(chk["after"] - after) <= tol * np.abs(before))


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("graph", [True, False])
def test_mass_check_in_batches(pcg, oracle_mod, precision, graph):
    """Contexts stepped by a batch keep their own per-step check: every other
    domain has it on, domains run different step budgets, and each checked
    domain's worst residual, step count and last totals match a single-domain
    checked run of the same problem (and its totals the oracle's)."""
    problems = [W.random_small(100 + k) for k in range(10)]
    budgets = [STEPS - (k % 3) for k in range(10)]
    batched = [W.apply(pcg.Solver(precision), p) for p in problems]
    for k, s in enumerate(batched):
        if k % 2 == 0:
            s.set_mass_check(True)
    b = pcg.Batch(batched)
    b.set_graph(graph)
    b.solve(STEPS, budgets=budgets)
    b.synchronize()
    tol = 1e-12 if precision == 1 else 1e-5
    for k, (p, s) in enumerate(zip(problems, batched)):
        if k % 2:
            with pytest.raises(pcg.PcgError):
                s.get_mass_check()
            continue
        chk = s.get_mass_check()
        assert chk["steps"] == budgets[k], (k, chk["steps"])
        assert np.all(chk["worst"] <= tol), (k, chk["worst"])
        single = W.apply(pcg.Solver(precision), p)
        single.set_mass_check(True)
        single.solve(budgets[k])
        ref = single.get_mass_check()
        scale = np.maximum(np.abs(ref["before"]), 1e-300)
        assert np.all(np.abs(chk["before"] - ref["before"]) <= tol * scale), k
        assert np.all(np.abs(chk["after"] - ref["after"]) <= tol * scale), k
        o = W.apply(oracle_mod.OracleSolver(threads=2), p)
        o.solve(budgets[k] - 1)
        before = o.mass()
        o.run_phases(oracle_mod.PHASE_DIFFUSION, False)
        assert np.all(np.abs(chk["before"] - before) <= tol * np.maximum(np.abs(before), 1e-300)), k
        assert np.all(np.abs(chk["after"] - o.mass()) <= tol * np.maximum(np.abs(before), 1e-300)), k
    b.close()
