"""Golden-value checks for every reference unit test of the BioFVM step.

Each `golden_*` function rebuilds one reference gtest with `make()` (an
OracleSolver or a GPU Solver factory), asserts the reference's expected values
with the reference's tolerances when `check` is true, and returns the arrays it
produced so that the GPU tests can also compare them with the oracle's.
"""
from __future__ import annotations

import numpy as np

import cases as C


def _near(actual, exp, what=""):
    assert abs(actual - exp["value"]) <= exp["tol"] * (1 + 1e-9), \
        f"{what} line {exp['line']}: {actual!r} vs {exp['value']} +- {exp['tol']}"


def _deq(actual, expected, what=""):
    # EXPECT_DOUBLE_EQ: within 4 ULPs
    actual, expected = np.asarray(actual, dtype=np.float64), np.asarray(expected, dtype=np.float64)
    ok = np.abs(actual - expected) <= 4 * np.spacing(np.abs(expected))
    assert np.all(ok), f"{what}: {actual[~ok] if actual.ndim else actual!r} != {expected!r}"


def golden_uniform(make, dims, check=True):
    s, exp = C.run_uniform(make, dims)
    f = s.get_field()
    if check:
        for sub in range(2):
            for v in f[..., sub].ravel():
                _near(v, exp[sub], f"Uniform{dims}D s{sub}")
    return {"field": f}


def golden_random(make, dims, check=True):
    s, exp = C.run_random(make, dims)
    f = s.get_field()
    if check:
        got = f.ravel()  # interleaved order == the test's index order
        assert got.size == exp.size
        bad = np.abs(got - exp) > 1e-6
        assert not bad.any(), f"Random{dims}D mismatches at {np.nonzero(bad)[0][:8]}: {got[bad][:8]} vs {exp[bad][:8]}"
    return {"field": f}


def golden_bulk(make, check=True):
    s, exp = C.run_bulk(make)
    f = s.get_field()
    if check:
        _near(f[1, 1, 1, 0], exp, "bulk (1,1,1,0)")
        mask = np.ones(f.shape[:3], dtype=bool)
        mask[1, 1, 1] = False
        _deq(f[..., 0][mask], 10.0, "bulk s0 elsewhere")
        _deq(f[..., 1], 1.0, "bulk s1")
    return {"field": f}


def golden_interior(make, dims, check=True):
    s, pts = C.run_interior(make, dims)
    f = s.get_field()
    if check:
        for idx, val in pts:
            x, y, z = idx
            _deq(f[z, y, x, 0], float(val), f"Interior{dims}D {idx}")
        # untouched voxels keep their initial conditions
        mask = np.ones(f.shape[:3], dtype=bool)
        for idx, _ in pts:
            mask[idx[2], idx[1], idx[0]] = False
        _deq(f[..., 0][mask], 1.0, "interior untouched s0")
        _deq(f[..., 1], 1.0, "interior s1")
    return {"field": f}


def golden_boundary(make, dims, check=True):
    s = C.run_boundary(make, dims)
    f = s.get_field()
    if check:
        nx, ny, nz = s.grid
        exp = C.boundary_expected(dims, nx, ny, nz)
        _deq(f[..., 0], exp, f"Boundary{dims}D s0")
        _deq(f[..., 1], 1.0, f"Boundary{dims}D s1")
    return {"field": f}


def golden_dynamic_boundary(make, check=True):
    """DirichletSolverTest.DynamicBoundaryModification (test_dirichlet_solver.cpp:355-392)."""
    s = C.builder_env(make, [(100.0, 0.01, 38.0)])
    s.set_dirichlet_boundary(0, 0, [160.0], [1])
    s.initialize()
    for _ in range(5):
        s.solve(1)
    s.set_dirichlet_boundary(0, 0, [20.0], [1])
    for _ in range(5):
        s.solve(1)
    f = s.get_field()
    if check:
        _deq(f[1, 1, 0, 0], 20.0, "x-min face after update")
    return {"field": f}


def golden_dynamic_interior(make, check=True):
    """DirichletSolverTest.DynamicInteriorVoxelModification (test_dirichlet_solver.cpp:394-425)."""
    s = C.builder_env(make, [(100.0, 0.01, 38.0), (50.0, 0.02, 5.0)])
    s.set_dirichlet_interior([5, 5, 5], [160.0, 50.0], [1, 1])
    s.initialize()
    for _ in range(5):
        s.solve(1)
    s.set_dirichlet_interior([5, 5, 5], [160.0, 0.0], [1, 1])  # update_dirichlet_interior_voxel s=1 -> 0
    for _ in range(5):
        s.solve(1)
    f = s.get_field()
    if check:
        _deq(f[5, 5, 5, 1], 0.0, "glucose source depleted")
        _deq(f[5, 5, 5, 0], 160.0, "oxygen source kept")
    return {"field": f}


def golden_disable_boundary(make, check=True):
    """DirichletSolverTest.DisableDirichletConditionsDynamically (test_dirichlet_solver.cpp:427-458).

    The reference asserts get_substrate_density(1, 0, 1, 1) != 160 on a one-substrate
    mesh; with S = 1 that index reads voxel (1,1,1).  Both that voxel and the face
    voxel (0,1,1) must have left 160 once the condition is off."""
    s = C.builder_env(make, [(100.0, 0.01, 38.0)])
    s.set_dirichlet_boundary(0, 0, [160.0], [1])
    s.initialize()
    for _ in range(5):
        s.solve(1)
    s.set_dirichlet_boundary(0, 0, [160.0], [0])
    for _ in range(5):
        s.solve(1)
    f = s.get_field()
    if check:
        assert f[1, 1, 1, 0] != 160.0
        assert f[1, 1, 0, 0] != 160.0
    return {"field": f}


def golden_multiple_substrates(make, check=True):
    """DirichletSolverTest.MultipleSubstrateModification (test_dirichlet_solver.cpp:460-505)."""
    s = C.builder_env(make, [(100.0, 0.01, 38.0), (50.0, 0.02, 5.0), (30.0, 0.015, 2.0)])
    s.set_dirichlet_interior([5, 5, 5], [160.0, 50.0, 10.0], [1, 1, 1])
    s.initialize()
    for _ in range(5):
        s.solve(1)
    # update_dirichlet_interior_voxel keeps existing nodes in place and appends new ones
    s.set_dirichlet_interior([5, 5, 5, 2, 2, 2], [80.0, 100.0, 0.0, 200.0, 60.0, 15.0], [1] * 6)
    for _ in range(5):
        s.solve(1)
    f = s.get_field()
    if check:
        for (x, y, z), vals in [((5, 5, 5), (80.0, 100.0, 0.0)), ((2, 2, 2), (200.0, 60.0, 15.0))]:
            for sub, v in enumerate(vals):
                _deq(f[z, y, x, sub], v, f"node {(x, y, z)} s{sub}")
    return {"field": f}


def _simple_cells(make, dims, internalized, recompute, check):
    name = {1: "RecomputeTest.Simple1D", 2: "RecomputeTest.Simple2D", 3: "RecomputeTest.Simple3D"}[dims]
    bbmax, positions = C.SIMPLE_MESH[dims]
    s = C.cell_env(make, dims, bbmax, internalized)
    agents = [C.default_agent(0, 1000), C.default_agent(400, 1000), C.default_agent(800, 1000)]
    C.set_agents(s, agents, positions, compute_internalized=internalized)
    s.initialize()
    diag = lambda f, k: f[k if dims > 2 else 0, k if dims > 1 else 0, k]
    out = {}
    s.run_phases(C.PHASE_CELLS, True)
    f1, i1 = s.get_field(), s.get_internalized()
    s.run_phases(C.PHASE_CELLS, recompute)
    f2, i2 = s.get_field(), s.get_internalized()
    s.release_internalized(0)
    f3, i3 = s.get_field(), s.get_internalized()
    out.update(field1=f1, int1=i1, field2=f2, int2=i2, field3=f3, int3=i3)
    if check:
        # in source order: 6 internalized, 6 density, 6 internalized, 6 density assertions
        near = [a for a in C.golden(name)["asserts"] if a["kind"] == "near"]
        assert len(near) == 24, (name, len(near))
        first_int, first_den, second_int, second_den = near[0:6], near[6:12], near[12:18], near[18:24]
        for (ints, dens, f, I) in [(first_int, first_den, f1, i1), (second_int, second_den, f2, i2)]:
            assert len(dens) == 6 and len(ints) == 6, (name, len(dens), len(ints))
            if internalized:
                for k, a in enumerate(ints):
                    _near(I[k // 2, k % 2], a, f"{name} internalized")
            for k, a in enumerate(dens):
                _near(diag(f, k // 2)[k % 2], a, f"{name} density")
        if internalized:
            _deq(diag(f3, 0)[0], 1.0, "released s0")
            _deq(diag(f3, 0)[1], 1.0, "released s1")
            _deq(i3[0], 0.0, "released internalized")
    return out


def golden_simple_cells(make, dims, internalized, recompute, check=True):
    return _simple_cells(make, dims, internalized, recompute, check)


def _conflict(make, agents, positions, internalized, recompute, check, grid_x):
    s = C.cell_env(make, 1, (grid_x * 20, 20, 20), internalized)
    C.set_agents(s, agents, positions, compute_internalized=internalized)
    s.initialize()
    active = [1] * len(agents)
    out = {}
    f0 = s.get_field()[0, 0]  # [nx, S]
    exp_d = C.serial_expected_densities_1d(f0, grid_x, agents, positions, active)
    s.run_phases(C.PHASE_CELLS, True)
    f1 = s.get_field()[0, 0]
    exp_i = C.serial_expected_internalized_1d(f1, agents, positions, np.zeros((len(agents), 2)))
    i1 = s.get_internalized()
    if check:
        assert np.all(np.abs(f1 - exp_d) <= 1e-6), np.max(np.abs(f1 - exp_d))
        if internalized:
            assert np.all(np.abs(i1 - exp_i) <= 1e-6), np.max(np.abs(i1 - exp_i))
    exp_d2 = C.serial_expected_densities_1d(f1, grid_x, agents, positions, active)
    s.run_phases(C.PHASE_CELLS, recompute)
    f2 = s.get_field()[0, 0]
    exp_i = C.serial_expected_internalized_1d(f2, agents, positions, exp_i)
    i2 = s.get_internalized()
    if check:
        assert np.all(np.abs(f2 - exp_d2) <= 1e-6), np.max(np.abs(f2 - exp_d2))
        if internalized:
            assert np.all(np.abs(i2 - exp_i) <= 1e-6), np.max(np.abs(i2 - exp_i))
    for i in range(len(agents)):
        s.release_internalized(i)
    f3 = s.get_field()[0, 0]
    if check and internalized:
        assert np.all(np.abs(f3 - 1.0) <= 1e-6), np.max(np.abs(f3 - 1.0))
    assert s.get_conflict()
    out.update(field1=f1, int1=i1, field2=f2, int2=i2, field3=f3, counts=s.get_counts())
    return out


def golden_conflict(make, internalized, recompute, check=True):
    """RecomputeTest.Conflict (test_cell_solver.cpp:396-491)."""
    agents, positions = C.conflict_agents()
    out = _conflict(make, agents, positions, internalized, recompute, check, 3)
    if check:
        assert out["counts"].ravel().tolist() == [1, 2, 3]
    return out


def golden_conflict_big(make, internalized, recompute, check=True):
    """RecomputeTest.ConflictBig (test_cell_solver.cpp:493-585)."""
    agents, positions = C.conflict_big_agents()
    out = _conflict(make, agents, positions, internalized, recompute, check, 100)
    if check:
        assert (out["counts"].ravel() == 50).all()
    return out


def golden_inactive_skip(make, check=True):
    """CellSolverTest.InactiveAgentsSkipSecretion (test_cell_solver.cpp:587-652)."""
    name = "CellSolverTest.InactiveAgentsSkipSecretion"
    s = C.cell_env(make, 1, (60, 20, 20), True)
    agents = [C.default_agent(0, 1000), C.default_agent(400, 1000), C.default_agent(800, 1000)]
    C.set_agents(s, agents, [(10, 0, 0), (30, 0, 0), (50, 0, 0)], active=[1, 0, 1], compute_internalized=True)
    s.initialize()
    s.run_phases(C.PHASE_CELLS, True)
    f = s.get_field()[0, 0]
    I = s.get_internalized()
    if check:
        _near(f[0, 0], C.expect(name, 626))
        _near(f[0, 1], C.expect(name, 627))
        _deq(f[1], 1.0, "inactive voxel untouched")
        _near(f[2, 0], C.expect(name, 634))
        _near(f[2, 1], C.expect(name, 635))
        _near(I[0, 0], C.expect(name, 641))
        _near(I[0, 1], C.expect(name, 642))
        _deq(I[1], 0.0, "inactive internalized")
        _near(I[2, 0], C.expect(name, 649))
        _near(I[2, 1], C.expect(name, 650))
        assert s.get_counts().ravel().tolist() == [1, 0, 1]
    return {"field": f, "int": I}


def golden_all_inactive(make, check=True):
    """CellSolverTest.AllInactiveAgentsNoSecretion (test_cell_solver.cpp:654-713)."""
    s = C.cell_env(make, 1, (60, 20, 20), True)
    agents = [C.default_agent(0, 1000), C.default_agent(400, 1000)]
    C.set_agents(s, agents, [(10, 0, 0), (30, 0, 0)], active=[0, 0], compute_internalized=True)
    s.initialize()
    before = s.get_field()
    s.run_phases(C.PHASE_CELLS, True)
    f = s.get_field()
    I = s.get_internalized()
    if check:
        _deq(f, before, "all inactive: densities unchanged")
        _deq(I, 0.0, "all inactive: internalized unchanged")
        assert int(s.get_counts().sum()) == 0
    return {"field": f, "int": I}


def golden_reactivation(make, check=True):
    """CellSolverTest.InactiveAgentReactivation (test_cell_solver.cpp:715-763)."""
    name = "CellSolverTest.InactiveAgentReactivation"
    s = C.cell_env(make, 1, (40, 20, 20), True)
    C.set_agents(s, [C.default_agent(0, 1000)], [(10, 0, 0)], active=[1], compute_internalized=True)
    s.initialize()
    s.run_phases(C.PHASE_CELLS, True)
    f1 = s.get_field()[0, 0, 0].copy()
    s.update_agents(is_active=[0])
    s.run_phases(C.PHASE_CELLS, True)
    f2 = s.get_field()[0, 0, 0].copy()
    s.update_agents(is_active=[1])
    s.run_phases(C.PHASE_CELLS, True)
    f3 = s.get_field()[0, 0, 0].copy()
    if check:
        _near(f1[0], C.expect(name, 743))
        _near(f1[1], C.expect(name, 744))
        _near(f2[0], C.expect(name, 752))
        _near(f2[1], C.expect(name, 753))
        _near(f3[0], C.expect(name, 761))
        _near(f3[1], C.expect(name, 762))
    return {"f1": f1, "f2": f2, "f3": f3}


ALL = (
    [(f"uniform{d}d", lambda make, check=True, d=d: golden_uniform(make, d, check)) for d in (1, 2, 3)]
    + [(f"random{d}d", lambda make, check=True, d=d: golden_random(make, d, check)) for d in (1, 2, 3)]
    + [("bulk", golden_bulk)]
    + [(f"interior{d}d", lambda make, check=True, d=d: golden_interior(make, d, check)) for d in (1, 2, 3)]
    + [(f"boundary{d}d", lambda make, check=True, d=d: golden_boundary(make, d, check)) for d in (1, 2, 3)]
    + [("dynamic_boundary", golden_dynamic_boundary), ("dynamic_interior", golden_dynamic_interior),
       ("disable_boundary", golden_disable_boundary), ("multiple_substrates", golden_multiple_substrates)]
    + [(f"simple{d}d_int{int(i)}_rec{int(r)}",
        lambda make, check=True, d=d, i=i, r=r: golden_simple_cells(make, d, i, r, check))
       for d in (1, 2, 3) for i in (True, False) for r in (True, False)]
    + [(f"conflict_int{int(i)}_rec{int(r)}", lambda make, check=True, i=i, r=r: golden_conflict(make, i, r, check))
       for i in (True, False) for r in (True, False)]
    + [(f"conflict_big_int{int(i)}_rec{int(r)}",
        lambda make, check=True, i=i, r=r: golden_conflict_big(make, i, r, check))
       for i in (True, False) for r in (True, False)]
    + [("inactive_skip", golden_inactive_skip), ("all_inactive", golden_all_inactive),
       ("reactivation", golden_reactivation)]
)
