"""Reference test scenarios, rebuilt for any solver with the Solver/OracleSolver API.

Each builder cites the reference gtest it restates (paths relative to
reactions-diffusion/biofvm/kernels/openmp_solver/tests/).  The expected values are
read from tests/golden/reference_golden.json (extracted from those files by
tests/golden/extract_golden.py), by test name and source line.
"""
from __future__ import annotations

import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = json.load(open(os.path.join(HERE, "golden", "reference_golden.json"), encoding="utf-8"))

PHASE_DIFFUSION, PHASE_DIRICHLET, PHASE_BULK, PHASE_CELLS, PHASE_ALL = 1, 2, 4, 8, 15


def golden(test: str) -> dict:
    return GOLDEN["tests"][test]


def expect(test: str, line: int) -> dict:
    for a in golden(test)["asserts"]:
        if a["line"] == line:
            return a
    raise KeyError(f"{test}:{line}")


def expected_array(test: str) -> np.ndarray:
    return np.asarray(golden(test)["arrays"][0]["values"])


# ---------------------------------------------------------------- environments

def default_microenv(make, dims, bbmax, voxel, dt=5.0, D=(4, 2), decay=(5, 3), init=(1, 1)):
    """test_diffusion_solver.cpp:12-34 (also dirichlet :15-37, bulk :14-36, cell :16-40)."""
    s = make()
    s.set_mesh(dims, (0, 0, 0), bbmax, voxel)
    s.set_substrates(dt, D, decay, init)
    return s


def biorobots_microenv(make, dims, bbmax, voxel):
    """test_diffusion_solver.cpp:36-58."""
    return default_microenv(make, dims, bbmax, voxel, dt=0.01, D=(1000, 1000), decay=(0.1, 0.4), init=(0, 0))


# ---------------------------------------------------------------- diffusion

UNIFORM = {  # test_diffusion_solver.cpp:61-134
    1: ("DiffusionSolverTest.Uniform1D", (80, 0, 0), (20, 0, 0), (81, 82)),
    2: ("DiffusionSolverTest.Uniform2D", (800, 800, 0), (20, 20, 0), (106, 107)),
    3: ("DiffusionSolverTest.Uniform3D", (200, 200, 200), (20, 20, 20), (131, 132)),
}


def run_uniform(make, dims):
    name, bbmax, voxel, lines = UNIFORM[dims]
    s = default_microenv(make, dims, bbmax, voxel)
    s.initialize()
    s.run_phases(PHASE_DIFFUSION, False)
    exp = [expect(name, ln) for ln in lines]
    return s, exp


RANDOM = {  # test_diffusion_solver.cpp:136-265
    1: ("DiffusionSolverTest.Random1D", (60, 0, 0)),
    2: ("DiffusionSolverTest.Random2D", (60, 60, 0)),
    3: ("DiffusionSolverTest.Random3D", (60, 60, 60)),
}


def run_random(make, dims):
    name, bbmax = RANDOM[dims]
    s = biorobots_microenv(make, dims, bbmax, (20, 20, 20))
    s.initialize()
    # field[index] = index, index = s + x*S + y*S*nx + z*S*nx*ny (the interleaved layout)
    s.set_field(np.arange(s.voxels * s.S, dtype=np.float64))
    s.run_phases(PHASE_DIFFUSION, False)
    return s, expected_array(name)


# ---------------------------------------------------------------- bulk

def run_bulk(make):
    """test_bulk_solver.cpp:39-98: supply 5, target 6, uptake 7 at (1,1,1,s=0) only."""
    s = default_microenv(make, 3, (100, 100, 100), (20, 20, 20), dt=0.01, init=(10, 1))
    nx, ny, nz = s.grid
    sup = np.zeros((s.S, nz, ny, nx))
    tgt = np.zeros_like(sup)
    upt = np.zeros_like(sup)
    sup[0, 1, 1, 1], tgt[0, 1, 1, 1], upt[0, 1, 1, 1] = 5, 6, 7
    s.set_bulk(2, sup.ravel(), upt.ravel(), tgt.ravel())
    s.initialize()
    s.run_phases(PHASE_BULK, False)
    return s, expect("BulkSolverTest.SimulateBulkSource", 92)


# ---------------------------------------------------------------- Dirichlet

def add_dirichlet_at(s, indices, values):
    """test_dirichlet_solver.cpp:39-60: only the first substrate has a condition."""
    K = len(indices)
    vox = np.array([idx[: s.dims] for idx in indices], dtype=np.uint64).ravel()
    vals = np.zeros((K, s.S))
    conds = np.zeros((K, s.S), dtype=np.uint8)
    vals[:, 0] = values
    conds[:, 0] = 1
    s.set_dirichlet_interior(vox, vals.ravel(), conds.ravel())


def add_boundary_dirichlet(s, faces):
    """test_dirichlet_solver.cpp:62-83: first substrate only; others 42 with no condition."""
    for axis, side, value in faces:
        vals = np.full(s.S, 42.0)
        conds = np.zeros(s.S, dtype=np.uint8)
        vals[0] = value
        conds[0] = 1
        s.set_dirichlet_boundary(axis, side, vals, conds)


INTERIOR = {  # test_dirichlet_solver.cpp:86-198
    1: ((100, 0, 0), (20, 0, 0), [(2, 0, 0)], [41]),
    2: ((60, 60, 0), (20, 20, 0), [(1, 1, 0), (2, 0, 0)], [10, 11]),
    3: ((60, 60, 60), (20, 20, 20), [(1, 1, 1), (1, 0, 2), (0, 1, 2)], [1000, 1001, 1002]),
}


def run_interior(make, dims):
    bbmax, voxel, idx, vals = INTERIOR[dims]
    s = default_microenv(make, dims, bbmax, voxel)
    add_dirichlet_at(s, idx, vals)
    s.initialize()
    s.run_phases(PHASE_DIRICHLET, False)
    return s, list(zip(idx, vals))


BOUNDARY_FACES = [(0, 0, 4), (0, 1, 5), (1, 0, 6), (1, 1, 7), (2, 0, 8), (2, 1, 9)]


def run_boundary(make, dims):
    """test_dirichlet_solver.cpp:200-353 on a 5^dims grid."""
    s = default_microenv(make, dims, (100, 100, 100), (20, 20, 20))
    add_boundary_dirichlet(s, BOUNDARY_FACES[: 2 * dims])
    s.initialize()
    s.run_phases(PHASE_DIRICHLET, False)
    return s


def boundary_expected(dims, nx, ny, nz):
    """The per-voxel substrate-0 value the reference tests assert (later faces win)."""
    exp = np.ones((nz, ny, nx))
    faces = BOUNDARY_FACES[: 2 * dims]
    for axis, side, val in faces:
        sl = [slice(None)] * 3
        n = (nx, ny, nz)[axis]
        sl[2 - axis] = n - 1 if side else 0
        exp[tuple(sl)] = val
    return exp


# ---------------------------------------------------------------- builder-level Dirichlet modification

def builder_env(make, densities, mesh_voxel=10):
    """microenvironment_builder defaults (microenvironment_builder.h:18, :40) with a
    100^3 box of 10-unit voxels, as test_dirichlet_solver.cpp:355-505 builds it."""
    s = make()
    s.set_mesh(3, (0, 0, 0), (100, 100, 100), (mesh_voxel,) * 3)
    s.set_substrates(0.01, [d[0] for d in densities], [d[1] for d in densities], [d[2] for d in densities])
    return s


# ---------------------------------------------------------------- cells

def default_agent(rates_offset, volume):
    """set_default_agent_values (test_cell_solver.cpp:104-126) for S = 2."""
    return dict(sec=[rates_offset + 100, 0], upt=[rates_offset + 200, 0], sat=[rates_offset + 300, 0],
                net=[0, rates_offset + 400], frac=[1, 1], vol=volume)


def set_agents(s, agents, positions, active=None, compute_internalized=False):
    A = len(agents)
    pos = np.array([p[: s.dims] for p in positions], dtype=np.float64).ravel()
    get = lambda k: np.array([a[k] for a in agents], dtype=np.float64).ravel()
    act = np.ones(A, dtype=np.uint8) if active is None else np.asarray(active, dtype=np.uint8)
    s.set_agents(pos, get("sec"), get("sat"), get("upt"), get("net"), get("vol"), act,
                 fraction_released=get("frac"), compute_internalized=compute_internalized)


SIMPLE_MESH = {  # test_cell_solver.cpp:135-391
    1: ((60, 20, 20), [(10, 0, 0), (30, 0, 0), (50, 0, 0)]),
    2: ((60, 60, 20), [(10, 10, 0), (30, 30, 0), (50, 50, 0)]),
    3: ((60, 60, 60), [(10, 10, 10), (30, 30, 30), (50, 50, 50)]),
}


def cell_env(make, dims, bbmax, compute_internalized):
    s = default_microenv(make, dims, bbmax, (20, 20, 20), dt=0.01)
    return s


def serial_expected_densities_1d(field_xs, grid_x, agents, positions, active, dt=0.01, Vv=8000.0):
    """compute_expected_agent_densities_1d (test_cell_solver.cpp:68-102)."""
    S = field_xs.shape[1]
    out = np.zeros_like(field_xs)
    vox = [int((p[0] - 0.0) / 20.0) for p in positions]
    for s in range(S):
        for x in range(grid_x):
            num = den = fac = 0.0
            for i, a in enumerate(agents):
                if vox[i] == x and active[i]:
                    num += a["sec"][s] * a["sat"][s] * dt * a["vol"] / Vv
                    den += (a["sec"][s] + a["upt"][s]) * dt * a["vol"] / Vv
                    fac += a["net"][s] * dt / Vv
            out[x, s] = (field_xs[x, s] + num) / (1 + den) + fac
    return out


def serial_expected_internalized_1d(field_xs, agents, positions, expected, dt=0.01, Vv=8000.0):
    """compute_expected_agent_internalized_1d (test_cell_solver.cpp:42-66)."""
    for i, a in enumerate(agents):
        x = int(positions[i][0] / 20.0)
        for s in range(field_xs.shape[1]):
            num = a["sec"][s] * a["sat"][s] * dt * a["vol"]
            denom = (a["sec"][s] + a["upt"][s]) * dt * a["vol"] / Vv
            factor = a["net"][s] * dt
            expected[i, s] -= (Vv * -denom * field_xs[x, s] + num) + factor
    return expected


def conflict_agents():
    """RecomputeTest.Conflict agents (test_cell_solver.cpp:411-418)."""
    agents = [default_agent(0, 500), default_agent(600, 1000), default_agent(1100, 1500),
              default_agent(1600, 2000), default_agent(2100, 2500), default_agent(2600, 3000)]
    positions = [(10, 0, 0), (30, 0, 0), (30, 0, 0), (50, 0, 0), (50, 0, 0), (50, 0, 0)]
    return agents, positions


def conflict_big_agents():
    """RecomputeTest.ConflictBig: 50 agents at each of 100 voxel centres (test_cell_solver.cpp:493-512)."""
    agents, positions = [], []
    for i in range(100):
        for _ in range(50):
            agents.append(default_agent(0, 500))
            positions.append((i * 20 + 10.0, 0, 0))
    return agents, positions
