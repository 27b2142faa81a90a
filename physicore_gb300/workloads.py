"""Seeded synthetic BioFVM problems.

One generator feeds both the GB300 path and the CPU oracle, so the two always
consume identical inputs.  Every array is produced by numpy's PCG64 generator,
which gives the same bits on x86 and Arm hosts.

Named workloads restate the benchmark configurations of this backend:
  plain_100     100^3 voxels of 20 um, 1 substrate, D=1000, decay 0.1, dt=0.01,
                field 0, Dirichlet 1.0 on all six faces, 1,000 interior agents
  large_320     320^3 voxels, 8 substrates with D log-uniform [10, 1e5] and
                decay log-uniform [1e-4, 1], field U[0,1], Dirichlet on the x faces
                plus 10,000 interior voxels, 1,000,000 agents
  dense_200     200^3 voxels, 4 substrates, 4,000,000 agents from a Gaussian
                cluster (sigma 200 um) at the domain centre
  batched_256   256 independent domains, each side log-uniform in [32, 160] voxels
                per axis, 1-6 substrates, 100-50,000 agents (log-uniform), with the
                per-domain recipe of large_320 (D, decay, field, x-face Dirichlet,
                interior nodes at the same density)
  served        a Poisson request stream of independent simulations (sides
                log-uniform [32, 256] per axis, 1-8 substrates, 0-200,000 agents,
                10-1,000 steps log-uniform)
A problem is a plain dict; `apply(solver, problem)` feeds it to any object with
the Solver call surface (physicore_gb300.Solver or the oracle).
"""
from __future__ import annotations

import math

import numpy as np

VOXEL = 20


def _rng(seed):
    return np.random.Generator(np.random.PCG64(seed))


def log_uniform(rng, lo, hi, size=None):
    return np.exp(rng.uniform(math.log(lo), math.log(hi), size))


def agents_block(rng, A, S, positions, secretion_hi=1.0, uptake_hi=0.5, volume=2494.0, active_frac=1.0,
                 net_export_hi=0.0):
    """Agent SoA with the rates of the plain benchmark: secretion U[0,1], saturation
    1.0, uptake U[0,0.5] per substrate, volume 2494 um^3."""
    sec = rng.uniform(0.0, secretion_hi, (A, S))
    upt = rng.uniform(0.0, uptake_hi, (A, S))
    sat = np.ones((A, S))
    net = rng.uniform(0.0, net_export_hi, (A, S)) if net_export_hi > 0 else np.zeros((A, S))
    vol = np.full(A, volume)
    active = (rng.random(A) < active_frac).astype(np.uint8) if active_frac < 1 else np.ones(A, np.uint8)
    return dict(positions=np.ascontiguousarray(positions, dtype=np.float64), secretion=sec, saturation=sat,
                uptake=upt, net_export=net, volumes=vol, is_active=active,
                fraction_released=np.ones((A, S)))


def uniform_positions(rng, A, dims, lo, hi):
    """U[lo, hi) per axis; never equal to hi (that would index past the grid)."""
    p = rng.uniform(lo, hi, (A, dims))
    return np.minimum(p, np.nextafter(np.asarray(hi, dtype=np.float64), -np.inf))


def plain_100(seed=0, n=100, agents=1000):
    """The plain single-domain workload (FP64 in the reference's own example)."""
    rng = _rng(seed)
    ext = n * VOXEL
    pos = uniform_positions(rng, agents, 3, VOXEL, ext - VOXEL)
    return dict(name=f"plain_{n}", dims=3, bbmin=(0, 0, 0), bbmax=(ext,) * 3, voxel=(VOXEL,) * 3, dt=0.01,
                D=[1000.0], decay=[0.1], initial=[0.0], field=None,
                boundary=[(a, s, [1.0], [1]) for a in range(3) for s in range(2)],
                interior=None, bulk=None, agents=agents_block(rng, agents, 1, pos), compute_internalized=True)


def large(seed=1, n=320, S=8, agents=1_000_000, interior=10_000, field_dtype=np.float32):
    rng = _rng(seed)
    ext = n * VOXEL
    D = log_uniform(rng, 10.0, 1e5, S)
    decay = log_uniform(rng, 1e-4, 1.0, S)
    field = rng.random((S, n, n, n), dtype=np.float32 if field_dtype == np.float32 else np.float64)
    faces = [(0, side, rng.random(S), [1] * S) for side in (0, 1)]
    vox = rng.integers(0, n, (interior, 3), dtype=np.uint64)
    # distinct interior nodes (the reference's update path never duplicates a node)
    lin = np.unique(vox[:, 0] + n * (vox[:, 1] + n * vox[:, 2]))
    vox = np.stack([lin % n, (lin // n) % n, lin // (n * n)], axis=1).astype(np.uint64)
    K = vox.shape[0]
    inter = (vox, rng.random((K, S)), np.ones((K, S), np.uint8))
    pos = uniform_positions(rng, agents, 3, 0.0, float(ext))
    return dict(name=f"large_{n}", dims=3, bbmin=(0, 0, 0), bbmax=(ext,) * 3, voxel=(VOXEL,) * 3, dt=0.01,
                D=D, decay=decay, initial=np.zeros(S), field=field, field_layout="planar", boundary=faces,
                interior=inter, bulk=None, agents=agents_block(rng, agents, S, pos), compute_internalized=True)


def dense(seed=2, n=200, S=4, agents=4_000_000, sigma=200.0):
    rng = _rng(seed)
    ext = n * VOXEL
    D = log_uniform(rng, 10.0, 1e5, S)
    decay = log_uniform(rng, 1e-4, 1.0, S)
    field = rng.random((S, n, n, n), dtype=np.float32)
    pos = rng.normal(ext / 2.0, sigma, (agents, 3))
    pos = np.clip(pos, 0.0, np.nextafter(float(ext), 0.0))
    return dict(name=f"dense_{n}", dims=3, bbmin=(0, 0, 0), bbmax=(ext,) * 3, voxel=(VOXEL,) * 3, dt=0.01,
                D=D, decay=decay, initial=np.zeros(S), field=field, field_layout="planar", boundary=[],
                interior=None, bulk=None, agents=agents_block(rng, agents, S, pos), compute_internalized=True)


def random_small(seed, max_side=24, max_S=9, max_agents=300, allow_bulk=True):
    """A small random problem that exercises every branch: dims 1..3, sides 1..max_side
    (n=1 axes included), S 1..max_S, random faces/conditions, interior nodes, bulk
    tables, colliding and inactive agents, internalized tracking on or off."""
    rng = _rng(seed)
    dims = int(rng.integers(1, 4))
    voxel = tuple(int(v) for v in rng.choice([5, 10, 20, 25], 3))
    sides = [int(rng.integers(1, max_side + 1)) if a < dims else 1 for a in range(3)]
    if rng.random() < 0.15:
        sides[int(rng.integers(0, dims))] = 1
    bbmin = tuple(int(v) for v in rng.integers(-100, 100, 3))
    # bbox extents that are not always a multiple of the voxel (ceil in the mesh)
    bbmax = tuple(bbmin[a] + max(1, sides[a] * voxel[a] - int(rng.integers(0, voxel[a]))) for a in range(3))
    S = int(rng.integers(1, max_S + 1))
    dt = float(rng.choice([0.01, 0.1, 1.0]))
    D = log_uniform(rng, 1.0, 1e4, S)
    decay = log_uniform(rng, 1e-3, 2.0, S)
    initial = rng.random(S)
    grid = [-(-(bbmax[a] - bbmin[a]) // voxel[a]) if a < dims else 1 for a in range(3)]
    nx, ny, nz = grid
    field = rng.random((nz, ny, nx, S)) * 10.0
    boundary = []
    for a in range(dims):
        for side in (0, 1):
            if rng.random() < 0.5:
                boundary.append((a, side, rng.random(S) * 5.0, (rng.random(S) < 0.7).astype(np.uint8)))
    interior = None
    V = nx * ny * nz
    if rng.random() < 0.6 and V > 1:
        K = int(rng.integers(1, min(V, 20) + 1))
        lin = rng.choice(V, K, replace=False)
        vox = np.stack([lin % nx, (lin // nx) % ny, lin // (nx * ny)], axis=1)[:, :dims].astype(np.uint64)
        interior = (vox, rng.random((K, S)) * 3.0, (rng.random((K, S)) < 0.7).astype(np.uint8))
    bulk = None
    if allow_bulk and rng.random() < 0.4:
        if rng.random() < 0.5:
            bulk = (1, rng.random(S), rng.random(S), rng.random(S) * 4)
        else:
            bulk = (2, rng.random(S * V), rng.random(S * V), rng.random(S * V) * 4)
    A = int(rng.integers(0, max_agents + 1))
    lo = np.array(bbmin[:dims], dtype=np.float64)
    hi = np.array([bbmin[a] + grid[a] * voxel[a] for a in range(dims)], dtype=np.float64)
    hi = np.minimum(hi, np.array(bbmax[:dims], dtype=np.float64))
    pos = uniform_positions(rng, A, dims, lo, hi)
    if A > 4:  # force collisions: copy some agents onto others' positions
        k = A // 3
        pos[rng.choice(A, k, replace=False)] = pos[rng.choice(A, k, replace=True)]
    ag = agents_block(rng, A, S, pos, secretion_hi=20.0, uptake_hi=10.0, volume=float(rng.uniform(100, 3000)),
                      active_frac=0.85, net_export_hi=2.0)
    ag["volumes"] = rng.uniform(100, 3000, A)
    return dict(name=f"random_{seed}", dims=dims, bbmin=bbmin, bbmax=bbmax, voxel=voxel, dt=dt, D=D, decay=decay,
                initial=initial, field=field, field_layout="interleaved", boundary=boundary, interior=interior,
                bulk=bulk, agents=ag, compute_internalized=bool(rng.random() < 0.6))


def apply(solver, p, with_field=True, with_agents=True, initialize=True):
    """Feeds problem `p` to `solver` and initialises it (with initialize=False the
    solver stays uninitialised, holding no device memory, and the initial field is
    the uniform initial conditions: a request for the simulation server)."""
    solver.set_mesh(p["dims"], p["bbmin"], p["bbmax"], p["voxel"])
    solver.set_substrates(p["dt"], p["D"], p["decay"], p["initial"])
    for axis, side, vals, conds in p["boundary"]:
        solver.set_dirichlet_boundary(axis, side, vals, conds)
    if p.get("interior") is not None:
        vox, vals, conds = p["interior"]
        solver.set_dirichlet_interior(vox[:, : p["dims"]], vals, conds)
    if p.get("bulk") is not None:
        solver.set_bulk(*p["bulk"])
    if with_agents and p.get("agents") is not None and len(p["agents"]["volumes"]):
        a = p["agents"]
        solver.set_agents(a["positions"], a["secretion"], a["saturation"], a["uptake"], a["net_export"],
                          a["volumes"], a["is_active"], fraction_released=a["fraction_released"],
                          compute_internalized=p["compute_internalized"])
    if not initialize:
        return solver
    solver.initialize()
    if with_field and p.get("field") is not None:
        f = p["field"]
        if p.get("field_layout") == "planar":
            solver.set_field(f, layout=1) if _takes_layout(solver) else solver.set_field(
                np.ascontiguousarray(np.moveaxis(f, 0, -1), dtype=np.float64))
        else:
            solver.set_field(f)
    return solver


def _takes_layout(solver):
    import inspect
    try:
        return "layout" in inspect.signature(solver.set_field).parameters
    except (TypeError, ValueError):
        return False


def _domain(rng, name, sides, S, A, interior_density=1e4 / 320 ** 3):
    """One 3-D domain with the per-domain recipe of large_320."""
    nx, ny, nz = sides
    ext = [n * VOXEL for n in sides]
    D = log_uniform(rng, 10.0, 1e5, S)
    decay = log_uniform(rng, 1e-4, 1.0, S)
    field = rng.random((S, nz, ny, nx), dtype=np.float32)
    faces = [(0, side, rng.random(S), [1] * S) for side in (0, 1)]
    V = nx * ny * nz
    K = int(round(V * interior_density))
    inter = None
    if K:
        lin = np.unique(rng.integers(0, V, K))
        vox = np.stack([lin % nx, (lin // nx) % ny, lin // (nx * ny)], axis=1).astype(np.uint64)
        inter = (vox, rng.random((vox.shape[0], S)), np.ones((vox.shape[0], S), np.uint8))
    pos = uniform_positions(rng, A, 3, np.zeros(3), np.array(ext, dtype=np.float64))
    return dict(name=name, dims=3, bbmin=(0, 0, 0), bbmax=tuple(ext), voxel=(VOXEL,) * 3, dt=0.01, D=D,
                decay=decay, initial=np.zeros(S), field=field, field_layout="planar", boundary=faces,
                interior=inter, bulk=None, agents=agents_block(rng, A, S, pos), compute_internalized=True)


def batched_sizes(seed=3, count=256, side_lo=32, side_hi=160, S_hi=6, agents_lo=100, agents_hi=50_000):
    """(sides, S, agents) of the batched workload's domains, without their arrays."""
    rng = _rng(seed)
    out = []
    for _ in range(count):
        sides = tuple(int(round(v)) for v in log_uniform(rng, side_lo, side_hi, 3))
        S = int(rng.integers(1, S_hi + 1))
        A = int(round(float(log_uniform(rng, agents_lo, agents_hi))))
        out.append((sides, S, A))
    return out


def batched_uneven(seed=3, count=256, **kw):
    """Yields the batched workload's domains one at a time (their fields are large
    together: about 1.8 GB of FP32 for 256 domains)."""
    for i, (sides, S, A) in enumerate(batched_sizes(seed, count, **kw)):
        yield _domain(_rng((seed, i)), f"batched_{i}", sides, S, A)


class ServedStream:
    """The served request stream: Poisson arrivals at `rate` per second for
    `duration` seconds; each request a 3-D domain with sides log-uniform in
    [32, 256] voxels per axis, 1-8 substrates, D and decay as large_320, initial
    conditions U[0,1], 0-200,000 uniform agents (internalized tracking on) and a
    step count log-uniform in [10, 1000].  Agent rates come from pools shared by all
    requests of a substrate count (synthetic inputs; only positions are drawn per
    request), so that building a request costs little host time."""

    def __init__(self, seed=4, rate=200.0, duration=10.0, side_lo=32, side_hi=256, S_hi=8, agents_hi=200_000,
                 steps_lo=10, steps_hi=1000):
        rng = _rng(seed)
        n = int(rng.poisson(rate * duration))
        self.arrivals = np.sort(rng.uniform(0.0, duration, n))
        self.sides = np.rint(log_uniform(rng, side_lo, side_hi, (n, 3))).astype(np.int64)
        self.S = rng.integers(1, S_hi + 1, n)
        self.A = rng.integers(0, agents_hi + 1, n)
        self.steps = np.rint(log_uniform(rng, steps_lo, steps_hi, n)).astype(np.int64)
        self.D = [log_uniform(rng, 10.0, 1e5, int(S)) for S in self.S]
        self.decay = [log_uniform(rng, 1e-4, 1.0, int(S)) for S in self.S]
        self.initial = [rng.random(int(S)) for S in self.S]
        self.seeds = rng.integers(0, 2 ** 31, n)
        self._unit = rng.random((agents_hi, 3))
        self._pools = {}
        for S in range(1, S_hi + 1):
            blk = agents_block(rng, agents_hi, S, np.zeros((agents_hi, 3)))
            self._pools[S] = {k: np.ascontiguousarray(blk[k]) for k in
                              ("secretion", "saturation", "uptake", "net_export", "volumes", "is_active",
                               "fraction_released")}

    def __len__(self):
        return len(self.arrivals)

    def vss(self, i):
        return int(np.prod(self.sides[i])) * int(self.S[i]) * int(self.steps[i])

    def request(self, solver, i):
        """Configures `solver` (not initialised) as request i."""
        nx, ny, nz = (int(v) for v in self.sides[i])
        S, A = int(self.S[i]), int(self.A[i])
        ext = np.array([nx, ny, nz], dtype=np.float64) * VOXEL
        solver.set_mesh(3, (0, 0, 0), tuple(int(v) for v in ext), (VOXEL,) * 3)
        solver.set_substrates(0.01, self.D[i], self.decay[i], self.initial[i])
        if A:
            pool = self._pools[S]
            pos = np.minimum(self._unit[:A] * ext, np.nextafter(ext, 0.0))
            solver.set_agents(pos, pool["secretion"][:A], pool["saturation"][:A], pool["uptake"][:A],
                              pool["net_export"][:A], pool["volumes"][:A], pool["is_active"][:A],
                              fraction_released=pool["fraction_released"][:A], compute_internalized=True)
        return solver
