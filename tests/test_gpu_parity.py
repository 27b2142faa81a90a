"""Randomised parity of the GB300 path against the FP64 oracle.

Small random problems cover every branch (dims 1-3, n = 1 axes, 1-9 substrates,
random faces and conditions, interior nodes, uniform and per-voxel bulk tables,
colliding and inactive agents, internalized tracking on and off, multi-step solves,
recompute after agent moves).  Tolerances: 1e-12 relative (FP64 build), 1e-5
relative (FP32 build), normalised per substrate by max |oracle|.  Ballot counts
and the conflict flag are integers and must be identical.
"""
import zlib

import numpy as np
import pytest

from physicore_gb300 import workloads as W
from test_gpu_golden import rel_err

pytestmark = pytest.mark.gpu

SEEDS = list(range(40))


def run_both(pcg, oracle_mod, p, precision, steps=(1, 2, 1), threads=2):
    g = W.apply(pcg.Solver(precision), p)
    o = W.apply(oracle_mod.OracleSolver(threads=threads), p)
    rng = np.random.default_rng(1000 + zlib.crc32(p["name"].encode()) % 1000)
    snaps = []
    for k, n in enumerate(steps):
        if k == 2 and g.A > 0:
            # agents move, one toggles activity; both solvers are told to recompute
            a = p["agents"]
            pos = a["positions"].copy()
            order = rng.permutation(g.A)
            pos = pos[order]
            act = a["is_active"].copy()
            act[rng.integers(0, g.A)] ^= 1
            for s in (g, o):
                s.update_agents(positions=pos, is_active=act)
                s.recompute_positional_data()
        g.solve(n)
        o.solve(n)
        snap = dict(field=(g.get_field(), o.get_field()))
        if g.A:
            snap["internalized"] = (g.get_internalized(), o.get_internalized())
            snap["counts"] = (g.get_counts(), o.get_counts())
            snap["conflict"] = (g.get_conflict(), o.get_conflict())
        snaps.append(snap)
    return snaps


def check(snaps, rtol, name, voxel_volume=None, den_max=0.0):
    """Fields: rtol relative per substrate.  With voxel_volume given (FP32 build),
    internalized amounts are held to rtol * Vv * max|field| * (1 + den_max): they are
    FP64 sums of FP32 densities, differenced (Vv*(D - D')) or, after a ballot
    conflict, multiplied by the agent's denominator (Vv*D'*den, cell_solver.cpp:
    140-142), so the FP32 rounding of D' enters scaled by Vv and by den."""
    for k, snap in enumerate(snaps):
        for key, (got, ref) in snap.items():
            if key in ("counts", "conflict"):
                assert np.array_equal(np.asarray(got), np.asarray(ref)), f"{name} step {k}: {key} differ"
            elif key == "internalized" and voxel_volume is not None:
                fmax = np.abs(snap["field"][1]).reshape(-1, ref.shape[-1]).max(axis=0)
                scale = np.maximum(voxel_volume * fmax * (1.0 + den_max), 1e-30)
                e = float((np.abs(got - ref) / scale).max()) if ref.size else 0.0
                assert e <= rtol, f"{name} step {k}: internalized error {e:.3e} of Vv*max|D| > {rtol}"
            else:
                e = rel_err(got, ref)
                assert e <= rtol, f"{name} step {k}: {key} relative error {e:.3e} > {rtol}"


@pytest.mark.parametrize("seed", SEEDS)
def test_random_fp64(pcg, oracle_mod, seed):
    p = W.random_small(seed)
    check(run_both(pcg, oracle_mod, p, pcg.FP64), 1e-12, p["name"])


def max_denominator(p):
    """Largest agent denominator (U+S)*dt*Vc/Vv of the problem (cell_solver.cpp:70-72)."""
    a = p.get("agents")
    if a is None or not len(a["volumes"]):
        return 0.0
    Vv = float(np.prod(p["voxel"]))
    den = (a["uptake"] + a["secretion"]) * p["dt"] * a["volumes"][:, None] / Vv
    return float(den.max())


@pytest.mark.parametrize("seed", SEEDS)
def test_random_fp32(pcg, oracle_mod, seed):
    p = W.random_small(seed)
    check(run_both(pcg, oracle_mod, p, pcg.FP32), 1e-5, p["name"], voxel_volume=float(np.prod(p["voxel"])),
          den_max=max_denominator(p))


@pytest.mark.parametrize("shape,S", [((6, 300, 5), 3), ((5, 4, 330), 2), ((4, 264, 250), 5), ((3, 7, 420), 1)])
def test_long_lines_with_faces(pcg, oracle_mod, shape, S):
    """y/z lines longer than the 216 points an FP32 tile keeps in shared memory
    (the rest of each line is held in registers), with Dirichlet on all six faces
    written by the last sweep, interior nodes and agents, against the oracle."""
    rng = np.random.default_rng(sum(shape) * 7 + S)
    nx, ny, nz = shape
    pos = rng.random((400, 3)) * np.array(shape) * 10.0
    ag = W.agents_block(rng, 400, S, pos)
    vox = np.stack([rng.integers(0, v, 30) for v in shape], axis=1).astype(np.uint64)
    lin = np.unique(vox[:, 0] + nx * (vox[:, 1] + ny * vox[:, 2]))
    vox = np.stack([lin % nx, (lin // nx) % ny, lin // (nx * ny)], axis=1).astype(np.uint64)
    p = dict(name=f"long_{nx}x{ny}x{nz}_{S}", dims=3, bbmin=(0, 0, 0), bbmax=(nx * 10, ny * 10, nz * 10),
             voxel=(10, 10, 10), dt=0.05, D=W.log_uniform(rng, 1, 1e4, S), decay=W.log_uniform(rng, 1e-3, 1, S),
             initial=np.zeros(S), field=rng.random((nz, ny, nx, S)), field_layout="interleaved",
             boundary=[(ax, side, rng.random(S), [1] * S) for ax in range(3) for side in (0, 1)],
             interior=(vox, rng.random((len(vox), S)), np.ones((len(vox), S), np.uint8)), bulk=None,
             agents=ag, compute_internalized=True)
    check(run_both(pcg, oracle_mod, p, pcg.FP32), 1e-5, p["name"], voxel_volume=1000.0, den_max=max_denominator(p))


@pytest.mark.parametrize("n,S", [(1, 1), (2, 3), (3, 5), (4, 2), (33, 7), (64, 1), (65, 4), (130, 2), (320, 1)])
def test_sweep_line_lengths(pcg, oracle_mod, n, S):
    """Line lengths around the 16-byte vector and 32-lane tile edges, in every axis."""
    rng = np.random.default_rng(n * 31 + S)
    for dims, shape in [(1, (n, 1, 1)), (2, (5, n, 1)), (3, (3, 4, n)), (3, (n, 3, 2))]:
        p = dict(name=f"lines_{n}_{S}_{dims}", dims=dims, bbmin=(0, 0, 0),
                 bbmax=tuple(shape[a] * 10 if a < dims else 0 for a in range(3)), voxel=(10, 10, 10), dt=0.05,
                 D=W.log_uniform(rng, 1, 1e4, S), decay=W.log_uniform(rng, 1e-3, 1, S), initial=np.zeros(S),
                 field=rng.random((shape[2], shape[1], shape[0], S)), field_layout="interleaved", boundary=[],
                 interior=None, bulk=None, agents=None, compute_internalized=False)
        for prec, tol in ((pcg.FP64, 1e-12), (pcg.FP32, 1e-5)):
            g = W.apply(pcg.Solver(prec), p)
            o = W.apply(oracle_mod.OracleSolver(threads=2), p)
            g.solve(3)
            o.solve(3)
            e = rel_err(g.get_field(), o.get_field())
            assert e <= tol, f"{p['name']} prec {prec}: {e:.3e}"


def test_layouts_round_trip(pcg):
    p = W.random_small(7)
    g = W.apply(pcg.Solver(pcg.FP64), p)
    f = g.get_field()
    planar = g.get_field(layout=pcg.LAYOUT_PLANAR)
    assert np.array_equal(np.moveaxis(planar, 0, -1), f)
    g.set_field(planar, layout=pcg.LAYOUT_PLANAR)
    assert np.array_equal(g.get_field(), f)
    f32 = g.get_field(dtype=np.float32)
    assert np.array_equal(f32, f.astype(np.float32))
    nx, ny, nz = g.grid
    for _ in range(5):
        s, x, y, z = [int(np.random.randint(0, m)) for m in (g.S, nx, ny, nz)]
        assert g.get_density(s, x, y, z) == f[z, y, x, s]


def test_layouts_pinned_host_buffers(pcg):
    """Pinned host buffers (copied without driver staging) give the same fields as
    pageable ones, in every layout and element type."""
    torch = pytest.importorskip("torch")
    for prec in (pcg.FP64, pcg.FP32):
        p = W.random_small(11)
        g = W.apply(pcg.Solver(prec), p)
        g.solve(2)
        for layout in (pcg.LAYOUT_INTERLEAVED, pcg.LAYOUT_PLANAR):
            for dt in (np.float32, np.float64):
                ref = g.get_field(layout=layout, dtype=dt)
                pinned = torch.empty(ref.shape, dtype=torch.float32 if dt == np.float32 else torch.float64,
                                     pin_memory=True).numpy()
                pinned[...] = -1
                g.get_field(layout=layout, dtype=dt, out=pinned)
                assert np.array_equal(pinned, ref), (prec, layout, dt)
        f = g.get_field()
        for layout in (pcg.LAYOUT_INTERLEAVED, pcg.LAYOUT_PLANAR):
            src = f if layout == pcg.LAYOUT_INTERLEAVED else np.ascontiguousarray(np.moveaxis(f, -1, 0))
            pinned = torch.empty(src.shape, dtype=torch.float64, pin_memory=True).numpy()
            pinned[...] = src * 0.5
            g.set_field(pinned, layout=layout)
            back = g.get_field()
            expect = (f * 0.5).astype(np.float32).astype(np.float64) if prec == pcg.FP32 else f * 0.5
            assert np.array_equal(back, expect), (prec, layout)
            g.set_field(f)


def test_field_readback_async(pcg):
    """Readbacks overlapped with the following steps (two staging slots in turn)
    deliver each step's field; a twin solver without agents (deterministic) gives
    the expected fields.  Pageable buffers fall back to a synchronous readback."""
    torch = pytest.importorskip("torch")
    p = W.random_small(12)
    p["agents"] = None
    g = W.apply(pcg.Solver(pcg.FP32), p)
    twin = W.apply(pcg.Solver(pcg.FP32), p)
    nx, ny, nz = g.grid
    shape = (g.S, nz, ny, nx)
    bufs = [torch.empty(shape, dtype=torch.float32, pin_memory=True).numpy() for _ in range(2)]
    expect, tickets = [], []
    for k in range(6):
        g.solve(1)
        twin.solve(1)
        expect.append(twin.get_field(layout=pcg.LAYOUT_PLANAR, dtype=np.float32))
        tickets.append(g.get_field_async(bufs[k % 2], layout=pcg.LAYOUT_PLANAR))
        if k:  # the previous step's field, read while this step's readback runs
            g.wait_field(tickets[k - 1])
            assert np.array_equal(bufs[(k - 1) % 2], expect[k - 1]), k - 1
    g.wait_field(tickets[-1])
    assert np.array_equal(bufs[5 % 2], expect[5])
    out = np.empty(shape, np.float32)
    g.wait_field(g.get_field_async(out, layout=pcg.LAYOUT_PLANAR))
    assert np.array_equal(out, expect[5])
    with pytest.raises(pcg.PcgError):
        g.wait_field(10 ** 6)


def test_mass_identity_pure_diffusion(pcg):
    """Without Dirichlet, bulk or agents each sweep scales the mass of substrate s by
    exactly 1/(1 + decay*dt/dims) (column sums of the ADI matrix)."""
    rng = np.random.default_rng(5)
    S = 3
    D = np.array([10.0, 1e3, 1e5])
    decay = np.array([0.1, 0.5, 1e-3])
    p = dict(name="mass", dims=3, bbmin=(0, 0, 0), bbmax=(400, 300, 200), voxel=(10, 10, 10), dt=0.01, D=D,
             decay=decay, initial=np.zeros(S), field=rng.random((20, 30, 40, S)), field_layout="interleaved",
             boundary=[], interior=None, bulk=None, agents=None, compute_internalized=False)
    g = W.apply(pcg.Solver(pcg.FP64), p)
    m0 = g.mass()
    g.solve(4)
    m1 = g.mass()
    expect = m0 * (1.0 / (1.0 + decay * 0.01 / 3)) ** (3 * 4)
    assert np.allclose(m1, expect, rtol=1e-12, atol=0)


def test_agent_outside_mesh_reports_error(pcg):
    p = W.random_small(3)
    g = W.apply(pcg.Solver(pcg.FP64), p)
    if g.A == 0:
        pytest.skip("no agents in this draw")
    pos = p["agents"]["positions"].copy()
    act = np.ones(g.A, np.uint8)
    pos[0, 0] = p["bbmax"][0] + 1e6  # far outside: the kernel flags it, never indexes with it
    g.update_agents(positions=pos, is_active=act)
    g.recompute_positional_data()
    g.solve(1)
    with pytest.raises(pcg.PcgError) as ei:
        g.synchronize()
    assert ei.value.code == 4 and "outside" in str(ei.value)
