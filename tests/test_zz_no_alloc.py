"""The allocation-free cell step (pcg_cells_noalloc).

pcg_cells_noalloc serves callers that cannot let a library allocate device memory
(frameworks that own all GPU memory through their own pool, loops that must avoid
cudaMalloc's synchronisation).  Here the caller's buffers are ordinary device
tensors; the entry point itself allocates nothing and takes its scratch from a
fixed device array shared by every call.

GPU tests: two cell passes in a row through the C ABI must match two passes of
the FP64 oracle's cell phase with the ballots rebuilt (run_phases(PHASE_CELLS,
recompute=1)), and two passes of the regular entry point (pcg_run_phases on an
FP32 context), within the FP32 tolerances of the other GPU tests; per-voxel
counts are not returned by this entry point, so the ballot is checked through the
densities.  Cases cover the scalar row path (S = 3, unpadded rows) and the 16-byte
row path (S = 4 and 8, padded rows whose padding must stay untouched), and a small
problem right after a large one on the shared scratch.

CPU tests: oversized, overflowing and malformed problems are rejected before any
device work.  This file is collected last.
"""
import ctypes

import numpy as np
import pytest

from physicore_gb300 import workloads as W

FP32_RTOL = 1e-5
PAD = 12345.0


def _problem(seed, S, n, agents, share=0.25):
    rng = np.random.default_rng(seed)
    pos = W.uniform_positions(rng, agents, 3, 0.0, np.array(n, dtype=np.float64) * 20.0)
    k = int(agents * share)
    pos[:k] = pos[k:2 * k]  # shared voxels: ballot conflicts
    ag = W.agents_block(rng, agents, S, pos, net_export_hi=0.5)
    ag["volumes"] = rng.uniform(500.0, 3000.0, agents)
    ag["is_active"][rng.integers(0, agents, max(1, agents // 50))] = 0
    return dict(name=f"noalloc_{seed}", dims=3, bbmin=(0, 0, 0), bbmax=tuple(v * 20 for v in n),
                voxel=(20, 20, 20), dt=0.01, D=np.geomspace(10.0, 1e4, S), decay=np.geomspace(1e-3, 0.5, S),
                initial=np.zeros(S), field=rng.random((n[2], n[1], n[0], S)), field_layout="interleaved",
                boundary=[], interior=None, bulk=None, agents=ag, compute_internalized=True)


def _fn(pcg):
    L = pcg.load_library()
    f = L.pcg_cells_noalloc
    P, u64 = ctypes.c_void_p, ctypes.c_uint64
    f.argtypes = [P, u64, ctypes.c_int, P, P, P, u64, ctypes.c_double, u64, P, P, P, P, P, P, P, P, ctypes.c_int, P]
    f.restype = ctypes.c_int
    return L, f


def _rel(got, ref):
    norm = np.maximum(np.abs(ref).reshape(-1, ref.shape[-1]).max(axis=0), 1e-30)
    return float((np.abs(got - ref).reshape(-1, ref.shape[-1]) / norm).max())


class Caller:
    """A caller's own device buffers for problem p, the field with row pitch `pitch`
    (padding filled with PAD)."""

    def __init__(self, torch, p, pitch):
        self.torch = torch
        nx, ny, nz = (p["bbmax"][d] // p["voxel"][d] for d in range(3))
        S = len(p["D"])
        self.grid, self.S, self.pitch, self.p = (nx, ny, nz), S, pitch, p
        dev = torch.device("cuda", 0)
        host = np.full((nz * ny, pitch), PAD, dtype=np.float32)
        host[:, : nx * S] = p["field"].reshape(nz * ny, nx * S).astype(np.float32)
        self.field = torch.from_numpy(host).to(dev)
        a = p["agents"]
        self.t = {k: torch.from_numpy(np.ascontiguousarray(a[k], dtype=np.float64).reshape(-1)).to(dev)
                  for k in ("positions", "secretion", "saturation", "uptake", "net_export", "volumes")}
        self.active = torch.from_numpy(a["is_active"].astype(np.uint8)).to(dev)
        self.internal = torch.zeros(len(a["volumes"]) * S, dtype=torch.float64, device=dev)
        self.bbmin = np.zeros(3, dtype=np.int64)
        self.voxel = np.array(p["voxel"], dtype=np.uint64)
        self.gridv = np.array(self.grid, dtype=np.uint64)

    def call(self, fn):
        t = self.t
        return fn(self.field.data_ptr(), self.pitch, 3, self.bbmin.ctypes.data, self.voxel.ctypes.data,
                  self.gridv.ctypes.data, self.S, self.p["dt"], len(self.p["agents"]["volumes"]),
                  t["positions"].data_ptr(), t["secretion"].data_ptr(), t["saturation"].data_ptr(),
                  t["uptake"].data_ptr(), t["net_export"].data_ptr(), t["volumes"].data_ptr(),
                  self.active.data_ptr(), self.internal.data_ptr(), 1,
                  self.torch.cuda.current_stream().cuda_stream)

    def get_field(self):
        nx, ny, nz = self.grid
        f = self.field.cpu().numpy()
        assert np.all(f[:, nx * self.S:] == PAD), "the row padding was written"
        return f[:, : nx * self.S].astype(np.float64).reshape(nz, ny, nx, self.S)

    def get_internalized(self):
        return self.internal.cpu().numpy().reshape(-1, self.S)


def _internalized_scale(p, field_ref):
    a = p["agents"]
    Vv = float(np.prod(p["voxel"]))
    den = (a["uptake"] + a["secretion"]) * p["dt"] * a["volumes"][:, None] / Vv
    # FP32 densities enter the internalized amounts scaled by Vv (and by den after a conflict)
    return Vv * np.abs(field_ref).reshape(-1, field_ref.shape[-1]).max(axis=0) * (1.0 + den.max())


def _check_two_calls(pcg, oracle_mod, torch, noalloc, L, p, pitch):
    caller = Caller(torch, p, pitch)
    regular = W.apply(pcg.Solver(pcg.FP32), p)
    oracle = W.apply(oracle_mod.OracleSolver(threads=4), p)
    for call in range(2):
        rc = caller.call(noalloc)
        assert rc == 0, L.pcg_last_error().decode()
        torch.cuda.synchronize()
        regular.run_phases(pcg.PHASE_CELLS, True)
        oracle.run_phases(pcg.PHASE_CELLS, True)
        f_got, f_ora, f_reg = caller.get_field(), oracle.get_field(), regular.get_field()
        e_ora, e_reg = _rel(f_got, f_ora), _rel(f_got, f_reg)
        assert e_ora <= FP32_RTOL, f"{p['name']} call {call}: field vs oracle {e_ora:.3e}"
        assert e_reg <= FP32_RTOL, f"{p['name']} call {call}: field vs pcg_run_phases {e_reg:.3e}"
        i_got, i_ora = caller.get_internalized(), oracle.get_internalized()
        scale = _internalized_scale(p, f_ora)
        ei = float((np.abs(i_got - i_ora) / scale).max())
        ei_reg = float((np.abs(i_got - regular.get_internalized()) / scale).max())
        assert ei <= FP32_RTOL, f"{p['name']} call {call}: internalized vs oracle {ei:.3e}"
        assert ei_reg <= FP32_RTOL, f"{p['name']} call {call}: internalized vs pcg_run_phases {ei_reg:.3e}"
    regular.close()
    oracle.close()


@pytest.mark.gpu
@pytest.mark.parametrize("S,padded", [(3, False), (4, True), (8, True)])
def test_noalloc_two_calls_match_oracle_and_regular_entry_point(pcg, oracle_mod, S, padded):
    torch = pytest.importorskip("torch")
    torch.cuda.set_device(0)
    L, noalloc = _fn(pcg)
    n = (24, 18, 12)
    p = _problem(40 + S, S, n, 2000)
    row = n[0] * S
    pitch = (row + 3) // 4 * 4 + 8 if padded else row
    _check_two_calls(pcg, oracle_mod, torch, noalloc, L, p, pitch)


@pytest.mark.gpu
def test_noalloc_small_problem_after_a_large_one(pcg, oracle_mod):
    """The scratch keeps the previous call's contents: a smaller mesh with fewer
    agents right after a larger one must not see stale ballots or sums."""
    torch = pytest.importorskip("torch")
    torch.cuda.set_device(0)
    L, noalloc = _fn(pcg)
    big = _problem(7, 8, (64, 48, 40), 60000, share=0.4)
    caller = Caller(torch, big, 64 * 8)
    assert caller.call(noalloc) == 0, L.pcg_last_error().decode()
    torch.cuda.synchronize()
    small = _problem(8, 4, (10, 9, 7), 300, share=0.5)
    _check_two_calls(pcg, oracle_mod, torch, noalloc, L, small, 10 * 4)


def _reject(pcg, dims=3, grid=(400, 400, 400), S=1, agents=10, pitch=None):
    L, noalloc = _fn(pcg)
    bbmin = np.zeros(3, dtype=np.int64)
    voxel = np.array([20, 20, 20], dtype=np.uint64)
    g = np.array(grid, dtype=np.uint64)
    dummy = ctypes.c_void_p(16)  # never dereferenced: validation comes before any device work
    pitch = grid[0] * S if pitch is None else pitch
    rc = noalloc(dummy, pitch, dims, bbmin.ctypes.data, voxel.ctypes.data, g.ctypes.data, S, 0.01, agents,
                 dummy, dummy, dummy, dummy, dummy, dummy, dummy, dummy, 0, None)
    return rc, L.pcg_last_error().decode()


def test_noalloc_rejects_oversized_problems(pcg):
    rc, msg = _reject(pcg)  # 64 M voxels: beyond the fixed scratch
    assert rc == 5 and "scratch" in msg
    rc, msg = _reject(pcg, grid=(100, 100, 100), S=8, agents=200_000)  # agents' terms beyond the scratch
    assert rc == 5 and "scratch" in msg


def test_noalloc_rejects_sizes_that_overflow(pcg):
    rc, msg = _reject(pcg, grid=(1 << 22, 1 << 22, 1 << 22))  # 2^66 voxels: the product overflows
    assert rc == 5 and "overflow" in msg
    rc, msg = _reject(pcg, grid=(1 << 16, 1 << 16, 1))  # exactly 2^32 voxels
    assert rc == 5 and "2^32" in msg
    rc, msg = _reject(pcg, grid=(64, 64, 64), agents=1 << 32)
    assert rc == 5 and "agents" in msg
    rc, msg = _reject(pcg, grid=(64, 1024, 1024), pitch=4096)  # pitch * ny * nz = 2^32 field elements
    assert rc == 5 and "pitch" in msg
    rc, msg = _reject(pcg, grid=(64, 64, 64), S=1 << 62, agents=8)  # nx * S overflows
    assert rc == 5 and "overflow" in msg


def test_noalloc_rejects_malformed_meshes(pcg):
    rc, msg = _reject(pcg, dims=2, grid=(16, 16, 5))  # z beyond dims must have one layer
    assert rc == 1 and "beyond dims" in msg
    rc, msg = _reject(pcg, grid=(16, 16, 16), S=2, pitch=31)  # a row needs 32 elements
    assert rc == 1 and "pitch" in msg
    rc, msg = _reject(pcg, grid=(16, 0, 16))
    assert rc == 1
