"""The allocation-free cell step (pcg_cells_noalloc) against the regular entry point.

pcg_cells_noalloc serves callers that cannot let a library allocate device memory
(frameworks that own all GPU memory through their own pool, loops that must avoid
cudaMalloc's synchronisation).  Here the caller's buffers are ordinary device
tensors; the entry point itself allocates nothing and takes its scratch from a
fixed device array.  Two cell passes in a row through the C ABI must match two
passes of pcg_run_phases(PCG_PHASE_CELLS, recompute=1) on the same inputs, within
the FP32 tolerances of the other GPU tests.  This file is collected last.
"""
import ctypes

import numpy as np
import pytest

from physicore_gb300 import workloads as W

pytestmark = pytest.mark.gpu

FP32_RTOL = 1e-5


def _problem():
    rng = np.random.default_rng(42)
    S, n = 3, (24, 18, 12)
    pos = W.uniform_positions(rng, 2000, 3, 0.0, np.array(n, dtype=np.float64) * 20.0)
    pos[:500] = pos[500:1000]  # shared voxels: ballot conflicts
    ag = W.agents_block(rng, 2000, S, pos, net_export_hi=0.5)
    return dict(name="noalloc", dims=3, bbmin=(0, 0, 0), bbmax=tuple(v * 20 for v in n), voxel=(20, 20, 20),
                dt=0.01, D=np.array([1e3, 50.0, 2e4]), decay=np.array([0.1, 0.5, 1e-3]), initial=np.zeros(S),
                field=rng.random((n[2], n[1], n[0], S)), field_layout="interleaved", boundary=[], interior=None,
                bulk=None, agents=ag, compute_internalized=True)


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


def test_noalloc_cells_match_regular_entry_point(pcg):
    torch = pytest.importorskip("torch")
    L, noalloc = _fn(pcg)
    p = _problem()
    ref = W.apply(pcg.Solver(pcg.FP32), p)
    a = p["agents"]
    nx, ny, nz = ref.grid
    S = ref.S
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)

    # the caller's own device buffers
    field = torch.from_numpy(ref.get_field(dtype=np.float32).reshape(-1).copy()).to(dev)
    t = {k: torch.from_numpy(np.ascontiguousarray(a[k], dtype=np.float64).reshape(-1)).to(dev)
         for k in ("positions", "secretion", "saturation", "uptake", "net_export", "volumes")}
    active = torch.from_numpy(a["is_active"].astype(np.uint8)).to(dev)
    internal = torch.zeros(len(a["volumes"]) * S, dtype=torch.float64, device=dev)
    bbmin = np.zeros(3, dtype=np.int64)
    voxel = np.array(p["voxel"], dtype=np.uint64)
    grid = np.array([nx, ny, nz], dtype=np.uint64)
    Vv = float(np.prod(p["voxel"]))
    den = (a["uptake"] + a["secretion"]) * p["dt"] * a["volumes"][:, None] / Vv

    for call in range(2):
        ref.run_phases(pcg.PHASE_CELLS, True)
        rc = noalloc(field.data_ptr(), nx * S, 3, bbmin.ctypes.data, voxel.ctypes.data, grid.ctypes.data, S,
                     p["dt"], len(a["volumes"]), t["positions"].data_ptr(), t["secretion"].data_ptr(),
                     t["saturation"].data_ptr(), t["uptake"].data_ptr(), t["net_export"].data_ptr(),
                     t["volumes"].data_ptr(), active.data_ptr(), internal.data_ptr(), 1,
                     torch.cuda.current_stream().cuda_stream)
        assert rc == 0, L.pcg_last_error().decode()
        torch.cuda.synchronize()
        f_ref = ref.get_field()
        f_got = field.cpu().numpy().astype(np.float64).reshape(nz, ny, nx, S)
        e = _rel(f_got, f_ref)
        assert e <= FP32_RTOL, f"call {call}: field relative error {e:.3e}"
        i_ref = ref.get_internalized()
        i_got = internal.cpu().numpy().reshape(-1, S)
        # internalized amounts: FP32 densities enter scaled by Vv (and by den after a conflict)
        scale = Vv * np.abs(f_ref).reshape(-1, S).max(axis=0) * (1.0 + den.max())
        ei = float((np.abs(i_got - i_ref) / scale).max())
        assert ei <= FP32_RTOL, f"call {call}: internalized error {ei:.3e}"


def test_noalloc_rejects_oversized_problems(pcg):
    L, noalloc = _fn(pcg)
    bbmin = np.zeros(3, dtype=np.int64)
    voxel = np.array([20, 20, 20], dtype=np.uint64)
    grid = np.array([400, 400, 400], dtype=np.uint64)  # 64 M voxels: beyond the fixed scratch
    dummy = ctypes.c_void_p(16)  # never dereferenced: the size check comes first
    rc = noalloc(dummy, 400, 3, bbmin.ctypes.data, voxel.ctypes.data, grid.ctypes.data, 1, 0.01, 10,
                 dummy, dummy, dummy, dummy, dummy, dummy, dummy, dummy, 0, None)
    assert rc == 5 and "scratch" in L.pcg_last_error().decode()
