"""physicore_gb300 -- GB300-native BioFVM reaction-diffusion backend.

The compute path is libphysicore_gb300.so (hand-written sm_103a CUDA behind the
C ABI declared in include/physicore_gb300.h).  This module is a thin ctypes
binding over that ABI for Python callers, tests and benchmarks; it holds no
compute of its own and raises if the native library is missing -- there is no
CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libphysicore_gb300.so")

FP32, FP64 = 0, 1
LAYOUT_INTERLEAVED, LAYOUT_PLANAR = 0, 1
DTYPE_F64, DTYPE_F32 = 0, 1
PHASE_DIFFUSION, PHASE_DIRICHLET, PHASE_BULK, PHASE_CELLS = 1, 2, 4, 8
PHASE_ALL = 15
BULK_NONE, BULK_UNIFORM, BULK_PER_VOXEL = 0, 1, 2
MAP_ROW, MAP_SUBSTRATE = 0, 1

ERRORS = {1: "invalid", 2: "cuda", 3: "nomem", 4: "device", 5: "unsupported"}


class PcgError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{ERRORS.get(code, code)}] {msg}")
        self.code = code


class KernelStat(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 32), ("launches", ctypes.c_uint64), ("total_ms", ctypes.c_double),
                ("algorithmic_bytes", ctypes.c_double)]


# (name, argtypes); every function returns int status unless noted
_P, _u64, _i32, _dbl, _u32 = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int, ctypes.c_double, ctypes.c_uint32
SIGNATURES = {
    "pcg_create": [_P, _i32, _i32],
    "pcg_destroy": [_P],
    "pcg_set_stream": [_P, _P],
    "pcg_get_stream": [_P, _P],
    "pcg_set_mesh": [_P, _i32, _P, _P, _P],
    "pcg_get_grid": [_P, _P],
    "pcg_set_substrates": [_P, _u64, _dbl, _P, _P, _P],
    "pcg_set_dirichlet_interior": [_P, _u64, _P, _P, _P],
    "pcg_set_dirichlet_boundary": [_P, _i32, _i32, _P, _P],
    "pcg_set_bulk": [_P, _i32, _P, _P, _P],
    "pcg_set_agents": [_P, _u64, _P, _P, _P, _P, _P, _P, _P, _P, _P, _i32],
    "pcg_update_agents": [_P, _P, _P],
    "pcg_set_internalized": [_P, _P],
    "pcg_initialize": [_P],
    "pcg_estimate_device_bytes": [_P, _P],
    "pcg_solve": [_P, _u64],
    "pcg_run_phases": [_P, _u32, _i32],
    "pcg_recompute_positional_data": [_P],
    "pcg_release_internalized": [_P, _u64],
    "pcg_get_field": [_P, _P, _i32, _i32],
    "pcg_get_field_async": [_P, _P, _i32, _i32, _P],
    "pcg_wait_field": [_P, _u64],
    "pcg_set_field": [_P, _P, _i32, _i32],
    "pcg_get_density": [_P, _u64, _u64, _u64, _u64, _P],
    "pcg_get_internalized": [_P, _P],
    "pcg_get_counts": [_P, _P],
    "pcg_get_conflict": [_P, _P],
    "pcg_mass": [_P, _P],
    "pcg_set_mass_check": [_P, ctypes.c_int],
    "pcg_set_sweep_fusion": [_P, ctypes.c_int, _u64, _u32],
    "pcg_get_mass_check": [_P, _P, _P, _P, _P],
    "pcg_synchronize": [_P],
    "pcg_get_field_device": [_P, _P, _P, _P],
    "pcg_get_agents_device": [_P, _P, _P],
    "pcg_set_kernel_timing": [_P, _i32],
    "pcg_get_kernel_stats": [_P, _P, _u64, _P],
    "pcg_reset_kernel_stats": [_P],
    "pcg_get_launch_count": [_P, _P],
    "pcg_batch_create": [_P, _P, _u64],
    "pcg_batch_destroy": [_P],
    "pcg_batch_solve": [_P, _u64],
    "pcg_batch_solve_budgets": [_P, _u64, _P],
    "pcg_batch_synchronize": [_P],
    "pcg_batch_get_stream": [_P, _P],
    "pcg_batch_set_graph": [_P, _i32],
    "pcg_batch_prepare": [_P],
    "pcg_batch_autotune": [_P],
    "pcg_batch_force_config": [_P, _i32, _i32, _u32],
    "pcg_batch_describe": [_P, _P, _u64, _P],
    "pcg_batch_set_kernel_timing": [_P, _i32],
    "pcg_batch_get_kernel_stats": [_P, _P, _u64, _P],
    "pcg_batch_reset_kernel_stats": [_P],
    "pcg_batch_get_launch_count": [_P, _P],
    "pcg_server_create": [_P, _i32, _i32, _P],
    "pcg_server_destroy": [_P],
    "pcg_server_submit": [_P, _P, _u64, _u64],
    "pcg_server_submit_readback": [_P, _P, _u64, _u64, _P, _i32, _i32],
    "pcg_server_cancel": [_P, _u64],
    "pcg_server_poll": [_P, _P, _u64, _P, _i32],
    "pcg_server_get_stats": [_P, _P],
}

_lib = None


def load_library(path: str | None = None):
    """Loads the native library (build it first with __graft_entry__.build())."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: the GB300 extension must be built (python -c "
                          "'import __graft_entry__ as g; g.build()'); there is no CPU fallback")
    L = ctypes.CDLL(path)
    L.pcg_last_error.restype = ctypes.c_char_p
    L.pcg_last_error.argtypes = []
    for name, args in SIGNATURES.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = ctypes.c_int
    _lib = L
    return L


def _ptr(a):
    return None if a is None else a.ctypes.data


def _f64(a, n=None):
    if a is None:
        return None
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float64))
    if n is not None and a.size != n:
        raise ValueError(f"expected {n} values, got {a.size}")
    return a


def _u8(a, n=None):
    if a is None:
        return None
    a = np.ascontiguousarray(np.asarray(a).astype(np.uint8))
    if n is not None and a.size != n:
        raise ValueError(f"expected {n} values, got {a.size}")
    return a


class Solver:
    """One BioFVM problem resident on one GB300 (a pcg_context)."""

    def __init__(self, precision: int = FP32, device: int = 0):
        self._L = load_library()
        h = ctypes.c_void_p()
        self._check(self._L.pcg_create(ctypes.byref(h), precision, device))
        self._h = h
        self.precision = precision
        self.dims = None
        self.grid = None
        self.S = None
        self.A = 0

    # -- plumbing -----------------------------------------------------------
    def _check(self, rc):
        if rc != 0:
            raise PcgError(rc, self._L.pcg_last_error().decode())

    def close(self):
        if getattr(self, "_h", None):
            self._L.pcg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    @property
    def voxels(self):
        return self.grid[0] * self.grid[1] * self.grid[2]

    # -- problem description -----------------------------------------------
    def set_mesh(self, dims, bbmin, bbmax, voxel):
        bmn = np.asarray(bbmin, dtype=np.int64)
        bmx = np.asarray(bbmax, dtype=np.int64)
        vx = np.asarray(voxel, dtype=np.uint64)
        self._check(self._L.pcg_set_mesh(self._h, dims, _ptr(bmn), _ptr(bmx), _ptr(vx)))
        g = np.zeros(3, dtype=np.uint64)
        self._check(self._L.pcg_get_grid(self._h, _ptr(g)))
        self.dims = dims
        self.grid = tuple(int(v) for v in g)

    def set_substrates(self, dt, D, decay, initial):
        D = _f64(D)
        self.S = D.size
        decay, initial = _f64(decay, self.S), _f64(initial, self.S)  # keep alive across the call
        self._check(self._L.pcg_set_substrates(self._h, self.S, float(dt), _ptr(D), _ptr(decay), _ptr(initial)))

    def set_dirichlet_interior(self, voxels, values, conditions):
        voxels = np.ascontiguousarray(np.asarray(voxels, dtype=np.uint64).reshape(-1))
        K = voxels.size // self.dims if voxels.size else 0
        vals = _f64(values, K * self.S) if K else None
        conds = _u8(conditions, K * self.S) if K else None
        self._check(self._L.pcg_set_dirichlet_interior(self._h, K, _ptr(voxels) if K else None, _ptr(vals),
                                                       _ptr(conds)))

    def set_dirichlet_boundary(self, axis, side, values, conditions):
        vals = _f64(values, self.S)
        conds = _u8(conditions, self.S) if values is not None else None
        self._check(self._L.pcg_set_dirichlet_boundary(self._h, axis, side, _ptr(vals), _ptr(conds)))

    def set_bulk(self, mode, supply=None, uptake=None, target=None):
        arrs = [_f64(supply), _f64(uptake), _f64(target)]
        self._check(self._L.pcg_set_bulk(self._h, mode, *[_ptr(a) for a in arrs]))

    def set_agents(self, positions, secretion, saturation, uptake, net_export, volumes, is_active,
                   internalized=None, fraction_released=None, compute_internalized=False):
        vol = _f64(volumes)
        A = vol.size
        S = self.S
        self.A = A
        arrs = [_f64(positions, A * self.dims), _f64(secretion, A * S), _f64(saturation, A * S),
                _f64(uptake, A * S), _f64(net_export, A * S), vol, _u8(is_active, A),
                _f64(internalized, A * S) if internalized is not None else None,
                _f64(fraction_released, A * S) if fraction_released is not None else None]
        self._check(self._L.pcg_set_agents(self._h, A, *[_ptr(a) if a is not None and a.size else None
                                                         for a in arrs], int(bool(compute_internalized))))

    def update_agents(self, positions=None, is_active=None):
        p = _f64(positions, self.A * self.dims) if positions is not None else None
        a = _u8(is_active, self.A) if is_active is not None else None
        self._check(self._L.pcg_update_agents(self._h, _ptr(p), _ptr(a)))

    # -- solver surface ----------------------------------------------------
    def initialize(self):
        self._check(self._L.pcg_initialize(self._h))

    def estimate_device_bytes(self):
        v = ctypes.c_uint64()
        self._check(self._L.pcg_estimate_device_bytes(self._h, ctypes.byref(v)))
        return v.value

    def solve(self, iterations=1):
        self._check(self._L.pcg_solve(self._h, iterations))

    def run_phases(self, phases, recompute_cells):
        self._check(self._L.pcg_run_phases(self._h, phases, int(bool(recompute_cells))))

    def recompute_positional_data(self):
        self._check(self._L.pcg_recompute_positional_data(self._h))

    def release_internalized(self, agent):
        self._check(self._L.pcg_release_internalized(self._h, agent))

    def synchronize(self):
        self._check(self._L.pcg_synchronize(self._h))

    # -- host access -------------------------------------------------------
    def get_field(self, layout=LAYOUT_INTERLEAVED, dtype=np.float64, out=None):
        """Field as [nz, ny, nx, S] (interleaved) or [S, nz, ny, nx] (planar)."""
        dt = np.dtype(dtype)
        code = DTYPE_F64 if dt == np.float64 else DTYPE_F32
        nx, ny, nz = self.grid
        shape = (nz, ny, nx, self.S) if layout == LAYOUT_INTERLEAVED else (self.S, nz, ny, nx)
        if out is None:
            out = np.empty(shape, dtype=dt)
        self._check(self._L.pcg_get_field(self._h, _ptr(out), layout, code))
        return out

    def get_field_async(self, out, layout=LAYOUT_INTERLEAVED):
        """Starts reading the field into `out` (a C-contiguous float32/float64 array
        of the layout's shape, ideally pinned memory) and returns a ticket for
        wait_field; `out` must stay alive and unread until then."""
        dt = np.dtype(out.dtype)
        code = DTYPE_F64 if dt == np.float64 else DTYPE_F32 if dt == np.float32 else None
        nx, ny, nz = self.grid
        shape = (nz, ny, nx, self.S) if layout == LAYOUT_INTERLEAVED else (self.S, nz, ny, nx)
        if code is None or tuple(out.shape) != shape or not out.flags["C_CONTIGUOUS"]:
            raise ValueError(f"out must be a C-contiguous float32/float64 array of shape {shape}")
        t = ctypes.c_uint64()
        self._check(self._L.pcg_get_field_async(self._h, _ptr(out), layout, code, ctypes.byref(t)))
        return t.value

    def wait_field(self, ticket):
        self._check(self._L.pcg_wait_field(self._h, ticket))

    def set_field(self, field, layout=LAYOUT_INTERLEAVED):
        f = np.ascontiguousarray(field)
        code = DTYPE_F32 if f.dtype == np.float32 else DTYPE_F64
        if code == DTYPE_F64:
            f = _f64(f)
        if f.size != self.voxels * self.S:
            raise ValueError("field size mismatch")
        self._check(self._L.pcg_set_field(self._h, _ptr(f), layout, code))

    def get_density(self, s, x, y, z):
        v = ctypes.c_double()
        self._check(self._L.pcg_get_density(self._h, s, x, y, z, ctypes.byref(v)))
        return v.value

    def get_internalized(self):
        out = np.empty(max(self.A * self.S, 1))
        self._check(self._L.pcg_get_internalized(self._h, _ptr(out)))
        return out[: self.A * self.S].reshape(self.A, self.S)

    def get_counts(self):
        out = np.empty(self.voxels, dtype=np.uint32)
        self._check(self._L.pcg_get_counts(self._h, _ptr(out)))
        return out.reshape(self.grid[2], self.grid[1], self.grid[0])

    def get_conflict(self):
        v = ctypes.c_int()
        self._check(self._L.pcg_get_conflict(self._h, ctypes.byref(v)))
        return bool(v.value)

    def mass(self):
        out = np.empty(self.S)
        self._check(self._L.pcg_mass(self._h, _ptr(out)))
        return out

    def set_mass_check(self, enable=True):
        """Per-step FP64 check of the sweeps' mass identity (pcg_set_mass_check)."""
        self._check(self._L.pcg_set_mass_check(self._h, int(bool(enable))))

    def set_sweep_fusion(self, enable=True, slab_bytes=0, lag=0):
        """x and y sweeps of 3-D meshes in one launch over z-slabs (pcg_set_sweep_fusion)."""
        self._check(self._L.pcg_set_sweep_fusion(self._h, int(bool(enable)), int(slab_bytes), int(lag)))

    def get_mass_check(self):
        """dict(before, after, worst, steps): the last checked step's totals before
        and after its sweeps, the worst relative residual, the steps checked."""
        before, after, worst = np.empty(self.S), np.empty(self.S), np.empty(self.S)
        steps = ctypes.c_uint64(0)
        self._check(self._L.pcg_get_mass_check(self._h, _ptr(before), _ptr(after), _ptr(worst),
                                               ctypes.byref(steps)))
        return dict(before=before, after=after, worst=worst, steps=int(steps.value))

    # -- device access and measurement -------------------------------------
    def field_device(self):
        p, eb, pitch = ctypes.c_void_p(), ctypes.c_uint64(), ctypes.c_uint64()
        self._check(self._L.pcg_get_field_device(self._h, ctypes.byref(p), ctypes.byref(eb), ctypes.byref(pitch)))
        return p.value, eb.value, pitch.value

    def agents_device(self):
        """(positions, is_active) device pointers of the agents (pcg_get_agents_device)."""
        pos, act = ctypes.c_void_p(), ctypes.c_void_p()
        self._check(self._L.pcg_get_agents_device(self._h, ctypes.byref(pos), ctypes.byref(act)))
        return pos.value, act.value

    def set_stream(self, stream_handle):
        """Queues this context's work on `stream_handle` (None: its own stream).  The
        stream must outlive its use by the context."""
        self._check(self._L.pcg_set_stream(self._h, ctypes.c_void_p(stream_handle)))

    def stream(self):
        s = ctypes.c_void_p()
        self._check(self._L.pcg_get_stream(self._h, ctypes.byref(s)))
        return s.value

    def set_kernel_timing(self, enable):
        self._check(self._L.pcg_set_kernel_timing(self._h, int(bool(enable))))

    def kernel_stats(self):
        arr = (KernelStat * 32)()
        cnt = ctypes.c_uint64()
        self._check(self._L.pcg_get_kernel_stats(self._h, arr, 32, ctypes.byref(cnt)))
        return {arr[i].name.decode(): {"launches": arr[i].launches, "ms": arr[i].total_ms,
                                       "bytes": arr[i].algorithmic_bytes} for i in range(min(cnt.value, 32))}

    def reset_kernel_stats(self):
        self._check(self._L.pcg_reset_kernel_stats(self._h))

    def launch_count(self):
        v = ctypes.c_uint64()
        self._check(self._L.pcg_get_launch_count(self._h, ctypes.byref(v)))
        return v.value


class Batch:
    """Many Solver contexts (one device, one precision) stepped together: every
    phase is one launch over all domains and the step replays from a CUDA graph.
    Results are read back through each Solver."""

    def __init__(self, solvers):
        self._L = load_library()
        self.solvers = list(solvers)  # the contexts must outlive the batch
        arr = (ctypes.c_void_p * len(self.solvers))(*[s.handle.value for s in self.solvers])
        h = ctypes.c_void_p()
        self._check(self._L.pcg_batch_create(ctypes.byref(h), arr, len(self.solvers)))
        self._h = h

    def _check(self, rc):
        if rc != 0:
            raise PcgError(rc, self._L.pcg_last_error().decode())

    def close(self):
        if getattr(self, "_h", None):
            self._L.pcg_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def solve(self, iterations=1, budgets=None):
        """`iterations` steps; with budgets, domain d takes part in the first budgets[d] only."""
        if budgets is None:
            self._check(self._L.pcg_batch_solve(self._h, iterations))
        else:
            b = np.ascontiguousarray(budgets, dtype=np.uint64)
            if b.size != len(self.solvers):
                raise ValueError("one budget per domain")
            self._check(self._L.pcg_batch_solve_budgets(self._h, iterations, b.ctypes.data))

    def synchronize(self):
        self._check(self._L.pcg_batch_synchronize(self._h))

    def stream(self):
        s = ctypes.c_void_p()
        self._check(self._L.pcg_batch_get_stream(self._h, ctypes.byref(s)))
        return s.value

    def set_graph(self, enable):
        self._check(self._L.pcg_batch_set_graph(self._h, int(bool(enable))))

    def prepare(self):
        """Descriptors built and step graphs captured now (pcg_batch_prepare)."""
        self._check(self._L.pcg_batch_prepare(self._h))

    def autotune(self):
        self._check(self._L.pcg_batch_autotune(self._h))

    def force_config(self, axis, mapping, rows=0):
        """mapping: MAP_ROW / MAP_SUBSTRATE (x only); -1 returns the axis to the tuner."""
        self._check(self._L.pcg_batch_force_config(self._h, axis, mapping, rows))

    def describe(self):
        import json
        need = ctypes.c_uint64()
        self._check(self._L.pcg_batch_describe(self._h, None, 0, ctypes.byref(need)))
        buf = ctypes.create_string_buffer(need.value)
        self._check(self._L.pcg_batch_describe(self._h, buf, need.value, ctypes.byref(need)))
        return json.loads(buf.value.decode())

    def set_kernel_timing(self, enable):
        self._check(self._L.pcg_batch_set_kernel_timing(self._h, int(bool(enable))))

    def kernel_stats(self):
        arr = (KernelStat * 32)()
        cnt = ctypes.c_uint64()
        self._check(self._L.pcg_batch_get_kernel_stats(self._h, arr, 32, ctypes.byref(cnt)))
        return {arr[i].name.decode(): {"launches": arr[i].launches, "ms": arr[i].total_ms,
                                       "bytes": arr[i].algorithmic_bytes} for i in range(min(cnt.value, 32))}

    def reset_kernel_stats(self):
        self._check(self._L.pcg_batch_reset_kernel_stats(self._h))

    def launch_count(self):
        v = ctypes.c_uint64()
        self._check(self._L.pcg_batch_get_launch_count(self._h, ctypes.byref(v)))
        return v.value


class ServerOptions(ctypes.Structure):
    _fields_ = [("max_active", ctypes.c_uint64), ("steps_per_tick", ctypes.c_uint64),
                ("reserve_bytes", ctypes.c_uint64), ("max_queue", ctypes.c_uint64),
                ("memory_limit_bytes", ctypes.c_uint64), ("autotune", ctypes.c_int)]


class ServerResult(ctypes.Structure):
    _fields_ = [("ctx", ctypes.c_void_p), ("tag", ctypes.c_uint64), ("steps", ctypes.c_uint64),
                ("status", ctypes.c_int), ("code", ctypes.c_int), ("t_submit", ctypes.c_double),
                ("t_admit", ctypes.c_double), ("t_done", ctypes.c_double), ("device_bytes", ctypes.c_uint64),
                ("error", ctypes.c_char * 160)]


class ServerStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in ("submitted", "admitted", "completed", "cancelled", "refused",
                                               "failed", "ticks", "rebuilds", "steps", "vss", "active_bytes",
                                               "queued", "active", "in_flight")] + [
        (n, ctypes.c_double) for n in ("uptime_s", "rebuild_s", "step_s", "admit_s")] + [
        ("prebuilds", ctypes.c_uint64), ("prebuild_s", ctypes.c_double)]


REQUEST_DONE, REQUEST_CANCELLED, REQUEST_REFUSED, REQUEST_FAILED = 0, 1, 2, 3
REQUEST_STATUS = {0: "done", 1: "cancelled", 2: "refused", 3: "failed"}


class Server:
    """Continuous batching of independent simulations on one device (pcg_server_*).

    submit() hands a configured, NOT initialised Solver to the server, which owns it
    until poll() returns it; the returned Solver holds the results and its device
    memory until it is closed."""

    def __init__(self, precision: int = FP32, device: int = 0, max_active: int = 0, steps_per_tick: int = 0,
                 reserve_bytes: int = 1 << 30, max_queue: int = 0, memory_limit_bytes: int = 0,
                 autotune: bool = False):
        self._L = load_library()
        opts = ServerOptions(max_active, steps_per_tick, reserve_bytes, max_queue, memory_limit_bytes,
                             int(bool(autotune)))
        h = ctypes.c_void_p()
        self._check(self._L.pcg_server_create(ctypes.byref(h), precision, device, ctypes.byref(opts)))
        self._h = h
        self._held = {}  # tag -> Solver owned by the server
        self._outs = {}  # tag -> host buffer the server writes the field into

    def _check(self, rc):
        if rc != 0:
            raise PcgError(rc, self._L.pcg_last_error().decode())

    def submit(self, solver: "Solver", steps: int, tag: int, out=None, layout: int = LAYOUT_INTERLEAVED):
        """Hands `solver` over for `steps` steps.  With `out` (a C-contiguous
        float32/float64 array of the layout's shape, ideally pinned) the server
        copies the final field into it before returning the request."""
        if tag in self._held:
            raise ValueError(f"tag {tag} is already in flight")
        if out is None:
            self._check(self._L.pcg_server_submit(self._h, solver.handle, steps, tag))
        else:
            nx, ny, nz = solver.grid
            shape = (nz, ny, nx, solver.S) if layout == LAYOUT_INTERLEAVED else (solver.S, nz, ny, nx)
            dt = np.dtype(out.dtype)
            if dt not in (np.float32, np.float64) or tuple(out.shape) != shape or not out.flags["C_CONTIGUOUS"]:
                raise ValueError(f"out must be a C-contiguous float32/float64 array of shape {shape}")
            code = DTYPE_F32 if dt == np.float32 else DTYPE_F64
            self._check(self._L.pcg_server_submit_readback(self._h, solver.handle, steps, tag, _ptr(out), layout,
                                                           code))
            self._outs[tag] = out  # kept alive until the request comes back
        self._held[tag] = solver

    def cancel(self, tag: int):
        self._check(self._L.pcg_server_cancel(self._h, tag))

    def poll(self, max_results: int = 256, wait_ms: int = 0):
        arr = (ServerResult * max_results)()
        n = ctypes.c_uint64()
        self._check(self._L.pcg_server_poll(self._h, arr, max_results, ctypes.byref(n), wait_ms))
        out = []
        for i in range(n.value):
            r = arr[i]
            self._outs.pop(r.tag, None)
            out.append({"solver": self._held.pop(r.tag), "tag": r.tag, "steps": r.steps,
                        "status": REQUEST_STATUS.get(r.status, r.status), "code": r.code,
                        "t_submit": r.t_submit, "t_admit": r.t_admit, "t_done": r.t_done,
                        "device_bytes": r.device_bytes, "error": r.error.decode()})
        return out

    def stats(self):
        st = ServerStats()
        self._check(self._L.pcg_server_get_stats(self._h, ctypes.byref(st)))
        return {name: getattr(st, name) for name, _ in ServerStats._fields_}

    def in_flight(self):
        return len(self._held)

    def close(self):
        if getattr(self, "_h", None):
            self._L.pcg_server_destroy(self._h)
            self._h = None
            for s in self._held.values():  # destroyed by the server
                s._h = None
            self._held.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
