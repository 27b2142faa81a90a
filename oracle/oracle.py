"""ctypes wrapper around the CPU oracle (biofvm_oracle.c).

TEST INFRASTRUCTURE ONLY: the oracle is the checker for the GB300 kernels and the
timed CPU baseline.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline leg import this module; the product package never does.

The oracle restates the reference OpenMP solver
(reactions-diffusion/biofvm/kernels/openmp_solver/src/*.cpp) in FP64; its field
layout is the reference's interleaved one, index = s + S*(x + nx*(y + ny*z)).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "liboracle.so")
SOURCES = [os.path.join(HERE, "biofvm_oracle.c")]

PHASE_DIFFUSION, PHASE_DIRICHLET, PHASE_BULK, PHASE_CELLS = 1, 2, 4, 8
PHASE_ALL = 15
BULK_NONE, BULK_UNIFORM, BULK_PER_VOXEL = 0, 1, 2


def build(force: bool = False) -> str:
    """Compile the oracle into oracle/_build/liboracle.so (gcc + OpenMP)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    newest_src = max(os.path.getmtime(p) for p in SOURCES + [os.path.join(HERE, "biofvm_oracle.h")])
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= newest_src:
        return LIB_PATH
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O3", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-fno-fast-math", "-o", tmp] + SOURCES + ["-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        u64, i32, dbl = ctypes.c_uint64, ctypes.c_int, ctypes.c_double
        L.orc_create.restype = P
        L.orc_destroy.argtypes = [P]
        L.orc_last_error.restype = ctypes.c_char_p
        for name, args in [
            ("orc_set_threads", [P, i32]),
            ("orc_set_mesh", [P, i32, P, P, P]),
            ("orc_get_grid", [P, P]),
            ("orc_set_substrates", [P, u64, dbl, P, P, P]),
            ("orc_set_dirichlet_interior", [P, u64, P, P, P]),
            ("orc_set_dirichlet_boundary", [P, i32, i32, P, P]),
            ("orc_set_bulk", [P, i32, P, P, P]),
            ("orc_set_agents", [P, u64, P, P, P, P, P, P, P, P, P, i32]),
            ("orc_update_agents", [P, P, P]),
            ("orc_initialize", [P]),
            ("orc_solve", [P, u64]),
            ("orc_run_phases", [P, ctypes.c_uint32, i32]),
            ("orc_recompute_positional_data", [P]),
            ("orc_release_internalized", [P, u64]),
            ("orc_get_field", [P, P]),
            ("orc_set_field", [P, P]),
            ("orc_get_internalized", [P, P]),
            ("orc_get_counts", [P, P]),
            ("orc_get_conflict", [P]),
            ("orc_mass", [P, P]),
            ("orc_precompute", [u64, u64, u64, u64, dbl, P, P, P, P, P]),
        ]:
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int
        _lib = L
    return _lib


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


class OracleError(RuntimeError):
    pass


def precompute(n, S, shape, dims, dt, D, decay):
    """diffusion_solver::precompute_values: returns (b', e, c) as [n,S], [n-1,S], [S]."""
    D, decay = _f64(D, S), _f64(decay, S)
    b = np.zeros(n * S)
    e = np.zeros(max(n - 1, 1) * S)
    c = np.zeros(S)
    lib().orc_precompute(n, S, shape, dims, dt, _ptr(D), _ptr(decay), _ptr(b), _ptr(e), _ptr(c))
    return b.reshape(n, S), e[: (n - 1) * S].reshape(max(n - 1, 0), S), c


class OracleSolver:
    """One BioFVM problem solved on the CPU, with the same call surface as the
    GB300 C-ABI wrapper (physicore_gb300.Solver)."""

    def __init__(self, threads: int = 0):
        self._L = lib()
        self._h = self._L.orc_create()
        if threads:
            self._L.orc_set_threads(self._h, threads)
        self.dims = None
        self.grid = None
        self.S = None
        self.A = 0

    def close(self):
        if self._h:
            self._L.orc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != 0:
            raise OracleError(self._L.orc_last_error().decode())

    def set_mesh(self, dims, bbmin, bbmax, voxel):
        bmn = np.asarray(bbmin, dtype=np.int64)
        bmx = np.asarray(bbmax, dtype=np.int64)
        vx = np.asarray(voxel, dtype=np.uint64)
        self._check(self._L.orc_set_mesh(self._h, dims, _ptr(bmn), _ptr(bmx), _ptr(vx)))
        g = np.zeros(3, dtype=np.uint64)
        self._L.orc_get_grid(self._h, _ptr(g))
        self.dims = dims
        self.grid = tuple(int(v) for v in g)

    def set_substrates(self, dt, D, decay, initial):
        D = _f64(D)
        S = D.size
        self.S = S
        decay, initial = _f64(decay, S), _f64(initial, S)  # keep alive across the call
        self._check(self._L.orc_set_substrates(self._h, S, float(dt), _ptr(D), _ptr(decay), _ptr(initial)))

    def set_dirichlet_interior(self, voxels, values, conditions):
        voxels = np.ascontiguousarray(np.asarray(voxels, dtype=np.uint64).reshape(-1))
        K = voxels.size // self.dims if voxels.size else 0
        vals = _f64(values, K * self.S) if K else np.zeros(1)
        conds = _u8(conditions, K * self.S) if K else np.zeros(1, np.uint8)
        self._check(self._L.orc_set_dirichlet_interior(self._h, K, _ptr(voxels) if K else None,
                                                       _ptr(vals), _ptr(conds)))

    def set_dirichlet_boundary(self, axis, side, values, conditions):
        vals = _f64(values, self.S)
        conds = _u8(conditions, self.S) if values is not None else None
        self._check(self._L.orc_set_dirichlet_boundary(self._h, axis, side, _ptr(vals), _ptr(conds)))

    def set_bulk(self, mode, supply=None, uptake=None, target=None):
        self._bulk = [_f64(supply), _f64(uptake), _f64(target)]
        self._check(self._L.orc_set_bulk(self._h, mode, *[_ptr(a) for a in self._bulk]))

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
        self._check(self._L.orc_set_agents(self._h, A, *[_ptr(a) if a is not None and a.size else None
                                                         for a in arrs], int(bool(compute_internalized))))

    def update_agents(self, positions=None, is_active=None):
        p = _f64(positions, self.A * self.dims) if positions is not None else None
        a = _u8(is_active, self.A) if is_active is not None else None
        self._check(self._L.orc_update_agents(self._h, _ptr(p), _ptr(a)))

    def initialize(self):
        self._check(self._L.orc_initialize(self._h))

    def solve(self, iterations=1):
        self._check(self._L.orc_solve(self._h, iterations))

    def run_phases(self, phases, recompute_cells):
        self._check(self._L.orc_run_phases(self._h, phases, int(bool(recompute_cells))))

    def recompute_positional_data(self):
        self._check(self._L.orc_recompute_positional_data(self._h))

    def release_internalized(self, agent):
        self._check(self._L.orc_release_internalized(self._h, agent))

    @property
    def voxels(self):
        return self.grid[0] * self.grid[1] * self.grid[2]

    def get_field(self):
        """Field in the reference layout, returned as an array [nz, ny, nx, S]."""
        out = np.empty(self.voxels * self.S)
        self._check(self._L.orc_get_field(self._h, _ptr(out)))
        return out.reshape(self.grid[2], self.grid[1], self.grid[0], self.S)

    def set_field(self, field):
        f = _f64(field, self.voxels * self.S)
        self._check(self._L.orc_set_field(self._h, _ptr(f)))

    def get_internalized(self):
        out = np.empty(max(self.A * self.S, 1))
        self._check(self._L.orc_get_internalized(self._h, _ptr(out)))
        return out[: self.A * self.S].reshape(self.A, self.S)

    def get_counts(self):
        out = np.empty(self.voxels, dtype=np.uint32)
        self._check(self._L.orc_get_counts(self._h, _ptr(out)))
        return out.reshape(self.grid[2], self.grid[1], self.grid[0])

    def get_conflict(self):
        return bool(self._L.orc_get_conflict(self._h))

    def mass(self):
        out = np.empty(self.S)
        self._check(self._L.orc_mass(self._h, _ptr(out)))
        return out


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
