"""ctypes wrapper of the FP64 oracle (liboracle.so).

TEST INFRASTRUCTURE: imported only by tests/, the smoke check and the CPU
baseline leg of bench.py, always as the checker.  The product never imports
it.  The scene crosses into the oracle through the same bcs_scene_desc struct
the product's C ABI takes.
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(REPO, "simulation-server_gb300"))

from bcs import SceneBuffers, Params  # noqa: E402  (ABI struct definitions only)

from build_oracle import LIB, build  # noqa: E402

_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(LIB)
        P = C.c_void_p
        D = C.POINTER(C.c_double)
        lib.bcso_create.argtypes = [P, C.POINTER(P)]
        lib.bcso_create.restype = C.c_int
        lib.bcso_destroy.argtypes = [P]
        lib.bcso_set_threads.argtypes = [P, C.c_int]
        lib.bcso_set_reference_order.argtypes = [P, C.c_int]
        lib.bcso_layout.restype = None
        lib.bcso_counts.argtypes = [P, P]
        lib.bcso_bounds.argtypes = [P, P, P]
        lib.bcso_set_particles.argtypes = [P, P, P, P]
        lib.bcso_set_particles.restype = C.c_int
        lib.bcso_get_particles.argtypes = [P, P, P, P]
        lib.bcso_set_vein.argtypes = [P, P, P]
        lib.bcso_get_vein.argtypes = [P, P, P, P]
        lib.bcso_step.argtypes = [P, C.c_int]
        lib.bcso_macro_step.argtypes = [P, C.c_int, C.c_int]
        lib.bcso_calculate_grids.argtypes = [P]
        lib.bcso_calculate_next_frame.argtypes = [P]
        lib.bcso_propagate_all.argtypes = [P]
        lib.bcso_get_grid.argtypes = [P, C.c_int, P, P, P, P]
        lib.bcso_grid_of_points.argtypes = [P, C.c_int, P, P, P, P, P, P]
        lib.bcso_layout.argtypes = [P, P, P, P]
        lib.bcso_vein_neighbors.argtypes = [P, P, P]
        lib.bcso_error_word.argtypes = [P, C.c_int]
        lib.bcso_error_word.restype = C.c_uint
        lib.bcso_steps_done.argtypes = [P]
        lib.bcso_steps_done.restype = C.c_longlong
        lib.bcso_philox4x32_10.argtypes = [P, P, P]
        lib.bcso_spring_scalar.argtypes = [D, D, C.c_double, C.c_double, C.c_double]
        lib.bcso_spring_scalar.restype = C.c_double
        lib.bcso_ray_triangle.argtypes = [D, D, D, D, D, D]
        lib.bcso_ray_triangle.restype = C.c_int
        lib.bcso_barycentric.argtypes = [D, D, D, D, D]
        lib.bcso_resilient.argtypes = [C.POINTER(Params), D, D, C.c_double, C.c_double, D]
        lib.bcso_environment.argtypes = [C.POINTER(Params), D, C.c_double, D]
        _lib = lib
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class OracleSim:
    """FP64 restatement of one scene; mirrors bcs.Simulation's calls."""

    def __init__(self, scene, threads: int | None = None):
        self.lib = load()
        self._bufs = SceneBuffers(scene)
        h = C.c_void_p()
        st = self.lib.bcso_create(C.addressof(self._bufs.desc), C.byref(h))
        if st != 0:
            raise ValueError(f"oracle rejected the scene (status {st})")
        self.h = h
        cnt = np.zeros(6, np.int32)
        self.lib.bcso_counts(self.h, cnt.ctypes.data)
        self.n, self.cells, self.nv, self.nt, self.grid_cells, self.tri_grid_cells = (int(x) for x in cnt)
        if threads:
            self.lib.bcso_set_threads(self.h, int(threads))
        self.set_particles(scene.positions, scene.velocities)

    def close(self):
        if getattr(self, "h", None):
            self.lib.bcso_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_threads(self, n: int):
        self.lib.bcso_set_threads(self.h, int(n))

    def set_reference_order(self, on: bool = True):
        """Read order of the reference's kernels run serially (pin mode)."""
        self.lib.bcso_set_reference_order(self.h, int(on))

    def layout(self, model_vertices: int, types: int):
        starts = np.empty((types, 3), np.int32)
        radius = np.empty(model_vertices, np.float32)
        r0 = np.empty(model_vertices, np.float64)
        self.lib.bcso_layout(self.h, starts.ctypes.data, radius.ctypes.data, r0.ctypes.data)
        return starts, radius, r0

    def set_particles(self, pos, vel, force=None):
        p = np.ascontiguousarray(pos, np.float32)
        v = np.ascontiguousarray(vel, np.float32)
        f = None if force is None else np.ascontiguousarray(force, np.float32)
        st = self.lib.bcso_set_particles(self.h, p.ctypes.data, v.ctypes.data, None if f is None else f.ctypes.data)
        if st != 0:
            raise ValueError("non-finite particle state")

    def get_particles(self):
        out = [np.empty((self.n, 3), np.float64) for _ in range(3)]
        self.lib.bcso_get_particles(self.h, *(a.ctypes.data for a in out))
        return tuple(out)

    def set_vein(self, pos=None, vel=None):
        p = None if pos is None else np.ascontiguousarray(pos, np.float32)
        v = None if vel is None else np.ascontiguousarray(vel, np.float32)
        self.lib.bcso_set_vein(self.h, None if p is None else p.ctypes.data, None if v is None else v.ctypes.data)

    def get_vein(self):
        out = [np.empty((self.nv, 3), np.float64) for _ in range(3)]
        self.lib.bcso_get_vein(self.h, *(a.ctypes.data for a in out))
        return tuple(out)

    def step(self, n: int = 1):
        self.lib.bcso_step(self.h, int(n))

    def macro_step(self, substeps: int, n: int = 1):
        """Multi-rate macro steps: collisions and the vein ray once per
        `substeps` sub-steps, cell springs every sub-step."""
        self.lib.bcso_macro_step(self.h, int(substeps), int(n))

    def calculate_grids(self):
        self.lib.bcso_calculate_grids(self.h)

    def calculate_next_frame(self):
        self.lib.bcso_calculate_next_frame(self.h)

    def propagate_all(self):
        self.lib.bcso_propagate_all(self.h)

    def get_grid(self, which=0, dense=True):
        cnt = self.n if which == 0 else self.nt
        cells = self.grid_cells if which == 0 else self.tri_grid_cells
        keys = np.empty(cnt, np.int32)
        ids = np.empty(cnt, np.int32)
        st = np.empty(cells, np.int32) if dense else None
        en = np.empty(cells, np.int32) if dense else None
        self.lib.bcso_get_grid(self.h, which, keys.ctypes.data, ids.ctypes.data,
                               None if st is None else st.ctypes.data, None if en is None else en.ctypes.data)
        return keys, ids, st, en

    def grid_of_points(self, pts, dense=False):
        pts = np.ascontiguousarray(pts, np.float32)
        n = len(pts)
        keys = np.empty(n, np.int32)
        ids = np.empty(n, np.int32)
        st = np.empty(self.grid_cells, np.int32) if dense else None
        en = np.empty(self.grid_cells, np.int32) if dense else None
        err = C.c_uint()
        self.lib.bcso_grid_of_points(self.h, n, pts.ctypes.data, keys.ctypes.data, ids.ctypes.data,
                                     None if st is None else st.ctypes.data, None if en is None else en.ctypes.data,
                                     C.byref(err))
        return keys, ids, st, en, int(err.value)

    def bounds(self):
        b = np.empty(6, np.float32)
        d = np.empty(6, np.int32)
        self.lib.bcso_bounds(self.h, b.ctypes.data, d.ctypes.data)
        return b, d

    def vein_neighbors(self):
        ids = np.empty((9, self.nv), np.int32)
        ln = np.empty((9, self.nv), np.float32)
        self.lib.bcso_vein_neighbors(self.h, ids.ctypes.data, ln.ctypes.data)
        return ids, ln

    def error_word(self, clear=False) -> int:
        return int(self.lib.bcso_error_word(self.h, int(clear)))

    def steps_done(self) -> int:
        return int(self.lib.bcso_steps_done(self.h))


def philox(ctr, key):
    c = np.asarray(ctr, np.uint32)
    k = np.asarray(key, np.uint32)
    out = np.empty(4, np.uint32)
    load().bcso_philox4x32_10(c.ctypes.data, k.ctypes.data, out.ctypes.data)
    return out
