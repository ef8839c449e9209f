"""bcs_grid_sort_static: grid keys and their stable sort with no device
allocation, for callers that cannot allocate (a host application that owns
all device memory, or a frame loop that must not stall on cudaMalloc).

Its output must equal the allocating path's (bcs_calculate_grids +
bcs_get_grid on a bcs_sim) exactly, on two calls in a row that share the
library's fixed scratch array.  Collected last, so that a failure here does
not hide any other test; it also passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

import bcs
import bcs_scenes as S

pytestmark = pytest.mark.gpu


def allocating_grid(scene, pos):
    sim = bcs.Simulation(scene)
    sim.set_particles(pos, np.zeros_like(pos))
    sim.calculate_grids()
    keys, ids, _, _ = sim.get_grid(0, dense=False)
    info = sim.info
    bounds = np.array([info.min_x, info.max_x, info.min_y, info.max_y, info.min_z, info.max_z], np.float32)
    cells = np.array([scene.params.cell_width, scene.params.cell_height, scene.params.cell_depth], np.float32)
    sim.close()
    return keys, ids, bounds, cells


def static_grid(lib, pos, bounds, cells):
    import torch
    n = len(pos)
    d = [torch.from_numpy(np.ascontiguousarray(pos[:, k])).cuda() for k in range(3)]
    out_k = torch.empty(n, dtype=torch.int32, device="cuda")
    out_i = torch.empty(n, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    fp = C.POINTER(C.c_float)
    st = lib.bcs_grid_sort_static(d[0].data_ptr(), d[1].data_ptr(), d[2].data_ptr(), n,
                                  bounds.ctypes.data_as(fp), cells.ctypes.data_as(fp),
                                  out_k.data_ptr(), out_i.data_ptr(), None)
    assert st == 0, bcs.STATUS.get(st, st)
    assert lib.bcs_synchronize is not None
    torch.cuda.synchronize()
    return out_k.cpu().numpy(), out_i.cpu().numpy()


def test_static_sort_matches_allocating_path_twice(lib):
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    bcs.set_device(0)
    small = S.straight_scene(cells=256, seed=21)
    k0, i0, b0, c0 = allocating_grid(small, small.positions)
    big = S.bifurcation_scene(cells_per_type=1000, seed=22)
    assert big.particle_count <= bcs.GRID_SORT_STATIC_MAX
    rng = np.random.default_rng(5)
    jitter = big.positions + rng.normal(0, 0.3, big.positions.shape).astype(np.float32)
    k1, i1, b1, c1 = allocating_grid(big, jitter)
    # two calls in a row through the shared scratch: small, then large
    sk0, si0 = static_grid(lib, small.positions, b0, c0)
    np.testing.assert_array_equal(sk0, k0)
    np.testing.assert_array_equal(si0, i0)
    sk1, si1 = static_grid(lib, jitter, b1, c1)
    np.testing.assert_array_equal(sk1, k1)
    np.testing.assert_array_equal(si1, i1)


def static_error_word(lib):
    w = C.c_uint32(0xFFFFFFFF)
    st = lib.bcs_grid_sort_static_error_word(None, C.byref(w))
    assert st == 0, bcs.STATUS.get(st, st)
    return w.value


def test_static_sort_reports_out_of_box_positions(lib):
    """A position outside the grid box is clamped to the edge cell, as on the
    allocating path, and the call's error word says so; the next in-box call
    clears it."""
    torch = pytest.importorskip("torch")
    assert torch.cuda.is_available()
    bcs.set_device(0)
    scene = S.straight_scene(cells=64, seed=23)
    pos = scene.positions.copy()
    k_in, i_in, b, c = allocating_grid(scene, pos)
    out = pos.copy()
    out[7] = (b[1] + 5.0, b[3] + 3.0, b[5] + 9.0)    # beyond every max face
    out[11] = (b[0] - 2.0, 0.5 * (b[2] + b[3]), b[4] - 1.0)
    k_out, i_out, _, _ = allocating_grid(scene, out)
    sk, si = static_grid(lib, out, b, c)
    np.testing.assert_array_equal(sk, k_out)
    np.testing.assert_array_equal(si, i_out)
    assert static_error_word(lib) == bcs.ERRW_OUT_OF_GRID
    sk, si = static_grid(lib, pos, b, c)
    np.testing.assert_array_equal(sk, k_in)
    np.testing.assert_array_equal(si, i_in)
    assert static_error_word(lib) == 0


def test_static_sort_rejects_oversize(lib):
    fp = C.POINTER(C.c_float)
    b = np.zeros(6, np.float32)
    c = np.ones(3, np.float32)
    st = lib.bcs_grid_sort_static(None, None, None, bcs.GRID_SORT_STATIC_MAX + 1, b.ctypes.data_as(fp),
                                  c.ctypes.data_as(fp), None, None, None)
    assert st == 1
