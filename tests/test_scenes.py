"""Scene generators: the shapes of the benchmark workloads (CPU only)."""
import numpy as np

import bcs_scenes as S


def test_cell_models():
    s = S.sphere_cell(3.0, 1)
    assert s.vertices.shape == (42, 3) and s.springs.shape == (120, 2)
    np.testing.assert_allclose(np.linalg.norm(s.vertices, axis=1), 3.0, rtol=1e-6)
    b = S.biconcave_cell(4.0, 2)
    assert b.vertices.shape == (162, 3) and b.springs.shape == (480, 2)
    assert abs(b.vertices[:, 0]).max() <= 4.0 + 1e-6 and abs(b.vertices[:, 1]).max() < 1.4


def test_straight_scene_shapes():
    sc = S.straight_scene()
    assert sc.particle_count == 256 * 42 == len(sc.positions)
    assert sc.vein_positions.shape == (6400, 3) and sc.vein_indices.shape == (12672, 3)
    # reference mesh order: (r+1)A+j, rA+j, rA+j+1 then (r+1)A+j, rA+j+1, (r+1)A+j+1
    assert list(sc.vein_indices[0]) == [64, 0, 1] and list(sc.vein_indices[1]) == [64, 1, 65]


def test_placement_has_no_overlap():
    sc = S.straight_scene(cells=64)
    cen = sc.positions.reshape(64, 42, 3).mean(1)
    d = np.linalg.norm(cen[:, None] - cen[None], axis=2) + np.eye(64) * 1e9
    assert d.min() >= 2 * 3.0 + 2 * 0.5
    r = np.linalg.norm(sc.positions[:, [0, 2]], axis=1)
    assert r.max() < 30.0 - 0.5


def test_triangle_normals_point_into_lumen():
    sc = S.straight_scene(cells=1)
    p = sc.vein_positions.astype(np.float64)
    t = sc.vein_indices.astype(np.int64)
    e1 = p[t[:, 1]] - p[t[:, 0]]
    e2 = p[t[:, 2]] - p[t[:, 0]]
    n = np.cross(e2, e1)
    c = p[t].mean(1)
    radial = c.copy()
    radial[:, 1] = 0
    assert np.all((n * radial).sum(1) < 0)


def test_bifurcation_small():
    sc = S.bifurcation_scene(cells_per_type=300, seed=3)
    assert sc.particle_count == 300 * 42 + 300 * 162
    assert len(sc.flow_segments) == 3
    assert len(sc.ending_radii) == 2


def test_batched_scenes_generator():
    scs = S.batched_scenes(4, seed=3, min_cells=20, max_cells=200, min_length=60.0, max_length=120.0)
    assert len(scs) == 4
    for sc in scs:
        n = sum(t.count for t in sc.types)
        assert 20 <= n <= 200
        L = -float(sc.vein_positions[:, 1].min())
        assert 60.0 <= L <= 120.0 + 1e-3
        assert len(sc.positions) == sum(t.count * len(t.vertices) for t in sc.types)
        # every cell inside the vessel radius
        r = np.hypot(sc.positions[:, 0], sc.positions[:, 2])
        assert r.max() < sc.params.cylinder_radius


def test_mixed_scene_grows_radius_to_fit():
    sc = S.mixed_straight_scene(400, 300, 60.0, seed=1, base_radius=10.0)
    assert sc.params.cylinder_radius > 10.0
    assert [t.count for t in sc.types] == [400, 300]


def test_scale_scene_small_and_subset():
    sc = S.scale_scene(600, seed=2, widen=2.0)
    assert [t.count for t in sc.types] == [300, 300]
    assert sc.params.cylinder_radius == 80.0
    assert len(sc.flow_segments) == 3
    sub = S.subset_scene(sc, 50, seed=4)
    assert sum(t.count for t in sub.types) == 50
    assert len(sub.positions) == sub.particle_count
    # every chosen cell is a whole cell of the full scene, in order
    full = {}
    start = 0
    for t in sc.types:
        pic = len(t.vertices)
        for c in range(t.count):
            full[sc.positions[start + c * pic].tobytes()] = sc.positions[start + c * pic:start + (c + 1) * pic]
        start += t.count * pic
    start = 0
    for t in sub.types:
        pic = len(t.vertices)
        for c in range(t.count):
            rows = sub.positions[start + c * pic:start + (c + 1) * pic]
            np.testing.assert_array_equal(full[rows[0].tobytes()], rows)
        start += t.count * pic


def test_scale_scene_key_space_at_one_million_cells():
    """The 1M-cell vessel's grid box at cell 1.0 stays inside 31-bit keys
    (computed from the vessel's segments, without building the scene)."""
    import math
    w = 6.0
    R, Rb = 40.0 * w, 28.0 * w
    # the length the generator settles on for 1M cells (checked on the host: 1269)
    L = 1269.3
    a = math.radians(15.0)
    ext_x = 2 * (L * math.sin(a) + Rb * math.cos(a)) + 80
    ext_y = L + L * math.cos(a) + Rb * math.sin(a) + 80
    ext_z = 2 * R + 80
    assert ext_x * ext_y * ext_z < 2 ** 31
