"""ctypes mirror of include/bcs.h and a thin host-side wrapper.

`Simulation` keeps the reference's vocabulary for the per-frame calls of
src/main.cu:175-208 — calculate_grids(), calculate_next_frame(),
propagate_all() — plus the fused step().  It loads libbcs.so from this
directory and raises if the library is missing or no CUDA device is usable:
there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libbcs.so")

BCS_OK = 0
STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA runtime error", 3: "out of device memory",
          4: "no CUDA device", 5: "unsupported", 6: "a bounded device wait expired"}
ERR_TIMEOUT = 6
GRID_UNIFORM, GRID_NONE = 0, 1
MEM_HOST, MEM_DEVICE = 0, 1
ERRW_OUT_OF_GRID, ERRW_NAN_NORMALIZE, ERRW_NONFINITE = 1, 2, 4

EXPORTED = [
    "bcs_default_params", "bcs_status_string", "bcs_abi_version", "bcs_set_device", "bcs_create", "bcs_destroy",
    "bcs_get_info", "bcs_set_particles", "bcs_get_particles", "bcs_set_vein", "bcs_get_vein",
    "bcs_calculate_grids", "bcs_calculate_next_frame", "bcs_propagate_all", "bcs_step",
    "bcs_get_grid", "bcs_export_render", "bcs_get_error_word", "bcs_synchronize", "bcs_time_steps",
    "bcs_profile_steps", "bcs_grid_sort_static", "bcs_grid_sort_static_error_word", "bcs_create_batch", "bcs_get_scene_info",
    "bcs_get_tuning", "bcs_set_tuning", "bcs_set_mover_sort", "bcs_autotune", "bcs_macro_step",
    "bcs_surrogate_create", "bcs_surrogate_destroy", "bcs_surrogate_collect", "bcs_surrogate_train",
    "bcs_surrogate_enable", "bcs_surrogate_get_stats", "bcs_surrogate_reset_stats", "bcs_surrogate_param_count",
    "bcs_surrogate_get_params", "bcs_surrogate_set_params", "bcs_surrogate_loss_grad", "bcs_surrogate_forward",
    "bcs_surrogate_get_scales", "bcs_surrogate_evaluate", "bcs_surrogate_set_scales", "bcs_time_macro_steps",
    "bcs_init_particles", "bcs_set_tensor_path", "bcs_tensor_wait_expiries", "bcs_get_particles_async",
    "bcs_wait_particles", "bcs_get_crowded", "bcs_set_tensor_wait_probe", "bcs_event_decode", "bcs_event_encode",
    "bcs_control_create", "bcs_control_destroy", "bcs_control_post", "bcs_control_post_event", "bcs_control_handle",
    "bcs_control_send", "bcs_control_take_outgoing", "bcs_run",
]
INIT_REFERENCE, INIT_LATTICE = 0, 1
STEP_SHAPES = ((256, 512, 3), (128, 256, 6), (384, 768, 2), (256, 512, 4), (256, 512, 2), (128, 256, 8))
GRID_SORT_STATIC_MAX = 262144
MAX_SUBSTEPS = 64
PHASES = ("grid", "vein_forces", "collisions", "particles", "vein_update")


class BcsError(RuntimeError):
    def __init__(self, status: int, what: str):
        super().__init__(f"{what}: {STATUS.get(status, status)} ({status})")
        self.status = status


class Vec3(C.Structure):
    _fields_ = [("x", C.c_void_p), ("y", C.c_void_p), ("z", C.c_void_p)]


class CellType(C.Structure):
    _fields_ = [("count", C.c_int), ("particles_in_cell", C.c_int), ("vertices", C.c_void_p),
                ("spring_count", C.c_int), ("springs", C.c_void_p), ("spring_lengths", C.c_void_p),
                ("collision_radius", C.c_void_p)]


class Vein(C.Structure):
    _fields_ = [("vertex_count", C.c_int), ("positions", C.c_void_p), ("triangle_count", C.c_int),
                ("indices", C.c_void_p), ("ending_count", C.c_int), ("ending_centers", C.c_void_p),
                ("ending_radii", C.c_void_p)]


class FlowSegment(C.Structure):
    _fields_ = [("origin", C.c_float * 3), ("direction", C.c_float * 3), ("length", C.c_float),
                ("radius", C.c_float), ("peak_force", C.c_float)]


class Params(C.Structure):
    _fields_ = [
        ("dt", C.c_float), ("use_blood_flow", C.c_int), ("enable_reaction_force", C.c_int),
        ("enable_big_cells_brake", C.c_int),
        ("cell_width", C.c_float), ("cell_height", C.c_float), ("cell_depth", C.c_float),
        ("cell_width_triangles", C.c_float), ("cell_height_triangles", C.c_float),
        ("cell_depth_triangles", C.c_float),
        ("bounding_spheres_coeff", C.c_float), ("grid_y_margin", C.c_float), ("grid_xz_margin", C.c_float),
        ("min_spawn_y", C.c_float), ("velocity_collision_damping", C.c_float), ("particle_k_sniff", C.c_float),
        ("vein_k_sniff", C.c_float), ("particle_d_fact", C.c_float), ("vein_d_fact", C.c_float),
        ("vein_collision_force_intensity", C.c_float), ("viscous_damping", C.c_float),
        ("collision_spring_coeff", C.c_float), ("collision_damping_coeff", C.c_float),
        ("collision_shear_coeff", C.c_float), ("max_cell_size_factor_before_brake", C.c_float),
        ("big_particle_braking_intensity", C.c_float), ("init_velocity", C.c_float * 3),
        ("vein_impact_distance", C.c_float), ("vein_impact_minimal_force_distance", C.c_float),
        ("gravity", C.c_float * 3), ("cylinder_radius", C.c_float), ("particle_grid", C.c_int),
        ("triangle_grid", C.c_int), ("vein_dynamic", C.c_int), ("refresh_triangle_centers", C.c_int),
        ("seed", C.c_uint64),
    ]


class SceneDesc(C.Structure):
    _fields_ = [("type_count", C.c_int), ("types", C.POINTER(CellType)), ("vein", Vein),
                ("flow_segment_count", C.c_int), ("flow_segments", C.POINTER(FlowSegment)),
                ("params", Params)]


class Info(C.Structure):
    _fields_ = [
        ("particle_count", C.c_int), ("blood_cell_count", C.c_int), ("type_count", C.c_int),
        ("vertex_count", C.c_int), ("triangle_count", C.c_int),
        ("min_x", C.c_float), ("max_x", C.c_float), ("min_y", C.c_float), ("max_y", C.c_float),
        ("min_z", C.c_float), ("max_z", C.c_float),
        ("cell_count_x", C.c_int), ("cell_count_y", C.c_int), ("cell_count_z", C.c_int),
        ("cell_count", C.c_int64),
        ("tri_cell_count_x", C.c_int), ("tri_cell_count_y", C.c_int), ("tri_cell_count_z", C.c_int),
        ("tri_cell_count", C.c_int64), ("steps_done", C.c_int64), ("device_bytes", C.c_size_t),
        ("kernels_per_step", C.c_int), ("scene_count", C.c_int),
    ]


class SceneInfo(C.Structure):
    _fields_ = [
        ("particle_start", C.c_int), ("particle_count", C.c_int),
        ("blood_cell_start", C.c_int), ("blood_cell_count", C.c_int),
        ("vertex_start", C.c_int), ("vertex_count", C.c_int),
        ("triangle_start", C.c_int), ("triangle_count", C.c_int),
        ("min_x", C.c_float), ("max_x", C.c_float), ("min_y", C.c_float), ("max_y", C.c_float),
        ("min_z", C.c_float), ("max_z", C.c_float),
        ("cell_count_x", C.c_int), ("cell_count_y", C.c_int), ("cell_count_z", C.c_int),
        ("cell_count", C.c_int64), ("cell_key_offset", C.c_int64),
        ("tri_cell_count_x", C.c_int), ("tri_cell_count_y", C.c_int), ("tri_cell_count_z", C.c_int),
        ("tri_cell_count", C.c_int64), ("tri_cell_key_offset", C.c_int64),
    ]


class InitDesc(C.Structure):
    _fields_ = [("kind", C.c_int), ("seed", C.c_uint64), ("velocity_sigma", C.c_float), ("gap", C.c_float)]


class Tuning(C.Structure):
    _fields_ = [("step_shape", C.c_int), ("persistent", C.c_int), ("spatial_order", C.c_int),
                ("full_sort", C.c_int), ("occupancy_filter", C.c_int), ("sorted_positions", C.c_int),
                ("grid_collisions", C.c_int)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class SurrogateDesc(C.Structure):
    _fields_ = [("cell_type", C.c_int), ("substeps", C.c_int), ("layers", C.c_int), ("max_samples", C.c_int),
                ("seed", C.c_uint64), ("tolerance", C.c_float), ("huber_delta", C.c_float)]


# control messages of the streaming server (bcs_event_type, bcs_event_state)
EVENT_NAMES = ("no_message", "camera_left", "camera_right", "camera_forward", "camera_back", "camera_ascend",
               "camera_descend", "camera_rotate_left", "camera_rotate_right", "camera_rotate_up",
               "camera_rotate_down", "toggle_polygon_mode", "toggle_springs_rendering", "toggle_spheres_rendering",
               "stream_successfully_ended", "stop_rendering", "new_connection", "peer_disconnected",
               "invalid_message")
EVENT = {n: i for i, n in enumerate(EVENT_NAMES)}
EVENT_START, EVENT_STOP, EVENT_NOT_RELEVANT = 0, 1, 2


class Event(C.Structure):
    _fields_ = [("type", C.c_int32), ("state", C.c_int32)]


class ControlState(C.Structure):
    _fields_ = [("held", C.c_uint32), ("polygon_mode_line", C.c_int32), ("springs_rendering", C.c_int32),
                ("spheres_rendering", C.c_int32), ("stop_requested", C.c_int32), ("connected", C.c_int32),
                ("handled", C.c_int64)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class SurrogateStats(C.Structure):
    _fields_ = [("cells", C.c_int64), ("samples", C.c_int64), ("valid_samples", C.c_int64),
                ("predicted_cells", C.c_int64), ("fallback_cells", C.c_int64), ("iterations", C.c_int64),
                ("parameters", C.c_int64), ("last_loss", C.c_float), ("tolerance", C.c_float),
                ("flops_per_cell", C.c_double), ("device_bytes", C.c_size_t)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


def load_library(path: str = LIB_PATH) -> C.CDLL:
    """Load libbcs.so (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with bcs_build.build() (no CPU fallback exists)")
    lib = C.CDLL(path)
    P = C.c_void_p
    sigs = {
        "bcs_default_params": ([C.POINTER(Params)], None),
        "bcs_status_string": ([C.c_int], C.c_char_p),
        "bcs_abi_version": ([], C.c_int),
        "bcs_set_device": ([C.c_int], C.c_int),
        "bcs_create": ([C.POINTER(SceneDesc), P, C.POINTER(P)], C.c_int),
        "bcs_create_batch": ([C.POINTER(SceneDesc), C.c_int, P, C.POINTER(P)], C.c_int),
        "bcs_get_scene_info": ([P, C.c_int, C.POINTER(SceneInfo)], C.c_int),
        "bcs_get_tuning": ([P, C.POINTER(Tuning)], C.c_int),
        "bcs_set_tuning": ([P, C.POINTER(Tuning)], C.c_int),
        "bcs_set_mover_sort": ([P, C.c_int], C.c_int),
        "bcs_autotune": ([P, C.c_int, C.POINTER(Tuning), C.POINTER(C.c_float)], C.c_int),
        "bcs_macro_step": ([P, C.c_int, C.c_int], C.c_int),
        "bcs_time_macro_steps": ([P, C.c_int, C.c_int, C.POINTER(C.c_float)], C.c_int),
        "bcs_init_particles": ([P, C.POINTER(InitDesc)], C.c_int),
        "bcs_set_tensor_path": ([C.c_int], C.c_int),
        "bcs_tensor_wait_expiries": ([], C.c_uint),
        "bcs_set_tensor_wait_probe": ([C.c_int], C.c_int),
        "bcs_surrogate_create": ([P, C.POINTER(SurrogateDesc), C.POINTER(P)], C.c_int),
        "bcs_surrogate_destroy": ([P], C.c_int),
        "bcs_surrogate_collect": ([P, C.c_int], C.c_int),
        "bcs_surrogate_train": ([P, C.c_int, C.c_int, C.c_float, C.POINTER(C.c_float)], C.c_int),
        "bcs_surrogate_enable": ([P, C.c_int], C.c_int),
        "bcs_surrogate_get_stats": ([P, C.POINTER(SurrogateStats)], C.c_int),
        "bcs_surrogate_reset_stats": ([P], C.c_int),
        "bcs_surrogate_param_count": ([P], C.c_int64),
        "bcs_surrogate_get_params": ([P, P, C.c_int64], C.c_int),
        "bcs_surrogate_set_params": ([P, P, C.c_int64], C.c_int),
        "bcs_surrogate_loss_grad": ([P, C.c_int, P, P, P, P, P], C.c_int),
        "bcs_surrogate_forward": ([P, C.c_int, P, P, P], C.c_int),
        "bcs_surrogate_get_scales": ([P, P], C.c_int),
        "bcs_surrogate_set_scales": ([P, P], C.c_int),
        "bcs_surrogate_evaluate": ([P, C.c_int, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)], C.c_int),
        "bcs_destroy": ([P], C.c_int),
        "bcs_get_info": ([P, C.POINTER(Info)], C.c_int),
        "bcs_set_particles": ([P, Vec3, Vec3, Vec3, C.c_int], C.c_int),
        "bcs_get_particles": ([P, Vec3, Vec3, Vec3, C.c_int], C.c_int),
        "bcs_get_particles_async": ([P, Vec3, Vec3, Vec3], C.c_int),
        "bcs_wait_particles": ([P], C.c_int),
        "bcs_get_crowded": ([P, C.POINTER(C.c_longlong)], C.c_int),
        "bcs_event_decode": ([C.POINTER(C.c_uint8), C.c_size_t], Event),
        "bcs_event_encode": ([Event, C.POINTER(C.c_uint8)], C.c_int),
        "bcs_control_create": ([C.POINTER(P)], C.c_int),
        "bcs_control_destroy": ([P], None),
        "bcs_control_post": ([P, C.POINTER(C.c_uint8), C.c_size_t], C.c_int),
        "bcs_control_post_event": ([P, Event], C.c_int),
        "bcs_control_handle": ([P, C.POINTER(ControlState)], C.c_int),
        "bcs_control_send": ([P, Event], C.c_int),
        "bcs_control_take_outgoing": ([P, C.POINTER(C.c_uint8)], C.c_int),
        "bcs_run": ([P, P, C.c_int, C.POINTER(C.c_int)], C.c_int),
        "bcs_set_vein": ([P, Vec3, Vec3, C.c_int], C.c_int),
        "bcs_get_vein": ([P, Vec3, Vec3, Vec3, C.c_int], C.c_int),
        "bcs_calculate_grids": ([P], C.c_int),
        "bcs_calculate_next_frame": ([P], C.c_int),
        "bcs_propagate_all": ([P], C.c_int),
        "bcs_step": ([P, C.c_int], C.c_int),
        "bcs_get_grid": ([P, C.c_int, P, P, P, P, C.c_int], C.c_int),
        "bcs_export_render": ([P, P, P, P, C.c_int], C.c_int),
        "bcs_get_error_word": ([P, C.POINTER(C.c_uint32), C.c_int], C.c_int),
        "bcs_synchronize": ([P], C.c_int),
        "bcs_time_steps": ([P, C.c_int, C.POINTER(C.c_float)], C.c_int),
        "bcs_profile_steps": ([P, C.c_int, C.POINTER(C.c_float)], C.c_int),
        "bcs_grid_sort_static": ([P, P, P, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_float), P, P, P], C.c_int),
        "bcs_grid_sort_static_error_word": ([P, C.POINTER(C.c_uint32)], C.c_int),
    }
    for name, (args, res) in sigs.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


# The reference's shipped constants (src/config/simulation.hpp:3-21,
# src/config/physics.hpp:4-34, src/meta_factory/vein_factory.hpp:88); the
# library's bcs_default_params returns the same values.
REFERENCE_DEFAULTS = dict(
    dt=0.008, use_blood_flow=1, enable_reaction_force=1, enable_big_cells_brake=1,
    cell_width=2.0, cell_height=2.0, cell_depth=2.0,
    cell_width_triangles=25.0, cell_height_triangles=25.0, cell_depth_triangles=25.0,
    bounding_spheres_coeff=3.0, grid_y_margin=40.0, grid_xz_margin=40.0, min_spawn_y=-20.0,
    velocity_collision_damping=0.96, particle_k_sniff=25.0, vein_k_sniff=0.1, particle_d_fact=10.0,
    vein_d_fact=0.7, vein_collision_force_intensity=0.005, viscous_damping=0.39, collision_spring_coeff=6.0,
    collision_damping_coeff=6.0, collision_shear_coeff=4.0, max_cell_size_factor_before_brake=1.5,
    big_particle_braking_intensity=0.8, init_velocity=(0.0, -80.0, 0.0), vein_impact_distance=6.0,
    vein_impact_minimal_force_distance=0.001, gravity=(0.0, -25.0, 0.0), cylinder_radius=50.0,
    particle_grid=GRID_UNIFORM, triangle_grid=GRID_UNIFORM, vein_dynamic=1, refresh_triangle_centers=0, seed=0,
)


def default_params() -> Params:
    """Params filled with the reference's shipped constants (pure Python)."""
    p = Params()
    for k, v in REFERENCE_DEFAULTS.items():
        if isinstance(v, tuple):
            getattr(p, k)[:] = v
        else:
            setattr(p, k, v)
    return p


def library_default_params() -> Params:
    """The same constants as evaluated by libbcs.so's bcs_default_params."""
    p = Params()
    load_library().bcs_default_params(C.byref(p))
    return p


def _ptr(a) -> int | None:
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return int(a.data_ptr())     # torch tensor


def _rows(a, n: int, what: str) -> np.ndarray:
    """A host array of n xyz rows as float32 (the library reads exactly n)."""
    a = np.asarray(a, dtype=np.float32)
    if a.shape != (n, 3):
        raise ValueError(f"{what}: expected shape ({n}, 3), got {a.shape}")
    return a


def _dev(t, n: int, what: str) -> int | None:
    """Device pointer of a contiguous float32 CUDA tensor of n elements."""
    if t is None:
        return None
    if isinstance(t, np.ndarray) or not getattr(t, "is_cuda", False):
        raise ValueError(f"{what}: expected a CUDA tensor")
    if str(t.dtype) != "torch.float32" or not t.is_contiguous() or t.numel() != n:
        raise ValueError(f"{what}: expected a contiguous float32 tensor of {n} elements")
    return int(t.data_ptr())


def _edges_per_cell(cell_type) -> int:
    """Directed spring edges of one cell as the library builds its graph:
    the dense spring matrix (a later spring overwrites an earlier one on the
    same pair, rest length 0 is no spring), self pairs left out."""
    dense = {}
    springs = np.asarray(cell_type.springs, np.int64).reshape(-1, 2)
    for (a, b), length in zip(springs, np.asarray(cell_type.spring_lengths, np.float32).reshape(-1)):
        dense[(int(a), int(b))] = length
        dense[(int(b), int(a))] = length
    return sum(1 for (a, b), length in dense.items() if a != b and length != 0.0)


def _check(status: int, what: str) -> None:
    if status != BCS_OK:
        raise BcsError(status, what)


def set_tensor_path(path: int) -> int:
    """0 = tcgen05 products (default), 1 = mma.sync; returns the previous path."""
    return int(load_library().bcs_set_tensor_path(int(path)))


def tensor_wait_expiries() -> int:
    return int(load_library().bcs_tensor_wait_expiries())


def set_tensor_wait_probe(polls: int) -> None:
    """Testing aid: with polls > 0 the first product wait of every CTA of the
    tcgen05 kernels gives up after that many polls of a barrier nothing
    arrives at; 0 restores the normal waits."""
    _check(load_library().bcs_set_tensor_wait_probe(int(polls)), "bcs_set_tensor_wait_probe")


class Control:
    """The streaming server's control messages (bcs_control): post received
    bytes, handle one message per frame, take the bytes to send."""

    def __init__(self):
        self.lib = load_library()
        self.h = C.c_void_p()
        _check(self.lib.bcs_control_create(C.byref(self.h)), "bcs_control_create")

    def post(self, data: bytes) -> None:
        buf = (C.c_uint8 * max(1, len(data))).from_buffer_copy(bytes(data) or b"\0")
        _check(self.lib.bcs_control_post(self.h, buf, len(data)), "bcs_control_post")

    def post_event(self, name: str, state: int = EVENT_NOT_RELEVANT) -> None:
        _check(self.lib.bcs_control_post_event(self.h, Event(EVENT[name], state)), "bcs_control_post_event")

    def handle(self) -> dict:
        st = ControlState()
        _check(self.lib.bcs_control_handle(self.h, C.byref(st)), "bcs_control_handle")
        return st.as_dict()

    def send(self, name: str, state: int = EVENT_NOT_RELEVANT) -> None:
        _check(self.lib.bcs_control_send(self.h, Event(EVENT[name], state)), "bcs_control_send")

    def take_outgoing(self) -> list:
        out, b = [], C.c_uint8()
        while self.lib.bcs_control_take_outgoing(self.h, C.byref(b)):
            out.append(int(b.value))
        return out

    def close(self) -> None:
        if self.h:
            self.lib.bcs_control_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def decode_event(data: bytes):
    buf = (C.c_uint8 * max(1, len(data))).from_buffer_copy(bytes(data) or b"\0")
    e = load_library().bcs_event_decode(buf, len(data))
    return EVENT_NAMES[e.type], e.state


def encode_event(name: str, state: int):
    b = C.c_uint8()
    ch = load_library().bcs_event_encode(Event(EVENT[name], state), C.byref(b))
    return (int(b.value), ch) if ch else (None, 0)


def set_device(device: int) -> None:
    _check(load_library().bcs_set_device(int(device)), "bcs_set_device")


class SceneBuffers:
    """Keeps the numpy arrays behind a SceneDesc alive."""

    def __init__(self, scene):
        self.keep = []
        types = (CellType * len(scene.types))()
        for i, t in enumerate(scene.types):
            verts = np.ascontiguousarray(t.vertices, dtype=np.float32)
            springs = np.ascontiguousarray(t.springs, dtype=np.int32).reshape(-1, 2)
            lengths = np.ascontiguousarray(t.spring_lengths, dtype=np.float32)
            rad = None if t.collision_radius is None else np.ascontiguousarray(t.collision_radius, dtype=np.float32)
            self.keep += [verts, springs, lengths, rad]
            types[i] = CellType(int(t.count), int(verts.shape[0]), verts.ctypes.data, int(springs.shape[0]),
                                springs.ctypes.data if springs.size else None,
                                lengths.ctypes.data if lengths.size else None,
                                None if rad is None else rad.ctypes.data)
        vp = np.ascontiguousarray(scene.vein_positions, dtype=np.float32)
        vi = np.ascontiguousarray(scene.vein_indices, dtype=np.uint32)
        ec = np.ascontiguousarray(scene.ending_centers, dtype=np.float32).reshape(-1, 3)
        er = np.ascontiguousarray(scene.ending_radii, dtype=np.float32).reshape(-1)
        self.keep += [vp, vi, ec, er, types]
        vein = Vein(int(vp.shape[0]), vp.ctypes.data, int(vi.shape[0]), vi.ctypes.data if vi.size else None,
                    int(er.shape[0]), ec.ctypes.data if er.size else None, er.ctypes.data if er.size else None)
        flows = (FlowSegment * max(1, len(scene.flow_segments)))()
        for i, f in enumerate(scene.flow_segments):
            flows[i] = FlowSegment((C.c_float * 3)(*f["origin"]), (C.c_float * 3)(*f["direction"]),
                                   f["length"], f["radius"], f["peak_force"])
        self.keep.append(flows)
        self.desc = SceneDesc(len(scene.types), types, vein, len(scene.flow_segments), flows, scene.params)


class Simulation:
    """One scene on the current CUDA device (≙ BloodCells + VeinTriangles +
    two UniformGrids + SimulationController of src/main.cu:122-138), or, given
    a list of scenes, a batch of independent scenes run by one set of
    launches (bcs_create_batch).  Batch state is scene-major: scene k owns
    the rows scene_info(k).particle_start .. + particle_count."""

    def __init__(self, scene, stream: int | None = None):
        self.lib = load_library()
        h = C.c_void_p()
        if isinstance(scene, (list, tuple)):
            self.scenes = list(scene)
            self.scene = self.scenes[0]
            self._bufs = [SceneBuffers(sc) for sc in self.scenes]
            descs = (SceneDesc * len(self._bufs))(*[b.desc for b in self._bufs])
            _check(self.lib.bcs_create_batch(descs, len(self._bufs), stream, C.byref(h)), "bcs_create_batch")
        else:
            self.scenes = [scene]
            self.scene = scene
            self._bufs = SceneBuffers(scene)
            _check(self.lib.bcs_create(C.byref(self._bufs.desc), stream, C.byref(h)), "bcs_create")
        self.h = h
        self._async_keep = []
        self.info = Info()
        _check(self.lib.bcs_get_info(self.h, C.byref(self.info)), "bcs_get_info")
        self.n = self.info.particle_count
        self.nv = self.info.vertex_count

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.bcs_destroy(self.h)
            self.h = None
            self._async_keep.clear()   # bcs_destroy waited for the reads

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---- state ------------------------------------------------------------
    def set_particles(self, pos, vel, force=None) -> None:
        """pos/vel/force: [N, 3] float32 numpy arrays (host)."""
        soa = [np.ascontiguousarray(_rows(a, self.n, k).T) for a, k in ((pos, "pos"), (vel, "vel"))]
        f = None if force is None else np.ascontiguousarray(_rows(force, self.n, "force").T)
        vecs = [Vec3(a[0].ctypes.data, a[1].ctypes.data, a[2].ctypes.data) for a in soa]
        fv = Vec3() if f is None else Vec3(f[0].ctypes.data, f[1].ctypes.data, f[2].ctypes.data)
        _check(self.lib.bcs_set_particles(self.h, vecs[0], vecs[1], fv, MEM_HOST), "bcs_set_particles")

    def get_particles(self):
        out = [np.empty((3, self.n), np.float32) for _ in range(3)]
        vecs = [Vec3(a[0].ctypes.data, a[1].ctypes.data, a[2].ctypes.data) for a in out]
        _check(self.lib.bcs_get_particles(self.h, vecs[0], vecs[1], vecs[2], MEM_HOST), "bcs_get_particles")
        return tuple(np.ascontiguousarray(a.T) for a in out)

    def get_particles_async(self, pos=None, vel=None, force=None) -> None:
        """Start reading the state into caller-owned host arrays without
        waiting (bcs_get_particles_async): each a C-contiguous float32 array
        of shape (3, n), rows x, y, z, kept alive and unread until
        wait_particles()."""
        def v3(a):
            if a is None:
                return Vec3()
            if a.dtype != np.float32 or a.shape != (3, self.n) or not a.flags.c_contiguous:
                raise ValueError("expected a C-contiguous float32 array of shape (3, n)")
            return Vec3(a[0].ctypes.data, a[1].ctypes.data, a[2].ctypes.data)
        vecs = (v3(pos), v3(vel), v3(force))
        self._async_keep.append((pos, vel, force))
        _check(self.lib.bcs_get_particles_async(self.h, *vecs), "bcs_get_particles_async")

    def crowded_particles(self) -> int:
        """Particles set aside as crowded, summed over all steps so far."""
        v = C.c_longlong()
        _check(self.lib.bcs_get_crowded(self.h, C.byref(v)), "bcs_get_crowded")
        return int(v.value)

    def wait_particles(self) -> None:
        _check(self.lib.bcs_wait_particles(self.h), "bcs_wait_particles")
        self._async_keep.clear()

    def init_particles(self, kind: int = INIT_LATTICE, seed: int = 0, velocity_sigma: float = 0.0,
                       gap: float = 0.2) -> None:
        """Initial state on the device (bcs_init_particles)."""
        d = InitDesc(int(kind), int(seed), float(velocity_sigma), float(gap))
        _check(self.lib.bcs_init_particles(self.h, C.byref(d)), "bcs_init_particles")

    def set_particles_device(self, x, y, z, vx, vy, vz) -> None:
        """Device pointers (torch CUDA tensors) in cudaVec3 SoA layout."""
        p = [_dev(a, self.n, "set_particles_device") for a in (x, y, z, vx, vy, vz)]
        if None in p:
            raise ValueError("set_particles_device: all six component tensors are required")
        _check(self.lib.bcs_set_particles(self.h, Vec3(*p[:3]), Vec3(*p[3:]), Vec3(), MEM_DEVICE), "bcs_set_particles")

    def get_particles_device(self, x, y, z, vx=None, vy=None, vz=None) -> None:
        p = [_dev(a, self.n, "get_particles_device") for a in (x, y, z, vx, vy, vz)]
        _check(self.lib.bcs_get_particles(self.h, Vec3(*p[:3]), Vec3(*p[3:]), Vec3(), MEM_DEVICE),
               "bcs_get_particles")

    def set_vein(self, pos=None, vel=None) -> None:
        keep = []

        def v3(a):
            if a is None:
                return Vec3()
            s = np.ascontiguousarray(_rows(a, self.nv, "set_vein").T)
            keep.append(s)
            return Vec3(s[0].ctypes.data, s[1].ctypes.data, s[2].ctypes.data)
        _check(self.lib.bcs_set_vein(self.h, v3(pos), v3(vel), MEM_HOST), "bcs_set_vein")

    def get_vein(self):
        out = [np.empty((3, self.nv), np.float32) for _ in range(3)]
        vecs = [Vec3(a[0].ctypes.data, a[1].ctypes.data, a[2].ctypes.data) for a in out]
        _check(self.lib.bcs_get_vein(self.h, vecs[0], vecs[1], vecs[2], MEM_HOST), "bcs_get_vein")
        return tuple(np.ascontiguousarray(a.T) for a in out)

    # ---- the frame ---------------------------------------------------------
    def calculate_grids(self) -> None:
        _check(self.lib.bcs_calculate_grids(self.h), "bcs_calculate_grids")

    def calculate_next_frame(self) -> None:
        _check(self.lib.bcs_calculate_next_frame(self.h), "bcs_calculate_next_frame")

    def propagate_all(self) -> None:
        _check(self.lib.bcs_propagate_all(self.h), "bcs_propagate_all")

    def step(self, nsteps: int = 1) -> None:
        _check(self.lib.bcs_step(self.h, int(nsteps)), "bcs_step")

    def run(self, max_frames: int, control=None) -> int:
        """The server loop (bcs_run): frames until a handled stopRendering
        message or max_frames + 1 frames; returns the frames run."""
        n = C.c_int()
        _check(self.lib.bcs_run(self.h, control.h if control is not None else None, int(max_frames), C.byref(n)),
               "bcs_run")
        return int(n.value)

    def macro_step(self, substeps: int, n: int = 1) -> None:
        """n multi-rate macro steps of `substeps` time steps each."""
        _check(self.lib.bcs_macro_step(self.h, int(substeps), int(n)), "bcs_macro_step")

    def time_macro_steps(self, substeps: int, n: int) -> float:
        ms = C.c_float()
        _check(self.lib.bcs_time_macro_steps(self.h, int(substeps), int(n), C.byref(ms)), "bcs_time_macro_steps")
        return ms.value

    def time_steps(self, nsteps: int) -> float:
        ms = C.c_float()
        _check(self.lib.bcs_time_steps(self.h, int(nsteps), C.byref(ms)), "bcs_time_steps")
        return ms.value

    def profile_steps(self, nsteps: int) -> dict:
        """Eager frames with CUDA events between phases: summed ms per phase."""
        ms = (C.c_float * len(PHASES))()
        _check(self.lib.bcs_profile_steps(self.h, int(nsteps), ms), "bcs_profile_steps")
        return dict(zip(PHASES, list(ms)))

    def synchronize(self) -> None:
        _check(self.lib.bcs_synchronize(self.h), "bcs_synchronize")

    # ---- inspection ---------------------------------------------------------
    def get_grid(self, which: int = 0, dense: bool = True):
        cnt = self.n if which == 0 else self.info.triangle_count
        cells = self.info.cell_count if which == 0 else self.info.tri_cell_count
        keys = np.empty(cnt, np.int32)
        ids = np.empty(cnt, np.int32)
        starts = np.empty(cells, np.int32) if dense else None
        ends = np.empty(cells, np.int32) if dense else None
        _check(self.lib.bcs_get_grid(self.h, which, keys.ctypes.data, ids.ctypes.data, _ptr(starts), _ptr(ends),
                                     MEM_HOST), "bcs_get_grid")
        return keys, ids, starts, ends

    def export_render(self):
        pv = np.empty((self.n, 6), np.float32)
        po = np.empty((self.n, 3), np.float32)
        vv = np.empty((self.nv, 6), np.float32)
        _check(self.lib.bcs_export_render(self.h, pv.ctypes.data, po.ctypes.data, vv.ctypes.data, MEM_HOST),
               "bcs_export_render")
        return pv, po, vv

    def error_word(self, clear: bool = False) -> int:
        w = C.c_uint32()
        _check(self.lib.bcs_get_error_word(self.h, C.byref(w), int(clear)), "bcs_get_error_word")
        return int(w.value)

    # ---- launch tuning ------------------------------------------------------
    def get_tuning(self) -> Tuning:
        t = Tuning()
        _check(self.lib.bcs_get_tuning(self.h, C.byref(t)), "bcs_get_tuning")
        return t

    def set_tuning(self, step_shape=0, persistent=0, spatial_order=0, full_sort=0, occupancy_filter=0,
                   sorted_positions=0, grid_collisions=3) -> None:
        t = Tuning(int(step_shape), int(persistent), int(spatial_order), int(full_sort), int(occupancy_filter),
                   int(sorted_positions), int(grid_collisions))
        _check(self.lib.bcs_set_tuning(self.h, C.byref(t)), "bcs_set_tuning")

    def set_mover_sort(self, mode: int) -> None:
        """0: by a recent frame's mover count, 1: movers by radix passes, 2: by one CTA,
        3: every pair from scratch (the same order in all)."""
        _check(self.lib.bcs_set_mover_sort(self.h, int(mode)), "bcs_set_mover_sort")

    def autotune(self, frames: int = 5):
        """Coordinate-descent search over the tuning; keeps the fastest, state unchanged."""
        t = Tuning()
        ms = C.c_float()
        _check(self.lib.bcs_autotune(self.h, int(frames), C.byref(t), C.byref(ms)), "bcs_autotune")
        return t, ms.value

    def scene_info(self, k: int) -> SceneInfo:
        out = SceneInfo()
        _check(self.lib.bcs_get_scene_info(self.h, int(k), C.byref(out)), "bcs_get_scene_info")
        return out

    def refresh_info(self) -> Info:
        _check(self.lib.bcs_get_info(self.h, C.byref(self.info)), "bcs_get_info")
        return self.info


class Surrogate:
    """The learned sub-step network of one cell model of `sim` (a
    bcs_surrogate handle)."""

    def __init__(self, sim: Simulation, cell_type: int = 0, substeps: int = 8, layers: int = 3,
                 max_samples: int = 4096, seed: int = 1, tolerance: float = 0.0, huber_delta: float = 0.0):
        self.lib = sim.lib
        self.sim = sim
        d = SurrogateDesc(int(cell_type), int(substeps), int(layers), int(max_samples), int(seed), float(tolerance),
                          float(huber_delta))
        h = C.c_void_p()
        _check(self.lib.bcs_surrogate_create(sim.h, C.byref(d), C.byref(h)), "bcs_surrogate_create")
        self.h = h
        self.substeps = int(substeps)
        t = sim.scene.types[cell_type]
        self.pic = len(t.vertices)
        self.edges = _edges_per_cell(t)

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.bcs_surrogate_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def collect(self, macro_steps: int) -> None:
        _check(self.lib.bcs_surrogate_collect(self.h, int(macro_steps)), "bcs_surrogate_collect")

    def train(self, iterations: int, batch_cells: int = 64, lr: float = 1e-3) -> float:
        loss = C.c_float()
        _check(self.lib.bcs_surrogate_train(self.h, int(iterations), int(batch_cells), float(lr), C.byref(loss)),
               "bcs_surrogate_train")
        return loss.value

    def enable(self, on: bool = True, fused: bool = True) -> None:
        """Use the network in macro steps (fused: one kernel per macro step)."""
        _check(self.lib.bcs_surrogate_enable(self.h, (1 if fused else 2) if on else 0), "bcs_surrogate_enable")

    def stats(self) -> dict:
        st = SurrogateStats()
        _check(self.lib.bcs_surrogate_get_stats(self.h, C.byref(st)), "bcs_surrogate_get_stats")
        return st.as_dict()

    def reset_stats(self) -> None:
        _check(self.lib.bcs_surrogate_reset_stats(self.h), "bcs_surrogate_reset_stats")

    def param_count(self) -> int:
        return int(self.lib.bcs_surrogate_param_count(self.h))

    def get_params(self) -> np.ndarray:
        out = np.empty(self.param_count(), np.float32)
        _check(self.lib.bcs_surrogate_get_params(self.h, out.ctypes.data, out.size), "bcs_surrogate_get_params")
        return out

    def set_params(self, p) -> None:
        p = np.ascontiguousarray(p, np.float32).reshape(-1)
        _check(self.lib.bcs_surrogate_set_params(self.h, p.ctypes.data, p.size), "bcs_surrogate_set_params")

    def _inputs(self, cells, features, edge_features, targets=None):
        """The host arrays of `cells` cells, checked against the sizes the
        library reads: (cells x pic, 16) node features, (cells x edges, 8)
        edge features, (cells x pic, 9) targets."""
        n, m = int(cells) * self.pic, int(cells) * self.edges
        want = [("features", features, (n, 16)), ("edge_features", edge_features, (m, 8))]
        if targets is not None:
            want.append(("targets", targets, (n, 9)))
        out = []
        for name, a, shape in want:
            a = np.ascontiguousarray(a, np.float32)
            if a.shape != shape:
                raise ValueError(f"{name}: expected shape {shape} for {cells} cells, got {a.shape}")
            out.append(a)
        return out

    def loss_grad(self, cells, features, edge_features, targets):
        f, e, t = self._inputs(cells, features, edge_features, targets)
        loss = np.zeros(1, np.float32)
        g = np.empty(self.param_count(), np.float32)
        _check(self.lib.bcs_surrogate_loss_grad(self.h, int(cells), f.ctypes.data, e.ctypes.data, t.ctypes.data,
                                                loss.ctypes.data, g.ctypes.data), "bcs_surrogate_loss_grad")
        return float(loss[0]), g

    def forward(self, cells, features, edge_features):
        f, e = self._inputs(cells, features, edge_features)
        y = np.empty((f.shape[0], 9), np.float32)
        _check(self.lib.bcs_surrogate_forward(self.h, int(cells), f.ctypes.data, e.ctypes.data, y.ctypes.data),
               "bcs_surrogate_forward")
        return y

    def evaluate(self, first: int, count: int):
        """(network error, extrapolation error) on stored samples [first, first + count)."""
        a, b = C.c_double(), C.c_double()
        _check(self.lib.bcs_surrogate_evaluate(self.h, int(first), int(count), C.byref(a), C.byref(b)),
               "bcs_surrogate_evaluate")
        return a.value, b.value

    def scales(self) -> np.ndarray:
        out = np.empty(53, np.float32)
        _check(self.lib.bcs_surrogate_get_scales(self.h, out.ctypes.data), "bcs_surrogate_get_scales")
        return out

    def set_scales(self, sc) -> None:
        sc = np.ascontiguousarray(sc, np.float32).reshape(-1)
        if sc.size != 53:
            raise ValueError(f"scales: expected 53 values, got {sc.size}")
        _check(self.lib.bcs_surrogate_set_scales(self.h, sc.ctypes.data), "bcs_surrogate_set_scales")
