"""Reference-format scene configuration: emit and import.

The reference's scene is compile-time C++: src/config/simulation.hpp and
physics.hpp hold scalar constants, blood_cells_definition.hpp lists
BloodCellDef<count, particlesInCell, indicesInCell, color, Springs, Vertices,
Indices, Normals> entries, blood_cell_presets.hpp defines those lists with
Spring<start, end, length> and mp_float3<x, y, z, precision> fixed-point
integers, and vein_definition.hpp holds the mesh as constexpr std::arrays plus
VeinEndingCenters / VeinEndingRadii (src/meta_factory/mp_helpers.hpp:24-36,
blood_cells_def_type.hpp:21-46).

emit_config() writes such a set for a runtime Scene so the reference can be
built on the identical scene; import_config() goes the other way, compiling
the reference's own meta_factory on a config set (g++, host only) and turning
its folded layout into a Scene.
"""
from __future__ import annotations

import os
import subprocess
import tempfile

import numpy as np

from bcs import REFERENCE_DEFAULTS, Params, default_params

SIMULATION_INT = ("cellWidth", "cellHeight", "cellDepth", "cellWidthTriangles", "cellHeightTriangles",
                  "cellDepthTriangles", "boundingSpheresCoeff")


def _f(x: float) -> str:
    s = f"{float(np.float32(x)):.9g}"
    return s if ("." in s or "e" in s or "inf" in s or "nan" in s) else s + ".0"


def simulation_hpp(p: Params, max_frames: int = 600) -> str:
    def i(v, name):
        if float(v) != int(v):
            raise ValueError(f"{name} must be integral in the reference's config ({v})")
        return int(v)
    return f"""#pragma once

inline constexpr int maxFrames = {max_frames};
inline constexpr int maxCudaStreams = 16;
inline constexpr float dt = {_f(p.dt)};
inline constexpr bool useBloodFlow = {int(bool(p.use_blood_flow))};
inline constexpr bool enableReactionForce = {int(bool(p.enable_reaction_force))};
inline constexpr bool enableBigCellsBrake = {int(bool(p.enable_big_cells_brake))};

inline constexpr int cellWidth = {i(p.cell_width, 'cell_width')};
inline constexpr int cellHeight = {i(p.cell_height, 'cell_height')};
inline constexpr int cellDepth  = {i(p.cell_depth, 'cell_depth')};

inline constexpr int cellWidthTriangles = {i(p.cell_width_triangles, 'cell_width_triangles')};
inline constexpr int cellHeightTriangles = {i(p.cell_height_triangles, 'cell_height_triangles')};
inline constexpr int cellDepthTriangles = {i(p.cell_depth_triangles, 'cell_depth_triangles')};

inline constexpr int boundingSpheresCoeff = {i(p.bounding_spheres_coeff, 'bounding_spheres_coeff')};
inline constexpr float gridYMargin = {_f(p.grid_y_margin)};
inline constexpr float gridXZMargin = {_f(p.grid_xz_margin)};
inline constexpr float minSpawnY = {_f(p.min_spawn_y)};
"""


def physics_hpp(p: Params) -> str:
    rows = [
        ("velocity_collision_damping", p.velocity_collision_damping), ("particle_k_sniff", p.particle_k_sniff),
        ("vein_k_sniff", p.vein_k_sniff), ("particle_d_fact", p.particle_d_fact), ("vein_d_fact", p.vein_d_fact),
        ("vein_boundaries_velocity_damping", 0.65), ("vein_collision_force_intensity", p.vein_collision_force_intensity),
        ("viscous_damping", p.viscous_damping), ("collisionSpringCoeff", p.collision_spring_coeff),
        ("collisionDampingCoeff", p.collision_damping_coeff), ("collistionShearCoeff", p.collision_shear_coeff),
        ("maxCellSizeFactorBeforeBrake", p.max_cell_size_factor_before_brake),
        ("bigParticleBrakingIntensity", p.big_particle_braking_intensity),
        ("initVelocityX", p.init_velocity[0]), ("initVelocityY", p.init_velocity[1]),
        ("initVelocityZ", p.init_velocity[2]), ("randomVelocityModifier", 0.894),
        ("veinImpactDistance", p.vein_impact_distance),
        ("veinImpactMinimalForceDistance", p.vein_impact_minimal_force_distance),
        ("Gx", p.gravity[0]), ("Gy", p.gravity[1]), ("Gz", p.gravity[2]),
    ]
    body = "\n".join(f"inline constexpr float {k} = {_f(v)};" for k, v in rows)
    return "#pragma once\n#include \"simulation.hpp\"\n\n" + body + "\n"


def vein_definition_hpp(positions, indices, ending_centers, ending_radii, precision: int = 5) -> str:
    pos = np.asarray(positions, np.float32).reshape(-1, 3)
    idx = np.asarray(indices, np.uint32).reshape(-1)
    lines = ["#pragma once", '#include "../meta_factory/mp_helpers.hpp"', '#include "../utilities/constexpr_vec.hpp"',
             "", "#include <array>", "#include <boost/mp11/list.hpp>", "", "using namespace boost::mp11;", "",
             f"inline constexpr std::array<cvec, {len(pos)}> veinPositions {{"]
    lines.append(",\n".join(", ".join(f"static_cast<float>({_f(c)})" for c in row) for row in pos))
    lines.append("};\n")
    lines.append(f"inline constexpr std::array<unsigned int, {len(idx)}> veinIndices {{")
    lines.append(",\n".join(", ".join(str(int(v)) for v in idx[k:k + 6]) for k in range(0, len(idx), 6)))
    lines.append("};\n")
    scale = 10 ** (precision - 1)

    def fixed(v):
        q = int(round(float(v) * scale))
        if abs(q) > 2**31 - 1:
            raise ValueError("vein ending does not fit the fixed-point format")
        return q
    cen = np.asarray(ending_centers, np.float64).reshape(-1, 3)
    rad = np.asarray(ending_radii, np.float64).reshape(-1)
    lines.append("using VeinEndingCenters = mp_list<")
    lines.append(",\n".join(f"mp_float3<{fixed(c[0])}, {fixed(c[1])}, {fixed(c[2])}, {precision}>" for c in cen))
    lines.append(">;\n")
    lines.append("using VeinEndingRadii = mp_list<")
    lines.append(",\n".join(f"mp_float<{fixed(r)}, {precision}>" for r in rad))
    lines.append(">;\n")
    return "\n".join(lines)


def preset_hpp(name: str, vertices, springs, spring_lengths, precision: int = 7) -> str:
    """One cell model as Spring / mp_float3 lists (fixed point, 10^(precision-1))."""
    scale = 10 ** (precision - 1)
    v = np.asarray(vertices, np.float64).reshape(-1, 3)
    sp = np.asarray(springs, np.int64).reshape(-1, 2)
    ln = np.asarray(spring_lengths, np.float64).reshape(-1)
    out = [f"using {name}_Springs = mp_list<"]
    out.append(",\n".join(f"\tSpring<{a}, {b}, {int(round(l * scale))}, {precision}>" for (a, b), l in zip(sp, ln)))
    out.append(">;\n")
    out.append(f"using {name}_Vertices = mp_list<")
    out.append(",\n".join(f"\tmp_float3<{int(round(x * scale))}, {int(round(y * scale))}, {int(round(z * scale))}, "
                          f"{precision}>" for x, y, z in v))
    out.append(">;\n")
    out.append(f"using {name}_Indices = mp_list<>;\nusing {name}_Normals = mp_list<>;\n")
    return "\n".join(out)


def blood_cells_definition_hpp(entries) -> str:
    """entries: (count, particles_in_cell, preset_name) in user order."""
    defs = ",\n\n".join(
        f"\tBloodCellDef<{c}, {pic}, 0, 0,\n\t\tpreset::{n}_Springs,\n\t\tpreset::{n}_Vertices,\n"
        f"\t\tpreset::{n}_Indices,\n\t\tpreset::{n}_Normals>" for c, pic, n in entries)
    return ('#pragma once\n\n#include "blood_cell_presets.hpp"\n#include "../meta_factory/blood_cells_def_type.hpp"\n\n'
            "#include <boost/mp11/list.hpp>\n\n\nnamespace\n{\n\tusing namespace boost::mp11;\n\n"
            f"\tusing UserDefinedBloodCellList = mp_list<\n{defs}\n\t> ;\n}}\n")


def emit_config(scene, out_dir: str, preset_names=None, keep_presets: bool = False) -> None:
    """Write a reference-format src/config set for `scene` into out_dir.  With
    keep_presets, blood_cell_presets.hpp is left alone and `preset_names` name
    existing presets for the scene's types."""
    os.makedirs(out_dir, exist_ok=True)
    names = preset_names or [f"Scene_type_{i}" for i in range(len(scene.types))]
    with open(os.path.join(out_dir, "simulation.hpp"), "w") as f:
        f.write(simulation_hpp(scene.params))
    with open(os.path.join(out_dir, "physics.hpp"), "w") as f:
        f.write(physics_hpp(scene.params))
    with open(os.path.join(out_dir, "vein_definition.hpp"), "w") as f:
        f.write(vein_definition_hpp(scene.vein_positions, scene.vein_indices, scene.ending_centers,
                                    scene.ending_radii))
    if not keep_presets:
        body = "\n".join(preset_hpp(n, t.vertices, t.springs, t.spring_lengths) for n, t in zip(names, scene.types))
        with open(os.path.join(out_dir, "blood_cell_presets.hpp"), "w") as f:
            f.write('#pragma once\n\n#include "../meta_factory/blood_cells_def_type.hpp"\n\n'
                    "#include <boost/mp11/list.hpp>\n#include <boost/mp11/mpl_tuple.hpp>\n#include <glm/vec3.hpp>\n\n"
                    "namespace preset\n{\n\tusing namespace boost::mp11;\n\n" + body + "\n}\n")
    with open(os.path.join(out_dir, "blood_cells_definition.hpp"), "w") as f:
        f.write(blood_cells_definition_hpp([(t.count, len(t.vertices), n) for t, n in zip(scene.types, names)]))


# ------------------------------------------------------------------ import --
def read_dump(d: str, name: str, dtype, shape=None):
    a = np.fromfile(os.path.join(d, name + ".bin"), dtype=dtype)
    return a.reshape(shape) if shape is not None else a


def layout_from_dump(d: str) -> dict:
    """The folded layout a layout-only run of the pin driver dumps."""
    ints = read_dump(d, "layout_ints", np.int32)
    out = dict(particle_count=int(ints[0]), blood_cell_count=int(ints[1]), type_count=int(ints[2]),
               model_vertex_count=int(ints[3]), graph_size=int(ints[4]), vein_vertex_count=int(ints[5]),
               triangle_count=int(ints[6]))
    out["particle_starts"] = read_dump(d, "particle_starts", np.int32)
    out["cell_type_starts"] = read_dump(d, "cell_type_starts", np.int32)
    out["model_starts"] = read_dump(d, "model_starts", np.int32)
    out["graph_starts"] = read_dump(d, "graph_starts", np.int32)
    out["spring_graph"] = read_dump(d, "spring_graph", np.float32)
    out["bounds"] = read_dump(d, "bounds", np.float32)
    tp = read_dump(d, "type_pic_count", np.int32).reshape(-1, 2)
    out["pic"], out["count"] = tp[:, 0].copy(), tp[:, 1].copy()
    out["models"] = read_dump(d, "models", np.float32).reshape(-1, 3)
    nv = out["vein_vertex_count"]
    out["vein_nb_ids"] = read_dump(d, "vein_nb_ids", np.int32).reshape(9, nv)
    out["vein_nb_len"] = read_dump(d, "vein_nb_len", np.float32).reshape(9, nv)
    out["bounding_spheres"] = read_dump(d, "bounding_spheres", np.float32)
    out["initial_radii"] = read_dump(d, "initial_radii", np.float32)
    return out


def springs_from_dense(graph: np.ndarray, pic: int):
    """(start, end) pairs with start < end and their rest lengths from one
    type's dense pic x pic graph (0 = no spring)."""
    g = graph.reshape(pic, pic)
    a, b = np.nonzero(np.triu(g, 1))
    return np.stack([a, b], 1).astype(np.int32), g[a, b].astype(np.float32)


def scene_from_layout(lay: dict, vein_positions, vein_indices, ending_centers, ending_radii, params: Params,
                      positions=None, velocities=None, name="reference-config"):
    from bcs_scenes import CellTypeSpec, Scene
    types = []
    for t in range(lay["type_count"]):
        pic = int(lay["pic"][t])
        m0 = int(lay["model_starts"][t])
        g0 = int(lay["graph_starts"][t])
        sp, ln = springs_from_dense(lay["spring_graph"][g0:g0 + pic * pic], pic)
        types.append(CellTypeSpec(int(lay["count"][t]), lay["models"][m0:m0 + pic].copy(), sp, ln, None,
                                  f"type{t}"))
    n = lay["particle_count"]
    pos = np.zeros((n, 3), np.float32) if positions is None else np.asarray(positions, np.float32)
    vel = np.zeros((n, 3), np.float32) if velocities is None else np.asarray(velocities, np.float32)
    return Scene(name, types, np.asarray(vein_positions, np.float32), np.asarray(vein_indices, np.uint32),
                 np.asarray(ending_centers, np.float32), np.asarray(ending_radii, np.float32), [], params, pos, vel)
