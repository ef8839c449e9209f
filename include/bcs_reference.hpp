// bcs_reference.hpp — adaptor for the reference's own build: fills a
// bcs_scene_desc from its compile-time scene.
//
// Include this from a translation unit of GPU-Blood-Cell-Simulation/
// Simulation-Server after its meta_factory headers; it reads the folded
// layout those headers define (BloodCellList, particleStarts,
// bloodCellModelStarts, accumulatedGraphSizes, springGraph —
// src/meta_factory/blood_cell_factory.hpp:117-328; veinPositions,
// veinIndices, VeinEndingCenters/Radii — src/config/vein_definition.hpp;
// the constants of src/config/simulation.hpp and physics.hpp), so the engine
// runs exactly the scene the reference was compiled for.  Springs come from
// the dense graph (0 = no spring), collision radii are left to the library
// (it derives them as generateBoundingSpheres does).
//
//   bcs_reference::Scene scene;           // keeps the arrays alive
//   bcs_sim* sim;
//   bcs_create(&scene.desc, nullptr, &sim);
#pragma once

#include <cstdint>
#include <vector>

#include "bcs.h"

namespace bcs_reference {

struct Scene {
    std::vector<bcs_cell_type> types;
    std::vector<std::vector<float>> vertices, lengths;
    std::vector<std::vector<int>> springs;
    std::vector<float> vein_positions, ending_centers, ending_radii;
    std::vector<uint32_t> vein_indices;
    bcs_scene_desc desc{};

    Scene() {
        using namespace boost::mp11;
        mp_for_each<mp_iota_c<bloodCellTypeCount>>([&](auto i) {
            using Def = mp_at_c<BloodCellList, i>;
            constexpr int pic = Def::particlesInCell;
            std::vector<float> v;
            mp_for_each<mp_iota_c<pic>>([&](auto j) {
                using P = mp_at_c<typename Def::Vertices, j>;
                v.push_back(P::x);
                v.push_back(P::y);
                v.push_back(P::z);
            });
            std::vector<int> s;
            std::vector<float> l;
            const int g0 = accumulatedGraphSizes[i];
            for (int a = 0; a < pic; ++a)
                for (int b = a + 1; b < pic; ++b) {
                    float len = springGraph[g0 + a * pic + b];
                    if (len != 0.0f) {
                        s.push_back(a);
                        s.push_back(b);
                        l.push_back(len);
                    }
                }
            vertices.push_back(std::move(v));
            springs.push_back(std::move(s));
            lengths.push_back(std::move(l));
            bcs_cell_type t{};
            t.count = Def::count;
            t.particles_in_cell = pic;
            types.push_back(t);
        });
        for (size_t k = 0; k < types.size(); ++k) {
            types[k].vertices = vertices[k].data();
            types[k].spring_count = (int)lengths[k].size();
            types[k].springs = springs[k].data();
            types[k].spring_lengths = lengths[k].data();
            types[k].collision_radius = nullptr;
        }
        for (auto& p : veinPositions) {
            vein_positions.push_back(p.x);
            vein_positions.push_back(p.y);
            vein_positions.push_back(p.z);
        }
        vein_indices.assign(veinIndices.begin(), veinIndices.end());
        mp_for_each<mp_iota_c<veinEndingCenterCount>>([&](auto i) {
            using E = mp_at_c<VeinEndingCenters, i>;
            ending_centers.push_back(E::x);
            ending_centers.push_back(E::y);
            ending_centers.push_back(E::z);
            ending_radii.push_back(mp_at_c<VeinEndingRadii, i>::value);
        });
        bcs_params& p = desc.params;
        bcs_default_params(&p);
        p.dt = dt;
        p.use_blood_flow = useBloodFlow;
        p.enable_reaction_force = enableReactionForce;
        p.enable_big_cells_brake = enableBigCellsBrake;
        p.cell_width = (float)cellWidth;
        p.cell_height = (float)cellHeight;
        p.cell_depth = (float)cellDepth;
        p.cell_width_triangles = (float)cellWidthTriangles;
        p.cell_height_triangles = (float)cellHeightTriangles;
        p.cell_depth_triangles = (float)cellDepthTriangles;
        p.bounding_spheres_coeff = (float)boundingSpheresCoeff;
        p.grid_y_margin = gridYMargin;
        p.grid_xz_margin = gridXZMargin;
        p.min_spawn_y = minSpawnY;
        p.velocity_collision_damping = velocity_collision_damping;
        p.particle_k_sniff = particle_k_sniff;
        p.vein_k_sniff = vein_k_sniff;
        p.particle_d_fact = particle_d_fact;
        p.vein_d_fact = vein_d_fact;
        p.vein_collision_force_intensity = vein_collision_force_intensity;
        p.viscous_damping = viscous_damping;
        p.collision_spring_coeff = collisionSpringCoeff;
        p.collision_damping_coeff = collisionDampingCoeff;
        p.collision_shear_coeff = collistionShearCoeff;
        p.max_cell_size_factor_before_brake = maxCellSizeFactorBeforeBrake;
        p.big_particle_braking_intensity = bigParticleBrakingIntensity;
        p.init_velocity[0] = initVelocityX;
        p.init_velocity[1] = initVelocityY;
        p.init_velocity[2] = initVelocityZ;
        p.vein_impact_distance = veinImpactDistance;
        p.vein_impact_minimal_force_distance = veinImpactMinimalForceDistance;
        p.gravity[0] = Gx;
        p.gravity[1] = Gy;
        p.gravity[2] = Gz;
        p.cylinder_radius = cylinderRadius;
        desc.type_count = (int)types.size();
        desc.types = types.data();
        desc.vein.vertex_count = (int)veinPositions.size();
        desc.vein.positions = vein_positions.data();
        desc.vein.triangle_count = (int)(vein_indices.size() / 3);
        desc.vein.indices = vein_indices.data();
        desc.vein.ending_count = (int)ending_radii.size();
        desc.vein.ending_centers = ending_centers.data();
        desc.vein.ending_radii = ending_radii.data();
        desc.flow_segment_count = 0;
        desc.flow_segments = nullptr;
    }
};

}  // namespace bcs_reference
