// Test helper of tests/test_ref_adaptor.py: compiled against a reference
// source tree whose src/config holds a generated scene, it builds the
// bcs_scene_desc that include/bcs_reference.hpp fills from the reference's
// compile-time scene (its meta_factory layout and config constants) and
// writes it to one binary file:
//   int32 type_count, then per type: int32 count, pic, spring_count,
//     float32 vertices[pic][3], int32 springs[spring_count][2],
//     float32 lengths[spring_count];
//   int32 vertex_count, triangle_count, ending_count, float32 positions[V][3],
//     uint32 indices[T][3], float32 ending_centers[E][3], ending_radii[E];
//   int32 sizeof(bcs_params), then the bcs_params bytes.
#include "config/physics.hpp"
#include "config/simulation.hpp"
#include "meta_factory/blood_cell_factory.hpp"
#include "meta_factory/vein_factory.hpp"

#include "bcs_reference.hpp"

#include <cstdio>

namespace {
FILE* out = nullptr;
template <class T>
void put(const T* p, size_t n) {
    if (n && std::fwrite(p, sizeof(T), n, out) != n) {
        std::perror("write");
        std::exit(2);
    }
}
void put_i(int v) { put(&v, 1); }
}  // namespace

int main(int argc, char** argv) {
    if (argc != 2) {
        std::fprintf(stderr, "usage: ref_adaptor_dump <out.bin>\n");
        return 1;
    }
    out = std::fopen(argv[1], "wb");
    if (!out) {
        std::perror(argv[1]);
        return 2;
    }
    bcs_reference::Scene scene;
    const bcs_scene_desc& d = scene.desc;
    put_i(d.type_count);
    for (int t = 0; t < d.type_count; ++t) {
        const bcs_cell_type& c = d.types[t];
        put_i(c.count);
        put_i(c.particles_in_cell);
        put_i(c.spring_count);
        put(c.vertices, 3 * (size_t)c.particles_in_cell);
        put(c.springs, 2 * (size_t)c.spring_count);
        put(c.spring_lengths, (size_t)c.spring_count);
    }
    put_i(d.vein.vertex_count);
    put_i(d.vein.triangle_count);
    put_i(d.vein.ending_count);
    put(d.vein.positions, 3 * (size_t)d.vein.vertex_count);
    put(d.vein.indices, 3 * (size_t)d.vein.triangle_count);
    put(d.vein.ending_centers, 3 * (size_t)d.vein.ending_count);
    put(d.vein.ending_radii, (size_t)d.vein.ending_count);
    put_i((int)sizeof(bcs_params));
    put(reinterpret_cast<const unsigned char*>(&d.params), sizeof(bcs_params));
    std::fclose(out);
    return 0;
}
