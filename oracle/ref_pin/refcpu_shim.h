// refcpu_shim.h — force-included when the reference's sources are compiled
// with g++ for the host (pin recipe, test infrastructure).  Kernels become
// plain functions (__global__/__device__ expand to ignored attributes in host
// compilation); the launch rewrite calls bcs_launch, which runs every
// (block, thread) of the grid serially, one after another.
#pragma once
#include <cmath>
#include <cstdio>
using std::isnan;
#include <cuda_runtime.h>

struct bcs_dims {
    dim3 grid, block;
};
template <class G, class B, class... R>
inline bcs_dims bcs_cfg(G g, B b, R...) {
    return bcs_dims{dim3(g), dim3(b)};
}

extern "C" {
extern uint3 threadIdx;
extern uint3 blockIdx;
extern dim3 blockDim;
extern dim3 gridDim;
}

template <class F>
inline void bcs_launch(bcs_dims d, F&& f) {
    gridDim = d.grid;
    blockDim = d.block;
    for (unsigned bz = 0; bz < d.grid.z; ++bz)
        for (unsigned by = 0; by < d.grid.y; ++by)
            for (unsigned bx = 0; bx < d.grid.x; ++bx)
                for (unsigned tz = 0; tz < d.block.z; ++tz)
                    for (unsigned ty = 0; ty < d.block.y; ++ty)
                        for (unsigned tx = 0; tx < d.block.x; ++tx) {
                            blockIdx = uint3{bx, by, bz};
                            threadIdx = uint3{tx, ty, tz};
                            f();
                        }
}
