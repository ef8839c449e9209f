// bcs_noalloc.cu — grid key + stable sort that allocates no device memory.
//
// Some callers cannot allocate: a host application that owns the whole
// device-memory budget and hands the library only its inputs and outputs, or
// a frame loop that must never stall on cudaMalloc/cudaFree (both can
// synchronise the device).  bcs_grid_sort_static gives them the particle
// grid's cell ids and stable order (the reference's calculateCellIdKernel +
// thrust::stable_sort_by_key, src/grids/uniform_grid.cu:24-49,144-147) with
// its scratch in a fixed array compiled into the library.
//
// The scratch is a file-scope __device__ array of
// BCS_GRID_SORT_STATIC_MAX pairs plus the radix histograms (about 2.1 MiB);
// every device that loads the library holds it until the process exits.  All
// calls share it, and it keeps the last call's contents, so calls that
// overlap on the GPU (different streams or threads without ordering) race.
// Every scratch word a call reads is written earlier in the same call, so
// nothing has to be cleared between calls.  A call's error word (positions
// outside the grid box, whose keys are clamped to the edge cells as in
// bcs_get_grid) stays in the array until the next call clears it;
// bcs_grid_sort_static_error_word reads it back.
#include <cuda_runtime.h>

#include <mutex>

#include "bcs_internal.cuh"

namespace bcs {
int radix_sort_pairs(const int* in_k, const int* in_v, int* a_k, int* a_v, int* b_k, int* b_v, int n, int bits,
                     unsigned* temp, cudaStream_t s);
}

namespace {

constexpr int kStaticMax = BCS_GRID_SORT_STATIC_MAX;
constexpr int kStaticTiles = (kStaticMax + 4095) / 4096;
constexpr size_t kStaticWords = 2 * (size_t)kStaticMax + 256 * (size_t)kStaticTiles + 256 + 1;

// Layout: [keys kStaticMax][ids kStaticMax][histograms 256*tiles][totals 256][error word]
static __device__ __align__(256) unsigned g_grid_sort_scratch[kStaticWords];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
unsigned* g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array for the current device, resolved once
// per device with that device current.
bcs_status scratch_for_current_device(unsigned** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return BCS_ERR_NO_DEVICE;
    if (dev < 0 || dev >= kMaxDevices) return BCS_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_grid_sort_scratch) != cudaSuccess) return BCS_ERR_CUDA;
        g_scratch_ptr[dev] = static_cast<unsigned*>(p);
    }
    *out = g_scratch_ptr[dev];
    return BCS_OK;
}

__global__ void k_keys_soa(const float* __restrict__ x, const float* __restrict__ y, const float* __restrict__ z,
                           int n, bcs::GridGeom g, int* keys, int* ids, unsigned* err) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    unsigned e = 0;
    keys[i] = bcs::grid_key(g, bcs::f3(x[i], y[i], z[i]), e);
    ids[i] = i;
    if (e) atomicOr(err, e);
}

}  // namespace

extern "C" bcs_status bcs_grid_sort_static(const float* x, const float* y, const float* z, int n,
                                           const float* bounds6, const float* cell3, int* cell_ids,
                                           int* object_ids, void* stream) {
    if (n < 0 || !bounds6 || !cell3 || (n > 0 && (!x || !y || !z || !cell_ids || !object_ids)))
        return BCS_ERR_INVALID_ARGUMENT;
    if (n > kStaticMax) return BCS_ERR_INVALID_ARGUMENT;
    if (!(cell3[0] > 0 && cell3[1] > 0 && cell3[2] > 0)) return BCS_ERR_INVALID_ARGUMENT;
    unsigned* scratch = nullptr;
    bcs_status st = scratch_for_current_device(&scratch);
    if (st != BCS_OK) return st;
    unsigned* err = scratch + 2 * (size_t)kStaticMax + 256 * (size_t)kStaticTiles + 256;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (cudaMemsetAsync(err, 0, sizeof(unsigned), s) != cudaSuccess) return BCS_ERR_CUDA;
    if (n == 0) return BCS_OK;

    // Grid geometry exactly as bcs_create derives it (FP32, uniform_grid.cu:83-104).
    bcs::GridGeom g{};
    g.lo[0] = bounds6[0]; g.hi[0] = bounds6[1];
    g.lo[1] = bounds6[2]; g.hi[1] = bounds6[3];
    g.lo[2] = bounds6[4]; g.hi[2] = bounds6[5];
    for (int k = 0; k < 3; ++k) {
        g.ext[k] = g.hi[k] - g.lo[k];
        g.cell[k] = cell3[k];
    }
    g.cx = (int)(g.ext[0] / g.cell[0]);
    g.cy = (int)(g.ext[1] / g.cell[1]);
    g.cz = (int)(g.ext[2] / g.cell[2]);
    g.cells = (long long)g.cx * g.cy * g.cz;
    if (g.cx < 1 || g.cy < 1 || g.cz < 1 || g.cells > INT32_MAX) return BCS_ERR_INVALID_ARGUMENT;
    int bits = 0;
    while (bits < 31 && (1LL << bits) < g.cells) ++bits;

    int* sk = reinterpret_cast<int*>(scratch);
    int* sv = sk + kStaticMax;
    unsigned* temp = scratch + 2 * (size_t)kStaticMax;
    // Keys land in the caller's outputs, which then serve as one ping-pong
    // buffer of the sort; the scratch pair is the other.
    k_keys_soa<<<(n + 255) / 256, 256, 0, s>>>(x, y, z, n, g, cell_ids, object_ids, err);
    if (bits > 0 && n > 1) {
        int which = bcs::radix_sort_pairs(cell_ids, object_ids, sk, sv, cell_ids, object_ids, n, bits, temp, s);
        if (which == 0) {
            if (cudaMemcpyAsync(cell_ids, sk, sizeof(int) * (size_t)n, cudaMemcpyDeviceToDevice, s) != cudaSuccess ||
                cudaMemcpyAsync(object_ids, sv, sizeof(int) * (size_t)n, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
                return BCS_ERR_CUDA;
        }
    }
    return cudaGetLastError() == cudaSuccess ? BCS_OK : BCS_ERR_CUDA;
}

extern "C" bcs_status bcs_grid_sort_static_error_word(void* stream, uint32_t* out) {
    if (!out) return BCS_ERR_INVALID_ARGUMENT;
    unsigned* scratch = nullptr;
    bcs_status st = scratch_for_current_device(&scratch);
    if (st != BCS_OK) return st;
    const unsigned* err = scratch + 2 * (size_t)kStaticMax + 256 * (size_t)kStaticTiles + 256;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    unsigned w = 0;
    if (cudaMemcpyAsync(&w, err, sizeof(unsigned), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return BCS_ERR_CUDA;
    *out = w;
    return BCS_OK;
}
