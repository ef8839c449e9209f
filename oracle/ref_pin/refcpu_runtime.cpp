// refcpu_runtime.cpp — host stand-ins for the CUDA runtime calls the
// reference's sources make (pin recipe, test infrastructure): device memory
// is host memory, copies are memcpy, synchronisation is a no-op.
#include <cuda_runtime.h>

#include <cstdlib>
#include <cstring>

extern "C" {
uint3 threadIdx;
uint3 blockIdx;
dim3 blockDim;
dim3 gridDim;

cudaError_t cudaMalloc(void** p, size_t n) {
    *p = std::calloc(n ? n : 1, 1);
    return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
cudaError_t cudaFree(void* p) {
    std::free(p);
    return cudaSuccess;
}
cudaError_t cudaMemcpy(void* d, const void* s, size_t n, cudaMemcpyKind) {
    std::memmove(d, s, n);
    return cudaSuccess;
}
cudaError_t cudaMemset(void* d, int v, size_t n) {
    std::memset(d, v, n);
    return cudaSuccess;
}
cudaError_t cudaSetDevice(int) { return cudaSuccess; }
cudaError_t cudaGetDevice(int* d) {
    *d = 0;
    return cudaSuccess;
}
cudaError_t cudaDeviceSynchronize(void) { return cudaSuccess; }
cudaError_t cudaStreamCreate(cudaStream_t* s) {
    *s = nullptr;
    return cudaSuccess;
}
cudaError_t cudaStreamDestroy(cudaStream_t) { return cudaSuccess; }
cudaError_t cudaStreamSynchronize(cudaStream_t) { return cudaSuccess; }
cudaError_t cudaGetLastError(void) { return cudaSuccess; }
const char* cudaGetErrorString(cudaError_t) { return "host stand-in"; }
}
