// tape_shim.h — force-included when the reference's host code is compiled
// with g++ to record its launch tape (test infrastructure: the recipe that
// lets the reference's own CUDA kernels be replayed on a GPU whose machine
// cannot build the reference).
//
// The recipe rewrites every `kernel<<<cfg>>>(args);` of a scratch copy of
// the reference's sources into `bcs_tape_launch(bcs_cfg(cfg), kernel, args);`
// and its one thrust::stable_sort_by_key call into bcs_tape_sort.  Nothing
// runs on the host: each launch is recorded with the kernel's address (named
// afterwards from the recorder's symbol table), its grid, block, dynamic
// shared memory and stream, and the bytes of every argument converted to the
// kernel's own parameter type, exactly as the CUDA runtime's launch stub
// would pass them.  Device allocations are fake addresses in a range no real
// pointer or value uses, so every pointer inside an argument is found and
// recorded as (allocation, offset) for the replay to patch.
#pragma once
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <new>
#include <utility>
using std::isnan;
#include <cuda_runtime.h>

struct bcs_dims {
    dim3 grid, block;
    size_t shmem = 0;
    cudaStream_t stream = nullptr;
};
template <class G, class B>
inline bcs_dims bcs_cfg(G g, B b) {
    return bcs_dims{dim3(g), dim3(b), 0, nullptr};
}
template <class G, class B, class S>
inline bcs_dims bcs_cfg(G g, B b, S shmem) {
    return bcs_dims{dim3(g), dim3(b), (size_t)shmem, nullptr};
}
template <class G, class B, class S>
inline bcs_dims bcs_cfg(G g, B b, S shmem, cudaStream_t s) {
    return bcs_dims{dim3(g), dim3(b), (size_t)shmem, s};
}

// Device-side builtins the reference's kernels name; never read on the host
// (kernels are recorded, not run).
extern "C" {
extern uint3 threadIdx;
extern uint3 blockIdx;
extern dim3 blockDim;
extern dim3 gridDim;
}

// tape_runtime.cpp
void bcs_tape_thunk(const void* fn, void (*thunk)(const void*, unsigned char* const*));
void bcs_tape_begin_launch(const void* fn, dim3 grid, dim3 block, size_t shmem, cudaStream_t stream, int params);
void bcs_tape_add_param(const void* bytes, size_t size);
void bcs_tape_end_launch();
void bcs_tape_sort(int* keys, int n, int* values);
void bcs_tape_fix_last_cell(const int* keys, int n, int* starts, int* ends);
void bcs_tape_mark(const char* label);
void bcs_tape_mark_buffer(const char* name, const void* device_ptr, size_t bytes);
int bcs_tape_write(const char* path);

// One argument, converted to the kernel's parameter type P the way a call
// would convert it (a class is copy-constructed, as the launch stub does).
// The storage is zeroed first so that padding bytes are reproducible.
template <class P, class A>
inline void bcs_tape_param(A&& a) {
    alignas(P) unsigned char storage[sizeof(P)];
    std::memset(storage, 0, sizeof(P));
    P* value = new (storage) P(std::forward<A>(a));
    bcs_tape_add_param(storage, sizeof(P));
    value->~P();
}

// The recorder's own CPU replay calls a kernel (a plain host function in
// the recorder's compile) with the bytes of its arguments through this thunk.
template <class... P, size_t... I>
inline void bcs_tape_invoke(void (*f)(P...), unsigned char* const* a, std::index_sequence<I...>) {
    f(*reinterpret_cast<P*>(a[I])...);
}
template <class... P>
void bcs_tape_call(const void* fn, unsigned char* const* a) {
    bcs_tape_invoke(reinterpret_cast<void (*)(P...)>(const_cast<void*>(fn)), a, std::index_sequence_for<P...>{});
}

template <class... P, class... A>
inline void bcs_tape_launch(bcs_dims d, void (*kernel)(P...), A&&... a) {
    static_assert(sizeof...(P) == sizeof...(A), "kernel argument count");
    bcs_tape_thunk(reinterpret_cast<const void*>(kernel), &bcs_tape_call<P...>);
    bcs_tape_begin_launch(reinterpret_cast<const void*>(kernel), d.grid, d.block, d.shmem, d.stream,
                          (int)sizeof...(P));
    (bcs_tape_param<P>(std::forward<A>(a)), ...);
    bcs_tape_end_launch();
}
