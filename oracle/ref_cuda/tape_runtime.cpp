// tape_runtime.cpp — recording stand-ins for the CUDA runtime calls the
// reference's host code makes (test infrastructure, see tape_shim.h).
//
// Device memory is a range of fake addresses starting at kBase: allocations
// are 256-byte aligned with a 256-byte gap between them, never dereferenced
// on the host.  Every call appends one op to the tape; bcs_tape_write saves
// it.  A copy from device to host cannot be recorded (its data would not
// exist yet), so it aborts the recording.
//
// Tape format (little-endian): "BCSTAPE1", then ops, each
//   u32 opcode, u64 payload bytes, payload
// with the payloads listed at the Op enum.  An address inside an argument or
// an op is always written as (u32 allocation id, u64 offset).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace {

constexpr uint64_t kBase = 0x5EC0000000000000ull;
constexpr uint64_t kAlign = 256;

enum Op : uint32_t {
    kAlloc = 1,        // u32 id, u64 bytes
    kFree = 2,         // u32 id
    kH2D = 3,          // u32 id, u64 off, u64 bytes, data
    kD2D = 4,          // u32 dst id, u64 dst off, u32 src id, u64 src off, u64 bytes
    kMemset = 5,       // u32 id, u64 off, i32 value, u64 bytes
    kStream = 6,       // u32 stream id (1, 2, ...; 0 is the legacy default stream)
    kLaunch = 7,       // u64 kernel address, u32 grid[3], u32 block[3], u32 shmem, u32 stream,
                       // u32 params, per param: u32 size, u32 relocations, bytes,
                       // per relocation: u32 offset in the param, u32 id, u64 off
    kSort = 8,         // u32 keys id, u64 off, u32 values id, u64 off, u32 n
    kSyncDevice = 9,   // -
    kSyncStream = 10,  // u32 stream id
    kMark = 11,        // label bytes
    kBuffer = 12,      // u32 id, u64 off, u64 bytes, name bytes
    kFixLastCell = 13, // u32 keys id, u64 off, u32 starts id, u64 off, u32 ends id, u64 off, u32 n
};

struct Alloc {
    uint32_t id;
    uint64_t addr, bytes;
    bool live;
};

struct Tape {
    std::vector<Alloc> allocs;
    uint64_t next = kBase;
    uint32_t streams = 0;
    std::vector<unsigned char> bytes;
    // launch being assembled
    std::vector<unsigned char> launch;
    int params_left = 0;
};

Tape& tape() {
    static Tape t;
    return t;
}

[[noreturn]] void fail(const char* what) {
    std::fprintf(stderr, "tape recorder: %s\n", what);
    std::exit(3);
}

template <class T>
void put(std::vector<unsigned char>& b, T v) {
    const unsigned char* p = reinterpret_cast<const unsigned char*>(&v);
    b.insert(b.end(), p, p + sizeof(T));
}

void put_bytes(std::vector<unsigned char>& b, const void* p, size_t n) {
    const unsigned char* c = static_cast<const unsigned char*>(p);
    b.insert(b.end(), c, c + n);
}

void emit(uint32_t op, const std::vector<unsigned char>& payload) {
    Tape& t = tape();
    put(t.bytes, op);
    put(t.bytes, (uint64_t)payload.size());
    put_bytes(t.bytes, payload.data(), payload.size());
}

bool in_range(uint64_t a) { return a >= kBase && a < tape().next; }

// (allocation id, offset) of a fake device address; one past the end of an
// allocation still belongs to it.
const Alloc* find(uint64_t a) {
    for (const Alloc& x : tape().allocs)
        if (a >= x.addr && a <= x.addr + x.bytes) return &x;
    return nullptr;
}

void put_addr(std::vector<unsigned char>& b, const void* p) {
    const uint64_t a = reinterpret_cast<uint64_t>(p);
    const Alloc* x = find(a);
    if (!x) fail("address outside every device allocation");
    put(b, x->id);
    put(b, a - x->addr);
}

uint32_t stream_id(cudaStream_t s) {
    if (!s) return 0;
    const uint64_t v = reinterpret_cast<uint64_t>(s);
    if (v == 0 || v > tape().streams) fail("unknown stream");
    return (uint32_t)v;
}

}  // namespace

extern "C" {
uint3 threadIdx;
uint3 blockIdx;
dim3 blockDim;
dim3 gridDim;

cudaError_t cudaMalloc(void** p, size_t n) {
    Tape& t = tape();
    const uint64_t bytes = n ? n : 1;
    Alloc a{(uint32_t)t.allocs.size(), t.next, bytes, true};
    t.allocs.push_back(a);
    t.next += (bytes + kAlign - 1) / kAlign * kAlign + kAlign;
    *p = reinterpret_cast<void*>(a.addr);
    std::vector<unsigned char> b;
    put(b, a.id);
    put(b, a.bytes);
    emit(kAlloc, b);
    return cudaSuccess;
}

cudaError_t cudaFree(void* p) {
    if (!p) return cudaSuccess;
    const Alloc* x = find(reinterpret_cast<uint64_t>(p));
    if (!x || x->addr != reinterpret_cast<uint64_t>(p)) fail("cudaFree of an address that was not allocated");
    std::vector<unsigned char> b;
    put(b, x->id);
    emit(kFree, b);
    return cudaSuccess;
}

cudaError_t cudaMemcpy(void* d, const void* s, size_t n, cudaMemcpyKind kind) {
    const bool dd = in_range(reinterpret_cast<uint64_t>(d)), sd = in_range(reinterpret_cast<uint64_t>(s));
    std::vector<unsigned char> b;
    if (dd && !sd && (kind == cudaMemcpyHostToDevice || kind == cudaMemcpyDefault)) {
        put_addr(b, d);
        put(b, (uint64_t)n);
        put_bytes(b, s, n);
        emit(kH2D, b);
    } else if (dd && sd && (kind == cudaMemcpyDeviceToDevice || kind == cudaMemcpyDefault)) {
        put_addr(b, d);
        put_addr(b, s);
        put(b, (uint64_t)n);
        emit(kD2D, b);
    } else if (!dd && !sd && kind == cudaMemcpyHostToHost) {
        std::memmove(d, s, n);
    } else {
        fail("a copy to the host cannot be recorded");
    }
    return cudaSuccess;
}

cudaError_t cudaMemset(void* d, int v, size_t n) {
    std::vector<unsigned char> b;
    put_addr(b, d);
    put(b, (int32_t)v);
    put(b, (uint64_t)n);
    emit(kMemset, b);
    return cudaSuccess;
}

cudaError_t cudaSetDevice(int) { return cudaSuccess; }
cudaError_t cudaGetDevice(int* d) {
    *d = 0;
    return cudaSuccess;
}
cudaError_t cudaDeviceSynchronize(void) {
    emit(kSyncDevice, {});
    return cudaSuccess;
}
cudaError_t cudaStreamCreate(cudaStream_t* s) {
    Tape& t = tape();
    const uint32_t id = ++t.streams;
    *s = reinterpret_cast<cudaStream_t>((uintptr_t)id);
    std::vector<unsigned char> b;
    put(b, id);
    emit(kStream, b);
    return cudaSuccess;
}
cudaError_t cudaStreamDestroy(cudaStream_t) { return cudaSuccess; }
cudaError_t cudaStreamSynchronize(cudaStream_t s) {
    std::vector<unsigned char> b;
    put(b, stream_id(s));
    emit(kSyncStream, b);
    return cudaSuccess;
}
cudaError_t cudaGetLastError(void) { return cudaSuccess; }
cudaError_t cudaPeekAtLastError(void) { return cudaSuccess; }
const char* cudaGetErrorString(cudaError_t) { return "tape recorder"; }
}

void bcs_tape_begin_launch(const void* fn, dim3 grid, dim3 block, size_t shmem, cudaStream_t stream, int params) {
    Tape& t = tape();
    if (t.params_left) fail("nested launch");
    t.launch.clear();
    put(t.launch, reinterpret_cast<uint64_t>(fn));
    for (unsigned v : {grid.x, grid.y, grid.z, block.x, block.y, block.z}) put(t.launch, (uint32_t)v);
    put(t.launch, (uint32_t)shmem);
    put(t.launch, stream_id(stream));
    put(t.launch, (uint32_t)params);
    t.params_left = params;
    if (!params) emit(kLaunch, t.launch);
}

void bcs_tape_add_param(const void* bytes, size_t size) {
    Tape& t = tape();
    if (t.params_left <= 0) fail("argument without a launch");
    std::vector<unsigned char> rel;
    uint32_t nrel = 0;
    // every 8-byte-aligned word that lies in the fake device range is a
    // device pointer (the range is chosen so that no value can fall there)
    for (size_t o = 0; o + 8 <= size; o += 8) {
        uint64_t w;
        std::memcpy(&w, static_cast<const unsigned char*>(bytes) + o, 8);
        if (!in_range(w)) continue;
        const Alloc* x = find(w);
        if (!x) fail("argument points between device allocations");
        put(rel, (uint32_t)o);
        put(rel, x->id);
        put(rel, w - x->addr);
        ++nrel;
    }
    put(t.launch, (uint32_t)size);
    put(t.launch, nrel);
    put_bytes(t.launch, bytes, size);
    put_bytes(t.launch, rel.data(), rel.size());
    if (--t.params_left == 0) emit(kLaunch, t.launch);
}

void bcs_tape_end_launch() {
    if (tape().params_left) fail("launch with missing arguments");
}

void bcs_tape_sort(int* keys, int n, int* values) {
    std::vector<unsigned char> b;
    put_addr(b, keys);
    put_addr(b, values);
    put(b, (uint32_t)n);
    emit(kSort, b);
}

void bcs_tape_fix_last_cell(const int* keys, int n, int* starts, int* ends) {
    std::vector<unsigned char> b;
    put_addr(b, keys);
    put_addr(b, starts);
    put_addr(b, ends);
    put(b, (uint32_t)n);
    emit(kFixLastCell, b);
}

void bcs_tape_mark(const char* label) {
    std::vector<unsigned char> b;
    put_bytes(b, label, std::strlen(label));
    emit(kMark, b);
}

void bcs_tape_mark_buffer(const char* name, const void* device_ptr, size_t bytes) {
    std::vector<unsigned char> b;
    put_addr(b, device_ptr);
    put(b, (uint64_t)bytes);
    put_bytes(b, name, std::strlen(name));
    emit(kBuffer, b);
}

int bcs_tape_write(const char* path) {
    FILE* f = std::fopen(path, "wb");
    if (!f) return 1;
    const Tape& t = tape();
    std::fwrite("BCSTAPE1", 1, 8, f);
    std::fwrite(t.bytes.data(), 1, t.bytes.size(), f);
    return std::fclose(f) == 0 ? 0 : 1;
}
