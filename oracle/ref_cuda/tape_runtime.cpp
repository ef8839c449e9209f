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
// with the opcodes and payloads listed in tape_format.h.  An address inside
// an argument or an op is always written as (u32 allocation id, u64 offset).
#include <cuda_runtime.h>

#include "tape_format.h"

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

using namespace bcs_tape;

namespace {

constexpr uint64_t kBase = 0x5EC0000000000000ull;
constexpr uint64_t kAlign = 256;


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

void bcs_tape_thunk(const void* fn, void (*thunk)(const void*, unsigned char* const*)) {
    static std::vector<const void*> seen;
    if (std::find(seen.begin(), seen.end(), fn) != seen.end()) return;
    seen.push_back(fn);
    std::vector<unsigned char> b;
    put(b, reinterpret_cast<uint64_t>(fn));
    put(b, reinterpret_cast<uint64_t>(thunk));
    emit(kThunk, b);
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

// ---------------------------------------------------------------------------
// CPU replay of a tape by the executable that recorded it (the kernel and
// thunk addresses on the tape are this executable's): allocations are host
// memory, every launch runs its grid serially through the kernel's thunk,
// the key sort is std::stable_sort.  This checks, without a GPU, that a tape
// holds everything the reference's kernels need, and that its arguments and
// relocations reproduce the reference's own host-driven run.
#include <map>
#include <numeric>

int bcs_tape_replay_cpu(const char* tape_path, const char* state_path, int frames, const char* out_path) {
    try {
        const std::vector<Op> ops = read(tape_path);
        std::vector<const Op*> setup, frame;
        segments(ops, setup, frame);
        std::vector<std::vector<unsigned char>> mem;
        std::map<uint64_t, uint64_t> thunk;
        std::map<std::string, std::pair<float*, uint64_t>> buffers;
        auto at = [&](const Addr& a, uint64_t bytes) -> unsigned char* {
            if (a.id >= mem.size() || a.off + bytes > mem[a.id].size()) throw std::runtime_error("op outside memory");
            return mem[a.id].data() + a.off;
        };
        auto run = [&](const Op& op) {
            switch (op.code) {
                case kAlloc: mem.emplace_back(op.bytes, 0); break;
                case kH2D: std::memcpy(at(op.a, op.bytes), op.data.data(), op.bytes); break;
                case kD2D: std::memmove(at(op.a, op.bytes), at(op.b, op.bytes), op.bytes); break;
                case kMemset: std::memset(at(op.a, op.bytes), op.value, op.bytes); break;
                case kThunk: thunk[op.kernel] = op.thunk; break;
                case kBuffer:
                    buffers[op.text] = {reinterpret_cast<float*>(at(op.a, op.bytes)), op.bytes};
                    break;
                case kSort: {
                    int* k = reinterpret_cast<int*>(at(op.a, 4ull * op.n));
                    int* v = reinterpret_cast<int*>(at(op.b, 4ull * op.n));
                    std::vector<uint32_t> idx(op.n);
                    std::iota(idx.begin(), idx.end(), 0u);
                    std::stable_sort(idx.begin(), idx.end(), [&](uint32_t x, uint32_t y) { return k[x] < k[y]; });
                    std::vector<int> ks(op.n), vs(op.n);
                    for (uint32_t i = 0; i < op.n; ++i) { ks[i] = k[idx[i]]; vs[i] = v[idx[i]]; }
                    std::memcpy(k, ks.data(), 4ull * op.n);
                    std::memcpy(v, vs.data(), 4ull * op.n);
                    break;
                }
                case kFixLastCell: {
                    const int* k = reinterpret_cast<const int*>(at(op.a, 4ull * op.n));
                    if (op.n == 0) break;
                    const int last = k[op.n - 1];
                    int first = (int)op.n - 1;
                    while (first > 0 && k[first - 1] == last) --first;
                    *reinterpret_cast<int*>(at(Addr{op.b.id, op.b.off + 4ull * last}, 4)) = first;
                    *reinterpret_cast<int*>(at(Addr{op.c.id, op.c.off + 4ull * last}, 4)) = (int)op.n - 1;
                    break;
                }
                case kLaunch: {
                    auto t = thunk.find(op.kernel);
                    if (t == thunk.end()) throw std::runtime_error("launch without a thunk");
                    std::vector<std::vector<unsigned char>> args(op.params.size());
                    std::vector<unsigned char*> ptrs(op.params.size());
                    for (size_t i = 0; i < op.params.size(); ++i) {
                        args[i] = op.params[i].bytes;
                        for (const Reloc& r : op.params[i].relocs) {
                            const uint64_t v = reinterpret_cast<uint64_t>(at(Addr{r.id, 0}, r.off) + r.off);
                            std::memcpy(&args[i][r.offset], &v, 8);
                        }
                        ptrs[i] = args[i].data();
                    }
                    auto call = reinterpret_cast<void (*)(const void*, unsigned char* const*)>(t->second);
                    gridDim = dim3(op.grid[0], op.grid[1], op.grid[2]);
                    blockDim = dim3(op.block[0], op.block[1], op.block[2]);
                    for (unsigned bz = 0; bz < op.grid[2]; ++bz)
                        for (unsigned by = 0; by < op.grid[1]; ++by)
                            for (unsigned bx = 0; bx < op.grid[0]; ++bx)
                                for (unsigned tz = 0; tz < op.block[2]; ++tz)
                                    for (unsigned ty = 0; ty < op.block[1]; ++ty)
                                        for (unsigned tx = 0; tx < op.block[0]; ++tx) {
                                            blockIdx = uint3{bx, by, bz};
                                            threadIdx = uint3{tx, ty, tz};
                                            call(reinterpret_cast<const void*>(op.kernel), ptrs.data());
                                        }
                    break;
                }
                default: break;   // frees, streams, synchronisation, marks
            }
        };
        for (const Op& op : ops)
            if (op.code == kThunk) run(op);
        for (const Op* op : setup) run(*op);
        const auto& px = buffers.at("positions.x");
        const size_t n = px.second / 4;
        const char* names[3] = {"positions", "velocities", "forces"};
        if (std::strcmp(state_path, "-") != 0) {
            std::vector<float> s(6 * n);
            FILE* f = std::fopen(state_path, "rb");
            if (!f || std::fread(s.data(), 4, s.size(), f) != s.size()) throw std::runtime_error("bad state file");
            std::fclose(f);
            for (int q = 0; q < 2; ++q)
                for (int c = 0; c < 3; ++c) {
                    float* b = buffers.at(std::string(names[q]) + "." + "xyz"[c]).first;
                    for (size_t i = 0; i < n; ++i) b[i] = s[3 * n * q + 3 * i + c];
                }
        }
        for (int f = 0; f < frames; ++f)
            for (const Op* op : frame) run(*op);
        std::vector<float> out(9 * n);
        for (int q = 0; q < 3; ++q)
            for (int c = 0; c < 3; ++c) {
                const float* b = buffers.at(std::string(names[q]) + "." + "xyz"[c]).first;
                for (size_t i = 0; i < n; ++i) out[3 * n * q + 3 * i + c] = b[i];
            }
        FILE* o = std::fopen(out_path, "wb");
        if (!o || std::fwrite(out.data(), 4, out.size(), o) != out.size()) throw std::runtime_error("cannot write");
        std::fclose(o);
        return 0;
    } catch (const std::exception& e) {
        std::fprintf(stderr, "tape CPU replay: %s\n", e.what());
        return 2;
    }
}
