// replay.cu — runs the reference's own CUDA kernels from a cubin and a launch
// tape (test infrastructure: the reference's CUDA build as a baseline where
// the reference itself cannot be compiled; see build_ref_cuda.py).
//
// Usage: ref_cuda_replay <dir> <reference|pinned> <state.bin|-> <frames> [<out.bin>]
//   dir        oracle/_ref/refcuda_<scene>: kernels.cubin, kernels.txt, <mode>.tape
//   state.bin  [N][3] positions then [N][3] velocities (float32), written into
//              the buffers the tape marks (forces start at zero); "-" keeps
//              the zeroed state
//   frames     frames replayed after the construction, each the tape's first
//              recorded frame (the recorder checks that its frames are equal)
//   out.bin    positions, velocities, forces ([N][3] float32 each) afterwards
// Prints one JSON line: frames run, ms per frame (the mean of one CUDA event
// pair per frame on the legacy stream, which also covers the tape's device
// synchronisations; the checks between frames are not timed), each frame's
// ms, launches per frame.
//
// Every launch is checked before it is issued: the cubin entry exists, its
// parameter count and sizes (cuFuncGetParamInfo) equal the recorded ones,
// every relocated pointer lies inside its allocation, and the block shape is
// legal.  A mismatch stops the replay before any kernel of it runs.
//
// The reference's grid key clamps with the box extent instead of the cell
// count (uniform_grid.cu:31-34), so a particle outside the grid box would
// make its kernels write past the cell tables.  Only the grid build at the
// start of a frame turns positions into table indices (the triangle grid's
// centres never move, Q8), so a frame is safe when every particle is inside
// the box as it starts.  Before every frame a check of our own (limits.txt:
// the box) confirms that every position is finite and inside the box shrunk
// by a guard band of a tenth of its smallest extent; otherwise the replay
// stops and reports the frames it ran.  The bound needs no assumption on
// speeds or forces.
#include <cuda.h>
#include <cuda_runtime.h>
#include <thrust/execution_policy.h>
#include <thrust/sort.h>

#include "tape_format.h"

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

namespace {

[[noreturn]] void die(const std::string& what) {
    std::fprintf(stderr, "ref_cuda_replay: %s\n", what.c_str());
    std::exit(2);
}

void check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) die(std::string(what) + ": " + cudaGetErrorString(e));
}

void check(CUresult r, const char* what) {
    if (r != CUDA_SUCCESS) {
        const char* s = nullptr;
        cuGetErrorString(r, &s);
        die(std::string(what) + ": " + (s ? s : "driver error"));
    }
}

using namespace bcs_tape;

// The last occupied cell's range (the reference never writes its end,
// uniform_grid.cu:78); the CPU pin sets it on the host after each build.
__global__ void k_fix_last_cell(const int* keys, int n, int* starts, int* ends, long long cells) {
    if (blockIdx.x != 0 || threadIdx.x != 0 || n <= 0) return;
    const int last = keys[n - 1];
    if (last < 0 || last >= cells) return;
    int first = n - 1;
    while (first > 0 && keys[first - 1] == last) --first;
    starts[last] = first;
    ends[last] = n - 1;
}

// Particles outside the guarded box, and the largest speed (as float bits;
// speeds are non-negative, so their bit patterns order like the values).
__global__ void k_guard(const float* x, const float* y, const float* z, const float* vx, const float* vy,
                        const float* vz, int n, float3 lo, float3 hi, unsigned* out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const bool inside = x[i] >= lo.x && x[i] <= hi.x && y[i] >= lo.y && y[i] <= hi.y && z[i] >= lo.z &&
                            z[i] <= hi.z;
        if (!inside) atomicAdd(&out[0], 1u);
        const float s = sqrtf(vx[i] * vx[i] + vy[i] * vy[i] + vz[i] * vz[i]);
        atomicMax(&out[1], s == s ? __float_as_uint(s) : 0x7F800000u);
    }
}

struct Replay {
    CUmodule module = nullptr;
    std::map<uint64_t, std::string> entry_of;
    std::map<uint64_t, CUfunction> fn;
    std::vector<void*> base;
    std::vector<uint64_t> size;
    std::vector<cudaStream_t> streams{nullptr};
    std::map<std::string, std::pair<void*, uint64_t>> buffers;
    long launches = 0;

    char* at(const Addr& a, uint64_t bytes) {
        if (a.id >= base.size() || !base[a.id]) die("tape names an allocation that does not exist");
        if (a.off + bytes > size[a.id]) die("tape op reaches past its allocation");
        return static_cast<char*>(base[a.id]) + a.off;
    }

    CUfunction function(uint64_t kernel) {
        auto it = fn.find(kernel);
        if (it != fn.end()) return it->second;
        auto e = entry_of.find(kernel);
        if (e == entry_of.end()) die("kernel without a cubin entry");
        CUfunction f;
        check(cuModuleGetFunction(&f, module, e->second.c_str()), e->second.c_str());
        fn[kernel] = f;
        return f;
    }

    // Every check a launch must pass, made for all launches of the tape
    // before any op runs.  `planned` holds each allocation's size and
    // `streams_made` the streams created before this launch.
    void validate(const Op& op, const std::vector<uint64_t>& planned, uint32_t streams_made) {
        CUfunction f = function(op.kernel);
        for (size_t i = 0; i < op.params.size(); ++i) {
            size_t off = 0, sz = 0;
            check(cuFuncGetParamInfo(f, i, &off, &sz), "cuFuncGetParamInfo");
            if (sz != op.params[i].bytes.size()) die("recorded argument size differs from the kernel's parameter");
            for (const Reloc& r : op.params[i].relocs) {
                if ((uint64_t)r.offset + 8 > op.params[i].bytes.size()) die("relocation outside its argument");
                if (r.id >= planned.size() || r.off > planned[r.id]) die("relocated pointer outside its allocation");
            }
        }
        size_t off = 0, sz = 0;
        if (cuFuncGetParamInfo(f, op.params.size(), &off, &sz) == CUDA_SUCCESS) die("kernel takes more parameters");
        const uint64_t threads = (uint64_t)op.block[0] * op.block[1] * op.block[2];
        if (threads == 0 || threads > 1024 || !op.grid[0] || !op.grid[1] || !op.grid[2]) die("illegal launch shape");
        if (op.shmem != 0) die("dynamic shared memory on a recorded launch");
        if (op.stream > streams_made) die("launch on a stream that was not created");
    }

    void launch(const Op& op) {
        std::vector<std::vector<unsigned char>> bufs(op.params.size());
        std::vector<void*> args(op.params.size());
        for (size_t i = 0; i < op.params.size(); ++i) {
            bufs[i] = op.params[i].bytes;
            for (const Reloc& r : op.params[i].relocs) {
                const uint64_t v = reinterpret_cast<uint64_t>(base[r.id]) + r.off;
                std::memcpy(&bufs[i][r.offset], &v, 8);
            }
            args[i] = bufs[i].data();
        }
        check(cuLaunchKernel(function(op.kernel), op.grid[0], op.grid[1], op.grid[2], op.block[0], op.block[1],
                             op.block[2], op.shmem, reinterpret_cast<CUstream>(streams[op.stream]), args.data(),
                             nullptr),
              "cuLaunchKernel");
        ++launches;
    }

    void run(const Op& op) {
        switch (op.code) {
            case kAlloc: {
                if (op.id != base.size()) die("allocations out of order");
                void* p = nullptr;
                check(cudaMalloc(&p, op.bytes), "cudaMalloc");
                check(cudaMemset(p, 0, op.bytes), "cudaMemset");   // fresh pages read as zero
                base.push_back(p);
                size.push_back(op.bytes);
                break;
            }
            case kFree: break;   // freed at exit
            case kH2D: check(cudaMemcpy(at(op.a, op.bytes), op.data.data(), op.bytes, cudaMemcpyHostToDevice), "h2d"); break;
            case kD2D: check(cudaMemcpy(at(op.a, op.bytes), at(op.b, op.bytes), op.bytes, cudaMemcpyDeviceToDevice), "d2d"); break;
            case kMemset: check(cudaMemset(at(op.a, op.bytes), op.value, op.bytes), "memset"); break;
            case kStream: {
                if (op.stream != streams.size()) die("streams out of order");
                cudaStream_t s;
                check(cudaStreamCreate(&s), "cudaStreamCreate");   // as the reference creates them
                streams.push_back(s);
                break;
            }
            case kLaunch: launch(op); break;
            case kSort: {
                int* k = reinterpret_cast<int*>(at(op.a, sizeof(int) * (uint64_t)op.n));
                int* v = reinterpret_cast<int*>(at(op.b, sizeof(int) * (uint64_t)op.n));
                thrust::stable_sort_by_key(thrust::device, k, k + op.n, v);   // uniform_grid.cu:144-147
                break;
            }
            case kSyncDevice: check(cudaDeviceSynchronize(), "cudaDeviceSynchronize"); break;
            case kSyncStream: check(cudaStreamSynchronize(streams.at(op.stream)), "cudaStreamSynchronize"); break;
            case kMark: break;
            case kBuffer: buffers[op.text] = {at(op.a, op.bytes), op.bytes}; break;
            case kThunk: break;   // host-side call thunks of the recorder's own CPU replay
            case kFixLastCell: {
                const int* k = reinterpret_cast<const int*>(at(op.a, sizeof(int) * (uint64_t)op.n));
                int* s = reinterpret_cast<int*>(at(op.b, 0));
                int* e = reinterpret_cast<int*>(at(op.c, 0));
                const long long cells = (long long)std::min(size[op.b.id] - op.b.off, size[op.c.id] - op.c.off) / 4;
                k_fix_last_cell<<<1, 1>>>(k, (int)op.n, s, e, cells);
                check(cudaGetLastError(), "k_fix_last_cell");
                break;
            }
        }
    }

    std::pair<float*, uint64_t> buffer(const std::string& name) {
        auto it = buffers.find(name);
        if (it == buffers.end()) die("tape marks no buffer " + name);
        return {static_cast<float*>(it->second.first), it->second.second};
    }
};

}  // namespace

int main(int argc, char** argv) {
    if (argc < 5) {
        std::fprintf(stderr, "usage: ref_cuda_replay <dir> <reference|pinned> <state.bin|-> <frames> [<out.bin>]\n");
        return 1;
    }
    const std::string dir = argv[1], mode = argv[2], state = argv[3];
    const int frames = std::atoi(argv[4]);
    if (mode != "reference" && mode != "pinned") die("mode is reference or pinned");
    Replay R;
    {
        std::ifstream k(dir + "/kernels.txt");
        if (!k) die("cannot open kernels.txt");
        std::string line;
        while (std::getline(k, line)) {
            std::istringstream ss(line);
            std::string addr, entry;
            if (ss >> addr >> entry) R.entry_of[std::stoull(addr, nullptr, 16)] = entry;
        }
    }
    std::vector<Op> ops;
    std::vector<const Op*> setup, frame;
    try {
        ops = read(dir + "/" + mode + ".tape");
        segments(ops, setup, frame);
    } catch (const std::exception& e) {
        die(e.what());
    }

    check(cudaSetDevice(0), "cudaSetDevice");
    check(cudaFree(nullptr), "context");
    check(cuModuleLoad(&R.module, (dir + "/kernels.cubin").c_str()), "cuModuleLoad");

    {
        // every launch of the construction and of the frame, checked against
        // the allocations and streams made before it, before anything runs
        std::vector<uint64_t> planned;
        uint32_t streams_made = 0;
        for (const std::vector<const Op*>* seg : {&setup, &frame})
            for (const Op* op : *seg) {
                if (op->code == kAlloc) {
                    if (op->id != planned.size()) die("allocations out of order");
                    planned.push_back(op->bytes);
                } else if (op->code == kStream) {
                    streams_made = std::max(streams_made, op->stream);
                } else if (op->code == kLaunch) {
                    R.validate(*op, planned, streams_made);
                }
            }
    }
    for (const Op* op : setup) R.run(*op);
    check(cudaDeviceSynchronize(), "construction");

    auto [px, n4] = R.buffer("positions.x");
    const size_t n = n4 / sizeof(float);
    if (state != "-") {
        std::ifstream f(state, std::ios::binary);
        std::vector<float> s(6 * n);
        if (!f.read(reinterpret_cast<char*>(s.data()), sizeof(float) * s.size())) die("state file too short");
        const char* names[2] = {"positions", "velocities"};
        for (int q = 0; q < 2; ++q)
            for (int c = 0; c < 3; ++c) {
                std::vector<float> comp(n);
                for (size_t i = 0; i < n; ++i) comp[i] = s[3 * n * q + 3 * i + c];
                auto b = R.buffer(std::string(names[q]) + "." + "xyz"[c]);
                if (b.second != sizeof(float) * n) die("buffer sizes differ");
                check(cudaMemcpy(b.first, comp.data(), b.second, cudaMemcpyHostToDevice), "state");
            }
    }
    check(cudaDeviceSynchronize(), "state");

    // the box and time step, and the guard band
    float box[6], dt = 0.f;
    {
        std::ifstream l(dir + "/limits.txt");
        if (!(l >> box[0] >> box[1] >> box[2] >> box[3] >> box[4] >> box[5] >> dt) || !(dt > 0.f))
            die("cannot read limits.txt");
    }
    const float guard = 0.1f * std::min({box[1] - box[0], box[3] - box[2], box[5] - box[4]});
    const float3 glo = make_float3(box[0] + guard, box[2] + guard, box[4] + guard);
    const float3 ghi = make_float3(box[1] - guard, box[3] - guard, box[5] - guard);
    unsigned* gword = nullptr;
    check(cudaMalloc(&gword, 2 * sizeof(unsigned)), "cudaMalloc");
    // true when every particle is finite and inside the guarded box
    auto inside = [&]() {
        check(cudaMemset(gword, 0, 2 * sizeof(unsigned)), "cudaMemset");
        auto b = [&](const char* nm) { return R.buffer(nm).first; };
        k_guard<<<std::max<size_t>(1, std::min<size_t>(4096, (n + 255) / 256)), 256>>>(
            b("positions.x"), b("positions.y"), b("positions.z"), b("velocities.x"), b("velocities.y"),
            b("velocities.z"), (int)n, glo, ghi, gword);
        unsigned h[2];
        check(cudaMemcpy(h, gword, sizeof(h), cudaMemcpyDeviceToHost), "guard");
        float vmax;
        std::memcpy(&vmax, &h[1], 4);
        return h[0] == 0 && vmax < 3.0e38f;
    };

    const long before = R.launches;
    cudaEvent_t e0, e1;
    check(cudaEventCreate(&e0), "event");
    check(cudaEventCreate(&e1), "event");
    double total_ms = 0.0;
    std::vector<float> per_frame;
    int done = 0;
    while (done < frames && inside()) {
        check(cudaEventRecord(e0, nullptr), "event");
        for (const Op* op : frame) R.run(*op);
        check(cudaEventRecord(e1, nullptr), "event");
        check(cudaEventSynchronize(e1), "frame");
        float ms = 0.f;
        check(cudaEventElapsedTime(&ms, e0, e1), "event");
        check(cudaGetLastError(), "frame");
        total_ms += ms;
        per_frame.push_back(ms);
        ++done;
    }

    if (argc > 5) {
        std::vector<float> out(9 * n);
        const char* names[3] = {"positions", "velocities", "forces"};
        for (int q = 0; q < 3; ++q)
            for (int c = 0; c < 3; ++c) {
                std::vector<float> comp(n);
                auto b = R.buffer(std::string(names[q]) + "." + "xyz"[c]);
                check(cudaMemcpy(comp.data(), b.first, b.second, cudaMemcpyDeviceToHost), "read back");
                for (size_t i = 0; i < n; ++i) out[3 * n * q + 3 * i + c] = comp[i];
            }
        std::ofstream o(argv[5], std::ios::binary);
        o.write(reinterpret_cast<const char*>(out.data()), sizeof(float) * out.size());
    }
    std::string list;
    for (size_t i = 0; i < per_frame.size(); ++i) {
        char b[32];
        std::snprintf(b, sizeof(b), "%s%.6f", i ? ", " : "", per_frame[i]);
        list += b;
    }
    std::printf("{\"frames\": %d, \"frames_requested\": %d, \"ms_per_frame\": %.6f, \"particles\": %zu, "
                "\"launches_per_frame\": %ld, \"ms_frames\": [%s]}\n",
                done, frames, done ? total_ms / done : 0.0, n, done ? (R.launches - before) / done : 0L,
                list.c_str());
    return 0;
}
