// tape_format.h — reader of the launch tapes tape_runtime.cpp writes (test
// infrastructure), shared by the GPU replay (replay.cu) and the recorder's
// own CPU replay.  A malformed tape throws std::runtime_error.
#pragma once
#include <cstdint>
#include <cstring>
#include <fstream>
#include <iterator>
#include <stdexcept>
#include <string>
#include <vector>

namespace bcs_tape {

// Opcodes and their payloads (an address is u32 allocation id, u64 offset).
enum Code : uint32_t {
    kAlloc = 1,        // u32 id, u64 bytes
    kFree = 2,         // u32 id
    kH2D = 3,          // address, u64 bytes, data
    kD2D = 4,          // destination address, source address, u64 bytes
    kMemset = 5,       // address, i32 value, u64 bytes
    kStream = 6,       // u32 stream id (1, 2, ...; 0 is the legacy default stream)
    kLaunch = 7,       // u64 kernel address, u32 grid[3], u32 block[3], u32 shmem, u32 stream,
                       // u32 params, per param: u32 size, u32 relocations, bytes,
                       // per relocation: u32 offset in the param, u32 id, u64 offset
    kSort = 8,         // keys address, values address, u32 n (stable, by key)
    kSyncDevice = 9,   // -
    kSyncStream = 10,  // u32 stream id
    kMark = 11,        // label bytes ("setup_end", "frame", "frame_end")
    kBuffer = 12,      // address, u64 bytes, name bytes
    kFixLastCell = 13, // keys address, starts address, ends address, u32 n
    kThunk = 14,       // u64 kernel address, u64 address of its call thunk (CPU replay only)
};

struct Addr {
    uint32_t id = 0;
    uint64_t off = 0;
};

struct Reloc {
    uint32_t offset = 0, id = 0;
    uint64_t off = 0;
};

struct Param {
    std::vector<unsigned char> bytes;
    std::vector<Reloc> relocs;
};

struct Op {
    uint32_t code = 0;
    uint32_t id = 0;              // alloc, free
    uint64_t bytes = 0;           // alloc, copies, memset, buffer
    Addr a, b, c;                 // copy / memset / sort / fix-last-cell / buffer operands
    int32_t value = 0;            // memset
    uint32_t n = 0;               // sort, fix-last-cell
    std::vector<unsigned char> data;   // h2d
    std::string text;             // mark, buffer name
    uint64_t kernel = 0, thunk = 0;    // launch, thunk
    uint32_t grid[3] = {}, block[3] = {}, shmem = 0, stream = 0;
    std::vector<Param> params;
};

namespace detail {
struct Cursor {
    const unsigned char* p;
    const unsigned char* end;
    template <class T>
    T take() {
        if (p + sizeof(T) > end) throw std::runtime_error("truncated tape");
        T v;
        std::memcpy(&v, p, sizeof(T));
        p += sizeof(T);
        return v;
    }
    Addr addr() {
        Addr a;
        a.id = take<uint32_t>();
        a.off = take<uint64_t>();
        return a;
    }
    std::vector<unsigned char> raw(size_t n) {
        if (p + n > end) throw std::runtime_error("truncated tape");
        std::vector<unsigned char> v(p, p + n);
        p += n;
        return v;
    }
};
}  // namespace detail

inline std::vector<Op> read(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("cannot open " + path);
    std::vector<unsigned char> d((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    if (d.size() < 8 || std::memcmp(d.data(), "BCSTAPE1", 8) != 0) throw std::runtime_error(path + " is not a tape");
    std::vector<Op> ops;
    size_t o = 8;
    while (o < d.size()) {
        if (o + 12 > d.size()) throw std::runtime_error("truncated tape");
        Op op;
        uint64_t size;
        std::memcpy(&op.code, &d[o], 4);
        std::memcpy(&size, &d[o + 4], 8);
        o += 12;
        if (size > d.size() - o) throw std::runtime_error("truncated tape");
        detail::Cursor c{d.data() + o, d.data() + o + size};
        o += size;
        switch (op.code) {
            case kAlloc: op.id = c.take<uint32_t>(); op.bytes = c.take<uint64_t>(); break;
            case kFree: op.id = c.take<uint32_t>(); break;
            case kH2D: op.a = c.addr(); op.bytes = c.take<uint64_t>(); op.data = c.raw(op.bytes); break;
            case kD2D: op.a = c.addr(); op.b = c.addr(); op.bytes = c.take<uint64_t>(); break;
            case kMemset: op.a = c.addr(); op.value = c.take<int32_t>(); op.bytes = c.take<uint64_t>(); break;
            case kStream: case kSyncStream: op.stream = c.take<uint32_t>(); break;
            case kLaunch: {
                op.kernel = c.take<uint64_t>();
                for (auto& g : op.grid) g = c.take<uint32_t>();
                for (auto& b : op.block) b = c.take<uint32_t>();
                op.shmem = c.take<uint32_t>();
                op.stream = c.take<uint32_t>();
                const uint32_t np = c.take<uint32_t>();
                for (uint32_t i = 0; i < np; ++i) {
                    Param prm;
                    const uint32_t sz = c.take<uint32_t>(), nr = c.take<uint32_t>();
                    prm.bytes = c.raw(sz);
                    for (uint32_t r = 0; r < nr; ++r) {
                        Reloc rl;
                        rl.offset = c.take<uint32_t>();
                        rl.id = c.take<uint32_t>();
                        rl.off = c.take<uint64_t>();
                        prm.relocs.push_back(rl);
                    }
                    op.params.push_back(std::move(prm));
                }
                break;
            }
            case kSort: op.a = c.addr(); op.b = c.addr(); op.n = c.take<uint32_t>(); break;
            case kSyncDevice: break;
            case kMark: { auto v = c.raw(size); op.text.assign(v.begin(), v.end()); break; }
            case kBuffer: {
                op.a = c.addr();
                op.bytes = c.take<uint64_t>();
                auto v = c.raw((size_t)(c.end - c.p));
                op.text.assign(v.begin(), v.end());
                break;
            }
            case kFixLastCell: op.a = c.addr(); op.b = c.addr(); op.c = c.addr(); op.n = c.take<uint32_t>(); break;
            case kThunk: op.kernel = c.take<uint64_t>(); op.thunk = c.take<uint64_t>(); break;
            default: throw std::runtime_error("unknown op in tape");
        }
        if (c.p != c.end) throw std::runtime_error("malformed op in tape");
        ops.push_back(std::move(op));
    }
    return ops;
}

// The ops before "setup_end" and those of the first "frame" .. "frame_end"
// (thunk records, emitted where a kernel first appears, belong to neither).
inline void segments(const std::vector<Op>& ops, std::vector<const Op*>& setup, std::vector<const Op*>& frame) {
    int phase = 0;   // 0 setup, 1 between, 2 first frame, 3 after it
    for (const Op& op : ops) {
        if (op.code == kThunk) continue;
        if (op.code == kMark) {
            if (op.text == "setup_end") phase = 1;
            else if (op.text == "frame" && phase == 1) phase = 2;
            else if (op.text == "frame_end" && phase == 2) phase = 3;
            continue;
        }
        if (phase == 0) setup.push_back(&op);
        else if (phase == 2) frame.push_back(&op);
    }
    if (phase != 3 || frame.empty()) throw std::runtime_error("tape holds no complete frame");
}

}  // namespace bcs_tape
