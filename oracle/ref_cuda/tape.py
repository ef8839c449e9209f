"""Reader of the launch tapes tape_runtime.cpp writes (test infrastructure).

read(path) returns the ops in order as dicts; an address is always an
(allocation id, offset) pair.  The opcodes and payloads are listed in
tape_format.h.
"""
from __future__ import annotations

import struct

OPS = {1: "alloc", 2: "free", 3: "h2d", 4: "d2d", 5: "memset", 6: "stream", 7: "launch", 8: "sort",
       9: "sync_device", 10: "sync_stream", 11: "mark", 12: "buffer", 13: "fix_last_cell", 14: "thunk"}


class _Reader:
    def __init__(self, b: bytes):
        self.b, self.o = b, 0

    def take(self, fmt: str):
        v = struct.unpack_from("<" + fmt, self.b, self.o)
        self.o += struct.calcsize("<" + fmt)
        return v if len(v) > 1 else v[0]

    def raw(self, n: int) -> bytes:
        v = self.b[self.o:self.o + n]
        self.o += n
        return v

    def addr(self):
        return self.take("IQ")


def read(path: str) -> list:
    data = open(path, "rb").read()
    if data[:8] != b"BCSTAPE1":
        raise ValueError(f"{path}: not a launch tape")
    ops, o = [], 8
    while o < len(data):
        code, size = struct.unpack_from("<IQ", data, o)
        o += 12
        r = _Reader(data[o:o + size])
        o += size
        name = OPS.get(code)
        if name is None:
            raise ValueError(f"{path}: unknown op {code}")
        op = {"op": name}
        if name == "alloc":
            op["id"], op["bytes"] = r.take("IQ")
        elif name == "free":
            op["id"] = r.take("I")
        elif name == "h2d":
            op["dst"] = r.addr()
            n = r.take("Q")
            op["data"] = r.raw(n)
        elif name == "d2d":
            op["dst"], op["src"] = r.addr(), r.addr()
            op["bytes"] = r.take("Q")
        elif name == "memset":
            op["dst"] = r.addr()
            op["value"], op["bytes"] = r.take("iQ")
        elif name in ("stream", "sync_stream"):
            op["stream"] = r.take("I")
        elif name == "launch":
            op["kernel"] = r.take("Q")
            op["grid"] = r.take("III")
            op["block"] = r.take("III")
            op["shmem"], op["stream"], n = r.take("III")
            params = []
            for _ in range(n):
                size, nrel = r.take("II")
                raw = r.raw(size)
                rel = [r.take("IIQ") for _ in range(nrel)]
                params.append({"bytes": raw, "relocs": [{"offset": a, "id": b, "off": c} for a, b, c in rel]})
            op["params"] = params
        elif name == "sort":
            op["keys"], op["values"] = r.addr(), r.addr()
            op["n"] = r.take("I")
        elif name == "mark":
            op["label"] = r.raw(len(r.b)).decode()
        elif name == "buffer":
            op["at"] = r.addr()
            op["bytes"] = r.take("Q")
            op["name"] = r.raw(len(r.b) - r.o).decode()
        elif name == "thunk":
            op["kernel"], op["thunk"] = r.take("QQ")
        elif name == "fix_last_cell":
            op["keys"], op["starts"], op["ends"] = r.addr(), r.addr(), r.addr()
            op["n"] = r.take("I")
        if r.o != len(r.b):
            raise ValueError(f"{path}: {name} op has {len(r.b) - r.o} trailing bytes")
        ops.append(op)
    return ops


def segments(ops: list) -> dict:
    """The ops before "setup_end" and between each "frame" / "frame_end"
    pair, without thunk records: {"setup": [...], "frames": [[...], ...]}."""
    setup, frames, cur, in_setup = [], [], None, True
    for op in ops:
        if op["op"] == "thunk":   # emitted where a kernel first appears; part of no segment
            continue
        if op["op"] == "mark":
            if op["label"] == "setup_end":
                in_setup = False
            elif op["label"] == "frame":
                cur = []
            elif op["label"] == "frame_end":
                frames.append(cur)
                cur = None
            continue
        if in_setup:
            setup.append(op)
        elif cur is not None:
            cur.append(op)
    return {"setup": setup, "frames": frames}
