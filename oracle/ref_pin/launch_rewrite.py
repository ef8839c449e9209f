"""Rewrite CUDA kernel launches `kernel<<<cfg>>>(args);` of a scratch copy of
the reference's sources so that it compiles with g++:

  form "cpu":  `bcs_launch(bcs_cfg(cfg), [&]() { kernel(args); });` runs the
               kernel on the CPU through the serial launch shim (refcpu_shim.h);
  form "tape": `bcs_tape_launch(bcs_cfg(cfg), kernel, args);` records the
               launch (oracle/ref_cuda/tape_shim.h).

Pin-recipe tooling: it only ever writes into the scratch directory it is
given."""
from __future__ import annotations

import re

_OPEN = re.compile(r"<<\s*<")


def _statement_start(text: str, pos: int) -> int:
    i = pos - 1
    depth = 0
    while i >= 0:
        c = text[i]
        if c in ")]>":
            depth += 1
        elif c in "([<":
            depth -= 1
        if depth <= 0 and c in ";{}":
            return i + 1
        if depth < 0:
            return i + 1
        i -= 1
    return 0


def rewrite(text: str, form: str = "cpu") -> tuple[str, int]:
    out = []
    last = 0
    count = 0
    for m in list(_OPEN.finditer(text)):
        if m.start() < last:
            continue
        start = _statement_start(text, m.start())
        # skip leading whitespace/newlines of the statement
        while start < m.start() and text[start].isspace():
            start += 1
        kernel = text[start:m.start()].strip()
        close = re.compile(r">>\s*>").search(text, m.end())
        cfg = text[m.end():close.start()]
        # argument list with matching parentheses
        p = text.index("(", close.end())
        depth = 0
        q = p
        while True:
            if text[q] == "(":
                depth += 1
            elif text[q] == ")":
                depth -= 1
                if depth == 0:
                    break
            q += 1
        args = text[p + 1:q]
        semi = text.index(";", q)
        out.append(text[last:start])
        if form == "tape":
            rest = f", {args}" if args.strip() else ""
            out.append(f"bcs_tape_launch(bcs_cfg({cfg}), {kernel}{rest});")
        else:
            out.append(f"bcs_launch(bcs_cfg({cfg}), [&]() {{ {kernel}({args}); }});")
        last = semi + 1
        count += 1
    out.append(text[last:])
    return "".join(out), count
