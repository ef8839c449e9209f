"""FP64 restatement of the learned sub-step network (test infrastructure).

The network is the project's own (it has no reference counterpart): a
message-passing network over one blood cell's spring graph.  Only the tests
use this file, as the checker of the CUDA forward and backward kernels:

    h0 = silu(f W_in + b_in)                     f: node features [n, 16]
    per layer l (3 layers, hidden 128):
        B   = silu(h W_b + b_b)                  node messages
        M_i = mean over the springs of i of B_j + ebar_i W_e + b_e
        h   = h + silu(h W_u + M W_v + b_u)
    y = h W_out + b_out                          y: [n, 9]
    loss = mean((y - t)^2)

ebar_i is the mean of node i's edge features e_ij (edge i <- j, 8 each).

`bf16=True` rounds what the GPU rounds: every weight, the activation
operands of the three hidden x hidden products of each layer (h before W_b
and W_u, M before W_v) and of their backward products, and B where the
aggregation reads it, to bfloat16 (round to nearest even); sums stay in
FP64.  The rounding of B passes gradients unchanged.
"""
from __future__ import annotations

import numpy as np

F_IN, E_IN, OUT = 16, 8, 9


def bf16(x):
    """Round to bfloat16 (nearest even), returned as float64."""
    a = np.ascontiguousarray(np.asarray(x, np.float32))
    b = a.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64).reshape(a.shape)


def silu(x):
    return x / (1.0 + np.exp(-x))


def dsilu(x):
    s = 1.0 / (1.0 + np.exp(-x))
    return s * (1.0 + x * (1.0 - s))


def param_names(layers):
    names = ["W_in", "b_in"]
    for l in range(layers):
        names += [f"Wb{l}", f"bb{l}", f"We{l}", f"be{l}", f"Wu{l}", f"Wv{l}", f"bu{l}"]
    return names + ["W_out", "b_out"]


def param_shapes(hidden, layers):
    H = hidden
    shapes = {"W_in": (F_IN, H), "b_in": (H,), "W_out": (H, OUT), "b_out": (OUT,)}
    for l in range(layers):
        shapes.update({f"Wb{l}": (H, H), f"bb{l}": (H,), f"We{l}": (E_IN, H), f"be{l}": (H,),
                       f"Wu{l}": (H, H), f"Wv{l}": (H, H), f"bu{l}": (H,)})
    return shapes


def _edge_mean(e, src, n):
    deg = np.bincount(src, minlength=n).astype(np.float64)
    ebar = np.zeros((n, e.shape[1]))
    np.add.at(ebar, src, np.asarray(e, np.float64))
    inv = 1.0 / np.maximum(deg, 1.0)
    return ebar * inv[:, None], inv


def forward(params, f, e, src, dst, layers, bf=False, keep=False):
    """f [n, F_IN], e [E, E_IN]; edge k runs src[k] <- dst[k] (src = the
    receiving node).  Returns y, or (y, cache) with keep=True."""
    P = {k: (bf16(v) if bf and k[0] == "W" else np.asarray(v, np.float64)) for k, v in params.items()}
    q = bf16 if bf else (lambda x: np.asarray(x, np.float64))
    n = f.shape[0]
    ebar, inv = _edge_mean(e, src, n)
    z0 = np.asarray(f, np.float64) @ P["W_in"] + P["b_in"]
    h = silu(z0)
    cache = {"z0": z0, "deg_inv": inv, "ebar": ebar, "P": P, "layers": []}
    for l in range(layers):
        hq = q(h)
        zb = hq @ P[f"Wb{l}"] + P[f"bb{l}"]
        B = q(silu(zb))
        M = np.zeros_like(B)
        np.add.at(M, src, B[dst])
        M = M * inv[:, None] + ebar @ P[f"We{l}"] + P[f"be{l}"]
        zu = hq @ P[f"Wu{l}"] + q(M) @ P[f"Wv{l}"] + P[f"bu{l}"]
        cache["layers"].append({"h": h, "zb": zb, "M": M, "zu": zu})
        h = h + silu(zu)
    y = h @ P["W_out"] + P["b_out"]
    cache["h_last"] = h
    return (y, cache) if keep else y


def loss_and_grads(params, f, e, src, dst, t, layers, bf=False):
    y, c = forward(params, f, e, src, dst, layers, bf=bf, keep=True)
    P = c["P"]
    q = bf16 if bf else (lambda x: np.asarray(x, np.float64))
    d = y - np.asarray(t, np.float64)
    loss = float(np.mean(d * d))
    g = {}
    dy = 2.0 * d / d.size
    g["W_out"] = c["h_last"].T @ dy
    g["b_out"] = dy.sum(0)
    dh = dy @ P["W_out"].T
    inv = c["deg_inv"]
    for l in reversed(range(layers)):
        L = c["layers"][l]
        h, zb, M, zu = L["h"], L["zb"], L["M"], L["zu"]
        hq, Mq = q(h), q(M)
        dzu = dh * dsilu(zu)
        dzq = q(dzu)
        g[f"Wu{l}"] = hq.T @ dzq
        g[f"Wv{l}"] = Mq.T @ dzq
        g[f"bu{l}"] = dzu.sum(0)
        dM = dzq @ P[f"Wv{l}"].T
        dh = dh + dzq @ P[f"Wu{l}"].T
        g[f"We{l}"] = c["ebar"].T @ dM
        g[f"be{l}"] = dM.sum(0)
        dB = np.zeros_like(dM)
        np.add.at(dB, dst, (dM * inv[:, None])[src])
        dzb = dB * dsilu(zb)
        dzbq = q(dzb)
        g[f"Wb{l}"] = hq.T @ dzbq
        g[f"bb{l}"] = dzb.sum(0)
        dh = dh + dzbq @ P[f"Wb{l}"].T
    dz0 = dh * dsilu(c["z0"])
    g["W_in"] = np.asarray(f, np.float64).T @ dz0
    g["b_in"] = dz0.sum(0)
    return loss, g


def init_params(hidden, layers, seed=0):
    """Uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) weights, zero biases."""
    rng = np.random.default_rng(seed)
    out = {}
    for k, shp in param_shapes(hidden, layers).items():
        if k[0] == "W":
            lim = 1.0 / np.sqrt(shp[0])
            out[k] = rng.uniform(-lim, lim, shp)
        else:
            out[k] = np.zeros(shp)
    return out


def graph_edges(adj_off, adj_nbr, cells, pic):
    """Directed edges (src <- dst) of `cells` copies of one cell's CSR graph,
    grouped by receiving node in node order."""
    src, dst = [], []
    for c in range(cells):
        for i in range(pic):
            for k in range(adj_off[i], adj_off[i + 1]):
                src.append(c * pic + i)
                dst.append(c * pic + adj_nbr[k])
    return np.asarray(src, np.int64), np.asarray(dst, np.int64)
