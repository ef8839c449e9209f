"""The FP64 network restatement (CPU): its gradients against finite
differences and its bfloat16 rounding against torch's."""
import numpy as np
import torch

import bcs_scenes as S
import mpnn_oracle as M


def graph(cells=2):
    m = S.sphere_cell(3.0, 1)
    pic = len(m.vertices)
    nb = [set() for _ in range(pic)]
    for a, b in m.springs:
        nb[a].add(b)
        nb[b].add(a)
    off = np.cumsum([0] + [len(x) for x in nb])
    nbr = np.concatenate([sorted(x) for x in nb])
    return M.graph_edges(off, nbr, cells, pic), pic


def test_gradients_follow_finite_differences():
    (src, dst), pic = graph()
    rng = np.random.default_rng(0)
    P = M.init_params(16, 2, 1)
    for k in P:
        if k[0] == "b":
            P[k] = rng.normal(0, 0.1, P[k].shape)
    f = rng.normal(size=(2 * pic, M.F_IN))
    e = rng.normal(size=(len(src), M.E_IN))
    t = rng.normal(size=(2 * pic, M.OUT))
    _, g = M.loss_and_grads(P, f, e, src, dst, t, 2)
    for k in P:
        for _ in range(2):
            idx = tuple(rng.integers(0, s) for s in P[k].shape)
            Pp = {q: v.copy() for q, v in P.items()}
            Pm = {q: v.copy() for q, v in P.items()}
            Pp[k][idx] += 1e-6
            Pm[k][idx] -= 1e-6
            fd = (M.loss_and_grads(Pp, f, e, src, dst, t, 2)[0] - M.loss_and_grads(Pm, f, e, src, dst, t, 2)[0]) / 2e-6
            assert abs(fd - g[k][idx]) <= 1e-5 * (abs(fd) + 1e-3), k


def test_bf16_rounding_matches_torch():
    x = np.random.default_rng(3).normal(0, 1e3, 100000).astype(np.float32)
    x[:10] = [0.0, -0.0, 1.0, 1.00390625, 1.005859375, 65504.0, 3.0e38, -1e-30, 1e-40, 2.5]
    want = torch.from_numpy(x).to(torch.bfloat16).to(torch.float64).numpy()
    np.testing.assert_array_equal(M.bf16(x), want)


def test_bf16_emulation_changes_little():
    (src, dst), pic = graph()
    rng = np.random.default_rng(5)
    P = M.init_params(128, 3, 2)
    f = rng.normal(size=(2 * pic, M.F_IN))
    e = rng.normal(size=(len(src), M.E_IN))
    y = M.forward(P, f, e, src, dst, 3)
    yb = M.forward(P, f, e, src, dst, 3, bf=True)
    assert np.abs(y - yb).max() < 5e-2 * np.abs(y).max()
