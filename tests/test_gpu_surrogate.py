"""The learned sub-step network: its CUDA forward and backward kernels
against the FP64 restatement in oracle/mpnn_oracle.py, training on data the
plain sub-steps generate, what the trained network gains over the
constant-force extrapolation it corrects, and the residual check with its
fallback inside macro steps.

Tolerances: the oracle rounds to bfloat16 exactly where the kernels do, so
GPU and oracle differ by FP32 against FP64 arithmetic plus the rare operand
that lands on the other side of a bfloat16 rounding boundary: 1e-2 of each
gradient tensor's norm, 2e-3 relative on the loss.
"""
import numpy as np
import pytest

import bcs
import bcs_scenes as S
import mpnn_oracle as M

pytestmark = pytest.mark.gpu


def sphere_scene(cells=24, seed=5, **kw):
    sc = S.straight_scene(cells=cells, seed=seed, radius=14.0, length=90.0, around=32, rings=40, **kw)
    sc.velocities[:] = np.random.default_rng(seed).normal(0, 6.0, sc.velocities.shape).astype(np.float32)
    return sc


def make(sc):
    sim = bcs.Simulation(sc)
    sim.set_particles(sc.positions, sc.velocities)
    return sim


def cell_graph(sc, t=0):
    """CSR graph of one cell of type t as the library builds it."""
    typ = sc.types[t]
    pic = len(typ.vertices)
    nb = [dict() for _ in range(pic)]
    for (a, b), L in zip(np.asarray(typ.springs).reshape(-1, 2), typ.spring_lengths):
        nb[a][b] = L
        nb[b][a] = L
    off = np.zeros(pic + 1, np.int64)
    nbr, ln = [], []
    for i in range(pic):
        ks = sorted(k for k in nb[i] if k != i and nb[i][k] != 0.0)
        nbr += ks
        ln += [nb[i][k] for k in ks]
        off[i + 1] = len(nbr)
    return off, np.asarray(nbr, np.int64), np.asarray(ln, np.float32)


def unflatten(flat, layers):
    out, o = {}, 0
    shapes = M.param_shapes(128, layers)
    for k in M.param_names(layers):
        n = int(np.prod(shapes[k]))
        out[k] = np.asarray(flat[o:o + n], np.float64).reshape(shapes[k])
        o += n
    assert o == len(flat)
    return out


def random_case(sur, sc, cells, seed):
    rng = np.random.default_rng(seed)
    off, nbr, _ = cell_graph(sc)
    pic = len(off) - 1
    src, dst = M.graph_edges(off, nbr, cells, pic)
    f = rng.normal(size=(cells * pic, M.F_IN)).astype(np.float32)
    e = rng.normal(size=(len(src), M.E_IN)).astype(np.float32)
    t = rng.normal(size=(cells * pic, M.OUT)).astype(np.float32)
    p = sur.get_params()
    p += rng.normal(0, 0.05, p.shape).astype(np.float32)   # non-zero biases
    sur.set_params(p)
    return f, e, t, src, dst, unflatten(p, 3)


def test_forward_matches_oracle(lib):
    sc = sphere_scene()
    sim = make(sc)
    sur = bcs.Surrogate(sim, max_samples=64)
    f, e, t, src, dst, P = random_case(sur, sc, 3, 1)
    y = sur.forward(3, f, e)
    yo = M.forward(P, f, e, src, dst, 3, bf=True)
    assert np.abs(y - yo).max() <= 2e-3 * (np.abs(yo).max() + 1e-6)


def test_gradients_match_oracle(lib):
    sc = sphere_scene()
    sim = make(sc)
    sur = bcs.Surrogate(sim, max_samples=64)
    f, e, t, src, dst, P = random_case(sur, sc, 2, 2)
    loss, g = sur.loss_grad(2, f, e, t)
    lo, go = M.loss_and_grads(P, f, e, src, dst, t, 3, bf=True)
    assert abs(loss - lo) <= 2e-3 * abs(lo)
    gg = unflatten(g, 3)
    for k in M.param_names(3):
        err = np.linalg.norm(gg[k] - go[k])
        assert err <= 1e-2 * np.linalg.norm(go[k]) + 1e-7, (k, err, np.linalg.norm(go[k]))
    # and the oracle itself follows its finite differences (FP64, no rounding)
    lf, gf = M.loss_and_grads(P, f, e, src, dst, t, 3)
    rng = np.random.default_rng(0)
    for k in ("Wb0", "We2", "bu1", "bb2", "W_in", "b_out"):
        idx = tuple(rng.integers(0, s) for s in P[k].shape)
        Pp = {q: v.copy() for q, v in P.items()}
        Pm = {q: v.copy() for q, v in P.items()}
        Pp[k][idx] += 1e-6
        Pm[k][idx] -= 1e-6
        fd = (M.loss_and_grads(Pp, f, e, src, dst, t, 3)[0] - M.loss_and_grads(Pm, f, e, src, dst, t, 3)[0]) / 2e-6
        assert abs(fd - gf[k][idx]) <= 1e-5 * (abs(fd) + 1e-3)


@pytest.fixture(scope="module")
def trained():
    """Plain macro steps of a moving 42-vertex-cell scene: 30 of them for
    training, 10 more held out."""
    sc = sphere_scene(cells=40, seed=8)
    sim = make(sc)
    sur = bcs.Surrogate(sim, substeps=8, max_samples=40 * 40, seed=3)
    sur.collect(30)
    train_n = sur.stats()["samples"]
    loss0 = sur.train(1, batch_cells=64, lr=1e-3)
    loss = sur.train(400, batch_cells=64, lr=1e-3)
    sur.collect(10)
    return sc, sim, sur, train_n, loss0, loss


def test_collect_and_train(lib, trained):
    sc, sim, sur, train_n, loss0, loss = trained
    st = sur.stats()
    assert train_n == 30 * 40 and st["samples"] == 40 * 40
    assert st["valid_samples"] > 0.9 * st["samples"]
    assert st["iterations"] == 401
    assert loss < 0.5 * loss0
    assert st["parameters"] == sur.param_count() == sum(int(np.prod(s)) for s in M.param_shapes(128, 3).values())
    assert abs(st["flops_per_cell"] - (2 * (42 * 16 * 128 + 3 * (3 * 42 * 128 * 128 + 42 * 8 * 128) + 42 * 128 * 9)
                                       + 3 * 240 * 128)) < 1


def test_trained_network_beats_the_extrapolation(lib, trained):
    sc, sim, sur, train_n, loss0, loss = trained
    net, base = sur.evaluate(train_n, 10 * 40)
    assert net < 0.7 * base, (net, base)


def test_residual_check_and_fallback(lib, trained):
    sc, sim, sur, train_n, loss0, loss = trained
    # a tolerance nothing meets: every cell falls back, so the macro steps
    # are the plain ones bit for bit
    a, b = make(sc), make(sc)
    strict = bcs.Surrogate(b, substeps=8, max_samples=40, seed=3, tolerance=1e-30)
    strict.set_params(sur.get_params())
    strict.set_scales(sur.scales())
    strict.enable(True)
    b.macro_step(8, 2)
    a.macro_step(8, 2)
    st = strict.stats()
    assert st["predicted_cells"] == 0 and st["fallback_cells"] == 2 * 40
    for x, y in zip(a.get_particles(), b.get_particles()):
        np.testing.assert_array_equal(x, y)
    strict.enable(False)


def test_surrogate_in_macro_steps(lib, trained):
    sc, sim, sur, train_n, loss0, loss = trained
    ref, run = make(sc), make(sc)
    s = bcs.Surrogate(run, substeps=8, max_samples=40, seed=3, tolerance=10.0)
    s.set_params(sur.get_params())
    s.set_scales(sur.scales())
    s.enable(True)
    run.macro_step(8, 4)
    ref.macro_step(8, 4)
    st = s.stats()
    assert st["predicted_cells"] + st["fallback_cells"] == 4 * 40
    assert st["predicted_cells"] > 0
    p, v, f = run.get_particles()
    assert np.isfinite(p).all() and np.isfinite(v).all() and np.isfinite(f).all()
    assert run.refresh_info().steps_done == ref.refresh_info().steps_done == 4 * 8
    pr = ref.get_particles()[0]
    assert np.median(np.linalg.norm(p - pr, axis=1)) < 0.05


def test_surrogate_arguments(lib):
    sim = make(sphere_scene(cells=4))
    for bad in (dict(cell_type=5), dict(substeps=1), dict(layers=0), dict(layers=5), dict(max_samples=0),
                dict(tolerance=-1.0)):
        with pytest.raises(bcs.BcsError):
            bcs.Surrogate(sim, **bad)
    sur = bcs.Surrogate(sim, max_samples=4)
    with pytest.raises(bcs.BcsError):
        sur.enable(True)      # not trained: no normalisation yet
    with pytest.raises(bcs.BcsError):
        sur.train(1)          # no samples yet


def test_surrogate_outlives_its_simulation(lib):
    """Destroying the simulation first detaches its surrogates: later calls
    on them are refused, destroying them still works."""
    sim = make(sphere_scene(cells=4))
    sur = bcs.Surrogate(sim, max_samples=16)
    sur.collect(1)
    other = bcs.Surrogate(sim, max_samples=16)
    other.close()                       # one destroyed while the simulation lives
    sim.close()
    with pytest.raises(bcs.BcsError) as e:
        sur.collect(1)
    assert e.value.status == 1
    with pytest.raises(bcs.BcsError):
        sur.stats()
    sur.close()


def test_fused_inference_matches_layer_kernels(lib, trained):
    sc, sim, sur, train_n, loss0, loss = trained
    out = []
    for fused in (True, False):
        run = make(sc)
        s = bcs.Surrogate(run, substeps=8, max_samples=40, seed=3, tolerance=10.0)
        s.set_params(sur.get_params())
        s.set_scales(sur.scales())
        s.enable(True, fused=fused)
        run.macro_step(8, 1)
        out.append((run.get_particles(), s.stats()))
    (a, sa), (b, sb) = out
    assert sa["predicted_cells"] == sb["predicted_cells"] == 40
    for x, y in zip(a, b):
        assert np.abs(x - y).max() <= 1e-4 * (np.abs(y).max() + 1.0)


@pytest.mark.parametrize("path", [0, 1])
def test_gradients_both_tensor_paths(lib, path):
    expired = bcs.tensor_wait_expiries()
    prev = bcs.set_tensor_path(path)
    try:
        sc = sphere_scene()
        sim = make(sc)
        sur = bcs.Surrogate(sim, max_samples=64)
        f, e, t, src, dst, P = random_case(sur, sc, 2, 11)
        loss, g = sur.loss_grad(2, f, e, t)
        lo, go = M.loss_and_grads(P, f, e, src, dst, t, 3, bf=True)
        assert abs(loss - lo) <= 2e-3 * abs(lo)
        gg = unflatten(g, 3)
        for k in M.param_names(3):
            assert np.linalg.norm(gg[k] - go[k]) <= 1e-2 * np.linalg.norm(go[k]) + 1e-7, k
        y = sur.forward(2, f, e)
        assert np.abs(y - M.forward(P, f, e, src, dst, 3, bf=True)).max() <= 2e-3 * (np.abs(y).max() + 1e-6)
    finally:
        bcs.set_tensor_path(prev)
    assert bcs.tensor_wait_expiries() == expired


def test_tensor_paths_agree(lib):
    sc = sphere_scene()
    sim = make(sc)
    sur = bcs.Surrogate(sim, max_samples=64)
    f, e, t, src, dst, P = random_case(sur, sc, 4, 12)
    prev = bcs.set_tensor_path(1)
    y1 = sur.forward(4, f, e)
    bcs.set_tensor_path(0)
    y0 = sur.forward(4, f, e)
    bcs.set_tensor_path(prev)
    assert np.abs(y0 - y1).max() <= 1e-4 * (np.abs(y1).max() + 1e-6)
    assert bcs.set_tensor_path(5) == -1


def test_fused_inference_matches_layer_kernels_disc_cells(lib):
    """The 162-vertex discs take the fused kernel's 11-warp shape (the other
    tests' 42-vertex cells take the 3-warp one): same comparison."""
    sc = S.mixed_straight_scene(4, 10, 60.0, seed=6, base_radius=14.0)
    sc.velocities[:] = np.random.default_rng(6).normal(0, 6.0, sc.velocities.shape).astype(np.float32)
    base = make(sc)
    sur = bcs.Surrogate(base, cell_type=1, substeps=8, max_samples=10 * 4, seed=5)
    sur.collect(3)
    sur.train(20, batch_cells=8, lr=1e-3)
    out = []
    for fused in (True, False):
        run = make(sc)
        s = bcs.Surrogate(run, cell_type=1, substeps=8, max_samples=10, seed=5, tolerance=10.0)
        s.set_params(sur.get_params())
        s.set_scales(sur.scales())
        s.enable(True, fused=fused)
        run.macro_step(8, 1)
        out.append((run.get_particles(), s.stats()))
    (a, sa), (b, sb) = out
    assert sa["predicted_cells"] == sb["predicted_cells"] == 10
    for x, y in zip(a, b):
        assert np.abs(x - y).max() <= 1e-4 * (np.abs(y).max() + 1.0)


def test_bounded_wait_gives_up_and_recovers(lib):
    """The tcgen05 products' bounded completion wait, made to run out: with
    the wait probe on, every CTA's first wait polls a barrier nothing arrives
    at, gives up, counts the expiry and skips its product (it still waits,
    bounded, for the products it issued before freeing tensor memory), and
    the call reports BCS_ERR_TIMEOUT.  With the probe off the next call
    matches the oracle again and counts nothing."""
    prev = bcs.set_tensor_path(0)
    try:
        sc = sphere_scene()
        sim = make(sc)
        sur = bcs.Surrogate(sim, max_samples=64)
        f, e, t, src, dst, P = random_case(sur, sc, 2, 21)
        before = bcs.tensor_wait_expiries()
        bcs.set_tensor_wait_probe(16)
        try:
            with pytest.raises(bcs.BcsError) as err:
                sur.loss_grad(2, f, e, t)
            assert err.value.status == bcs.ERR_TIMEOUT
            with pytest.raises(bcs.BcsError) as err:
                sur.forward(2, f, e)
            assert err.value.status == bcs.ERR_TIMEOUT
        finally:
            bcs.set_tensor_wait_probe(0)
        after = bcs.tensor_wait_expiries()
        assert after > before
        loss, g = sur.loss_grad(2, f, e, t)
        lo, go = M.loss_and_grads(P, f, e, src, dst, t, 3, bf=True)
        assert abs(loss - lo) <= 2e-3 * abs(lo)
        gg = unflatten(g, 3)
        for k in M.param_names(3):
            assert np.linalg.norm(gg[k] - go[k]) <= 1e-2 * np.linalg.norm(go[k]) + 1e-7, k
        assert bcs.tensor_wait_expiries() == after
    finally:
        bcs.set_tensor_path(prev)
