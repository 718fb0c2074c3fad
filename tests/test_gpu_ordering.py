"""Learned ordering of overlap tests on the GPU.

* the tensor-core inference and the training kernels against the FP32 restatement of the
  network (oracle/mlp_ref.py), with the tolerances written below;
* pair logging and training: the logged pairs carry both labels and training lowers the
  loss;
* decisions: a sweep that pre-tests ranked partners (network or centre distance) leaves
  the FP64 state bit-identical to the plain sweep's, and its logged moves replay on the
  CPU oracle with identical outcome codes — the ordering only removes pair tests."""
import numpy as np
import pytest

import pyoracle as po
import systems
from oracle import mlp_ref
from rampack_gb300 import _lib

pytestmark = pytest.mark.gpu

# logits: |y_gpu - y_ref| <= ATOL + RTOL |y_ref| (FP32 accumulation order on the tensor
# cores vs float64, and BF16 re-rounding of hidden units that sit on a rounding tie)
PRED_ATOL, PRED_RTOL = 2e-2, 2e-2
# gradient: relative L2 error of the whole gradient vector
GRAD_REL = 2e-2


def gpu_packing(cfg):
    from rampack_gb300.packing import GpuPacking
    kind, prm, pos, rot, box = cfg
    return GpuPacking(kind, prm, pos, rot, box)


def random_pairs(n, seed, frac=0.3):
    rng = np.random.default_rng(seed)
    d = rng.uniform(-1.0, 1.0, (n, 3)) * 3.0
    ai = rng.normal(size=(n, 3))
    ai /= np.linalg.norm(ai, axis=1, keepdims=True)
    aj = rng.normal(size=(n, 3))
    aj /= np.linalg.norm(aj, axis=1, keepdims=True)
    return mlp_ref.features(d, ai, aj, 1.0 / 3.0), (rng.uniform(size=n) < frac).astype(np.uint8)


@pytest.mark.parametrize("n", [1, 15, 16, 33, 1000])
def test_predict_matches_oracle(engine, n):
    cfg = systems.sc_l2()
    f, _ = random_pairs(n, 10 + n)
    w = mlp_ref.init_params(7)
    with gpu_packing(cfg) as g:
        g.set_mlp_params(w)
        assert np.array_equal(g.mlp_params(), w)
        y = g.mlp_predict(f)
    want, _ = mlp_ref.forward(f, w)
    assert np.all(np.abs(y - want) <= PRED_ATOL + PRED_RTOL * np.abs(want)), np.max(np.abs(y - want))


@pytest.mark.parametrize("n", [1, 31, 32, 777, 20000])
def test_gradient_matches_oracle(engine, n):
    cfg = systems.sc_l2()
    f, lab = random_pairs(n, 20 + n)
    w = mlp_ref.init_params(8)
    with gpu_packing(cfg) as g:
        g.set_mlp_params(w)
        grad, loss = g.mlp_gradient(f, lab)
    want_loss, want = mlp_ref.loss_and_grad(f, lab, w)
    assert abs(loss - want_loss) <= 1e-4 + 1e-4 * abs(want_loss)
    assert np.linalg.norm(grad - want) <= GRAD_REL * np.linalg.norm(want)


def test_init_is_seeded(engine):
    cfg = systems.sc_l2()
    with gpu_packing(cfg) as g:
        g.mlp_init(5)
        a = g.mlp_params()
        g.mlp_init(5)
        b = g.mlp_params()
        g.mlp_init(6)
        c = g.mlp_params()
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    w1 = a[mlp_ref.W1:mlp_ref.B1].reshape(64, 16)
    assert np.all(w1[:, 13:] == 0) and np.all(a[mlp_ref.B1:mlp_ref.W2] == 0)


def collect(g, sweeps, seed=11, every=1):
    g.pair_log_enable(400_000, every)
    for c in range(sweeps):
        g.sweep(0.2, 0.2, seed=seed, counter=c)
    return g.pair_log()


def test_pair_log_and_training(engine):
    cfg = systems.sc_l2_dense()
    with gpu_packing(cfg) as g:
        f, lab = collect(g, 6)
        assert len(f) > 1000
        assert 0 < lab.mean() < 1
        assert np.all(np.isfinite(f)) and np.all(f[:, 13:] == 0)
        # pre-move separations of pairs that reached the segment test lie within about
        # one interaction range (plus the move)
        assert np.all(f[:, 9] < 1.5)
        np.testing.assert_allclose(np.linalg.norm(f[:, 3:6], axis=1), 1, atol=1e-3)
        _, l0 = g.mlp_gradient(f, lab)
        l1 = g.mlp_train(epochs=10, batch=512, lr=2e-3, seed=1)
        _, l2 = g.mlp_gradient(f, lab)
        assert l2 < 0.8 * l0, (l0, l1, l2)
        g.pair_log_clear()
        assert len(g.pair_log()[0]) == 0


@pytest.mark.parametrize("name", ["sc_l2_dense", "hs_dense"])
def test_ordered_sweeps_leave_the_plain_state(engine, name):
    cfg = systems.ALL[name]()
    t, r = (0.1, 0.0) if cfg[0] == 0 else (0.2, 0.2)
    results = {}
    for mode in (_lib.ORDER_OFF, _lib.ORDER_DISTANCE, _lib.ORDER_MLP):
        with gpu_packing(cfg) as g:
            if mode == _lib.ORDER_MLP and cfg[0] == 1:
                # spheres reach no segment test, so only spherocylinders log pairs
                collect(g, 3, seed=99)
                g.mlp_train(epochs=8, batch=512, lr=2e-3, seed=2)
                g.pair_log_enable(0)
                g.upload(*cfg[2:])
            g.set_ordering(mode, every=2)
            acc = pairs = 0
            for c in range(5):
                st = g.sweep(t, r, seed=31, counter=c)
                acc += st["accepted"]
                pairs += st["pair_tests"]
            results[mode] = (g.state(), acc, pairs)
    (p0, r0, b0), acc0, pairs0 = results[_lib.ORDER_OFF]
    for mode in (_lib.ORDER_DISTANCE, _lib.ORDER_MLP):
        (p, rr, b), acc, pairs = results[mode]
        assert np.array_equal(p, p0) and np.array_equal(rr, r0), f"mode {mode}: state differs"
        assert acc == acc0
        if cfg[0] == 1:
            # spherocylinders find most overlaps in the segment stage: pre-testing the
            # ranked partners skips most of the scan of a rejected move
            assert pairs < pairs0, (mode, pairs, pairs0)


def test_ordered_sweep_log_replays_on_oracle(oracle, engine):
    cfg = systems.sc_l2_dense()
    kind, prm, pos, rot, box = cfg
    cpu = po.CpuPacking("oracle", kind, prm, pos, rot, box, threads=1)
    with gpu_packing(cfg) as g:
        g.set_ordering(_lib.ORDER_MLP, every=1)
        for cycle in range(2):
            g.sweep(0.2, 0.2, seed=404, counter=cycle, log=True)
            moves, codes = g.sweep_log()
            _, _, bounds = g.grid()
            want, _ = cpu.replay(moves, bounds)
            assert np.array_equal(codes, want)
        gp, gr, _ = g.state()
        cp, cr, _ = cpu.state()
        assert np.array_equal(gp, cp) and np.array_equal(gr, cr)


# ---- multi-centre bodies (bent chains and bent rods) ----------------------------------
def test_body_pair_log_and_training(engine):
    """Pairs of bent chains logged by the sweep carry the body-frame features (unit axes of
    the other body, |b|^2 and the squared separation across the primary axis consistent with
    the separation) and both labels; training on them lowers the loss."""
    cfg = systems.poly_dense()
    with gpu_packing(cfg) as g:
        f, lab = collect(g, 4)
        assert len(f) > 1000
        assert 0 < lab.mean() < 1
        assert np.all(np.isfinite(f)) and np.all(f[:, 13:] == 0)
        np.testing.assert_allclose(np.linalg.norm(f[:, 3:6], axis=1), 1, atol=1e-3)
        np.testing.assert_allclose(np.linalg.norm(f[:, 6:9], axis=1), 1, atol=1e-3)
        np.testing.assert_allclose(f[:, 9], (f[:, 0:3] ** 2).sum(1), rtol=1e-4, atol=1e-6)
        np.testing.assert_allclose(f[:, 12], (f[:, 0:2] ** 2).sum(1), rtol=1e-4, atol=1e-6)
        assert np.all(f[:, 9] < 1.5)  # within about one body reach before the move
        _, l0 = g.mlp_gradient(f, lab)
        g.mlp_train(epochs=10, batch=512, lr=2e-3, seed=1)
        _, l2 = g.mlp_gradient(f, lab)
        assert l2 < 0.8 * l0, (l0, l2)


@pytest.mark.parametrize("name", ["poly_dense", "psc_bent"])
def test_ordered_body_sweeps_leave_the_plain_state(engine, name):
    cfg = systems.ALL[name]()
    results = {}
    for mode in (_lib.ORDER_OFF, _lib.ORDER_DISTANCE, _lib.ORDER_MLP):
        with gpu_packing(cfg) as g:
            if mode == _lib.ORDER_MLP:
                collect(g, 3, seed=99)
                g.mlp_train(epochs=8, batch=512, lr=2e-3, seed=2)
                g.pair_log_enable(0)
                g.upload(*cfg[2:])
            g.set_ordering(mode, every=2)
            acc = pairs = 0
            for c in range(5):
                st = g.sweep(0.2, 0.2, seed=31, counter=c)
                acc += st["accepted"]
                pairs += st["pair_tests"]
            results[mode] = (g.state(), acc, pairs)
    (p0, r0, b0), acc0, pairs0 = results[_lib.ORDER_OFF]
    for mode in (_lib.ORDER_DISTANCE, _lib.ORDER_MLP):
        (p, rr, b), acc, pairs = results[mode]
        assert np.array_equal(p, p0) and np.array_equal(rr, r0), f"mode {mode}: state differs"
        assert acc == acc0
        if name == "poly_dense":
            # dense chains reject most moves, and the pre-tested partners find most of those
            # overlaps (the bent rods reject few moves, so the pre-test saves nothing there)
            assert pairs < pairs0, (mode, pairs, pairs0)


@pytest.mark.parametrize("name", ["poly_dense", "psc_bent"])
def test_ordered_body_sweep_log_replays_on_oracle(oracle, engine, name):
    cfg = systems.ALL[name]()
    kind, prm, pos, rot, box = cfg
    cpu = po.CpuPacking("oracle", kind, prm, pos, rot, box, threads=1)
    with gpu_packing(cfg) as g:
        collect(g, 2, seed=5)
        g.mlp_train(epochs=4, batch=512, lr=2e-3, seed=3)
        g.pair_log_enable(0)
        g.upload(pos, rot, box)
        g.set_ordering(_lib.ORDER_MLP, every=1)
        for cycle in range(2):
            g.sweep(0.2, 0.2, seed=404, counter=cycle, log=True)
            moves, codes = g.sweep_log()
            _, _, bounds = g.grid()
            want, _ = cpu.replay(moves, bounds)
            assert np.array_equal(codes, want)
        gp, gr, _ = g.state()
        cp, cr, _ = cpu.state()
        assert np.array_equal(gp, cp) and np.array_equal(gr, cr)
