"""CPU checks of the ranking network's restatement (oracle/mlp_ref.py): BF16 rounding
against torch's conversion, and the backward pass against finite differences."""
import numpy as np
import pytest

from oracle import mlp_ref


def test_bf16_rounding_matches_torch():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.normal(0, 1, 4096), rng.normal(0, 1e-3, 1024), rng.normal(0, 1e4, 1024),
                        [0.0, -0.0, 1.0, 1.00390625, 1.005859375, -3.0e38]]).astype(np.float32)
    want = torch.from_numpy(x).to(torch.bfloat16).to(torch.float32).numpy()
    got = mlp_ref.bf16(x)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def _pairs(n, seed):
    rng = np.random.default_rng(seed)
    d = rng.uniform(-1.0, 1.0, (n, 3))
    ai = rng.normal(size=(n, 3))
    ai /= np.linalg.norm(ai, axis=1, keepdims=True)
    aj = rng.normal(size=(n, 3))
    aj /= np.linalg.norm(aj, axis=1, keepdims=True)
    f = mlp_ref.features(d * 3.0, ai, aj, 1.0 / 3.0)
    lab = (rng.uniform(size=n) < 0.3).astype(np.uint8)
    return f, lab


def test_features_layout():
    f, _ = _pairs(5, 1)
    assert f.shape == (5, 16) and np.all(f[:, 13:] == 0)
    np.testing.assert_allclose(f[:, 9], (f[:, :3] ** 2).sum(1), rtol=1e-6)
    np.testing.assert_allclose(np.linalg.norm(f[:, 3:6], axis=1), 1, rtol=1e-6)


def test_gradient_matches_finite_differences():
    f, lab = _pairs(48, 2)
    w = mlp_ref.init_params(3).astype(np.float64)
    _, g = mlp_ref.loss_and_grad(f, lab, w, rounding=False)
    rng = np.random.default_rng(4)
    idx = np.concatenate([rng.choice(np.arange(mlp_ref.W1, mlp_ref.B1).reshape(64, 16)[:, :13].ravel(), 12),
                          rng.choice(np.arange(mlp_ref.B1, mlp_ref.NPARAM), 36, replace=False)])
    eps = 1e-6
    for k in idx:
        wp, wm = w.copy(), w.copy()
        wp[k] += eps
        wm[k] -= eps
        fd = (mlp_ref.loss(f, lab, wp, rounding=False) - mlp_ref.loss(f, lab, wm, rounding=False)) / (2 * eps)
        assert abs(fd - g[k]) <= 1e-6 + 1e-4 * abs(fd), (k, fd, g[k])


def test_rounded_gradient_close_to_unrounded():
    # the straight-through BF16 gradient differs from the exact one by BF16-sized terms only
    f, lab = _pairs(256, 5)
    w = mlp_ref.init_params(6)
    _, g0 = mlp_ref.loss_and_grad(f, lab, w, rounding=False)
    _, g1 = mlp_ref.loss_and_grad(f, lab, w, rounding=True)
    assert np.linalg.norm(g1 - g0) <= 0.05 * np.linalg.norm(g0)
