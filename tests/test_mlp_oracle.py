"""The CPU oracle of the surrogate network: bf16 rounding, gradients, Adam."""
import numpy as np
import pytest

from oracle import mlp


def _net(rng, dims):
    Ws = [rng.standard_normal((dims[l + 1], dims[l])) / np.sqrt(dims[l])
          for l in range(len(dims) - 1)]
    bs = [0.1 * rng.standard_normal(dims[l + 1]) for l in range(len(dims) - 1)]
    return Ws, bs


def test_bf16_round_matches_torch():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.standard_normal(10000) * 10.0 ** rng.integers(-30, 30, 10000),
                        [0.0, -0.0, 1.0, 1.00390625, 1.01171875, 3.0e38]])
    want = torch.from_numpy(x.astype(np.float32)).to(torch.bfloat16).to(torch.float64).numpy()
    np.testing.assert_array_equal(mlp.bf16_round(x), want)


def test_gradients_match_finite_differences():
    rng = np.random.default_rng(1)
    dims = [7, 16, 16, 5]
    Ws, bs = _net(rng, dims)
    X = rng.standard_normal((11, 7))
    Tg = rng.standard_normal((11, 5))
    loss, gW, gb = mlp.loss_and_grads(X, Tg, Ws, bs, bf16=False)
    h = 1e-6
    for l in range(len(Ws)):
        for (i, j) in [(0, 0), (dims[l + 1] - 1, dims[l] - 1), (2, 3)]:
            Wp = [w.copy() for w in Ws]
            Wp[l][i, j] += h
            Wm = [w.copy() for w in Ws]
            Wm[l][i, j] -= h
            fd = (mlp.loss_and_grads(X, Tg, Wp, bs, False)[0]
                  - mlp.loss_and_grads(X, Tg, Wm, bs, False)[0]) / (2 * h)
            assert abs(fd - gW[l][i, j]) <= 1e-7 * max(1.0, abs(fd)), (l, i, j)
        bp = [b.copy() for b in bs]
        bp[l][1] += h
        bm = [b.copy() for b in bs]
        bm[l][1] -= h
        fd = (mlp.loss_and_grads(X, Tg, Ws, bp, False)[0]
              - mlp.loss_and_grads(X, Tg, Ws, bm, False)[0]) / (2 * h)
        assert abs(fd - gb[l][1]) <= 1e-7 * max(1.0, abs(fd))


def test_bf16_emulation_is_close_to_exact():
    rng = np.random.default_rng(2)
    dims = [55, 64, 64, 53]
    Ws, bs = _net(rng, dims)
    X = rng.standard_normal((64, 55))
    Tg = rng.standard_normal((64, 53))
    l64, g64, _ = mlp.loss_and_grads(X, Tg, Ws, bs, bf16=False)
    l16, g16, _ = mlp.loss_and_grads(X, Tg, Ws, bs, bf16=True)
    assert abs(l16 - l64) <= 0.02 * l64
    for a, b in zip(g16, g64):
        assert np.linalg.norm(a - b) <= 0.05 * np.linalg.norm(b)


def test_adam_first_step_moves_by_lr():
    p = np.array([1.0, -2.0, 0.5])
    g = np.array([0.3, -1e-3, 0.0])
    p1, m, v = mlp.adam(p, g, np.zeros(3), np.zeros(3), 1, 0.01)
    # bias-corrected first step: p - lr * sign(g) (up to eps)
    np.testing.assert_allclose(p1[:2], p[:2] - 0.01 * np.sign(g[:2]), rtol=0, atol=1e-7)
    assert p1[2] == p[2]
