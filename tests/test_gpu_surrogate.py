"""Surrogate network kernels against the CPU oracle, and the gated surrogate.

* one layer's forward GEMM + epilogue against torch (fp32 math on the same
  bf16 operands);
* the full backward pass (all weight and bias gradients) and the Adam update
  against the float64 oracle in oracle/mlp.py with bf16 rounding emulated;
* training lowers the loss on held-out states;
* the gate: tol = 0 sends every state to the exact kernel (result identical
  to CRS_MODE_FP64), states outside the training box always fall back, and
  the network's answer is returned unchanged where the gate passes;
* the gain over the method without it: calibrated for an error bound on
  held-out states labelled by the exact kernel, the gated surrogate (two
  networks, the error network's estimate and their disagreement in the
  gate) keeps the error of every state it serves within the bound on fresh
  states and evaluates them faster than the plain FP64 kernel alone.
"""
import ctypes
import tempfile

import numpy as np
import pytest

from create_rate_subs_gb300 import _lib, synth
from create_rate_subs_gb300.mechanism import Mechanism
from oracle import mlp as omlp

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

GRAD_TOL = 2e-2   # relative Frobenius error of gradients (fp32 vs fp64 sums, bf16 ties)
FWD_TOL = 1e-3    # relative error of one layer's fp32 output vs torch fp32


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _s():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


@pytest.fixture(scope="module")
def rs():
    from create_rate_subs_gb300.rates import RateSubs
    d = tempfile.mkdtemp(prefix="crs_sur_")
    return RateSubs(Mechanism.from_chemkin(*synth.write_mechanism("gri53", d)))


def test_forward_layer_matches_torch():
    lib = _lib.load()
    g = torch.Generator(device="cuda").manual_seed(0)
    M, K, N, n_valid = 384, 128, 256, 250
    X = torch.randn((M, K), generator=g, device="cuda").to(torch.bfloat16)
    W = torch.randn((N, K), generator=g, device="cuda").to(torch.bfloat16) * 0.1
    b = torch.randn(N, generator=g, device="cuda") * 0.1
    Z = torch.full((M, n_valid), float("nan"), device="cuda")
    A = torch.zeros((M, N), dtype=torch.bfloat16, device="cuda")
    AT = torch.zeros((N, M), dtype=torch.bfloat16, device="cuda")
    m_valid = 300
    assert lib.crs_mlp_forward(_p(X), _p(W), _p(b), M, N, K, m_valid, n_valid, 1,
                               _p(Z), n_valid, _p(A), N, _p(AT), M, None, 0, _s()) == 0, \
        _lib.last_error()
    ref = X.float() @ W.float().t() + b
    z = Z[:m_valid]
    err = (z - ref[:m_valid, :n_valid]).abs().max() / ref.abs().max()
    assert err <= FWD_TOL
    # SiLU in fp32 then one rounding to bf16: at most one bf16 step from torch
    a_ref = torch.nn.functional.silu(z)
    a = A[:m_valid, :n_valid].float()
    assert bool(((a - a_ref).abs() <= 2.0 ** -8 * a_ref.abs() + 1e-30).all())
    assert torch.equal(AT[:n_valid, :m_valid], A[:m_valid, :n_valid].t())
    assert torch.isnan(Z[m_valid:]).all()          # rows past m untouched
    assert (A[:, n_valid:] == 0).all() and (A[m_valid:] == 0).all()


@pytest.mark.parametrize("dims,m", [([55, 256, 256, 256, 53], 1000),
                                    ([55, 64, 128, 53], 300),
                                    ([55, 256, 53], 129),
                                    ([130, 128, 64, 256, 40], 513)])
def test_fused_inference_matches_layers(dims, m):
    """crs_mlp_infer (all layers in one kernel, activations on chip) against
    the layer-by-layer forward (activations through HBM) on the same bf16
    operands: the same fp32 sums in the same order, the same epilogue."""
    from create_rate_subs_gb300.surrogate import MLP
    net = MLP(dims, seed=11)
    assert net.fused_ok()
    M = (m + 127) // 128 * 128
    g = torch.Generator(device="cuda").manual_seed(5)
    X = torch.zeros((M, net.pad[0]), dtype=torch.bfloat16, device="cuda")
    X[:m, : dims[0]] = torch.randn((m, dims[0]), generator=g, device="cuda").to(torch.bfloat16)
    ref = torch.full((m, net.pad[-1]), float("nan"), device="cuda")
    got = torch.full((m, net.pad[-1]), float("nan"), device="cuda")
    net.forward(X, m, ref)
    net.infer(X, m, got)
    torch.cuda.synchronize()
    n = dims[-1]
    assert torch.isfinite(got[:, :n]).all()
    assert torch.isnan(got[:, n:]).all()          # columns past the output untouched
    err = float(((got[:, :n] - ref[:, :n]).abs().max() / ref[:, :n].abs().max()))
    print(dims, "max diff / max |y| =", err)
    assert err <= 1e-6


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("M,splits", [(256, 4), (1024, 16)])
def test_backward_matches_oracle(M, splits):
    from create_rate_subs_gb300.surrogate import MLP
    dims = [55, 256, 256, 256, 53]
    net = MLP(dims, seed=3)
    rng = np.random.default_rng(M)
    Xh = rng.standard_normal((M, 55)).astype(np.float32)
    Th = rng.standard_normal((M, 53)).astype(np.float32)
    X = torch.zeros((M, 64), dtype=torch.bfloat16, device="cuda")
    X[:, :55] = torch.from_numpy(Xh).cuda().to(torch.bfloat16)
    XT = X.t().contiguous()
    Tg = torch.from_numpy(Th).cuda()
    Ws = [omlp.bf16_round(w.cpu().numpy()) for w in net.W32]
    bs = [b.cpu().numpy().astype(np.float64) for b in net.b32]
    loss_ref, gW_ref, gb_ref = omlp.loss_and_grads(
        X[:, :55].float().cpu().numpy().astype(np.float64), Th.astype(np.float64), Ws, bs)
    loss = torch.zeros(1, device="cuda")
    W32_before = [w.clone() for w in net.W32]
    net.train_step(X, XT, Tg, lr=1e-3, loss_slot=loss, splits=splits)
    torch.cuda.synchronize()
    assert abs(loss.item() - loss_ref) <= 1e-3 * loss_ref
    for l in range(4):
        assert _rel(net.gW[l].cpu().numpy(), gW_ref[l]) <= GRAD_TOL, ("W", l)
        assert _rel(net.gb[l].cpu().numpy(), gb_ref[l]) <= GRAD_TOL, ("b", l)
    # the Adam update applied to the kernel's own gradient
    for l in range(4):
        p1, _, _ = omlp.adam(W32_before[l].cpu().numpy().astype(np.float64),
                             net.gW[l].cpu().numpy().astype(np.float64),
                             np.zeros(net.gW[l].shape), np.zeros(net.gW[l].shape), 1, 1e-3)
        np.testing.assert_allclose(net.W32[l].cpu().numpy(), p1, rtol=0, atol=2e-6)
        # bf16 copies refreshed from the new master weights
        w16 = net.W32[l].to(torch.bfloat16)
        assert torch.equal(net.W[l][: dims[l + 1], : dims[l]], w16)
        assert torch.equal(net.WT[l][: dims[l], : dims[l + 1]], w16.t())


def test_split_count_does_not_change_gradient_much():
    from create_rate_subs_gb300.surrogate import MLP
    M = 1024
    g = torch.Generator(device="cuda").manual_seed(5)
    X = torch.zeros((M, 64), dtype=torch.bfloat16, device="cuda")
    X[:, :55] = torch.randn((M, 55), generator=g, device="cuda").to(torch.bfloat16)
    XT = X.t().contiguous()
    Tg = torch.randn((M, 53), generator=g, device="cuda")
    grads = []
    for splits in (1, 16):
        net = MLP([55, 256, 256, 256, 53], seed=7)
        net.train_step(X, XT, Tg, lr=1e-3, splits=splits)
        grads.append([w.clone() for w in net.gW])
    for a, b in zip(*grads):
        assert float((a - b).norm() / b.norm()) <= 1e-5


@pytest.fixture(scope="module")
def trained(rs):
    from create_rate_subs_gb300.surrogate import Surrogate
    sur = Surrogate(rs, seed=0, batch=8192)
    untrained = Surrogate(rs, seed=0, batch=8192)
    T, P, Y = sur.sample_states(1 << 14, seed=77)       # held-out states
    losses = sur.fit(n_train=1 << 18, epochs=6, lr=2e-3, seed=11)
    for k in ("mu", "sd", "lo", "hi"):                    # same inputs, same scales
        getattr(untrained, k).copy_(getattr(sur, k))
    untrained.set_scale(sur.scale.cpu().numpy())
    before = untrained.loss(T, P, Y)                      # the initial weights
    after = sur.loss(T, P, Y)
    return sur, untrained, (T, P, Y), before, after, losses


def test_training_lowers_loss(trained):
    sur, _, _, before, after, losses = trained
    assert np.all(np.isfinite(losses))
    assert losses[-1] < losses[0]
    assert after < 0.5 * before, (before, after)


def test_gate_tol_zero_is_exact(rs, trained):
    sur, _, (T, P, Y), _, _, _ = trained
    w, nfb = sur.wdot(T, P, Y, tol=0.0)
    exact = rs.wdot(T, P, Y, mode="fp64")
    assert nfb == T.shape[0]
    assert torch.equal(w, exact)


def test_gate_out_of_box_falls_back(rs, trained):
    sur, _, (T, P, Y), _, _, _ = trained
    n = 1000
    T2 = T[:n].clone()
    T2[::3] = 4000.0          # far outside the training box
    P2, Y2 = P[:n].contiguous(), Y[:, :n].contiguous()
    raw, _ = sur.wdot(T2, P2, Y2, tol=float("inf"), with_fallback=False)
    w, nfb = sur.wdot(T2, P2, Y2, tol=float("inf"))
    exact = rs.wdot(T2, P2, Y2, mode="fp64")
    hot = torch.zeros(n, dtype=torch.bool, device="cuda")
    hot[::3] = True
    assert nfb >= int(hot.sum())
    assert torch.equal(w[:, hot], exact[:, hot])
    # in-box states with an infinite tolerance keep the network's answer
    inbox = ~hot
    same = (w[:, inbox] == raw[:, inbox]).all(dim=0) | (w[:, inbox] == exact[:, inbox]).all(dim=0)
    assert bool(same.all())


# error bound of the gain test (e = max_k |w_k - w_k,exact| / (|w_k,exact| +
# s_k)), and the fraction of it the calibration aims at on held-out states
GAIN_BOUND = 0.2
GAIN_MARGIN = 0.5


@pytest.fixture(scope="module")
def gated(rs):
    from create_rate_subs_gb300.surrogate import Surrogate
    sur = Surrogate(rs, seed=0, batch=16384)
    sur.fit(n_train=1 << 22, epochs=8, lr=2e-3, lr_final=2e-5, seed=21)
    sur.fit_gate(n=1 << 21, epochs=12, seed=22)
    cal = sur.calibrate(GAIN_BOUND, n=1 << 21, seed=23, margin=GAIN_MARGIN)
    return sur, cal


def _ms(fn, reps=3):
    fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def test_gated_surrogate_bounds_error_and_beats_plain_fp64(rs, gated):
    """On 2^20 fresh states the gated surrogate's result is within
    GAIN_BOUND of the exact FP64 kernel's on every state, and it is faster
    than evaluating every state with that kernel."""
    sur, cal = gated
    n = 1 << 20
    T, P, Y = sur.sample_states(n, seed=24)
    Y = Y[: rs.n_species - 1].contiguous()
    exact = rs.wdot(T, P, Y, mode="fp64")
    w, nfb = sur.wdot(T, P, Y)
    err = sur.served_error(w, exact)
    out = torch.empty_like(exact)
    ms_sur = _ms(lambda: sur.wdot(T, P, Y, out=out))
    ms_plain = _ms(lambda: rs.wdot(T, P, Y, mode="fp64", out=out))
    print("calibration %s; fresh states: fallback %.3f, max error %.4f, p99 %.4f; "
          "%.2f ms gated vs %.2f ms plain FP64" % (cal, nfb / n, float(err.max()),
                                                  float(err.quantile(0.99)), ms_sur, ms_plain))
    assert 0 < nfb < n
    assert float(err.max()) <= GAIN_BOUND
    assert ms_sur < ms_plain
