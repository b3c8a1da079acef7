"""Learned surrogate for wdot with exact fallback.

Two multilayer perceptrons ("members", different initial weights and batch
order, same training states) map a state's features -- T, ln P and
ln(Y_k + 1e-12) for every species, standardised -- to the species
production rates, each normalised by its standard deviation over the
training states and passed through sign(x) log(1 + |x|):

    y_k = sign(w_k / s_k) log1p(|w_k| / s_k),   s_k = std(w_k)

The served y is the members' mean.  The default network is
55 -> 256 -> 256 -> 256 -> 53 (SiLU) for the 53-species mechanism.  Weights
are bf16 on the tensor cores with fp32 accumulation and fp32 master
copies; training (forward, backward, Adam) and inference run entirely in
libcrs's own kernels (crs_mlp_*, crs_adam_step, crs_surrogate_*).
Training states are drawn like the benchmark states and labelled by the
exact FP64 kernel.

Error measure reported for the surrogate: e = max_k |w_k - w_k,exact| /
(|w_k,exact| + s_k), i.e. relative error where a rate is large and error in
units of the species' typical rate where it is small.  In y space a change
dy moves w by |dy| (|w| + s) to first order, so e is about max_k |dy_k|.

Every evaluation is gated.  A state goes back to the exact kernel
(CRS_MODE_FP64 on the gathered states, results scattered into place) when

* one of its features lies outside the box spanned by the training states
  (widened by 2 % of each feature's range), or
* its element residual max_e |sum_k a_ek w_k| / sum_k a_ek (|w_k| + s_k)
  exceeds ``tol`` (exact production rates conserve every element), or
* its error score exceeds ``stol``: the output of an error network
  (56 -> 256 -> 256 -> 1: the 55 features and the members' disagreement
  D = max_k |y_k,a - y_k,b| as log10(D + 1e-4), standardised) trained on
  held-out states, labelled by the exact kernel, to predict log10(e + 1e-4)
  of the served result.  Before ``fit_gate`` the score is log10(D + 1e-4)
  alone.

``calibrate(bound)`` sets ``stol`` from a further held-out set labelled by
the exact kernel: the largest score up to which every calibration state
has e <= margin * bound (margin 0.5 by default).  The plain kernel is thus both the fallback and the arbiter
of the surrogate's error; the bound holds on the calibration states and is
measured again on fresh states by the tests and bench.py.

The reference has no surrogate; this module is the learned part that sits
beside its four functions.
"""
import ctypes
import math

import numpy as np

from . import _lib

__all__ = ["MLP", "Surrogate", "surrogate_error"]

ACT_NONE, ACT_SILU = 0, 1
Y_FLOOR = 1e-12


def _torch():
    import torch
    return torch


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _r(x, m):
    return (x + m - 1) // m * m


def _stream(device):
    return ctypes.c_void_p(_torch().cuda.current_stream(device).cuda_stream)


class MLP(object):
    """Weights, Adam moments and work buffers of a bf16 perceptron.

    dims = [n_in, h_1, ..., n_out].  Layer l holds fp32 master weights
    W32[l] (n_out x n_in) and bias b32[l], their bf16 copies W[l]
    (padded to 64 x 64 multiples, zero outside) and WT[l] (transposed), and
    Adam moments.  Hidden widths must be multiples of 64 up to 256 or
    multiples of 256."""

    def __init__(self, dims, seed=0, device=None):
        torch = _torch()
        self.lib = _lib.load()
        if device is None:
            device = torch.cuda.current_device()
        self.device = device if isinstance(device, torch.device) else torch.device("cuda", device)
        self.dims = [int(d) for d in dims]
        self.L = len(self.dims) - 1
        self.pad = [_r(d, 64) for d in self.dims]
        for h in self.pad[1:-1]:
            if not (h in (64, 128, 256) or h % 256 == 0):
                raise ValueError("hidden width %d not supported" % h)
        g = torch.Generator().manual_seed(seed)
        f32 = dict(dtype=torch.float32, device=self.device)
        bf = dict(dtype=torch.bfloat16, device=self.device)
        self.W32, self.b32, self.W, self.WT = [], [], [], []
        self.mW, self.vW, self.mb, self.vb, self.gW, self.gb = [], [], [], [], [], []
        for l in range(self.L):
            nin, nout = self.dims[l], self.dims[l + 1]
            bound = 1.0 / math.sqrt(nin)
            w = (torch.rand((nout, nin), generator=g, dtype=torch.float32) * 2 - 1) * bound
            b = (torch.rand((nout,), generator=g, dtype=torch.float32) * 2 - 1) * bound
            self.W32.append(w.to(self.device))
            self.b32.append(b.to(self.device))
            self.W.append(torch.zeros((self.pad[l + 1], self.pad[l]), **bf))
            self.WT.append(torch.zeros((self.pad[l], self.pad[l + 1]), **bf))
            for lst, shape in ((self.mW, (nout, nin)), (self.vW, (nout, nin)),
                               (self.gW, (nout, nin)), (self.mb, (nout,)),
                               (self.vb, (nout,)), (self.gb, (nout,))):
                lst.append(torch.zeros(shape, **f32))
        self.step = 0
        self.refresh_bf16()
        self._train = None
        self._infer = None

    # -- weights ---------------------------------------------------------
    def refresh_bf16(self):
        """bf16 copies from the fp32 master weights (round to nearest)."""
        for l in range(self.L):
            nin, nout = self.dims[l], self.dims[l + 1]
            self.W[l][:nout, :nin] = self.W32[l].to(self.W[l].dtype)
            self.WT[l][:nin, :nout] = self.W32[l].t().to(self.W[l].dtype)

    def state_dict(self):
        """Everything needed to resume training (host numpy arrays)."""
        d = {"dims": np.array(self.dims), "step": np.array(self.step)}
        for l in range(self.L):
            for name in ("W32", "b32", "mW", "vW", "mb", "vb"):
                d["%s_%d" % (name, l)] = getattr(self, name)[l].cpu().numpy()
        return d

    def load_state_dict(self, d):
        torch = _torch()
        if [int(x) for x in d["dims"]] != self.dims:
            raise ValueError("checkpoint dims %s != %s" % (list(d["dims"]), self.dims))
        self.step = int(d["step"])
        for l in range(self.L):
            for name in ("W32", "b32", "mW", "vW", "mb", "vb"):
                getattr(self, name)[l].copy_(torch.from_numpy(d["%s_%d" % (name, l)]))
        self.refresh_bf16()

    # -- buffers ---------------------------------------------------------
    def _train_bufs(self, M_pad, splits):
        torch = _torch()
        key = (M_pad, splits)
        if self._train is not None and self._train["key"] == key:
            return self._train
        f32 = dict(dtype=torch.float32, device=self.device)
        bf = dict(dtype=torch.bfloat16, device=self.device)
        L, d, p = self.L, self.dims, self.pad
        b = {"key": key}
        b["Z"] = [torch.zeros((M_pad, d[l + 1]), **f32) for l in range(L - 1)]
        b["A"] = [torch.zeros((M_pad, p[l + 1]), **bf) for l in range(L - 1)]
        b["AT"] = [torch.zeros((p[l + 1], M_pad), **bf) for l in range(L - 1)]
        b["dZ"] = [torch.zeros((M_pad, p[l + 1]), **bf) for l in range(L)]
        b["dZT"] = [torch.zeros((_r(p[l + 1], 128), M_pad), **bf) for l in range(L)]
        b["Yh"] = torch.zeros((M_pad, p[L]), **f32)
        b["partial"] = torch.zeros(
            (splits * max(_r(p[l + 1], 128) * p[l] for l in range(L)),), **f32)
        self._train = b
        return b

    def _infer_bufs(self, M_pad):
        torch = _torch()
        if self._infer is not None and self._infer["M_pad"] >= M_pad:
            return self._infer
        bf = dict(dtype=torch.bfloat16, device=self.device)
        w = max(self.pad[1:-1])
        b = {"M_pad": M_pad,
             "A": [torch.empty((M_pad * w,), **bf), torch.empty((M_pad * w,), **bf)]}
        self._infer = b
        return b

    # -- passes ----------------------------------------------------------
    def forward(self, X, m, Y, stream=None):
        """Y[:m, :n_out] (fp32, unit column stride) = network(X); X bf16
        (M_pad, pad[0]) with M_pad = m rounded up to 128 (rows >= m are
        ignored).  Rows of Y a multiple of 4 floats apart store fastest."""
        s = stream if stream is not None else _stream(self.device)
        M_pad = X.shape[0]
        if M_pad % 128 or M_pad < m or X.shape[1] != self.pad[0]:
            raise ValueError("X must be (m rounded up to 128, %d)" % self.pad[0])
        if Y.dim() != 2 or Y.shape[0] < m or Y.shape[1] < self.dims[-1] or Y.stride(1) != 1:
            raise ValueError("Y must be (m, >= %d) with unit column stride" % self.dims[-1])
        b = self._infer_bufs(M_pad)
        a = X
        L, d, p = self.L, self.dims, self.pad
        for l in range(L):
            last = l == L - 1
            out = None if last else b["A"][l % 2][: M_pad * p[l + 1]].view(M_pad, p[l + 1])
            _lib.check(self.lib.crs_mlp_forward(
                _p(a), _p(self.W[l]), _p(self.b32[l]), M_pad, p[l + 1], p[l], m, d[l + 1],
                ACT_NONE if last else ACT_SILU, None, 0, _p(out), p[l + 1] if out is not None else 0,
                None, 0, _p(Y) if last else None, Y.stride(0) if last else 0, s))
            a = out
        return Y

    def fused_ok(self):
        """True when infer() runs the whole network in one kernel: at most
        6 layers, every padded width <= 256."""
        return self.L <= 6 and max(self.pad) <= 256

    def infer(self, X, m, Y, stream=None):
        """forward() for inference: the whole network in one kernel per tile
        of 128 states (crs_mlp_infer), the activations kept on chip, when
        fused_ok(); the layer-by-layer forward() otherwise.  Same arguments
        and result."""
        if not self.fused_ok():
            return self.forward(X, m, Y, stream)
        s = stream if stream is not None else _stream(self.device)
        M_pad = X.shape[0]
        if M_pad % 128 or M_pad < m or X.shape[1] != self.pad[0] or not X.is_contiguous():
            raise ValueError("X must be a contiguous (m rounded up to 128, %d)" % self.pad[0])
        if Y.dim() != 2 or Y.shape[0] < m or Y.shape[1] < self.dims[-1] or Y.stride(1) != 1:
            raise ValueError("Y must be (m, >= %d) with unit column stride" % self.dims[-1])
        L = self.L
        args = (ctypes.c_int64 * (L + 1))(*self.dims), (ctypes.c_int64 * (L + 1))(*self.pad), \
            (ctypes.c_void_p * L)(*[w.data_ptr() for w in self.W]), \
            (ctypes.c_void_p * L)(*[b.data_ptr() for b in self.b32])
        _lib.check(self.lib.crs_mlp_infer(_p(X), M_pad, m, L, *args, _p(Y), Y.stride(0),
                                          None, s))
        return Y

    def train_step(self, X, XT, Tg, lr, loss_slot=None, splits=32, b1=0.9, b2=0.999,
                   eps=1e-8, stream=None):
        """One Adam step on the batch (X: bf16 (M, pad[0]), XT: bf16
        (pad[0], M), Tg: fp32 (M, n_out) targets; M a multiple of 128).
        The batch's mean squared error is added to loss_slot (fp32 device
        scalar) when given."""
        s = stream if stream is not None else _stream(self.device)
        M = X.shape[0]
        if M % 128 or XT.shape != (self.pad[0], M) or Tg.shape != (M, self.dims[-1]):
            raise ValueError("bad batch shapes")
        while splits > 1 and (M // 64) % splits:
            splits //= 2
        b = self._train_bufs(M, splits)
        L, d, p = self.L, self.dims, self.pad
        lib = self.lib
        a = X
        for l in range(L):
            last = l == L - 1
            _lib.check(lib.crs_mlp_forward(
                _p(a), _p(self.W[l]), _p(self.b32[l]), M, p[l + 1], p[l], M, d[l + 1],
                ACT_NONE if last else ACT_SILU,
                None if last else _p(b["Z"][l]), d[l + 1],
                None if last else _p(b["A"][l]), p[l + 1],
                None if last else _p(b["AT"][l]), M,
                _p(b["Yh"]) if last else None, p[L], s))
            if not last:
                a = b["A"][l]
        _lib.check(lib.crs_mlp_loss_grad(
            _p(b["Yh"]), p[L], _p(Tg), d[L], M, d[L], p[L], 1.0 / (M * d[L]),
            _p(b["dZ"][L - 1]), p[L], _p(b["dZT"][L - 1]), M, _p(loss_slot), s))
        for l in range(L - 1, -1, -1):
            aT = XT if l == 0 else b["AT"][l - 1]
            _lib.check(lib.crs_mlp_backward_weight(
                _p(b["dZT"][l]), _p(aT), _r(p[l + 1], 128), p[l], M, d[l + 1], d[l],
                splits, _p(b["partial"]), _p(self.gW[l]), s))
            _lib.check(lib.crs_mlp_row_sums(_p(b["dZT"][l]), M, d[l + 1], M,
                                            _p(self.gb[l]), s))
            if l > 0:
                _lib.check(lib.crs_mlp_backward_data(
                    _p(b["dZ"][l]), _p(self.WT[l]), M, p[l], p[l + 1], M, d[l],
                    _p(b["Z"][l - 1]), d[l], _p(b["dZ"][l - 1]), p[l],
                    _p(b["dZT"][l - 1]), M, s))
        self.step += 1
        for l in range(L):
            _lib.check(lib.crs_adam_step(
                _p(self.W32[l]), _p(self.gW[l]), _p(self.mW[l]), _p(self.vW[l]),
                d[l + 1], d[l], lr, b1, b2, eps, self.step,
                _p(self.W[l]), p[l], _p(self.WT[l]), p[l + 1], s))
            _lib.check(lib.crs_adam_step(
                _p(self.b32[l]), _p(self.gb[l]), _p(self.mb[l]), _p(self.vb[l]),
                1, d[l + 1], lr, b1, b2, eps, self.step, None, 0, None, 0, s))
        return b

    def launches_per_step(self):
        """Kernels one train_step launches."""
        return self.L + 1 + 2 * self.L + self.L + (self.L - 1) + 2 * self.L


def surrogate_error(w, w_exact, scale):
    """Per-state max_k |w - w_exact| / (|w_exact| + s_k) (numpy, (N, n))."""
    s = np.asarray(scale, dtype=np.float64)[:, None]
    return np.max(np.abs(w - w_exact) / (np.abs(w_exact) + s), axis=0)


class Surrogate(object):
    """wdot(T, P, Y) from the trained networks, with gated exact fallback.

    ``rs`` is a RateSubs (the exact kernel: labels, fallback and arbiter).
    ``members``: 2 (served y = mean of two networks, their disagreement in
    the gate) or 1."""

    def __init__(self, rs, hidden=(256, 256, 256), seed=0, batch=16384, members=2,
                 err_hidden=(256, 256)):
        torch = _torch()
        if rs.mech is None:
            raise ValueError("the surrogate needs the Mechanism (element counts)")
        if members not in (1, 2):
            raise ValueError("members must be 1 or 2")
        self.rs = rs
        self.lib = rs.lib
        self.device = rs.device
        N = rs.n_species
        self.N = N
        self.n_in = 2 + N
        self.nets = [MLP([self.n_in] + list(hidden) + [N], seed=seed + 7919 * j,
                         device=self.device) for j in range(members)]
        self.net = self.nets[0]
        # the error network reads the features and, in the first padding
        # column, the members' standardised log10 disagreement
        self.err_net = MLP([self.n_in + 1] + list(err_hidden) + [1], seed=seed + 104729,
                           device=self.device)
        if self.err_net.pad[0] != self.net.pad[0]:
            raise ValueError("the feature rows need a free padding column")
        self.err_trained = False
        self.gate_mu, self.gate_sd = 0.0, 1.0
        self.stol = float("inf")   # gate threshold on the error score
        self.bound = None          # the calibrated error bound, if any
        self.batch = int(batch)
        if self.batch % 128:
            raise ValueError("batch must be a multiple of 128")
        _, A = rs.mech.element_matrix()
        self.atoms = np.rint(A)
        self.n_elem = A.shape[0]
        if self.n_elem > 8:
            raise ValueError("at most 8 elements")
        f32 = dict(dtype=torch.float32, device=self.device)
        self.mu = torch.zeros(self.n_in, **f32)
        self.sd = torch.ones(self.n_in, **f32)
        self.lo = torch.full((self.n_in,), -np.inf, **f32)
        self.hi = torch.full((self.n_in,), np.inf, **f32)
        self.set_scale(np.ones(N))
        self.history = []

    def set_scale(self, scale):
        """Species scales s_k (float64; rates exceed the fp32 range) and the
        tables the output kernel derives from them."""
        torch = _torch()
        s = np.asarray(scale, dtype=np.float64)
        if s.shape != (self.N,) or not np.all(np.isfinite(s)) or np.any(s <= 0):
            raise ValueError("scales must be N positive finite numbers")
        self.scale = torch.from_numpy(s.copy()).to(self.device)
        m, e = np.frexp(s)                          # s = m 2^e, m in [0.5, 1)
        self._scale_m = torch.from_numpy(m.astype(np.float32)).to(self.device)
        self._scale_e = torch.from_numpy(e.astype(np.int32)).to(self.device)
        c = self.atoms * s[None, :]
        c = c / np.maximum(c.max(axis=1, keepdims=True), 1e-300)
        self._cons = torch.from_numpy(np.ascontiguousarray(c, dtype=np.float32)).to(self.device)

    # -- data ------------------------------------------------------------
    def sample_states(self, n, seed):
        """Seeded states on the device, distributed like synth.make_states:
        T ~ U[800, 2800] K, P log-uniform in [1, 50] atm, Y ~ Dirichlet(0.5)."""
        torch = _torch()
        from . import chem
        g = torch.Generator(device=self.device).manual_seed(int(seed))
        f64 = dict(dtype=torch.float64, device=self.device)
        T = torch.rand(n, generator=g, **f64) * 2000.0 + 800.0
        P = torch.exp(torch.rand(n, generator=g, **f64) * math.log(50.0)) * chem.PA
        Y = torch.empty((self.N, n), **f64)
        with torch.random.fork_rng(devices=[self.device]):
            torch.cuda.manual_seed(int(seed) + 1)
            Y.copy_(torch._standard_gamma(torch.full((self.N, n), 0.5, **f64)))
        Y /= Y.sum(dim=0, keepdim=True)
        return T, P, Y

    def features(self, T, P, Y, ld, n, X, XT=None, ldxt=0, out_of_box=None, raw=None,
                 box=True):
        _lib.check(self.lib.crs_surrogate_features(
            n, _p(T), _p(P), _p(Y), ld, self.N, _p(self.mu), _p(self.sd),
            _p(self.lo) if box else None, _p(self.hi) if box else None, _p(X),
            self.net.pad[0], _p(XT), ldxt, self.net.pad[0], _p(out_of_box), _p(raw),
            _stream(self.device)))

    def targets(self, W):
        """(n, N) fp32 training targets from exact wdot (N, n)."""
        torch = _torch()
        x = W / self.scale[:, None]
        return (torch.sign(x) * torch.log1p(torch.abs(x))).t().contiguous().float()

    def _batches(self, T, P, Y, n):
        """Features of n states (a multiple of the batch) as X (n, pad) and
        the per-batch transposes XT (nb, pad, B) that training reads."""
        torch = _torch()
        B = self.batch
        nb = n // B
        X = torch.zeros((n, self.net.pad[0]), dtype=torch.bfloat16, device=self.device)
        XT = torch.zeros((nb, self.net.pad[0], B), dtype=torch.bfloat16, device=self.device)
        for j in range(nb):
            o = j * B
            self.features(T[o:], P[o:], Y[:, o:], Y.stride(0), B, X[o:], XT[j], B, box=False)
        return X, XT

    def _train(self, net, X, XT, Tg, epochs, lr, lr_final, seed):
        """Adam with a cosine learning-rate schedule over shuffled batches;
        returns the mean loss per epoch."""
        torch = _torch()
        B = self.batch
        nb = X.shape[0] // B
        losses = torch.zeros(epochs * nb, dtype=torch.float32, device=self.device)
        rng = np.random.default_rng(seed)
        total = epochs * nb
        for e in range(epochs):
            order = rng.permutation(nb)
            for i, j in enumerate(order):
                st = e * nb + i
                lr_s = lr_final + 0.5 * (lr - lr_final) * (1 + math.cos(math.pi * st / total))
                o = int(j) * B
                net.train_step(X[o:o + B], XT[int(j)], Tg[o:o + B], lr_s,
                               loss_slot=losses[st:st + 1])
        return losses.view(epochs, nb).mean(dim=1).cpu().numpy().tolist()

    # -- training --------------------------------------------------------
    def fit(self, n_train=1 << 20, epochs=4, lr=1e-3, lr_final=1e-5, seed=1,
            states=None):
        """Label n_train states with the exact kernel and train every member
        on them (member j shuffles with seed + j).  Returns the members'
        mean training loss per epoch."""
        torch = _torch()
        B = self.batch
        n = _r(n_train, B)
        T, P, Y = states if states is not None else self.sample_states(n, seed)
        n = T.shape[0]
        if n % B:
            raise ValueError("number of training states must be a multiple of the batch")
        W = self.rs.wdot(T, P, Y, mode="fp64")
        sd = W.std(dim=1).cpu().numpy()
        self.set_scale(np.where(np.isfinite(sd) & (sd > 0), sd, 1.0))
        # feature statistics and the training box from the raw features
        f32 = dict(dtype=torch.float32, device=self.device)
        X = torch.zeros((n, self.net.pad[0]), dtype=torch.bfloat16, device=self.device)
        raw = torch.empty((n, self.n_in), **f32)
        self.mu.zero_()
        self.sd.fill_(1.0)
        self.features(T, P, Y, n, n, X, raw=raw, box=False)
        self.mu.copy_(raw.mean(dim=0))
        self.sd.copy_(raw.std(dim=0).clamp_min(1e-6))
        lo, hi = raw.min(dim=0).values, raw.max(dim=0).values
        self.lo.copy_(lo - 0.02 * (hi - lo))
        self.hi.copy_(hi + 0.02 * (hi - lo))
        del raw, X
        X, XT = self._batches(T, P, Y, n)
        Tg = self.targets(W)
        del W
        per = [self._train(net, X, XT, Tg, epochs, lr, lr_final, seed + j)
               for j, net in enumerate(self.nets)]
        per_epoch = np.mean(np.array(per), axis=0).tolist()
        self.history.extend(per_epoch)
        # the error network and the gate threshold belong to the old weights
        self.err_trained = False
        self.stol, self.bound = float("inf"), None
        return per_epoch

    def served_error(self, w, W):
        """Per-state e = max_k |w_k - W_k| / (|W_k| + s_k) (device, (n,))."""
        return ((w - W).abs() / (W.abs() + self.scale[:, None])).amax(dim=0)

    def fit_gate(self, n=1 << 22, epochs=12, lr=2e-3, lr_final=2e-5, seed=2, states=None,
                 top=0.1, copies=3):
        """Train the error network on n held-out states (seed: their draw,
        unless ``states`` is given) labelled by the exact kernel: target
        log10(e + 1e-4), e the error of the served (members' mean) result.
        The fraction ``top`` of the states with the largest errors is seen
        ``copies`` more times (the gate has to rank the tail; on 2^24 fresh
        states this cut the fallback at a 0.1 bound from 60% to 48%).  The
        epochs are scaled so that the number of steps stays that of plain
        training.  Returns the loss per epoch."""
        torch = _torch()
        B = self.batch
        n = _r(n, B)
        T, P, Y = states if states is not None else self.sample_states(n, seed)
        n = T.shape[0]
        if n % B:
            raise ValueError("number of states must be a multiple of the batch")
        Yr = Y[: self.N - 1].contiguous()
        W = self.rs.wdot(T, P, Yr, mode="fp64")
        w, _, g = self._serve(T, P, Yr, stol=float("inf"), use_err=False)  # g: log10(D+1e-4)
        e = self.served_error(w, W)
        del W, w
        self.gate_mu = float(g.mean())
        self.gate_sd = max(float(g.std()), 1e-6)
        X = torch.zeros((n, self.net.pad[0]), dtype=torch.bfloat16, device=self.device)
        self.features(T, P, Yr, Yr.stride(0), n, X, box=False)
        X[:, self.n_in] = ((g - self.gate_mu) / self.gate_sd).to(torch.bfloat16)
        idx = torch.arange(n, device=self.device)
        k = int(top * n)
        if k > 0 and copies > 0:
            worst = torch.argsort(e, descending=True)[:k]
            idx = torch.cat([idx] + [worst] * copies)
        gen = torch.Generator(device=self.device).manual_seed(int(seed))
        idx = idx[torch.randperm(idx.numel(), device=self.device, generator=gen)]
        idx = idx[: idx.numel() // B * B]
        n2 = idx.numel()
        Xs = X[idx].contiguous()
        del X
        tgt = torch.log10(e + 1e-4).float()[idx][:, None].contiguous()
        del e, g
        nb = n2 // B
        XT = torch.empty((nb, self.net.pad[0], B), dtype=torch.bfloat16, device=self.device)
        for j in range(nb):
            XT[j].copy_(Xs[j * B:(j + 1) * B].t())
        ep = max(1, int(round(epochs * n / n2)))
        losses = self._train(self.err_net, Xs, XT, tgt, ep, lr, lr_final, seed)
        self.err_trained = True
        return losses

    def gate_scores(self, T, P, Y):
        """(served wdot (N, n), gate score g (n,), error e (n,)) of the
        network path on states labelled here by the exact kernel."""
        Yr = Y[: self.N - 1].contiguous() if Y.shape[0] == self.N else Y
        W = self.rs.wdot(T, P, Yr, mode="fp64")
        w, _, g = self._serve(T, P, Yr, stol=float("inf"))
        return w, g, self.served_error(w, W)

    @staticmethod
    def threshold(g, e, bound):
        """Largest score such that every state scoring at or below it has
        e <= bound (-inf when even the best-scored state exceeds it)."""
        torch = _torch()
        order = torch.argsort(g)
        bad = torch.nonzero(e[order] > bound)
        first = int(bad[0]) if bad.numel() else int(g.numel())
        if first == 0:
            return float("-inf")
        # states tied with the first bad score must not be served
        tau = float(g[order[first - 1]])
        if first < g.numel() and float(g[order[first]]) == tau:
            below = g[order[:first]] < tau
            tau = float(g[order[:first]][below].max()) if bool(below.any()) else float("-inf")
        return tau

    def calibrate(self, bound, n=1 << 22, seed=3, margin=0.5, states=None):
        """Set the gate threshold ``stol`` so that every one of n held-out
        states labelled by the exact kernel that the network would serve has
        e <= margin * bound.  The margin covers the tail of fresh states: a
        threshold calibrated at the bound itself on 2^22 states let errors
        up to 1.65x the bound through on 2^24 fresh ones.  Returns the
        calibration summary."""
        torch = _torch()
        T, P, Y = states if states is not None else self.sample_states(n, seed)
        _, g, e = self.gate_scores(T, P, Y)
        tau = self.threshold(g, e, margin * bound)
        self.stol, self.bound = tau, float(bound)
        served = g <= tau
        return {"bound": float(bound), "margin": float(margin), "stol": tau,
                "states": int(g.numel()),
                "fallback_fraction": 1.0 - float(served.double().mean()),
                "served_max": float(e[served].max()) if bool(served.any()) else 0.0}

    def loss(self, T, P, Y):
        """Mean squared error of the served network output on states
        (exact labels)."""
        W = self.rs.wdot(T, P, Y, mode="fp64")
        Yh = self.predict(T, P, Y)
        return float(((Yh - self.targets(W)) ** 2).mean())

    def predict(self, T, P, Y):
        """Served network outputs (n, N) fp32: the members' mean."""
        torch = _torch()
        n = T.shape[0]
        M = _r(max(n, 1), 128)
        X = torch.zeros((M, self.net.pad[0]), dtype=torch.bfloat16, device=self.device)
        self.features(T, P, Y, Y.stride(0), n, X, box=False)
        acc = None
        for net in self.nets:
            Yh = torch.empty((n, net.pad[-1]), dtype=torch.float32, device=self.device)
            net.infer(X, n, Yh)
            acc = Yh[:, : self.N] if acc is None else acc + Yh[:, : self.N]
        return acc / len(self.nets)

    # -- evaluation ------------------------------------------------------
    def _serve(self, T, P, Y, tol=float("inf"), stol=None, out=None, use_err=True):
        """The network path: (wdot (N, n), fallback flags (n,) uint8, gate
        score (n,)).  Y holds the N - 1 independent mass fractions."""
        torch = _torch()
        n, ld = self.rs._check_states(T, P, Y)
        s = _stream(self.device)
        N = self.N
        if out is None:
            out = torch.empty((N, n), dtype=torch.float64, device=self.device)
        elif out.shape != (N, n) or not out.is_contiguous():
            raise ValueError("out must be a contiguous (species, n) float64 tensor")
        stol = self.stol if stol is None else stol
        f32 = dict(dtype=torch.float32, device=self.device)
        flag = torch.empty(n, dtype=torch.uint8, device=self.device)
        gate = torch.empty(n, **f32)
        if n == 0:
            return out, flag, gate
        M = _r(n, 128)
        X = torch.empty((M, self.net.pad[0]), dtype=torch.bfloat16, device=self.device)
        box = torch.empty(n, dtype=torch.uint8, device=self.device)
        self.features(T, P, Y, ld, n, X, out_of_box=box)
        Yh = [torch.empty((n, net.pad[-1]), **f32) for net in self.nets]
        for net, y in zip(self.nets, Yh):
            net.infer(X, n, y, s)
        est = None
        if use_err and self.err_trained:
            _lib.check(self.lib.crs_surrogate_disagreement(
                n, _p(Yh[0]), _p(Yh[-1]), Yh[0].stride(0), N, self.gate_mu, self.gate_sd,
                _p(X), X.stride(0), self.n_in, s))
            est = torch.empty((n, 4), **f32)
            self.err_net.infer(X, n, est, s)
        _lib.check(self.lib.crs_surrogate_output2(
            n, _p(Yh[0]), _p(Yh[-1]), Yh[0].stride(0), N, _p(self._scale_m), _p(self._scale_e),
            _p(self._cons), self.n_elem, tol, 0.0 if est is not None else 1.0, _p(est),
            est.stride(0) if est is not None else 0, stol, _p(box), _p(out), n, _p(flag),
            _p(gate), s))
        return out, flag, gate

    def wdot(self, T, P, Y, tol=0.05, stol=None, out=None, with_fallback=True):
        """wdot (N, n) for every state: the networks where the gate passes,
        the exact FP64 kernel elsewhere.  ``stol``: gate threshold on the
        error score (default: the calibrated one; infinite before
        ``calibrate``).  Returns (wdot, n_fallback)."""
        torch = _torch()
        out, flag, _ = self._serve(T, P, Y, tol=tol, stol=stol, out=out)
        n = out.shape[1]
        if n == 0:
            return out, 0
        if not with_fallback:
            return out, int(flag.sum())
        s = _stream(self.device)
        N = self.N
        ld = Y.stride(0)
        idx = torch.empty(n, dtype=torch.int64, device=self.device)
        cnt = torch.zeros(1, dtype=torch.int64, device=self.device)
        _lib.check(self.lib.crs_select(n, _p(flag), _p(idx), _p(cnt), s))
        m = int(cnt.item())
        if m:
            f64 = dict(dtype=torch.float64, device=self.device)
            Tc, Pc = torch.empty(m, **f64), torch.empty(m, **f64)
            Yc = torch.empty((N - 1, m), **f64)
            _lib.check(self.lib.crs_gather_states(m, _p(idx), _p(T), _p(P), _p(Y), ld, N - 1,
                                                  _p(Tc), _p(Pc), _p(Yc), m, s))
            Wc = self.rs.wdot(Tc, Pc, Yc, mode="fp64")
            _lib.check(self.lib.crs_scatter_wdot(m, _p(idx), _p(Wc), m, N, _p(out), n, s))
        return out, m

    def save(self, path):
        d = {}
        for j, net in enumerate(self.nets):
            for k, v in net.state_dict().items():
                d["m%d_%s" % (j, k)] = v
        for k, v in self.err_net.state_dict().items():
            d["err_%s" % k] = v
        for k in ("mu", "sd", "lo", "hi", "scale"):
            d[k] = getattr(self, k).cpu().numpy()
        d["history"] = np.array(self.history)
        d["gate"] = np.array([self.stol, np.nan if self.bound is None else self.bound,
                              float(self.err_trained), self.gate_mu, self.gate_sd])
        np.savez(path, **d)

    def load(self, path):
        torch = _torch()
        d = dict(np.load(path))
        for j, net in enumerate(self.nets):
            net.load_state_dict({k[len("m%d_" % j):]: v for k, v in d.items()
                                 if k.startswith("m%d_" % j)})
        self.err_net.load_state_dict({k[4:]: v for k, v in d.items() if k.startswith("err_")})
        for k in ("mu", "sd", "lo", "hi"):
            getattr(self, k).copy_(torch.from_numpy(d[k]))
        self.set_scale(d["scale"])
        self.history = list(d.get("history", []))
        stol, bound, trained, self.gate_mu, self.gate_sd = (float(x) for x in d["gate"])
        self.stol, self.bound = stol, (None if math.isnan(bound) else bound)
        self.err_trained = bool(trained)
