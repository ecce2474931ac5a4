"""MLP on the project's own kernels: FP32 training (forward, backward, Adam)
and BF16 inference.  Weights are (in, out) row-major; y = GELU(x W + b)
between hidden layers, linear output."""
from __future__ import annotations

import numpy as np

from .. import _lib
from ..device import ptr, require_cuda, stream_handle


class MLP:
    def __init__(self, sizes=(20, 128, 128, 128, 3), seed=0):
        t = require_cuda()
        self.t = t
        self.sizes = tuple(int(s) for s in sizes)
        rng = np.random.default_rng(seed)
        self.W, self.b = [], []
        for i in range(len(self.sizes) - 1):
            fan_in, fan_out = self.sizes[i], self.sizes[i + 1]
            w = rng.standard_normal((fan_in, fan_out)) * np.sqrt(2.0 / fan_in)
            if i == len(self.sizes) - 2:
                w *= 0.1
            self.W.append(t.from_numpy(w.astype(np.float32)).cuda())
            self.b.append(t.zeros(fan_out, device="cuda"))
        self.params = self.W + self.b
        self.m = [t.zeros_like(p) for p in self.params]
        self.v = [t.zeros_like(p) for p in self.params]
        self.step_count = 0
        self.lib = _lib.load()
        self._bf16 = None

    @property
    def n_layers(self):
        return len(self.W)

    # -- training ------------------------------------------------------------
    def forward(self, X):
        """X: CUDA float32 (B, F).  Returns y (B, out) and keeps the tape."""
        t = self.t
        X = X.contiguous()
        B = X.shape[0]
        self._inputs, self._pre = [], []
        h = X
        for i in range(self.n_layers):
            fi, fo = self.sizes[i], self.sizes[i + 1]
            last = i == self.n_layers - 1
            out = t.empty((B, fo), device="cuda")
            pre = None if last else t.empty((B, fo), device="cuda")
            _lib.check(self.lib.mlp_gemm(0, 0, B, fo, fi, ptr(h), fi, ptr(self.W[i]), fo, ptr(out), fo,
                                         ptr(self.b[i]), 0 if last else 1, ptr(pre), 0, stream_handle()))
            self._inputs.append(h)
            self._pre.append(pre)
            h = out
        return h

    def backward(self, dy):
        """Gradients of the loss w.r.t. every parameter (list, like self.params)."""
        t = self.t
        B = dy.shape[0]
        gW = [None] * self.n_layers
        gb = [None] * self.n_layers
        d = dy.contiguous()
        for i in reversed(range(self.n_layers)):
            fi, fo = self.sizes[i], self.sizes[i + 1]
            if self._pre[i] is not None:
                dz = t.empty_like(d)
                _lib.check(self.lib.mlp_gelu_backward(ptr(d), ptr(self._pre[i]), ptr(dz), d.numel(),
                                                      stream_handle()))
            else:
                dz = d
            x = self._inputs[i]
            gW[i] = t.empty((fi, fo), device="cuda")
            _lib.check(self.lib.mlp_gemm(1, 0, fi, fo, B, ptr(x), fi, ptr(dz), fo, ptr(gW[i]), fo, None, 0,
                                         None, 0, stream_handle()))
            gb[i] = t.empty(fo, device="cuda")
            _lib.check(self.lib.mlp_bias_grad(ptr(dz), B, fo, ptr(gb[i]), stream_handle()))
            if i > 0:
                dx = t.empty((B, fi), device="cuda")
                _lib.check(self.lib.mlp_gemm(0, 1, B, fi, fo, ptr(dz), fo, ptr(self.W[i]), fo, ptr(dx), fi,
                                             None, 0, None, 0, stream_handle()))
                d = dx
        return gW + gb

    def loss(self, y, target, col_weight=None):
        t = self.t
        dy = t.empty_like(y)
        out = t.empty(1, device="cuda")
        w = None if col_weight is None else t.as_tensor(col_weight, dtype=t.float32, device="cuda")
        _lib.check(self.lib.mlp_mse_loss(ptr(y), ptr(target), ptr(w), y.numel(), y.shape[1], ptr(dy), ptr(out),
                                         stream_handle()))
        return out, dy

    def adam(self, grads, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8, weight_decay=0.0):
        self.step_count += 1
        for p, g, m, v in zip(self.params, grads, self.m, self.v):
            _lib.check(self.lib.mlp_adam_step(ptr(p), ptr(g), ptr(m), ptr(v), p.numel(), lr, beta1, beta2, eps,
                                              self.step_count, weight_decay, stream_handle()))
        self._bf16 = None

    def fit(self, X, Y, epochs=400, batch=256, lr=2e-3, col_weight=None, seed=0, lr_decay=0.995,
            weight_decay=1e-4, verbose=False):
        """Minibatch Adam on host arrays X (N, F), Y (N, out); returns the loss curve."""
        t = self.t
        Xd = t.from_numpy(np.ascontiguousarray(X, np.float32)).cuda()
        Yd = t.from_numpy(np.ascontiguousarray(Y, np.float32)).cuda()
        rng = np.random.default_rng(seed)
        N = X.shape[0]
        curve = []
        for ep in range(epochs):
            order = t.from_numpy(rng.permutation(N)).cuda()
            tot = 0.0
            for s in range(0, N, batch):
                idx = order[s:s + batch]
                y = self.forward(Xd[idx])
                l, dy = self.loss(y, Yd[idx].contiguous(), col_weight)
                self.adam(self.backward(dy), lr=lr, weight_decay=weight_decay)
                tot += float(l.item()) * idx.numel()
            lr *= lr_decay
            curve.append(tot / N)
            if verbose and ep % 50 == 0:
                print(f"epoch {ep} loss {curve[-1]:.5f}")
        return np.asarray(curve)

    # -- inference -----------------------------------------------------------
    def predict(self, X):
        """FP32 forward on host inputs -> host outputs."""
        t = self.t
        return self.forward(t.from_numpy(np.ascontiguousarray(X, np.float32)).cuda()).cpu().numpy()

    def predict_bf16(self, X):
        """BF16 inference: weights and layer inputs rounded to bfloat16,
        FP32 accumulation and bias/GELU epilogue."""
        t = self.t
        if self._bf16 is None:
            self._bf16 = []
            for W in self.W:
                wb = t.empty(W.shape, dtype=t.bfloat16, device="cuda")
                _lib.check(self.lib.mlp_to_bf16(ptr(W), ptr(wb), W.numel(), stream_handle()))
                self._bf16.append(wb)
        h = t.from_numpy(np.ascontiguousarray(X, np.float32)).cuda()
        B = h.shape[0]
        for i in range(self.n_layers):
            fi, fo = self.sizes[i], self.sizes[i + 1]
            hb = t.empty((B, fi), dtype=t.bfloat16, device="cuda")
            _lib.check(self.lib.mlp_to_bf16(ptr(h), ptr(hb), h.numel(), stream_handle()))
            out = t.empty((B, fo), device="cuda")
            last = i == self.n_layers - 1
            _lib.check(self.lib.mlp_gemm_bf16(0, 0, B, fo, fi, ptr(hb), fi, ptr(self._bf16[i]), fo, ptr(out), fo,
                                              ptr(self.b[i]), 0 if last else 1, stream_handle()))
            h = out
        return h.cpu().numpy()

    # -- persistence ---------------------------------------------------------
    def state(self):
        return {f"W{i}": W.cpu().numpy() for i, W in enumerate(self.W)} | \
            {f"b{i}": b.cpu().numpy() for i, b in enumerate(self.b)} | {"sizes": np.asarray(self.sizes)}

    def save(self, path, **extra):
        np.savez_compressed(path, **self.state(), **extra)

    @classmethod
    def load(cls, path):
        d = np.load(path)
        m = cls(tuple(int(s) for s in d["sizes"]))
        t = m.t
        for i in range(m.n_layers):
            m.W[i].copy_(t.from_numpy(d[f"W{i}"]))
            m.b[i].copy_(t.from_numpy(d[f"b{i}"]))
        return m, {k: d[k] for k in d.files if not k[0] in "Wb" and k != "sizes"}
