"""The join-proposal MLP (32-256-256-128-1, ReLU) on the project's own BF16
tensor-core kernels (csrc/mlp.cu): forward, backward and Adam, with FP32
master weights and FP32 accumulation.  No reference counterpart: this is
the learned proposal that orders the candidate joins of a search pass."""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import native

DIMS = (32, 256, 256, 128, 1)


def _lib():
    L = native.lib()
    vp, i32, i64, f32 = C.c_void_p, C.c_int32, C.c_int64, C.c_float
    L.poyd_gemm_bf16.argtypes = [vp, i32, i32, vp, i32, i32, i32, i32, i32, vp, i32, vp, vp,
                                 i32, i32, vp]
    L.poyd_relu_grad_bf16.argtypes = [vp, vp, vp, i64, vp]
    L.poyd_colsum_bf16.argtypes = [vp, i32, i32, vp, vp]
    L.poyd_mlp_head_forward.argtypes = [vp, vp, vp, i32, i32, vp, vp]
    L.poyd_mlp_head_backward.argtypes = [vp, vp, vp, vp, i32, i32, vp, vp, vp, vp, vp]
    L.poyd_adam_step.argtypes = [vp, vp, vp, vp, vp, i64, f32, f32, f32, f32, i32, vp]
    L.poyd_to_bf16.argtypes = [vp, vp, i64, vp]
    return L


def _p(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _st():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


class MLP:
    """Parameters: W_l [in, out] row-major (fp32 master + bf16 copy), b_l fp32."""

    def __init__(self, seed: int = 0, device="cuda"):
        self.dev = torch.device(device)
        rng = np.random.default_rng(seed)
        self.W, self.W16, self.b = [], [], []
        for i in range(4):
            fan_in, fan_out = DIMS[i], DIMS[i + 1]
            w = rng.normal(0, np.sqrt(2.0 / fan_in), size=(fan_in, fan_out)).astype(np.float32)
            self.W.append(torch.from_numpy(w).to(self.dev))
            self.b.append(torch.zeros(fan_out, dtype=torch.float32, device=self.dev))
        self.W16 = [w.to(torch.bfloat16) for w in self.W]
        self.mW = [torch.zeros_like(w) for w in self.W]
        self.vW = [torch.zeros_like(w) for w in self.W]
        self.mb = [torch.zeros_like(b) for b in self.b]
        self.vb = [torch.zeros_like(b) for b in self.b]
        self.steps = 0
        self.L = _lib()

    def state(self):
        return {"W": [w.cpu().numpy() for w in self.W], "b": [b.cpu().numpy() for b in self.b]}

    def _gemm(self, A, tA, lda, B, tB, ldb, M, N, K, bias=None, relu=False, c32=None, c16=None,
              ldc=None, acc=False):
        native.check(self.L.poyd_gemm_bf16(_p(A), lda, tA, _p(B), ldb, tB, M, N, K, _p(bias),
                                           int(relu), _p(c32), _p(c16), ldc, int(acc), _st()))

    def forward(self, X16: torch.Tensor):
        """X16 [B, 32] bf16 -> predictions [B] fp32 (activations kept)."""
        B = X16.shape[0]
        self.X16 = X16
        self.H = []
        a = X16
        for i in range(3):
            K, N = DIMS[i], DIMS[i + 1]
            h = torch.empty((B, N), dtype=torch.bfloat16, device=self.dev)
            self._gemm(a, 0, K, self.W16[i], 0, N, B, N, K, bias=self.b[i], relu=True, c16=h,
                       ldc=N)
            self.H.append(h)
            a = h
        y = torch.empty(B, dtype=torch.float32, device=self.dev)
        native.check(self.L.poyd_mlp_head_forward(_p(a), _p(self.W16[3]), _p(self.b[3]), B,
                                                  DIMS[3], _p(y), _st()))
        self.y = y
        return y

    def backward(self, target: torch.Tensor):
        """Gradients of mean squared error; returns (loss, gW list, gb list)."""
        B = self.X16.shape[0]
        gW = [torch.empty_like(w) for w in self.W]
        gb = [torch.empty_like(b) for b in self.b]
        loss = torch.zeros(1, dtype=torch.float32, device=self.dev)
        dZ = torch.empty((B, DIMS[3]), dtype=torch.bfloat16, device=self.dev)
        native.check(self.L.poyd_mlp_head_backward(_p(self.H[2]), _p(self.W16[3]), _p(self.y),
                                                   _p(target), B, DIMS[3], _p(dZ),
                                                   _p(gW[3]), _p(gb[3]), _p(loss), _st()))
        for i in (2, 1, 0):
            K, N = DIMS[i], DIMS[i + 1]
            a_in = self.X16 if i == 0 else self.H[i - 1]
            # dW_i = a_in^T dZ  ([K, N], reduction over the batch)
            self._gemm(a_in, 1, K, dZ, 0, N, K, N, B, c32=gW[i], ldc=N)
            native.check(self.L.poyd_colsum_bf16(_p(dZ), B, N, _p(gb[i]), _st()))
            if i > 0:
                dH = torch.empty((B, K), dtype=torch.bfloat16, device=self.dev)
                # dH = dZ W_i^T  ([B, K])
                self._gemm(dZ, 0, N, self.W16[i], 1, N, B, K, N, c16=dH, ldc=K)
                dZn = torch.empty_like(dH)
                native.check(self.L.poyd_relu_grad_bf16(_p(dH), _p(self.H[i - 1]), _p(dZn),
                                                        dH.numel(), _st()))
                dZ = dZn
        return loss, gW, gb

    def step(self, gW, gb, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        self.steps += 1
        for i in range(4):
            native.check(self.L.poyd_adam_step(_p(self.W[i]), _p(self.W16[i]), _p(gW[i]),
                                               _p(self.mW[i]), _p(self.vW[i]), self.W[i].numel(),
                                               lr, b1, b2, eps, self.steps, _st()))
            native.check(self.L.poyd_adam_step(_p(self.b[i]), None, _p(gb[i]), _p(self.mb[i]),
                                               _p(self.vb[i]), self.b[i].numel(), lr, b1, b2, eps,
                                               self.steps, _st()))

    def fit(self, X: torch.Tensor, y: torch.Tensor, epochs=3, batch=4096, lr=1e-3, seed=0):
        """Mini-batch Adam on (X fp32 [n, 32], y fp32 [n]); returns losses."""
        g = torch.Generator(device="cpu").manual_seed(seed)
        n = X.shape[0]
        X16 = X.to(torch.bfloat16)
        losses = []
        for _ in range(epochs):
            perm = torch.randperm(n, generator=g).to(self.dev)
            for s in range(0, n - batch + 1, batch):
                idx = perm[s:s + batch]
                self.forward(X16[idx].contiguous())
                loss, gW, gb = self.backward(y[idx].contiguous())
                self.step(gW, gb, lr=lr)
                losses.append(loss)
        return [float(l.item()) for l in losses[-10:]]

    def predict(self, X: torch.Tensor) -> torch.Tensor:
        """Predictions for the rows of X (fp32 [n, 32]) in one fused launch
        (``poyd_mlp_forward``), equal to ``forward``'s."""
        X16 = X.to(torch.bfloat16).contiguous()
        y = torch.empty(X16.shape[0], dtype=torch.float32, device=self.dev)
        if X16.shape[0] == 0:
            return y
        Wt = [w.t().contiguous() for w in self.W16[:3]]
        native.check(self.L.poyd_mlp_forward(_p(X16), X16.shape[0], _p(Wt[0]), _p(self.b[0]),
                                             _p(Wt[1]), _p(self.b[1]), _p(Wt[2]), _p(self.b[2]),
                                             _p(self.W16[3]), _p(self.b[3]), _p(y), _st()))
        return y
