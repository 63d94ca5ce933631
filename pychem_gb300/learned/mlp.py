"""The pair network: 40 -> 256 -> 256 -> 256 -> 29, SiLU, BF16 weights used by the
GEMMs with FP32 accumulation and FP32 master weights for Adam.  Forward and backward
run on the library's kernels (pcg_mlp_*)."""
import ctypes

import numpy as np
import torch

from .. import _lib
from .blocks import NFEAT, NPARAM

DIMS = [NFEAT, 256, 256, 256, NPARAM]


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _s():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class PairMLP:
    def __init__(self, device="cuda", seed=0, dims=DIMS):
        self.dims = list(dims)
        self.dev = torch.device(device)
        g = torch.Generator().manual_seed(seed)
        self.W, self.b = [], []
        for k in range(len(dims) - 1):
            fan_in = dims[k]
            w = torch.randn(dims[k], dims[k + 1], generator=g) * (2.0 / fan_in) ** 0.5
            if k == len(dims) - 2:
                w *= 0.1
            self.W.append(w.to(self.dev))
            self.b.append(torch.zeros(dims[k + 1], device=self.dev))
        self.refresh_bf16()
        self.mW = [torch.zeros_like(w) for w in self.W]
        self.vW = [torch.zeros_like(w) for w in self.W]
        self.mb = [torch.zeros_like(b) for b in self.b]
        self.vb = [torch.zeros_like(b) for b in self.b]
        self.step_count = 0
        self.mean = torch.zeros(NPARAM, device=self.dev)
        self.std = torch.ones(NPARAM, device=self.dev)

    def refresh_bf16(self):
        self.Wb = [w.to(torch.bfloat16).contiguous() for w in self.W]

    @property
    def nlayers(self):
        return len(self.W)

    def forward(self, X, keep=False):
        """X (M, NFEAT) float32 -> (M, NPARAM) normalised outputs."""
        M = X.shape[0]
        A = X.contiguous()
        cache = []
        for k in range(self.nlayers):
            K, N = self.dims[k], self.dims[k + 1]
            act = 1 if k < self.nlayers - 1 else 0
            C = torch.empty(M, N, dtype=torch.float32, device=self.dev)
            Z = torch.empty(M, N, dtype=torch.float32, device=self.dev) if (keep and act) else None
            _lib.call("pcg_mlp_gemm", M, N, K, _p(A), K, 1, _p(self.Wb[k]), 1, N, 1, _p(C), N, 0, _p(self.b[k]),
                      _p(Z), act, _s())
            cache.append((A, Z))
            A = C
        return A, cache

    def backward(self, dY, cache):
        """Gradients (dW, db) per layer for output gradient dY (M, NPARAM)."""
        M = dY.shape[0]
        G = dY.contiguous()
        grads = [None] * self.nlayers
        for k in reversed(range(self.nlayers)):
            K, N = self.dims[k], self.dims[k + 1]
            A, Z = cache[k]
            if Z is not None:
                _lib.call("pcg_mlp_dsilu", M * N, _p(G), _p(Z), _s())
            dW = torch.empty(K, N, dtype=torch.float32, device=self.dev)
            _lib.call("pcg_mlp_gemm", K, N, M, _p(A), 1, K, _p(G), 0, N, 1, _p(dW), N, 0, None, None, 0, _s())
            db = torch.empty(N, dtype=torch.float32, device=self.dev)
            _lib.call("pcg_mlp_colsum", M, N, _p(G), _p(db), _s())
            grads[k] = (dW, db)
            if k > 0:
                dA = torch.empty(M, K, dtype=torch.float32, device=self.dev)
                _lib.call("pcg_mlp_gemm", M, K, N, _p(G), N, 1, _p(self.Wb[k]), 1, 1, N, _p(dA), K, 0, None, None, 0,
                          _s())
                G = dA
        return grads

    def loss_grad(self, Y, T, mask):
        n = Y.numel()
        cnt = float(mask.sum())
        dY = torch.empty_like(Y)
        loss = torch.zeros(1, dtype=torch.float32, device=self.dev)
        _lib.call("pcg_mlp_mse", n, _p(Y), _p(T), _p(mask), ctypes.c_float(1.0 / max(cnt, 1.0)), _p(dY), _p(loss),
                  _s())
        return loss, dY

    def adam(self, grads, lr, b1=0.9, b2=0.999, eps=1e-8):
        self.step_count += 1
        for k, (dW, db) in enumerate(grads):
            _lib.call("pcg_mlp_adam", self.W[k].numel(), _p(self.W[k]), _p(dW), _p(self.mW[k]), _p(self.vW[k]),
                      _p(self.Wb[k]), ctypes.c_float(lr), ctypes.c_float(b1), ctypes.c_float(b2), ctypes.c_float(eps),
                      self.step_count, _s())
            _lib.call("pcg_mlp_adam", self.b[k].numel(), _p(self.b[k]), _p(db), _p(self.mb[k]), _p(self.vb[k]), None,
                      ctypes.c_float(lr), ctypes.c_float(b1), ctypes.c_float(b2), ctypes.c_float(eps), self.step_count,
                      _s())

    def predict(self, X):
        Y, _ = self.forward(X)
        return Y * self.std + self.mean

    def state(self):
        d = {"dims": np.array(self.dims), "mean": self.mean.cpu().numpy(), "std": self.std.cpu().numpy()}
        for k in range(self.nlayers):
            d["W%d" % k] = self.W[k].cpu().numpy()
            d["b%d" % k] = self.b[k].cpu().numpy()
        return d

    def save(self, path, **extra):
        np.savez_compressed(path, **self.state(), **extra)

    @classmethod
    def load(cls, path, device="cuda"):
        z = np.load(path)
        net = cls(device=device, dims=[int(x) for x in z["dims"]])
        for k in range(net.nlayers):
            net.W[k] = torch.as_tensor(z["W%d" % k], device=net.dev)
            net.b[k] = torch.as_tensor(z["b%d" % k], device=net.dev)
        net.refresh_bf16()
        net.mean = torch.as_tensor(z["mean"], device=net.dev)
        net.std = torch.as_tensor(z["std"], device=net.dev)
        return net
