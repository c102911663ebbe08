"""CPU oracle of the learned predictor's network (test infrastructure only).

numpy restatement of the library's multilayer perceptron (vefem_mlp_* in
include/vefem.h): layers in -> width (GELU, erf form) x hidden -> out,
weights rounded to BF16 (nearest even) in the products, FP32 activations,
mean squared error, full-batch Adam (beta1 0.9, beta2 0.999, eps 1e-8).  The
network has no counterpart in the reference, whose arclength predictor is the
tangent step of updateSolutionArclength (Continuation_Arclength_mod.F90:339-379);
the tests check the GPU forward pass, the gradients of the GPU backward
kernels and the Adam update against this file.  Products accumulate in
float64 here, so the tests compare with a tolerance.
"""
from __future__ import annotations

import numpy as np
from scipy.special import erf


def bf16_round(a: np.ndarray) -> np.ndarray:
    """Round float32 values to the nearest BF16 (ties to even), as float32."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


class MLPRef:
    def __init__(self, in_dim: int, out_dim: int, width: int = 256, hidden: int = 3):
        self.dims = [in_dim] + [width] * hidden + [out_dim]
        self.layers = [(self.dims[i], self.dims[i + 1]) for i in range(hidden + 1)]
        self.n_params = sum(i * o + o for i, o in self.layers)
        self.params = np.zeros(self.n_params, np.float32)
        self.m = np.zeros(self.n_params, np.float64)
        self.v = np.zeros(self.n_params, np.float64)
        self.t = 0

    def init_params(self, seed: int):
        """The library's initialisation: weights uniform in +-sqrt(1/in) from a
        64-bit linear congruential stream, biases zero."""
        M = (1 << 64) - 1
        A, C = 6364136223846793005, 1442695040888963407
        st = (seed * A + C) & M
        parts = []
        for i, n in self.layers:
            w = np.empty(i * n, np.float64)
            bound = np.sqrt(1.0 / i)
            for k in range(i * n):
                st = (st * A + C) & M
                w[k] = (2.0 * ((st >> 11) * (1.0 / 9007199254740992.0)) - 1.0) * bound
            parts += [w.astype(np.float32), np.zeros(n, np.float32)]
        self.params = np.concatenate(parts)
        return self.params

    def reset_optimizer(self):
        self.m[:] = 0.0
        self.v[:] = 0.0
        self.t = 0

    def get_params(self):
        return self.params.copy()

    def set_params(self, p):
        self.params = np.asarray(p, np.float32).copy()

    def unpack(self, p=None):
        p = self.params if p is None else p
        out, o = [], 0
        for i, n in self.layers:
            W = p[o:o + i * n].reshape(n, i)
            o += i * n
            b = p[o:o + n]
            o += n
            out.append((W, b))
        return out

    @staticmethod
    def gelu(z):
        return 0.5 * z * (1.0 + erf(z / np.sqrt(2.0)))

    @staticmethod
    def gelu_prime(z):
        return 0.5 * (1.0 + erf(z / np.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / np.sqrt(2.0 * np.pi)

    def forward(self, X, keep=False):
        a = np.asarray(X, np.float64)
        cache = []
        L = self.unpack()
        for k, (W, b) in enumerate(L):
            Wb = bf16_round(W).astype(np.float64)
            z = a @ Wb.T + b.astype(np.float64)
            cache.append((a, z, Wb))
            a = self.gelu(z) if k + 1 < len(L) else z
        return (a, cache) if keep else a

    def loss_grad(self, X, T):
        Y, cache = self.forward(X, keep=True)
        T = np.asarray(T, np.float64)
        cnt = Y.size
        loss = float(np.sum((Y - T) ** 2) / cnt)
        d = 2.0 * (Y - T) / cnt
        grads = []
        for k in range(len(cache) - 1, -1, -1):
            a, z, Wb = cache[k]
            if k + 1 < len(cache):
                d = d * self.gelu_prime(z)
            grads.append((d.T @ a, d.sum(axis=0)))
            d = d @ Wb
        grads.reverse()
        g = np.concatenate([np.concatenate([gW.reshape(-1), gb]) for gW, gb in grads])
        return loss, g

    def adam_step(self, X, T, lr=1e-3):
        loss, g = self.loss_grad(X, T)
        b1, b2, eps = 0.9, 0.999, 1e-8
        self.t += 1
        self.m = b1 * self.m + (1 - b1) * g
        self.v = b2 * self.v + (1 - b2) * g * g
        mh = self.m / (1 - b1 ** self.t)
        vh = self.v / (1 - b2 ** self.t)
        self.params = (self.params - lr * mh / (np.sqrt(vh) + eps)).astype(np.float32)
        return loss

    def train(self, X, T, iters, lr=1e-3):
        loss = None
        for _ in range(iters):
            loss = self.adam_step(X, T, lr)
        return loss
