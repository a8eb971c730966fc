"""CPU oracle of the learned CG preconditioner network (TEST INFRASTRUCTURE
ONLY: the product never imports this file).

Restates in numpy FP64 the network the GPU layers compute
(seismic_engine/precond.py, csrc/st_precond.cu, csrc/st_conv.cu):
    h0 = relu(C_in([s r, s dinv r])),  h_k = relu(conv_k(h_{k-1}) + h_{k-1}),
    zhat = C_out(h_K),  z = dinv r + s_out zhat,
3x3x3 convolutions with zero padding, tap = (kd*3 + kh)*3 + kw, weights
[out][in][27]. With bf16=True the BF16 storage of the GPU path is emulated
(activations, their gradients and the tensor-core layers' weights rounded to
BF16, round-to-nearest-even), leaving FP32-vs-FP64 accumulation as the only
difference. The network is new in this project (the reference has no
learned preconditioner), so parity here is against this restatement.
"""
from __future__ import annotations

import numpy as np

TAPS = [(kd - 1, kh - 1, kw - 1) for kd in range(3) for kh in range(3) for kw in range(3)]


def bf16(a):
    """Round to BF16 (nearest even) and back to FP64."""
    f = np.ascontiguousarray(a, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return u.view(np.float32).astype(np.float64)


def shift(x, d):
    """y[..., i] = x[..., i + d] with zeros outside (x: (..., D, H, W))."""
    out = np.zeros_like(x)
    sl_out, sl_in = [], []
    for ax, s in enumerate(d):
        n = x.shape[-3 + ax]
        if s >= 0:
            sl_out.append(slice(0, n - s))
            sl_in.append(slice(s, n))
        else:
            sl_out.append(slice(-s, n))
            sl_in.append(slice(0, n + s))
    out[(Ellipsis, *sl_out)] = x[(Ellipsis, *sl_in)]
    return out


def conv(x, w):
    """x (Ci, D, H, W), w (Co, Ci, 27) -> (Co, D, H, W)."""
    out = np.zeros((w.shape[0],) + x.shape[1:])
    for t, d in enumerate(TAPS):
        out += np.einsum("oi,idhw->odhw", w[:, :, t], shift(x, d))
    return out


def conv_t(g, w):
    """Adjoint of conv: g (Co, D, H, W) -> (Ci, D, H, W)."""
    out = np.zeros((w.shape[1],) + g.shape[1:])
    for t, d in enumerate(TAPS):
        out += shift(np.einsum("oi,odhw->idhw", w[:, :, t], g), tuple(-s for s in d))
    return out


def wgrad(x, g):
    """dL/dw for conv(x, w) with output gradient g: (Co, Ci, 27)."""
    return np.stack([np.einsum("odhw,idhw->oi", g, shift(x, d)) for d in TAPS], axis=-1)


class Net:
    def __init__(self, w_in, w_k, w_out, bf16_storage=True):
        self.w_in = np.asarray(w_in, np.float64)
        self.w_out = np.asarray(w_out, np.float64)
        self.q = bf16 if bf16_storage else (lambda a: np.asarray(a, np.float64))
        self.w_k = [self.q(np.asarray(w, np.float64)) for w in w_k]

    def forward(self, r, dinv, shape):
        D, H, W = shape
        r = np.asarray(r, np.float64).reshape(D, H, W)
        dinv = np.asarray(dinv, np.float64).reshape(D, H, W)
        s = 1.0 / np.sqrt(np.mean(np.float32(r) ** 2))
        x = np.stack([s * r, s * dinv * r])
        h = [self.q(np.maximum(conv(x, self.w_in), 0.0))]
        for w in self.w_k:
            h.append(self.q(np.maximum(conv(h[-1], w) + h[-1], 0.0)))
        zhat = conv(h[-1], self.w_out[None])[0]
        self.cache = (x, h)
        return zhat.reshape(-1)

    def backward(self, dzhat, shape):
        x, h = self.cache
        dz = np.asarray(dzhat, np.float64).reshape((1,) + tuple(shape))
        d_out = wgrad(h[-1], dz)[0]
        dh = self.q(conv_t(dz, self.w_out[None]))
        d_k = [None] * len(self.w_k)
        for k in range(len(self.w_k), 0, -1):
            g = self.q(dh * (h[k] > 0))
            d_k[k - 1] = wgrad(h[k - 1], g)
            dh = self.q(conv_t(g, self.w_k[k - 1]) + g)
        g0 = self.q(dh * (h[0] > 0))
        d_in = wgrad(x, g0)
        return d_in, d_k, d_out
