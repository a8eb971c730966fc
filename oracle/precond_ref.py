"""CPU oracle of the learned CG preconditioner network (TEST INFRASTRUCTURE
ONLY: the product never imports this file).

Restates in numpy FP64 the preconditioner the GPU layers compute
(seismic_engine/precond.py, csrc/st_precond.cu, csrc/st_conv.cu):
    z = D r + S G^T G S r,  G = (I + conv_K)...(I + conv_1) C^T,
D = diag(dinv), S = sqrt(D), input scaled by 1 / rms(r) and output back;
3x3x3 convolutions with zero padding, tap = (kd*3 + kh)*3 + kw, weights
[out][in][27]. With bf16_storage the BF16 storage of the GPU path is
emulated (activations, their gradients and the tensor-core layers' weights
rounded to BF16, round-to-nearest-even), leaving FP32-vs-FP64 accumulation
as the only difference. The network is new in this project (the reference has no
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
    """z = D r + S G^T G S r, G = (I + conv_K)...(I + conv_1) C^T (see the
    module docstring of seismic_engine/precond.py)."""

    def __init__(self, w_c, w_k, bf16_storage=True):
        self.q = bf16 if bf16_storage else (lambda a: np.asarray(a, np.float64))
        self.w_c = np.asarray(w_c, np.float64)[None]  # (1, 32, 27)
        self.w_k = [self.q(np.asarray(w, np.float64)) for w in w_k]

    def forward(self, r, dinv, shape):
        q = self.q
        r = np.asarray(r, np.float64).reshape(shape)
        dinv = np.asarray(dinv, np.float64).reshape(shape)
        s = 1.0 / np.sqrt(np.mean(np.float32(r).astype(np.float64) ** 2))
        sq = np.sqrt(dinv)
        a = (s * sq * r)[None]
        u = [q(conv_t(a, self.w_c))]
        for w in self.w_k:
            u.append(q(u[-1] + conv(u[-1], w)))
        v = [None] * len(self.w_k) + [u[-1]]
        for k in range(len(self.w_k), 0, -1):
            v[k - 1] = q(v[k] + conv_t(v[k], self.w_k[k - 1]))
        y = conv(v[0], self.w_c)[0]
        self.cache = (a, u, v, sq, s)
        return (dinv * r + sq * y / s).reshape(-1)

    def backward(self, dz, shape):
        q = self.q
        a, u, v, sq, s = self.cache
        dy = (sq * np.asarray(dz, np.float64).reshape(shape) / s)[None]
        d_c = wgrad(v[0], dy)[0]
        d = q(conv_t(dy, self.w_c))
        d_k = [np.zeros_like(w) for w in self.w_k]
        for k in range(1, len(self.w_k) + 1):
            d_k[k - 1] += wgrad(d, v[k])
            d = q(d + conv(d, self.w_k[k - 1]))
        for k in range(len(self.w_k), 0, -1):
            d_k[k - 1] += wgrad(u[k - 1], d)
            d = q(d + conv_t(d, self.w_k[k - 1]))
        d_c = d_c + wgrad(d, a)[0]
        return d_c, d_k
