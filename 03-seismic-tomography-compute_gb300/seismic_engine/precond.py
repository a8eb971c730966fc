"""Learned preconditioner for CG on the damped tomography normal equations
(A^T A + lam I) x = A^T b, and the flexible CG that runs it.

The network (no reference counterpart; the reference solves with plain or
Jacobi CG, sparse/sparse_ops.cpp:8-113) maps a residual r on the cell grid to
a correction
    z = dinv * r + s_out * N(s_in r, s_in dinv r),
    N = C_out o (relu(conv_k(h) + h))^K o relu(C_in),
dinv the Jacobi diagonal, s_in = 1 / rms(r), s_out = rms(r) * mean(dinv).
N has no biases, so z scales with r, and C_out starts at zero, so the
untrained network is exactly Jacobi. The K 32 -> 32 layers run on the tensor
cores (st_conv3d_bf16: tcgen05, BF16 operands, FP32 accumulation) forward
and for the input gradient; weight gradients and the 2 -> 32 / 32 -> 1 layers
are CUDA-core kernels (st_precond.cu). Training uses pairs (r_k,
e_k = x* - x_k) taken from plain-CG solves of other systems and minimises
the A-norm error of the correction, ||z_k - e_k||_A^2 / ||e_k||_A^2 =
(z.Az - 2 z.r + e.r) / e.r (A e_k = r_k), the quantity CG itself reduces;
its gradient 2 (A z - r) / e.r needs one operator product per sample. Adam
on FP32 master weights. Flexible CG (one-term A-orthogonalisation)
tolerates the nonlinear preconditioner; the true residual judges
convergence, and plain Jacobi-CG remains the fallback.
"""
from __future__ import annotations

import ctypes as C
import math

import torch

from . import _lib
from ._lib import call

CH = 32


def _p(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


class LearnedPreconditioner:
    def __init__(self, nx: int, ny: int, nz: int, layers: int = 4, seed: int = 0):
        self.shape = (nx, ny, nz)
        self.n = nx * ny * nz
        self.layers = layers
        g = torch.Generator().manual_seed(seed)
        dev = "cuda"
        self.w_in = (torch.randn((CH, 2, 27), generator=g) * math.sqrt(2.0 / 54)).to(dev)
        self.w_k = [(torch.randn((CH, CH, 27), generator=g) * (0.5 * math.sqrt(2.0 / (27 * CH)))).to(dev)
                    for _ in range(layers)]
        self.w_out = torch.zeros((CH, 27), device=dev)
        self.params = [self.w_in, *self.w_k, self.w_out]
        pad = (nx + 2, ny + 2, nz + 2, CH)
        self.h = [torch.zeros(pad, dtype=torch.bfloat16, device=dev) for _ in range(layers + 1)]
        self.dh = torch.zeros(pad, dtype=torch.bfloat16, device=dev)
        self.g = torch.zeros(pad, dtype=torch.bfloat16, device=dev)
        self.packed = [torch.empty(27 * CH * CH, dtype=torch.bfloat16, device=dev) for _ in range(layers)]
        self.packed_t = [torch.empty(27 * CH * CH, dtype=torch.bfloat16, device=dev) for _ in range(layers)]
        self.zhat = torch.zeros(self.n, device=dev)
        self.s_in = torch.zeros(1, device=dev)
        self.s_out = torch.zeros(1, device=dev)
        self._adam = None
        self.pack()

    # ------------------------------------------------------------------ weights
    def _stream(self):
        return C.c_void_p(torch.cuda.current_stream().cuda_stream)

    def pack(self):
        st = self._stream()
        for w, p, pt in zip(self.w_k, self.packed, self.packed_t):
            call("st_conv3d_pack_weights", _p(w), _p(p), 0, st)
            call("st_conv3d_pack_weights", _p(w), _p(pt), 1, st)

    def state_dict(self):
        return {"w_in": self.w_in.cpu(), "w_k": [w.cpu() for w in self.w_k], "w_out": self.w_out.cpu()}

    def load_state_dict(self, sd):
        self.w_in.copy_(sd["w_in"])
        for w, s in zip(self.w_k, sd["w_k"]):
            w.copy_(s)
        self.w_out.copy_(sd["w_out"])
        self.pack()

    # ------------------------------------------------------------------ forward
    def _scales(self, r, dinv):
        rms = torch.sqrt(torch.mean(r.double() ** 2)).float().clamp_min(1e-30)
        self.s_in.copy_((1.0 / rms).reshape(1))
        self.s_out.copy_((rms * dinv.double().mean().float()).reshape(1))

    def forward(self, r, dinv, z=None):
        """zhat = N(r) (kept in self.zhat, activations in self.h); z (optional)
        receives dinv * r + s_out * zhat."""
        nx, ny, nz = self.shape
        st = self._stream()
        self._scales(r, dinv)
        call("st_pc_in_conv", _p(r), _p(dinv), _p(self.s_in), _p(self.w_in), _p(self.h[0]), nx, ny, nz, st)
        for k in range(self.layers):
            call("st_conv3d_bf16", _p(self.h[k]), _p(self.packed[k]), None, _p(self.h[k]), _p(self.h[k + 1]), 0,
                 nx, ny, nz, 1, st)
        call("st_pc_out_conv", _p(self.h[-1]), _p(self.w_out), _p(r), _p(dinv), _p(self.s_out), _p(self.zhat),
             _p(z), nx, ny, nz, st)
        return self.zhat

    __call__ = forward

    # ------------------------------------------------------------------ backward
    def backward(self, dzhat, r, dinv, grads):
        """Accumulates dL/dw into grads (list like self.params) for the
        activations of the last forward."""
        nx, ny, nz = self.shape
        st = self._stream()
        call("st_pc_out_conv_bwd", _p(dzhat), _p(self.h[-1]), _p(self.w_out), _p(self.dh), _p(grads[-1]), nx, ny,
             nz, st)
        for k in range(self.layers, 0, -1):
            call("st_pc_relu_mask", _p(self.dh), _p(self.h[k]), _p(self.g), nx, ny, nz, st)
            call("st_conv3d_wgrad", _p(self.h[k - 1]), _p(self.g), _p(grads[k]), nx, ny, nz, st)
            # dh_{k-1} = conv_k^T(g) + g (the residual connection), tensor cores
            call("st_conv3d_bf16", _p(self.g), _p(self.packed_t[k - 1]), None, _p(self.g), _p(self.dh), 0, nx, ny,
                 nz, 0, st)
        call("st_pc_relu_mask", _p(self.dh), _p(self.h[0]), _p(self.g), nx, ny, nz, st)
        call("st_pc_in_conv_wgrad", _p(r), _p(dinv), _p(self.s_in), _p(self.g), _p(grads[0]), nx, ny, nz, st)

    def check(self):
        call("st_conv3d_check", self._stream())

    # ------------------------------------------------------------------ training
    def a_norm_loss(self, r, e, dinv, op, grads=None, weight=1.0):
        """||z - e||_A^2 / ||e||_A^2 for z = dinv r + s_out N(r), with A e = r
        (so ||e||_A^2 = e.r). With grads, accumulates weight * dL/dw."""
        z = torch.empty_like(r)
        self.forward(r, dinv, z)
        az = op(z, torch.empty_like(r))
        ee = float(torch.dot(e.double(), r.double()))
        loss = (float(torch.dot(z.double(), az.double())) - 2.0 * float(torch.dot(z.double(), r.double())) + ee) / ee
        if grads is not None:
            # dL/dz = 2 (A z - r) / e.r ; dL/dzhat = s_out dL/dz
            dz = (az - r).mul_(2.0 * weight / ee).mul_(self.s_out)
            self.backward(dz, r, dinv, grads)
        return loss

    def train_step(self, batch, lr=1e-3, betas=(0.9, 0.999), eps=1e-8):
        """One Adam step on a list of (r, e, dinv, op) samples (pairs from
        plain-CG solves, op the system's NormalOperator); returns the mean
        A-norm loss before the step."""
        grads = [torch.zeros_like(p) for p in self.params]
        total = 0.0
        for r, e, dinv, op in batch:
            total += self.a_norm_loss(r, e, dinv, op, grads, 1.0 / len(batch))
        if self._adam is None:
            self._adam = {"t": 0, "m": [torch.zeros_like(p) for p in self.params],
                          "v": [torch.zeros_like(p) for p in self.params]}
        a = self._adam
        a["t"] += 1
        b1, b2 = betas
        for p, gr, m, v in zip(self.params, grads, a["m"], a["v"]):
            m.mul_(b1).add_(gr, alpha=1 - b1)
            v.mul_(b2).addcmul_(gr, gr, value=1 - b2)
            mh = m / (1 - b1 ** a["t"])
            vh = v / (1 - b2 ** a["t"])
            p.sub_(lr * mh / (vh.sqrt() + eps))
        self.pack()
        return total / len(batch)


def training_pairs(A, d, lam, iterations=(5, 20, 50, 100, 200, 400), tol=1e-7, max_iter=20000):
    """(r_k, e_k = x* - x_k) pairs from the plain Jacobi-CG solver on one
    system: x* from a solve to tol, x_k after k iterations from x = 0."""
    from .sparse import normal_cg_device
    n = A.cols()
    op = NormalOperator(A, lam)
    rhs = torch.zeros(n, device="cuda")
    A.spmv_device(d, rhs, transpose=True)
    torch.cuda.synchronize()
    xs = torch.zeros(n, device="cuda")
    normal_cg_device(A, d, lam, xs, max_iter, tol, True)
    out = []
    for k in iterations:
        xk = torch.zeros(n, device="cuda")
        it, _, _ = normal_cg_device(A, d, lam, xk, int(k), 1e-30, True)
        if it < k:
            break
        rk = rhs - op(xk, torch.empty_like(xk))
        out.append((rk, xs - xk))
    return op, out


# ---------------------------------------------------------------------- solvers

class NormalOperator:
    """q = (A^T A + lam I) p with the GPU SpMV kernels, on the matrix's stream."""

    def __init__(self, A, lam):
        self.A = A
        self.lam = float(lam)
        self.t = torch.zeros(A.rows(), device="cuda")
        self.stream = torch.cuda.ExternalStream(A.stream_ptr())

    def __call__(self, p, q):
        torch.cuda.current_stream().synchronize()
        self.A.spmv_device(p, self.t)
        self.A.spmv_device(self.t, q, transpose=True)
        torch.cuda.synchronize()
        q.add_(p, alpha=self.lam)
        return q

    def jacobi(self):
        d = torch.zeros(self.A.cols(), device="cuda")
        call("st_csr_normal_jacobi", self.A.handle, self.lam, _p(d))
        torch.cuda.synchronize()
        return d


def flexible_cg(op: NormalOperator, rhs, precond=None, dinv=None, tol=1e-6, max_iter=10000, x=None):
    """Flexible CG (one-term A-orthogonalisation of the search directions),
    FP64 scalars, stopping on the true residual ||rhs - op(x)|| / ||rhs||
    (recomputed every 50 iterations and at the end). precond(r, z) fills z;
    None = Jacobi with dinv. Returns (x, iterations, true relative residual)."""
    n = rhs.numel()
    x = torch.zeros(n, device="cuda") if x is None else x
    r = rhs.clone() if not x.any() else rhs - op(x, torch.zeros_like(rhs))
    bn = float(torch.linalg.norm(rhs.double()))
    if bn == 0.0:
        return x, 0, 0.0
    z = torch.zeros_like(rhs)
    q = torch.zeros_like(rhs)

    def apply(r_, z_):
        if precond is None:
            torch.mul(dinv, r_, out=z_)
        else:
            precond(r_, dinv, z_)

    def apply_safe(r_, z_):
        # a preconditioned direction that is not a descent direction falls back to Jacobi
        apply(r_, z_)
        if precond is not None and float(torch.dot(z_.double(), r_.double())) <= 0.0:
            torch.mul(dinv, r_, out=z_)

    apply_safe(r, z)
    p = z.clone()
    op(p, q)
    it = 0
    rel = 1.0
    while it < max_iter:
        pq = float(torch.dot(p.double(), q.double()))
        if abs(pq) < 1e-300:
            break
        alpha = float(torch.dot(p.double(), r.double())) / pq
        x.add_(p, alpha=alpha)
        r.add_(q, alpha=-alpha)
        it += 1
        rel = float(torch.linalg.norm(r.double())) / bn
        if rel <= tol or it % 50 == 0:
            true = rhs - op(x, torch.zeros_like(rhs))
            rel = float(torch.linalg.norm(true.double())) / bn
            r.copy_(true)
            if rel <= tol:
                break
        apply_safe(r, z)
        beta = float(torch.dot(z.double(), q.double())) / pq
        p.mul_(-beta).add_(z)
        op(p, q)
    return x, it, rel
