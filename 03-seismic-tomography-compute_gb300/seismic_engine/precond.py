"""Learned preconditioner for CG on the damped tomography normal equations
(A^T A + lam I) x = A^T b, and the flexible CG that runs it.

The preconditioner (no reference counterpart; the reference solves with
plain or Jacobi CG, sparse/sparse_ops.cpp:8-113) is linear and symmetric
positive (semi)definite by construction:
    z = M r = D r + S G^T G S r,   D = diag(dinv) (Jacobi), S = sqrt(D),
    G = (I + conv_K) ... (I + conv_1) C^T,
C^T a 1 -> 32 channel 3x3x3 layer and conv_k 32 -> 32 channel 3x3x3 layers.
So CG keeps its theory (a fixed SPD preconditioner), and the untrained
network (small weights) is Jacobi plus a small correction. The 2K 32 -> 32
layers of G and G^T run on the tensor cores (st_conv3d_bf16: tcgen05, BF16
operands, FP32 accumulation; G^T through the transposed weight packing),
forward and in the backward pass, and so do their weight gradients
(st_conv3d_wgrad: a tcgen05 implicit GEMM contracting over the voxels); C,
C^T, their weight gradients and the scalings are CUDA-core kernels
(st_precond.cu). Activations are BF16, and
the input is scaled by 1 / rms(r) and the output back (z stays linear in r).

Training uses pairs (r_k, e_k = x* - x_k) from plain Jacobi-CG solves of
other systems and minimises 1 - (z.r)^2 / ((z.Az)(e.r)) (A e_k = r_k): the
A-norm error of the best multiple of z relative to ||e||_A^2, i.e. how much
one preconditioned step can reduce the error (CG picks the step length).
Adam on FP32 master weights; the weights of G and G^T are tied.
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
    def __init__(self, nx: int, ny: int, nz: int, layers: int = 2, seed: int = 0, init_scale: float = 0.05):
        self.shape = (nx, ny, nz)
        self.n = nx * ny * nz
        self.layers = layers
        g = torch.Generator().manual_seed(seed)
        dev = "cuda"
        self.w_c = (torch.randn((CH, 27), generator=g) * (init_scale / math.sqrt(27))).to(dev)
        self.w_k = [(torch.randn((CH, CH, 27), generator=g) * (0.5 / math.sqrt(27 * CH))).to(dev)
                    for _ in range(layers)]
        self.params = [self.w_c, *self.w_k]
        pad = (nx + 2, ny + 2, nz + 2, CH)
        self.u = [torch.zeros(pad, dtype=torch.bfloat16, device=dev) for _ in range(layers + 1)]
        self.v = [torch.zeros(pad, dtype=torch.bfloat16, device=dev) for _ in range(layers)] + [self.u[-1]]
        self.d0 = torch.zeros(pad, dtype=torch.bfloat16, device=dev)
        self.d1 = torch.zeros(pad, dtype=torch.bfloat16, device=dev)
        self.packed = [torch.empty(27 * CH * CH, dtype=torch.bfloat16, device=dev) for _ in range(layers)]
        self.packed_t = [torch.empty(27 * CH * CH, dtype=torch.bfloat16, device=dev) for _ in range(layers)]
        self.a = torch.zeros(self.n, device=dev)
        self.y = torch.zeros(self.n, device=dev)
        self.acc = torch.zeros(2, dtype=torch.float64, device=dev)
        self.scales = torch.zeros(2, device=dev)
        self.inv_scales = torch.zeros(2, device=dev)
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
        return {"w_c": self.w_c.cpu(), "w_k": [w.cpu() for w in self.w_k]}

    def load_state_dict(self, sd):
        self.w_c.copy_(sd["w_c"])
        for w, s in zip(self.w_k, sd["w_k"]):
            w.copy_(s)
        self.pack()

    # ------------------------------------------------------------------ forward
    def _tc(self, x, packed, out):
        """out = x + conv(x) on the tensor cores."""
        nx, ny, nz = self.shape
        call("st_conv3d_bf16", _p(x), _p(packed), None, _p(x), _p(out), 0, nx, ny, nz, 0, self._stream())

    def forward(self, r, dinv, z):
        """z = D r + S G^T G S r (activations kept for backward)."""
        nx, ny, nz = self.shape
        st = self._stream()
        call("st_pc_scales", _p(r), _p(dinv), _p(self.acc), _p(self.scales), self.n, st)
        call("st_pc_scale_in", _p(r), _p(dinv), _p(self.scales), _p(self.a), self.n, st)
        call("st_pc_tconv1", _p(self.a), _p(self.w_c), _p(self.u[0]), nx, ny, nz, st)
        for k in range(self.layers):
            self._tc(self.u[k], self.packed[k], self.u[k + 1])
        for k in range(self.layers, 0, -1):
            self._tc(self.v[k], self.packed_t[k - 1], self.v[k - 1])
        call("st_pc_out_conv", _p(self.v[0]), _p(self.w_c), None, None, None, _p(self.y), None, nx, ny, nz, st)
        call("st_pc_combine", _p(self.y), _p(r), _p(dinv), _p(self.scales), _p(z), self.n, st)
        return z

    def __call__(self, r, dinv, z):
        return self.forward(r, dinv, z)

    # ------------------------------------------------------------------ backward
    def backward(self, dz, r, dinv, grads):
        """Accumulates dL/dw into grads ([dw_c, dw_1, ...]) for the
        activations of the last forward, given dL/dz."""
        nx, ny, nz = self.shape
        st = self._stream()
        # dy = sqrt(dinv) dz / s_in
        torch.reciprocal(self.scales, out=self.inv_scales)
        dy = torch.empty_like(dz)
        call("st_pc_scale_in", _p(dz), _p(dinv), _p(self.inv_scales), _p(dy), self.n, st)
        # y = C(v0): dv0 = C^T(dy), dw_c += sum dy * v0[.+tap]
        call("st_pc_out_conv_bwd", _p(dy), _p(self.v[0]), _p(self.w_c), _p(self.d0), _p(grads[0]), nx, ny, nz, st)
        d, e = self.d0, self.d1
        # v_{k-1} = (I + conv_k^T) v_k: dw_k += wgrad(x = dv_{k-1}, g = v_k); dv_k = (I + conv_k) dv_{k-1}
        for k in range(1, self.layers + 1):
            call("st_conv3d_wgrad", _p(d), _p(self.v[k]), _p(grads[k]), nx, ny, nz, st)
            self._tc(d, self.packed[k - 1], e)
            d, e = e, d
        # u_k = (I + conv_k) u_{k-1}: dw_k += wgrad(x = u_{k-1}, g = du_k); du_{k-1} = (I + conv_k^T) du_k
        for k in range(self.layers, 0, -1):
            call("st_conv3d_wgrad", _p(self.u[k - 1]), _p(d), _p(grads[k]), nx, ny, nz, st)
            self._tc(d, self.packed_t[k - 1], e)
            d, e = e, d
        # u_0 = C^T(a): dw_c += sum a * du_0[.+tap]
        call("st_pc_conv1_wgrad", _p(self.a), _p(d), _p(grads[0]), nx, ny, nz, st)

    def check(self):
        call("st_conv3d_check", self._stream())

    # ------------------------------------------------------------------ training
    def a_norm_loss(self, r, e, dinv, op, grads=None, weight=1.0):
        """1 - (z.r)^2 / ((z.Az)(e.r)) for z = M r, with A e = r. With grads,
        accumulates weight * dL/dw."""
        z = torch.empty_like(r)
        self.forward(r, dinv, z)
        az = op(z, torch.empty_like(r))
        er = float(torch.dot(e.double(), r.double()))
        zr = float(torch.dot(z.double(), r.double()))
        zaz = float(torch.dot(z.double(), az.double()))
        loss = 1.0 - zr * zr / (zaz * er)
        if grads is not None:
            # dL/dz = -2 (z.r) / ((z.Az)(e.r)) * (r - (z.r)/(z.Az) Az)
            dz = (r - az * (zr / zaz)).mul_(-2.0 * weight * zr / (zaz * er))
            self.backward(dz, r, dinv, grads)
        return loss

    def train_step(self, batch, lr=1e-3, betas=(0.9, 0.999), eps=1e-8):
        """One Adam step on a list of (r, e, dinv, op) samples (pairs from
        plain-CG solves, op the system's NormalOperator); returns the mean
        loss before the step."""
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


class NativeNetwork:
    """The trained network as a native handle (st_pcnet): applied inside the
    native flexible CG without Python in the loop."""

    def __init__(self, net: LearnedPreconditioner, device: int = 0):
        h = C.c_void_p()
        call("st_pcnet_create", *net.shape, net.layers, device, C.byref(h))
        self._h = h
        self.update(net)

    def update(self, net: LearnedPreconditioner):
        wk = torch.stack(net.w_k).contiguous() if net.layers else torch.zeros(1, device="cuda")
        torch.cuda.synchronize()
        call("st_pcnet_set_weights", self._h, _p(net.w_c.contiguous()), _p(wk))

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None):
            _lib.load().st_pcnet_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def normal_fcg_device(A, d, lam, x, max_iter=20000, tol=1e-6, network: NativeNetwork | None = None):
    """Native flexible CG on (A^T A + lam I) x = A^T d (torch CUDA FP32 d, x),
    preconditioned by the network or, with network=None, by Jacobi. Returns
    (iterations, true relative residual)."""
    it = C.c_int()
    rel = C.c_double()
    call("st_normal_fcg_device", A.handle, _p(d), float(lam), int(max_iter), float(tol),
         network.handle if network is not None else None, _p(x), C.byref(it), C.byref(rel))
    return it.value, rel.value


def ray_system(n: int, n_rays: int, seed: int, lam: float = 1e-2, noise: float = 0.01):
    """One synthetic traveltime system (workloads.ray_endpoints geometry):
    (CSRMatrix A, device data d) with d = A x_true + noise (x_true smooth,
    sigma = 0.03 n cells)."""
    import numpy as np
    from . import workloads as wl
    from .sparse import CSRMatrix
    A = CSRMatrix()
    A.build_ray_matrix(wl.ray_endpoints(n_rays, n, seed), n, n, n)
    xt = torch.from_numpy(wl.smooth_model(n, max(1.0, 0.03 * n), seed + 36).astype(np.float32)).cuda()
    ax = torch.zeros(A.rows(), device="cuda")
    A.spmv_device(xt, ax)
    torch.cuda.synchronize()
    b = wl.noisy_data(ax.double().cpu().numpy(), noise, seed + 40)
    return A, torch.from_numpy(b.astype(np.float32)).cuda()


def train_on_ray_systems(n: int = 32, n_rays: int = 60000, seeds=range(1000, 1064), lam: float = 1e-2,
                         layers: int = 2, steps: int = 300, batch: int = 4, lr: float = 1e-3, seed: int = 0,
                         log=None):
    """Trains a LearnedPreconditioner on (r_k, e_k) pairs from plain Jacobi-CG
    solves of the given seeded ray systems (n^3 cells, n_rays rays each);
    the network is convolutional and scale-normalised, so it applies to
    other grid sizes with the same ray density. Returns (network, stats)."""
    import time
    import numpy as np
    t0 = time.perf_counter()
    samples, keep = [], []
    for s in seeds:
        A, d = ray_system(n, n_rays, s, lam)
        op, pairs = training_pairs(A, d, lam)
        dinv = op.jacobi()
        keep.append(A)
        samples += [(r, e, dinv, op) for r, e in pairs]
    t_data = time.perf_counter() - t0
    net = LearnedPreconditioner(n, n, n, layers=layers, seed=seed)
    base = float(np.mean([net.a_norm_loss(*smp) for smp in samples]))
    rng = np.random.default_rng(seed)
    t1 = time.perf_counter()
    for step in range(steps):
        idx = rng.choice(len(samples), min(batch, len(samples)), replace=False)
        loss = net.train_step([samples[i] for i in idx], lr=lr if step < 0.7 * steps else 0.25 * lr)
        if log is not None and (step % 50 == 0 or step == steps - 1):
            log(f"step {step}: loss {loss:.4f}")
    net.check()
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t1
    final = float(np.mean([net.a_norm_loss(*smp) for smp in samples]))
    stats = {"systems": len(list(seeds)), "pairs": len(samples), "grid": n, "rays": n_rays, "layers": layers,
             "steps": steps, "data_s": t_data, "train_s": t_train, "loss_jacobi": base, "loss_trained": final}
    return net, stats


def fit_stencil_weights(n: int = 50, n_rays: int = 500_000, seeds=(2001,), lam: float = 1e-2, tol: float = 1e-6,
                        max_iter: int = 20000, common=(0.05, 0.1, 0.2, 0.3, 0.5, 0.8, 1.2), factors=(0.6, 1.6),
                        sweeps: int = 2):
    """Fits the three axis weights w of the stencil preconditioner
    M r = D r + S K_w (S r) (st_normal_pcg_stencil_device, the symmetric form
    D + S G^T G S with G the weighted axis differences) on training systems:
    the weights that minimise the mean PCG iteration count to `tol` over
    seeded ray systems (`ray_system`, other seeds than the system the weights
    are used on). A search over one common weight, then per-axis coordinate
    descent over the given factors. Returns (w, stats)."""
    import time
    from .sparse import normal_cg_device, normal_pcg_stencil_device
    t0 = time.perf_counter()
    systems = [ray_system(n, n_rays, s, lam) for s in seeds]
    evals = 0

    def iters(w):
        nonlocal evals
        tot = 0
        for A, d in systems:
            x = torch.zeros(n ** 3, device="cuda")
            if w is None:
                it, _, _ = normal_cg_device(A, d, lam, x, max_iter, tol, True)
            else:
                it, _, _ = normal_pcg_stencil_device(A, d, lam, w, (n, n, n), x, max_iter, tol)
            tot += it
        evals += 1
        return tot / len(systems)

    base = iters(None)
    best_w, best = (0.0, 0.0, 0.0), base
    for a in common:
        c = iters((a, a, a))
        if c < best:
            best_w, best = (a, a, a), c
    for _ in range(sweeps):
        for axis in range(3):
            for f in factors:
                w = list(best_w)
                w[axis] *= f
                c = iters(tuple(w))
                if c < best:
                    best_w, best = tuple(w), c
    for A, _ in systems:
        A.close()
    stats = {"systems": len(systems), "grid": n, "rays": n_rays, "jacobi_iterations": base,
             "fitted_iterations": best, "evaluations": evals, "fit_s": time.perf_counter() - t0}
    return best_w, stats
