"""Learned CG preconditioner on the GPU: its forward pass and the gradients
of all its layers (tensor-core forward, input-gradient and 32 -> 32
weight-gradient convolutions; CUDA-core 1 <-> 32 channel layers) against
the CPU oracle's FP64 restatement with
BF16 storage emulated (relative L2 <= 1e-2), and the preconditioned flexible
CG against Jacobi-CG on a small ray system after a short training."""
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def se():
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "st_build", os.path.join(REPO, "03-seismic-tomography-compute_gb300", "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build()
    import seismic_engine
    import seismic_engine.precond  # noqa: F401
    return seismic_engine


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def test_network_forward_and_gradients_match_oracle(se):
    import torch
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import precond_ref as pr
    shape = (6, 7, 9)
    n = int(np.prod(shape))
    net = se.precond.LearnedPreconditioner(*shape, layers=2, seed=3, init_scale=0.5)
    g = torch.Generator().manual_seed(4)
    r = torch.randn(n, generator=g).cuda()
    dinv = (torch.rand(n, generator=g) + 0.5).cuda()
    z = torch.zeros(n, device="cuda")
    net.forward(r, dinv, z)
    dz = torch.randn(n, generator=g).cuda()
    grads = [torch.zeros_like(p) for p in net.params]
    net.backward(dz, r, dinv, grads)
    net.check()
    torch.cuda.synchronize()
    ref = pr.Net(net.w_c.cpu().numpy(), [w.cpu().numpy() for w in net.w_k])
    zr = ref.forward(r.cpu().numpy(), dinv.cpu().numpy(), shape)
    corr = z.cpu().numpy() - (dinv * r).cpu().numpy()  # the learned part, compared on its own
    assert rel(corr, zr - (dinv * r).cpu().numpy()) < 1e-2
    d_c, d_k = ref.backward(dz.cpu().numpy(), shape)
    errs = [rel(grads[0].cpu().numpy(), d_c)] + [rel(grads[1 + k].cpu().numpy(), d_k[k]) for k in range(2)]
    print("network gradient errors vs oracle:", ["%.2e" % e for e in errs])
    assert max(errs) < 1e-2


def test_native_fcg_and_trained_preconditioner(se):
    """Native flexible CG: with Jacobi it reaches the same solution as the
    native Jacobi-CG; the network trained on CG pairs from other systems
    lowers its training loss below Jacobi's and still converges (the printed
    iteration counts are what it gains, or costs, against Jacobi)."""
    import torch
    pc = se.precond
    n, rays = 20, 16000
    net, stats = pc.train_on_ray_systems(n=n, n_rays=rays, seeds=range(1000, 1004), steps=60, layers=1)
    assert stats["loss_trained"] < stats["loss_jacobi"], stats
    A, d = pc.ray_system(n, rays, 7)
    x_cg = torch.zeros(n ** 3, device="cuda")
    it_cg, _, tr_cg = se.normal_cg_device(A, d, 1e-2, x_cg, 20000, 1e-6, True)
    x_j = torch.zeros(n ** 3, device="cuda")
    it_j, rel_j = pc.normal_fcg_device(A, d, 1e-2, x_j, 20000, 1e-6)
    native = pc.NativeNetwork(net)
    x_l = torch.zeros(n ** 3, device="cuda")
    it_l, rel_l = pc.normal_fcg_device(A, d, 1e-2, x_l, 20000, 1e-6, native)
    print(f"{n}^3 ray system: Jacobi-CG {it_cg} it, Jacobi-FCG {it_j} it, learned FCG {it_l} it; "
          f"training loss {stats['loss_jacobi']:.4f} -> {stats['loss_trained']:.4f}")
    assert tr_cg <= 2e-6 and rel_j <= 1e-6 and rel_l <= 1e-6
    assert abs(it_j - it_cg) <= 0.1 * it_cg + 16
    assert float(torch.linalg.norm(x_j - x_cg)) <= 2e-2 * float(torch.linalg.norm(x_cg))
    assert float(torch.linalg.norm(x_l - x_cg)) <= 2e-2 * float(torch.linalg.norm(x_cg))


def test_conv3d_wgrad_tensor_cores_match_fp64(se):
    """st_conv3d_wgrad (tcgen05 implicit GEMM over the padded rows, split over
    CTAs) against an FP64 sum over the interior voxels of the same BF16
    values; the output gradient's border rows hold garbage, which the kernel
    must ignore. Shapes: small, ragged, and large enough for long K ranges."""
    import torch
    from seismic_engine._lib import call
    st = torch.cuda.current_stream().cuda_stream
    for shape in ((6, 7, 9), (17, 12, 30), (40, 33, 50)):
        D, H, W = shape
        gen = torch.Generator().manual_seed(D)
        x = torch.zeros((D + 2, H + 2, W + 2, 32))
        x[1:-1, 1:-1, 1:-1] = torch.randn((D, H, W, 32), generator=gen)
        g = torch.randn((D + 2, H + 2, W + 2, 32), generator=gen)
        xb, gb = x.bfloat16(), g.bfloat16()
        xd, gd = xb.cuda(), gb.cuda()
        dw = torch.zeros(32 * 32 * 27, device="cuda")
        call("st_conv3d_wgrad", xd.data_ptr(), gd.data_ptr(), dw.data_ptr(), D, H, W, st)
        call("st_conv3d_check", st)
        xf, gi = xb.double(), gb.double()[1:-1, 1:-1, 1:-1]
        ref = np.zeros((32, 32, 27))
        for tap in range(27):
            kd, kh, kw = tap // 9, (tap // 3) % 3, tap % 3
            xs = xf[kd:kd + D, kh:kh + H, kw:kw + W]
            ref[:, :, tap] = torch.einsum("dhwo,dhwi->oi", gi, xs).numpy()
        got = dw.cpu().numpy().reshape(32, 32, 27)
        assert rel(got, ref) < 1e-5, (shape, rel(got, ref))
