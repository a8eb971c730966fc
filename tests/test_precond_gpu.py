"""Learned CG preconditioner on the GPU: its forward pass and the gradients
of all its layers (tensor-core forward and input-gradient convolutions,
CUDA-core weight gradients) against the CPU oracle's FP64 restatement with
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
    net = se.precond.LearnedPreconditioner(*shape, layers=2, seed=3)
    g = torch.Generator().manual_seed(4)
    net.w_out.copy_(torch.randn((32, 27), generator=g) * 0.1)
    net.pack()
    r = torch.randn(n, generator=g).cuda()
    dinv = (torch.rand(n, generator=g) + 0.5).cuda()
    zhat = net.forward(r, dinv).clone()
    dz = torch.randn(n, generator=g).cuda()
    grads = [torch.zeros_like(p) for p in net.params]
    net.backward(dz, r, dinv, grads)
    net.check()
    torch.cuda.synchronize()
    ref = pr.Net(net.w_in.cpu().numpy(), [w.cpu().numpy() for w in net.w_k], net.w_out.cpu().numpy())
    zr = ref.forward(r.cpu().numpy(), dinv.cpu().numpy(), shape)
    assert rel(zhat.cpu().numpy(), zr) < 1e-2
    d_in, d_k, d_out = ref.backward(dz.cpu().numpy(), shape)
    errs = [rel(grads[0].cpu().numpy(), d_in)] + [rel(grads[1 + k].cpu().numpy(), d_k[k]) for k in range(2)] + \
        [rel(grads[-1].cpu().numpy(), d_out)]
    print("network gradient errors vs oracle:", ["%.2e" % e for e in errs])
    assert max(errs) < 1e-2
