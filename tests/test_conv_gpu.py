"""The tensor-core 3x3x3 convolution (tcgen05, BF16 operands, FP32
accumulation) against a PyTorch FP64 conv3d of the same BF16-rounded inputs
and weights: relative L2 <= 1e-5 for FP32 output (FP32 accumulation of 864
exact BF16 products), <= 8e-3 for BF16 output (one BF16 rounding); the
transposed (input-gradient) packing satisfies <conv(x), y> = <x, conv^T(y)>
to 1e-5; border rows of every output stay zero."""
import ctypes as C
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    import importlib.util
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    spec = importlib.util.spec_from_file_location(
        "st_build", os.path.join(repo, "03-seismic-tomography-compute_gb300", "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build()
    from seismic_engine import _lib
    return _lib.load()


def padded(x):
    """(32, D, H, W) torch tensor -> padded channels-last BF16 on the GPU."""
    import torch
    c, d, h, w = x.shape
    p = torch.zeros((d + 2, h + 2, w + 2, c), dtype=torch.bfloat16, device="cuda")
    p[1:-1, 1:-1, 1:-1, :] = x.permute(1, 2, 3, 0).to(torch.bfloat16).cuda()
    return p


def unpad(p):
    """padded channels-last (any dtype) -> (32, D, H, W) FP64 CPU."""
    return p[1:-1, 1:-1, 1:-1, :].permute(3, 0, 1, 2).double().cpu()


def run_conv(lib, xin, wpk, bias, add, D, H, W, relu, f32):
    import torch
    out = torch.full((D + 2, H + 2, W + 2, 32), 7.0, dtype=torch.float32 if f32 else torch.bfloat16, device="cuda")
    out[0] = 0  # planes 0 and D+1 are the caller's (zero once); the kernel writes every row in between
    out[-1] = 0
    st = torch.cuda.current_stream().cuda_stream
    rc = lib.st_conv3d_bf16(C.c_void_p(xin.data_ptr()), C.c_void_p(wpk.data_ptr()),
                            C.c_void_p(bias.data_ptr()) if bias is not None else None,
                            C.c_void_p(add.data_ptr()) if add is not None else None, C.c_void_p(out.data_ptr()),
                            int(f32), D, H, W, int(relu), C.c_void_p(st))
    assert rc == 0, lib.st_last_error()
    assert lib.st_conv3d_check(C.c_void_p(st)) == 0, lib.st_last_error()
    return out


def pack(lib, w, transpose=False):
    import torch
    wpk = torch.empty(27 * 32 * 32, dtype=torch.bfloat16, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    assert lib.st_conv3d_pack_weights(C.c_void_p(w.data_ptr()), C.c_void_p(wpk.data_ptr()), int(transpose),
                                      C.c_void_p(st)) == 0
    return wpk


def rel(a, b):
    return float((a - b).norm() / max(float(b.norm()), 1e-300))


# (25, 40, 40): units of 3 planes (the last of 1) march along d through the window ring
@pytest.mark.parametrize("D,H,W", [(3, 5, 7), (5, 13, 100), (2, 9, 156), (3, 4, 269), (4, 33, 31), (25, 40, 40)])
def test_conv_matches_torch(lib, D, H, W):
    import torch
    import torch.nn.functional as F
    g = torch.Generator().manual_seed(D * 1000 + H * 10 + W)
    x = torch.randn((32, D, H, W), generator=g)
    w = (torch.randn((32, 32, 3, 3, 3), generator=g) / 30).cuda()
    bias = torch.randn(32, generator=g).cuda()
    xin = padded(x)
    wpk = pack(lib, w)
    xb = unpad(xin)
    wb = w.to(torch.bfloat16).double().cpu()
    ref = F.conv3d(xb[None], wb, bias.double().cpu(), padding=1)[0]
    out = run_conv(lib, xin, wpk, bias, None, D, H, W, relu=False, f32=True)
    torch.cuda.synchronize()
    assert rel(unpad(out), ref) < 1e-5
    border = out.clone()
    border[1:-1, 1:-1, 1:-1, :] = 0
    assert not border.any()
    # fused residual input + ReLU, BF16 output
    addv = torch.randn((32, D, H, W), generator=g)
    add = padded(addv)
    out16 = run_conv(lib, xin, wpk, bias, add, D, H, W, relu=True, f32=False)
    ref16 = torch.relu(ref + unpad(add))
    assert rel(unpad(out16), ref16) < 8e-3


def test_transposed_packing_is_the_adjoint(lib):
    import torch
    D, H, W = 4, 11, 19
    g = torch.Generator().manual_seed(5)
    w = (torch.randn((32, 32, 3, 3, 3), generator=g) / 30).cuda()
    x = padded(torch.randn((32, D, H, W), generator=g))
    y = padded(torch.randn((32, D, H, W), generator=g))
    fwd = run_conv(lib, x, pack(lib, w), None, None, D, H, W, relu=False, f32=True)
    bwd = run_conv(lib, y, pack(lib, w, transpose=True), None, None, D, H, W, relu=False, f32=True)
    lhs = float((unpad(fwd) * unpad(y)).sum())
    rhs = float((unpad(x) * unpad(bwd)).sum())
    assert abs(lhs - rhs) <= 1e-5 * abs(lhs)


def test_too_wide_volume_is_refused(lib):
    import torch
    from seismic_engine import _lib
    D, H, W = 2, 3, 270  # the widest accepted is 269 (four plane windows of 128 + 2 (W + 3) rows)
    x = torch.zeros((D + 2, H + 2, W + 2, 32), dtype=torch.bfloat16, device="cuda")
    y = torch.zeros_like(x)
    wpk = torch.zeros(27 * 32 * 32, dtype=torch.bfloat16, device="cuda")
    rc = lib.st_conv3d_bf16(C.c_void_p(x.data_ptr()), C.c_void_p(wpk.data_ptr()), None, None, C.c_void_p(y.data_ptr()),
                            0, D, H, W, 0, None)
    assert rc == _lib.ST_ERR_UNSUPPORTED
