"""The CPU restatement of the learned-preconditioner network (test
infrastructure) against its own definition: conv_t is the adjoint of conv,
and the backward pass matches finite differences of the loss."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import precond_ref as pr  # noqa: E402


def test_conv_transpose_is_adjoint():
    rng = np.random.default_rng(0)
    x = rng.standard_normal((3, 4, 5, 6))
    y = rng.standard_normal((2, 4, 5, 6))
    w = rng.standard_normal((2, 3, 27))
    assert abs(np.sum(pr.conv(x, w) * y) - np.sum(x * pr.conv_t(y, w))) < 1e-10


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(1)
    shape = (4, 3, 5)
    n = int(np.prod(shape))
    w_in = rng.standard_normal((32, 2, 27)) * 0.2
    w_k = [rng.standard_normal((32, 32, 27)) * 0.02 for _ in range(2)]
    w_out = rng.standard_normal((32, 27)) * 0.1
    r = rng.standard_normal(n)
    dinv = rng.random(n) + 0.5
    t = rng.standard_normal(n)

    def loss(wi, wk, wo):
        net = pr.Net(wi, wk, wo, bf16_storage=False)
        z = net.forward(r, dinv, shape)
        return 0.5 * float(np.sum((z - t) ** 2)), net

    l0, net = loss(w_in, w_k, w_out)
    d_in, d_k, d_out = net.backward(net.forward(r, dinv, shape) - t, shape)
    eps = 1e-6
    for (name, idx) in [("in", (3, 1, 13)), ("k0", (5, 7, 2)), ("k1", (31, 0, 26)), ("out", (9, 4))]:
        wi, wk, wo = w_in.copy(), [w.copy() for w in w_k], w_out.copy()
        if name == "in":
            wi[idx] += eps
            an = d_in[idx]
        elif name == "out":
            wo[idx] += eps
            an = d_out[idx]
        else:
            k = int(name[1])
            wk[k][idx] += eps
            an = d_k[k][idx]
        fd = (loss(wi, wk, wo)[0] - l0) / eps
        assert abs(fd - an) <= 1e-4 * max(1.0, abs(an)), (name, fd, an)
