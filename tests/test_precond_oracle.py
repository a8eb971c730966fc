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
    w_c = rng.standard_normal((32, 27)) * 0.1
    w_k = [rng.standard_normal((32, 32, 27)) * 0.02 for _ in range(2)]
    r = rng.standard_normal(n)
    dinv = rng.random(n) + 0.5
    t = rng.standard_normal(n)

    def loss(wc, wk):
        net = pr.Net(wc, wk, bf16_storage=False)
        z = net.forward(r, dinv, shape)
        return 0.5 * float(np.sum((z - t) ** 2)), net

    l0, net = loss(w_c, w_k)
    d_c, d_k = net.backward(net.forward(r, dinv, shape) - t, shape)
    eps = 1e-5
    for (name, idx) in [("c", (3, 13)), ("c", (31, 0)), ("k0", (5, 7, 2)), ("k1", (31, 0, 26))]:
        fd = 0.0
        for sign in (1.0, -1.0):  # central differences: the loss is far from linear in w_c
            wc, wk = w_c.copy(), [w.copy() for w in w_k]
            if name == "c":
                wc[idx] += sign * eps
            else:
                wk[int(name[1])][idx] += sign * eps
            fd += sign * loss(wc, wk)[0] / (2 * eps)
        an = d_c[idx] if name == "c" else d_k[int(name[1])][idx]
        assert abs(fd - an) <= 1e-6 * max(1.0, abs(an)), (name, fd, an)


def test_preconditioner_is_symmetric_positive():
    rng = np.random.default_rng(2)
    shape = (5, 4, 6)
    n = int(np.prod(shape))
    net = pr.Net(rng.standard_normal((32, 27)) * 0.2, [rng.standard_normal((32, 32, 27)) * 0.05], bf16_storage=False)
    dinv = rng.random(n) + 0.5
    x, y = rng.standard_normal(n), rng.standard_normal(n)
    # M is linear (the 1/rms scaling cancels): <M x, y> = <x, M y>, <M x, x> > 0
    mx, my = net.forward(x, dinv, shape), net.forward(y, dinv, shape)
    assert abs(np.dot(mx, y) - np.dot(x, my)) <= 1e-10 * np.linalg.norm(mx) * np.linalg.norm(y)
    assert np.dot(mx, x) > 0
    assert np.allclose(net.forward(3.0 * x, dinv, shape), 3.0 * mx)
