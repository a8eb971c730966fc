"""Host logic of the stencil-preconditioner weight fit
(seismic_engine.precond.fit_stencil_weights) without a GPU: the solver
calls are replaced by a synthetic iteration count with a known minimum, and
the search (one common weight, then per-axis coordinate descent) must move
to it and report its statistics; a weight set that gains nothing keeps
Jacobi (all zero)."""
import os
import sys
import types

import pytest

torch = pytest.importorskip("torch")

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(REPO, "03-seismic-tomography-compute_gb300"))


class _FakeMatrix:
    def close(self):
        pass


def _patched(monkeypatch, cost):
    from seismic_engine import precond, sparse
    monkeypatch.setattr(precond, "ray_system", lambda n, rays, seed, lam=1e-2: (_FakeMatrix(), None))
    monkeypatch.setattr(torch, "zeros", lambda *a, **k: None)
    monkeypatch.setattr(sparse, "normal_cg_device", lambda A, d, lam, x, mi, tol, jac: (cost(None), 0.0, 0.0))
    monkeypatch.setattr(sparse, "normal_pcg_stencil_device",
                        lambda A, d, lam, w, grid, x, mi, tol: (cost(tuple(w)), 0.0, 0.0))
    return precond


def test_search_moves_to_the_minimum(monkeypatch):
    target = (0.15, 0.4, 0.3)

    def cost(w):
        if w is None:
            return 1000.0
        return 800.0 + 400.0 * sum((a - b) ** 2 for a, b in zip(w, target))

    precond = _patched(monkeypatch, cost)
    w, stats = precond.fit_stencil_weights(n=8, n_rays=10, seeds=(1, 2), sweeps=3)
    assert stats["jacobi_iterations"] == 1000.0
    assert stats["fitted_iterations"] == cost(w) < 1000.0
    assert stats["systems"] == 2 and stats["evaluations"] == 1 + 7 + 3 * 3 * 2
    # the coordinate search ends within a factor step of the minimum on each axis
    for a, b in zip(w, target):
        assert b / 1.6 <= a <= b * 1.6, (w, target)


def test_no_gain_keeps_jacobi(monkeypatch):
    precond = _patched(monkeypatch, lambda w: 500.0 if w is None else 500.0 + 10.0 * sum(w))
    w, stats = precond.fit_stencil_weights(n=8, n_rays=10, seeds=(1,))
    assert w == (0.0, 0.0, 0.0) and stats["fitted_iterations"] == 500.0
