"""Generates solver_api_small.npz by running the reference's own
WaveEquationSolver (src/cpp/solver/wave_equation.cpp of
13262233692/03-seismic-tomography-compute, compiled in place by
oracle/build_ref.sh) through the harness entry points in
oracle/ref_harness.cpp, on the seeded 14x12x16 grid of prop_small.npz.

    SEISMIC_REFERENCE_DIR=<reference checkout> python tests/golden/make_golden_solver_api.py

Contents (FP64 reference outputs, halo-padded reference layout):
  adj_*      adjoint_propagate (wave_equation.cpp:154-194) on a fresh solver,
             with a residual shorter than nt and one NaN sample (skipped by
             inject_source)
  adjfp_*    forward_propagate(wavelet) then adjoint_propagate on the same
             solver (adjoint_propagate keeps the fields)
  bb_*       configure_rtm(enable_rtm, ring_buffer_capacity 4), then per step
             inject_source(centre) + step_forward, store_forward_wavefield_for_rtm
             (ops bit 1), apply_rtm_step (bit 2; bit 4 = with_snapshot) and
             apply_sponge_layer (bit 8); finalize_image; the image,
             illumination, reflectivity, final fields and the
             snapshots_captured / snapshots_dropped counts
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.join(REPO, "03-seismic-tomography-compute_gb300"))

from oracle import Reference, build_ref  # noqa: E402
from seismic_engine import workloads as wl  # noqa: E402


def main():
    if build_ref() is None:
        raise SystemExit("reference sources unavailable: cannot generate fixtures")
    ref = Reference()
    rng = np.random.default_rng(777)
    w = wl.small_case(n=(14, 12, 16), nt=50, seed=11, sponge_width=4)
    vel = wl.to_reference_layout(w.vel)
    g = (w.nx, w.ny, w.nz, w.d, w.d, w.d, w.dt)
    out = dict(n=np.array([w.nx, w.ny, w.nz]), d=w.d, dt=w.dt, sw=w.sponge_width, damp=w.sponge_damping, vel=vel,
               wavelet=w.shots[0].wavelet)
    nt = 40
    resid = rng.standard_normal(nt - 7) * 1e-2
    resid[11] = np.nan
    a = ref.adjoint_propagate(*g, nt, w.sponge_width, w.sponge_damping, vel, resid)
    out.update(adj_nt=nt, adj_resid=resid, adj_cur=a["cur"], adj_prev=a["prev"],
               adj_result=np.array([a["status"], a["nan"], a["repaired"], a["steps"], int(a["ok"])]))
    b = ref.adjoint_propagate(*g, nt, w.sponge_width, w.sponge_damping, vel, resid,
                              fwd_wavelet=w.shots[0].wavelet[:nt])
    out.update(adjfp_cur=b["cur"], adjfp_prev=b["prev"],
               adjfp_result=np.array([b["status"], b["nan"], b["repaired"], b["steps"], int(b["ok"])]))
    nsteps = 30
    ops = np.array([(1 if (t >= 5 and t % 3 == 0) else 0) | (2 if t % 2 == 0 else 0) | (4 if t % 4 == 0 else 0)
                    | (8 if t in (17, 25) else 0) for t in range(nsteps)], np.int32)
    r = ref.rtm_building_blocks(*g, w.sponge_width, w.sponge_damping, vel, w.shots[0].wavelet[:nsteps], ops, 4)
    out.update(bb_ops=ops, bb_ring=4, bb_image=r["image"], bb_illum=r["illum"], bb_refl=r["refl"], bb_cur=r["cur"],
               bb_prev=r["prev"], bb_counts=np.array([r["captured"], r["dropped"]]))
    np.savez_compressed(os.path.join(HERE, "solver_api_small.npz"), **out)
    print("solver_api_small.npz", os.path.getsize(os.path.join(HERE, "solver_api_small.npz")))
    print("adjoint result", out["adj_result"], out["adjfp_result"], "counts", out["bb_counts"])


if __name__ == "__main__":
    main()
