"""Generates the golden fixtures in this directory by running the reference's
own C++ (src/cpp of 13262233692/03-seismic-tomography-compute, compiled in
place by oracle/build_ref.sh into oracle/_ref/libseismic_ref.so) on small
seeded inputs. The reference sources exist only where this script is run;
the fixtures it writes are what the tests (and the GPU machine) use.

    python tests/golden/make_golden.py

Fixtures (all FP64 reference outputs):
  prop_small.npz     inject_source + step_forward stepping with a source and
                     receivers; the same with step_adjoint and per-receiver
                     injection (the reference's adjoint semantics)
  fwdprop_small.npz  forward_propagate (centre source, snapshots, CFL check)
  rtm_small.npz      RTMEngine::apply_image_condition + finalize_image
  csr_small.npz      CSRMatrix::build_from_triplets + spmv (rows >= 8 entries,
                     so the shipped pad_to_alignment never fires)
  fault_small.npz    FaultTolerance::repair_field_nan / clamp_field / count_nan_inf
  config_small.npz   load_config on config/default.yaml and on an edited copy
"""
from __future__ import annotations

import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.join(REPO, "03-seismic-tomography-compute_gb300"))

from oracle import Reference, build_ref  # noqa: E402
from seismic_engine import workloads as wl  # noqa: E402

REFERENCE = os.environ.get("SEISMIC_REFERENCE_DIR", "/root/reference")


def prop_case():
    w = wl.small_case(n=(14, 12, 16), nt=50, seed=11, sponge_width=4)
    shot = w.shots[0]
    vel = wl.to_reference_layout(w.vel)
    rec = shot.rec.coords()
    return w, shot, vel, rec


def main():
    if build_ref() is None:
        raise SystemExit("reference sources unavailable: cannot generate fixtures")
    ref = Reference()
    rng = np.random.default_rng(1234)

    # -- propagator stepping (forward and the reference's adjoint stepping)
    w, shot, vel, rec = prop_case()
    src = np.array([shot.src], np.int64)
    f = ref.run_steps(w.nx, w.ny, w.nz, w.d, w.d, w.d, w.dt, w.sponge_width, w.sponge_damping, vel, w.nt, src,
                      shot.wavelet[:, None], rec)
    resid = rng.standard_normal((w.nt, rec.shape[0])) * 1e-2
    a = ref.run_steps(w.nx, w.ny, w.nz, w.d, w.d, w.d, w.dt, w.sponge_width, w.sponge_damping, vel, w.nt, rec,
                      resid, src, adjoint=True)
    np.savez_compressed(os.path.join(HERE, "prop_small.npz"),
                        n=np.array([w.nx, w.ny, w.nz]), d=w.d, dt=w.dt, sw=w.sponge_width, damp=w.sponge_damping,
                        vel=vel, src=src, wavelet=shot.wavelet, rec=rec,
                        seis=f["seis"], cur=f["cur"], prev=f["prev"], status=f["status"],
                        adj_resid=resid, adj_seis=a["seis"], adj_cur=a["cur"], adj_prev=a["prev"],
                        adj_status=a["status"])

    # -- forward_propagate (centre source, snapshots every 7 steps)
    fp = ref.forward_propagate(w.nx, w.ny, w.nz, w.d, w.d, w.d, w.dt, 30, w.sponge_width, w.sponge_damping, 7,
                               vel, shot.wavelet[:30])
    bad = ref.forward_propagate(w.nx, w.ny, w.nz, w.d, w.d, w.d, 10 * w.dt, 30, w.sponge_width, w.sponge_damping,
                                7, vel, shot.wavelet[:30])
    np.savez_compressed(os.path.join(HERE, "fwdprop_small.npz"), nt=30, snap_interval=7, dt=w.dt,
                        status=fp["status"], steps=fp["steps"], ok=fp["ok"], cur=fp["cur"], prev=fp["prev"],
                        snapshots=fp["snapshots"], cfl_bad_status=bad["status"], cfl_bad_steps=bad["steps"])

    # -- RTM imaging condition
    nx, ny, nz = 6, 5, 7
    npad = (nx + 2) * (ny + 2) * (nz + 2)
    F = rng.standard_normal((4, npad))
    A = rng.standard_normal((4, npad))
    F[1, 100] = np.nan
    A[2, 150] = np.inf
    img, ill, refl = ref.rtm_image(nx, ny, nz, F, A)
    np.savez_compressed(os.path.join(HERE, "rtm_small.npz"), n=np.array([nx, ny, nz]), fwd=F, adj=A, image=img,
                        illum=ill, refl=refl)

    # -- CSR build: 40 rows x 33 cols, >= 10 distinct columns per row, duplicate
    # (row,col) pairs with dyadic values (exact sums), out-of-range entries dropped
    rows, cols = 40, 33
    R, Cc, V = [], [], []
    for r in range(rows):
        cs = rng.choice(cols, size=10 + (r % 5), replace=False)
        for c in cs:
            R.append(r); Cc.append(c); V.append(rng.integers(-64, 64) / 16.0)
        for c in rng.choice(cs, size=3):
            R.append(r); Cc.append(c); V.append(rng.integers(-64, 64) / 16.0)
    R += [-1, rows, 3, 4]
    Cc += [2, 2, -1, cols]
    V += [1.0, 1.0, 1.0, 1.0]
    perm = rng.permutation(len(R))
    R = np.array(R, np.int64)[perm]
    Cc = np.array(Cc, np.int64)[perm]
    V = np.array(V, np.float64)[perm]
    rp, col, val = ref.csr_build(rows, cols, R, Cc, V)
    x = rng.standard_normal(cols)
    y = ref.csr_spmv(x, rows)
    np.savez_compressed(os.path.join(HERE, "csr_small.npz"), rows=rows, cols=cols, r=R, c=Cc, v=V, row_ptr=rp,
                        col=col, val=val, x=x, y=y)

    # -- fault tolerance helpers on a padded field with NaN/Inf cells
    nx, ny, nz = 7, 6, 8
    g = rng.standard_normal((nx + 2) * (ny + 2) * (nz + 2)) * 1e3
    for i in (150, 151, 152 + (nz + 2), 300, 7):
        g[i] = np.nan
    g[200] = np.inf
    g[201] = -np.inf
    rep = ref.repair_field_nan(g, nx + 2, ny + 2, nz + 2, 1, 0.0)
    cl = ref.clamp_field(g, -500.0, 500.0)
    np.savez_compressed(os.path.join(HERE, "fault_small.npz"), n=np.array([nx, ny, nz]), field=g, repaired=rep,
                        clamped=cl, nan_count=ref.count_nan_inf(g))

    # -- configuration parser
    default_yaml = os.path.join(REFERENCE, "config", "default.yaml")
    with open(default_yaml) as fh:
        text = fh.read()
    edited = (text.replace("dt: 0.001", "dt: 0.0005").replace("nt: 5000", "nt: 1234")
              .replace("sponge_width: 20", "sponge_width: 12").replace("initial_vp: 1500.0", "initial_vp: 1490.0")
              .replace("snapshot_interval: 100", "snapshot_interval: 50")
              .replace("regularization_lambda: 0.0001", "regularization_lambda: 0.25"))
    with tempfile.NamedTemporaryFile("w", suffix=".yaml", delete=False) as fh:
        fh.write(edited + "\n# comment line\nunknown_section:\n  foo: 1\n")
        edited_path = fh.name
    vals_default = ref.load_config(default_yaml)
    vals_edited = ref.load_config(edited_path)
    vals_missing = ref.load_config("/nonexistent/path.yaml")
    os.unlink(edited_path)
    np.savez_compressed(os.path.join(HERE, "config_small.npz"), default_yaml=np.array(text),
                        edited_yaml=np.array(edited + "\n# comment line\nunknown_section:\n  foo: 1\n"),
                        default=vals_default, edited=vals_edited, missing=vals_missing)
    for fn in sorted(os.listdir(HERE)):
        if fn.endswith(".npz"):
            print(fn, os.path.getsize(os.path.join(HERE, fn)))


if __name__ == "__main__":
    main()
