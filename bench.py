#!/usr/bin/env python
"""Benchmark of the GB300 seismic hot path on its headline workload.

Workload (one bench step = one shot): reverse-time migration on a 256^3 grid,
2000 time steps -- the forward pass with a fused BF16 (+per-snapshot scale)
snapshot store of every step, then the exact-adjoint backward pass with the
zero-lag cross-correlation imaging fused in, then the reflectivity. The
metric is stencil throughput in Gpts/s (interior points x time steps of both
passes per second); HBM GB/s and the roofline fraction of the dominant kernel
are reported beside it. Inputs are seeded synthetic models (4 layers
1500-4500 m/s, two +-10% Gaussian anomalies, 15 Hz Ricker at (128,128,5),
128x128 receivers on z = 5; observed data modelled on the true model,
migration on the model smoothed with sigma 6 cells).

    python bench.py [--gpus N --steps K --warmup W] [--impl reference]

Multi-GPU (torchrun): every rank migrates its own shot (shot-parallel, no
collective on the data path); value = all ranks' points / max rank time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

REPO = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(REPO, "03-seismic-tomography-compute_gb300")
for _p in (PKG, os.path.join(REPO, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

SNAP_BYTES = {"bf16": 2, "fp16": 2, "fp32": 4}


def alg_bytes(snap, paired):
    """Algorithmic HBM bytes per interior point per launch of the forward and
    the adjoint+imaging kernels. One step per launch: read u, prev, c + write
    out (16) + the snapshot store (forward) or read (adjoint) + image and
    illumination read-modify-write (16, adjoint). Two steps per launch: read
    u, prev, c (12) + write both steps' fields (8) + two snapshots + the image
    and illumination read-modify-write once (16, adjoint)."""
    es = SNAP_BYTES[snap]
    if paired:
        return 20 + 2 * es, 36 + 2 * es
    return 16 + es, 32 + es
METRIC = "stencil Gpts/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--nt", type=int, default=2000, help="time steps per shot (2000 = the workload)")
    ap.add_argument("--n", type=int, default=256, help="grid edge (256 = the workload)")
    ap.add_argument("--snap", choices=["bf16", "fp16", "fp32"], default="bf16")
    ap.add_argument("--fused-steps", type=int, choices=[1, 2], default=2,
                    help="time steps per launch of the forward and imaging passes (results are identical)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="target CPU sample time")
    ap.add_argument("--workload", choices=["rtm", "large"], default="rtm",
                    help="large: one 512^3, 8-shot adjoint tomography iteration (not the headline line)")
    ap.add_argument("--segment", type=int, default=200, help="checkpoint segment length of --workload large")
    ap.add_argument("--compare", action="store_true",
                    help="--workload large: also time FP32 segment snapshots and unpreconditioned CG")
    ap.add_argument("--kernel", choices=["conv", "wgrad", "fwigrad", "spmv", "rays"], default=None,
                    help="time one kernel alone (profiling runs) instead of the workload")
    ap.add_argument("--no-tomo", action="store_true", help="skip the tomography CG measurement")
    ap.add_argument("--tomo-n", type=int, default=100, help="cell grid edge of the --kernel spmv matrix")
    ap.add_argument("--tomo-rays", type=int, default=2_000_000, help="rays of the --kernel spmv matrix")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-preconditioner solve")
    ap.add_argument("--no-rays", action="store_true", help="skip the sampled-ray forward/gradient measurement")
    ap.add_argument("--no-512", action="store_true", help="skip the 512^3 roofline leg")
    ap.add_argument("--no-large", action="store_true", help="skip the 512^3 adjoint tomography iteration")
    ap.add_argument("--dry-run", action="store_true",
                    help="check the multi-process plumbing only (set-up, barrier, max over ranks); no GPU work")
    return ap.parse_args()


def workload(n, nt):
    from seismic_engine import workloads as wl
    if n == 256:
        w = wl.rtm_256(nt)
    else:
        w = wl.rtm_256(nt)
        v = wl.layered(n, n, n, [1500.0, 2500.0, 3500.0, 4500.0])
        wl.random_anomalies(v, 2, seed=2)
        w.nx = w.ny = w.nz = n
        w.vel = v
        w.dt = wl.cfl_dt(10.0, float(v.max()))
        rec = wl.ReceiverGrid(0, 2, n // 2, 0, 2, n // 2, 5)
        w.shots = [wl.ShotSpec((n // 2, n // 2, 5), wl.ricker(15.0, w.dt, nt), rec)]
        w.name = f"rtm-{n}^3"
    w.vel_migration = wl.smooth(w.vel, 6.0)
    return w


def config_dict(w, snap, n_gpus):
    return {
        "workload": f"{w.name} x {w.nt} steps (forward + exact adjoint with fused imaging)",
        "grid": [w.nx, w.ny, w.nz], "nt": w.nt, "dx_m": w.d, "dt_s": w.dt,
        "snapshots": f"{snap}+per-snapshot scale, store-all",
        "receivers": f"{w.shots[0].rec.nx}x{w.shots[0].rec.ny} on z={w.shots[0].rec.z}",
        "sponge": [w.sponge_width, w.sponge_damping, w.sponge_mode],
        "l2": "inputs larger than L2: 4 FP32 fields of %.0f MB each + %.0f GB of snapshots" % (
            (w.nx + 2) * (w.ny + 2) * (w.nz + 8) * 4 / 1e6,
            w.nx * w.ny * w.nz * w.nt * (4 if snap == "fp32" else 2) / 1e9),
        "parallelism": "shot-parallel replicas" if n_gpus > 1 else "single GPU, one device-resident domain",
    }


def dist_setup(args):
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    elif torch.cuda.is_available():
        torch.cuda.set_device(local)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.dev = device_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-i", str(self.dev),
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in getattr(self, "lines", []):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic(kernel_key):
    """DRAM bytes per launch of a kernel from the committed ncu summary, or None."""
    p = os.path.join(REPO, "profiles", "traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        d = json.load(f)
    e = d.get(kernel_key)
    return None if e is None else e.get("bytes_per_launch_full")


# ---------------------------------------------------------------- CPU legs
def cpu_rtm_sample(w, nt_sample):
    """Oracle port (the reference's step restated in C, OpenMP over the host
    cores): forward stepping with states kept + exact adjoint with imaging,
    nt_sample steps of each on the workload's grid. Returns seconds."""
    from oracle import Oracle
    from seismic_engine import workloads as wl
    o = Oracle()
    g = o.grid(w.nx, w.ny, w.nz, w.d, w.d, w.d, w.dt, w.sponge_width, w.sponge_damping, sponge_mode=w.sponge_mode)
    shot = w.shots[0]
    vel = wl.to_reference_layout(w.vel_migration)
    rec = shot.rec.coords()
    data = np.random.default_rng(0).standard_normal((nt_sample, rec.shape[0])) * 1e-3
    t0 = time.perf_counter()
    f = o.run(g, vel, nt_sample, np.array([shot.src]), shot.wavelet[:nt_sample, None], rec, keep_states=True)
    o.adjoint(g, vel, nt_sample, rec, data, states=f["states"], want_image=True)
    return time.perf_counter() - t0, o.num_threads()


def cpu_baseline(w, target_s):
    """Blocks of up to 60 forward + 60 adjoint/imaging steps (the forward
    states of a block are kept in host memory, 137 MB each at 256^3),
    repeated until about target_s of CPU work has run."""
    probe_steps = 2
    t, cores = cpu_rtm_sample(w, probe_steps)
    per_step = t / probe_steps
    nt_s = int(max(2, min(60, target_s / per_step)))
    total, blocks = 0.0, 0
    while blocks < 1 or (total < target_s and blocks < 8):
        t, cores = cpu_rtm_sample(w, nt_s)
        total += t
        blocks += 1
    pts = 2.0 * nt_s * blocks * w.nx * w.ny * w.nz
    return {"value": pts / total / 1e9, "unit": "Gpts/s", "cores": cores, "kind": "port",
            "sample": f"{blocks} blocks of {nt_s} forward + {nt_s} adjoint/imaging steps of the {w.nx}^3 "
                      f"workload in FP64 ({total:.1f} s; the reference's CPU step restated in C, OpenMP over "
                      f"{cores} threads)"}


def _ref_note():
    import platform
    if platform.machine() in ("x86_64", "AMD64"):
        return "the reference's own single-threaded C++ is the oracle's pin, not timed here"
    return (f"the reference's own C++ uses x86 intrinsics (immintrin.h) and does not build on this "
            f"{platform.machine()} host")


def run_reference(args):
    world, rank, _ = int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")), 0
    if rank != 0:
        return 0
    w = workload(args.n, args.nt)
    # each step: a bounded RTM sample sized so the whole run ends in minutes
    probe, cores = cpu_rtm_sample(w, 2)
    nt_s = int(max(2, min(40, 20.0 / (probe / 2))))
    times = []
    for i in range(args.warmup + args.steps):
        t, cores = cpu_rtm_sample(w, nt_s)
        if i >= args.warmup:
            times.append(t)
    el = sum(times)
    pts = 2.0 * nt_s * w.nx * w.ny * w.nz * args.steps
    value = pts / el / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Gpts/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded layered model + Gaussian anomalies)",
        "config": config_dict(w, args.snap, world),
        "cpu_baseline": {"value": value, "unit": "Gpts/s", "cores": cores, "kind": "port",
                         "sample": f"each step: {nt_s} forward + {nt_s} adjoint/imaging steps of the "
                                   f"{w.nx}^3 workload in FP64 (the reference's CPU step restated in C, "
                                   f"OpenMP over {cores} threads; {_ref_note()})"},
        "e2e": {"value": value, "unit": "Gpts/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------- tomography
def run_tomography(args):
    """Traveltime tomography on 100^3 cells with 2M straight rays: the ray
    matrix build, SpMV / SpMV^T bandwidth, and time to a 1e-6 true relative
    residual of (A^T A + 1e-2 I) x = A^T b for the Jacobi-CG, for plain CG
    (no preconditioner), for the PCG with the fitted stencil preconditioner
    and for the flexible CG with the learned preconditioner (trained first on
    64 smaller seeded systems; training and fitting times reported
    separately)."""
    import torch
    import seismic_engine as se
    from seismic_engine import precond as pc
    tp = se.workloads.tomography_100()
    n = tp.n
    A = se.CSRMatrix()
    ends = torch.from_numpy(tp.ends).cuda()
    A.build_ray_matrix(ends, n, n, n)  # warm-up build
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    nnz = A.build_ray_matrix(ends, n, n, n)
    torch.cuda.synchronize()
    build_ms = 1e3 * (time.perf_counter() - t0)
    xt = torch.from_numpy(tp.x_true.astype(np.float32)).cuda()
    ax = torch.zeros(A.rows(), device="cuda")
    A.spmv_device(xt, ax)
    torch.cuda.synchronize()
    d = torch.from_numpy(se.workloads.noisy_data(ax.double().cpu().numpy(), tp.noise_level,
                                                 tp.noise_seed).astype(np.float32)).cuda()
    stream = torch.cuda.ExternalStream(A.stream_ptr())
    hbm_peak, peak_kind = measured_peaks()
    spmv = {}
    for name, tr, x, y in (("A", False, xt, ax), ("A^T", True, ax, torch.zeros(n ** 3, device="cuda"))):
        for _ in range(3):
            A.spmv_device(x, y, transpose=tr)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(10):
            A.spmv_device(x, y, transpose=tr)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / 10
        rows = A.cols() if tr else A.rows()
        alg = nnz * 8 + rows * 16  # FP32 value + int32 column per entry, int64 row pointer + FP32 output per row
        spmv[name] = {"ms": ms, "achieved": alg / ms / 1e6, "peak": hbm_peak, "unit": "GB/s",
                      "frac": alg / ms / 1e6 / hbm_peak, "alg_bytes": alg}
    out = {"workload": f"{n}^3 cells, {A.rows()} straight rays (surface to 4 boreholes), lam {tp.lam}, "
                       f"b = A x_true + 1% noise, tol 1e-6 on the true residual",
           "nnz": nnz, "nnz_per_row": nnz / A.rows(), "build_ms": build_ms, "spmv": spmv,
           "peak_kind": f"{peak_kind} copy bandwidth"}
    x = torch.zeros(n ** 3, device="cuda")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    it, rel, true_rel = se.normal_cg_device(A, d, tp.lam, x, 20000, 1e-6, True, confirm_true=True)
    torch.cuda.synchronize()
    t_cg = time.perf_counter() - t0
    out["jacobi_cg"] = {"iterations": it, "seconds": t_cg, "ms_per_iteration": 1e3 * t_cg / max(it, 1),
                        "true_rel": true_rel}
    # plain CG (no preconditioner, sparse_ops.cpp:8-50 on the normal equations): the baseline the
    # learned preconditioner's time target is stated against
    x = torch.zeros(n ** 3, device="cuda")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    it_p, rel_p, true_p = se.normal_cg_device(A, d, tp.lam, x, 20000, 1e-6, False, confirm_true=True)
    torch.cuda.synchronize()
    t_plain = time.perf_counter() - t0
    out["plain_cg"] = {"iterations": it_p, "seconds": t_plain, "ms_per_iteration": 1e3 * t_plain / max(it_p, 1),
                       "true_rel": true_p}
    # the fitted stencil preconditioner: weights learned on another seeded system of the same ray
    # density (50^3 cells, 500k rays), then applied here
    w_st, st_stats = pc.fit_stencil_weights()
    x = torch.zeros(n ** 3, device="cuda")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    it_s, rel_s, true_s = se.normal_pcg_stencil_device(A, d, tp.lam, w_st, (n, n, n), x, 20000, 1e-6, confirm_true=True)
    torch.cuda.synchronize()
    t_s = time.perf_counter() - t0
    out["stencil_pcg"] = {"iterations": it_s, "seconds": t_s, "ms_per_iteration": 1e3 * t_s / max(it_s, 1),
                          "true_rel": true_s, "time_ratio_vs_jacobi_cg": t_s / t_cg,
                          "time_ratio_vs_plain_cg": t_s / t_plain, "weights": list(w_st),
                          "fit": st_stats}
    if not args.no_learned:
        net, stats = pc.train_on_ray_systems(n=32, n_rays=60000, seeds=range(1000, 1064), lam=tp.lam)
        big = pc.LearnedPreconditioner(n, n, n, layers=net.layers)
        big.load_state_dict(net.state_dict())
        native = pc.NativeNetwork(big)
        del big
        x = torch.zeros(n ** 3, device="cuda")
        pc.normal_fcg_device(A, d, tp.lam, x, 3, 1e-6, native)  # warm-up
        x.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        it_l, rel_l = pc.normal_fcg_device(A, d, tp.lam, x, 20000, 1e-6, native)
        torch.cuda.synchronize()
        t_l = time.perf_counter() - t0
        out["learned_fcg"] = {"iterations": it_l, "seconds": t_l, "ms_per_iteration": 1e3 * t_l / max(it_l, 1),
                              "true_rel": rel_l, "time_ratio_vs_jacobi_cg": t_l / t_cg,
                              "time_ratio_vs_plain_cg": t_l / t_plain, "training": stats}
        native.close()
    A.close()
    return out


def run_sampled_rays(args):
    """The reference's Python inversion driver's traveltime forward model and
    gradient (midpoint-sampled straight rays, inversion.py:329-433) on 100^3
    cells of 200 m with 2000 sources x 1000 ocean-bottom stations (2M picks):
    pick-set build, device forward and gradient (CUDA events on the pick
    set's stream), the same through the host API (numpy in and out), and the
    oracle's single-thread C restatement on a bounded sample of the picks."""
    import torch
    import seismic_engine as se
    ps = se.workloads.obs_picks()
    t0 = time.perf_counter()
    rays = se.SampledRays(ps.model, ps.src_xyz, ps.sta_xyz, ps.weight)
    build_ms = 1e3 * (time.perf_counter() - t0)
    vp = torch.from_numpy(ps.vp.reshape(-1)).cuda()
    rng = np.random.default_rng(3)
    res = torch.from_numpy(rng.standard_normal(rays.n_picks) * 0.05).cuda()
    times = torch.empty(rays.n_picks, dtype=torch.float64, device="cuda")
    grad = torch.empty(rays.n_cells, dtype=torch.float64, device="cuda")
    stream = torch.cuda.ExternalStream(rays.stream_ptr())
    out = {"workload": f"{ps.name}: {rays.n_picks} picks, {rays.n_samples} midpoint samples on "
                       f"{ps.model[0]}^3 cells of {ps.model[3]:.0f} m (FP64, bit-exact vs the reference's formulas)",
           "n_picks": rays.n_picks, "n_samples": rays.n_samples, "build_ms": build_ms}
    for name, fn in (("forward", lambda: rays.forward_model(vp, out=times)),
                     ("gradient", lambda: rays.compute_gradient(vp, res, out=grad))):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(10):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / 10
        out[name] = {"ms": ms, "gsamples_per_s": rays.n_samples / ms / 1e6}
    vp_h = ps.vp.reshape(-1).copy()
    res_h = res.cpu().numpy()
    rays.forward_model(vp_h)
    t0 = time.perf_counter()
    t_h = rays.forward_model(vp_h)
    g_h = rays.compute_gradient(vp_h, res_h)
    out["host_api_ms"] = {"forward_plus_gradient": 1e3 * (time.perf_counter() - t0),
                          "h2d_bytes": int(2 * vp_h.nbytes + res_h.nbytes), "d2h_bytes": int(t_h.nbytes + g_h.nbytes)}
    out["host_matches_device"] = bool(np.array_equal(t_h, times.cpu().numpy()) and
                                      np.array_equal(g_h, grad.cpu().numpy()))
    # the whole driver (inversion.py:118-274) on the device: 3 iterations of forward, misfit, gradient,
    # smoothing, regularisation, normalisation and a 10-trial line search, observed times = the
    # forward model of a perturbed model
    from types import SimpleNamespace
    from seismic_engine.inversion import AdjointStateInversion
    n = ps.model[0]
    model = SimpleNamespace(nx=n, ny=n, nz=n, dx=ps.model[3], dy=ps.model[4], dz=ps.model[5],
                            origin_x=0.0, origin_y=0.0, origin_z=0.0, vp=ps.vp.copy(), vp_min=1450.0,
                            vp_max=8500.0)
    t_obs = rays.forward_model(vp * 1.02).cpu().numpy()
    obs = SimpleNamespace(picks=[])
    # one untimed iteration first: the first use of each torch operation in a process loads its kernels
    warm_model = SimpleNamespace(**{**vars(model), "vp": model.vp.copy()})  # the driver updates model.vp
    warm = AdjointStateInversion(warm_model, obs, None, max_iterations=1, step_length=10.0, smoothing_sigma=2.0,
                                 misfit_type="l2", rays=rays, observed=t_obs, weights=ps.weight)
    warm.run()
    inv = AdjointStateInversion(model, obs, None, max_iterations=3, step_length=10.0, smoothing_sigma=2.0,
                                misfit_type="l2", rays=rays, observed=t_obs, weights=ps.weight)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    res_inv = inv.run()
    torch.cuda.synchronize()
    out["driver"] = {"iterations": res_inv["iterations"], "ms_per_iteration": 1e3 * (time.perf_counter() - t0) /
                     max(res_inv["iterations"], 1), "misfit_history": res_inv["misfit_history"]}
    if not args.no_cpu_baseline:
        from oracle import Oracle
        orc = Oracle()
        k = 100_000
        n = np.array(ps.model[:3])
        d = np.array(ps.model[3:6])
        o = np.array(ps.model[6:9])
        t0 = time.perf_counter()
        orc.sampled_traveltimes(n, d, o, ps.src_xyz[:k], ps.sta_xyz[:k], None, ps.vp)
        orc.sampled_gradient(n, d, o, ps.src_xyz[:k], ps.sta_xyz[:k], None, ps.weight[:k], ps.vp, res_h[:k])
        cpu_s = (time.perf_counter() - t0) * rays.n_picks / k
        gpu_s = (out["forward"]["ms"] + out["gradient"]["ms"]) / 1e3
        out["cpu_baseline"] = {"kind": "port", "cores": 1, "sample": f"first {k} picks, scaled to all",
                               "forward_plus_gradient_s": cpu_s, "gpu_speedup": cpu_s / gpu_s}
    rays.close()
    return out


# ---------------------------------------------------------------- GPU leg
def run_gpu(args):
    import torch
    import seismic_engine as se
    from seismic_engine import _lib

    world, rank, local = dist_setup(args)
    w = workload(args.n, args.nt)
    shot = w.shots[0]
    rec = shot.rec
    snap_kind = {"bf16": _lib.ST_SNAP_BF16, "fp16": _lib.ST_SNAP_FP16, "fp32": _lib.ST_SNAP_FP32}[args.snap]
    grid = se.GridParams(w.nx, w.ny, w.nz, w.d, w.d, w.d)
    cfg = se.SolverConfig(dt=w.dt, nt=w.nt, sponge_width=w.sponge_width, sponge_damping=w.sponge_damping,
                          sponge_mode=w.sponge_mode)
    s = se.WaveEquationSolver(grid, cfg, device=torch.cuda.current_device())
    s.set_step_fusion(args.fused_steps)
    vel_true = se.workloads.to_reference_layout(w.vel)
    vel_mig = se.workloads.to_reference_layout(w.vel_migration)
    # observed data (input preparation, untimed)
    s.set_velocity_field(vel_true)
    data = torch.zeros((w.nt, rec.count), device="cuda")
    se.shot_forward(s, shot.src, shot.wavelet, w.nt, rec, seis=data)
    s.set_velocity_field(vel_mig)
    npts = w.nx * w.ny * w.nz
    image = torch.zeros(npts, device="cuda")
    illum = torch.zeros(npts, device="cuda")
    refl = torch.zeros(npts, device="cuda")
    stream = torch.cuda.ExternalStream(s.stream_ptr())
    L = _lib.load()

    def step():
        se.rtm_shot(s, shot.src, shot.wavelet, w.nt, rec, data, image, illum, refl, snap_kind=snap_kind)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    import ctypes as C
    lc0 = C.c_longlong()
    L.st_launch_count(C.byref(lc0))
    ph = (C.c_float * 2)()
    fwd_ms, bwd_ms = [], []
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(torch.cuda.current_device()) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            step()
            L.st_solver_last_phase_ms(s.handle, ph)
            fwd_ms.append(ph[0])
            bwd_ms.append(ph[1])
        ev1.record(stream)
        torch.cuda.synchronize()
    barrier(world)
    el_ms = max_over_ranks(ev0.elapsed_time(ev1), world)
    lc1 = C.c_longlong()
    L.st_launch_count(C.byref(lc1))
    launches = lc1.value - lc0.value
    pts_step = 2.0 * w.nt * npts
    value = world * pts_step * args.steps / (el_ms / 1e3) / 1e9
    hbm_peak, peak_kind = measured_peaks()
    # both passes run nt / 2 two-step launches (an odd nt adds one single step)
    paired = args.fused_steps == 2 and w.nt % 2 == 0 and w.nz % 8 == 0
    fwd_bytes, bwd_bytes = alg_bytes(args.snap, paired)
    snap = args.snap.upper()
    if paired:
        bwd_kernel = f"fd_step2_kernel<adjoint, {snap}> (two adjoint steps + imaging)"
        fwd_kernel = f"fd_step2_kernel<forward, {snap}> (two forward steps + snapshot stores)"
        launches_per_pass, traffic_key = w.nt // 2, "fd_step2_image_bf16_256"
        traffic_key_fwd = "fd_step2_forward_bf16_256"
    else:
        bwd_kernel = f"fd_step_kernel<SNAP_NONE, {snap}, imaging> (adjoint step + imaging)"
        fwd_kernel = f"fd_step_kernel<{snap}, NONE> (forward step + snapshot store)"
        launches_per_pass, traffic_key = w.nt, "fd_step_adjoint_image_bf16_256"
        traffic_key_fwd = "fd_step_forward_bf16_256"
    bwd_launch_ms = statistics.mean(bwd_ms) / launches_per_pass
    fwd_launch_ms = statistics.mean(fwd_ms) / launches_per_pass
    bw_bwd = bwd_bytes * npts / (bwd_launch_ms / 1e3) / 1e9
    bw_fwd = fwd_bytes * npts / (fwd_launch_ms / 1e3) / 1e9
    alg_total = (fwd_bytes + bwd_bytes) * launches_per_pass * npts * args.steps
    traffic = profile_traffic(traffic_key) if args.snap == "bf16" and w.nx == 256 else None
    traffic_fwd = profile_traffic(traffic_key_fwd) if args.snap == "bf16" and w.nx == 256 else None
    line = {
        "metric": METRIC, "value": value, "unit": "Gpts/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": el_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded layered model + Gaussian anomalies, Ricker source)",
        "config": config_dict(w, args.snap, world),
        "hbm_gbs_algorithmic": alg_total / (el_ms / 1e3) / 1e9,
        "roofline": {"bound": "hbm", "kernel": bwd_kernel,
                     "achieved": bw_bwd, "peak": hbm_peak, "unit": "GB/s", "frac": bw_bwd / hbm_peak,
                     "peak_kind": f"{peak_kind} copy bandwidth", "traffic": traffic,
                     "alg_bytes_per_launch": bwd_bytes * npts, "launch_ms": bwd_launch_ms,
                     "steps_per_launch": 2 if paired else 1},
        "roofline_forward": {"bound": "hbm", "kernel": fwd_kernel,
                             "achieved": bw_fwd, "peak": hbm_peak, "unit": "GB/s", "frac": bw_fwd / hbm_peak,
                             "traffic": traffic_fwd, "alg_bytes_per_launch": fwd_bytes * npts, "launch_ms": fwd_launch_ms,
                             "steps_per_launch": 2 if paired else 1},
        "phases_ms_per_step": {"forward": statistics.mean(fwd_ms), "backward": statistics.mean(bwd_ms)},
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    if not args.no_e2e:
        # the same metric through the host C-ABI entry: velocity and receiver data copied in from pinned
        # host memory, the image copied out, every step
        vel_pin = torch.from_numpy(vel_mig).pin_memory()
        data_pin = data.cpu().pin_memory()
        img_pin = torch.empty(npts, dtype=torch.float64).pin_memory()  # the caller's reused image buffer
        times = []
        out = None
        for i in range(1 + args.steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            out = se.rtm_shot_host(s, vel_pin.numpy(), shot.src, shot.wavelet, w.nt, rec, data_pin.numpy(),
                                   snap_kind=snap_kind, want=("image",), out={"image": img_pin.numpy()})
            torch.cuda.synchronize()
            if i > 0:
                times.append(time.perf_counter() - t0)
        e2e_s = max_over_ranks(sum(times), world)
        line["e2e"] = {"value": world * pts_step * args.steps / e2e_s / 1e9, "unit": "Gpts/s",
                       "h2d_bytes_per_step": int(vel_mig.nbytes + data_pin.numel() * 4),
                       "d2h_bytes_per_step": int(npts * 8),
                       "api": "st_rtm_shot_host (include/seismic_gb300.h)"}
        img_dev = image.cpu().numpy().astype(np.float64)
        line["e2e"]["matches_device_path"] = bool(
            np.allclose(out["image"], img_dev, rtol=1e-5, atol=1e-6 * np.abs(img_dev).max()))
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(w, args.cpu_seconds)
    s.close()
    if rank == 0 and world == 1 and not args.no_512:
        del image, illum, refl, data
        torch.cuda.empty_cache()
        line["roofline_512"] = run_512_leg(args)
    if rank == 0 and world == 1 and not args.no_large:
        torch.cuda.empty_cache()
        line["large_iteration"] = large_iteration(args)
    if rank == 0 and world == 1 and not args.no_tomo:
        torch.cuda.empty_cache()
        line["tomography"] = run_tomography(args)
    if rank == 0 and world == 1 and not args.no_rays:
        torch.cuda.empty_cache()
        line["sampled_rays"] = run_sampled_rays(args)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def run_512_leg(args, nt=200):
    """The propagator kernels at 512^3 (the large workload's grid and model,
    its first shot and 256x256 receivers): a 200-step BF16 RTM shot with two
    steps per launch and one with one step per launch; per-launch times from
    the passes' CUDA events, algorithmic bytes as the headline roofline."""
    import torch
    import seismic_engine as se
    from seismic_engine import _lib
    import ctypes as C
    w = se.workloads.large_512(nt=nt)
    sh = w.shots[0]
    n = w.nx
    cfg = se.SolverConfig(dt=w.dt, nt=nt, sponge_width=w.sponge_width, sponge_damping=w.sponge_damping,
                          sponge_mode=w.sponge_mode)
    s = se.WaveEquationSolver(se.GridParams(n, n, n, w.d, w.d, w.d), cfg)
    s.set_velocity_field(se.workloads.to_reference_layout(w.vel))
    data = torch.randn((nt, sh.rec.count), device="cuda", generator=torch.Generator("cuda").manual_seed(5)) * 1e-3
    npts = n ** 3
    image, illum = torch.zeros(npts, device="cuda"), torch.zeros(npts, device="cuda")
    L = _lib.load()
    peak, kind = measured_peaks()
    out = {"workload": f"{w.name} model, shot 0, {nt} steps, BF16 snapshots, {sh.rec.nx}x{sh.rec.ny} receivers",
           "peak": peak, "peak_kind": f"{kind} copy bandwidth", "unit": "GB/s"}
    for fused in (2, 1):
        s.set_step_fusion(fused)
        ph = (C.c_float * 2)()
        fwd, bwd, tot = [], [], []
        for i in range(3):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            st = torch.cuda.ExternalStream(s.stream_ptr())
            e0.record(st)
            se.rtm_shot(s, sh.src, sh.wavelet, nt, sh.rec, data, image, illum, snap_kind=_lib.ST_SNAP_BF16)
            e1.record(st)
            torch.cuda.synchronize()
            L.st_solver_last_phase_ms(s.handle, ph)
            if i > 0:
                fwd.append(ph[0])
                bwd.append(ph[1])
                tot.append(e0.elapsed_time(e1))
        launches = nt // fused
        fb, bb = alg_bytes("bf16", fused == 2)
        f_ms, b_ms = statistics.mean(fwd) / launches, statistics.mean(bwd) / launches
        key = "pair" if fused == 2 else "one_step"
        out[key] = {
            "forward": {"launch_ms": f_ms, "alg_bytes_per_launch": fb * npts,
                        "achieved": fb * npts / f_ms / 1e6, "frac": fb * npts / f_ms / 1e6 / peak},
            "adjoint_imaging": {"launch_ms": b_ms, "alg_bytes_per_launch": bb * npts,
                                "achieved": bb * npts / b_ms / 1e6, "frac": bb * npts / b_ms / 1e6 / peak},
            "shot_gpts_per_s": 2.0 * nt * npts / (statistics.mean(tot) / 1e3) / 1e9,
        }
    s.close()
    return out


def large_iteration(args):
    """One iteration of the large workload (512^3, 8 shots x 4000 steps,
    checkpointed BF16 adjoint gradient, PCG update on 256^3) as in
    `--workload large`; returns its timing dictionary."""
    import types
    a = types.SimpleNamespace(**vars(args))
    a.nt, a.compare = 4000, False
    return _large(a)


def run_kernel(args):
    """Single-kernel timing for profiling: 'conv' = the tensor-core 3x3x3
    32 -> 32 convolution on a 100^3 volume; 'wgrad' = its tensor-core weight
    gradient on the same volume; 'fwigrad' = one shot's FWI gradient on the 256^3
    workload (--nt steps, 400 by default); 'spmv' = A x and A^T y of the
    100^3 / 2M-ray tomography matrix; 'rays' = the sampled-ray forward model
    and gradient of 2M picks. Prints one JSON line."""
    import ctypes as C
    import torch
    import seismic_engine as se
    from seismic_engine import _lib
    L = _lib.load()
    st = torch.cuda.current_stream()
    res = {"kernel": args.kernel, "steps": args.steps, "warmup": args.warmup}
    if args.kernel == "conv":
        n = 100
        g = torch.Generator(device="cuda").manual_seed(0)
        x = torch.zeros((n + 2, n + 2, n + 2, 32), dtype=torch.bfloat16, device="cuda")
        x[1:-1, 1:-1, 1:-1] = torch.randn((n, n, n, 32), device="cuda", generator=g).to(torch.bfloat16)
        y = torch.zeros_like(x)
        w = torch.randn((32, 32, 3, 3, 3), device="cuda", generator=g) / 30
        wp = torch.empty(27 * 32 * 32, dtype=torch.bfloat16, device="cuda")
        L.st_conv3d_pack_weights(C.c_void_p(w.data_ptr()), C.c_void_p(wp.data_ptr()), 0, C.c_void_p(st.cuda_stream))

        def one():
            rc = L.st_conv3d_bf16(C.c_void_p(x.data_ptr()), C.c_void_p(wp.data_ptr()), None, C.c_void_p(x.data_ptr()),
                                  C.c_void_p(y.data_ptr()), 0, n, n, n, 0, C.c_void_p(st.cuda_stream))
            assert rc == 0
        flops = 2.0 * n ** 3 * 32 * 32 * 27
        res.update({"workload": f"3x3x3 conv, 32 -> 32 channels, BF16 operands, {n}^3 voxels", "flops": flops})
    elif args.kernel == "wgrad":
        n = 100
        g = torch.Generator(device="cuda").manual_seed(0)
        x = torch.zeros((n + 2, n + 2, n + 2, 32), dtype=torch.bfloat16, device="cuda")
        x[1:-1, 1:-1, 1:-1] = torch.randn((n, n, n, 32), device="cuda", generator=g).to(torch.bfloat16)
        gy = torch.zeros_like(x)
        gy[1:-1, 1:-1, 1:-1] = torch.randn((n, n, n, 32), device="cuda", generator=g).to(torch.bfloat16)
        dw = torch.zeros(32 * 32 * 27, device="cuda")

        def one():
            rc = L.st_conv3d_wgrad(C.c_void_p(x.data_ptr()), C.c_void_p(gy.data_ptr()), C.c_void_p(dw.data_ptr()), n, n,
                                   n, C.c_void_p(st.cuda_stream))
            assert rc == 0
        # the GEMM runs over every padded row (the border rows contribute zero)
        flops = 2.0 * (n + 2) ** 3 * 32 * 32 * 27
        res.update({"workload": f"3x3x3 conv weight gradient, 32 -> 32 channels, BF16 operands, {n}^3 voxels",
                    "flops": flops})
    elif args.kernel == "fwigrad":
        import seismic_engine.fwi as fwi
        nt_ = args.nt if args.nt != 2000 else 400
        w = se.workloads.rtm_256(nt=nt_)
        cfg = se.SolverConfig(dt=w.dt, nt=nt_, sponge_width=w.sponge_width, sponge_damping=w.sponge_damping,
                              sponge_mode=w.sponge_mode)
        s = se.WaveEquationSolver(se.GridParams(w.nx, w.ny, w.nz, w.d, w.d, w.d), cfg)
        fwi.set_velocity_device(s, torch.from_numpy(w.vel.astype(np.float32)).cuda())
        sh = w.shots[0]
        d_obs = torch.zeros((nt_, sh.rec.count), device="cuda")
        se.shot_forward(s, sh.src, sh.wavelet, nt_, sh.rec, seis=d_obs)
        d_obs *= 1.01
        gv = torch.zeros(w.points, device="cuda")
        st = torch.cuda.ExternalStream(s.stream_ptr())

        def one():
            fwi.fwi_gradient(s, sh.src, sh.wavelet, nt_, sh.rec, d_obs, gv, snap_kind=_lib.ST_SNAP_BF16)
        res.update({"workload": f"FWI gradient of one shot, {w.name}, {nt_} steps, BF16 snapshots (forward + "
                                f"adjoint with the gradient epilogue)", "steps_per_call": nt_})
    elif args.kernel == "rays":
        ps = se.workloads.obs_picks()
        rays = se.SampledRays(ps.model, ps.src_xyz, ps.sta_xyz, ps.weight)
        vp = torch.from_numpy(ps.vp.reshape(-1)).cuda()
        rs = torch.from_numpy(np.random.default_rng(3).standard_normal(rays.n_picks) * 0.05).cuda()
        tt = torch.empty(rays.n_picks, dtype=torch.float64, device="cuda")
        gg = torch.empty(rays.n_cells, dtype=torch.float64, device="cuda")

        def one():
            rays.forward_model(vp, out=tt)
            rays.compute_gradient(vp, rs, out=gg)
        res.update({"workload": f"sampled-ray forward + gradient, {rays.n_picks} picks, {rays.n_samples} samples"})
        st = torch.cuda.ExternalStream(rays.stream_ptr())
        one()
        torch.cuda.synchronize()
        for name, fn in (("forward_ms", lambda: rays.forward_model(vp, out=tt)),
                         ("gradient_ms", lambda: rays.compute_gradient(vp, rs, out=gg))):
            f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            f0.record(st)
            for _ in range(max(args.steps, 1)):
                fn()
            f1.record(st)
            torch.cuda.synchronize()
            res[name] = f0.elapsed_time(f1) / max(args.steps, 1)
    else:
        nt_, nr_ = args.tomo_n, args.tomo_rays
        A = se.CSRMatrix()
        nnz = A.build_ray_matrix(torch.from_numpy(se.workloads.ray_endpoints(nr_, nt_, 4)).cuda(), nt_, nt_, nt_)
        xv = torch.randn(A.cols(), device="cuda")
        yv = torch.zeros(A.rows(), device="cuda")
        zv = torch.zeros(A.cols(), device="cuda")

        def one():
            A.spmv_device(xv, yv)
            A.spmv_device(yv, zv, transpose=True)
        res.update({"workload": f"A x and A^T y, {A.rows()} x {A.cols()}, nnz {nnz}",
                    "alg_bytes": 2 * nnz * 8 + (A.rows() + A.cols()) * 16})
        st = torch.cuda.ExternalStream(A.stream_ptr())  # the SpMV kernels run on the matrix's stream
        one()
        torch.cuda.synchronize()
        for name, fn in (("A_ms", lambda: A.spmv_device(xv, yv)),
                         ("AT_ms", lambda: A.spmv_device(yv, zv, transpose=True))):
            f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            f0.record(st)
            for _ in range(max(args.steps, 1)):
                fn()
            f1.record(st)
            torch.cuda.synchronize()
            res[name] = f0.elapsed_time(f1) / max(args.steps, 1)
    for _ in range(args.warmup):
        one()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(args.steps):
        one()
    e1.record(st)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    res["ms"] = ms
    if "flops" in res:
        res["tflops"] = res["flops"] / ms / 1e9
    if "alg_bytes" in res:
        res["gbs"] = res["alg_bytes"] / ms / 1e6
    if "steps_per_call" in res:
        res["ms_per_step"] = ms / res["steps_per_call"]
    if args.kernel == "conv":
        assert L.st_conv3d_check(C.c_void_p(st.cuda_stream)) == 0
    print(json.dumps(res), flush=True)
    return 0


def laplacian_csr(n, mu=1.0):
    """sqrt(mu) L for the 7-point Laplacian L on an n^3 grid (Dirichlet), built
    by the FD-stencil builder with v dt / d = 1 (off-diagonals 1, diagonal
    2 - 6) and a diagonal shift of -2."""
    import seismic_engine as se
    A = se.CSRMatrix()
    A.build_fd_stencil_7point(n, n, n, np.full(n ** 3, 1.0), 1.0, 1.0, 1.0, 1.0)
    A.add_diagonal(-2.0)
    if mu != 1.0:
        A.scale(float(np.sqrt(mu)))
    return A


def run_large(args):
    """One adjoint tomography iteration on the 512^3 workload (see _large).
    Prints one JSON line."""
    line = _large(args)
    print(json.dumps(line), flush=True)
    return 0


def _large(args):
    """One adjoint tomography iteration on the 512^3 workload: 8 shots one
    after another, each forward + checkpointed adjoint gradient (BF16 segment
    snapshots), the summed velocity gradient restricted to a 256^3 inversion
    grid (2x2x2 means) and a Jacobi-PCG model update (I + mu L^T L) x = g,
    L the 7-point Laplacian (mu = 1)."""
    import torch
    import seismic_engine as se
    import seismic_engine.fwi as fwi
    nt = args.nt if args.nt != 2000 else 4000
    w = se.workloads.large_512(nt=nt)
    n = w.nx
    cfg = se.SolverConfig(dt=w.dt, nt=nt, sponge_width=w.sponge_width, sponge_damping=w.sponge_damping,
                          sponge_mode=w.sponge_mode)
    s = se.WaveEquationSolver(se.GridParams(n, n, n, w.d, w.d, w.d), cfg)
    s.set_step_fusion(args.fused_steps)
    v_true = torch.from_numpy(w.vel.astype(np.float32)).cuda()
    v0 = torch.from_numpy(se.workloads.smooth(w.vel, 6.0).astype(np.float32)).cuda()
    fwi.set_velocity_device(s, v_true)
    d_obs = []
    for sh in w.shots:  # observed data (input preparation, untimed)
        d = torch.zeros((nt, sh.rec.count), device="cuda")
        se.shot_forward(s, sh.src, sh.wavelet, nt, sh.rec, seis=d)
        d_obs.append(d)
    torch.cuda.synchronize()
    fwi.set_velocity_device(s, v0)
    L = laplacian_csr(n // 2)
    slots = -(-nt // args.segment)

    def iteration(kind, jacobi):
        g = torch.zeros(w.points, device="cuda")
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        misfit = 0.0
        for sh, d in zip(w.shots, d_obs):
            misfit += fwi.fwi_gradient(s, sh.src, sh.wavelet, nt, sh.rec, d, g, snap_kind=kind,
                                       checkpoint=(args.segment, slots))
        torch.cuda.synchronize()
        t_grad = time.perf_counter() - t0
        gr = torch.nn.functional.avg_pool3d(g.reshape(1, 1, n, n, n), 2).reshape(-1).contiguous()
        x = torch.zeros_like(gr)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        it, rel, true_rel = se.normal_cg_device(L, None, 1.0, x, 5000, 1e-6, jacobi, rhs=gr.clone())
        torch.cuda.synchronize()
        t_cg = time.perf_counter() - t1
        return {"seconds": t_grad + t_cg, "gradient_s": t_grad, "cg_s": t_cg, "cg_iterations": it,
                "cg_true_rel": true_rel, "misfit": misfit}

    res = iteration(_snap("bf16"), True)
    # forward sweep + recompute + adjoint steps of every shot
    pts = float(w.points) * nt * 3 * len(w.shots)
    line = {"metric": "adjoint tomography iteration", "value": res["seconds"], "unit": "s",
            "higher_is_better": False, "n_gpus": 1, "dtype": "f32",
            "config": {"workload": f"{w.name} x {nt} steps, {len(w.shots)} shots, 256x256 receivers, "
                                   f"checkpointed adjoint (segments of {args.segment}, BF16 snapshots), "
                                   f"PCG (I + L^T L) update on a {n // 2}^3 grid"},
           "gpts_per_s": pts / res["gradient_s"] / 1e9, "bf16_checkpointed_pcg": res}
    if args.compare:
        line["fp32_checkpointed"] = iteration(_snap("fp32"), True)
        line["plain_cg"] = iteration(_snap("bf16"), False)
    s.close()
    L.close()
    return line


def _snap(name):
    from seismic_engine import _lib
    return {"bf16": _lib.ST_SNAP_BF16, "fp16": _lib.ST_SNAP_FP16, "fp32": _lib.ST_SNAP_FP32}[name]


def launch_replicas(n, argv):
    """`--gpus N` run outside torchrun: start N replica processes through
    torch.distributed.run (one per GPU, LOCAL_RANK = device, rendezvous on
    127.0.0.1); rank 0 prints the JSON line. Returns their exit status."""
    import socket
    with socket.socket() as so:
        so.bind(("127.0.0.1", 0))
        port = so.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={n}",
           "--master-addr", "127.0.0.1", f"--master-port={port}", os.path.abspath(__file__), *argv]
    return subprocess.call(cmd)


def run_dry(args):
    """The replica plumbing of run_gpu without GPU work: each rank times a
    token sleep; the line carries the max over ranks."""
    world, rank, _ = dist_setup(args)
    barrier(world)
    t0 = time.perf_counter()
    time.sleep(0.01 * (1 + rank))
    el = max_over_ranks(time.perf_counter() - t0, world)
    barrier(world)
    if rank == 0:
        print(json.dumps({"dry_run": True, "n_gpus": world, "max_rank_seconds": el}), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        return launch_replicas(args.gpus, sys.argv[1:])
    if args.dry_run:
        return run_dry(args)
    if args.kernel:
        return run_kernel(args)
    if args.workload == "large":
        return run_large(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
