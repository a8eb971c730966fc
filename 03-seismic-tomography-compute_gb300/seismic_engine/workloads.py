"""Seeded synthetic inputs of the benchmark workloads: layered velocity models
with Gaussian anomalies, the CFL time-step rule, the Ricker wavelet and the
surface receiver grids. There is no public dataset for this path; these
generators stand in for field data with the stated shapes and value ranges.

Velocity arrays are (nx, ny, nz) with z as depth (z fastest, the reference's
index order, core/grid.cpp:45-49); `to_reference_layout` pads them to the
reference's halo-padded layout with edge values.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np


def ricker(f0: float, dt: float, nt: int, t0: float | None = None) -> np.ndarray:
    """w(t) = (1 - 2 pi^2 f0^2 tau^2) exp(-pi^2 f0^2 tau^2), tau = n dt - t0,
    t0 = 1.2 / f0 by default."""
    t0 = 1.2 / f0 if t0 is None else t0
    tau = np.arange(nt) * dt - t0
    a = (math.pi * f0 * tau) ** 2
    return (1.0 - 2.0 * a) * np.exp(-a)


def cfl_dt(d: float, vmax: float, courant: float = 0.45) -> float:
    """dt = floor_1e-6(courant * d / vmax); the reference accepts
    vmax dt / d <= 0.49 per axis (core/fault_tolerance.cpp:49-70)."""
    return math.floor(courant * d / vmax * 1e6) / 1e6


def layered(nx: int, ny: int, nz: int, velocities) -> np.ndarray:
    """Equal-thickness horizontal layers along z (depth)."""
    v = np.empty((nx, ny, nz), np.float64)
    L = len(velocities)
    bounds = [int(math.ceil(k * nz / L)) for k in range(L + 1)]
    for k, vel in enumerate(velocities):
        v[:, :, bounds[k]:bounds[k + 1]] = vel
    return v


def add_gaussian(v: np.ndarray, centre, amp: float, sigma: float) -> np.ndarray:
    """v *= 1 + amp exp(-r^2 / (2 sigma^2)) around centre (cell units)."""
    nx, ny, nz = v.shape
    x = np.arange(nx)[:, None, None] - centre[0]
    y = np.arange(ny)[None, :, None] - centre[1]
    z = np.arange(nz)[None, None, :] - centre[2]
    v *= 1.0 + amp * np.exp(-(x * x + y * y + z * z) / (2.0 * sigma * sigma))
    return v


def random_anomalies(v: np.ndarray, count: int, seed: int, amp: float = 0.10, sigma: float = 8.0):
    """`count` anomalies with centres uniform in the central 50% of each axis
    and amplitude +-amp (random sign)."""
    rng = np.random.default_rng(seed)
    n = np.array(v.shape)
    for _ in range(count):
        c = rng.uniform(0.25 * n, 0.75 * n)
        s = 1.0 if rng.random() < 0.5 else -1.0
        add_gaussian(v, c, s * amp, sigma)
    return v


def smooth(v: np.ndarray, sigma: float) -> np.ndarray:
    from scipy.ndimage import gaussian_filter
    return gaussian_filter(v, sigma=sigma, mode="nearest")


def to_reference_layout(v: np.ndarray) -> np.ndarray:
    """(nx,ny,nz) interior -> flat (nx+2)*(ny+2)*(nz+2) padded array (edge halo)."""
    return np.ascontiguousarray(np.pad(v, 1, mode="edge")).reshape(-1)


@dataclass
class ReceiverGrid:
    """Receiver q = irx*ny + iry at (x0 + irx*sx, y0 + iry*sy, z)."""
    x0: int
    sx: int
    nx: int
    y0: int
    sy: int
    ny: int
    z: int

    @property
    def count(self) -> int:
        return self.nx * self.ny

    def coords(self) -> np.ndarray:
        ix = self.x0 + self.sx * np.arange(self.nx)
        iy = self.y0 + self.sy * np.arange(self.ny)
        X, Y = np.meshgrid(ix, iy, indexing="ij")
        return np.stack([X.ravel(), Y.ravel(), np.full(X.size, self.z)], axis=1).astype(np.int64)


@dataclass
class ShotSpec:
    src: tuple
    wavelet: np.ndarray
    rec: ReceiverGrid


@dataclass
class Workload:
    name: str
    nx: int
    ny: int
    nz: int
    d: float
    dt: float
    nt: int
    vel: np.ndarray          # (nx,ny,nz) true model
    shots: list
    sponge_width: int = 20
    sponge_damping: float = 0.015
    vel_migration: np.ndarray | None = None
    # "reference": the reference's sponge rule, which diverges on a 20-cell,
    # 0.015 sponge within a few hundred steps; "stable": the Cerjan form.
    sponge_mode: str = "reference"

    @property
    def points(self) -> int:
        return self.nx * self.ny * self.nz


def forward_128(nt: int = 1000) -> Workload:
    """128^3 forward modelling: 3 layers 1500/2500/3500 m/s, +10% Gaussian
    anomaly (sigma 8 cells) at the centre, 15 Hz Ricker at (64,64,5), 64x64
    receivers every 2nd cell on z = 5."""
    n = 128
    v = layered(n, n, n, [1500.0, 2500.0, 3500.0])
    add_gaussian(v, (64, 64, 64), 0.10, 8.0)
    dt = cfl_dt(10.0, 3500.0)
    rec = ReceiverGrid(0, 2, 64, 0, 2, 64, 5)
    return Workload("forward-128^3", n, n, n, 10.0, dt, nt, v, [ShotSpec((64, 64, 5), ricker(15.0, dt, nt), rec)])


def rtm_256(nt: int = 2000) -> Workload:
    """256^3 single-shot RTM: 4 layers 1500..4500 m/s, two seeded (seed 2)
    +-10% anomalies, source (128,128,5), 128x128 receivers every 2nd cell on
    z = 5, migration velocity = true model smoothed with sigma 6 cells."""
    n = 256
    v = layered(n, n, n, [1500.0, 2500.0, 3500.0, 4500.0])
    random_anomalies(v, 2, seed=2)
    vmax = float(v.max())
    dt = cfl_dt(10.0, vmax)
    rec = ReceiverGrid(0, 2, 128, 0, 2, 128, 5)
    w = Workload("rtm-256^3", n, n, n, 10.0, dt, nt, v, [ShotSpec((128, 128, 5), ricker(15.0, dt, nt), rec)],
                 sponge_mode="stable")
    return w


def fwi_192(nt: int = 1500) -> Workload:
    """192^3 FWI: 4 layers + 2 seeded (seed 3) anomalies; 4 shots on a 2x2
    surface grid; start model = true model smoothed with sigma 6 cells."""
    n = 192
    v = layered(n, n, n, [1500.0, 2500.0, 3500.0, 4500.0])
    random_anomalies(v, 2, seed=3)
    dt = cfl_dt(10.0, float(v.max()))
    rec = ReceiverGrid(0, 2, 96, 0, 2, 96, 5)
    w = ricker(15.0, dt, nt)
    shots = [ShotSpec((sx, sy, 5), w, rec) for sx in (64, 128) for sy in (64, 128)]
    return Workload("fwi-192^3", n, n, n, 10.0, dt, nt, v, shots, sponge_mode="stable")


def large_512(nt: int = 4000) -> Workload:
    """512^3: 6 layers 1500..5000 m/s + 6 seeded (seed 5) anomalies, 20 Hz
    Ricker, 8 shots on a 2x4 surface grid at z = 5, 256x256 receivers."""
    n = 512
    v = layered(n, n, n, list(np.linspace(1500.0, 5000.0, 6)))
    random_anomalies(v, 6, seed=5)
    dt = cfl_dt(10.0, float(v.max()))
    rec = ReceiverGrid(0, 2, 256, 0, 2, 256, 5)
    w = ricker(20.0, dt, nt)
    shots = [ShotSpec((int(sx), int(sy), 5), w, rec) for sx in (170, 341) for sy in (102, 204, 307, 409)]
    return Workload("large-512^3", n, n, n, 10.0, dt, nt, v, shots, sponge_mode="stable")


def small_case(n=(24, 20, 28), nt: int = 80, seed: int = 7, sponge_width: int = 6) -> Workload:
    """Small seeded case for parity tests (the oracle finishes it in
    milliseconds): 2 layers + one anomaly, Ricker at the upper centre,
    receivers every 3rd cell on z = 3."""
    nx, ny, nz = n
    v = layered(nx, ny, nz, [1500.0, 2400.0])
    rng = np.random.default_rng(seed)
    add_gaussian(v, (nx / 2, ny / 2, nz / 2), 0.1, 3.0)
    v *= 1.0 + 0.02 * rng.standard_normal(v.shape)
    dt = cfl_dt(10.0, float(v.max()))
    rec = ReceiverGrid(1, 3, (nx - 2) // 3, 1, 3, (ny - 2) // 3, 3)
    w = ricker(25.0, dt, nt)
    return Workload("small", nx, ny, nz, 10.0, dt, nt, v,
                    [ShotSpec((nx // 2, ny // 2, 4), w, rec)], sponge_width=sponge_width)


# ------------------------------------------------------------ traveltime tomography

@dataclass
class RayTomography:
    """Straight-ray traveltime tomography on an n^3 cell grid: ray endpoints
    (cell units), the true model x_true, the damping lam, and the seeds of
    the data noise."""
    name: str
    n: int
    ends: np.ndarray      # [n_rays, 6] FP64: x0 y0 z0 x1 y1 z1
    x_true: np.ndarray    # n^3 FP64, x slowest
    lam: float
    noise_seed: int
    noise_level: float = 0.01


def _morton2(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Interleaved bits of two non-negative integer arrays (Z-order key)."""
    key = np.zeros(a.shape, np.uint64)
    a = a.astype(np.uint64)
    b = b.astype(np.uint64)
    for bit in range(16):
        key |= ((a >> np.uint64(bit)) & np.uint64(1)) << np.uint64(2 * bit + 1)
        key |= ((b >> np.uint64(bit)) & np.uint64(1)) << np.uint64(2 * bit)
    return key


def ray_endpoints(n_rays: int, n: int = 100, seed: int = 4, spatial_order: bool = True) -> np.ndarray:
    """Sources uniform on the surface z = 0; receivers in one of four vertical
    boreholes at cells (0.1n, 0.1n), (0.1n, 0.9n), (0.9n, 0.1n), (0.9n, 0.9n)
    (cell centres), depth uniform in [0, n). Each ray goes to the borehole
    diagonally opposite its source quadrant, which lengthens the paths to
    about 1.8 n cells crossed per ray.

    spatial_order lists the rays by borehole, then source cell in Z order,
    then receiver depth, so rays that share cells sit close together (a
    better cache footprint for the SpMV gathers). The set of rays is the
    same; the damped normal equations do not depend on their order."""
    rng = np.random.default_rng(seed)
    xs = rng.uniform(0.0, n, n_rays)
    ys = rng.uniform(0.0, n, n_rays)
    zr = rng.uniform(0.0, n, n_rays)
    near, far = int(0.1 * n) + 0.5, int(0.9 * n) + 0.5
    bx = np.where(xs < 0.5 * n, far, near)
    by = np.where(ys < 0.5 * n, far, near)
    ends = np.stack([xs, ys, np.zeros(n_rays), bx, by, zr], axis=1)
    if spatial_order:
        hole = (bx > 0.5 * n).astype(np.int64) * 2 + (by > 0.5 * n).astype(np.int64)
        src = _morton2(np.floor(xs).astype(np.int64), np.floor(ys).astype(np.int64))
        order = np.lexsort((zr, src, hole))
        ends = ends[order]
    return ends


def smooth_model(n: int, sigma: float, seed: int) -> np.ndarray:
    """Seeded white noise smoothed with a Gaussian (sigma cells), unit std."""
    from scipy.ndimage import gaussian_filter
    x = gaussian_filter(np.random.default_rng(seed).standard_normal((n, n, n)), sigma, mode="nearest")
    return (x / x.std()).reshape(-1)


def tomography_100(n_rays: int = 2_000_000, seed: int = 4) -> RayTomography:
    """100^3 cells (1M unknowns), 2M straight surface-to-borehole rays,
    (A^T A + 1e-2 I) x = A^T b with b = A x_true + 1% noise (seed 44)."""
    n = 100
    return RayTomography("tomo-100^3-2M-rays", n, ray_endpoints(n_rays, n, seed), smooth_model(n, 5.0, seed + 36),
                         1e-2, 44)


def tomography_small(n: int = 20, n_rays: int = 3000, seed: int = 7) -> RayTomography:
    return RayTomography(f"tomo-{n}^3", n, ray_endpoints(n_rays, n, seed), smooth_model(n, 2.0, seed + 36), 1e-2,
                         seed + 40)


def noisy_data(A_x: np.ndarray, level: float, seed: int) -> np.ndarray:
    """b = A x_true + level * std(A x_true) * N(0, 1)."""
    noise = np.random.default_rng(seed).standard_normal(A_x.size)
    return A_x + level * float(np.std(A_x)) * noise


# ------------------------------------------- midpoint-sampled traveltime picks

@dataclass
class PickSet:
    """Picks of the reference's Python inversion driver (one per source-station
    pair): model = (nx, ny, nz, dx, dy, dz, origin_x, origin_y, origin_z),
    world coordinates in metres, velocities vp (nx, ny, nz) FP64 in m/s."""
    name: str
    model: tuple
    src_xyz: np.ndarray   # [n_picks, 3]
    sta_xyz: np.ndarray   # [n_picks, 3]
    weight: np.ndarray    # [n_picks]
    vp: np.ndarray        # (nx, ny, nz)


def gradient_model(nx: int, ny: int, nz: int, dz: float, water_depth: float = 4000.0) -> np.ndarray:
    """VelocityModel.initialize_gradient_model's vp (model.py:46-64): water
    (1500 m/s) above water_depth, below it 3000 (1 + 0.3 depth / 5000) capped
    at 8500."""
    z = np.arange(nz) * dz
    col = np.where(z < water_depth, 1500.0, np.minimum(3000.0 * (1.0 + 0.3 * (z - water_depth) / 5000.0), 8500.0))
    return np.broadcast_to(col, (nx, ny, nz)).copy()


def obs_picks(n: int = 100, d: float = 200.0, n_sources: int = 2000, n_stations: int = 1000,
              seed: int = 9) -> PickSet:
    """n^3 cells of d metres; sources (earthquakes) uniform in the volume below
    the seafloor, ocean-bottom stations uniform on the seafloor at 4000 m; one
    pick per source-station pair (n_sources * n_stations picks, in source-major
    order), weights uniform in [0.5, 1.5]; vp = the gradient model plus a
    smooth 5% perturbation."""
    rng = np.random.default_rng(seed)
    ext = n * d
    src = np.stack([rng.uniform(0, ext, n_sources), rng.uniform(0, ext, n_sources),
                    rng.uniform(4000.0, ext, n_sources)], axis=1)
    sta = np.stack([rng.uniform(0, ext, n_stations), rng.uniform(0, ext, n_stations),
                    np.full(n_stations, 4000.0)], axis=1)
    src_xyz = np.repeat(src, n_stations, axis=0)
    sta_xyz = np.tile(sta, (n_sources, 1))
    weight = rng.uniform(0.5, 1.5, n_sources * n_stations)
    vp = gradient_model(n, n, n, d) * (1.0 + 0.05 * smooth_model(n, 4.0, seed + 1).reshape(n, n, n))
    return PickSet(f"picks-{n}^3-{n_sources}x{n_stations}", (n, n, n, d, d, d, 0.0, 0.0, 0.0), src_xyz, sta_xyz,
                   weight, vp)
