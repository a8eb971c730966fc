"""GPU midpoint-sampled straight-ray forward model and gradient (the
reference's AdjointStateInversion._forward_model / _compute_gradient,
seismic_tomography/inversion.py:329-433) through the C ABI: bit-exact FP64
against the reference's own outputs (golden fixtures) and against the oracle
on larger seeded pick sets, on the host and the device (torch) paths; the
sampled-ray CSR against the oracle's triplet build; refusals and empty sets."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def se():
    import importlib.util
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    spec = importlib.util.spec_from_file_location(
        "st_build", os.path.join(repo, "03-seismic-tomography-compute_gb300", "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build()
    import seismic_engine
    return seismic_engine


def fixture(golden_dir, name):
    return dict(np.load(os.path.join(golden_dir, name)))


def model_of(z):
    return tuple(int(v) for v in z["n"]) + tuple(float(v) for v in z["d"]) + tuple(float(v) for v in z["origin"])


@pytest.mark.parametrize("name", ["rays_small.npz", "rays_medium.npz"])
def test_bit_exact_against_reference(se, golden_dir, name):
    z = fixture(golden_dir, name)
    rays = se.SampledRays(model_of(z), z["src_xyz"], z["sta_xyz"], z["weight"], z["valid"], z["dist"])
    t = rays.forward_model(z["vp"])
    g = rays.compute_gradient(z["vp"], z["residuals"])
    assert np.array_equal(t, z["times"]), np.abs(t - z["times"]).max()
    assert np.array_equal(g, z["gradient"]), np.abs(g - z["gradient"]).max()


class _Obj:
    def __init__(self, **kw):
        self.__dict__.update(kw)


def test_reference_objects_path(se, golden_dir):
    """forward_model / compute_gradient on objects with the reference's
    attribute names (VelocityModel, OBSDataCoordinator, OBSPick, ...)."""
    from seismic_engine import rays as R
    z = fixture(golden_dir, "rays_small.npz")
    nx, ny, nz, dx, dy, dz, ox, oy, oz = model_of(z)
    model = _Obj(nx=nx, ny=ny, nz=nz, dx=dx, dy=dy, dz=dz, origin_x=ox, origin_y=oy, origin_z=oz, vp=z["vp"])
    sources, stations, picks = {}, {}, []
    for i in range(z["valid"].size):
        sid, rid = (f"S{i}", f"R{i}") if z["valid"][i] else (f"S{i}", "unknown")
        sources[sid] = _Obj(x=z["src_xyz"][i, 0], y=z["src_xyz"][i, 1], z=z["src_xyz"][i, 2])
        if z["valid"][i]:
            stations[rid] = _Obj(x=z["sta_xyz"][i, 0], y=z["sta_xyz"][i, 1], z=z["sta_xyz"][i, 2])
        picks.append(_Obj(source_id=sid, station_id=rid, weight=float(z["weight"][i])))
    obs = _Obj(picks=picks, sources=sources, stations=stations)
    rays = R.SampledRays.from_reference_objects(model, obs)
    assert np.array_equal(R.forward_model(model, obs, rays), z["times"])
    assert np.array_equal(R.compute_gradient(model, obs, z["residuals"], rays), z["gradient"])


def random_case(seed, n=(36, 28, 22), n_src=40, n_sta=60):
    rng = np.random.default_rng(seed)
    d = np.array([40.0, 100.0, 80.0])  # n = dist / (5 dx): about 7 samples per ray
    o = np.array([-300.0, 0.0, 50.0])
    ext = np.array(n) * d
    src = o + rng.uniform(-0.1, 1.1, (n_src, 3)) * ext
    sta = o + rng.uniform(0.0, 1.0, (n_sta, 3)) * ext
    s = np.repeat(src, n_sta, axis=0)
    r = np.tile(sta, (n_src, 1))
    vp = rng.uniform(1500.0, 7000.0, n)
    bad = rng.integers(0, vp.size, 40)
    vp.reshape(-1)[bad[:10]] = np.nan
    vp.reshape(-1)[bad[10:20]] = -1.0
    vp.reshape(-1)[bad[20:30]] = 0.0
    vp.reshape(-1)[bad[30:]] = np.inf
    valid = (rng.uniform(size=s.shape[0]) > 0.02).astype(np.uint8)
    w = rng.uniform(0.5, 1.5, s.shape[0])
    res = rng.standard_normal(s.shape[0])
    res[rng.integers(0, res.size, 20)] = np.nan
    return np.array(n), d, o, s, r, valid, w, vp, res


def test_bit_exact_against_oracle_random(se, oracle):
    import torch
    n, d, o, s, r, valid, w, vp, res = random_case(5)
    model = tuple(int(v) for v in n) + tuple(d) + tuple(o)
    rays = se.SampledRays(model, s, r, w, valid)
    t_ref = oracle.sampled_traveltimes(n, d, o, s, r, valid, vp)
    g_ref = oracle.sampled_gradient(n, d, o, s, r, valid, w, vp, res)
    assert rays.n_samples > 5 * s.shape[0]
    assert np.array_equal(rays.forward_model(vp), t_ref)
    assert np.array_equal(rays.compute_gradient(vp, res), g_ref)
    # device path: torch FP64 tensors, ordered after the current stream
    vt = torch.from_numpy(vp.reshape(-1)).cuda()
    rt = torch.from_numpy(res).cuda()
    tt = rays.forward_model(vt)
    gt = rays.compute_gradient(vt, rt)
    assert np.array_equal(tt.cpu().numpy(), t_ref)
    assert np.array_equal(gt.cpu().numpy(), g_ref)


def test_sampled_matrix_matches_oracle_triplets(se, oracle):
    n, d, o, s, r, valid, w, vp, res = random_case(6, n_src=20, n_sta=30)
    model = tuple(int(v) for v in n) + tuple(d) + tuple(o)
    rays = se.SampledRays(model, s, r, w, valid)
    A = rays.matrix()
    rp, col, val = A.row_ptr(), A.col_ind(), A.values()
    assert A.rows() == s.shape[0] and A.cols() == int(np.prod(n))
    # the oracle's triplets: one per sample, (pick, cell, ds), duplicates summed
    good = np.where(np.isfinite(vp) & (vp > 0), vp, 1500.0)
    inv_v = 1.0 / good.reshape(-1)
    t = oracle.sampled_traveltimes(n, d, o, s, r, valid, good)
    y = A.spmv(inv_v)
    np.testing.assert_allclose(y, t, rtol=2e-6)
    for i in range(0, s.shape[0], 97):  # per-row structure: ascending unique columns
        c = col[rp[i]:rp[i + 1]]
        assert np.all(np.diff(c) > 0)
        if not valid[i]:
            assert c.size == 0


def test_refusals_and_empty(se):
    from seismic_engine import SeismicError
    model = (8, 8, 8, 10.0, 10.0, 10.0, 0.0, 0.0, 0.0)
    with pytest.raises(SeismicError):
        se.SampledRays(model, [[np.nan, 0, 0]], [[1.0, 1.0, 1.0]], [1.0])
    with pytest.raises(SeismicError):  # 2e7 samples in one ray
        se.SampledRays(model, [[0.0, 0.0, 0.0]], [[1e9, 0.0, 0.0]], [1.0])
    with pytest.raises(SeismicError):
        se.SampledRays((8, 8, 8, 0.0, 10.0, 10.0, 0.0, 0.0, 0.0), [[0.0, 0, 0]], [[1.0, 1, 1]], [1.0])
    e = se.SampledRays(model, np.zeros((0, 3)), np.zeros((0, 3)), np.zeros(0))
    assert e.n_picks == 0 and e.n_samples == 0
    assert e.forward_model(np.full(512, 2000.0)).size == 0
    assert np.all(e.compute_gradient(np.full(512, 2000.0), np.zeros(0)) == 0.0)
    # invalid picks only: time 0, no gradient, no samples
    v = se.SampledRays(model, [[5.0, 5, 5]], [[75.0, 75, 75]], [1.0], valid=[0])
    assert v.n_samples == 0 and v.forward_model(np.full(512, 2000.0))[0] == 0.0


def test_full_size_matrix_properties(se):
    """At the benchmark's size (2M picks, 26.8M samples on 100^3 cells): the
    forward model equals A (1/v) with the sampled-ray CSR, and the gradient
    equals -(A^T (w r)) / v^2 (all velocities valid, residuals finite), to
    the FP32 precision of the matrix and the SpMV."""
    import torch
    ps = se.workloads.obs_picks()
    rays = se.SampledRays(ps.model, ps.src_xyz, ps.sta_xyz, ps.weight)
    vp = torch.from_numpy(ps.vp.reshape(-1)).cuda()
    res = torch.from_numpy(np.random.default_rng(1).standard_normal(rays.n_picks) * 0.05).cuda()
    t = rays.forward_model(vp)
    g = rays.compute_gradient(vp, res)
    A = rays.matrix()
    assert A.rows() == rays.n_picks and A.cols() == rays.n_cells
    y = torch.zeros(rays.n_picks, device="cuda")
    s = (1.0 / vp).float()
    A.spmv_device(s, y)
    r32 = (torch.from_numpy(ps.weight).cuda() * res).float()
    z = torch.zeros(rays.n_cells, device="cuda")
    A.spmv_device(r32, z, transpose=True)
    torch.cuda.synchronize()
    torch.cuda.ExternalStream(A.stream_ptr()).synchronize()
    e_t = float(torch.linalg.norm(y.double() - t) / torch.linalg.norm(t))
    g_ref = -z.double() / (vp * vp)
    e_g = float(torch.linalg.norm(g_ref - g) / torch.linalg.norm(g))
    print(f"full size: forward vs A(1/v) {e_t:.2e}, gradient vs -A^T(wr)/v^2 {e_g:.2e}")
    assert e_t < 1e-6 and e_g < 1e-5
    A.close()
    rays.close()
