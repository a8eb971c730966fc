"""Oracle restatement of the straight-ray path-length matrix (voxel
traversal) against its definition: row sums are the ray lengths, every
entry is a cell the segment crosses, and a dense sampling of the segment
gives the same per-cell lengths."""
import numpy as np


def test_ray_matrix_row_sums_and_cells(oracle):
    from seismic_engine import workloads as wl
    n = 12
    ends = wl.ray_endpoints(400, n, seed=3)
    rp, col, val = oracle.ray_matrix(ends, n, n, n, h=2.5)
    assert rp[0] == 0 and rp[-1] == col.size and np.all(np.diff(rp) > 0)
    assert col.min() >= 0 and col.max() < n ** 3 and np.all(val > 0)
    lengths = 2.5 * np.linalg.norm(ends[:, 3:] - ends[:, :3], axis=1)
    sums = np.add.reduceat(val, rp[:-1])
    np.testing.assert_allclose(sums, lengths, rtol=1e-12)
    for i in range(rp.size - 1):  # columns ascending within each row
        assert np.all(np.diff(col[rp[i]:rp[i + 1]]) > 0)


def test_ray_matrix_matches_dense_sampling(oracle):
    from seismic_engine import workloads as wl
    n = 10
    ends = wl.ray_endpoints(12, n, seed=5)
    rp, col, val = oracle.ray_matrix(ends, n, n, n)
    m = 200_000
    for i in range(ends.shape[0]):
        p0, p1 = ends[i, :3], ends[i, 3:]
        t = (np.arange(m) + 0.5) / m
        pts = p0[None, :] + t[:, None] * (p1 - p0)[None, :]
        c = np.clip(np.floor(pts).astype(np.int64), 0, n - 1)
        idx = (c[:, 0] * n + c[:, 1]) * n + c[:, 2]
        u, cnt = np.unique(idx, return_counts=True)
        approx = cnt * np.linalg.norm(p1 - p0) / m
        got = dict(zip(col[rp[i]:rp[i + 1]], val[rp[i]:rp[i + 1]]))
        big = {k: v for k, v in zip(u, approx) if v > 1e-3}
        for k, v in big.items():
            assert abs(got.get(k, 0.0) - v) < 2e-4 * np.linalg.norm(p1 - p0) + 1e-4, (i, k)


def test_ray_endpoints_geometry():
    from seismic_engine import workloads as wl
    e = wl.ray_endpoints(1000, 100, seed=4)
    assert e.shape == (1000, 6)
    assert np.all(e[:, 2] == 0.0) and np.all((e[:, 5] >= 0) & (e[:, 5] < 100))
    assert set(np.unique(e[:, 3])) <= {10.5, 90.5} and set(np.unique(e[:, 4])) <= {10.5, 90.5}
