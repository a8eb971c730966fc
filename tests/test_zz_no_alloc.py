"""st_cg_device_static: the CG entry point for callers that cannot allocate
device memory while they run (its scratch is a fixed file-scope device
array). Called twice in a row through the C ABI, it must give the solution
and iteration count of the allocating entry point st_cg_device within the
tolerance the CG tests use (1e-5 relative). This file is named to be
collected last, so a run that stops at the first failure has already run
every other test; it also passes on its own in a fresh process."""
import ctypes as C
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


def spd_matrix(se, nx, ny, nz):
    vel = np.full(nx * ny * nz, 2000.0)
    dt = 0.25 * 10.0 / 2000.0  # diagonally dominant, symmetric 7-point matrix
    return se.compute_fd_stencil(nx, ny, nz, vel, 10.0, 10.0, 10.0, dt)


def solve(lib, name, m, b, x, jacobi):
    it = C.c_int(-1)
    rel = C.c_double(-1.0)
    rc = getattr(lib, name)(m.handle, C.c_void_p(b.data_ptr()), C.c_void_p(x.data_ptr()), 500, C.c_double(1e-6),
                            int(jacobi), C.byref(it), C.byref(rel))
    assert rc == 0, lib.st_last_error()
    return it.value, rel.value


@pytest.mark.parametrize("jacobi", [False, True])
def test_static_cg_matches_allocating_cg(se, jacobi):
    import torch
    from seismic_engine import _lib
    lib = _lib.load()
    m = spd_matrix(se, 24, 20, 28)
    n = m.rows()
    rng = np.random.default_rng(31 + int(jacobi))
    x_ref = torch.zeros(n, device="cuda")
    x_sta = torch.zeros(n, device="cuda")
    for call in range(2):  # two calls in a row share (and must re-initialise) the static scratch
        b = torch.from_numpy(rng.standard_normal(n).astype(np.float32)).cuda()
        it_ref, rel_ref = solve(lib, "st_cg_device", m, b, x_ref, jacobi)
        it_sta, rel_sta = solve(lib, "st_cg_device_static", m, b, x_sta, jacobi)
        torch.cuda.synchronize()
        assert it_ref > 0 and abs(it_sta - it_ref) <= 1, (call, it_sta, it_ref)
        assert rel_sta < 1e-6
        xr, xs = x_ref.cpu().numpy(), x_sta.cpu().numpy()
        assert np.linalg.norm(xs - xr) <= 1e-5 * np.linalg.norm(xr), call
    # and it allocates nothing: the device's free memory is the same before and
    # after a further call (the static scratch was set up by the calls above)
    free0 = torch.cuda.mem_get_info()[0]
    solve(lib, "st_cg_device_static", m, b, x_sta, jacobi)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0


def test_static_cg_rejects_oversized_system(se):
    import torch
    from seismic_engine import _lib
    lib = _lib.load()
    m = spd_matrix(se, 128, 128, 65)  # 1,064,960 unknowns > ST_CG_STATIC_MAX_N = 1,048,576
    n = m.rows()
    assert n > 1048576
    b = torch.ones(n, device="cuda")
    x = torch.zeros(n, device="cuda")
    it = C.c_int(-1)
    rel = C.c_double(-1.0)
    rc = lib.st_cg_device_static(m.handle, C.c_void_p(b.data_ptr()), C.c_void_p(x.data_ptr()), 10, C.c_double(1e-6),
                                 0, C.byref(it), C.byref(rel))
    assert rc == _lib.ST_ERR_ARG
    assert b"at most 1048576 unknowns" in lib.st_last_error()
