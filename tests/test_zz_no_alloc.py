"""ptf_calcN2d_noalloc against ptf_calcN, both through the C ABI.

The no-allocation entry point serves callers that may not have a library
allocate device memory (a host whose memory pool owns the device, or a loop
that cannot absorb cudaFree's device-wide synchronisation).  It must give the
same advective term as the handle-based ptf_calcN, call after call, while its
intermediates live in the library's fixed device scratch.  This file is
collected last so a failure here leaves every other test already run.
"""
import ctypes as ct

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-13  # the FP64 calcN tolerance of tests/test_gpu_parity.py


def _field(grid, seed):
    rng = np.random.default_rng(seed)
    X, Y = np.meshgrid(grid.x, grid.y)
    x0, y0 = rng.uniform(-1, 1, 2)
    c = np.exp(-((X - x0) ** 2 + (Y - y0) ** 2) / (2 * 0.3 ** 2)) + 0.2 * np.sin(2 * X + seed) * np.cos(3 * Y)
    return np.fft.rfft2(c)


@pytest.mark.parametrize("nx,ny,Lx,Ly", [(64, 64, 2 * np.pi, 2 * np.pi), (256, 128, 2 * np.pi, 3.0),
                                         (512, 512, 2 * np.pi, 2 * np.pi)])
def test_noalloc_matches_calcN_twice(gpu, nx, ny, Lx, Ly):
    import torch
    from ptf_gb300 import _lib as L
    lib = L.load()
    u = lambda x, y: np.cos(x) * np.sin(2 * y)
    v = lambda x, y: -0.5 * np.sin(x) * np.cos(2 * y)
    prob = gpu.Problem(gpu.GPU(), gpu.TwoDAdvectingFlow(u=u, v=v), nx=nx, ny=ny, Lx=Lx, Ly=Ly)
    X, Y = gpu.gridpoints(prob.grid)
    ud = torch.from_numpy(np.ascontiguousarray(u(X, Y))).cuda()
    vd = torch.from_numpy(np.ascontiguousarray(v(X, Y))).cuda()
    stream = torch.cuda.current_stream()
    for seed in (1, 2):  # two calls in a row: the shared scratch keeps the first call's contents
        sol = _field(prob.grid, seed)
        ref = np.empty_like(sol)
        rc = lib.ptf_calcN(prob._h, sol.ctypes.data_as(ct.c_void_p), ref.ctypes.data_as(ct.c_void_p), L.PTF_HOST)
        L.check(rc, prob._h)
        sol_d = torch.from_numpy(sol.view(np.float64).copy()).cuda()
        out_d = torch.full_like(sol_d, float("nan"))
        rc = lib.ptf_calcN2d_noalloc(nx, ny, Lx, Ly, ct.c_void_p(sol_d.data_ptr()), ct.c_void_p(ud.data_ptr()),
                                     ct.c_void_p(vd.data_ptr()), ct.c_void_p(out_d.data_ptr()),
                                     ct.c_void_p(stream.cuda_stream))
        L.check(rc, None)
        torch.cuda.synchronize()
        got = out_d.cpu().numpy().view(np.complex128).reshape(ref.shape)
        err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
        assert err <= TOL, (seed, err)


def test_noalloc_rejects_oversized_grid(gpu):
    import torch
    from ptf_gb300 import _lib as L
    lib = L.load()
    buf = torch.zeros(16, dtype=torch.float64, device="cuda")
    p = ct.c_void_p(buf.data_ptr())
    rc = lib.ptf_calcN2d_noalloc(1024, 1024, 2 * np.pi, 2 * np.pi, p, p, p, p, None)
    assert rc == L.PTF_ERR_MEMORY
    assert "scratch" in lib.ptf_last_error(None).decode()
    rc = lib.ptf_calcN2d_noalloc(100, 64, 2 * np.pi, 2 * np.pi, p, p, p, p, None)
    assert rc == L.PTF_ERR_ARG
