"""GPU test of the allocation-free residual entry point.

fdfd_residual_noalloc serves callers that may not let a library call
cudaMalloc/cudaFree (memory-pool runtimes, code avoiding the synchronisation
those calls imply).  It keeps its block partial sums in a fixed device array
of the library and takes every buffer from the caller.  Here the caller's
buffers are torch tensors.  Its output must match the handle path's operator
product (fdfd_apply) on two calls in a row, so a stale scratch array would show.
This file runs last so that a failure here leaves every other test already run.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12   # both paths run the same FP64 stencil kernel


def rel(a, b):
    return float(np.linalg.norm(np.ravel(a - b)) / np.linalg.norm(np.ravel(b)))


def test_noalloc_residual_matches_handle_path(lib, fdfd):
    import torch

    L = fdfd._lib
    Nx, Ny, nrhs = 37, 29, 3
    rng = np.random.default_rng(0)
    eps = rng.uniform(1, 4, (Nx, Ny)) + 0.05j
    h = L.Handle(Nx, Ny, 4, 4, 0.05, 0.05, 1e-6, 4.0, np.log(1e-8), L.FDFD_TM, L.FDFD_PREC_FP64)
    h.set_eps(eps)
    h.factor(1.2e15)
    dev = torch.device("cuda")
    d_st = torch.from_numpy(L.natural(h.stencil()).reshape(-1)).to(dev)
    for call in range(2):
        x = rng.standard_normal((nrhs, Nx, Ny)) + 1j * rng.standard_normal((nrhs, Nx, Ny))
        b = rng.standard_normal((nrhs, Nx, Ny)) + 1j * rng.standard_normal((nrhs, Nx, Ny))
        ref_r = b - h.apply(x)                       # existing entry point
        d_x = torch.from_numpy(L.natural(x).reshape(-1)).to(dev)
        d_b = torch.from_numpy(L.natural(b).reshape(-1)).to(dev)
        d_r = torch.empty_like(d_x)
        d_n = torch.full((2 * nrhs,), float("nan"), dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        rc = lib.fdfd_residual_noalloc(Nx, Ny, nrhs, d_st.data_ptr(), d_x.data_ptr(), d_b.data_ptr(),
                                       d_r.data_ptr(), d_n.data_ptr(), None)
        assert rc == L.FDFD_OK, (call, rc)
        r = L.from_natural(d_r.cpu().numpy(), Nx, Ny)
        assert rel(r, ref_r) <= TOL, (call, rel(r, ref_r))
        norms = d_n.cpu().numpy()
        for k in range(nrhs):
            assert norms[2 * k] == pytest.approx(np.linalg.norm(ref_r[k]) ** 2, rel=TOL)
            assert norms[2 * k + 1] == pytest.approx(np.linalg.norm(b[k]) ** 2, rel=TOL)
    # b = NULL: r = A x and the |b|² norms are 0, here on a stream of the caller's
    x = rng.standard_normal((nrhs, Nx, Ny)) + 1j * rng.standard_normal((nrhs, Nx, Ny))
    ref_ax = h.apply(x)
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        d_x = torch.from_numpy(L.natural(x).reshape(-1)).to(dev, non_blocking=False)
        d_r = torch.empty_like(d_x)
        d_n = torch.full((2 * nrhs,), float("nan"), dtype=torch.float64, device=dev)
    stream.synchronize()
    rc = lib.fdfd_residual_noalloc(Nx, Ny, nrhs, d_st.data_ptr(), d_x.data_ptr(), None, d_r.data_ptr(),
                                   d_n.data_ptr(), stream.cuda_stream)
    assert rc == L.FDFD_OK, rc
    r = L.from_natural(d_r.cpu().numpy(), Nx, Ny)
    assert rel(r, ref_ax) <= TOL, rel(r, ref_ax)
    norms = d_n.cpu().numpy()
    for k in range(nrhs):
        assert norms[2 * k] == pytest.approx(np.linalg.norm(ref_ax[k]) ** 2, rel=TOL)
        assert norms[2 * k + 1] == 0.0
    # sizes beyond the fixed scratch, or more right-hand sides than the launch's grid y
    # allows, are rejected before any device work
    assert lib.fdfd_residual_noalloc(4096, 4096, 2, d_st.data_ptr(), d_x.data_ptr(), d_b.data_ptr(),
                                     d_r.data_ptr(), d_n.data_ptr(), None) == L.FDFD_EINVAL
    assert lib.fdfd_residual_noalloc(4, 4, 65536, d_st.data_ptr(), d_x.data_ptr(), d_b.data_ptr(),
                                     d_r.data_ptr(), d_n.data_ptr(), None) == L.FDFD_EINVAL
    h.close()
