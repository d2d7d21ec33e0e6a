"""Failure paths of the GPU solve, in forms that fault, trap or hang no GPU.

* FDFD_ETIMEOUT: the tensor-core GEMM's pipeline waits are bounded; with the
  handle's wait limit set to 1 ns a wait runs out before its copies land, the
  CTA lets its own copies and MMAs finish, frees its tensor memory and exits,
  and the factorization reports the timeout.  With the default limit back, the
  same handle factors and solves to the oracle's field.
* FDFD_ESINGULAR: a permittivity whose ω²ϵ₀ϵᵣ term overflows makes a pivot of
  the first-step block inversion non-finite, which the pivot check reports.
* FDFD_ENOMEM: a device budget below what the factorization needs fails the
  allocation on the host, before any device work; the handle stays usable.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_RES = 1e-10


def rel(a, b):
    return float(np.linalg.norm(np.ravel(a - b)) / np.linalg.norm(np.ravel(b)))


def problem(Nx=300, Ny=260):
    from fdfd_gb300 import workloads as W
    return W.design_guide(Nx, Ny, design=(64, 64), seed=7, npml=12)


def handle(fdfd, p, prec):
    h = fdfd._lib.Handle(p.Nx, p.Ny, p.npml[0], p.npml[1], p.dx, p.dy, 1e-6, p.pml_m, p.pml_lnR, fdfd.TM, prec)
    h.set_refinement(TOL_RES, 60)
    return h


def oracle_fields(oracle, p):
    g = oracle.Grid((p.Nx, p.Ny), p.npml, ((0.0, 0.0), (p.Nx * p.dx, p.Ny * p.dy)))
    return oracle.solve(g, p.eps, p.src, p.omega, oracle.TM, p.pml_m, p.pml_lnR)


def test_gemm_wait_timeout_reports_etimeout_and_recovers(lib, fdfd, oracle):
    p = problem()
    h = handle(fdfd, p, fdfd.FDFD_PREC_MIXED)
    h.set_eps(p.eps)
    h.set_wait_limit(1)
    with pytest.raises(fdfd.FDFDError) as e:
        h.factor(p.omega)
    assert e.value.code == fdfd._lib.FDFD_ETIMEOUT, e.value
    h.set_wait_limit(0)
    h.factor(p.omega)
    f1, f2, f3, st = h.solve(p.src)
    h.close()
    assert st.tc_gemm == 1 and st.rel_residual <= TOL_RES
    ref = oracle_fields(oracle, p)
    assert max(rel(f1, ref[0]), rel(f2, ref[1]), rel(f3, ref[2])) <= 1e-8


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_nonfinite_pivot_reports_esingular(lib, fdfd, prec):
    """ϵᵣ = 1e300 (FP64: ω²ϵ₀ϵᵣ overflows in the assembly) or 1e42 (mixed:
    the scaled diagonal overflows FP32) at one cell: FDFD_ESINGULAR.  The next
    factorization of a regular ϵᵣ on the same handle succeeds."""
    p = problem(96, 64)
    P = fdfd.FDFD_PREC_FP64 if prec == "fp64" else fdfd.FDFD_PREC_MIXED
    h = handle(fdfd, p, P)
    eps = p.eps.copy()
    eps[p.Nx // 2, p.Ny // 2] = 1e300 if prec == "fp64" else 1e42
    h.set_eps(eps)
    with pytest.raises(fdfd.FDFDError) as e:
        h.factor(p.omega)
    assert e.value.code == fdfd._lib.FDFD_ESINGULAR, e.value
    h.set_eps(p.eps)
    h.factor(p.omega)
    _, _, _, st = h.solve(p.src)
    h.close()
    assert st.rel_residual <= TOL_RES


def test_device_budget_reports_enomem(lib, fdfd):
    p = problem(96, 64)
    h = handle(fdfd, p, fdfd.FDFD_PREC_MIXED)
    h.set_eps(p.eps)
    h.set_device_budget(1 << 20)          # below the handle's own buffers and the factor pools
    with pytest.raises(fdfd.FDFDError) as e:
        h.factor(p.omega)
    assert e.value.code == fdfd._lib.FDFD_ENOMEM, e.value
    assert "budget" in str(e.value)
    h.set_device_budget(0)
    h.factor(p.omega)
    _, _, _, st = h.solve(p.src)
    h.close()
    assert st.rel_residual <= TOL_RES


# ---------------------------------------------------------------------------
# checkpointing of block factors to host memory (capacity beyond HBM)
# ---------------------------------------------------------------------------
def ckpt_problem():
    from fdfd_gb300 import workloads as W
    return W.design_guide(300, 200, design=(60, 60), seed=8, npml=12)


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_checkpoint_mode_matches_resident(lib, fdfd, prec):
    """Forced checkpoint mode (couplings and X blocks in pinned host memory, copied back by every
    sweep) gives the same fields as the resident layout, with less device memory."""
    p = ckpt_problem()
    P = fdfd.FDFD_PREC_FP64 if prec == "fp64" else fdfd.FDFD_PREC_MIXED
    out = {}
    for mode in (-1, 1):
        h = handle(fdfd, p, P)
        h.set_checkpoint(mode)
        h.set_eps(p.eps)
        h.factor(p.omega)
        f1, f2, f3, st = h.solve(p.src)
        out[mode] = (f1, f2, f3, st.device_bytes, h.checkpoint_info(), st.rel_residual)
        h.close()
    res, ck = out[-1], out[1]
    assert not res[4]["active"] and ck[4]["active"]
    assert ck[4]["host_bytes"] > 0 and ck[4]["copied_bytes"] > ck[4]["host_bytes"]
    assert ck[3] < res[3]
    assert ck[5] <= TOL_RES
    for a, c in zip(res[:3], ck[:3]):
        assert rel(c, a) <= 1e-14


def test_checkpoint_engages_under_device_budget(lib, fdfd):
    """Automatic mode: with a device budget between the checkpointed and the resident footprint
    the handle checkpoints by itself and solves; below the checkpointed footprint it reports
    FDFD_ENOMEM."""
    p = ckpt_problem()
    tot = {}
    for mode in (-1, 1):
        h = handle(fdfd, p, fdfd.FDFD_PREC_MIXED)
        h.set_checkpoint(mode)
        h.set_eps(p.eps)
        h.factor(p.omega)
        _, _, _, st = h.solve(p.src)
        tot[mode] = st.device_bytes
        h.close()
    h = handle(fdfd, p, fdfd.FDFD_PREC_MIXED)
    h.set_device_budget((tot[-1] + tot[1]) // 2)
    h.set_eps(p.eps)
    h.factor(p.omega)
    _, _, _, st = h.solve(p.src)
    assert h.checkpoint_info()["active"] and st.rel_residual <= TOL_RES
    h.close()
    h = handle(fdfd, p, fdfd.FDFD_PREC_MIXED)
    h.set_device_budget(tot[1] // 2)
    h.set_eps(p.eps)
    with pytest.raises(fdfd.FDFDError) as e:
        h.factor(p.omega)
    assert e.value.code == fdfd._lib.FDFD_ENOMEM
    h.close()
