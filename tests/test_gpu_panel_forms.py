"""Alternative kernel forms against the default ones, through the C ABI: the
Gauss-Jordan panel forms against the one-CTA lane-quad form, the bulk-copy
sweep products against the register-load kernel, and split-K Schur products
against unsplit ones.

* cluster form: one matrix's panel split over 2, 4 or 8 CTAs of a thread-block
  cluster (FDFD_GJ_CL, read when the handle is created; -1 picks the size per
  level from its matrix count, -2 (the default) clusters of 8 for the deep levels);
* row form: one row per thread, software-pipelined column steps (FDFD_GJ_FORM=1).

Each form takes the same pivots and performs the same arithmetic per element, so
a factorization and solve with every panel in that form gives the fields of the
lane-quad form bit for bit, in both precisions, for matrices up to 512 rows (32-
and 16-column panels) and above (16- and 8-column panels).  The default form's
fields also match the oracle.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_RES = 1e-10
FORMS = [("FDFD_GJ_CL", "2"), ("FDFD_GJ_CL", "4"), ("FDFD_GJ_CL", "8"), ("FDFD_GJ_CL", "-1"), ("FDFD_GJ_CL", "-2"),
         ("FDFD_GJ_FORM", "1")]


def rel(a, b):
    return float(np.linalg.norm(np.ravel(a - b)) / np.linalg.norm(np.ravel(b)))


def run(fdfd, monkeypatch, p, prec, env):
    for name in ("FDFD_GJ_CL", "FDFD_GJ_FORM"):
        monkeypatch.delenv(name, raising=False)
    for name, val in env:
        monkeypatch.setenv(name, val)
    h = fdfd._lib.Handle(p.Nx, p.Ny, p.npml[0], p.npml[1], p.dx, p.dy, 1e-6, p.pml_m, p.pml_lnR, fdfd.TM, prec)
    h.set_refinement(TOL_RES, 60)
    h.set_eps(p.eps)
    h.factor(p.omega)
    f1, f2, f3, st = h.solve(p.src)
    h.close()
    return f1, f2, f3, st


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
@pytest.mark.parametrize("size", [(260, 200), (560, 600)])
def test_panel_forms_match_quad_form(lib, fdfd, oracle, monkeypatch, prec, size):
    from fdfd_gb300 import workloads as W
    p = W.design_guide(size[0], size[1], design=(48, 48), seed=11, npml=12)
    P = fdfd.FDFD_PREC_FP64 if prec == "fp64" else fdfd.FDFD_PREC_MIXED
    base = run(fdfd, monkeypatch, p, P, [("FDFD_GJ_CL", "1"), ("FDFD_GJ_FORM", "0")])
    assert base[3].rel_residual <= TOL_RES
    for env in FORMS:
        got = run(fdfd, monkeypatch, p, P, [env])
        assert got[3].iterations == base[3].iterations, env
        for a, b in zip(got[:3], base[:3]):
            assert np.array_equal(a, b), (env, rel(a, b))
    auto = run(fdfd, monkeypatch, p, P, [])
    for a, b in zip(auto[:3], base[:3]):
        assert np.array_equal(a, b), rel(a, b)
    g = oracle.Grid((p.Nx, p.Ny), p.npml, ((0.0, 0.0), (p.Nx * p.dx, p.Ny * p.dy)))
    ref = oracle.solve(g, p.eps, p.src, p.omega, oracle.TM, p.pml_m, p.pml_lnR)
    tol = 1e-8 if prec == "mixed" else 1e-10
    assert max(rel(auto[0], ref[0]), rel(auto[1], ref[1]), rel(auto[2], ref[2])) <= tol


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
@pytest.mark.parametrize("size", [(260, 200), (301, 197)])
def test_bulk_copy_sweep_matches_register_form(lib, fdfd, monkeypatch, prec, size):
    """The N-form sweep products through the bulk-copy pipeline (the default where it fits)
    give the fields of the register-load kernel bit for bit (b = 200: 16-byte rows; b = 197:
    a row end inside a 16-byte vector)."""
    from fdfd_gb300 import workloads as W
    p = W.design_guide(size[0], size[1], design=(48, 48), seed=12, npml=12)
    P = fdfd.FDFD_PREC_FP64 if prec == "fp64" else fdfd.FDFD_PREC_MIXED
    monkeypatch.setenv("FDFD_GEMV_BULK", "0")
    ref = run(fdfd, monkeypatch, p, P, [])
    monkeypatch.setenv("FDFD_GEMV_BULK", "1")
    got = run(fdfd, monkeypatch, p, P, [])
    assert got[3].iterations == ref[3].iterations and got[3].rel_residual <= TOL_RES
    for a, b in zip(got[:3], ref[:3]):
        assert np.array_equal(a, b), rel(a, b)


def test_splitk_schur_products_match(lib, fdfd, oracle, monkeypatch):
    """Split-K Schur products (the default for products whose tiles fill less than half of the
    SMs: partial products over K slices, then their sum in a fixed order) give the fields of
    the unsplit products to within the mixed form's rounding, and the oracle's; the result is
    the same on a second run (deterministic)."""
    from fdfd_gb300 import workloads as W
    p = W.design_guide(600, 300, design=(64, 64), seed=13, npml=12)   # b = 300: the deep levels split
    P = fdfd.FDFD_PREC_MIXED
    monkeypatch.setenv("FDFD_SPLITK", "0")
    ref = run(fdfd, monkeypatch, p, P, [])
    monkeypatch.setenv("FDFD_SPLITK", "1")
    got = run(fdfd, monkeypatch, p, P, [])
    got2 = run(fdfd, monkeypatch, p, P, [])
    assert got[3].rel_residual <= TOL_RES and abs(got[3].iterations - ref[3].iterations) <= 1
    for a, b, c in zip(got[:3], ref[:3], got2[:3]):
        assert rel(a, b) <= 1e-9 and np.array_equal(a, c)
    g = oracle.Grid((p.Nx, p.Ny), p.npml, ((0.0, 0.0), (p.Nx * p.dx, p.Ny * p.dy)))
    o = oracle.solve(g, p.eps, p.src, p.omega, oracle.TM, p.pml_m, p.pml_lnR)
    assert max(rel(got[0], o[0]), rel(got[1], o[1]), rel(got[2], o[2])) <= 1e-8
