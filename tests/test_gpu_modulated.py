"""GPU parity of the modulated-device solve (solve(d::ModulatedDevice),
src/solver/modulation.jl:35-119) through the C ABI against the FP64 oracle."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden")
TOL_RES = 1e-10
TOL_FIELD_MIXED = 1e-8
TOL_FIELD_FP64 = 1e-10


def rel(a, b):
    return float(np.linalg.norm(np.ravel(a - b)) / np.linalg.norm(np.ravel(b)))


def grid_of(oracle, p):
    return oracle.Grid((p.Nx, p.Ny), tuple(p.npml), ((0.0, 0.0), (p.Nx * p.dx, p.Ny * p.dy)))


def mf_handle(fdfd, p, prec, s, shared):
    h = fdfd._lib.ModulatedHandle(p.Nx, p.Ny, p.npml[0], p.npml[1], p.dx, p.dy, s, 1e-6, p.pml_m, p.pml_lnR,
                                  shared, prec)
    h.set_refinement(TOL_RES, 60)
    h.set_eps(p.eps)
    h.set_deps(p.extra["deps"])
    return h


@pytest.mark.parametrize("s,shared", [(1, True), (2, False)])
def test_mf_apply_matches_oracle(lib, fdfd, oracle, s, shared):
    """The coupled operator (sideband stencils + Δϵ couplings) applied on the
    device equals the oracle's sparse matrix."""
    from fdfd_gb300 import workloads as W
    p = W.modulated_waveguide(dh=0.05, L=4.0)
    h = mf_handle(fdfd, p, fdfd.FDFD_PREC_FP64, s, shared)
    h.factor(p.omega, p.extra["Omega"])
    K = 2 * s + 1
    rng = np.random.default_rng(9)
    x = rng.standard_normal((K, p.Nx, p.Ny)) + 1j * rng.standard_normal((K, p.Nx, p.Ny))
    y = h.apply(x)
    h.close()
    A, _, _ = oracle.modulated_system(grid_of(oracle, p), p.eps, p.extra["deps"], p.omega, p.extra["Omega"], s,
                                      shared, p.pml_m, p.pml_lnR)
    ref = A @ np.concatenate([oracle.vec(x[j]) for j in range(K)])
    got = np.concatenate([oracle.vec(y[j]) for j in range(K)])
    assert rel(got, ref) <= 1e-13


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_mf_golden(lib, fdfd, prec):
    """Stored FP64 answer of the reference's modulated-waveguide setup at 125x50."""
    g = np.load(os.path.join(GOLD, "tm_modulated_125x50.npz"))
    Nx, Ny, s = int(g["Nx"]), int(g["Ny"]), int(g["nsidebands"])
    pr = fdfd.FDFD_PREC_FP64 if prec == "fp64" else fdfd.FDFD_PREC_MIXED
    h = fdfd._lib.ModulatedHandle(Nx, Ny, int(g["npml"][0]), int(g["npml"][1]), float(g["dx"]), float(g["dy"]), s,
                                  1e-6, float(g["pml_m"]), float(g["pml_lnR"]), bool(g["sharedpml"]), pr)
    h.set_refinement(TOL_RES, 60)
    h.set_eps(g["eps"])
    h.set_deps(g["deps"])
    h.factor(float(g["omega"]), float(g["Omega"]))
    ez, _, _, st = h.solve(g["src"])
    h.close()
    assert st.rel_residual <= TOL_RES
    assert rel(ez, g["ez"]) <= (TOL_FIELD_FP64 if prec == "fp64" else TOL_FIELD_MIXED)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("s,shared", [(1, True), (1, False), (2, True)])
def test_mf_solve_matches_oracle(lib, fdfd, oracle, prec, s, shared):
    """Ez, Hx, Hy of every sideband against the oracle's direct solve of the
    coupled system (reference setup at 250x100, shared or per-sideband PML)."""
    from fdfd_gb300 import workloads as W
    p = W.modulated_waveguide(dh=0.02, nsidebands=s, sharedpml=shared)
    pr = fdfd.FDFD_PREC_FP64 if prec == "fp64" else fdfd.FDFD_PREC_MIXED
    h = mf_handle(fdfd, p, pr, s, shared)
    h.factor(p.omega, p.extra["Omega"])
    ez, hx, hy, st = h.solve(p.src)
    h.close()
    ref = oracle.solve_modulated(grid_of(oracle, p), p.eps, p.extra["deps"], p.src, p.omega, p.extra["Omega"], s,
                                 shared, p.pml_m, p.pml_lnR)
    tol = TOL_FIELD_FP64 if prec == "fp64" else TOL_FIELD_MIXED
    assert st.rel_residual <= TOL_RES and st.nrhs == 1
    # errors relative to the whole coupled field (the quantity the residual
    # bound controls; a weak sideband alone carries a larger relative error)
    for c, got in enumerate((ez, hx, hy)):
        want = np.stack([ref[j][c] for j in range(2 * s + 1)])
        assert rel(got, want) <= tol, (c, rel(got, want))


def test_mf_errors(lib, fdfd):
    from fdfd_gb300 import workloads as W
    p = W.modulated_waveguide(dh=0.05, L=4.0)
    h = mf_handle(fdfd, p, fdfd.FDFD_PREC_MIXED, 1, True)
    E = fdfd._lib.FDFD_EINVAL
    with pytest.raises(fdfd.FDFDError) as e:
        h.solve(p.src)                                   # before fdfd_mf_factor
    assert e.value.code == E
    with pytest.raises(fdfd.FDFDError) as e:
        h.factor(p.omega, 1.5 * p.omega)                 # ω - Ω < 0
    assert e.value.code == E
    with pytest.raises(fdfd.FDFDError) as e:
        fdfd._lib.Handle.factor(h, p.omega)              # single-frequency entry point
    assert e.value.code == E
    bad = p.extra["deps"].copy()
    bad[3, 3] = np.inf
    with pytest.raises(fdfd.FDFDError) as e:
        h.set_deps(bad)
    assert e.value.code == E
    h.close()
