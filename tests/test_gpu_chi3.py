"""GPU parity of the χ³ nonlinear solve (solve(d::χ3Device, method),
src/solver/nonlinear.jl) through the C ABI against the FP64 oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def problem(oracle, strength=0.05):
    """60x40 point-source guide; χ on the guide rows, scaled so that the χ³ term
    reaches `strength` of the linear ω²ϵ term where the linear field peaks."""
    from fdfd_gb300 import workloads as W
    p = W.point_source_guide(60, 40, npml=8)
    g = oracle.Grid((p.Nx, p.Ny), p.npml, ((0.0, 0.0), (p.Nx * p.dx, p.Ny * p.dy)))
    chi = np.zeros((p.Nx, p.Ny))
    chi[:, 15:25] = 1.0
    ez = oracle.solve(g, p.eps, p.src, p.omega, oracle.TM, p.pml_m, p.pml_lnR)[0]
    c = oracle.chi3_coeff(g, chi, p.omega).max() * np.abs(ez[chi > 0]).max() ** 2
    lin = p.omega ** 2 * oracle.EPS0 * g.L0 * 12.25
    return p, g, chi * strength * lin / c


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("method", ["born", "newton"])
def test_chi3_matches_oracle(lib, fdfd, oracle, method, prec):
    p, g, chi = problem(oracle)
    ref, err_ref = oracle.solve_chi3(g, p.eps, chi, p.src, p.omega, method, p.pml_m, p.pml_lnR)
    pr = fdfd.FDFD_PREC_FP64 if prec == "fp64" else fdfd.FDFD_PREC_MIXED
    h = fdfd._lib.Handle(p.Nx, p.Ny, p.npml[0], p.npml[1], p.dx, p.dy, 1e-6, p.pml_m, p.pml_lnR, fdfd.TM, pr)
    h.set_refinement(1e-10, 60)
    h.set_eps(p.eps)
    h.factor(p.omega)
    code = fdfd._lib.FDFD_CHI3_BORN if method == "born" else fdfd._lib.FDFD_CHI3_NEWTON
    ez, hx, hy, err, st = h.chi3_solve(chi, p.src, code, 1e-12, 50)
    h.close()
    assert err[0] == 1.0 and err[-1] <= 1e-12
    assert abs(len(err) - len(err_ref)) <= 1, (len(err), len(err_ref))
    for got, want in zip((ez, hx, hy), ref):
        assert np.linalg.norm(got - want) <= 1e-9 * np.linalg.norm(want)


def test_chi3_newton_converges_quadratically(lib, fdfd, oracle):
    """At 20% nonlinearity Newton needs far fewer steps than Born, and both reach
    the same field."""
    p, g, chi = problem(oracle, 0.2)
    h = fdfd._lib.Handle(p.Nx, p.Ny, p.npml[0], p.npml[1], p.dx, p.dy, 1e-6, p.pml_m, p.pml_lnR, fdfd.TM,
                         fdfd.FDFD_PREC_MIXED)
    h.set_eps(p.eps)
    h.factor(p.omega)
    e_b, _, _, err_b, _ = h.chi3_solve(chi, p.src, fdfd._lib.FDFD_CHI3_BORN, 1e-11, 200)
    e_n, _, _, err_n, _ = h.chi3_solve(chi, p.src, fdfd._lib.FDFD_CHI3_NEWTON, 1e-11, 50)
    h.close()
    assert len(err_n) < len(err_b) and err_n[-1] <= 1e-11
    assert np.linalg.norm(e_b - e_n) <= 1e-9 * np.linalg.norm(e_n)


def test_chi3_host_mirror_and_errors(lib, fdfd, oracle):
    p, g, chi = problem(oracle)
    grid = fdfd.Grid.from_cells(p.Nx, p.Ny, p.dx, p.dy, p.npml)
    d = fdfd.Chi3Device(grid, p.omega, eps=p.eps.copy(), chi=chi, src=p.src.copy())
    f = fdfd.solve(d, fdfd.IterativeMethodGN)
    ref, _ = oracle.solve_chi3(g, p.eps, chi, p.src, p.omega, "newton", 3.5, -12.0)
    assert np.linalg.norm(f["Ez"] - ref[0]) <= 1e-9 * np.linalg.norm(ref[0])
    h = fdfd._lib.Handle(p.Nx, p.Ny, p.npml[0], p.npml[1], p.dx, p.dy, 1e-6, p.pml_m, p.pml_lnR, fdfd.TM,
                         fdfd.FDFD_PREC_MIXED)
    h.set_eps(p.eps)
    with pytest.raises(fdfd.FDFDError) as e:          # not factored
        h.chi3_solve(chi, p.src)
    assert e.value.code == fdfd._lib.FDFD_EINVAL
    h.factor(p.omega)
    with pytest.raises(fdfd.FDFDError) as e:          # two Born steps are not enough
        h.chi3_solve(chi, p.src, fdfd._lib.FDFD_CHI3_BORN, 1e-12, 2)
    assert e.value.code == fdfd._lib.FDFD_ENOCONV
    _, _, _, st = h.solve(p.src)                      # the handle is a linear solver again
    h.close()
    assert st.rel_residual <= 1e-10
