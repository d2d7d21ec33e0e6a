"""GPU parity on the full-size benchmark configurations and on the eigenfield
recovery, against the FP64 oracle (through the C ABI).

* the 800 x 480 design-guide solve (the benchmark's workload) in both
  precisions against the oracle's SuperLU solve;
* the 1000 x 600 adjoint gradient against the oracle's FP64 adjoint and
  against central finite differences on 32 seeded design pixels;
* the 280 x 280 rod-lattice cavity eigenfrequencies with the FP64 and the
  mixed factor;
* TM and TE eigenfrequencies and their recovered fields (eigen.jl:89-93 and
  :97-114) against the oracle's ARPACK solve.
The full-size oracle solves run in spawned processes (tests/_big_oracle.py)
while the other GPU tests run.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_RES = 1e-10
TOL_FIELD_MIXED = 1e-8
TOL_FIELD_FP64 = 1e-10


def rel(a, b):
    return float(np.linalg.norm(np.ravel(a - b)) / np.linalg.norm(np.ravel(b)))


def make(fdfd, p, pol, prec, tol=TOL_RES, max_iter=80):
    h = fdfd._lib.Handle(p.Nx, p.Ny, p.npml[0], p.npml[1], p.dx, p.dy, 1e-6, p.pml_m, p.pml_lnR, pol, prec)
    h.set_refinement(tol, max_iter)
    return h


# ---------------------------------------------------------------------------
# 800 x 480 design guide (the benchmark's workload)
# ---------------------------------------------------------------------------
@pytest.mark.big_oracle("design_guide")
@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_design_guide_800x480_vs_oracle(lib, fdfd, big_oracle, prec):
    """Field error of the GPU solve against the FP64 SuperLU solve of the same
    800 x 480 problem: <= 1e-8 (mixed factor + FP64 FGMRES to 1e-10) and
    <= 1e-10 (FP64 factor)."""
    from fdfd_gb300 import workloads as W
    p = W.design_guide()
    P = fdfd.FDFD_PREC_MIXED if prec == "mixed" else fdfd.FDFD_PREC_FP64
    h = make(fdfd, p, fdfd.TM, P)
    h.set_eps(p.eps)
    h.factor(p.omega)
    f1, f2, f3, st = h.solve(p.src)
    h.close()
    ref = big_oracle("design_guide")
    tol = TOL_FIELD_MIXED if prec == "mixed" else TOL_FIELD_FP64
    assert st.rel_residual <= TOL_RES
    errs = [rel(f, r) for f, r in zip((f1, f2, f3), ref)]
    assert max(errs) <= tol, errs


# ---------------------------------------------------------------------------
# 1000 x 600 adjoint gradient
# ---------------------------------------------------------------------------
@pytest.mark.big_oracle("adjoint")
def test_adjoint_1000x600_vs_oracle_and_finite_differences(lib, fdfd, big_oracle):
    """Gradient of J = |mᵀE|² over the 300 x 300 design (mixed factor, FP64
    refinement to 1e-10) against the oracle's FP64 adjoint (SuperLU forward and
    transposed solves), then central differences with step 1e-4 in ϵᵣ on 32
    seeded design pixels, each J from a fresh factorization refined to 1e-13
    (FP64-accurate J; the mixed factor keeps the 64 factorizations to seconds):
    |fd - g| <= 1e-5 |g| + 1e-9 J per pixel, the floor being the resolution of
    a difference of two J values accurate to ~1e-13."""
    from fdfd_gb300 import workloads as W
    p = W.adjoint_problem()
    h = make(fdfd, p, fdfd.TM, fdfd.FDFD_PREC_MIXED)
    h.set_eps(p.eps)
    h.factor(p.omega)
    J, grad, ez, st = h.adjoint(p.src, p.extra["mvec"])
    assert st.rel_residual <= TOL_RES
    J0, grad0, E0 = big_oracle("adjoint")
    assert abs(J - J0) <= TOL_FIELD_MIXED * J0
    assert rel(ez, E0) <= TOL_FIELD_MIXED
    x0, y0, dwx, dwy = p.extra["design_box"]
    gd, gd0 = grad[x0:x0 + dwx, y0:y0 + dwy], grad0[x0:x0 + dwx, y0:y0 + dwy]
    assert rel(gd, gd0) <= 1e-7, rel(gd, gd0)

    h.set_refinement(1e-13, 80)
    rng = np.random.default_rng(32)
    flat = rng.choice(dwx * dwy, size=32, replace=False)
    pix = [(x0 + int(k) // dwy, y0 + int(k) % dwy) for k in flat]
    hstep = 1e-4
    fd, g = [], []
    for (i, j) in pix:
        Js = []
        for d in (hstep, -hstep):
            e = p.eps.copy()
            e[i, j] += d
            h.set_eps(e)
            h.factor(p.omega)
            Js.append(h.adjoint(p.src, p.extra["mvec"])[0])
        fd.append((Js[0] - Js[1]) / (2 * hstep))
        g.append(grad[i, j])
    h.close()
    fd, g = np.array(fd), np.array(g)
    bad = [(pix[k], fd[k], g[k]) for k in range(len(pix)) if abs(fd[k] - g[k]) > 1e-5 * abs(g[k]) + 1e-9 * J]
    assert not bad, bad
    assert np.linalg.norm(fd - g) <= 1e-5 * np.linalg.norm(g)


# ---------------------------------------------------------------------------
# eigenfrequencies
# ---------------------------------------------------------------------------
def match_eigs(om, ref):
    """max relative distance from each reference eigenfrequency to the nearest computed one"""
    return max(np.min(np.abs(om - r)) / abs(r) for r in ref)


@pytest.mark.big_oracle("cavity")
@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_eigfreq_phc_cavity_280(lib, fdfd, big_oracle, prec):
    """12 x 12 rod-lattice cavity (ϵ = 8.9, r = 0.2a, 20 cells per a, 20-cell
    PML): the six eigenfrequencies nearest ωa/2πc = 0.38 with the FP64 factor
    and with the mixed factor refined inside every Arnoldi step."""
    from fdfd_gb300 import workloads as W
    p, w0 = W.phc_cavity()
    P = fdfd.FDFD_PREC_MIXED if prec == "mixed" else fdfd.FDFD_PREC_FP64
    h = make(fdfd, p, fdfd.TM, P)
    h.set_eps(p.eps)
    om, lam, f, st = h.eigfreq(w0, 6)
    h.close()
    assert match_eigs(om, big_oracle("cavity")) <= 1e-8


def eigen_problem(pol):
    """A 52 x 44 grid, 8 PML cells, a seeded random dielectric block: the four
    eigenvalues nearest σ are simple and separated by >= 0.6 % of |σ|."""
    rng = np.random.default_rng(11)
    Nx, Ny, npml, dx = 52, 44, 8, 0.05
    eps = np.ones((Nx, Ny), complex)
    eps[14:38, 12:32] = rng.uniform(1, 8, (24, 20))
    w0 = 2 * np.pi * 299792458.0 / 1.0e-6
    return Nx, Ny, npml, dx, eps, w0


def phase_normalised(f1, f2, f3):
    """Unit-norm f1 with its largest entry real and positive, the same factor on f2, f3."""
    k = np.argmax(np.abs(f1))
    c = np.conj(f1.flat[k]) / abs(f1.flat[k]) / np.linalg.norm(f1)
    return f1 * c, f2 * c, f3 * c


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("pol", ["TM", "TE"])
def test_eigfreq_and_fields_vs_oracle(lib, fdfd, oracle, pol, prec):
    """Eigenfrequencies and recovered eigenfields against the oracle's ARPACK
    shift-invert: TM H from forward differences (eigen.jl:89-93), TE
    Ex = Tϵx⁻¹ δyb Hz / iω, Ey = -Tϵy⁻¹ δxb Hz / iω (eigen.jl:106-114), both
    scaled like the mode (unit norm, largest entry real and positive)."""
    Nx, Ny, npml, dx, eps, w0 = eigen_problem(pol)
    P = fdfd.FDFD_PREC_MIXED if prec == "mixed" else fdfd.FDFD_PREC_FP64
    opol = oracle.TM if pol == "TM" else oracle.TE
    h = fdfd._lib.Handle(Nx, Ny, npml, npml, dx, dx, 1e-6, 4.0, np.log(1e-8), opol, P)
    h.set_refinement(1e-12, 80)
    h.set_eps(eps)
    nev = 4
    om, lam, f, st = h.eigfreq(w0, nev, tol=1e-12)
    h.close()
    g = oracle.Grid((Nx, Ny), (npml, npml), ((0.0, 0.0), (Nx * dx, Ny * dx)))
    w_ref, f_ref, _ = oracle.eigenfrequency(g, eps, w0, opol, nev, "LM", 4.0, np.log(1e-8),
                                            v0=np.ones(Nx * Ny, dtype=complex))
    assert match_eigs(om, w_ref) <= 1e-10
    for q in range(nev):
        k = int(np.argmin(np.abs(w_ref - om[q])))
        got = phase_normalised(f[q, 0], f[q, 1], f[q, 2])
        ref = phase_normalised(*f_ref[k])
        errs = [rel(a, b) for a, b in zip(got, ref)]
        assert max(errs) <= 1e-8, (q, errs)


@pytest.mark.parametrize("which", ["LR", "SR", "LI"])
def test_eigfreq_which_vs_oracle(lib, fdfd, oracle, which):
    """Arpack's `which` in shift-invert mode ranks θ = 1/(λ - σ): the selections
    other than :LM against scipy's ARPACK with the same `which` and shift."""
    Nx, Ny, npml, dx, eps, w0 = eigen_problem("TM")
    h = fdfd._lib.Handle(Nx, Ny, npml, npml, dx, dx, 1e-6, 4.0, np.log(1e-8), oracle.TM, fdfd.FDFD_PREC_FP64)
    h.set_refinement(1e-12, 80)
    h.set_eps(eps)
    code = {"LM": 0, "LR": 1, "SM": 2, "SR": 3, "LI": 4, "SI": 5}[which]
    nev = 3
    om, lam, f, st = h.eigfreq(w0, nev, which=code, tol=1e-12)
    h.close()
    g = oracle.Grid((Nx, Ny), (npml, npml), ((0.0, 0.0), (Nx * dx, Ny * dx)))
    w_ref, _, _ = oracle.eigenfrequency(g, eps, w0, oracle.TM, nev, which, 4.0, np.log(1e-8),
                                        v0=np.ones(Nx * Ny, dtype=complex))
    assert match_eigs(om, w_ref) <= 1e-10
