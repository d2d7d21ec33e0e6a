"""GPU parity of the CUDA solve path (through the C ABI) against the FP64 oracle."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden")
DRIVEN = ["tm_point_guide_60x40", "tm_design_48x72", "te_design_64x40"]

# tolerances (relative 2-norm errors)
TOL_RES = 1e-10        # ||b - A x|| / ||b||
TOL_FIELD_MIXED = 1e-8  # field error vs FP64 oracle, mixed precision
TOL_FIELD_FP64 = 1e-10  # field error vs FP64 oracle, FP64 factorization


def rel(a, b):
    return float(np.linalg.norm(np.ravel(a - b)) / np.linalg.norm(np.ravel(b)))


def handle_for(fdfd, Nx, Ny, npml, dx, dy, m, lnR, pol, prec):
    h = fdfd._lib.Handle(Nx, Ny, npml[0], npml[1], dx, dy, 1e-6, m, lnR, pol, prec)
    h.set_refinement(TOL_RES, 40)
    return h


def oracle_solve(oracle, p, pol):
    g = oracle.Grid((p.Nx, p.Ny), tuple(p.npml), ((0.0, 0.0), (p.Nx * p.dx, p.Ny * p.dy)))
    return oracle.solve(g, p.eps, p.src, p.omega, pol, p.pml_m, p.pml_lnR)


# ---------------------------------------------------------------------------
# block GEMM kernels
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("M,N,K", [(100, 70, 40), (128, 256, 32), (480, 480, 480), (300, 520, 96)])
@pytest.mark.parametrize("kind", ["tc", "tc64", "tc128", "tc128x2", "tc256", "tcs", "tcs64", "tcs128x2", "tcs256",
                                  "simt32", "simt64"])
def test_block_gemm(lib, fdfd, M, N, K, kind):
    """tc: the tensor-core kernel with the launcher's tile width, residual
    planes formed in shared memory; tcNN forces 128 x NN tiles (tc128x2: the 128-column
    tile sized for two CTAs per SM); tcs*: operands
    passed pre-split (four planes); simt32/simt64: the CUDA-core kernels."""
    rng = np.random.default_rng(M * 7 + N * 3 + K)
    A = rng.standard_normal((M, K)) + 1j * rng.standard_normal((M, K))
    B = rng.standard_normal((N, K)) + 1j * rng.standard_normal((N, K))
    ref = A @ B.T
    prec = fdfd.FDFD_PREC_FP64 if kind == "simt64" else fdfd.FDFD_PREC_MIXED
    use_tc = {"tc": 1, "tc64": 64, "tc128": 128, "tc128x2": 129, "tc256": 256, "tcs": -1, "tcs64": -64,
              "tcs128x2": -129, "tcs256": -256}.get(kind, 0)
    C, ms = fdfd._lib.debug_gemm(A, B, prec, use_tc)
    err = rel(C, ref)
    # FP32 inputs carry 6e-8 relative rounding; 3xTF32 products keep ~2^-21 per
    # product, and the tensor core's FP32 accumulation (truncating, measured
    # 9e-7 at K=32, 7.5e-6 at K=480, 1.5e-5 at K=1024) grows about linearly in K.
    tol = 2.5e-8 * K + 1e-6 if kind.startswith("tc") else {"simt32": 1e-6, "simt64": 1e-13}[kind]
    assert err <= tol, (kind, err)


# ---------------------------------------------------------------------------
# assembly
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("name", DRIVEN)
def test_stencil_matches_oracle(lib, fdfd, name):
    g = np.load(os.path.join(GOLD, name + ".npz"))
    Nx, Ny = int(g["Nx"]), int(g["Ny"])
    h = handle_for(fdfd, Nx, Ny, g["npml"], float(g["dx"]), float(g["dy"]), float(g["pml_m"]),
                   float(g["pml_lnR"]), int(g["pol"]), fdfd.FDFD_PREC_FP64)
    h.set_eps(g["eps"])
    h.factor(float(g["omega"]))
    st = h.stencil()
    h.close()
    ref = np.swapaxes(g["stencil"].reshape(5, Ny, Nx), 1, 2)
    scale = np.abs(ref).max()
    assert np.abs(st - ref).max() <= 1e-14 * scale


# ---------------------------------------------------------------------------
# driven solves
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("name", DRIVEN)
def test_solve_golden(lib, fdfd, name, prec):
    g = np.load(os.path.join(GOLD, name + ".npz"))
    Nx, Ny = int(g["Nx"]), int(g["Ny"])
    P = fdfd.FDFD_PREC_FP64 if prec == "fp64" else fdfd.FDFD_PREC_MIXED
    h = handle_for(fdfd, Nx, Ny, g["npml"], float(g["dx"]), float(g["dy"]), float(g["pml_m"]),
                   float(g["pml_lnR"]), int(g["pol"]), P)
    h.set_eps(g["eps"])
    h.factor(float(g["omega"]))
    f1, f2, f3, st = h.solve(g["src"])
    h.close()
    tol = TOL_FIELD_FP64 if prec == "fp64" else TOL_FIELD_MIXED
    assert st.rel_residual <= TOL_RES
    for f, k in ((f1, "f1"), (f2, "f2"), (f3, "f3")):
        assert rel(f, g[k]) <= tol, (k, rel(f, g[k]))


@pytest.mark.parametrize("shape", [(3, 3), (5, 7), (7, 5), (16, 3), (3, 16), (33, 17), (17, 33), (40, 41),
                                   (64, 64), (61, 37)])
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_solve_ring_shapes(lib, fdfd, oracle, shape, prec):
    """Odd/even ring sizes, both block orientations, tiny grids, complex ϵᵣ."""
    Nx, Ny = shape
    rng = np.random.default_rng(Nx * 100 + Ny)
    npml = (min(4, Nx // 4), min(4, Ny // 4))
    eps = rng.uniform(1, 4, (Nx, Ny)) + 1j * rng.uniform(0, 0.1, (Nx, Ny))
    src = rng.standard_normal((Nx, Ny)) + 1j * rng.standard_normal((Nx, Ny))
    dx = dy = 0.05
    omega = 2 * np.pi * oracle.C0 / 1.55e-6
    P = fdfd.FDFD_PREC_FP64 if prec == "fp64" else fdfd.FDFD_PREC_MIXED
    h = handle_for(fdfd, Nx, Ny, npml, dx, dy, 4.0, np.log(1e-8), fdfd.TM, P)
    h.set_eps(eps)
    h.factor(omega)
    f1, f2, f3, st = h.solve(src)
    h.close()
    g = oracle.Grid((Nx, Ny), npml, ((0.0, 0.0), (Nx * dx, Ny * dy)))
    r1, r2, r3 = oracle.solve(g, eps, src, omega, oracle.TM, 4.0, np.log(1e-8))
    tol = TOL_FIELD_FP64 if prec == "fp64" else TOL_FIELD_MIXED
    assert st.rel_residual <= TOL_RES
    assert rel(f1, r1) <= tol and rel(f2, r2) <= tol and rel(f3, r3) <= tol


def test_point_guide_200x120(lib, fdfd, oracle):
    """Plain FP64 TM solve: 200x120 straight guide, Jz=1 point source."""
    from fdfd_gb300 import workloads as W
    p = W.point_source_guide()
    ref = oracle_solve(oracle, p, oracle.TM)
    for prec, tol in ((fdfd.FDFD_PREC_FP64, TOL_FIELD_FP64), (fdfd.FDFD_PREC_MIXED, TOL_FIELD_MIXED)):
        h = handle_for(fdfd, p.Nx, p.Ny, p.npml, p.dx, p.dy, p.pml_m, p.pml_lnR, fdfd.TM, prec)
        h.set_eps(p.eps)
        h.factor(p.omega)
        f1, f2, f3, st = h.solve(p.src)
        h.close()
        assert st.rel_residual <= TOL_RES
        assert max(rel(f1, ref[0]), rel(f2, ref[1]), rel(f3, ref[2])) <= tol


def test_fp64_fallback(lib, fdfd, oracle):
    """A MIXED handle whose refinement cannot reach tol within max_iter solves
    (one fewer than the FP32 factor needs) factors the operator again in FP64
    and finishes with it; with the fallback off the call reports
    FDFD_ENOCONV, and the next factorization is FP32 again."""
    from fdfd_gb300 import workloads as W
    p = W.point_source_guide()
    ref = oracle_solve(oracle, p, oracle.TM)
    h = handle_for(fdfd, p.Nx, p.Ny, p.npml, p.dx, p.dy, p.pml_m, p.pml_lnR, fdfd.TM, fdfd.FDFD_PREC_MIXED)
    h.set_eps(p.eps)
    h.factor(p.omega)
    _, _, _, st = h.solve(p.src)
    n_mixed = st.iterations
    assert st.fp64_fallback == 0 and st.factor_precision == fdfd.FDFD_PREC_MIXED and n_mixed >= 3
    h.set_refinement(TOL_RES, n_mixed - 1)
    f1, f2, f3, st = h.solve(p.src)
    assert st.fp64_fallback == 1 and st.factor_precision == fdfd.FDFD_PREC_FP64
    assert st.rel_residual <= TOL_RES
    assert max(rel(f1, ref[0]), rel(f2, ref[1]), rel(f3, ref[2])) <= TOL_FIELD_FP64
    h.set_fallback(False)
    h.factor(p.omega)
    with pytest.raises(fdfd.FDFDError) as e:
        h.solve(p.src)
    assert e.value.code == fdfd._lib.FDFD_ENOCONV
    h.set_refinement(TOL_RES, 40)
    _, _, _, st = h.solve(p.src)
    h.close()
    assert st.fp64_fallback == 0 and st.factor_precision == fdfd.FDFD_PREC_MIXED and st.rel_residual <= TOL_RES


def test_block_size_above_512(lib, fdfd):
    """Blocks of more than 512 unknowns take the two-rows-per-thread panel
    kernels (FP32 panel width 16, FP64 width 8).  Both factorizations must
    reach the residual bound, and the two fields must agree."""
    Nx, Ny = 530, 516
    rng = np.random.default_rng(5)
    eps = rng.uniform(1, 3, (Nx, Ny)) + 1j * rng.uniform(0, 0.05, (Nx, Ny))
    src = np.zeros((Nx, Ny), complex)
    src[Nx // 3, Ny // 2] = 1j
    src[2 * Nx // 3, Ny // 3] = 0.5
    omega = 2 * np.pi * 299792458.0 / 1.55e-6
    out = {}
    for prec in (fdfd.FDFD_PREC_FP64, fdfd.FDFD_PREC_MIXED):
        h = handle_for(fdfd, Nx, Ny, (12, 12), 0.05, 0.05, 4.0, np.log(1e-8), fdfd.TM, prec)
        h.set_eps(eps)
        h.factor(omega)
        f1, _, _, st = h.solve(src)
        h.close()
        assert st.block == 516 and st.rel_residual <= TOL_RES
        out[prec] = f1
    assert rel(out[fdfd.FDFD_PREC_MIXED], out[fdfd.FDFD_PREC_FP64]) <= TOL_FIELD_MIXED


def test_profile_classes(lib, fdfd):
    """Per-class device timing: every class of a mixed solve is populated."""
    from fdfd_gb300 import workloads as W
    p = W.point_source_guide()
    h = handle_for(fdfd, p.Nx, p.Ny, p.npml, p.dx, p.dy, p.pml_m, p.pml_lnR, fdfd.TM, fdfd.FDFD_PREC_MIXED)
    h.set_eps(p.eps)
    h.set_profiling(True)
    h.factor(p.omega)
    _, _, _, st = h.solve(p.src)
    prof = h.profile()
    h.close()
    gk = "gemm_tc" if st.tc_gemm else "gemm_simt"
    for k in (gk, "gj_panel", "gj_update", "sweep", "residual", "level1"):
        assert prof[k]["launches"] > 0 and prof[k]["ms"] > 0, k
    assert prof[gk]["work"] > 0 and prof["gj_update"]["work"] > 0 and prof["level1"]["work"] > 0


def test_multi_rhs_matches_single(lib, fdfd, oracle):
    from fdfd_gb300 import workloads as W
    p = W.design_guide(96, 64, design=(24, 24), seed=3, npml=10)
    rng = np.random.default_rng(1)
    srcs = rng.standard_normal((3, p.Nx, p.Ny)) + 1j * rng.standard_normal((3, p.Nx, p.Ny))
    h = handle_for(fdfd, p.Nx, p.Ny, p.npml, p.dx, p.dy, p.pml_m, p.pml_lnR, fdfd.TM, fdfd.FDFD_PREC_MIXED)
    h.set_eps(p.eps)
    h.factor(p.omega)
    F1, _, _, st = h.solve(srcs)
    assert st.rel_residual <= TOL_RES
    for k in range(3):
        f1, _, _, _ = h.solve(srcs[k])
        assert rel(F1[k], f1) <= 1e-9
    h.close()


def test_reference_dipole_problem(lib, fdfd, oracle):
    """The reference's own test problem (test/runtests.jl:7-21): 6x6 µm, dh = 0.01,
    15 PML cells, ω = 2π·200 THz, point source 1im at (0, 0), default PML
    grading; the GPU solve must agree with the FP64 direct solve as the
    reference's two solvers must (√eps relative), here to the mixed tolerance."""
    d = fdfd.Device(fdfd.Grid(0.01, [15, 15], [-3, 3], [-3, 3]), 2 * np.pi * 200e12)
    fdfd.setup_src(d, fdfd.Point(0, 0))
    field = fdfd.solve(d, fdfd.TM, precision="mixed")
    g = oracle.Grid.from_ranges(0.01, [15, 15], [-3, 3], [-3, 3])
    src = np.zeros(g.N, dtype=complex)
    src[g.x2ind(0), g.y2ind(0)] = 1j
    r = oracle.solve(g, np.ones(g.N, dtype=complex), src, 2 * np.pi * 200e12, oracle.TM)
    assert rel(field["Ez"], r[0]) <= TOL_FIELD_MIXED
    assert rel(field["Hx"], r[1]) <= TOL_FIELD_MIXED
    assert rel(field["Hy"], r[2]) <= TOL_FIELD_MIXED


# ---------------------------------------------------------------------------
# adjoint gradient
# ---------------------------------------------------------------------------
def adjoint_problem_small():
    from fdfd_gb300 import workloads as W
    p = W.adjoint_problem(Nx=64, Ny=48, design=(16, 16), seed=9, waist=4.0, npml=8)
    return p


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_adjoint_matches_oracle(lib, fdfd, oracle, prec):
    p = adjoint_problem_small()
    P = fdfd.FDFD_PREC_FP64 if prec == "fp64" else fdfd.FDFD_PREC_MIXED
    h = handle_for(fdfd, p.Nx, p.Ny, p.npml, p.dx, p.dy, p.pml_m, p.pml_lnR, fdfd.TM, P)
    h.set_eps(p.eps)
    h.factor(p.omega)
    J, grad, ez, st = h.adjoint(p.src, p.extra["mvec"])
    h.close()
    g = oracle.Grid((p.Nx, p.Ny), p.npml, ((0.0, 0.0), (p.Nx * p.dx, p.Ny * p.dy)))
    J0, grad0, E0 = oracle.adjoint_gradient(g, p.eps, p.src, p.omega, p.extra["mvec"], p.pml_m, p.pml_lnR)
    tol = TOL_FIELD_FP64 if prec == "fp64" else TOL_FIELD_MIXED
    assert st.rel_residual <= TOL_RES
    assert abs(J - J0) <= tol * J0
    assert rel(ez, E0) <= tol
    assert rel(grad, grad0) <= 10 * tol


def test_adjoint_matches_finite_differences(lib, fdfd):
    """Central differences (step 1e-4 in ϵᵣ, FP64 solves) on seeded design pixels, ≤ 1e-5 relative."""
    p = adjoint_problem_small()
    h = handle_for(fdfd, p.Nx, p.Ny, p.npml, p.dx, p.dy, p.pml_m, p.pml_lnR, fdfd.TM, fdfd.FDFD_PREC_FP64)
    h.set_eps(p.eps)
    h.factor(p.omega)
    J, grad, _, _ = h.adjoint(p.src, p.extra["mvec"])
    x0, y0, dwx, dwy = p.extra["design_box"]
    rng = np.random.default_rng(17)
    pix = [(x0 + rng.integers(dwx), y0 + rng.integers(dwy)) for _ in range(4)]
    for (i, j) in pix:
        Js = []
        for d in (1e-4, -1e-4):
            e = p.eps.copy()
            e[i, j] += d
            h.set_eps(e)
            h.factor(p.omega)
            Js.append(h.adjoint(p.src, p.extra["mvec"])[0])
        fd = (Js[0] - Js[1]) / 2e-4
        assert abs(fd - grad[i, j]) <= 1e-5 * abs(grad[i, j]) + 1e-9 * J, (i, j, fd, grad[i, j])
    h.close()


# ---------------------------------------------------------------------------
# eigenfrequency
# ---------------------------------------------------------------------------
def match_eigs(om, ref):
    """max relative distance from each reference eigenfrequency to the nearest computed one"""
    return max(np.min(np.abs(om - r)) / abs(r) for r in ref)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_eigfreq_golden(lib, fdfd, prec):
    g = np.load(os.path.join(GOLD, "tm_phc_eigen_56.npz"))
    Nx, Ny = int(g["Nx"]), int(g["Ny"])
    P = fdfd.FDFD_PREC_FP64 if prec == "fp64" else fdfd.FDFD_PREC_MIXED
    h = handle_for(fdfd, Nx, Ny, g["npml"], float(g["dx"]), float(g["dy"]), float(g["pml_m"]),
                   float(g["pml_lnR"]), int(g["pol"]), P)
    h.set_eps(g["eps"])
    nev = len(g["omega"])
    om, lam, f, st = h.eigfreq(float(g["omega0"]), nev)
    assert match_eigs(om, g["omega"]) <= 1e-8
    # eigenvectors: (A - σI) y = (λ - σ) y with the assembled shifted operator
    sigma = -float(g["omega0"]) ** 2 * (fdfd.MU0 * 1e-6) * (fdfd.EPS0 * 1e-6)   # eigen.jl:86
    ay = h.apply(f[:, 0])
    for q in range(nev):
        r = ay[q] - (lam[q] - sigma) * f[q, 0]
        assert np.linalg.norm(r) <= 1e-7 * abs(lam[q] - sigma) * np.linalg.norm(f[q, 0])
    h.close()


# ---------------------------------------------------------------------------
# error behaviour
# ---------------------------------------------------------------------------
def test_errors(lib, fdfd):
    h = handle_for(fdfd, 20, 16, (2, 2), 0.05, 0.05, 4.0, np.log(1e-8), fdfd.TM, fdfd.FDFD_PREC_MIXED)
    with pytest.raises(fdfd.FDFDError) as e:
        h.solve(np.ones((20, 16)))
    assert e.value.code == fdfd._lib.FDFD_EINVAL
    eps = np.ones((20, 16), dtype=complex)
    eps[3, 4] = np.nan
    with pytest.raises(fdfd.FDFDError) as e:
        h.set_eps(eps)
    assert e.value.code == fdfd._lib.FDFD_EINVAL and "non-finite entry at 83" in str(e.value)   # 3 + 20 * 4, x fastest
    h.set_eps(np.ones((20, 16)))
    with pytest.raises(fdfd.FDFDError):
        h.factor(-1.0)
    h.close()


def test_rejected_inputs_leave_the_handle_unchanged(lib, fdfd):
    """ϵᵣ and sources are validated on the device after the copy: a rejected ϵᵣ (NaN, inf or a
    complex zero) leaves the previous permittivity in place, a rejected source leaves the factors,
    and the handle then solves as before."""
    h = handle_for(fdfd, 40, 30, (6, 6), 0.05, 0.05, 4.0, np.log(1e-8), fdfd.TM, fdfd.FDFD_PREC_MIXED)
    eps = np.ones((40, 30), dtype=complex)
    eps[15:25, 10:20] = 6.0
    src = np.zeros((40, 30), dtype=complex)
    src[10, 15] = 1.0
    h.set_eps(eps)
    h.factor(2 * np.pi * 299792458.0 / 1.55e-6)
    ref = h.solve(src)[:3]
    for bad, msg in ((np.inf, "non-finite entry at 501"), (0.0, "is zero at 501")):
        e2 = eps.copy()
        e2[21, 12] = bad                      # index 21 + 40 * 12 = 501 in the x-fastest order
        with pytest.raises(fdfd.FDFDError) as e:
            h.set_eps(e2)
        assert e.value.code == fdfd._lib.FDFD_EINVAL and msg in str(e.value), str(e.value)
    s2 = src.copy()
    s2[3, 3] = np.nan
    with pytest.raises(fdfd.FDFDError) as e:
        h.solve(s2)
    assert e.value.code == fdfd._lib.FDFD_EINVAL
    got = h.solve(src)[:3]                    # same factors
    h.factor(2 * np.pi * 299792458.0 / 1.55e-6)
    again = h.solve(src)[:3]                  # refactored from the kept permittivity
    h.close()
    for a, b, c in zip(ref, got, again):
        assert np.array_equal(a, b) and np.array_equal(a, c)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_adjoint_vjp_matches_objective_and_oracle(lib, fdfd, oracle, prec):
    """The vector-Jacobian product (the rrule pullback) for g = 2·conj(mᵀE)·m is the
    gradient of J = |mᵀE|²; for an arbitrary cotangent it matches the oracle's
    -Re(ω²ϵ₀ λ⊙E) with λ = A⁻ᵀ g from a transposed SuperLU solve."""
    import scipy.sparse.linalg as spla
    p = adjoint_problem_small()
    P = fdfd.FDFD_PREC_FP64 if prec == "fp64" else fdfd.FDFD_PREC_MIXED
    h = handle_for(fdfd, p.Nx, p.Ny, p.npml, p.dx, p.dy, p.pml_m, p.pml_lnR, fdfd.TM, P)
    h.set_eps(p.eps)
    h.factor(p.omega)
    m = p.extra["mvec"]
    J, grad, ez, _ = h.adjoint(p.src, m)
    s = np.sum(m * ez)
    gvjp, ez2, st = h.adjoint_vjp(p.src, 2 * np.conj(s) * m)
    tol = TOL_FIELD_FP64 if prec == "fp64" else TOL_FIELD_MIXED
    assert st.rel_residual <= TOL_RES
    assert rel(gvjp, grad) <= 10 * tol
    rng = np.random.default_rng(4)
    g = rng.standard_normal((p.Nx, p.Ny)) + 1j * rng.standard_normal((p.Nx, p.Ny))
    gr, E, _ = h.adjoint_vjp(p.src, g)
    h.close()
    og = oracle.Grid((p.Nx, p.Ny), p.npml, ((0.0, 0.0), (p.Nx * p.dx, p.Ny * p.dy)))
    A = oracle.assemble(og, p.eps, p.omega, oracle.TM, p.pml_m, p.pml_lnR)
    lu = spla.splu(A.tocsc())
    E0 = lu.solve(1j * p.omega * oracle.vec(p.src))
    lam = lu.solve(oracle.vec(g), trans="T")
    eps0 = oracle.normalize_parameters(1e-6)[0]
    g0 = oracle.unvec(-np.real(p.omega ** 2 * eps0 * lam * E0), (p.Nx, p.Ny))
    assert rel(gr, g0) <= 10 * tol
