"""CPU checks that pin the FP64 oracle (no GPU needed).

The reference holds no golden vectors (its test/runtests.jl only checks that
two FP64 direct solvers agree), so the oracle is pinned by hand-derived
operator entries, solver agreement, an analytic Green's-function answer and
the committed golden fixtures (regression).
"""
import os

import numpy as np
import pytest
import scipy.sparse as sp
from scipy.special import hankel2

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def small_grid(oracle, N=(4, 3), npml=(1, 1), d=(0.1, 0.2)):
    return oracle.Grid(N, npml, ((0.0, 0.0), (N[0] * d[0], N[1] * d[1])))


def test_constants(oracle):
    # src/types.jl:6-9
    assert oracle.EPS0 == 8.85418782e-12 and oracle.MU0 == 1.25663706e-6
    assert oracle.C0 == pytest.approx(299792458.0, rel=1e-8)
    assert oracle.normalize_parameters(1e-6) == (oracle.EPS0 * 1e-6, oracle.MU0 * 1e-6, oracle.C0 / 1e-6)


def test_grid_round_half_even(oracle):
    # src/grid.jl:28: N = round(L/dh), Julia rounds half to even
    g = oracle.Grid.from_ranges(1.0, [0, 0], [0.0, 2.5], [0.0, 3.5])
    assert g.N == (2, 4)
    assert np.allclose(g.xc(), [0.625, 1.875])


def test_delta_hand_entries(oracle):
    g = small_grid(oracle)
    dx, dy = g.dx(), g.dy()
    f1 = np.array([[-1, 1, 0, 0], [0, -1, 1, 0], [0, 0, -1, 1], [1, 0, 0, -1]]) / dx
    b1 = np.array([[1, 0, 0, -1], [-1, 1, 0, 0], [0, -1, 1, 0], [0, 0, -1, 1]]) / dx
    assert np.array_equal(oracle.delta(oracle.X, oracle.FORWARD, g).toarray(), np.kron(np.eye(3), f1))
    assert np.array_equal(oracle.delta(oracle.X, oracle.BACKWARD, g).toarray(), np.kron(np.eye(3), b1))
    fy = np.array([[-1, 1, 0], [0, -1, 1], [1, 0, -1]]) / dy
    by = np.array([[1, 0, -1], [-1, 1, 0], [0, -1, 1]]) / dy
    assert np.array_equal(oracle.delta(oracle.Y, oracle.FORWARD, g).toarray(), np.kron(fy, np.eye(4)))
    assert np.array_equal(oracle.delta(oracle.Y, oracle.BACKWARD, g).toarray(), np.kron(by, np.eye(4)))
    # backward difference is minus the transpose of forward (periodic)
    D = oracle.delta(oracle.X, oracle.FORWARD, g)
    assert np.array_equal(oracle.delta(oracle.X, oracle.BACKWARD, g).toarray(), -D.T.toarray())


def test_grid_average_periodic(oracle):
    a = np.arange(12.0).reshape(4, 3)
    gx = oracle.grid_average(a, oracle.X)
    assert gx[0, 0] == (a[0, 0] + a[3, 0]) / 2 and gx[2, 1] == (a[2, 1] + a[1, 1]) / 2
    gy = oracle.grid_average(a, oracle.Y)
    assert gy[1, 0] == (a[1, 0] + a[1, 2]) / 2


def test_sfactor_hand_values(oracle):
    # src/pml.jl:1-31 with N=10 cells, 3 PML cells, dw = 0.1, m = 3.5, lnR = -12
    g = oracle.Grid((10, 10), (3, 3), ((0.0, 0.0), (1.0, 1.0)))
    w = 2e15
    eps0 = oracle.EPS0 * 1e-6
    T = 3 * 0.1   # Npml * dw, as pml.jl:4 computes it
    smax = -(3.5 + 1) * (-12) / (2 * oracle.ETA0 * T)
    S = lambda l: 1 - 1j * smax * (l / T) ** 3.5 / (w * eps0)
    f = oracle.create_sfactor(oracle.X, oracle.FORWARD, g, w)
    b = oracle.create_sfactor(oracle.X, oracle.BACKWARD, g, w)
    ap = lambda v: pytest.approx(v, rel=1e-14)
    assert f[0] == ap(S(0.1 * 2.5)) and f[2] == ap(S(0.1 * 0.5)) and f[3] == 1 and f[9] == ap(S(0.1 * 2.5))
    assert b[0] == ap(S(0.3)) and b[2] == ap(S(0.1)) and b[7] == 1 and b[8] == ap(S(0.1)) and b[9] == ap(S(0.2))


def test_tm_operator_is_P_symmetric(oracle):
    """P·A is complex symmetric for P = diag(s_xf s_yf): the identity the adjoint uses."""
    g = oracle.Grid((12, 9), (3, 2), ((0.0, 0.0), (1.2, 0.9)))
    rng = np.random.default_rng(0)
    eps = rng.uniform(1, 5, g.N) + 0.1j
    w = 1.2e15
    A = oracle.assemble(g, eps, w, oracle.TM)
    sxf = oracle.create_sfactor(oracle.X, oracle.FORWARD, g, w)
    syf = oracle.create_sfactor(oracle.Y, oracle.FORWARD, g, w)
    P = sp.diags(oracle.vec(sxf[:, None] * syf[None, :]))
    PA = (P @ A).toarray()
    assert np.abs(PA - PA.T).max() <= 1e-15 * np.abs(PA).max()


@pytest.mark.parametrize("pol", [1, 2])
def test_solver_agreement(oracle, pol):
    """The reference's test pattern (test/runtests.jl:7-21): two independent FP64
    direct solvers agree; here SuperLU vs dense LAPACK on a small problem."""
    g = oracle.Grid((30, 24), (5, 5), ((0.0, 0.0), (1.5, 1.2)))
    rng = np.random.default_rng(pol)
    eps = rng.uniform(1, 12, g.N) + 0j
    src = np.zeros(g.N, dtype=complex)
    src[10, 12] = 1j
    w = 2 * np.pi * oracle.C0 / 1.55e-6
    A = oracle.assemble(g, eps, w, pol, 4.0, np.log(1e-8))
    b = 1j * w * oracle.vec(src)
    x1 = oracle.dolinearsolve(A, b)
    x2 = np.linalg.solve(A.toarray(), b)
    assert np.linalg.norm(x1 - x2) <= 1e-12 * np.linalg.norm(x2)


@pytest.mark.parametrize("pol", [1, 2])
def test_driven_plane_wave_closed_form(oracle, pol):
    """Driven solve (src/solver/driven.jl:4-59) without PML, uniform ϵᵣ, source e^{i(θx·i + θy·j)}:
    the operator is diagonal in that discrete Fourier mode, so
      TM: Ez = iω·src / (-k²/μ₀ + ω²ϵ₀ϵᵣ),  Hx = -δyb Ez/(iωμ₀),  Hy = δxb Ez/(iωμ₀)   (:35-41)
      TE: Hz = iω·src / (-k²/(ϵ₀ϵᵣ) + ω²μ₀), Ex = Tϵyi δyb Hz/(iω), Ey = -Tϵxi δxb Hz/(iω)   (:45-51)
    with k² = (2/dx·sin(θx/2))² + (2/dy·sin(θy/2))² and δb e^{iθj} = e^{iθj}(1 - e^{-iθ})/dh."""
    Nx, Ny, dx, dy, er = 20, 16, 0.05, 0.04, 2.25
    g = oracle.Grid((Nx, Ny), (0, 0), ((0.0, 0.0), (Nx * dx, Ny * dy)))
    eps0, mu0, _ = oracle.normalize_parameters(g.L0)
    w = 2 * np.pi * oracle.C0 / 1.55e-6
    I, J = np.meshgrid(np.arange(Nx), np.arange(Ny), indexing="ij")
    tx, ty = 2 * np.pi * 3 / Nx, 2 * np.pi * 2 / Ny
    src = np.exp(1j * (tx * I + ty * J))
    k2 = (2 / dx * np.sin(tx / 2)) ** 2 + (2 / dy * np.sin(ty / 2)) ** 2
    bx, by = (1 - np.exp(-1j * tx)) / dx, (1 - np.exp(-1j * ty)) / dy
    f = oracle.solve(g, np.full((Nx, Ny), er, dtype=complex), src, w, pol)
    if pol == oracle.TM:
        ez = 1j * w * src / (-k2 / mu0 + w ** 2 * eps0 * er)
        want = (ez, -ez * by / (1j * w * mu0), ez * bx / (1j * w * mu0))
    else:
        hz = 1j * w * src / (-k2 / (eps0 * er) + w ** 2 * mu0)
        want = (hz, hz * by / (1j * w * eps0 * er), -hz * bx / (1j * w * eps0 * er))
    for got, ref in zip(f, want):
        assert np.abs(got - ref).max() <= 1e-11 * np.abs(ref).max()


def test_dipole_matches_greens_function(oracle):
    """Known answer: a point current 1im in free space radiates
    Ez = -(i/4)·ω·μ₀·dx·dy·H0⁽²⁾(k r) (outgoing under the e^{+iωt} convention
    implied by the PML stretch s = 1 - iσ/(ωϵ₀), pml.jl:10)."""
    dx = 0.025
    N = 240
    g = oracle.Grid((N, N), (20, 20), ((-N * dx / 2, -N * dx / 2), (N * dx / 2, N * dx / 2)))
    w = 2 * np.pi * oracle.C0 / 1.55e-6
    src = np.zeros(g.N, dtype=complex)
    src[N // 2, N // 2] = 1j
    ez, _, _ = oracle.solve(g, np.ones(g.N, dtype=complex), src, w, oracle.TM, 4.0, np.log(1e-8))
    eps0, mu0, _ = oracle.normalize_parameters(1e-6)
    k = w * np.sqrt(mu0 * eps0)
    xs = g.xc()
    c = N // 2
    worst = 0.0
    for off in (40, 60, 80):
        r = abs(xs[c + off] - xs[c])
        ana = -0.25j * w * mu0 * dx * dx * hankel2(0, k * r)
        worst = max(worst, abs(ez[c + off, c] - ana) / abs(ana))
    assert worst <= 0.03, worst


@pytest.mark.parametrize("name", ["tm_point_guide_60x40", "tm_design_48x72", "te_design_64x40"])
def test_golden_regression(oracle, name):
    g = np.load(os.path.join(GOLD, name + ".npz"))
    Nx, Ny = int(g["Nx"]), int(g["Ny"])
    grid = oracle.Grid((Nx, Ny), tuple(g["npml"]), ((0.0, 0.0), (Nx * float(g["dx"]), Ny * float(g["dy"]))))
    f = oracle.solve(grid, g["eps"], g["src"], float(g["omega"]), int(g["pol"]), float(g["pml_m"]),
                     float(g["pml_lnR"]))
    for i, k in enumerate(("f1", "f2", "f3")):
        assert np.linalg.norm(f[i] - g[k]) <= 1e-12 * np.linalg.norm(g[k])


def test_adjoint_gradient_matches_fd(oracle):
    """FP64 adjoint of J = |mᵀE|² against central differences (step 1e-4 in ϵᵣ)."""
    g = oracle.Grid((28, 22), (4, 4), ((0.0, 0.0), (28 * 0.0775, 22 * 0.0775)))
    rng = np.random.default_rng(5)
    eps = rng.uniform(1, 12.25, g.N) + 0j
    src = np.zeros(g.N, dtype=complex)
    src[7, :] = np.exp(-((np.arange(22) - 11) / 4.0) ** 2)
    m = np.zeros(g.N, dtype=complex)
    m[20, :] = np.exp(-((np.arange(22) - 11) / 4.0) ** 2)
    w = 2 * np.pi * oracle.C0 / 1.55e-6
    J, grad, _ = oracle.adjoint_gradient(g, eps, src, w, m, 4.0, np.log(1e-8))
    for (i, j) in [(12, 9), (14, 11), (16, 13)]:
        ep, em = eps.copy(), eps.copy()
        ep[i, j] += 1e-4
        em[i, j] -= 1e-4
        fd = (oracle.objective(g, ep, src, w, m, 4.0, np.log(1e-8)) -
              oracle.objective(g, em, src, w, m, 4.0, np.log(1e-8))) / 2e-4
        assert abs(fd - grad[i, j]) <= 1e-5 * abs(grad[i, j]) + 1e-12 * J


# ---------------------------------------------------------------------------
# modulated device (src/solver/modulation.jl)
# ---------------------------------------------------------------------------
def test_modulated_blocks(oracle):
    """Block structure of the coupled sideband matrix (modulation.jl:79-101):
    diagonal blocks differ only by (ωₙ² - ω₀²)Tϵ under a shared PML, block
    (n, n+1) is ½ωₙ² conj(TΔϵ), block (n+1, n) is ½ωₙ₊₁² TΔϵ."""
    g = small_grid(oracle, N=(6, 5), npml=(1, 1), d=(0.1, 0.2))
    rng = np.random.default_rng(1)
    eps = rng.uniform(1, 4, g.N) + 0j
    deps = rng.standard_normal(g.N) + 1j * rng.standard_normal(g.N)
    w, W = 2.0e15, 3.0e14
    A, wn, _ = oracle.modulated_system(g, eps, deps, w, W, 1, True, 4.0, -18.0)
    A = A.toarray()
    N = 30
    eps0 = oracle.EPS0 * g.L0
    blk = lambda i, j: A[i * N:(i + 1) * N, j * N:(j + 1) * N]
    Te = np.diag(eps0 * oracle.vec(eps))
    TDe = np.diag(eps0 * oracle.vec(deps))
    assert np.allclose(wn, [w - W, w, w + W])
    for n in range(3):
        assert np.allclose(blk(n, n) - wn[n] ** 2 * Te, blk(1, 1) - wn[1] ** 2 * Te, rtol=0, atol=1e-9 * abs(A).max())
    for n in range(2):
        assert np.allclose(blk(n, n + 1), 0.5 * wn[n] ** 2 * TDe.conj(), rtol=1e-14, atol=0)
        assert np.allclose(blk(n + 1, n), 0.5 * wn[n + 1] ** 2 * TDe, rtol=1e-14, atol=0)
    assert not blk(0, 2).any() and not blk(2, 0).any()


def test_sideband_operator_entries(oracle):
    """Row of Sxb δxb μ₀⁻¹ Sxf δxf (modulation.jl:82): x-neighbour entries
    sxb_i sxf_i/(dx²μ₀) (i+1) and sxb_i sxf_{i-1}/(dx²μ₀) (i-1), diagonal minus
    their sum, with 1/s factors of S_create."""
    g = small_grid(oracle, N=(6, 5), npml=(2, 1), d=(0.1, 0.2))
    w = 2.0e15
    eps = np.ones(g.N) + 0j
    A, _, _ = oracle.modulated_system(g, eps, np.zeros(g.N), w, 0.0, 0, True, 4.0, -18.0)
    A = A.tocsr()
    _, mu0, _ = oracle.normalize_parameters(g.L0)
    eps0 = oracle.EPS0 * g.L0
    sxf = 1 / oracle.create_sfactor(oracle.X, oracle.FORWARD, g, w, 4.0, -18.0)
    sxb = 1 / oracle.create_sfactor(oracle.X, oracle.BACKWARD, g, w, 4.0, -18.0)
    syf = 1 / oracle.create_sfactor(oracle.Y, oracle.FORWARD, g, w, 4.0, -18.0)
    syb = 1 / oracle.create_sfactor(oracle.Y, oracle.BACKWARD, g, w, 4.0, -18.0)
    dx, dy = g.dx(), g.dy()
    Nx, Ny = g.N
    for ix, iy in [(0, 0), (2, 3), (5, 4), (1, 2)]:
        k = ix + Nx * iy
        kp, km = (ix + 1) % Nx + Nx * iy, (ix - 1) % Nx + Nx * iy
        kyp, kym = ix + Nx * ((iy + 1) % Ny), ix + Nx * ((iy - 1) % Ny)
        cxp = sxb[ix] * sxf[ix] / dx ** 2 / mu0
        cxm = sxb[ix] * sxf[ix - 1] / dx ** 2 / mu0
        cyp = syb[iy] * syf[iy] / dy ** 2 / mu0
        cym = syb[iy] * syf[iy - 1] / dy ** 2 / mu0
        assert np.isclose(A[k, kp], cxp, rtol=1e-13) and np.isclose(A[k, km], cxm, rtol=1e-13)
        assert np.isclose(A[k, kyp], cyp, rtol=1e-13) and np.isclose(A[k, kym], cym, rtol=1e-13)
        assert np.isclose(A[k, k], -(cxp + cxm + cyp + cym) + w ** 2 * eps0, rtol=1e-12)


def test_modulated_without_pml_or_modulation_is_driven(oracle):
    """Without PML the backward-outer sideband operator equals the driven TM
    operator (periodic differences commute); with Δϵ = 0 the centre sideband
    of solve(::ModulatedDevice) is then the driven field and the other
    sidebands vanish."""
    g = oracle.Grid((24, 18), (0, 0), ((0.0, 0.0), (24 * 0.08, 18 * 0.08)))
    rng = np.random.default_rng(3)
    eps = rng.uniform(1, 4, g.N) + 1j * rng.uniform(0.01, 0.1, g.N)
    src = np.zeros(g.N, complex)
    src[7, 9] = 1j
    w = 2 * np.pi * oracle.C0 / 1.55e-6
    out = oracle.solve_modulated(g, eps, np.zeros(g.N), src, w, 0.2 * w, 1, True)
    ref = oracle.solve(g, eps, src, w, oracle.TM)
    assert np.linalg.norm(out[1][0] - ref[0]) <= 1e-10 * np.linalg.norm(ref[0])
    assert np.abs(out[0][0]).max() == 0 and np.abs(out[2][0]).max() == 0


def test_modulated_plane_wave_closed_form(oracle):
    """solve(d::ModulatedDevice) (src/solver/modulation.jl:35-119) without PML, with uniform ϵᵣ and
    Δϵᵣ and a discrete plane-wave source: each sideband field is c_n·src, where c solves the
    K x K tridiagonal system of that Fourier mode:
      diagonal -k²/μ₀ + ωₙ²ϵ₀ϵᵣ, (n, n+1) = ½ωₙ²ϵ₀ conj(Δϵᵣ), (n+1, n) = ½ωₙ₊₁²ϵ₀ Δϵᵣ   (:79-101),
      right-hand side iω in the centre sideband (:67-69);
    H is the forward-difference recovery at ωₙ (:110-114), δf e^{iθj} = e^{iθj}(e^{iθ} - 1)/dh."""
    Nx, Ny, dx, dy, er, de = 20, 16, 0.05, 0.04, 2.25, 0.3 + 0.2j
    g = oracle.Grid((Nx, Ny), (0, 0), ((0.0, 0.0), (Nx * dx, Ny * dy)))
    eps0, mu0, _ = oracle.normalize_parameters(g.L0)
    w = 2 * np.pi * oracle.C0 / 1.55e-6
    Om, s = 0.05 * w, 2
    K = 2 * s + 1
    I, J = np.meshgrid(np.arange(Nx), np.arange(Ny), indexing="ij")
    tx, ty = 2 * np.pi * 3 / Nx, 2 * np.pi * 2 / Ny
    src = np.exp(1j * (tx * I + ty * J))
    k2 = (2 / dx * np.sin(tx / 2)) ** 2 + (2 / dy * np.sin(ty / 2)) ** 2
    wn = w + Om * np.arange(-s, s + 1)
    M = np.diag(-k2 / mu0 + wn ** 2 * eps0 * er).astype(complex)
    for j in range(K - 1):
        M[j, j + 1] = 0.5 * wn[j] ** 2 * eps0 * np.conj(de)
        M[j + 1, j] = 0.5 * wn[j + 1] ** 2 * eps0 * de
    rhs = np.zeros(K, dtype=complex)
    rhs[s] = 1j * w
    c = np.linalg.solve(M, rhs)
    out = oracle.solve_modulated(g, np.full((Nx, Ny), er, dtype=complex), np.full((Nx, Ny), de), src, w, Om, s)
    fx, fy = (np.exp(1j * tx) - 1) / dx, (np.exp(1j * ty) - 1) / dy
    got = [np.stack(f) for f in out]
    ref = [np.stack((c[j] * src, -c[j] * src * fy / (1j * wn[j] * mu0), c[j] * src * fx / (1j * wn[j] * mu0)))
           for j in range(K)]
    for comp in range(3):
        a = np.stack([x[comp] for x in got])
        b = np.stack([x[comp] for x in ref])
        assert np.linalg.norm(a - b) <= 1e-11 * np.linalg.norm(b)


def test_modulated_golden_regression(oracle):
    g = np.load(os.path.join(GOLD, "tm_modulated_125x50.npz"))
    Nx, Ny = int(g["Nx"]), int(g["Ny"])
    grid = oracle.Grid((Nx, Ny), tuple(g["npml"]), ((0.0, 0.0), (Nx * float(g["dx"]), Ny * float(g["dy"]))))
    out = oracle.solve_modulated(grid, g["eps"], g["deps"], g["src"], float(g["omega"]), float(g["Omega"]),
                                 int(g["nsidebands"]), bool(g["sharedpml"]), float(g["pml_m"]), float(g["pml_lnR"]))
    ez = np.stack([o[0] for o in out])
    assert np.linalg.norm(ez - g["ez"]) <= 1e-12 * np.linalg.norm(g["ez"])


@pytest.mark.parametrize("pol", [1, 2])
def test_eigenfrequency_discrete_dispersion(oracle, pol):
    """eigenfrequency (src/solver/eigen.jl:69-115) on a periodic grid without PML and with
    uniform ϵᵣ: the 5-point operator's eigenvalues are known in closed form,
    k² = (2/dx·sin(πm/Nx))² + (2/dy·sin(πn/Ny))², ω = c₀k/(L₀√ϵᵣ), for TM (ω = √(-λ/μ₀ϵ₀))
    and TE (ω = √(-λ/μ₀)) alike.  The four modes nearest ω₀ must be on that set."""
    Nx, Ny, dh, er = 24, 18, 0.05, 2.25
    g = oracle.Grid((Nx, Ny), (0, 0), ((0.0, 0.0), (Nx * dh, Ny * dh)))
    _, _, c0n = oracle.normalize_parameters(g.L0)
    m, n = np.arange(Nx)[:, None], np.arange(Ny)[None, :]
    k2 = (2 / dh * np.sin(np.pi * m / Nx)) ** 2 + (2 / dh * np.sin(np.pi * n / Ny)) ** 2
    w_an = np.sort(np.sqrt(k2.ravel()) * c0n / np.sqrt(er))
    w, _, _ = oracle.eigenfrequency(g, np.full((Nx, Ny), er, dtype=complex), 1.02 * w_an[5], pol, 4)
    for x in w:
        assert np.min(np.abs(w_an - x)) <= 1e-12 * abs(x)
    assert np.allclose(w, w_an[5], rtol=1e-12)   # the (±m, ±n) mode nearest ω₀ is four-fold


# ---------------------------------------------------------------------------
# mode sources (src/device.jl:112-149, src/solver/eigen.jl:6-29)
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("pol", [1, 2])
def test_eigenmode_arpack_matches_dense(oracle, pol):
    """The ARPACK shift-invert restatement of eigenmode returns the eigenpair
    of the dense eigendecomposition nearest the shift."""
    rng = np.random.default_rng(4 + pol)
    e = rng.uniform(1, 12, 41) + 1j * rng.uniform(0, 0.2, 41)
    w = 2 * np.pi * oracle.C0 / 1.55e-6
    b1, v1 = oracle.eigenmode_1d(e, 0.03, w, pol, 2.5)
    b2, v2 = oracle.eigenmode_1d(e, 0.03, w, pol, 2.5, dense=True)
    assert abs(b1[0] - b2[0]) <= 1e-12 * abs(b2[0])
    a1, a2 = np.abs(v1[:, 0]), np.abs(v2[:, 0])
    assert np.linalg.norm(a1 / np.linalg.norm(a1) - a2 / np.linalg.norm(a2)) <= 1e-9


def test_eigenmode_slab_dispersion(oracle):
    """Known answer: the fundamental TM (Ez) mode of a symmetric slab of index
    n1 = 3.5, width d = 0.22 µm in n2 = 1 satisfies κ tan(κd/2) = γ with
    κ² = k₀²n1² − β², γ² = β² − k₀²n2²; the second-order finite differences
    reach it to O(dh²)."""
    from scipy.optimize import brentq
    lam, d, n1, n2, dh = 1.55, 0.22, 3.5, 1.0, 0.002
    k0 = 2 * np.pi / lam
    f = lambda b: np.sqrt(k0 ** 2 * n1 ** 2 - b ** 2) * np.tan(np.sqrt(k0 ** 2 * n1 ** 2 - b ** 2) * d / 2) \
        - np.sqrt(b ** 2 - k0 ** 2 * n2 ** 2)
    lo = max(k0 * n2, np.sqrt(max(k0 ** 2 * n1 ** 2 - (np.pi / d) ** 2, 0))) + 1e-9
    b_exact = brentq(f, lo, k0 * n1 - 1e-9)
    y = (np.arange(1000) + 0.5) * dh - 1.0
    e = np.where(np.abs(y) <= d / 2, n1 ** 2, n2 ** 2).astype(complex)
    w = 2 * np.pi * oracle.C0 / (lam * 1e-6)
    b, _ = oracle.eigenmode_1d(e, dh, w, 1, 3.0)
    assert abs(b[0].real - b_exact) <= 2e-3 * b_exact and abs(b[0].imag) <= 1e-9 * b_exact


def test_setup_mode_adds_normalized_abs(oracle):
    """setup_mode! adds normalize(abs.(v)) on the slice and nothing elsewhere."""
    g = oracle.Grid((30, 40), (4, 4), ((0.0, 0.0), (30 * 0.05, 40 * 0.05)))
    e = np.ones(g.N, complex)
    e[:, 17:23] = 12.25
    src = np.zeros(g.N, complex)
    w = 2 * np.pi * oracle.C0 / 1.55e-6
    oracle.setup_mode(src, g, e, 1, w, 3.0, 6, 20, oracle.X, 0.8)
    indx, indy, _ = oracle.mode_slice(g, 6, 20, oracle.X, 0.8)
    assert len(indy) == 17 and np.isclose(np.linalg.norm(src), 1.0)
    mask = np.zeros(g.N, bool)
    mask[indx, indy] = True
    assert not src[~mask].any() and np.all(src[mask].real > 0)


# ---------------------------------------------------------------------------
# Poynting flux (src/flux.jl)
# ---------------------------------------------------------------------------
def test_poynting_energy_balance(oracle):
    """Known answer: for a lossless medium with a point source, the flux
    through a closed box around the source equals the power the source
    delivers, P = -½Re(∫ E·J*)·dA (J = src, E = Ez); the discrete identity
    holds to discretisation accuracy (a few percent at 20 cells/λ)."""
    g = oracle.Grid((120, 120), (20, 20), ((0.0, 0.0), (120 * 0.05, 120 * 0.05)))
    eps = np.ones(g.N, complex)
    src = np.zeros(g.N, complex)
    src[60, 60] = 1.0
    w = 2 * np.pi * oracle.C0 / 1.55e-6
    ez, hx, hy = oracle.solve(g, eps, src, w, oracle.TM, 4.0, np.log(1e-8))
    Sx, Sy = oracle.poynting(ez, hx, hy, oracle.TM)
    lo, hi = 40, 80
    dx, dy = g.dx(), g.dy()
    out = (Sx[hi, lo:hi].sum() - Sx[lo, lo:hi].sum()) * dy + (Sy[lo:hi, hi].sum() - Sy[lo:hi, lo].sum()) * dx
    delivered = abs(0.5 * np.real(np.sum(ez * np.conj(src)))) * dx * dy
    assert out > 0 and abs(out - delivered) <= 0.1 * delivered, (out, delivered)


def test_flux_integral_matches_poynting_columns(oracle):
    """flux_surface_integral (x̂) sums -½Re(Ez̄ Hy*)·dy over the rows with Ez
    averaged over columns x and x+1 (poynting averages x and x-1).  Checked on
    a random field by direct evaluation; the ŷ normal raises."""
    rng = np.random.default_rng(2)
    g = oracle.Grid((16, 12), (2, 2), ((0.0, -0.3), (16 * 0.05, 12 * 0.05 - 0.3)))
    f = [rng.standard_normal(g.N) + 1j * rng.standard_normal(g.N) for _ in range(3)]
    x, rows = oracle.flux_line_indices(g, (0.41, 0.0), 0.1)
    assert abs(g.xc()[x] - 0.41) <= g.dx() / 2 and np.all(np.abs(g.yc()[rows]) <= 0.1 + 1e-12) and len(rows) == 4
    v = oracle.flux_surface_integral(g, f[0], f[2], oracle.TM, (0.41, 0.0), 0.1, oracle.X)
    ref = sum(-0.5 * np.real(0.5 * (f[0][x, j] + f[0][x + 1, j]) * np.conj(f[2][x, j])) for j in rows) * g.dy()
    assert np.isclose(v, ref, rtol=1e-13)
    with pytest.raises(NotImplementedError):
        oracle.flux_surface_integral(g, f[0], f[2], oracle.TM, (0.41, 0.0), 0.1, oracle.Y)


@pytest.mark.parametrize("method", ["born", "newton"])
def test_chi3_plane_wave_closed_form(oracle, method):
    """solve(d::χ3Device, method) (src/solver/nonlinear.jl:36-129) without PML, with uniform ϵᵣ
    and χ and a unit-modulus plane-wave source: |e|² stays uniform, so the field is a·src with
    the scalar fixed point (L + c|a|²)a = iω, L = -k²/μ₀ + ω²ϵ₀ϵᵣ, c = ω²ϵ₀·3χ/L₀ (:71).
    χ is set so that c|a|² ≈ 0.01|L|: the amplitude moves 1 % from the linear a₀ = iω/L, which
    both iterations must reproduce (Born on this grid diverges at 0.1: other Fourier modes lie
    near resonance, and the Born map amplifies them; Newton does not)."""
    Nx, Ny, dx, dy, er = 20, 16, 0.05, 0.04, 2.25
    g = oracle.Grid((Nx, Ny), (0, 0), ((0.0, 0.0), (Nx * dx, Ny * dy)))
    eps0, mu0, _ = oracle.normalize_parameters(g.L0)
    w = 2 * np.pi * oracle.C0 / 1.55e-6
    I, J = np.meshgrid(np.arange(Nx), np.arange(Ny), indexing="ij")
    tx, ty = 2 * np.pi * 3 / Nx, 2 * np.pi * 2 / Ny
    src = np.exp(1j * (tx * I + ty * J))
    L = -((2 / dx * np.sin(tx / 2)) ** 2 + (2 / dy * np.sin(ty / 2)) ** 2) / mu0 + w ** 2 * eps0 * er
    a0 = 1j * w / L
    chi = 0.01 * abs(L) / (abs(a0) ** 2 * w ** 2 * eps0 * 3 / g.L0)
    c = w ** 2 * eps0 * 3 * chi / g.L0
    a = a0
    for _ in range(200):
        a = 1j * w / (L + c * abs(a) ** 2)
    assert abs(a - a0) > 5e-3 * abs(a0)
    (ez, _, _), err = oracle.solve_chi3(g, np.full((Nx, Ny), er, dtype=complex), np.full((Nx, Ny), chi), src, w,
                                        method)
    assert err[-1] <= 1e-12
    assert np.abs(ez - a * src).max() <= 1e-10 * abs(a)


@pytest.mark.parametrize("pol", [1, 2])
def test_poynting_plane_wave_closed_form(oracle, pol):
    """poynting (src/flux.jl:15-29) of a discrete plane wave f1 = a·e^{i(θx·i + θy·j)} with
    f2 = α·f1, f3 = β·f1: grid_average over the previous cell multiplies f1 by (1 + e^{-iθ})/2, so
      TM: Sx = -½|a|²Re(½(1 + e^{-iθx})·conj(β)),  Sy = ½|a|²Re(½(1 + e^{-iθy})·conj(α))
      TE: Sx = ½|a|²Re(β·conj(½(1 + e^{-iθx}))),  Sy = -½|a|²Re(α·conj(½(1 + e^{-iθy})))
    uniform over the grid (the average wraps periodically, grid.jl:157-162)."""
    Nx, Ny = 12, 10
    I, J = np.meshgrid(np.arange(Nx), np.arange(Ny), indexing="ij")
    tx, ty = 2 * np.pi * 2 / Nx, 2 * np.pi * 3 / Ny
    a, al, be = 0.7 - 1.1j, 0.3 + 2.0j, -1.4 + 0.6j
    f1 = a * np.exp(1j * (tx * I + ty * J))
    Sx, Sy = oracle.poynting(f1, al * f1, be * f1, pol)
    hx, hy = (1 + np.exp(-1j * tx)) / 2, (1 + np.exp(-1j * ty)) / 2
    a2 = abs(a) ** 2
    if pol == oracle.TM:
        want = (-0.5 * a2 * (hx * np.conj(be)).real, 0.5 * a2 * (hy * np.conj(al)).real)
    else:
        want = (0.5 * a2 * (be * np.conj(hx)).real, -0.5 * a2 * (al * np.conj(hy)).real)
    assert np.allclose(Sx, want[0], rtol=1e-13, atol=0) and np.allclose(Sy, want[1], rtol=1e-13, atol=0)
