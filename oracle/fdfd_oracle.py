"""FP64 CPU oracle for the FDFD solve path.  TEST INFRASTRUCTURE ONLY.

This module restates, in numpy/scipy, the arithmetic of fancompute/FDFD.jl on
the path that the GPU library replaces: unit normalisation, the Yee-grid
difference operators, the SC-PML stretch factors, the TM/TE driven system and
field recovery, and the TM/TE eigenfrequency problem.  Each function cites the
reference file and line range it follows (paths relative to the FDFD.jl
project root).

Only the tests, ``__graft_entry__.smoke()`` and the CPU baseline leg of
``bench.py`` may import this file, and only as the checker.  The product path
(the CUDA library and its host wrapper) never imports or calls it.

Parity status: the reference is Julia and cannot run in this environment, and
its own test suite holds no golden vectors (``test/runtests.jl:7-63`` only
checks that two FP64 direct solvers agree to sqrt(eps)).  Parity of this
restatement with the reference is therefore UNPINNED at the level of exact
field values.  It is cross-checked instead against (a) hand-derived operator
entries on tiny grids, (b) an independent dense FP64 solve, mirroring the
reference's own solver-agreement test, (c) the analytic 2-D free-space
Green's function for the reference's dipole test problem, and (d) closed-form
discrete solutions on periodic grids without PML (plane-wave driven TM/TE
fields, the sideband system per Fourier mode, the χ³ scalar fixed point, and
the eigenfrequencies of a uniform grid).

Third-party arithmetic that the reference delegates (not vendored in the
reference tree, and unpinned there: ``Project.toml`` has no [compat] section
and there is no Manifest):
  * SparseArrays ``lu(A)\\b`` -> SuiteSparse UMFPACK (``src/solver/solver.jl:35``),
    MKL Pardiso ``COMPLEX_NONSYM`` (``solver.jl:19-32``): restated with
    ``scipy.sparse.linalg.splu`` (SuperLU), another FP64 sparse direct LU.
  * Arpack.jl ``eigs(A, nev, sigma, which)`` (``src/solver/eigen.jl:86,104``):
    restated with ``scipy.sparse.linalg.eigs`` (ARPACK-ng shift-invert).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

# --- constants: src/types.jl:6-9 -------------------------------------------
EPS0 = 8.85418782e-12
MU0 = 1.25663706e-6
C0 = math.sqrt(1 / EPS0 / MU0)
ETA0 = math.sqrt(MU0 / EPS0)
DEFAULT_L0 = 1e-6  # src/grid.jl:5 (DEFAULT_L₀)

TM, TE = 1, 2  # src/types.jl:20 (@enum Polarization TM=1 TE=2)
X, Y = 1, 2    # src/types.jl:18 (@enum Direction x̂=1 ŷ=2)
FORWARD, BACKWARD = 1, 2  # src/types.jl:19


def normalize_parameters(L0: float = DEFAULT_L0):
    """(ϵ₀L₀, μ₀L₀, c₀/L₀): src/device.jl:40."""
    return EPS0 * L0, MU0 * L0, C0 / L0


@dataclass
class Grid:
    """2-D grid: src/grid.jl:7-13 (fields), :26-33 (constructor)."""
    N: tuple       # (Nx, Ny)
    Npml: tuple    # (Npx, Npy)
    bounds: tuple  # ((x1, y1), (x2, y2))
    L0: float = DEFAULT_L0

    @classmethod
    def from_ranges(cls, dh, Npml, xrange, yrange, L0=DEFAULT_L0):
        """src/grid.jl:26-33: N = round(L/dh) (round-half-even, as Julia)."""
        L = (float(xrange[1] - xrange[0]), float(yrange[1] - yrange[0]))
        N = (int(round(L[0] / dh)), int(round(L[1] / dh)))
        return cls(N, (int(Npml[0]), int(Npml[1])),
                   ((float(xrange[0]), float(yrange[0])),
                    (float(xrange[1]), float(yrange[1]))), L0)

    @property
    def L(self):
        return (self.bounds[1][0] - self.bounds[0][0],
                self.bounds[1][1] - self.bounds[0][1])

    def dx(self):  # src/grid.jl:68-70
        return (self.bounds[1][0] - self.bounds[0][0]) / self.N[0]

    def dy(self):  # src/grid.jl:72-74
        return (self.bounds[1][1] - self.bounds[0][1]) / self.N[1]

    def dh(self, w):  # src/grid.jl:63-66
        return self.dx() if w == X else self.dy()

    def xc(self):  # src/grid.jl:76-78
        return self.bounds[0][0] + self.dx() * (np.arange(self.N[0]) + 0.5)

    def yc(self):  # src/grid.jl:80-82
        return self.bounds[0][1] + self.dy() * (np.arange(self.N[1]) + 0.5)

    def x2ind(self, x):
        """src/grid.jl:112-117, returned 0-based."""
        ind = int(round((x - self.bounds[0][0]) / self.L[0] * self.N[0]) + 1)
        ind = min(max(ind, 1), self.N[0])
        return ind - 1

    def y2ind(self, y):
        """src/grid.jl:120-125, returned 0-based."""
        ind = int(round((y - self.bounds[0][1]) / self.L[1] * self.N[1]) + 1)
        ind = min(max(ind, 1), self.N[1])
        return ind - 1


def vec(a: np.ndarray) -> np.ndarray:
    """Julia ``a[:]``: column-major flatten, x fastest (driven.jl:21)."""
    return np.asarray(a).reshape(-1, order="F")


def unvec(v: np.ndarray, shape) -> np.ndarray:
    return np.asarray(v).reshape(shape, order="F")


def delta(w: int, s: int, g: Grid) -> sp.csr_matrix:
    """Periodic first differences: src/grid.jl:128-154.

    x: kron(I_Ny, δx), y: kron(δy, I_Nx); forward has +1 on the super-diagonal
    and at (N,1); backward has -1 on the sub-diagonal and at (1,N).
    """
    Nx, Ny = g.N

    def d1(N, h, forward):
        if forward:  # spdiagm(1 => ones(N-1), 0 => -ones(N), -N+1 => [1])
            m = sp.diags([np.ones(N - 1), -np.ones(N)], [1, 0], shape=(N, N), format="lil")
            m[N - 1, 0] += 1.0
        else:        # spdiagm(-1 => -ones(N-1), 0 => ones(N), N-1 => [-1])
            m = sp.diags([-np.ones(N - 1), np.ones(N)], [-1, 0], shape=(N, N), format="lil")
            m[0, N - 1] += -1.0
        return (1 / h) * m.tocsr()

    if w == X:
        return sp.kron(sp.identity(Ny, format="csr"), d1(Nx, g.dx(), s == FORWARD), format="csr")
    return sp.kron(d1(Ny, g.dy(), s == FORWARD), sp.identity(Nx, format="csr"), format="csr")


def grid_average(center: np.ndarray, w: int) -> np.ndarray:
    """src/grid.jl:157-162: (a + circshift(a, 1 along w))/2, periodic."""
    if center.ndim == 1:
        return (center + np.roll(center, 1)) / 2
    if w == X:
        return (center + np.roll(center, 1, axis=0)) / 2
    return (center + np.roll(center, 1, axis=1)) / 2


def create_sfactor(w: int, s: int, g: Grid, omega: float, m: float = 3.5,
                   lnR: float = -12.0) -> np.ndarray:
    """1-D complex stretch factors s(l) = 1 - iσ(l)/(ωϵ₀): src/pml.jl:1-31."""
    eps0, _, _ = normalize_parameters(g.L0)
    dw = g.dh(w)
    Nw_pml = g.Npml[w - 1]
    Nw = g.N[w - 1]
    Tw = Nw_pml * dw
    out = np.ones(Nw, dtype=np.complex128)
    if Nw_pml == 0:
        return out
    sigmax = -(m + 1) * lnR / (2 * ETA0 * Tw)

    def S(l):
        return 1 - 1j * (sigmax * (l / Tw) ** m) / (omega * eps0)

    for i in range(1, Nw + 1):
        if s == FORWARD:
            if i <= Nw_pml:
                out[i - 1] = S(dw * (Nw_pml - i + 0.5))
            elif i > Nw - Nw_pml:
                out[i - 1] = S(dw * (i - (Nw - Nw_pml) - 0.5))
        else:
            if i <= Nw_pml:
                out[i - 1] = S(dw * (Nw_pml - i + 1))
            elif i > Nw - Nw_pml:
                out[i - 1] = S(dw * (i - (Nw - Nw_pml) - 1))
    return out


def S_create(g: Grid, omega: float, m: float = 3.5, lnR: float = -12.0):
    """Diagonal 1/s matrices (Sx_f, Sx_b, Sy_f, Sy_b): src/pml.jl:33-63.

    The reference does not forward m/lnR (pml.jl:35-38); here they are
    explicit so that the same restatement serves both the defaults and the
    m=4, R=1e-8 PML used by the benchmark problems.
    """
    Nx, Ny = g.N
    sxf = create_sfactor(X, FORWARD, g, omega, m, lnR)
    sxb = create_sfactor(X, BACKWARD, g, omega, m, lnR)
    syf = create_sfactor(Y, FORWARD, g, omega, m, lnR)
    syb = create_sfactor(Y, BACKWARD, g, omega, m, lnR)
    Sxf = np.broadcast_to((sxf ** -1)[:, None], (Nx, Ny))
    Sxb = np.broadcast_to((sxb ** -1)[:, None], (Nx, Ny))
    Syf = np.broadcast_to((syf ** -1)[None, :], (Nx, Ny))
    Syb = np.broadcast_to((syb ** -1)[None, :], (Nx, Ny))
    return tuple(sp.diags(vec(a), 0, format="csr") for a in (Sxf, Sxb, Syf, Syb))


def stretched_deltas(g: Grid, omega: float, m=3.5, lnR=-12.0):
    """δxb, δxf, δyb, δyf with PML rows applied: src/solver/driven.jl:25-31."""
    Sxf, Sxb, Syf, Syb = S_create(g, omega, m, lnR)
    return (Sxb @ delta(X, BACKWARD, g), Sxf @ delta(X, FORWARD, g),
            Syb @ delta(Y, BACKWARD, g), Syf @ delta(Y, FORWARD, g))


def assemble(g: Grid, eps_r: np.ndarray, omega: float, pol: int, m=3.5, lnR=-12.0):
    """Driven system matrix A (CSC): src/solver/driven.jl:21-45.

    TM: A = δxf μ₀⁻¹ δxb + δyf μ₀⁻¹ δyb + ω² Tϵ               (driven.jl:35)
    TE: A = δxf Tϵxi δxb + δyf Tϵyi δyb + ω² μ₀ I              (driven.jl:45;
        the reference's ``speye`` is restated as a sparse identity)
    """
    eps0, mu0, _ = normalize_parameters(g.L0)
    eps_r = np.asarray(eps_r, dtype=np.complex128)
    dxb, dxf, dyb, dyf = stretched_deltas(g, omega, m, lnR)
    if pol == TM:
        Te = sp.diags(eps0 * vec(eps_r), 0)
        A = dxf * mu0 ** -1 @ dxb + dyf * mu0 ** -1 @ dyb + omega ** 2 * Te
    else:
        Texi = sp.diags(1 / vec(grid_average(eps0 * eps_r, X)), 0)
        Teyi = sp.diags(1 / vec(grid_average(eps0 * eps_r, Y)), 0)
        n = g.N[0] * g.N[1]
        A = dxf @ Texi @ dxb + dyf @ Teyi @ dyb + omega ** 2 * mu0 * sp.identity(n)
    return A.tocsc()


def dolinearsolve(A: sp.spmatrix, b: np.ndarray) -> np.ndarray:
    """``lu(A)\\b``: src/solver/solver.jl:35 (SuperLU stands in for UMFPACK)."""
    lu = spla.splu(sp.csc_matrix(A))
    return lu.solve(np.asarray(b, dtype=np.complex128))


def solve(g: Grid, eps_r, src, omega: float, pol: int = TM, m=3.5, lnR=-12.0,
          return_system=False):
    """Driven solve for one frequency: src/solver/driven.jl:4-59.

    ``src`` is the current array J (Nx x Ny); the right-hand side is
    b = iω·src (driven.jl:36,46).  Returns (f1, f2, f3) as Nx x Ny arrays:
    TM -> (Ez, Hx, Hy) with backward-difference H recovery (driven.jl:40-41);
    TE -> (Hz, Ex, Ey) (driven.jl:50-51).
    """
    eps0, mu0, _ = normalize_parameters(g.L0)
    eps_r = np.asarray(eps_r, dtype=np.complex128)
    A = assemble(g, eps_r, omega, pol, m, lnR)
    b = 1j * omega * vec(np.asarray(src, dtype=np.complex128))
    x = dolinearsolve(A, b)
    f = recover_driven(g, eps_r, omega, x, pol, m, lnR)
    if return_system:
        return f, A, b
    return f


def recover_driven(g: Grid, eps_r, omega, x, pol, m=3.5, lnR=-12.0):
    """H (TM) or E (TE) recovery of the driven solve: src/solver/driven.jl:40-51."""
    eps0, mu0, _ = normalize_parameters(g.L0)
    dxb, dxf, dyb, dyf = stretched_deltas(g, omega, m, lnR)
    shp = g.N
    if pol == TM:
        hx = -1 / 1j / omega / mu0 * (dyb @ x)
        hy = 1 / 1j / omega / mu0 * (dxb @ x)
        return unvec(x, shp), unvec(hx, shp), unvec(hy, shp)
    eps_r = np.asarray(eps_r, dtype=np.complex128)
    Texi = sp.diags(1 / vec(grid_average(eps0 * eps_r, X)), 0)
    Teyi = sp.diags(1 / vec(grid_average(eps0 * eps_r, Y)), 0)
    ex = 1 / 1j / omega * (Teyi @ (dyb @ x))
    ey = 1 / 1j / omega * (Texi @ (-(dxb @ x)))
    return unvec(x, shp), unvec(ex, shp), unvec(ey, shp)


def eigen_operator(g: Grid, eps_r, omega0: float, pol: int, m=3.5, lnR=-12.0):
    """Eigen-operator A and shift σ: src/solver/eigen.jl:69-104.

    TM: A = Tϵᵣ⁻¹ δxf δxb + Tϵᵣ⁻¹ δyf δyb, σ = -ω₀² μ₀ ϵ₀   (eigen.jl:83-86)
    TE: A = δxf Tϵx⁻¹ δxb + δyf Tϵy⁻¹ δyb, σ = -ω₀² μ₀      (eigen.jl:100-104)
    """
    eps0, mu0, _ = normalize_parameters(g.L0)
    eps_r = np.asarray(eps_r, dtype=np.complex128)
    dxb, dxf, dyb, dyf = stretched_deltas(g, omega0, m, lnR)
    if pol == TM:
        Tri = sp.diags(1 / vec(eps_r), 0)
        A = Tri @ dxf @ dxb + Tri @ dyf @ dyb
        sigma = -omega0 ** 2 * mu0 * eps0
    else:
        Txi = sp.diags(1 / vec(grid_average(eps0 * eps_r, X)), 0)
        Tyi = sp.diags(1 / vec(grid_average(eps0 * eps_r, Y)), 0)
        A = dxf @ Txi @ dxb + dyf @ Tyi @ dyb
        sigma = -omega0 ** 2 * mu0
    return A.tocsc(), sigma


def eigenfrequency(g: Grid, eps_r, omega0: float, pol: int, nev: int, which="LM",
                   m=3.5, lnR=-12.0, tol=0.0, v0=None):
    """Shift-invert eigenfrequencies and fields: src/solver/eigen.jl:69-115.

    Returns (omega, fields) with omega = sqrt(-λ/(μ₀ϵ₀)) for TM (eigen.jl:87)
    or sqrt(-λ/μ₀) for TE (eigen.jl:105); fields use FORWARD differences for
    TM H recovery (eigen.jl:90-91) and Tϵx⁻¹/Tϵy⁻¹ for TE (eigen.jl:108-109).
    """
    eps0, mu0, _ = normalize_parameters(g.L0)
    eps_r = np.asarray(eps_r, dtype=np.complex128)
    A, sigma = eigen_operator(g, eps_r, omega0, pol, m, lnR)
    lam, vecs = spla.eigs(A, k=nev, sigma=sigma, which=which, tol=tol, v0=v0)
    dxb, dxf, dyb, dyf = stretched_deltas(g, omega0, m, lnR)
    shp = g.N
    if pol == TM:
        w = np.sqrt(-lam / mu0 / eps0)
        fields = []
        for i in range(nev):
            ez = vecs[:, i]
            hx = -1 / 1j / w[i] / mu0 * (dyf @ ez)
            hy = 1 / 1j / w[i] / mu0 * (dxf @ ez)
            fields.append((unvec(ez, shp), unvec(hx, shp), unvec(hy, shp)))
        return w, fields, lam
    w = np.sqrt(-lam / mu0)
    Txi = sp.diags(1 / vec(grid_average(eps0 * eps_r, X)), 0)
    Tyi = sp.diags(1 / vec(grid_average(eps0 * eps_r, Y)), 0)
    fields = []
    for i in range(nev):
        hz = vecs[:, i]
        ex = 1 / 1j / w[i] * (Txi @ (dyb @ hz))
        ey = 1 / 1j / w[i] * (Tyi @ (-(dxb @ hz)))
        fields.append((unvec(hz, shp), unvec(ex, shp), unvec(ey, shp)))
    return w, fields, lam


# --- adjoint (no counterpart in the reference: it has no gradient code) ------

def adjoint_gradient(g: Grid, eps_r, src, omega: float, mvec: np.ndarray,
                     m=3.5, lnR=-12.0):
    """FP64 adjoint gradient of J = |mᵀE|² with respect to real ϵᵣ (TM).

    E = A⁻¹ b with A from ``assemble`` and b = iω·src.  Since
    ∂A/∂ϵᵣ_k = ω²ϵ₀ e_k e_kᵀ, dJ/dϵᵣ_k = 2·Re(conj(mᵀE)·mᵀ ∂E/∂ϵᵣ_k) and
    ∂E/∂ϵᵣ_k = -A⁻¹(ω²ϵ₀ E_k e_k), so with λ = A⁻ᵀ m:
        dJ/dϵᵣ_k = -2·Re(conj(mᵀE) · ω²ϵ₀ · λ_k · E_k).
    Returns (J, grad (Nx x Ny), E (Nx x Ny)).
    """
    eps0, _, _ = normalize_parameters(g.L0)
    A = assemble(g, eps_r, omega, TM, m, lnR)
    b = 1j * omega * vec(np.asarray(src, dtype=np.complex128))
    lu = spla.splu(A)
    E = lu.solve(b)
    mv = vec(mvec).astype(np.complex128)
    s = mv @ E
    J = abs(s) ** 2
    lam = lu.solve(mv, trans="T")
    grad = -2.0 * np.real(np.conj(s) * omega ** 2 * eps0 * lam * E)
    return J, unvec(grad, g.N), unvec(E, g.N)


def objective(g: Grid, eps_r, src, omega, mvec, m=3.5, lnR=-12.0):
    """J = |mᵀE|² for the finite-difference check of ``adjoint_gradient``."""
    A = assemble(g, eps_r, omega, TM, m, lnR)
    b = 1j * omega * vec(np.asarray(src, dtype=np.complex128))
    E = spla.splu(A).solve(b)
    return abs(vec(mvec).astype(np.complex128) @ E) ** 2


# --- mode sources: src/device.jl:112-149, src/solver/eigen.jl:6-29 ----------

def eigenmode_1d(eps_slice, dh: float, omega: float, pol: int, neff, nev: int = 1, L0: float = DEFAULT_L0,
                 dense=False):
    """eigenmode(d::AbstractDevice{1}, pol, neff, nev): src/solver/eigen.jl:6-29.

    1-D periodic grid of len(eps_slice) cells of size dh, no PML (the
    ``Grid(N, xrange)`` constructor, grid.jl:53-59).  TM: A = ω²μ₀Tϵ + δxf δxb;
    TE: A = ω²μ₀Tϵ + Tϵ δxf Tϵxinv δxb.  ARPACK's shift-invert eigs(A, nev,
    sigma=(ω n_eff/c₀)²) (scipy's ARPACK-ng here; ``dense`` picks the nearest
    eigenvalues of a dense eig instead).  Returns (β = √λ, vectors (n, nev))."""
    eps0, mu0, c0 = normalize_parameters(L0)
    e = np.asarray(eps_slice, dtype=np.complex128).ravel()
    n = e.size
    g = Grid((n, 1), (0, 0), ((0.0, 0.0), (n * dh, dh)), L0)
    Te = sp.diags(eps0 * e, 0)
    dxb, dxf = delta(X, BACKWARD, g), delta(X, FORWARD, g)
    if pol == TM:
        A = omega ** 2 * mu0 * Te + dxf @ dxb
    else:
        Txi = sp.diags(1 / (eps0 * grid_average(e, X)), 0)
        A = omega ** 2 * mu0 * Te + Te @ dxf @ Txi @ dxb
    sigma = (omega / c0 * neff) ** 2
    if dense:
        w, v = np.linalg.eig(A.toarray())
        idx = np.argsort(np.abs(w - sigma))[:nev]
        vals, vecs = w[idx], v[:, idx]
    else:
        vals, vecs = spla.eigs(A.astype(np.complex128).tocsc(), k=nev, sigma=sigma,
                               v0=np.ones(n, dtype=np.complex128))
    return np.sqrt(vals.astype(np.complex128)), vecs


def mode_slice(g: Grid, ix: int, iy: int, normal: int, width: float):
    """Slice indices of get_modes (device.jl:125-142), 0-based: srcpoints =
    round(width/dh) made odd, M = (srcpoints-1)/2 cells each side of (ix, iy)."""
    dh = g.dy() if normal == X else g.dx()
    pts = int(round(width / dh))
    if pts % 2 == 0:
        pts += 1
    M = (pts - 1) // 2
    if normal == X:
        return ix, np.arange(iy - M, iy + M + 1), dh
    return np.arange(ix - M, ix + M + 1), iy, dh


def get_modes(g: Grid, eps_r, pol: int, omega: float, neff, nmodes: int, ix: int, iy: int, normal: int,
              width: float, dense=False):
    """get_modes(d, pol, ω, neff, nmodes, pt, slicenormal, slicewidth): src/device.jl:124-149
    with (ix, iy) = coord2ind(grid, pt) - 1.  Returns (β, vectors, indx, indy)."""
    indx, indy, dh = mode_slice(g, ix, iy, normal, width)
    e = np.asarray(eps_r)[indx, indy]
    beta, vecs = eigenmode_1d(e, dh, omega, pol, neff, nmodes, g.L0, dense)
    return beta, vecs, indx, indy


def setup_mode(src, g: Grid, eps_r, pol: int, omega: float, neff, ix: int, iy: int, normal: int, width: float):
    """setup_mode!(d, pol, ω, neff, pt, srcnormal, srcwidth): src/device.jl:118-121,
    src[indx, indy] += normalize(abs.(vector[:])) (in place)."""
    _, vecs, indx, indy = get_modes(g, eps_r, pol, omega, neff, 1, ix, iy, normal, width)
    a = np.abs(vecs[:, 0])
    src[indx, indy] += a / np.linalg.norm(a)
    return src


# --- χ³ nonlinear driven solve: src/solver/nonlinear.jl --------------------------

def chi3_coeff(g: Grid, chi, omega: float):
    """coeff = ω²ϵ₀·3χ/L₀ with ϵ₀ normalised (nonlinear.jl:71)."""
    eps0, _, _ = normalize_parameters(g.L0)
    return omega ** 2 * eps0 * 3 * vec(np.asarray(chi, dtype=np.float64)) / g.L0


def born(A, b, coeff, ez, tol=1e-12, maxiterations=50):
    """_doborn (nonlinear.jl:92-106): ez ← (A + diag(coeff·|ez|²))⁻¹ b until
    ||ez_new − ez||/||ez|| ≤ tol.  The reference misplaces a parenthesis in
    the solve call (``sparse(Diagonal(...), b, CNSym)``); the evident intent,
    dolinearsolve(A + Diagonal(coeff.*ez.*conj.(ez)), b), is restated."""
    err = [1.0]
    i = 1
    while err[-1] > tol and i <= maxiterations:
        new = dolinearsolve((A + sp.diags(coeff * ez * np.conj(ez))).tocsc(), b)
        err.append(np.linalg.norm(new - ez) / np.linalg.norm(ez))
        ez = new
        i += 1
    return ez, err


def newton(A, b, coeff, ez, tol=1e-12, maxiterations=50):
    """_donewton (nonlinear.jl:108-129): Newton on the stacked unknown [ez; conj(ez)]
    with F = (A + diag(coeff|ez|²))ez − b, J = [J1 J2; conj(J2) conj(J1)],
    J1 = A + diag(2coeff|ez|²), J2 = diag(coeff ez²); err = ||δ||/||[ez; conj ez]||."""
    M = ez.size
    z = np.concatenate([ez, np.conj(ez)])
    err = [1.0]
    i = 1
    while err[-1] > tol and i <= maxiterations:
        e1 = z[:M]
        F = (A + sp.diags(coeff * e1 * np.conj(e1))) @ e1 - b
        J1 = A + sp.diags(2 * coeff * np.conj(e1) * e1)
        J2 = sp.diags(coeff * e1 * e1)
        J = sp.bmat([[J1, J2], [J2.conj(), J1.conj()]], format="csc")
        d = dolinearsolve(J, np.concatenate([F, np.conj(F)]))
        nz = np.linalg.norm(z)
        z = z - d
        err.append(np.linalg.norm(d) / nz)
        i += 1
    return z[:M], err


def solve_chi3(g: Grid, eps_r, chi, src, omega: float, method: str, m=3.5, lnR=-12.0, tol=1e-12,
               maxiterations=50):
    """solve(d::χ3Device, which_method): src/solver/nonlinear.jl:36-90 (TM): the
    linear solve, then Born (``"born"``) or Gauss-Newton (``"newton"``), then
    the driven H recovery.  Returns ((Ez, Hx, Hy), err history)."""
    A = assemble(g, eps_r, omega, TM, m, lnR)
    b = 1j * omega * vec(np.asarray(src, dtype=np.complex128))
    ez = dolinearsolve(A, b)
    coeff = chi3_coeff(g, chi, omega)
    if method == "born":
        ez, err = born(A, b, coeff, ez, tol, maxiterations)
    else:
        ez, err = newton(A, b, coeff, ez, tol, maxiterations)
    return recover_driven(g, eps_r, omega, ez, TM, m, lnR), err


# --- Poynting flux: src/flux.jl -------------------------------------------------

def poynting(f1, f2, f3, pol: int):
    """poynting(field): src/flux.jl:15-29.  TM (Ez, Hx, Hy): Sx = -½Re(avgx(Ez)·Hy*),
    Sy = ½Re(avgy(Ez)·Hx*).  TE (Hz, Ex, Ey): Sx = ½Re(Ey·avgx(Hz)*),
    Sy = -½Re(Ex·avgy(Hz)*) — the reference reads ``field.Hz_x``/``field.Hz_y``
    (flux.jl:26-27), which a FieldTE does not have; the averages computed on the
    lines before are meant."""
    ax, ay = grid_average(f1, X), grid_average(f1, Y)
    if pol == TM:
        return -0.5 * np.real(ax * np.conj(f3)), 0.5 * np.real(ay * np.conj(f2))
    return 0.5 * np.real(f3 * np.conj(ax)), -0.5 * np.real(f2 * np.conj(ay))


def flux_line_indices(g: Grid, center, width):
    """Indices of flux_surface_integral (flux.jl:39-42), 0-based: the column whose
    centre lies within dx/2 of center.x (AxisArrays ``atvalue``), and the rows
    whose centres lie in the closed interval [center.y - width, center.y + width]."""
    xc, yc = g.xc(), g.yc()
    hit = np.nonzero(np.abs(xc - center[0]) <= g.dx() / 2)[0]
    if hit.size == 0:
        raise ValueError("no grid column at center.x")
    rows = np.nonzero((yc >= center[1] - width) & (yc <= center[1] + width))[0]
    return int(hit[0]), rows


def flux_surface_integral(g: Grid, f1, f3, pol: int, center, width, normal: int):
    """flux_surface_integral(field, center, width, normal): src/flux.jl:37-66.
    x̂ normal: Σ -½Re(½(f1[x]+f1[x+1])·f3[x]*)·dy over the rows, f1/f3 = Ez/Hy
    (TM) or Hz/Ey (TE: the reference names an undefined ``pt`` and reads :Hy,
    flux.jl:49,54; the column of ``center`` and :Ey are meant; its sign is kept).
    ŷ normal raises, as the reference."""
    if normal == Y:
        raise NotImplementedError("ŷ normal %s calculation not yet implemented" % ("TM" if pol == TM else "TE"))
    x, rows = flux_line_indices(g, center, width)
    av = 0.5 * (f1[x, rows] + f1[x + 1, rows])
    if pol == TM:
        return float(np.sum(-0.5 * np.real(av * np.conj(f3[x, rows]))) * g.dy())
    return float(np.sum(-0.5 * np.real(f3[x, rows] * np.conj(av))) * g.dy())


# --- multi-frequency (modulated) driven solve: src/solver/modulation.jl ------

def modulated_system(g: Grid, eps_r, deps_r, omega: float, Omega: float, nsidebands: int,
                     sharedpml=True, m=3.5, lnR=-12.0):
    """Coupled sideband system of ``solve(d::ModulatedDevice)``:
    src/solver/modulation.jl:35-119 (TM only, as the reference).

    Frequencies ωₙ = ω + nΩ, n = -s..s (:41,49).  Per sideband
    Aₙ = Sxb δxb μ₀⁻¹ Sxf δxf + Syb δyb μ₀⁻¹ Syf δyf + ωₙ² Tϵ with the PML at ω
    (shared, :79-85) or at ωₙ (:86-91).  Couplings: block (n, n+1) =
    ½ωₙ² conj(TΔϵ), block (n+1, n) = ½ωₙ₊₁² TΔϵ (:93-101).  Returns
    (A, omegas, S) with S = [(Sxf, Syf)] per sideband (one entry when shared)."""
    eps0, mu0, _ = normalize_parameters(g.L0)
    K = 2 * nsidebands + 1
    wn = omega + Omega * np.arange(-nsidebands, nsidebands + 1)
    Te = sp.diags(eps0 * vec(np.asarray(eps_r, dtype=np.complex128)), 0)
    TDe = sp.diags(eps0 * vec(np.asarray(deps_r, dtype=np.complex128)), 0)
    dxb, dxf = delta(X, BACKWARD, g), delta(X, FORWARD, g)
    dyb, dyf = delta(Y, BACKWARD, g), delta(Y, FORWARD, g)
    blocks, S = [], []
    for j in range(K if not sharedpml else 1):
        Sxf, Sxb, Syf, Syb = S_create(g, omega if sharedpml else wn[j], m, lnR)
        S.append((Sxf, Syf, Sxb @ dxb * (1 / mu0) @ Sxf @ dxf + Syb @ dyb * (1 / mu0) @ Syf @ dyf))
    for j in range(K):
        A1 = S[0 if sharedpml else j][2]
        blocks.append(A1 + wn[j] ** 2 * Te)
    A = sp.block_diag(blocks, format="csr")
    if nsidebands > 0:
        Cp = sp.kron(sp.diags(0.5 * wn[:-1] ** 2, 1), TDe.conj())
        Cm = sp.kron(sp.diags(0.5 * wn[1:] ** 2, -1), TDe)
        A = A + Cp + Cm
    return A.tocsc(), wn, [(a, b) for a, b, _ in S]


def solve_modulated(g: Grid, eps_r, deps_r, src, omega: float, Omega: float, nsidebands: int,
                    sharedpml=True, m=3.5, lnR=-12.0):
    """``solve(d::ModulatedDevice)`` for one ω: src/solver/modulation.jl:35-119.

    b = iω·src in the centre sideband block (:67-69); Ez per sideband and
    H with forward differences, hx = -Syf δyf ez/(iωₙμ₀), hy = Sxf δxf ez/(iωₙμ₀)
    (:110-114).  Returns a list of K (Ez, Hx, Hy) triples, n = -s..s."""
    eps0, mu0, _ = normalize_parameters(g.L0)
    A, wn, S = modulated_system(g, eps_r, deps_r, omega, Omega, nsidebands, sharedpml, m, lnR)
    N = g.N[0] * g.N[1]
    K = len(wn)
    b = np.zeros(K * N, dtype=np.complex128)
    b[nsidebands * N:(nsidebands + 1) * N] = 1j * omega * vec(np.asarray(src, dtype=np.complex128))
    ez = dolinearsolve(A, b)
    dxf, dyf = delta(X, FORWARD, g), delta(Y, FORWARD, g)
    out = []
    for j in range(K):
        e = ez[j * N:(j + 1) * N]
        Sxf, Syf = S[0 if sharedpml else j]
        hx = -1 / 1j / wn[j] / mu0 * (Syf @ (dyf @ e))
        hy = 1 / 1j / wn[j] / mu0 * (Sxf @ (dxf @ e))
        out.append((unvec(e, g.N), unvec(hx, g.N), unvec(hy, g.N)))
    return out


def relative_residual(A, x, b):
    return np.linalg.norm(b - A @ x) / np.linalg.norm(b)
