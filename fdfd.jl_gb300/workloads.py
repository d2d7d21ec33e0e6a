"""Seeded synthetic FDFD problems (permittivity, source, frequency).

The problems follow the benchmark conventions of the GPU solve path:
free-space wavelength λ₀ = 1.55 µm, cell size dl = λ₀/20, length unit
L₀ = 1 µm, angular frequency ω = 2πc₀/λ (SI rad/s), 20 PML cells on every
side graded with m = 4 and target reflection R = 1e-8 (lnR = ln 1e-8),
background ϵᵣ = 1, silicon-like guides ϵᵣ = 12.25, random design pixels drawn
i.i.d. uniform in [1, 12.25] from ``numpy.random.default_rng(seed)``.

A Gaussian line source has the profile src(iy) = exp(-((iy - y0)/w)²) with the
waist w and centre y0 given in cells; it lies on the grid column ix = Npml+30.

Arrays are (Nx, Ny) complex128, x the first axis; flattened column-major
(x fastest) they match the unknown ordering of the reference's ``A[:]``.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

EPS0 = 8.85418782e-12
MU0 = 1.25663706e-6
C0 = math.sqrt(1 / EPS0 / MU0)

LAMBDA0 = 1.55          # µm
DL = LAMBDA0 / 20       # µm
NPML = 20
PML_M = 4.0
PML_LNR = math.log(1e-8)
EPS_GUIDE = 12.25
GUIDE_CELLS = 10


def omega_of(lam_um: float) -> float:
    return 2 * math.pi * C0 / (lam_um * 1e-6)


@dataclass
class Problem:
    """One driven problem: grid sizes and spacing, PML, ϵᵣ, source(s), ω."""
    name: str
    Nx: int
    Ny: int
    dx: float
    dy: float
    npml: tuple
    eps: np.ndarray             # (Nx, Ny) complex128
    src: np.ndarray             # (Nx, Ny) or (nrhs, Nx, Ny) complex128
    omega: float
    pml_m: float = PML_M
    pml_lnR: float = PML_LNR
    L0: float = 1e-6
    extra: dict = field(default_factory=dict)

    @property
    def xrange(self):
        return (0.0, self.Nx * self.dx)

    @property
    def yrange(self):
        return (0.0, self.Ny * self.dy)


def gaussian_line(Ny: int, y0: float, waist: float) -> np.ndarray:
    iy = np.arange(Ny, dtype=np.float64)
    return np.exp(-((iy - y0) / waist) ** 2)


def _guide_rows(Ny):
    lo = Ny // 2 - GUIDE_CELLS // 2
    return lo, lo + GUIDE_CELLS


def waveguide_eps(Nx, Ny, design=None, seed=0, arms="through"):
    """ϵᵣ with a guide along x centred in y and an optional centred random
    design region of (dwx, dwy) cells.  arms="through" runs the guide over the
    whole length; "split" stops it at the design region (input + output arms).
    """
    eps = np.ones((Nx, Ny), dtype=np.complex128)
    g0, g1 = _guide_rows(Ny)
    if design is None or arms == "through":
        eps[:, g0:g1] = EPS_GUIDE
    if design is not None:
        dwx, dwy = design
        x0 = Nx // 2 - dwx // 2
        y0 = Ny // 2 - dwy // 2
        if arms == "split":
            eps[:x0, g0:g1] = EPS_GUIDE
            eps[x0 + dwx:, g0:g1] = EPS_GUIDE
        rng = np.random.default_rng(seed)
        eps[x0:x0 + dwx, y0:y0 + dwy] = rng.uniform(1.0, EPS_GUIDE, size=(dwx, dwy))
    return eps


def design_box(Nx, Ny, design):
    dwx, dwy = design
    x0 = Nx // 2 - dwx // 2
    y0 = Ny // 2 - dwy // 2
    return x0, y0, dwx, dwy


def point_source_guide(Nx=200, Ny=120, npml=NPML, name="point_guide"):
    """Plain FP64 TM solve problem: straight guide, Jz=1 point source 30 cells
    inside the left PML edge, at the guide centre."""
    eps = waveguide_eps(Nx, Ny)
    src = np.zeros((Nx, Ny), dtype=np.complex128)
    src[npml + 30, Ny // 2] = 1.0
    return Problem(name, Nx, Ny, DL, DL, (npml, npml), eps, src, omega_of(LAMBDA0))


def design_guide(Nx=800, Ny=480, design=(200, 200), seed=2, waist=8.0, npml=NPML,
                 name="design_guide"):
    """Input and output guide arms around a seeded random design region,
    Gaussian line source across the input guide."""
    eps = waveguide_eps(Nx, Ny, design=design, seed=seed, arms="split")
    src = np.zeros((Nx, Ny), dtype=np.complex128)
    g0, g1 = _guide_rows(Ny)
    src[npml + 30, :] = gaussian_line(Ny, 0.5 * (g0 + g1 - 1), waist)
    return Problem(name, Nx, Ny, DL, DL, (npml, npml), eps, src, omega_of(LAMBDA0),
                   extra={"design": design, "seed": seed, "waist": waist})


def frequency_sweep(Nx=400, Ny=400, design=(160, 160), seed=3, n_freq=64, n_src=8,
                    waist=6.0, npml=NPML, lam_range=(1.45, 1.65)):
    """Batched sweep: one seeded design, n_freq wavelengths uniform in
    lam_range, each with n_src Gaussian line sources at seeded y-offsets.
    Returns (problem at the first wavelength with all sources stacked, lams)."""
    eps = waveguide_eps(Nx, Ny, design=design, seed=seed, arms="split")
    rng = np.random.default_rng(seed + 1000)
    lams = rng.uniform(lam_range[0], lam_range[1], size=n_freq)
    g0, g1 = _guide_rows(Ny)
    yc = 0.5 * (g0 + g1 - 1)
    offs = rng.uniform(-Ny / 8, Ny / 8, size=n_src)
    src = np.zeros((n_src, Nx, Ny), dtype=np.complex128)
    for k in range(n_src):
        src[k, npml + 30, :] = gaussian_line(Ny, yc + offs[k], waist)
    p = Problem("frequency_sweep", Nx, Ny, DL, DL, (npml, npml), eps, src,
                omega_of(lams[0]), extra={"lams": lams, "offsets": offs, "seed": seed})
    return p, lams


def mixed_size_batch(n=32, sizes=(128, 256, 512, 1024), seed=5, npml=NPML):
    """n independent square problems, side drawn from ``sizes`` (seeded);
    each a split guide with a centred random design of half the side."""
    rng = np.random.default_rng(seed)
    sides = rng.choice(np.asarray(sizes), size=n)
    probs = []
    for k, s in enumerate(sides):
        s = int(s)
        p = design_guide(s, s, design=(s // 2, s // 2), seed=seed * 1000 + k, waist=6.0,
                         npml=npml, name=f"mixed_{k}_{s}")
        probs.append(p)
    return probs


def adjoint_problem(Nx=1000, Ny=600, design=(300, 300), seed=4, waist=8.0, npml=NPML):
    """Adjoint gradient problem: objective J = |Σ_line m·Ez|² with m a Gaussian
    (waist 8 cells) on the column 40 cells before the right PML."""
    p = design_guide(Nx, Ny, design=design, seed=seed, waist=waist, npml=npml,
                     name="adjoint")
    g0, g1 = _guide_rows(Ny)
    mvec = np.zeros((Nx, Ny), dtype=np.complex128)
    mvec[Nx - npml - 40, :] = gaussian_line(Ny, 0.5 * (g0 + g1 - 1), waist)
    p.extra["mvec"] = mvec
    p.extra["design_box"] = design_box(Nx, Ny, design)
    return p


def phc_cavity(n_cells=12, res=20, eps_rod=8.9, radius=0.2, npml=NPML, a_um=1.0,
               freq_norm=0.38):
    """Square lattice of n_cells x n_cells rods (radius·a, ϵᵣ=eps_rod) in air
    with the rod at the origin removed, `res` cells per lattice constant a.
    Rod centres sit at (i - n_cells//2)·a for i = 0..n_cells-1 on both axes;
    the domain spans the lattice plus half a period on each side plus the PML.
    Returns (problem, ω₀) with ω₀ a/(2πc) = freq_norm."""
    dx = a_um / res
    n_in = n_cells * res
    N = n_in + 2 * npml
    x0 = -(n_cells // 2 + 0.5) * a_um - npml * dx  # left edge of the domain
    xc = x0 + dx * (np.arange(N) + 0.5)
    X, Y = np.meshgrid(xc, xc, indexing="ij")
    eps = np.ones((N, N), dtype=np.complex128)
    centres = [(i - n_cells // 2) * a_um for i in range(n_cells)]
    r2 = (radius * a_um) ** 2
    for cx in centres:
        for cy in centres:
            if abs(cx) < 1e-12 and abs(cy) < 1e-12:
                continue
            eps[(X - cx) ** 2 + (Y - cy) ** 2 <= r2] = eps_rod
    omega0 = 2 * math.pi * freq_norm * C0 / (a_um * 1e-6)
    src = np.zeros((N, N), dtype=np.complex128)
    p = Problem("phc_cavity", N, N, dx, dx, (npml, npml), eps, src, omega0,
                extra={"x0": x0})
    return p, omega0


def modulated_waveguide(dh=0.02, L=5.0, nsidebands=1, npml=(15, 15), waist_um=0.2, sharedpml=True,
                        mod_range=None):
    """Interband photonic transition in a modulated waveguide, the setup of the
    reference's own modulated-device test (test/runtests.jl:40-63): x ∈ [0, L],
    y ∈ [-1, 1] µm at cell size dh, 15 PML cells, carrier ω = 2π·193.9 THz,
    modulation Ω = 4.541e14 rad/s, a guide of width a = 0.2202 µm (ϵᵣ = 12.25)
    and Δϵᵣ = exp(i q x), q = 2.9263 µm⁻¹, on the lower half of the guide for
    x in ``mod_range`` (default [1, L-1]).  The reference drives the guide with a
    mode source; here a Gaussian line source of waist ``waist_um`` across the
    guide at x = 0.2 µm stands in.  PML grading is the reference default
    (m = 3.5, lnR = -12).  ``extra`` holds deps, Omega, nsidebands, sharedpml."""
    if np.isscalar(npml):
        npml = (int(npml), int(npml))
    x0, x1 = mod_range if mod_range is not None else (1.0, L - 1.0)
    Nx, Ny = int(round(L / dh)), int(round(2.0 / dh))
    xc = 0.0 + dh * (np.arange(Nx) + 0.5)
    yc = -1.0 + dh * (np.arange(Ny) + 0.5)
    X, Y = np.meshgrid(xc, yc, indexing="ij")
    a, q = 0.2202, 2.9263
    eps = np.ones((Nx, Ny), dtype=np.complex128)
    eps[(-a / 2 <= Y) & (Y <= a / 2)] = 12.25
    deps = np.zeros((Nx, Ny), dtype=np.complex128)
    reg = (x0 <= X) & (X <= x1) & (-a / 2 <= Y) & (Y <= 0.0)
    deps[reg] = np.exp(1j * q * X[reg])
    src = np.zeros((Nx, Ny), dtype=np.complex128)
    ix = int(round(0.2 / dh))
    src[ix, :] = np.exp(-(yc / waist_um) ** 2)
    return Problem(f"modulated_waveguide_{Nx}x{Ny}", Nx, Ny, dh, dh, tuple(npml), eps, src,
                   2 * math.pi * 1.939e14, pml_m=3.5, pml_lnR=-12.0,
                   extra={"deps": deps, "Omega": 4.541e14, "nsidebands": nsidebands, "sharedpml": sharedpml})


def modulated_notebook(nsidebands=1):
    """The modulated-waveguide example of the reference's notebook
    (notebooks/Example_simulations.ipynb, the ModulatedDevice cell): dh = 0.01 µm,
    x ∈ [0, 15], y ∈ [-1, 1] (1500 x 200 cells), PML 15 x 10 cells, modulation on
    1.5 ≤ x ≤ 11.7, one sideband on each side of the carrier."""
    return modulated_waveguide(dh=0.01, L=15.0, nsidebands=nsidebands, npml=(15, 10), mod_range=(1.5, 11.7))
