"""fdfd_gb300 — GB300 solve path for 2-D FDFD problems, host-side mirror of
the FDFD.jl interface on that path.

The reference (fancompute/FDFD.jl) exposes ``Grid``, ``Device``,
``setup_ϵᵣ!``, ``setup_src!``, ``solve(d, pol)`` and
``eigenfrequency(d, pol, nev; which)`` returning ``FieldTM``/``FieldTE``
(src/grid.jl, src/device.jl, src/solver/driven.jl, src/solver/eigen.jl,
src/data.jl).  This module keeps those names, argument meanings and return
shapes and runs every solve through ``libfdfd_cuda`` (the C ABI in
include/fdfd_cuda.h) — the role ``ENV["FDFD_SOLVER"] = "cuda"`` plays for a
Julia caller.  There is no CPU fallback: without the CUDA library every solve
raises.

Arrays are numpy (Nx, Ny) with x the first axis, i.e. the reference's Julia
column-major layout.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import FDFDError, FDFD_PREC_FP64, FDFD_PREC_MIXED  # noqa: F401

__all__ = ["EPS0", "MU0", "C0", "ETA0", "TM", "TE", "X", "Y", "Grid", "Device", "ModulatedDevice", "Point", "Mode",
           "setup_eps", "setup_src", "setup_deps", "add_mode", "setup_mode", "get_modes", "solve", "eigenfrequency",
           "FieldTM", "FieldTE", "Flux", "probe_field", "poynting", "flux_surface_integral", "unwrap", "Chi3Device", "setup_chi",
           "IterativeMethodGN", "IterativeMethodB", "normalize_parameters", "FDFDError"]

# src/types.jl:6-9
EPS0 = 8.85418782e-12
MU0 = 1.25663706e-6
C0 = math.sqrt(1 / EPS0 / MU0)
ETA0 = math.sqrt(MU0 / EPS0)
DEFAULT_L0 = 1e-6          # src/grid.jl:5
TM, TE = _lib.FDFD_TM, _lib.FDFD_TE   # src/types.jl:20
X, Y = _lib.FDFD_X, _lib.FDFD_Y       # src/types.jl:18 (x̂, ŷ)
IterativeMethodGN, IterativeMethodB = _lib.FDFD_CHI3_NEWTON, _lib.FDFD_CHI3_BORN   # src/solver/nonlinear.jl:5


@dataclass
class Point:
    """src/types.jl:23-26."""
    x: float
    y: float


class Grid:
    """2-D grid (src/grid.jl:7-33): N = round(L/dh) cells per axis, Npml PML
    cells per side, bounds ((x1, y1), (x2, y2)) in units of L₀."""

    def __init__(self, dh, Npml, xrange, yrange, L0=DEFAULT_L0):
        L = (float(xrange[1] - xrange[0]), float(yrange[1] - yrange[0]))
        self.N = (int(round(L[0] / dh)), int(round(L[1] / dh)))
        self.Npml = (int(Npml[0]), int(Npml[1]))
        self.bounds = ((float(xrange[0]), float(yrange[0])), (float(xrange[1]), float(yrange[1])))
        self.L = L
        self.L0 = float(L0)

    @classmethod
    def from_cells(cls, Nx, Ny, dx, dy, Npml, x0=0.0, y0=0.0, L0=DEFAULT_L0):
        g = cls.__new__(cls)
        g.N = (int(Nx), int(Ny))
        g.Npml = (int(Npml[0]), int(Npml[1]))
        g.bounds = ((float(x0), float(y0)), (float(x0 + Nx * dx), float(y0 + Ny * dy)))
        g.L = (g.bounds[1][0] - g.bounds[0][0], g.bounds[1][1] - g.bounds[0][1])
        g.L0 = float(L0)
        return g

    def size(self):
        return self.N

    def dx(self):  # src/grid.jl:68-70
        return (self.bounds[1][0] - self.bounds[0][0]) / self.N[0]

    def dy(self):  # src/grid.jl:72-74
        return (self.bounds[1][1] - self.bounds[0][1]) / self.N[1]

    def xc(self):  # src/grid.jl:76-78
        return self.bounds[0][0] + self.dx() * (np.arange(self.N[0]) + 0.5)

    def yc(self):  # src/grid.jl:80-82
        return self.bounds[0][1] + self.dy() * (np.arange(self.N[1]) + 0.5)

    def dh(self, w):  # src/grid.jl:63-66
        return self.dx() if w == X else self.dy()

    def xe(self):  # src/grid.jl:89-91: the N+1 cell edges along x
        return self.bounds[0][0] + self.dx() * np.arange(self.N[0] + 1)

    def ye(self):  # src/grid.jl:93-95
        return self.bounds[0][1] + self.dy() * np.arange(self.N[1] + 1)

    def x2ind(self, x):
        """0-based index of the cell nearest x, clamped to the grid (src/grid.jl:112-117;
        Julia's round and Python's both round half to even)."""
        i = int(round((x - self.bounds[0][0]) / self.L[0] * self.N[0]) + 1)
        return min(max(i, 1), self.N[0]) - 1

    def y2ind(self, y):  # src/grid.jl:120-125, 0-based
        i = int(round((y - self.bounds[0][1]) / self.L[1] * self.N[1]) + 1)
        return min(max(i, 1), self.N[1]) - 1

    def coord2ind(self, pt: Point):
        """0-based (ix, iy), src/grid.jl:103-125."""
        return self.x2ind(pt.x), self.y2ind(pt.y)


@dataclass
class Mode:
    """src/device.jl:5-11: polarization, slice normal (X or Y), effective-index
    guess, centre point and slice width (L₀ units)."""
    pol: int
    dir: int
    neff: complex
    pt: Point
    width: float


def normalize_parameters(g: Grid):
    """(ϵ₀L₀, μ₀L₀, c₀/L₀): src/device.jl:40."""
    return EPS0 * g.L0, MU0 * g.L0, C0 / g.L0


@dataclass
class Device:
    """src/device.jl:19-35: grid, complex ϵᵣ and src arrays, frequencies ω."""
    grid: Grid
    omega: list
    eps: np.ndarray = None
    src: np.ndarray = None
    modes: list = field(default_factory=list)

    def __post_init__(self):
        if np.isscalar(self.omega):
            self.omega = [float(self.omega)]
        if self.eps is None:
            self.eps = np.ones(self.grid.N, dtype=np.complex128)
        if self.src is None:
            self.src = np.zeros(self.grid.N, dtype=np.complex128)


@dataclass
class ModulatedDevice:
    """src/solver/modulation.jl:4-26: a Device with a modulation amplitude Δϵᵣ
    (zero by default), modulation frequency Ω, the number of sidebands on each
    side of the carrier and whether the sidebands share the carrier's PML."""
    grid: Grid
    omega: list
    Omega: float
    nsidebands: int
    sharedpml: bool = True
    eps: np.ndarray = None
    deps: np.ndarray = None
    src: np.ndarray = None
    modes: list = field(default_factory=list)

    def __post_init__(self):
        if np.isscalar(self.omega):
            self.omega = [float(self.omega)]
        if self.eps is None:
            self.eps = np.ones(self.grid.N, dtype=np.complex128)
        if self.deps is None:
            self.deps = np.zeros(self.grid.N, dtype=np.complex128)
        if self.src is None:
            self.src = np.zeros(self.grid.N, dtype=np.complex128)


@dataclass
class Chi3Device:
    """src/solver/nonlinear.jl:9-27: a Device with a real χ⁽³⁾ array (zero by default)."""
    grid: Grid
    omega: list
    eps: np.ndarray = None
    chi: np.ndarray = None
    src: np.ndarray = None
    modes: list = field(default_factory=list)

    def __post_init__(self):
        if np.isscalar(self.omega):
            self.omega = [float(self.omega)]
        if self.eps is None:
            self.eps = np.ones(self.grid.N, dtype=np.complex128)
        if self.chi is None:
            self.chi = np.zeros(self.grid.N, dtype=np.float64)
        if self.src is None:
            self.src = np.zeros(self.grid.N, dtype=np.complex128)


def _mask(d, region):
    X, Y = np.meshgrid(d.grid.xc(), d.grid.yc(), indexing="ij")
    return np.vectorize(region)(X, Y).astype(bool), X, Y


def setup_eps(d: Device, region, value):
    """setup_ϵᵣ!(d, region, value): src/device.jl:63-89 (region and value may be callables of (x, y))."""
    m, X, Y = _mask(d, region)
    d.eps[m] = np.vectorize(value)(X, Y)[m] if callable(value) else value


def setup_src(d: Device, where, value=None):
    """setup_src!(d, pt) puts 1im at the point (src/device.jl:95-98);
    setup_src!(d, pt, srcnormal) puts 1im on the whole grid line through the
    point normal to srcnormal, X or Y (device.jl:101-108);
    setup_src!(d, region, value) fills a region (device.jl:92)."""
    if isinstance(where, Point):
        ix, iy = d.grid.coord2ind(where)
        if value is None:
            d.src[ix, iy] = 1j
        elif value == X:
            d.src[ix, :] = 1j
        elif value == Y:
            d.src[:, iy] = 1j
        else:
            raise FDFDError(_lib.FDFD_EINVAL, "srcnormal must be X or Y")
        return
    m, xs, ys = _mask(d, where)
    d.src[m] = np.vectorize(value)(xs, ys)[m] if callable(value) else value


def setup_deps(d: ModulatedDevice, region, value):
    """setup_Δϵᵣ!(d, region, value): src/solver/modulation.jl:31-32 (region and value may be callables)."""
    m, X, Y = _mask(d, region)
    d.deps[m] = np.vectorize(value)(X, Y)[m] if callable(value) else value


def setup_chi(d: Chi3Device, region, value):
    """setup_χ!(d, region, value): src/solver/nonlinear.jl:32-33."""
    m, X_, Y_ = _mask(d, region)
    d.chi[m] = np.vectorize(value)(X_, Y_)[m] if callable(value) else value


globals()["setup_χ"] = setup_chi


def add_mode(d, mode: Mode):
    """add_mode!(d, mode): src/device.jl:112-115."""
    d.modes.append(mode)


def _mode_spec(d, m: Mode, pol=None):
    ix, iy = d.grid.coord2ind(m.pt if isinstance(m.pt, Point) else Point(*m.pt))
    return (m.pol if pol is None else pol, m.dir, ix, iy, m.width, m.neff)


def _mode_handle(d):
    g = d.grid
    h = _lib.Handle(g.N[0], g.N[1], g.Npml[0], g.Npml[1], g.dx(), g.dy(), g.L0, 3.5, -12.0, TM, FDFD_PREC_MIXED)
    h.set_eps(d.eps)
    return h


def get_modes(d, pol, omega, neff, nmodes, pt: Point, slicenormal, slicewidth):
    """get_modes(d, pol, ω, neff, nmodes, pt, slicenormal, slicewidth): src/device.jl:124-149, computed on
    the GPU (nmodes = 1).  Returns (β, vector, indx, indy) with 0-based slice indices."""
    if nmodes != 1:
        raise FDFDError(_lib.FDFD_EINVAL, "get_modes: the GPU mode solver returns one mode (nmodes = 1)")
    h = _mode_handle(d)
    try:
        ix, iy = d.grid.coord2ind(pt if isinstance(pt, Point) else Point(*pt))
        beta, v = h.get_mode(omega, pol, slicenormal, ix, iy, slicewidth, neff)
    finally:
        h.close()
    M = (v.size - 1) // 2
    if slicenormal == X:
        return beta, v, ix, np.arange(iy - M, iy + M + 1)
    return beta, v, np.arange(ix - M, ix + M + 1), iy


def setup_mode(d, pol, omega, neff, pt: Point, srcnormal, srcwidth):
    """setup_mode!(d, pol, ω, neff, pt, srcnormal, srcwidth): src/device.jl:118-121 — adds
    normalize(abs.(v)) to d.src on the slice."""
    h = _mode_handle(d)
    try:
        m = Mode(pol, srcnormal, neff, pt, srcwidth)
        d.src = d.src + h.mode_sources([omega], [_mode_spec(d, m)])[0]
    finally:
        h.close()


globals()["setup_ϵᵣ"] = setup_eps
globals()["setup_Δϵᵣ"] = setup_deps


class _Field:
    components = ()

    def __init__(self, grid, omega, data):
        self.grid = grid
        self.omega = complex(omega)
        self.data = data            # (Nx, Ny, 3) complex

    def __getitem__(self, comp):
        if isinstance(comp, str):
            return self.data[:, :, self.components.index(comp)]
        return self.data[comp]

    @property
    def shape(self):
        return self.data.shape


class FieldTM(_Field):
    """src/data.jl:50-63: Nx x Ny x 3 with components [:Ez, :Hx, :Hy]."""
    components = ("Ez", "Hx", "Hy")


class FieldTE(_Field):
    """src/data.jl:65-78: Nx x Ny x 3 with components [:Hz, :Ex, :Ey]."""
    components = ("Hz", "Ex", "Ey")


@dataclass
class Flux:
    """src/data.jl (Flux): grid, ω and the Poynting components Sx, Sy (Nx x Ny)."""
    grid: Grid
    omega: complex
    Sx: np.ndarray
    Sy: np.ndarray


def _field_handle(field):
    g = field.grid
    return _lib.Handle(g.N[0], g.N[1], g.Npml[0], g.Npml[1], g.dx(), g.dy(), g.L0, 3.5, -12.0, TM, FDFD_PREC_MIXED)


def _pol_of(field):
    return TM if isinstance(field, FieldTM) else TE


def unwrap(v, inplace=False):
    """unwrap(v, inplace=false): src/FDFD.jl:19-31.  Phase unwrapping in the
    reference's order: each entry is shifted by 2π while it differs from the
    already unwrapped previous entry by ≥ π (then ≤ -π).  Non-finite entries are
    left as they are (the reference's loops would not end on ±Inf)."""
    u = v if inplace else np.array(v, dtype=np.float64, copy=True)
    for i in range(1, len(u)):
        if not (math.isfinite(u[i]) and math.isfinite(u[i - 1])):
            continue
        while u[i] - u[i - 1] >= math.pi:
            u[i] -= 2 * math.pi
        while u[i] - u[i - 1] <= -math.pi:
            u[i] += 2 * math.pi
    return u


def probe_field(field, component: str, pt: Point):
    """probe_field(field, component, pt): src/flux.jl:6-12.  The value of
    `component` ("Ez", "Hx", "Hy" for TM; "Hz", "Ex", "Ey" for TE) in the cell
    whose centre lies within half a cell of pt on each axis, as AxisArrays'
    atvalue(…, atol = dh/2) selects it; the first such cell on a tie."""
    g = field.grid
    ix = np.nonzero(np.abs(g.xc() - pt.x) <= g.dx() / 2)[0]
    iy = np.nonzero(np.abs(g.yc() - pt.y) <= g.dy() / 2)[0]
    if ix.size == 0 or iy.size == 0:
        raise FDFDError(_lib.FDFD_EINVAL, f"no grid cell centre within half a cell of ({pt.x}, {pt.y})")
    if component not in field.components:
        raise FDFDError(_lib.FDFD_EINVAL, "%s is invalid for the %s polarization. Valid options are %s" %
                        (component, "TM" if isinstance(field, FieldTM) else "TE",
                         ", ".join(":" + c for c in field.components)))
    return complex(field[component][ix[0], iy[0]])


def poynting(field):
    """poynting(field::Field): src/flux.jl:15-29, on the GPU."""
    h = _field_handle(field)
    try:
        Sx, Sy = h.poynting(_pol_of(field), field.data[:, :, 0], field.data[:, :, 1], field.data[:, :, 2])
    finally:
        h.close()
    return Flux(field.grid, field.omega, Sx, Sy)


def flux_surface_integral(field, center: Point, width, normal):
    """flux_surface_integral(field, center, width, normal): src/flux.jl:37-66, on the GPU.
    The column is the one whose centre lies within dx/2 of center.x; the rows are
    those whose centres lie in [center.y - width, center.y + width]."""
    g = field.grid
    if normal == Y:
        raise FDFDError(_lib.FDFD_EINVAL, "ŷ normal %s calculation not yet implemented" %
                        ("TM" if _pol_of(field) == TM else "TE"))
    xc, yc = g.xc(), g.yc()
    hit = np.nonzero(np.abs(xc - center.x) <= g.dx() / 2)[0]
    if hit.size == 0:
        raise FDFDError(_lib.FDFD_EINVAL, "no grid column at center.x")
    rows = np.nonzero((yc >= center.y - width) & (yc <= center.y + width))[0]
    if rows.size == 0:
        raise FDFDError(_lib.FDFD_EINVAL, "no grid row in the interval")
    h = _field_handle(field)
    try:
        out = h.flux_integral(_pol_of(field), field.data[:, :, 0], field.data[:, :, 2],
                              [(int(hit[0]), int(rows[0]), int(rows[-1]))], normal)
    finally:
        h.close()
    return float(out[0])


def _prec(precision):
    if isinstance(precision, str):
        return {"fp64": FDFD_PREC_FP64, "mixed": FDFD_PREC_MIXED}[precision]
    return int(precision)


def make_handle(d: Device, pol=TM, precision="mixed", pml_m=3.5, pml_lnR=-12.0, tol=1e-10, max_iter=40):
    g = d.grid
    h = _lib.Handle(g.N[0], g.N[1], g.Npml[0], g.Npml[1], g.dx(), g.dy(), g.L0, pml_m, pml_lnR, pol,
                    _prec(precision))
    h.set_refinement(tol, max_iter)
    h.set_eps(d.eps)
    return h


def solve(d: Device, pol=TM, precision="mixed", pml_m=3.5, pml_lnR=-12.0, tol=1e-10, max_iter=40,
          return_stats=False, frequencies_per_launch=1, autotune=False):
    """solve(d::Device, pol) — src/solver/driven.jl:4-59.

    One factorization per frequency (as the reference re-factors per ω) and a
    refined solve for d.src.  ``pml_m``/``pml_lnR`` default to the values the
    reference hard-wires (src/pml.jl:1, S_create does not forward them).
    Returns a FieldTM/FieldTE, or a list when len(d.omega) > 1 (driven.jl:57-58).
    A ModulatedDevice takes the coupled-sideband path (``solve_modulated``).

    ``frequencies_per_launch`` > 1 (several frequencies, no mode sources): that many
    handles are factored together, one frequency each, by one CUDA-graph launch
    (fdfd_batch_factor), and their solves run concurrently.  ``autotune`` runs the
    launch-shape autotuner on every handle first.
    """
    if isinstance(d, ModulatedDevice):
        return solve_modulated(d, precision, pml_m, pml_lnR, tol, max_iter, return_stats)
    if isinstance(d, Chi3Device):
        # solve(d::χ3Device, which_method): the second argument is the iterative method
        return solve_chi3(d, pol, precision, pml_m, pml_lnR, max_iter=max_iter, return_stats=return_stats)
    if frequencies_per_launch > 1 and len(d.omega) > 1 and not d.modes:
        return _solve_batched(d, pol, precision, pml_m, pml_lnR, tol, max_iter, return_stats,
                              int(frequencies_per_launch), autotune)
    h = make_handle(d, pol, precision, pml_m, pml_lnR, tol, max_iter)
    if autotune:
        h.autotune()
    out, stats = [], []
    try:
        if d.modes:
            # driven.jl:15-19: per ω the source is reset and rebuilt from the modes
            # (TM profiles, as the reference's loop passes TM); all ω in one launch
            srcs = h.mode_sources(d.omega, [_mode_spec(d, m, TM) for m in d.modes])
        for i, w in enumerate(d.omega):
            if d.modes:
                d.src = srcs[i].copy()
            h.factor(w)
            f1, f2, f3, st = h.solve(d.src)
            cls = FieldTM if pol == TM else FieldTE
            out.append(cls(d.grid, w, np.stack([f1, f2, f3], axis=-1)))
            stats.append(st.as_dict())
    finally:
        h.close()
    res = out[0] if len(out) == 1 else out
    return (res, stats) if return_stats else res


def _solve_batched(d, pol, precision, pml_m, pml_lnR, tol, max_iter, return_stats, width, autotune):
    """solve() for many frequencies: `width` handles, one CUDA-graph launch factoring a wave of
    `width` frequencies, then their solves concurrently (the driver's threads wait in the library,
    outside the interpreter lock)."""
    import concurrent.futures as cf
    omegas = list(d.omega)
    width = min(width, len(omegas))
    hs = [make_handle(d, pol, precision, pml_m, pml_lnR, tol, max_iter) for _ in range(width)]
    cls = FieldTM if pol == TM else FieldTE
    out, stats = [None] * len(omegas), [None] * len(omegas)
    batch = None
    try:
        if autotune:
            for h in hs:
                h.autotune()
        batch = _lib.Batch(hs)
        with cf.ThreadPoolExecutor(max_workers=width) as ex:
            for w0 in range(0, len(omegas), width):
                wave = omegas[w0:w0 + width]
                if len(wave) == width:
                    batch.factor(wave)
                else:                        # a short last wave: its handles factor one by one
                    for h, w in zip(hs, wave):
                        h.factor(w)
                res = list(ex.map(lambda h: h.solve(d.src), hs[:len(wave)]))
                for k, (w, (f1, f2, f3, st)) in enumerate(zip(wave, res)):
                    out[w0 + k] = cls(d.grid, w, np.stack([f1, f2, f3], axis=-1))
                    stats[w0 + k] = st.as_dict()
    finally:
        if batch is not None:
            batch.close()
        for h in hs:
            h.close()
    res = out[0] if len(out) == 1 else out
    return (res, stats) if return_stats else res


def solve_chi3(d: Chi3Device, method=IterativeMethodGN, precision="mixed", pml_m=3.5, pml_lnR=-12.0,
               tol=1e-12, maxiterations=50, max_iter=40, return_stats=False):
    """solve(d::χ3Device, which_method) — src/solver/nonlinear.jl:36-90 (TM): per ω one
    factorization of the linear operator, reused by every Born or Newton step."""
    g = d.grid
    h = _lib.Handle(g.N[0], g.N[1], g.Npml[0], g.Npml[1], g.dx(), g.dy(), g.L0, pml_m, pml_lnR, TM,
                    _prec(precision))
    out, stats = [], []
    try:
        h.set_refinement(1e-10, max_iter)
        h.set_eps(d.eps)
        if d.modes:
            srcs = h.mode_sources(d.omega, [_mode_spec(d, m, TM) for m in d.modes])
        for i, w in enumerate(d.omega):
            if d.modes:
                d.src = srcs[i].copy()
            h.factor(w)
            ez, hx, hy, err, st = h.chi3_solve(d.chi, d.src, method, tol, maxiterations)
            out.append(FieldTM(g, w, np.stack([ez, hx, hy], axis=-1)))
            stats.append(dict(st.as_dict(), step_errors=err.tolist()))
    finally:
        h.close()
    res = out[0] if len(out) == 1 else out
    return (res, stats) if return_stats else res


def solve_modulated(d: ModulatedDevice, precision="mixed", pml_m=3.5, pml_lnR=-12.0, tol=1e-10, max_iter=60,
                    return_stats=False):
    """solve(d::ModulatedDevice) — src/solver/modulation.jl:35-119 (TM).

    Per carrier ω one factorization of the 2s+1 sideband operators and a
    refined solve of the coupled system.  Returns an Nω x (2s+1) nested list of
    FieldTM (the reference's ``Array{FieldTM}(undef, Nω, nfrequencies)``), the
    field of sideband n = -s..s carrying ωₙ = ω + nΩ."""
    g = d.grid
    h = _lib.ModulatedHandle(g.N[0], g.N[1], g.Npml[0], g.Npml[1], g.dx(), g.dy(), d.nsidebands, g.L0, pml_m,
                             pml_lnR, d.sharedpml, _prec(precision))
    out, stats = [], []
    try:
        h.set_refinement(tol, max_iter)
        h.set_eps(d.eps)
        h.set_deps(d.deps)
        if d.modes:
            srcs = h.mode_sources(d.omega, [_mode_spec(d, m, TM) for m in d.modes])   # modulation.jl:51-55
        for i, w in enumerate(d.omega):
            if d.modes:
                d.src = srcs[i].copy()
            h.factor(w, d.Omega)
            ez, hx, hy, st = h.solve(d.src)
            wn = [w + d.Omega * n for n in range(-d.nsidebands, d.nsidebands + 1)]
            out.append([FieldTM(g, wn[j], np.stack([ez[j], hx[j], hy[j]], axis=-1)) for j in range(len(wn))])
            stats.append(st.as_dict())
    finally:
        h.close()
    return (out, stats) if return_stats else out


def eigenfrequency(d: Device, pol, nev, which="LM", precision="mixed", pml_m=3.5, pml_lnR=-12.0, tol=1e-10):
    """eigenfrequency(d, pol, nev; which) — src/solver/eigen.jl:69-115."""
    h = make_handle(d, pol, precision, pml_m, pml_lnR, tol)
    try:
        N = d.grid.N[0] * d.grid.N[1]
        om = np.empty(nev, dtype=np.complex128)
        lam = np.empty(nev, dtype=np.complex128)
        flds = np.empty((nev, 3, N), dtype=np.complex128)
        st = _lib.Stats()
        import ctypes as C
        which_code = {"LM": 0, "LR": 1, "SM": 2, "SR": 3, "LI": 4, "SI": 5}[str(which).lstrip(":")]
        rc = h.lib.fdfd_eigfreq(h.h, float(d.omega[0]), int(nev), which_code, float(tol), _lib.cptr(om),
                                _lib.cptr(lam), _lib.cptr(flds), C.byref(st))
        h._check(rc)
        cls = FieldTM if pol == TM else FieldTE
        fields = []
        for i in range(nev):
            comps = [_lib.from_natural(flds[i, c], d.grid.N[0], d.grid.N[1])[0] for c in range(3)]
            fields.append(cls(d.grid, om[i], np.stack(comps, axis=-1)))
        return om, fields
    finally:
        h.close()
