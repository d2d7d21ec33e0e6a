"""ctypes binding of libfdfd_cuda (include/fdfd_cuda.h).

This is the same binding a Julia ``ccall`` shim makes: plain pointers and
sizes, complex arrays as interleaved float64 pairs, x fastest.  Loading the
library never falls back to anything else: a missing or unloadable
``libfdfd_cuda.so`` raises immediately.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfdfd_cuda.so")

FDFD_OK, FDFD_EINVAL, FDFD_ENOMEM, FDFD_ESINGULAR, FDFD_ENOCONV, FDFD_ETIMEOUT, FDFD_ECUDA = range(7)
STATUS_NAMES = {0: "FDFD_OK", 1: "FDFD_EINVAL", 2: "FDFD_ENOMEM", 3: "FDFD_ESINGULAR", 4: "FDFD_ENOCONV",
                5: "FDFD_ETIMEOUT", 6: "FDFD_ECUDA"}
FDFD_TM, FDFD_TE = 1, 2
FDFD_PREC_FP64, FDFD_PREC_MIXED = 0, 1
FDFD_REFINE_GMRES, FDFD_REFINE_CLASSIC = 0, 1
FDFD_X, FDFD_Y = 1, 2
FDFD_CHI3_NEWTON, FDFD_CHI3_BORN = 1, 2
FDFD_MODE_MAX_POINTS = 1023

# every symbol include/fdfd_cuda.h declares
EXPORTS = ["fdfd_version", "fdfd_create", "fdfd_destroy", "fdfd_last_error", "fdfd_set_refinement",
           "fdfd_set_fallback", "fdfd_set_restart", "fdfd_set_wait_limit", "fdfd_set_device_budget",
           "fdfd_set_checkpoint", "fdfd_checkpoint_info", "fdfd_mf_create", "fdfd_mf_set_deps", "fdfd_mf_factor",
           "fdfd_mf_solve", "fdfd_get_mode", "fdfd_mode_sources", "fdfd_poynting", "fdfd_poynting_device",
           "fdfd_flux_integral", "fdfd_chi3_solve",
           "fdfd_set_eps", "fdfd_factor", "fdfd_solve", "fdfd_solve_device", "fdfd_adjoint", "fdfd_adjoint_vjp", "fdfd_eigfreq",
           "fdfd_batch_create", "fdfd_batch_factor", "fdfd_batch_stats", "fdfd_batch_last_error",
           "fdfd_batch_destroy", "fdfd_autotune", "fdfd_get_tuning", "fdfd_get_stencil", "fdfd_apply", "fdfd_set_profiling", "fdfd_get_profile", "fdfd_residual_noalloc",
           "fdfd_debug_hessenberg_eig", "fdfd_debug_gemm"]
PROF_CLASSES = ["gemm_tc", "gemm_simt", "gj_panel", "sweep", "residual", "other", "gj_update", "level1"]


class Stats(C.Structure):
    _fields_ = [("iterations", C.c_int), ("nrhs", C.c_int), ("rel_residual", C.c_double),
                ("t_assemble_ms", C.c_double), ("t_factor_ms", C.c_double), ("t_solve_ms", C.c_double),
                ("t_recover_ms", C.c_double), ("t_total_ms", C.c_double), ("factor_flops", C.c_double),
                ("block", C.c_int), ("nblocks", C.c_int), ("levels", C.c_int), ("tc_gemm", C.c_int),
                ("device_bytes", C.c_longlong), ("gpu_launches", C.c_longlong),
                ("factor_precision", C.c_int), ("fp64_fallback", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Mode(C.Structure):
    """fdfd_mode: one mode source (Mode, src/device.jl:5-11)."""
    _fields_ = [("pol", C.c_int), ("normal", C.c_int), ("ix", C.c_int), ("iy", C.c_int), ("width", C.c_double),
                ("neff_re", C.c_double), ("neff_im", C.c_double)]


class Profile(C.Structure):
    _fields_ = [("ms", C.c_double * 8), ("work", C.c_double * 8), ("launches", C.c_longlong * 8)]

    def as_dict(self):
        return {k: {"ms": self.ms[i], "work": self.work[i], "launches": self.launches[i]}
                for i, k in enumerate(PROF_CLASSES)}


class FDFDError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


_lib = None


def load(path: str = LIB_PATH) -> C.CDLL:
    """Load libfdfd_cuda.so and declare its signatures (raises if absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise FileNotFoundError(f"{path} is missing: run __graft_entry__.build() (nvcc, sm_103a) first")
    lib = C.CDLL(path)
    vp, dp, ip = C.c_void_p, C.POINTER(C.c_double), C.c_int
    lib.fdfd_version.restype = C.c_char_p
    lib.fdfd_version.argtypes = []
    lib.fdfd_create.restype = ip
    lib.fdfd_create.argtypes = [C.POINTER(vp), ip, ip, ip, ip, C.c_double, C.c_double, C.c_double, C.c_double,
                                C.c_double, ip, ip]
    lib.fdfd_destroy.restype = None
    lib.fdfd_destroy.argtypes = [vp]
    lib.fdfd_last_error.restype = C.c_char_p
    lib.fdfd_last_error.argtypes = [vp]
    lib.fdfd_set_refinement.restype = ip
    lib.fdfd_set_refinement.argtypes = [vp, C.c_double, ip, ip]
    lib.fdfd_set_fallback.restype = ip
    lib.fdfd_set_fallback.argtypes = [vp, ip]
    lib.fdfd_set_restart.restype = ip
    lib.fdfd_set_restart.argtypes = [vp, ip]
    lib.fdfd_set_wait_limit.restype = ip
    lib.fdfd_set_wait_limit.argtypes = [vp, C.c_longlong]
    lib.fdfd_set_device_budget.restype = ip
    lib.fdfd_set_device_budget.argtypes = [vp, C.c_longlong]
    lib.fdfd_set_checkpoint.restype = ip
    lib.fdfd_set_checkpoint.argtypes = [vp, ip]
    lib.fdfd_checkpoint_info.restype = ip
    lib.fdfd_checkpoint_info.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]
    lib.fdfd_mf_create.restype = ip
    lib.fdfd_mf_create.argtypes = [C.POINTER(vp), ip, ip, ip, ip, C.c_double, C.c_double, C.c_double, C.c_double,
                                   C.c_double, ip, ip, ip]
    lib.fdfd_mf_set_deps.restype = ip
    lib.fdfd_mf_set_deps.argtypes = [vp, dp]
    lib.fdfd_mf_factor.restype = ip
    lib.fdfd_mf_factor.argtypes = [vp, C.c_double, C.c_double]
    lib.fdfd_mf_solve.restype = ip
    lib.fdfd_mf_solve.argtypes = [vp, dp, dp, dp, dp, C.POINTER(Stats)]
    lib.fdfd_get_mode.restype = ip
    lib.fdfd_get_mode.argtypes = [vp, C.c_double, C.POINTER(Mode), ip, dp, dp, C.POINTER(C.c_int)]
    lib.fdfd_mode_sources.restype = ip
    lib.fdfd_mode_sources.argtypes = [vp, ip, dp, ip, C.POINTER(Mode), dp]
    lib.fdfd_poynting.restype = ip
    lib.fdfd_poynting.argtypes = [vp, ip, dp, dp, dp, dp, dp]
    lib.fdfd_poynting_device.restype = ip
    lib.fdfd_poynting_device.argtypes = [vp, ip, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.fdfd_flux_integral.restype = ip
    lib.fdfd_flux_integral.argtypes = [vp, ip, dp, dp, ip, ip, C.POINTER(C.c_int), dp]
    lib.fdfd_chi3_solve.restype = ip
    lib.fdfd_chi3_solve.argtypes = [vp, dp, dp, ip, C.c_double, ip, dp, dp, dp, dp, C.POINTER(C.c_int),
                                    C.POINTER(Stats)]
    lib.fdfd_set_eps.restype = ip
    lib.fdfd_set_eps.argtypes = [vp, dp]
    lib.fdfd_factor.restype = ip
    lib.fdfd_factor.argtypes = [vp, C.c_double]
    lib.fdfd_solve.restype = ip
    lib.fdfd_solve.argtypes = [vp, dp, ip, dp, dp, dp, C.POINTER(Stats)]
    lib.fdfd_solve_device.restype = ip
    lib.fdfd_solve_device.argtypes = [vp, C.c_void_p, ip, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(Stats)]
    lib.fdfd_adjoint.restype = ip
    lib.fdfd_adjoint.argtypes = [vp, dp, dp, dp, dp, dp, C.POINTER(Stats)]
    lib.fdfd_adjoint_vjp.restype = ip
    lib.fdfd_adjoint_vjp.argtypes = [vp, dp, dp, dp, dp, C.POINTER(Stats)]
    lib.fdfd_eigfreq.restype = ip
    lib.fdfd_eigfreq.argtypes = [vp, C.c_double, ip, ip, C.c_double, dp, dp, dp, C.POINTER(Stats)]
    lib.fdfd_batch_create.restype = ip
    lib.fdfd_batch_create.argtypes = [C.POINTER(vp), ip, C.POINTER(vp)]
    lib.fdfd_batch_factor.restype = ip
    lib.fdfd_batch_factor.argtypes = [vp, dp, C.POINTER(C.c_int)]
    lib.fdfd_batch_stats.restype = ip
    lib.fdfd_batch_stats.argtypes = [vp, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong), dp]
    lib.fdfd_batch_last_error.restype = C.c_char_p
    lib.fdfd_batch_last_error.argtypes = [vp]
    lib.fdfd_batch_destroy.restype = None
    lib.fdfd_batch_destroy.argtypes = [vp]
    lib.fdfd_autotune.restype = ip
    lib.fdfd_autotune.argtypes = [vp]
    lib.fdfd_get_tuning.restype = ip
    lib.fdfd_get_tuning.argtypes = [vp, C.c_char_p, ip]
    lib.fdfd_get_stencil.restype = ip
    lib.fdfd_get_stencil.argtypes = [vp, dp]
    lib.fdfd_apply.restype = ip
    lib.fdfd_apply.argtypes = [vp, dp, ip, dp]
    lib.fdfd_set_profiling.restype = ip
    lib.fdfd_set_profiling.argtypes = [vp, ip]
    lib.fdfd_get_profile.restype = ip
    lib.fdfd_get_profile.argtypes = [vp, C.POINTER(Profile)]
    lib.fdfd_residual_noalloc.restype = ip
    lib.fdfd_residual_noalloc.argtypes = [ip, ip, ip, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                          C.c_void_p]
    lib.fdfd_debug_hessenberg_eig.restype = ip
    lib.fdfd_debug_hessenberg_eig.argtypes = [ip, dp, dp, dp]
    lib.fdfd_debug_gemm.restype = ip
    lib.fdfd_debug_gemm.argtypes = [ip, ip, ip, dp, dp, dp, ip, ip, dp]
    _lib = lib
    return lib


def cptr(a: np.ndarray):
    """Pointer to a C-contiguous complex128/float64 array as double*."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"] and a.dtype in (np.complex128, np.float64)
    return a.ctypes.data_as(C.POINTER(C.c_double))


def natural(a: np.ndarray) -> np.ndarray:
    """(..., Nx, Ny) array -> contiguous buffer in the library's x-fastest order."""
    a = np.asarray(a, dtype=np.complex128)
    return np.ascontiguousarray(np.swapaxes(a, -1, -2))


def from_natural(buf: np.ndarray, Nx: int, Ny: int) -> np.ndarray:
    """Inverse of ``natural``: x-fastest buffer holding k*Nx*Ny values -> (k, Nx, Ny)."""
    k = buf.size // (Nx * Ny)
    return np.swapaxes(np.reshape(buf, (k, Ny, Nx)), -1, -2)


class Handle:
    """Owning wrapper of one fdfd_handle (create ... destroy)."""

    def __init__(self, Nx, Ny, Npx, Npy, dx, dy, L0=1e-6, pml_m=3.5, pml_lnR=-12.0, pol=FDFD_TM,
                 precision=FDFD_PREC_MIXED):
        self.lib = load()
        self.h = C.c_void_p()
        rc = self.lib.fdfd_create(C.byref(self.h), int(Nx), int(Ny), int(Npx), int(Npy), float(dx), float(dy),
                                  float(L0), float(pml_m), float(pml_lnR), int(pol), int(precision))
        if rc != FDFD_OK:
            raise FDFDError(rc, "fdfd_create failed")
        self.Nx, self.Ny, self.pol = int(Nx), int(Ny), int(pol)

    def _check(self, rc):
        if rc != FDFD_OK:
            raise FDFDError(rc, self.lib.fdfd_last_error(self.h).decode())

    def close(self):
        if self.h:
            self.lib.fdfd_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
        return False

    def set_refinement(self, tol=1e-10, max_iter=40, mode=FDFD_REFINE_GMRES):
        self._check(self.lib.fdfd_set_refinement(self.h, float(tol), int(max_iter), int(mode)))

    def set_restart(self, m=0):
        """FGMRES basis length (0: automatic)."""
        self._check(self.lib.fdfd_set_restart(self.h, int(m)))

    def set_fallback(self, on=True):
        """FP64 re-factorization when a MIXED handle's refinement stalls (default on)."""
        self._check(self.lib.fdfd_set_fallback(self.h, int(bool(on))))

    def set_wait_limit(self, ns=0):
        """Pipeline wait limit of the tensor-core GEMM in ns (0: the default, 2 s)."""
        self._check(self.lib.fdfd_set_wait_limit(self.h, int(ns)))

    def set_device_budget(self, nbytes=0):
        """Device bytes the handle may hold (0: no limit); beyond it allocations fail with FDFD_ENOMEM."""
        self._check(self.lib.fdfd_set_device_budget(self.h, int(nbytes)))

    def autotune(self):
        """Time the candidate launch shapes of this handle's GEMMs and sweep products and keep the
        fastest; overwrites the factor storage.  Returns the record of the choices (text)."""
        self._check(self.lib.fdfd_autotune(self.h))
        return self.tuning()

    def tuning(self):
        n = self.lib.fdfd_get_tuning(self.h, None, 0)
        buf = C.create_string_buffer(n + 1)
        self.lib.fdfd_get_tuning(self.h, buf, n + 1)
        return buf.value.decode()

    def set_checkpoint(self, mode=0):
        """Block factors in pinned host memory: 0 automatic (default), 1 always, -1 never."""
        self._check(self.lib.fdfd_set_checkpoint(self.h, int(mode)))

    def checkpoint_info(self):
        a, hb, cb = C.c_int(0), C.c_longlong(0), C.c_longlong(0)
        self._check(self.lib.fdfd_checkpoint_info(self.h, C.byref(a), C.byref(hb), C.byref(cb)))
        return {"active": bool(a.value), "host_bytes": hb.value, "copied_bytes": cb.value}

    def set_eps(self, eps):
        buf = natural(eps)
        self._check(self.lib.fdfd_set_eps(self.h, cptr(buf)))

    def factor(self, omega):
        self._check(self.lib.fdfd_factor(self.h, float(omega)))

    def solve(self, src, fields=3):
        """src (nrhs, Nx, Ny) or (Nx, Ny) -> (f1, f2, f3, stats) arrays shaped like src."""
        src = np.asarray(src, dtype=np.complex128)
        single = src.ndim == 2
        s3 = src[None] if single else src
        nrhs = s3.shape[0]
        buf = natural(s3)
        outs = [np.empty_like(buf) if i < fields else None for i in range(3)]
        st = Stats()
        self._check(self.lib.fdfd_solve(self.h, cptr(buf), nrhs, cptr(outs[0]), cptr(outs[1]), cptr(outs[2]),
                                        C.byref(st)))
        res = [from_natural(o, self.Nx, self.Ny) if o is not None else None for o in outs]
        if single:
            res = [r[0] if r is not None else None for r in res]
        return res[0], res[1], res[2], st

    def adjoint(self, src, mvec):
        """Gradient of J = |Σ m·Ez|² w.r.t. real ϵᵣ -> (J, grad (Nx, Ny), Ez (Nx, Ny), stats)."""
        s = natural(src)
        m = natural(mvec)
        grad = np.empty((self.Ny, self.Nx), dtype=np.float64)
        ez = np.empty_like(s)
        J = C.c_double(0)
        st = Stats()
        self._check(self.lib.fdfd_adjoint(self.h, cptr(s), cptr(m), C.byref(J), cptr(grad), cptr(ez), C.byref(st)))
        return J.value, grad.T.copy(), from_natural(ez, self.Nx, self.Ny)[0], st

    def adjoint_vjp(self, src, g):
        """Pullback of Ez = solve(ϵᵣ) for the conjugated cotangent g = conj(ΔEz):
        -> (grad (Nx, Ny) = -Re(ω²ϵ₀ λ⊙E) with λ = A⁻ᵀ g, Ez (Nx, Ny), stats)."""
        s = natural(src)
        gv = natural(g)
        grad = np.empty((self.Ny, self.Nx), dtype=np.float64)
        ez = np.empty_like(s)
        st = Stats()
        self._check(self.lib.fdfd_adjoint_vjp(self.h, cptr(s), cptr(gv), cptr(grad), cptr(ez), C.byref(st)))
        return grad.T.copy(), from_natural(ez, self.Nx, self.Ny)[0], st

    def eigfreq(self, omega0, nev, which=0, tol=1e-10):
        """Shift-invert eigenfrequencies -> (omega[nev], lambda[nev], fields (nev, 3, Nx, Ny), stats)."""
        N = self.Nx * self.Ny
        om = np.empty(nev, dtype=np.complex128)
        lam = np.empty(nev, dtype=np.complex128)
        flds = np.empty((nev, 3, N), dtype=np.complex128)
        st = Stats()
        self._check(self.lib.fdfd_eigfreq(self.h, float(omega0), int(nev), int(which), float(tol), cptr(om),
                                          cptr(lam), cptr(flds), C.byref(st)))
        f = np.stack([np.stack([from_natural(flds[i, c], self.Nx, self.Ny)[0] for c in range(3)])
                      for i in range(nev)])
        return om, lam, f, st

    def get_mode(self, omega, pol, normal, ix, iy, width, neff):
        """Guided mode of the slice -> (beta (complex), vector (npts,) complex)."""
        m = Mode(int(pol), int(normal), int(ix), int(iy), float(width), float(np.real(neff)), float(np.imag(neff)))
        vec = np.empty(FDFD_MODE_MAX_POINTS, dtype=np.complex128)
        beta = np.empty(1, dtype=np.complex128)
        npts = C.c_int(0)
        self._check(self.lib.fdfd_get_mode(self.h, float(omega), C.byref(m), vec.size, cptr(beta), cptr(vec),
                                           C.byref(npts)))
        return complex(beta[0]), vec[:npts.value].copy()

    def mode_sources(self, omegas, modes):
        """modes: sequence of (pol, normal, ix, iy, width, neff) -> src (nw, Nx, Ny) complex."""
        om = np.ascontiguousarray(np.atleast_1d(np.asarray(omegas, dtype=np.float64)))
        arr = (Mode * len(modes))(*[Mode(int(p), int(nrm), int(ix), int(iy), float(w), float(np.real(n)),
                                         float(np.imag(n))) for p, nrm, ix, iy, w, n in modes])
        out = np.empty(om.size * self.Nx * self.Ny, dtype=np.complex128)
        self._check(self.lib.fdfd_mode_sources(self.h, om.size, cptr(om), len(modes), arr, cptr(out)))
        return from_natural(out, self.Nx, self.Ny)

    def poynting(self, pol, f1, f2, f3):
        """(Sx, Sy), each (Nx, Ny), of the field (f1, f2, f3)."""
        b = [natural(f) for f in (f1, f2, f3)]
        Sx = np.empty((self.Ny, self.Nx), dtype=np.float64)
        Sy = np.empty_like(Sx)
        self._check(self.lib.fdfd_poynting(self.h, int(pol), *[cptr(x) for x in b], cptr(Sx), cptr(Sy)))
        return Sx.T.copy(), Sy.T.copy()

    def flux_integral(self, pol, f1, f3, lines, normal=FDFD_X):
        """x̂-normal line integrals; lines: sequence of (xind, iy0, iy1) -> array of fluxes."""
        b1, b3 = natural(f1), natural(f3)
        ln = np.ascontiguousarray(np.asarray(lines, dtype=np.int32).reshape(-1, 3))
        out = np.empty(ln.shape[0], dtype=np.float64)
        self._check(self.lib.fdfd_flux_integral(self.h, int(pol), cptr(b1), cptr(b3), int(normal), ln.shape[0],
                                                ln.ctypes.data_as(C.POINTER(C.c_int)), cptr(out)))
        return out

    def chi3_solve(self, chi, src, method=FDFD_CHI3_NEWTON, tol=1e-12, maxit=50):
        """χ³ solve of the factored TM operator -> (Ez, Hx, Hy, err history, stats)."""
        c = np.ascontiguousarray(np.asarray(chi, dtype=np.float64).T)
        b = natural(src)
        outs = [np.empty_like(b) for _ in range(3)]
        err = np.empty(maxit + 1, dtype=np.float64)
        nerr = C.c_int(0)
        st = Stats()
        self._check(self.lib.fdfd_chi3_solve(self.h, cptr(c), cptr(b), int(method), float(tol), int(maxit),
                                             *[cptr(o) for o in outs], cptr(err), C.byref(nerr), C.byref(st)))
        f = [from_natural(o, self.Nx, self.Ny)[0] for o in outs]
        return f[0], f[1], f[2], err[:min(nerr.value, maxit + 1)].copy(), st

    def set_profiling(self, on=True):
        self._check(self.lib.fdfd_set_profiling(self.h, 1 if on else 0))

    def profile(self):
        p = Profile()
        self._check(self.lib.fdfd_get_profile(self.h, C.byref(p)))
        return p.as_dict()

    def solve_device(self, d_src: int, nrhs: int, d_f1: int, d_f2: int, d_f3: int):
        """fdfd_solve_device on raw device pointers (ints); returns Stats."""
        st = Stats()
        self._check(self.lib.fdfd_solve_device(self.h, C.c_void_p(d_src), int(nrhs), C.c_void_p(d_f1),
                                               C.c_void_p(d_f2), C.c_void_p(d_f3), C.byref(st)))
        return st

    def stencil(self):
        out = np.empty((5, self.Ny, self.Nx), dtype=np.complex128)
        self._check(self.lib.fdfd_get_stencil(self.h, cptr(out)))
        return np.swapaxes(out, 1, 2)

    def apply(self, x):
        x = np.asarray(x, dtype=np.complex128)
        single = x.ndim == 2
        x3 = x[None] if single else x
        buf = natural(x3)
        out = np.empty_like(buf)
        self._check(self.lib.fdfd_apply(self.h, cptr(buf), x3.shape[0], cptr(out)))
        y = from_natural(out, self.Nx, self.Ny)
        return y[0] if single else y


class ModulatedHandle(Handle):
    """Owning wrapper of a modulated-device handle (fdfd_mf_create): K = 2s+1
    coupled sidebands, TM (solve(d::ModulatedDevice), modulation.jl:35-119)."""

    def __init__(self, Nx, Ny, Npx, Npy, dx, dy, nsidebands, L0=1e-6, pml_m=3.5, pml_lnR=-12.0,
                 shared_pml=True, precision=FDFD_PREC_MIXED):
        self.lib = load()
        self.h = C.c_void_p()
        rc = self.lib.fdfd_mf_create(C.byref(self.h), int(Nx), int(Ny), int(Npx), int(Npy), float(dx), float(dy),
                                     float(L0), float(pml_m), float(pml_lnR), int(nsidebands),
                                     1 if shared_pml else 0, int(precision))
        if rc != FDFD_OK:
            raise FDFDError(rc, "fdfd_mf_create failed")
        self.Nx, self.Ny, self.pol = int(Nx), int(Ny), FDFD_TM
        self.K = 2 * int(nsidebands) + 1

    def set_deps(self, deps):
        buf = natural(deps)
        self._check(self.lib.fdfd_mf_set_deps(self.h, cptr(buf)))

    def factor(self, omega, Omega):
        self._check(self.lib.fdfd_mf_factor(self.h, float(omega), float(Omega)))

    def solve(self, src):
        """src (Nx, Ny) -> (Ez, Hx, Hy, stats), each field (K, Nx, Ny), sideband n = -s..s."""
        buf = natural(src)
        outs = [np.empty(self.K * self.Nx * self.Ny, dtype=np.complex128) for _ in range(3)]
        st = Stats()
        self._check(self.lib.fdfd_mf_solve(self.h, cptr(buf), cptr(outs[0]), cptr(outs[1]), cptr(outs[2]),
                                           C.byref(st)))
        f = [from_natural(o, self.Nx, self.Ny) for o in outs]
        return f[0], f[1], f[2], st

    def apply(self, x):
        """Coupled operator product: x (K, Nx, Ny) -> y (K, Nx, Ny)."""
        buf = natural(x)
        out = np.empty_like(buf)
        self._check(self.lib.fdfd_apply(self.h, cptr(buf), 1, cptr(out)))
        return from_natural(out, self.Nx, self.Ny)


def hessenberg_eig(H):
    """Eigenvalues and unit eigenvectors of a complex upper Hessenberg matrix (host QR in the library)."""
    lib = load()
    H = np.ascontiguousarray(H, dtype=np.complex128)
    n = H.shape[0]
    w = np.empty(n, dtype=np.complex128)
    V = np.empty((n, n), dtype=np.complex128)
    rc = lib.fdfd_debug_hessenberg_eig(n, cptr(H), cptr(w), cptr(V))
    if rc != FDFD_OK:
        raise FDFDError(rc, "fdfd_debug_hessenberg_eig failed")
    return w, V


def debug_gemm(A, B, precision=FDFD_PREC_MIXED, use_tc=1):
    """C = A @ B.T through the library's block GEMM kernels (returns C, kernel ms)."""
    lib = load()
    A = np.ascontiguousarray(A, dtype=np.complex128)
    B = np.ascontiguousarray(B, dtype=np.complex128)
    M, K = A.shape
    N = B.shape[0]
    Cm = np.empty((M, N), dtype=np.complex128)
    ms = C.c_double(0)
    rc = lib.fdfd_debug_gemm(M, N, K, cptr(A), cptr(B), cptr(Cm), int(precision), int(use_tc), C.byref(ms))
    if rc != FDFD_OK:
        raise FDFDError(rc, "fdfd_debug_gemm failed")
    return Cm, ms.value


class Batch:
    """Handles factored together: one CUDA graph launch per fdfd_batch_factor after the first
    call (which factors them one by one and captures the graph).  The handles must outlive it."""

    def __init__(self, handles):
        self.lib = load()
        self.handles = list(handles)
        self.b = C.c_void_p()
        arr = (C.c_void_p * len(self.handles))(*[h.h for h in self.handles])
        rc = self.lib.fdfd_batch_create(C.byref(self.b), len(self.handles), arr)
        if rc != FDFD_OK:
            raise FDFDError(rc, "fdfd_batch_create failed")

    def factor(self, omegas):
        """Factor handle i at omegas[i]; returns the per-handle status codes (raises on error)."""
        om = np.ascontiguousarray(np.asarray(omegas, dtype=np.float64))
        if om.size != len(self.handles):
            raise ValueError("one frequency per handle")
        st = (C.c_int * len(self.handles))()
        rc = self.lib.fdfd_batch_factor(self.b, om.ctypes.data_as(C.POINTER(C.c_double)), st)
        if rc != FDFD_OK:
            raise FDFDError(rc, self.lib.fdfd_batch_last_error(self.b).decode())
        return list(st)

    def stats(self):
        k, n, ms = C.c_longlong(0), C.c_longlong(0), C.c_double(0)
        self.lib.fdfd_batch_stats(self.b, C.byref(k), C.byref(n), C.byref(ms))
        return {"graph_kernels": k.value, "graph_launches": n.value, "last_graph_ms": ms.value}

    def close(self):
        if self.b:
            self.lib.fdfd_batch_destroy(self.b)
            self.b = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
        return False
