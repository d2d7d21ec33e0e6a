"""CPU checks of the C ABI: the library builds, loads and exports every symbol
that include/fdfd_cuda.h declares; argument validation needs no GPU."""
import ctypes as C
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "fdfd_cuda.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(fdfd_[a-z_0-9]+)\s*\(", text)))


def test_header_matches_binding(fdfd):
    assert declared_functions() == sorted(fdfd._lib.EXPORTS)


def test_library_exports_every_declared_symbol(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_version(lib):
    assert lib.fdfd_version().decode().startswith("fdfd_cuda")


def test_create_rejects_bad_arguments_without_touching_the_gpu(lib, fdfd):
    h = C.c_void_p()
    args = dict(Nx=20, Ny=16, Npx=2, Npy=2, dx=0.05, dy=0.05, L0=1e-6, m=4.0, lnR=-18.4, pol=1, prec=1)

    def create(**kw):
        a = dict(args, **kw)
        return lib.fdfd_create(C.byref(h), a["Nx"], a["Ny"], a["Npx"], a["Npy"], a["dx"], a["dy"], a["L0"],
                               a["m"], a["lnR"], a["pol"], a["prec"])

    E = fdfd._lib.FDFD_EINVAL
    assert create(Nx=2) == E          # the ring needs at least three lines
    assert create(Ny=0) == E
    assert create(Npx=11) == E        # PML wider than half the grid
    assert create(dx=0.0) == E
    assert create(pol=3) == E
    assert create(prec=7) == E
    assert create(m=float("nan")) == E
    assert lib.fdfd_create(None, 20, 16, 2, 2, 0.05, 0.05, 1e-6, 4.0, -18.4, 1, 1) == E


def test_null_handle_calls_fail_cleanly(lib, fdfd):
    E = fdfd._lib.FDFD_EINVAL
    assert lib.fdfd_set_eps(None, None) == E
    assert lib.fdfd_factor(None, 1.0) == E
    assert lib.fdfd_solve(None, None, 1, None, None, None, None) == E
    assert lib.fdfd_set_refinement(None, 1e-10, 10, 0) == E
    assert lib.fdfd_set_fallback(None, 1) == E
    assert lib.fdfd_set_restart(None, 20) == E
    lib.fdfd_destroy(None)


def test_extension_entry_points_reject_bad_arguments(lib, fdfd):
    """The modulated-device, mode, flux and χ³ entry points validate their
    arguments before any device work (no GPU needed)."""
    import ctypes as C
    L = fdfd._lib
    E = L.FDFD_EINVAL
    h = C.c_void_p()
    assert lib.fdfd_mf_create(None, 40, 30, 4, 4, 0.05, 0.05, 1e-6, 4.0, -18.4, 1, 1, 1) == E
    assert lib.fdfd_mf_create(C.byref(h), 40, 30, 4, 4, 0.05, 0.05, 1e-6, 4.0, -18.4, -1, 1, 1) == E   # sidebands
    assert lib.fdfd_mf_create(C.byref(h), 40, 30, 4, 4, 0.05, 0.05, 1e-6, 4.0, -18.4, 17, 1, 1) == E   # K > 33
    assert lib.fdfd_mf_set_deps(None, None) == E
    assert lib.fdfd_mf_factor(None, 1.0, 0.1) == E
    assert lib.fdfd_mf_solve(None, None, None, None, None, None) == E
    m = L.Mode(1, 1, 5, 5, 0.5, 3.0, 0.0)
    beta = (C.c_double * 2)()
    npts = C.c_int(0)
    assert lib.fdfd_get_mode(None, 1.0, C.byref(m), 0, beta, beta, C.byref(npts)) == E
    assert lib.fdfd_mode_sources(None, 1, beta, 1, C.byref(m), beta) == E
    assert lib.fdfd_poynting(None, 1, None, None, None, None, None) == E
    assert lib.fdfd_poynting_device(None, 1, None, None, None, None, None) == E
    assert lib.fdfd_flux_integral(None, 1, None, None, 1, 1, None, None) == E
    assert lib.fdfd_chi3_solve(None, None, None, 1, 1e-12, 10, None, None, None, None, None, None) == E

