"""GPU parity of the Poynting flux and its line integral (src/flux.jl)
through the C ABI against the FP64 oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def solved(fdfd, oracle, pol):
    from fdfd_gb300 import workloads as W
    p = W.design_guide(160, 100, design=(40, 30), seed=13, npml=12)
    g = oracle.Grid((p.Nx, p.Ny), p.npml, ((0.0, -0.5 * p.Ny * p.dy), (p.Nx * p.dx, 0.5 * p.Ny * p.dy)))
    f = oracle.solve(g, p.eps, p.src, p.omega, pol, p.pml_m, p.pml_lnR)
    h = fdfd._lib.Handle(p.Nx, p.Ny, p.npml[0], p.npml[1], p.dx, p.dy, 1e-6, p.pml_m, p.pml_lnR, pol,
                         fdfd.FDFD_PREC_MIXED)
    return g, f, h


@pytest.mark.parametrize("pol", [1, 2])
def test_poynting_matches_oracle(lib, fdfd, oracle, pol):
    g, f, h = solved(fdfd, oracle, pol)
    Sx, Sy = h.poynting(pol, *f)
    h.close()
    rx, ry = oracle.poynting(*f, pol)
    assert np.linalg.norm(Sx - rx) <= 1e-14 * np.linalg.norm(rx)
    assert np.linalg.norm(Sy - ry) <= 1e-14 * np.linalg.norm(ry)


@pytest.mark.parametrize("pol", [1, 2])
def test_flux_integral_matches_oracle(lib, fdfd, oracle, pol):
    g, f, h = solved(fdfd, oracle, pol)
    centers = [(1.0, 0.0, 0.4), (3.0, 0.1, 0.8), (6.0, -0.2, 0.3), (g.xc()[-2], 0.0, 10.0)]
    lines, ref = [], []
    for cx, cy, w in centers:
        x, rows = oracle.flux_line_indices(g, (cx, cy), w)
        lines.append((x, rows[0], rows[-1]))
        ref.append(oracle.flux_surface_integral(g, f[0], f[2], pol, (cx, cy), w, oracle.X))
    got = h.flux_integral(pol, f[0], f[2], lines)
    h.close()
    assert np.allclose(got, ref, rtol=1e-12, atol=1e-14 * max(abs(r) for r in ref))


def test_poynting_device_pointers(lib, fdfd, oracle):
    """fdfd_poynting_device on device-resident fields (no host copies)."""
    torch = pytest.importorskip("torch")
    g, f, h = solved(fdfd, oracle, 1)
    dev = [torch.from_numpy(np.ascontiguousarray(x.T).view(np.float64)).cuda() for x in f]
    Sx = torch.empty(g.N[1], g.N[0], dtype=torch.float64, device="cuda")
    Sy = torch.empty_like(Sx)
    rc = h.lib.fdfd_poynting_device(h.h, 1, *[d.data_ptr() for d in dev], Sx.data_ptr(), Sy.data_ptr())
    h._check(rc)
    rx, ry = oracle.poynting(*f, 1)
    h.close()
    assert np.linalg.norm(Sx.cpu().numpy().T - rx) <= 1e-14 * np.linalg.norm(rx)
    assert np.linalg.norm(Sy.cpu().numpy().T - ry) <= 1e-14 * np.linalg.norm(ry)


def test_host_mirror_flux(lib, fdfd, oracle):
    """poynting(field) and flux_surface_integral(field, ...) of the host mirror."""
    g = fdfd.Grid(0.05, (10, 10), (0.0, 6.0), (-2.0, 2.0))
    d = fdfd.Device(g, 2 * np.pi * 200e12)
    fdfd.setup_eps(d, lambda x, y: abs(y) <= 0.15, 12.0)
    fdfd.setup_src(d, fdfd.Point(1.0, 0.0))
    field = fdfd.solve(d, fdfd.TM)
    fl = fdfd.poynting(field)
    rx, ry = oracle.poynting(field["Ez"], field["Hx"], field["Hy"], 1)
    assert np.allclose(fl.Sx, rx, rtol=1e-13, atol=1e-14 * np.abs(rx).max())
    og = oracle.Grid(g.N, g.Npml, g.bounds)
    v = fdfd.flux_surface_integral(field, fdfd.Point(4.0, 0.0), 0.5, fdfd.X)
    ref = oracle.flux_surface_integral(og, field["Ez"], field["Hy"], 1, (4.0, 0.0), 0.5, oracle.X)
    assert np.isclose(v, ref, rtol=1e-12)
    with pytest.raises(fdfd.FDFDError):
        fdfd.flux_surface_integral(field, fdfd.Point(4.0, 0.0), 0.5, fdfd.Y)


def test_flux_errors(lib, fdfd, oracle):
    g, f, h = solved(fdfd, oracle, 1)
    E = fdfd._lib.FDFD_EINVAL
    for lines, normal in [([(159, 0, 10)], 1), ([(5, 20, 10)], 1), ([(5, 0, 100)], 1), ([(5, 0, 10)], 2)]:
        with pytest.raises(fdfd.FDFDError) as e:
            h.flux_integral(1, f[0], f[2], lines, normal)
        assert e.value.code == E
    h.close()
