"""GPU parity of the guided-mode solver and the mode sources
(get_modes / setup_mode!, src/device.jl:112-149; eigenmode, src/solver/eigen.jl:6-29)
through the C ABI against the FP64 oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

W0 = 2 * np.pi * 299792458.0 / 1.55e-6


def guide_problem(oracle, Nx=120, Ny=90, dh=0.02, rng_seed=0):
    g = oracle.Grid((Nx, Ny), (10, 10), ((0.0, 0.0), (Nx * dh, Ny * dh)))
    eps = np.ones((Nx, Ny), complex)
    eps[:, Ny // 2 - 6:Ny // 2 + 5] = 12.25               # guide along x
    eps[Nx // 2 - 5:Nx // 2 + 6, :] = 11.0                # guide along y
    rng = np.random.default_rng(rng_seed)
    eps[70:90, 10:30] = rng.uniform(1, 12, (20, 20)) + 1j * rng.uniform(0, 0.3, (20, 20))
    return g, eps


def handle(fdfd, g, eps):
    h = fdfd._lib.Handle(g.N[0], g.N[1], g.Npml[0], g.Npml[1], g.dx(), g.dy(), 1e-6, 4.0, np.log(1e-8), fdfd.TM,
                         fdfd.FDFD_PREC_MIXED)
    h.set_eps(eps)
    return h


def phase_aligned(v, ref):
    k = np.argmax(np.abs(ref))
    return v * (ref[k] / v[k]) / abs(ref[k] / v[k])


CASES = [  # pol, normal, ix, iy, width, neff
    (1, 1, 12, 45, 0.8, 3.5),       # TM, slice across the x-guide
    (2, 1, 12, 45, 0.8, 3.0),       # TE, same slice
    (1, 2, 60, 8, 0.7, 3.3),        # TM, slice across the y-guide
    (2, 2, 60, 80, 1.1, 2.9),       # TE, wider slice
    (1, 1, 80, 20, 0.34, 2.0 + 0.05j),   # lossy random region, complex n_eff guess
    (2, 2, 78, 19, 0.3, 1.5),
]


@pytest.mark.parametrize("case", CASES)
def test_get_mode_matches_oracle(lib, fdfd, oracle, case):
    g, eps = guide_problem(oracle)
    pol, normal, ix, iy, width, neff = case
    h = handle(fdfd, g, eps)
    beta, v = h.get_mode(W0, pol, normal, ix, iy, width, neff)
    h.close()
    b_ref, v_ref, _, _ = oracle.get_modes(g, eps, pol, W0, neff, 1, ix, iy, normal, width)
    v_ref = v_ref[:, 0] / np.linalg.norm(v_ref[:, 0])
    assert v.shape == v_ref.shape
    assert abs(beta - b_ref[0]) <= 1e-10 * abs(b_ref[0])
    assert np.isclose(np.linalg.norm(v), 1.0, rtol=1e-12)
    assert np.linalg.norm(phase_aligned(v, v_ref) - v_ref) <= 1e-8


def test_mode_sources_match_oracle(lib, fdfd, oracle):
    """Several frequencies, two modes each (one TM slice per guide), all in one
    launch; per frequency the source is the sum of normalize(abs.(v))."""
    g, eps = guide_problem(oracle)
    modes = [(1, 1, 12, 45, 0.8, 3.5), (1, 2, 60, 8, 0.7, 3.3)]
    omegas = W0 * np.array([0.9, 1.0, 1.07])
    h = handle(fdfd, g, eps)
    src = h.mode_sources(omegas, modes)
    h.close()
    assert src.shape == (3, g.N[0], g.N[1])
    for k, w in enumerate(omegas):
        ref = np.zeros(g.N, complex)
        for pol, normal, ix, iy, width, neff in modes:
            oracle.setup_mode(ref, g, eps, pol, w, neff, ix, iy, normal, width)
        assert np.linalg.norm(src[k] - ref) <= 1e-9 * np.linalg.norm(ref)


def test_solve_with_mode_source(lib, fdfd, oracle):
    """The reference's waveguide test setup (test/runtests.jl:23-38): a guide
    (ϵᵣ = 12, 0.3 µm wide) driven by a TM mode source at x = 1 µm, solved
    through the host mirror's solve() against the oracle."""
    g = fdfd.Grid(0.02, (15, 15), (0.0, 10.0), (-1.0, 1.0))
    d = fdfd.Device(g, 2 * np.pi * 200e12)
    fdfd.setup_eps(d, lambda x, y: abs(y) <= 0.15, 12.0)
    fdfd.add_mode(d, fdfd.Mode(fdfd.TM, fdfd.X, 3.5, fdfd.Point(1.0, 0.0), 0.8))
    f = fdfd.solve(d, fdfd.TM, precision="mixed")
    og = oracle.Grid(g.N, g.Npml, g.bounds)
    ix, iy = g.coord2ind(fdfd.Point(1.0, 0.0))
    src = np.zeros(g.N, complex)
    oracle.setup_mode(src, og, d.eps, 1, d.omega[0], 3.5, ix, iy, oracle.X, 0.8)
    assert np.linalg.norm(d.src - src) <= 1e-9 * np.linalg.norm(src)
    ref = oracle.solve(og, d.eps, src, d.omega[0], oracle.TM)
    for c, k in enumerate(("Ez", "Hx", "Hy")):
        assert np.linalg.norm(f[k] - ref[c]) <= 1e-8 * np.linalg.norm(ref[c])


def test_mode_errors(lib, fdfd, oracle):
    g, eps = guide_problem(oracle)
    h = handle(fdfd, g, eps)
    E = fdfd._lib.FDFD_EINVAL
    for bad in [(1, 1, 12, 2, 0.8, 3.5),      # slice leaves the grid
                (1, 3, 12, 45, 0.8, 3.5),     # no such normal
                (1, 1, 12, 45, 0.02, 3.5),    # one cell
                (1, 1, 12, 45, 30.0, 3.5)]:   # wider than the grid
        with pytest.raises(fdfd.FDFDError) as e:
            h.get_mode(W0, *bad)
        assert e.value.code == E
    h.close()
