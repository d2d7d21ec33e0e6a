"""Batched factorizations in one CUDA graph (fdfd_batch_*), through the C ABI.

Handles of uneven sizes, both polarizations and both precisions are factored
together: the first fdfd_batch_factor factors them one by one and captures the
graph, later calls replay it with new frequencies.  After each batch call every
handle must solve exactly as after its own fdfd_factor at that frequency.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_RES = 1e-10


def rel(a, b):
    return float(np.linalg.norm(np.ravel(a - b)) / np.linalg.norm(np.ravel(b)))


def problems():
    from fdfd_gb300 import workloads as W
    return [(W.design_guide(96, 64, design=(24, 24), seed=3, npml=10), 1, 1),      # TM mixed
            (W.design_guide(70, 130, design=(30, 30), seed=4, npml=10), 1, 0),     # TM FP64, transposed layout
            (W.design_guide(80, 80, design=(32, 32), seed=5, npml=10), 2, 1),      # TE mixed
            (W.point_source_guide(200, 120), 1, 1)]                                 # the plain 200 x 120 problem


def make(fdfd, p, pol, prec):
    h = fdfd._lib.Handle(p.Nx, p.Ny, p.npml[0], p.npml[1], p.dx, p.dy, 1e-6, p.pml_m, p.pml_lnR, pol, prec)
    h.set_refinement(TOL_RES, 60)
    h.set_eps(p.eps)
    return h


def test_batch_graph_matches_individual_factorizations(lib, fdfd):
    L = fdfd._lib
    from fdfd_gb300 import workloads as W
    probs = problems()
    hs = [make(fdfd, p, pol, prec) for p, pol, prec in probs]
    refs = [make(fdfd, p, pol, prec) for p, pol, prec in probs]
    batch = L.Batch(hs)
    for call, lam in enumerate((1.55, 1.50, 1.62)):
        om = [W.omega_of(lam + 0.01 * i) for i in range(len(hs))]
        assert batch.factor(om) == [0] * len(hs)
        st = batch.stats()
        if call == 0:
            assert st["graph_launches"] == 0 and st["graph_kernels"] > 100 * len(hs)
        else:
            assert st["graph_launches"] == call and st["last_graph_ms"] > 0
        for i, (p, pol, prec) in enumerate(probs):
            f1, f2, f3, s1 = hs[i].solve(p.src)
            refs[i].factor(om[i])
            g1, g2, g3, s2 = refs[i].solve(p.src)
            assert s1.rel_residual <= TOL_RES and s2.rel_residual <= TOL_RES
            tol = 1e-9 if prec == 1 else 1e-11
            assert max(rel(f1, g1), rel(f2, g2), rel(f3, g3)) <= tol, (call, i)
    # a new permittivity on one handle is picked up by the next replay
    p0 = probs[0][0]
    e2 = p0.eps.copy()
    e2[40:50, 20:30] = 4.0
    hs[0].set_eps(e2)
    refs[0].set_eps(e2)
    om = [W.omega_of(1.58)] * len(hs)
    batch.factor(om)
    f1, _, _, _ = hs[0].solve(p0.src)
    refs[0].factor(om[0])
    g1, _, _, _ = refs[0].solve(p0.src)
    assert rel(f1, g1) <= 1e-9
    batch.close()
    for h in hs + refs:
        h.close()


def test_batch_rejects_bad_arguments(lib, fdfd):
    import ctypes as C
    L = fdfd._lib
    p, pol, prec = problems()[0]
    h = make(fdfd, p, pol, prec)
    arr = (C.c_void_p * 2)(h.h, h.h)
    b = C.c_void_p()
    assert lib.fdfd_batch_create(C.byref(b), 2, arr) == L.FDFD_EINVAL    # a handle twice
    batch = L.Batch([h])
    with pytest.raises(fdfd.FDFDError) as e:
        batch.factor([-1.0])
    assert e.value.code == L.FDFD_EINVAL
    batch.close()
    h.close()


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_autotune_records_choices_and_keeps_results(lib, fdfd, oracle, prec):
    """The autotuner times every GEMM shape (tensor-core path) and sweep product of the plan, keeps
    the fastest launch shapes, and the handle then factors and solves to the oracle's field."""
    from fdfd_gb300 import workloads as W
    p = W.design_guide(160, 96, design=(40, 40), seed=6, npml=12)
    P = fdfd.FDFD_PREC_MIXED if prec == "mixed" else fdfd.FDFD_PREC_FP64
    h = make(fdfd, p, 1, P)
    log = h.autotune()
    assert "gemv" in log and (("gemm" in log) == (prec == "mixed")), log
    for line in log.splitlines():
        assert "->" in line and "ms" in line
    h.factor(p.omega)
    f1, f2, f3, st = h.solve(p.src)
    h.close()
    g = oracle.Grid((p.Nx, p.Ny), p.npml, ((0.0, 0.0), (p.Nx * p.dx, p.Ny * p.dy)))
    ref = oracle.solve(g, p.eps, p.src, p.omega, oracle.TM, p.pml_m, p.pml_lnR)
    tol = 1e-8 if prec == "mixed" else 1e-10
    assert st.rel_residual <= TOL_RES
    assert max(rel(f1, ref[0]), rel(f2, ref[1]), rel(f3, ref[2])) <= tol


def test_mirror_solve_batches_frequencies(lib, fdfd):
    """solve(d, TM, frequencies_per_launch=4) on a device with six frequencies (one graph wave
    of four, a short wave of two) gives the fields of the frequency-by-frequency solve."""
    g = fdfd.Grid(0.05, (10, 10), (-3.0, 3.0), (-2.0, 2.0))
    lams = np.linspace(1.45, 1.65, 6)
    d = fdfd.Device(g, [2 * np.pi * 299792458.0 / (l * 1e-6) for l in lams])
    fdfd.setup_eps(d, lambda x, y: abs(y) < 0.25, 12.25)
    fdfd.setup_src(d, fdfd.Point(-2.0, 0.0))
    ref = fdfd.solve(d, fdfd.TM)
    got, st = fdfd.solve(d, fdfd.TM, frequencies_per_launch=4, autotune=True, return_stats=True)
    assert len(got) == 6
    for a, b in zip(got, ref):
        for c in ("Ez", "Hx", "Hy"):
            assert rel(a[c], b[c]) <= 1e-8
    assert max(s["rel_residual"] for s in st) <= TOL_RES


def test_factor_graph_replay_matches_plain_factorization(lib, fdfd, monkeypatch):
    """fdfd_factor captures its own work on the second consecutive factorization at one ω and
    replays it afterwards (ϵᵣ read from device memory): the fields equal those of plain launches
    bit for bit, also after a new permittivity, and a new ω falls back to plain launches.  New
    launch shapes (autotune) drop the graph; the tuner's timing-based choices can differ between
    the two runs, so that last step is compared to rounding."""
    from fdfd_gb300 import workloads as W
    p = W.design_guide(160, 96, design=(40, 40), seed=9, npml=12)
    e2 = p.eps.copy()
    e2[60:80, 40:60] = 3.0

    def runs(graph):
        monkeypatch.setenv("FDFD_FACTOR_GRAPH", "1" if graph else "0")
        h = make(fdfd, p, 1, fdfd.FDFD_PREC_MIXED)
        out = []
        for eps, om in ((p.eps, p.omega), (p.eps, p.omega), (p.eps, p.omega), (e2, p.omega),
                        (e2, p.omega * 1.02), (e2, p.omega)):
            h.set_eps(eps)
            h.factor(om)
            out.append(h.solve(p.src)[:3])
        h.autotune()
        h.factor(p.omega)
        out.append(h.solve(p.src)[:3])
        h.close()
        return out

    plain, graph = runs(False), runs(True)
    for k, (a, b) in enumerate(zip(plain, graph)):
        for x, y in zip(a, b):
            if k < 6:
                assert np.array_equal(x, y), (k, rel(x, y))
            else:   # after autotune: the two runs' timing-based choices may differ (split-K, tiles)
                assert rel(x, y) <= 1e-9, (k, rel(x, y))
