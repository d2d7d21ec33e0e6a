"""Host-side parts of the Python mirror that need no GPU."""
import numpy as np
import pytest


def _field(fdfd, cls):
    g = fdfd.Grid(0.1, (2, 2), (-1.0, 1.0), (0.0, 1.5))       # 20 x 15 cells
    data = (np.arange(g.N[0] * g.N[1] * 3, dtype=np.float64) * (1 + 0.5j)).reshape(g.N[0], g.N[1], 3)
    return g, cls(g, 1.0, data)


def test_probe_field_picks_the_cell_within_half_a_cell(fdfd):
    """probe_field (src/flux.jl:6-12): atvalue with atol = dh/2 on each axis."""
    g, f = _field(fdfd, fdfd.FieldTM)
    ix, iy = 7, 4                                            # centre (-0.25, 0.45)
    pt = fdfd.Point(g.xc()[ix] + 0.04, g.yc()[iy] - 0.049)
    assert fdfd.probe_field(f, "Hx", pt) == f.data[ix, iy, 1]
    assert fdfd.probe_field(f, "Ez", fdfd.Point(g.xc()[0], g.yc()[-1])) == f.data[0, -1, 0]


def test_probe_field_errors_as_the_reference(fdfd):
    g, f = _field(fdfd, fdfd.FieldTE)
    with pytest.raises(fdfd.FDFDError, match="Ez is invalid for the TE polarization. Valid options are :Hz, :Ex, :Ey"):
        fdfd.probe_field(f, "Ez", fdfd.Point(0.0, 0.5))
    assert fdfd.probe_field(f, "Ey", fdfd.Point(0.01, 0.52)) == f.data[10, 5, 2]   # centre (0.05, 0.55)
    with pytest.raises(fdfd.FDFDError):
        fdfd.probe_field(f, "Hz", fdfd.Point(5.0, 0.5))   # outside the grid


def test_grid_and_indices_follow_the_reference(fdfd):
    """Grid (src/grid.jl:26-33), xc/yc (:76-82) and coord2ind (:103-125, clamped, 1-based there)."""
    g = fdfd.Grid(0.05, (20, 20), (-5.0, 5.0), (-3.0, 3.0))
    assert g.N == (200, 120)
    assert np.isclose(g.xc()[0], -5.0 + 0.025) and np.isclose(g.yc()[-1], 3.0 - 0.025)
    assert g.coord2ind(fdfd.Point(-3.0, 0.0)) == (40, 60)
    assert g.coord2ind(fdfd.Point(-99.0, 99.0)) == (0, 119)


def test_grid_edges_and_axis_indices(fdfd):
    """dh, xe/ye (src/grid.jl:63-66, 89-95) and x2ind/y2ind (:112-125)."""
    g = fdfd.Grid(0.1, (2, 2), (-1.0, 1.0), (0.0, 1.5))
    assert g.dh(fdfd.X) == g.dx() and g.dh(fdfd.Y) == g.dy()
    assert len(g.xe()) == g.N[0] + 1 and np.isclose(g.xe()[-1], 1.0)
    assert len(g.ye()) == g.N[1] + 1 and np.isclose(g.ye()[0], 0.0)
    assert g.x2ind(-1.0) == 0 and g.x2ind(0.0) == 10 and g.x2ind(7.0) == g.N[0] - 1
    assert g.y2ind(0.26) == 3 and g.y2ind(-3.0) == 0


def test_line_source(fdfd):
    """setup_src!(d, pt, srcnormal) (src/device.jl:101-108): 1im on the grid line normal to srcnormal."""
    g = fdfd.Grid(0.1, (2, 2), (-1.0, 1.0), (0.0, 1.5))
    d = fdfd.Device(g, 1e15)
    fdfd.setup_src(d, fdfd.Point(-0.5, 0.7), fdfd.X)
    ix, iy = g.coord2ind(fdfd.Point(-0.5, 0.7))
    assert np.all(d.src[ix, :] == 1j) and np.count_nonzero(d.src) == g.N[1]
    d2 = fdfd.Device(g, 1e15)
    fdfd.setup_src(d2, fdfd.Point(-0.5, 0.7), fdfd.Y)
    assert np.all(d2.src[:, iy] == 1j) and np.count_nonzero(d2.src) == g.N[0]


def test_unwrap_follows_the_reference_loop(fdfd):
    """unwrap (src/FDFD.jl:19-31): shifts by 2π against the already unwrapped previous entry."""
    import math
    v = np.array([0.0, 3.0, -3.0, 0.5, 3.1416, -3.1416])
    u = fdfd.unwrap(v)
    assert np.all(v == np.array([0.0, 3.0, -3.0, 0.5, 3.1416, -3.1416]))   # not in place
    # 0.5 - 3.28 > -π: no shift at index 3, as the reference's loop decides it
    assert np.allclose(u, [0.0, 3.0, -3.0 + 2 * math.pi, 0.5, 3.1416, -3.1416 + 2 * math.pi])
    assert np.all(np.abs(np.diff(u)) < math.pi)
    w = v.copy()
    assert fdfd.unwrap(w, True) is w and np.allclose(w, u)


def test_handle_is_a_context_manager(fdfd):
    """`with Handle(...)` releases the library handle on exit (a closed handle is a NULL pointer)."""
    H = fdfd._lib.Handle
    assert hasattr(H, "__enter__") and hasattr(H, "__exit__")
    h = H.__new__(H)               # no GPU here: exercise the protocol on an unopened handle
    import ctypes
    h.h = ctypes.c_void_p()
    h.lib = None
    with h as same:
        assert same is h
    assert not h.h
