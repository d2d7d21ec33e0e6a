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
