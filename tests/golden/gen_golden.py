"""Generate the golden fixtures under tests/golden/ with the FP64 oracle.

Each fixture is a small seeded problem (inputs and oracle outputs) so that the
GPU tests compare against stored FP64 answers and the CPU tests pin the oracle
against regressions.  Run: python tests/golden/gen_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, ROOT)
import __graft_entry__  # noqa: E402

__graft_entry__.load_package()
import fdfd_oracle as O  # noqa: E402
from fdfd_gb300 import workloads as W  # noqa: E402


def grid_of(p):
    return O.Grid((p.Nx, p.Ny), p.npml, ((0.0, 0.0), (p.Nx * p.dx, p.Ny * p.dy)))


def stencil_from_csc(A, Nx, Ny):
    A = A.tocsr()
    N = Nx * Ny
    idx = np.arange(N)
    ix, iy = idx % Nx, idx // Nx
    out = []
    for di, dj in [(0, 0), (-1, 0), (1, 0), (0, -1), (0, 1)]:
        col = ((ix + di) % Nx) + Nx * ((iy + dj) % Ny)
        out.append(np.asarray(A[idx, col]).ravel())
    return np.stack(out)   # (5, N), natural order


def driven_case(name, p, pol):
    g = grid_of(p)
    f, A, b = O.solve(g, p.eps, p.src, p.omega, pol, p.pml_m, p.pml_lnR, return_system=True)
    st = stencil_from_csc(A, p.Nx, p.Ny)
    # the five periodic diagonals hold every entry of A
    assert np.isclose(abs(A).sum(), np.abs(st).sum(), rtol=1e-12)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), Nx=p.Nx, Ny=p.Ny, npml=np.array(p.npml), dx=p.dx,
                        dy=p.dy, omega=p.omega, pml_m=p.pml_m, pml_lnR=p.pml_lnR, pol=pol, eps=p.eps, src=p.src,
                        f1=f[0], f2=f[1], f3=f[2], stencil=st)


def eigen_case(name, p, omega0, pol, nev):
    g = grid_of(p)
    w, fields, lam = O.eigenfrequency(g, p.eps, omega0, pol, nev, "LM", p.pml_m, p.pml_lnR,
                                      v0=np.ones(p.Nx * p.Ny, dtype=complex))
    _, sigma = O.eigen_operator(g, p.eps, omega0, pol, p.pml_m, p.pml_lnR)
    order = np.argsort(np.abs(lam - sigma))
    np.savez_compressed(os.path.join(HERE, name + ".npz"), Nx=p.Nx, Ny=p.Ny, npml=np.array(p.npml), dx=p.dx,
                        dy=p.dy, omega0=omega0, pml_m=p.pml_m, pml_lnR=p.pml_lnR, pol=pol, eps=p.eps,
                        omega=w[order], lam=lam[order])


def modulated_case(name, p):
    g = grid_of(p)
    e = p.extra
    out = O.solve_modulated(g, p.eps, e["deps"], p.src, p.omega, e["Omega"], e["nsidebands"], e["sharedpml"],
                            p.pml_m, p.pml_lnR)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), Nx=p.Nx, Ny=p.Ny, npml=np.array(p.npml), dx=p.dx,
                        dy=p.dy, omega=p.omega, Omega=e["Omega"], nsidebands=e["nsidebands"],
                        sharedpml=e["sharedpml"], pml_m=p.pml_m, pml_lnR=p.pml_lnR, eps=p.eps, deps=e["deps"],
                        src=p.src, ez=np.stack([o[0] for o in out]))


def main():
    driven_case("tm_point_guide_60x40", W.point_source_guide(60, 40, npml=8), O.TM)
    driven_case("tm_design_48x72", W.design_guide(48, 72, design=(16, 20), seed=7, npml=8), O.TM)
    driven_case("te_design_64x40", W.design_guide(64, 40, design=(20, 12), seed=11, npml=8), O.TE)
    p, w0 = W.phc_cavity(n_cells=5, res=8, npml=8)
    eigen_case("tm_phc_eigen_56", p, w0, O.TM, 4)
    modulated_case("tm_modulated_125x50", W.modulated_waveguide(dh=0.04, nsidebands=1))
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
