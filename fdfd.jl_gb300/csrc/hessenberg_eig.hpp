// Eigen-decomposition of a small complex upper Hessenberg matrix (host code).
//
// Used for the Ritz pairs of the shift-invert Arnoldi iteration of
// fdfd_eigfreq.  Complex single-shift QR iteration with Wilkinson shifts and
// deflation on the Hessenberg form, accumulating the Schur vectors, followed
// by back-substitution for the eigenvectors of the triangular Schur factor
// (the textbook algorithm of Golub & Van Loan, Matrix Computations, §7.5).
#pragma once
#include <cmath>
#include <complex>
#include <vector>

namespace hess {

typedef std::complex<double> zc;

// H: n x n row-major upper Hessenberg (entries below the subdiagonal ignored).
// On success w[i] holds the eigenvalues and V (n x n row-major, column i)
// the unit-norm eigenvector of w[i].  Returns false if the QR iteration did
// not converge within 60 n sweeps.
inline bool eig(int n, const std::vector<zc>& H, std::vector<zc>& w, std::vector<zc>& V) {
    std::vector<zc> T(H), Z((size_t)n * n, zc(0, 0));
    auto t = [&](int i, int j) -> zc& { return T[(size_t)i * n + j]; };
    auto z = [&](int i, int j) -> zc& { return Z[(size_t)i * n + j]; };
    for (int i = 0; i < n; ++i) {
        z(i, i) = 1;
        for (int j = 0; j + 1 < i; ++j) t(i, j) = 0;
    }
    double hnorm = 0;
    for (auto& v : T) hnorm = std::max(hnorm, std::abs(v));
    const double eps = 2.220446049250313e-16;
    int hi = n - 1, its = 0, total = 0;
    while (hi > 0) {
        int l = hi;
        while (l > 0) {
            double s = std::abs(t(l - 1, l - 1)) + std::abs(t(l, l));
            if (s == 0) s = hnorm;
            if (std::abs(t(l, l - 1)) <= eps * s) break;
            --l;
        }
        if (l == hi) {            // 1x1 block converged
            if (hi > 0) t(hi, hi - 1) = 0;
            --hi;
            its = 0;
            continue;
        }
        if (l > 0) t(l, l - 1) = 0;
        if (++total > 60 * n) return false;
        // Wilkinson shift from the trailing 2x2 of the active block, exceptional shift every 10 sweeps
        zc shift;
        const zc a = t(hi - 1, hi - 1), b = t(hi - 1, hi), c = t(hi, hi - 1), d = t(hi, hi);
        if (its > 0 && its % 10 == 0) {
            shift = d + zc(std::abs(c.real()) + std::abs(t(hi - 1, std::max(hi - 2, 0)).real()), 0);
        } else {
            const zc hm = 0.5 * (a - d);
            const zc disc = std::sqrt(hm * hm + b * c);
            const zc m1 = 0.5 * (a + d) + disc, m2 = 0.5 * (a + d) - disc;
            shift = std::abs(m1 - d) < std::abs(m2 - d) ? m1 : m2;
        }
        ++its;
        zc x = t(l, l) - shift, y = t(l + 1, l);
        for (int k = l; k < hi; ++k) {
            // Givens G = [[c, s], [-conj(s), c]] with G·[x; y] = [r; 0]
            const double ax = std::abs(x), r = std::hypot(ax, std::abs(y));
            double cs;
            zc sn;
            if (r == 0) { cs = 1; sn = 0; }
            else if (ax == 0) { cs = 0; sn = 1; }
            else { cs = ax / r; sn = (x / ax) * std::conj(y) / r; }
            for (int j = (k > l ? k - 1 : l); j < n; ++j) {     // rows k, k+1
                const zc t1 = t(k, j), t2 = t(k + 1, j);
                t(k, j) = cs * t1 + sn * t2;
                t(k + 1, j) = -std::conj(sn) * t1 + cs * t2;
            }
            const int rmax = std::min(k + 2, hi);
            for (int i = 0; i <= rmax; ++i) {                   // columns k, k+1 (times Gᴴ)
                const zc t1 = t(i, k), t2 = t(i, k + 1);
                t(i, k) = cs * t1 + std::conj(sn) * t2;
                t(i, k + 1) = -sn * t1 + cs * t2;
            }
            for (int i = 0; i < n; ++i) {                       // Schur vectors Z·Gᴴ
                const zc z1 = z(i, k), z2 = z(i, k + 1);
                z(i, k) = cs * z1 + std::conj(sn) * z2;
                z(i, k + 1) = -sn * z1 + cs * z2;
            }
            if (k + 1 < hi) { x = t(k + 1, k); y = t(k + 2, k); }
        }
    }
    w.resize(n);
    for (int i = 0; i < n; ++i) w[i] = t(i, i);
    // eigenvectors of the triangular Schur factor, then back to H's basis
    V.assign((size_t)n * n, zc(0, 0));
    const double small = eps * std::max(hnorm, 1e-300);
    std::vector<zc> xv(n);
    for (int i = 0; i < n; ++i) {
        for (int j = 0; j < n; ++j) xv[j] = 0;
        xv[i] = 1;
        for (int j = i - 1; j >= 0; --j) {
            zc s = 0;
            for (int k = j + 1; k <= i; ++k) s += t(j, k) * xv[k];
            zc den = t(j, j) - w[i];
            if (std::abs(den) < small) den = small;
            xv[j] = -s / den;
        }
        double nrm = 0;
        for (int r = 0; r < n; ++r) {
            zc acc = 0;
            for (int k = 0; k <= i; ++k) acc += z(r, k) * xv[k];
            V[(size_t)r * n + i] = acc;
            nrm += std::norm(acc);
        }
        nrm = std::sqrt(nrm);
        if (nrm > 0)
            for (int r = 0; r < n; ++r) V[(size_t)r * n + i] /= nrm;
    }
    return true;
}

}  // namespace hess
