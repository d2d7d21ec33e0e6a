// Guided modes of 1-D grid slices and the mode sources built from them.
//
// The reference computes a mode source per frequency before each driven solve
// (src/solver/driven.jl:15-19): get_modes (src/device.jl:124-149) cuts the ϵᵣ
// slice of a Mode, eigenmode (src/solver/eigen.jl:6-29) builds the periodic 1-D
// operator
//   TM: A = ω²μ₀Tϵ + δxf δxb            TE: A = ω²μ₀Tϵ + Tϵ δxf Tϵxinv δxb
// and ARPACK's shift-invert `eigs(A, nev=1, sigma=(ω n_eff/c₀)²)` returns the
// eigenpair nearest the shift; setup_mode! (device.jl:118-121) adds
// normalize(abs.(v)) to the source on the slice.
//
// Here every (frequency, mode) pair is one job of one warp, in FP64, all in
// shared memory:
//  * A − σI = T0 + a0·e_0·e_{n-1}ᵀ + cN·e_{n-1}·e_0ᵀ with T0 tridiagonal.  Lane 0
//    factors T0 with partial pivoting (the recurrences of LAPACK's xGTTRF);
//    lanes 0 and 1 solve T0 z0 = e_0, T0 zN = e_{n-1}; the periodic corners are
//    handled by the Sherman-Morrison-Woodbury identity with the 2x2 capacitance
//    matrix S = I + [[a0 z0[n-1], cN zN[n-1]], [a0 z0[0], cN zN[0]]].
//  * Inverse iteration with the fixed shift σ converges to the eigenvector of
//    the eigenvalue nearest σ — the pair ARPACK's shift-invert mode returns for
//    nev = 1.  Each step: lane 0 runs the two triangular recurrences, the warp
//    applies the Woodbury correction, normalises, forms the Rayleigh quotient
//    λ = yᴴAy and the residual ||Ay − λy||.  The loop stops when the residual
//    reaches 1e-13·||A||, or stagnates below 1e-9·||A||, within 4000 steps.
//  * β = √λ (principal branch, Julia's `sqrt`), the vector scaled to unit norm
//    with its largest entry real and positive (ARPACK's phase is arbitrary; the
//    source uses |v| only).
#include "common.cuh"
#include "kernels.cuh"

namespace {

__device__ __forceinline__ cplx<double> csqrt_principal(cplx<double> z) {
    // principal square root: Re ≥ 0, branch cut on the negative real axis
    const double r = hypot(z.re, z.im);
    if (r == 0.0) return cmk(0.0, 0.0);
    if (z.re >= 0.0) {
        const double t = sqrt(0.5 * (r + z.re));
        return cmk(t, z.im / (2.0 * t));
    }
    const double t = sqrt(0.5 * (r - z.re));
    return cmk(fabs(z.im) / (2.0 * t), copysign(t, z.im));
}

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

}  // namespace

// Shared memory per job (nmax = largest slice): 11 complex arrays and the pivots.
size_t mode_smem_bytes(int nmax) { return (size_t)nmax * (11 * sizeof(cplx<double>) + sizeof(int)); }

__global__ void __launch_bounds__(32) mode_kernel(const ModeJob* __restrict__ jobs, int nmax,
                                                  const cplx<double>* __restrict__ eps, double eps0n, double mu0n,
                                                  cplx<double>* __restrict__ beta, cplx<double>* __restrict__ vecs,
                                                  int* __restrict__ iters, unsigned* err) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const ModeJob J = jobs[blockIdx.x];
    const int n = J.n;
    const int lane = threadIdx.x;
    cplx<double>* lo = reinterpret_cast<cplx<double>*>(smem_raw);   // A[i][i-1] (periodic)
    cplx<double>* dg = lo + nmax;                                    // A[i][i]
    cplx<double>* up = dg + nmax;                                    // A[i][i+1] (periodic)
    cplx<double>* dl = up + nmax;                                    // xGTTRF factors of T0
    cplx<double>* du = dl + nmax;
    cplx<double>* du2 = du + nmax;
    cplx<double>* dinv = du2 + nmax;
    cplx<double>* z0 = dinv + nmax;
    cplx<double>* zN = z0 + nmax;
    cplx<double>* x = zN + nmax;
    cplx<double>* y = x + nmax;
    int* ipiv = reinterpret_cast<int*>(y + nmax);
    const cplx<double> zero = cmk(0.0, 0.0), one = cmk(1.0, 0.0);
    const cplx<double> sig = cmk(J.sig_re, J.sig_im);
    const double h2 = 1.0 / (J.dh * J.dh);
    const double w2mu = J.omega * J.omega * mu0n;

    // ---- the 1-D operator (eigen.jl:16-21) ----
    for (int i = lane; i < n; i += 32) {
        const cplx<double> e = eps[J.k0 + (long long)i * J.stride];
        const cplx<double> te = cscale(e, eps0n);                                 // Tϵ_i
        if (J.pol == 1) {
            lo[i] = cmk(h2, 0.0);
            up[i] = cmk(h2, 0.0);
            dg[i] = cadd(cscale(te, w2mu), cmk(-2.0 * h2, 0.0));
        } else {
            // Tϵxinv_i = 1/(ϵ₀(ϵ_i + ϵ_{i-1})/2), periodic (grid_average, 1-D)
            const int im = i == 0 ? n - 1 : i - 1, ip = i + 1 == n ? 0 : i + 1;
            const cplx<double> em = eps[J.k0 + (long long)im * J.stride];
            const cplx<double> ep = eps[J.k0 + (long long)ip * J.stride];
            const cplx<double> ti = cinv(cscale(cadd(e, em), 0.5 * eps0n));
            const cplx<double> tp = cinv(cscale(cadd(ep, e), 0.5 * eps0n));
            up[i] = cscale(cmul(te, tp), h2);
            lo[i] = cscale(cmul(te, ti), h2);
            dg[i] = csub(cscale(te, w2mu), cadd(up[i], lo[i]));
        }
    }
    __syncwarp();
    // ||A||_inf for the stopping rule
    double an = 0.0;
    for (int i = lane; i < n; i += 32) an = fmax(an, cabs1(lo[i]) + cabs1(dg[i]) + cabs1(up[i]));
    for (int o = 16; o > 0; o >>= 1) an = fmax(an, __shfl_xor_sync(0xffffffffu, an, o));
    // T0 = A − σI without the corners: diagonal in dinv, T0[i+1][i] in dl, T0[i][i+1] in du
    for (int i = lane; i < n; i += 32) {
        dinv[i] = csub(dg[i], sig);
        dl[i] = i + 1 < n ? lo[i + 1] : zero;
        du[i] = i + 1 < n ? up[i] : zero;
        du2[i] = zero;
    }
    __syncwarp();
    int bad = 0;
    if (lane == 0) {
        cplx<double> d = dinv[0];
        for (int i = 0; i + 1 < n; ++i) {
            cplx<double> l = dl[i];
            cplx<double> dn = dinv[i + 1];
            const cplx<double> u = du[i];
            int ip = i;
            if (cabs1(d) >= cabs1(l)) {
                cplx<double> f = zero;
                if (cabs1(d) > 0.0) {
                    f = cmul(l, cinv(d));
                    dn = csub(dn, cmul(f, u));
                }
                l = f;
            } else {
                const cplx<double> f = cmul(d, cinv(l));
                d = l;
                du[i] = dn;
                dn = csub(u, cmul(f, dn));
                if (i + 2 < n) {
                    du2[i] = du[i + 1];
                    du[i + 1] = cneg(cmul(f, du[i + 1]));
                }
                l = f;
                ip = i + 1;
            }
            if (!(cabs1(d) > 0.0) || !isfinite(cabs1(d))) { bad = 1; d = one; }
            dl[i] = l;
            dinv[i] = cinv(d);
            ipiv[i] = ip;
            d = dn;
        }
        if (!(cabs1(d) > 0.0) || !isfinite(cabs1(d))) { bad = 1; d = one; }
        dl[n - 1] = zero;
        du[n - 1] = zero;
        dinv[n - 1] = cinv(d);
        ipiv[n - 1] = n - 1;
    }
    bad = __shfl_sync(0xffffffffu, bad, 0);
    __syncwarp();
    // T0 v = e solved in place (L with the neighbour interchanges, then U)
    auto t0_solve = [&](cplx<double>* v) {
        for (int i = 0; i + 1 < n; ++i) {
            if (ipiv[i] == i) {
                v[i + 1] = csub(v[i + 1], cmul(dl[i], v[i]));
            } else {
                const cplx<double> t = v[i];
                v[i] = v[i + 1];
                v[i + 1] = csub(t, cmul(dl[i], v[i]));
            }
        }
        cplx<double> v1 = cmul(v[n - 1], dinv[n - 1]), v2 = zero;
        v[n - 1] = v1;
        for (int i = n - 2; i >= 0; --i) {
            const cplx<double> vi = cmul(csub(csub(v[i], cmul(du[i], v1)), cmul(du2[i], v2)), dinv[i]);
            v[i] = vi;
            v2 = v1;
            v1 = vi;
        }
    };
    for (int i = lane; i < n; i += 32) {
        z0[i] = i == 0 ? one : zero;
        zN[i] = i == n - 1 ? one : zero;
    }
    __syncwarp();
    if (lane < 2) t0_solve(lane == 0 ? z0 : zN);
    __syncwarp();
    const cplx<double> a0 = lo[0];        // A[0][n-1]
    const cplx<double> cN = up[n - 1];    // A[n-1][0]
    const cplx<double> s00 = cadd(one, cmul(a0, z0[n - 1])), s01 = cmul(cN, zN[n - 1]);
    const cplx<double> s10 = cmul(a0, z0[0]), s11 = cadd(one, cmul(cN, zN[0]));
    const cplx<double> det = csub(cmul(s00, s11), cmul(s01, s10));
    if (!(cabs1(det) > 0.0) || !isfinite(cabs1(det))) bad = 1;
    const cplx<double> idet = bad ? zero : cinv(det);
    // start vector: deterministic, no symmetry in i (reaches odd and even modes)
    for (int i = lane; i < n; i += 32) {
        const double t = (double)i;
        x[i] = cmk(1.0 + 0.37 * sin(1.7 * t + 0.3) + 0.11 * cos(0.23 * t * t), 0.29 * cos(2.3 * t + 0.1));
    }
    __syncwarp();
    cplx<double> lam = zero;
    double res = 0.0, prev = 1e300;
    int it = 0, conv = 0, flat = 0;
    const int kMaxIter = 4000;
    for (; !bad && it < kMaxIter; ++it) {
        for (int i = lane; i < n; i += 32) y[i] = x[i];
        __syncwarp();
        if (lane == 0) t0_solve(y);
        __syncwarp();
        // Woodbury: y -= [a0 z0, cN zN] S⁻¹ [y[n-1], y[0]]
        const cplx<double> r0 = y[n - 1], r1 = y[0];
        const cplx<double> c0 = cmul(idet, csub(cmul(s11, r0), cmul(s01, r1)));
        const cplx<double> c1 = cmul(idet, csub(cmul(s00, r1), cmul(s10, r0)));
        __syncwarp();
        double nn = 0.0;
        for (int i = lane; i < n; i += 32) {
            const cplx<double> v = csub(csub(y[i], cmul(cmul(c0, a0), z0[i])), cmul(cmul(c1, cN), zN[i]));
            y[i] = v;
            nn += v.re * v.re + v.im * v.im;
        }
        nn = warp_sum(nn);
        if (!(nn > 0.0) || !isfinite(nn)) { bad = 1; break; }
        const double inv = 1.0 / sqrt(nn);
        for (int i = lane; i < n; i += 32) y[i] = cscale(y[i], inv);
        __syncwarp();
        // λ = yᴴ A y and ||A y − λ y||
        double qr = 0.0, qi = 0.0;
        for (int i = lane; i < n; i += 32) {
            const int im = i == 0 ? n - 1 : i - 1, ip = i + 1 == n ? 0 : i + 1;
            const cplx<double> w = cadd(cadd(cmul(lo[i], y[im]), cmul(dg[i], y[i])), cmul(up[i], y[ip]));
            const cplx<double> yc = cmk(y[i].re, -y[i].im);
            const cplx<double> p = cmul(yc, w);
            qr += p.re;
            qi += p.im;
            x[i] = w;   // A y, kept for the residual
        }
        lam = cmk(warp_sum(qr), warp_sum(qi));
        __syncwarp();
        double rr = 0.0;
        for (int i = lane; i < n; i += 32) {
            const cplx<double> r = csub(x[i], cmul(lam, y[i]));
            rr += r.re * r.re + r.im * r.im;
            x[i] = y[i];
        }
        res = sqrt(warp_sum(rr));
        __syncwarp();
        if (res <= 1e-13 * an) { conv = 1; ++it; break; }
        flat = res >= 0.98 * prev ? flat + 1 : 0;
        if (flat >= 8 && res <= 1e-9 * an) { conv = 1; ++it; break; }
        prev = fmin(prev, res);
    }
    if (bad && lane == 0) dev_error(err, FDFD_DEVERR_SINGULAR);
    // phase: largest entry real and positive
    double best = -1.0;
    int bi = 0;
    for (int i = lane; i < n; i += 32) {
        const double m = x[i].re * x[i].re + x[i].im * x[i].im;
        if (m > best) { best = m; bi = i; }
    }
    for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
    }
    const cplx<double> pk = x[bi];
    const double pm = sqrt(pk.re * pk.re + pk.im * pk.im);
    const cplx<double> ph = pm > 0.0 ? cmk(pk.re / pm, -pk.im / pm) : one;
    for (int i = lane; i < n; i += 32) vecs[J.out_off + i] = cmul(x[i], ph);
    if (lane == 0) {
        beta[blockIdx.x] = csqrt_principal(lam);
        iters[blockIdx.x] = conv ? it : -it;
    }
}

// Mode sources (device.jl:118-121, driven.jl:15-19): src[w] = Σ over the modes of
// frequency w of |v| on the slice (v has unit norm, so |v| is normalize(abs.(v))).
// One block per frequency; modes are added in order, a block-wide barrier
// between modes (slices may overlap).
__global__ void mode_src_kernel(const ModeJob* __restrict__ jobs, const int* __restrict__ job_start,
                                const cplx<double>* __restrict__ vecs, long long N, cplx<double>* __restrict__ src) {
    const int w = blockIdx.x;
    cplx<double>* s = src + (size_t)w * N;
    for (int j = job_start[w]; j < job_start[w + 1]; ++j) {
        const ModeJob J = jobs[j];
        for (int i = threadIdx.x; i < J.n; i += blockDim.x) {
            const cplx<double> v = vecs[J.out_off + i];
            const long long k = J.k0 + (long long)i * J.stride;
            s[k] = cadd(s[k], cmk(sqrt(v.re * v.re + v.im * v.im), 0.0));
        }
        __syncthreads();
    }
}

int launch_modes(cudaStream_t s, int njobs, int nmax, const ModeJob* jobs, const cplx<double>* eps, double eps0n,
                 double mu0n, cplx<double>* beta, cplx<double>* vecs, int* iters, unsigned* err) {
    const size_t smem = mode_smem_bytes(nmax);
    static const cudaError_t attr =
        cudaFuncSetAttribute(mode_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)mode_smem_bytes(FDFD_MODE_MAX_POINTS));
    if (attr != cudaSuccess) return (int)attr;
    mode_kernel<<<njobs, 32, smem, s>>>(jobs, nmax, eps, eps0n, mu0n, beta, vecs, iters, err);
    return (int)cudaGetLastError();
}

void launch_mode_src(cudaStream_t s, int nw, const ModeJob* jobs, const int* job_start, const cplx<double>* vecs,
                     long long N, cplx<double>* src) {
    mode_src_kernel<<<nw, 256, 0, s>>>(jobs, job_start, vecs, N, src);
}
