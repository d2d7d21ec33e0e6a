// FP64 operator assembly, matrix-free stencil products and field recovery.
//
// The operator is the reference's 5-point FDFD matrix, assembled per unknown
// instead of as sparse products.  Unknown k = ix + Nx*iy (x fastest, the
// column-major `A[:]` ordering of src/solver/driven.jl:21).  All neighbours are
// periodic, exactly as the reference's difference matrices (src/grid.jl:138-151,
// the ±(N-1) corner entries).
#include <algorithm>

#include "common.cuh"
#include "kernels.cuh"

// ---------------------------------------------------------------------------
// 1-D stretch factors, src/pml.jl:1-31 (create_sfactor).  Writes, per axis,
// s (forward/backward) and 1/s (the entries of S_create's diagonals,
// pml.jl:33-63).  Layout of `out`: [sxf | sxb | syf | syb] then the inverses
// [1/sxf | 1/sxb | 1/syf | 1/syb]; each block has Nx or Ny entries.
// ---------------------------------------------------------------------------
__device__ cplx<double> sfactor_value(int i1, int Nw, int Npml, double dw, bool forward,
                                      double omega, double eps0n, double eta0,
                                      double m, double lnR) {
    // i1 is the 1-based index of the reference loop (pml.jl:14-28).
    if (Npml == 0) return cmk(1.0, 0.0);
    double Tw = Npml * dw;
    double sigmax = -(m + 1) * lnR / (2 * eta0 * Tw);
    double l;
    if (forward) {
        if (i1 <= Npml) l = dw * (Npml - i1 + 0.5);
        else if (i1 > Nw - Npml) l = dw * (i1 - (Nw - Npml) - 0.5);
        else return cmk(1.0, 0.0);
    } else {
        if (i1 <= Npml) l = dw * (Npml - i1 + 1);
        else if (i1 > Nw - Npml) l = dw * (i1 - (Nw - Npml) - 1);
        else return cmk(1.0, 0.0);
    }
    double sig = sigmax * pow(l / Tw, m);
    // S(l) = 1 - 1im*σ(l)/(ω ϵ₀)  (pml.jl:10)
    return cmk(1.0, -(sig / (omega * eps0n)));
}

// the arguments live in device memory, so that a captured factorization is replayed
// for another frequency by rewriting them before the launch
__global__ void sfactor_kernel(const SFactorArgs* __restrict__ pa, cplx<double>* out) {
    const SFactorArgs a = *pa;
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    int tot = 2 * a.Nx + 2 * a.Ny;
    if (t >= tot) return;
    cplx<double> s;
    if (t < a.Nx) s = sfactor_value(t + 1, a.Nx, a.Npx, a.dx, true, a.omega, a.eps0n, a.eta0, a.m, a.lnR);
    else if (t < 2 * a.Nx) s = sfactor_value(t - a.Nx + 1, a.Nx, a.Npx, a.dx, false, a.omega, a.eps0n, a.eta0, a.m, a.lnR);
    else if (t < 2 * a.Nx + a.Ny) s = sfactor_value(t - 2 * a.Nx + 1, a.Ny, a.Npy, a.dy, true, a.omega, a.eps0n, a.eta0, a.m, a.lnR);
    else s = sfactor_value(t - 2 * a.Nx - a.Ny + 1, a.Ny, a.Npy, a.dy, false, a.omega, a.eps0n, a.eta0, a.m, a.lnR);
    out[t] = s;
    out[tot + t] = cinv(s);
}

// ---------------------------------------------------------------------------
// Stencil assembly.  For unknown (ix, iy) writes the five coefficients
// [self, (ix-1,iy), (ix+1,iy), (ix,iy-1), (ix,iy+1)] of the operator selected
// by `op`, evaluated in the order the reference's sparse products evaluate them
// (products without FMA contraction, as Julia does).
//   OP_TM_DRIVEN  A = δxf μ₀⁻¹ δxb + δyf μ₀⁻¹ δyb + ω² Tϵ          driven.jl:35
//   OP_TE_DRIVEN  A = δxf Tϵxi δxb + δyf Tϵyi δyb + ω² μ₀ I         driven.jl:45
//   OP_TM_EIGEN   A = Tϵᵣ⁻¹δxf δxb + Tϵᵣ⁻¹δyf δyb - σ I             eigen.jl:84
//   OP_TE_EIGEN   A = δxf Tϵx⁻¹ δxb + δyf Tϵy⁻¹ δyb - σ I           eigen.jl:102
//   OP_TM_SIDEBAND  Aₙ = Sxb δxb μ₀⁻¹ Sxf δxf + Syb δyb μ₀⁻¹ Syf δyf + ωₙ² Tϵ
//                 (one sideband of a modulated device, modulation.jl:82-90:
//                 backward difference outside, forward inside)
// with δxf = Sxf·δ(x̂,Forward) etc. (driven.jl:28-31) and the Tϵ averages
// of grid_average (grid.jl:157-162).
// ---------------------------------------------------------------------------
__device__ __forceinline__ cplx<double> eps_avg_inv(const cplx<double>* eps, int ix, int iy, int Nx, int Ny,
                                                    bool alongx, double eps0n) {
    // 1 ./ grid_average(ϵ₀ϵᵣ, w): (a + circshift(a, 1 along w))/2, periodic.
    int jx = alongx ? (ix + Nx - 1) % Nx : ix;
    int jy = alongx ? iy : (iy + Ny - 1) % Ny;
    cplx<double> a = cscale_rn(eps[ix + (size_t)Nx * iy], eps0n);
    cplx<double> b = cscale_rn(eps[jx + (size_t)Nx * jy], eps0n);
    cplx<double> s = cadd_rn(a, b);
    s = cmk(s.re / 2, s.im / 2);
    return cinv(s);
}

__global__ void stencil_kernel(const StencilArgs* __restrict__ pa, const cplx<double>* __restrict__ eps,
                               const cplx<double>* __restrict__ sf, cplx<double>* __restrict__ st) {
    const StencilArgs a = *pa;
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long N = (long long)a.Nx * a.Ny;
    if (k >= N) return;
    int ix = (int)(k % a.Nx), iy = (int)(k / a.Nx);
    int ixp = (ix + 1) % a.Nx, iyp = (iy + 1) % a.Ny;
    const int tot = 2 * a.Nx + 2 * a.Ny;
    const cplx<double>* inv = sf + tot;            // 1/s blocks
    cplx<double> sxf = inv[ix], sxb = inv[a.Nx + ix], sxbp = inv[a.Nx + ixp];
    cplx<double> syf = inv[2 * a.Nx + iy], syb = inv[2 * a.Nx + a.Ny + iy],
                 sybp = inv[2 * a.Nx + a.Ny + iyp];
    // backward operator entries: (Sxb δxb)_{i,i} = sxb_i/dx, (.)_{i+1,i} = -sxb_{i+1}/dx
    cplx<double> bx = cscale_rn(sxb, a.idx), bxp = cscale_rn(sxbp, a.idx);
    cplx<double> by = cscale_rn(syb, a.idy), byp = cscale_rn(sybp, a.idy);
    cplx<double> self, cxm, cxp, cym, cyp;
    if (a.op == OP_TM_SIDEBAND) {
        // row i of Sxb δxb μ₀⁻¹ Sxf δxf: (sxb_i/dx)μ₀⁻¹ [sxf_i/dx (v_{i+1} - v_i) - sxf_{i-1}/dx (v_i - v_{i-1})]
        const int ixm = (ix + a.Nx - 1) % a.Nx, iym = (iy + a.Ny - 1) % a.Ny;
        cplx<double> ox = cscale_rn(bx, a.imu0), oy = cscale_rn(by, a.imu0);
        cxp = cmul_rn(ox, cscale_rn(sxf, a.idx));
        cxm = cmul_rn(ox, cscale_rn(inv[ixm], a.idx));
        cyp = cmul_rn(oy, cscale_rn(syf, a.idy));
        cym = cmul_rn(oy, cscale_rn(inv[2 * a.Nx + iym], a.idy));
        cplx<double> sx = cneg(cadd_rn(cxp, cxm)), sy = cneg(cadd_rn(cyp, cym));
        cplx<double> e = cscale_rn(eps[k], a.eps0n);
        self = cadd_rn(cadd_rn(sx, sy), cscale_rn(e, a.omega2));
    } else if (a.op == OP_TM_DRIVEN || a.op == OP_TM_EIGEN) {
        // forward row factor f = (Sxf δxf)_{i,i+1} = sxf_i/dx, times μ₀⁻¹ (driven) or
        // pre-multiplied by ϵᵣ⁻¹ (eigen: Tϵᵣ⁻¹*δxf).
        cplx<double> fx = cscale_rn(sxf, a.idx), fy = cscale_rn(syf, a.idy);
        if (a.op == OP_TM_DRIVEN) {
            fx = cscale_rn(fx, a.imu0);
            fy = cscale_rn(fy, a.imu0);
        } else {
            cplx<double> rinv = cinv(eps[k]);
            fx = cmul_rn(rinv, fx);
            fy = cmul_rn(rinv, fy);
        }
        cplx<double> p1 = cmul_rn(fx, bx), p2 = cmul_rn(fx, bxp);
        cplx<double> q1 = cmul_rn(fy, by), q2 = cmul_rn(fy, byp);
        cxm = p1; cxp = p2; cym = q1; cyp = q2;
        cplx<double> sx = cneg(cadd_rn(p1, p2)), sy = cneg(cadd_rn(q1, q2));
        self = cadd_rn(sx, sy);
        if (a.op == OP_TM_DRIVEN) {
            // ω^2 * (ϵ₀ ϵᵣ)
            cplx<double> e = cscale_rn(eps[k], a.eps0n);
            self = cadd_rn(self, cscale_rn(e, a.omega2));
        } else {
            self = cmk(self.re - a.sigma_re, self.im - a.sigma_im);
        }
    } else {
        // TE: (δxf Tϵxi)_{i,k} = (Sxf δxf)_{i,k} * t_k, then * δxb.
        cplx<double> fx = cscale_rn(sxf, a.idx), fy = cscale_rn(syf, a.idy);
        cplx<double> tx = eps_avg_inv(eps, ix, iy, a.Nx, a.Ny, true, a.eps0n);
        cplx<double> txp = eps_avg_inv(eps, ixp, iy, a.Nx, a.Ny, true, a.eps0n);
        cplx<double> ty = eps_avg_inv(eps, ix, iy, a.Nx, a.Ny, false, a.eps0n);
        cplx<double> typ = eps_avg_inv(eps, ix, iyp, a.Nx, a.Ny, false, a.eps0n);
        cplx<double> p1 = cmul_rn(cmul_rn(fx, tx), bx), p2 = cmul_rn(cmul_rn(fx, txp), bxp);
        cplx<double> q1 = cmul_rn(cmul_rn(fy, ty), by), q2 = cmul_rn(cmul_rn(fy, typ), byp);
        cxm = p1; cxp = p2; cym = q1; cyp = q2;
        cplx<double> sx = cneg(cadd_rn(p1, p2)), sy = cneg(cadd_rn(q1, q2));
        self = cadd_rn(sx, sy);
        if (a.op == OP_TE_DRIVEN) self = cmk(__dadd_rn(self.re, a.omega2mu0), self.im);
        else self = cmk(self.re - a.sigma_re, self.im - a.sigma_im);
    }
    st[k] = self;
    st[N + k] = cxm;
    st[2 * N + k] = cxp;
    st[3 * N + k] = cym;
    st[4 * N + k] = cyp;
}

// ---------------------------------------------------------------------------
// Matrix-free residual r = b - A x (or y = A x when b == nullptr) for nrhs
// stacked vectors, FP64, fused with per-block partial sums of |r|² and |b|².
// One thread per unknown; neighbour loads are periodic in x and y.
// Partial sums go to part[rhs][block][2]; reduce_partials_kernel folds them.
// ---------------------------------------------------------------------------
__global__ void residual_kernel(int Nx, int Ny, int nrhs, const cplx<double>* __restrict__ st,
                                const cplx<double>* __restrict__ x, const cplx<double>* __restrict__ b,
                                cplx<double>* __restrict__ r, double* __restrict__ part) {
    long long N = (long long)Nx * Ny;
    int rhs = blockIdx.y;
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double rr = 0.0, bb = 0.0;
    if (k < N) {
        int ix = (int)(k % Nx), iy = (int)(k / Nx);
        long long kxm = (ix == 0) ? k + Nx - 1 : k - 1;
        long long kxp = (ix == Nx - 1) ? k - (Nx - 1) : k + 1;
        long long kym = (iy == 0) ? k + N - Nx : k - Nx;
        long long kyp = (iy == Ny - 1) ? k - (N - Nx) : k + Nx;
        const cplx<double>* xv = x + (size_t)rhs * N;
        // four FMAs per term: FP64 issue, not HBM, bounds this kernel on this part
        cplx<double> acc = cmul(st[k], xv[k]);
        cmac<false>(acc, st[N + k], xv[kxm]);
        cmac<false>(acc, st[2 * N + k], xv[kxp]);
        cmac<false>(acc, st[3 * N + k], xv[kym]);
        cmac<false>(acc, st[4 * N + k], xv[kyp]);
        if (b) {
            cplx<double> bv = b[(size_t)rhs * N + k];
            acc = csub(bv, acc);
            bb = bv.re * bv.re + bv.im * bv.im;
        }
        rr = acc.re * acc.re + acc.im * acc.im;
        r[(size_t)rhs * N + k] = acc;
    }
    if (!part) return;
    // block reduction (deterministic order)
    __shared__ double s_rr[32], s_bb[32];
    for (int o = 16; o > 0; o >>= 1) {
        rr += __shfl_down_sync(0xffffffffu, rr, o);
        bb += __shfl_down_sync(0xffffffffu, bb, o);
    }
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) { s_rr[w] = rr; s_bb[w] = bb; }
    __syncthreads();
    if (w == 0) {
        int nw = blockDim.x >> 5;
        rr = l < nw ? s_rr[l] : 0.0;
        bb = l < nw ? s_bb[l] : 0.0;
        for (int o = 16; o > 0; o >>= 1) {
            rr += __shfl_down_sync(0xffffffffu, rr, o);
            bb += __shfl_down_sync(0xffffffffu, bb, o);
        }
        if (l == 0) {
            part[((size_t)rhs * gridDim.x + blockIdx.x) * 2 + 0] = rr;
            part[((size_t)rhs * gridDim.x + blockIdx.x) * 2 + 1] = bb;
        }
    }
}

// Residual of the coupled sideband system (modulation.jl:93-101), nrhs = 1:
// r_n = b_n - (A_n x_n + ½ωₙ²ϵ₀ conj(Δϵ)⊙x_{n+1} + ½ωₙ²ϵ₀ Δϵ⊙x_{n-1}); vectors are
// sideband-major (x_n at offset n·Nx·Ny).  Grid (blocks, K); partial sums of
// |r|², |b|² per (sideband, block) in part[n][block][2].
__global__ void residual_mf_kernel(MfResidualArgs a, const cplx<double>* __restrict__ deps,
                                   const cplx<double>* __restrict__ x, const cplx<double>* __restrict__ b,
                                   cplx<double>* __restrict__ r, double* __restrict__ part) {
    const long long N = (long long)a.Nx * a.Ny;
    const int n = blockIdx.y;
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double rr = 0.0, bb = 0.0;
    if (k < N) {
        const int ix = (int)(k % a.Nx), iy = (int)(k / a.Nx);
        const long long kxm = (ix == 0) ? k + a.Nx - 1 : k - 1;
        const long long kxp = (ix == a.Nx - 1) ? k - (a.Nx - 1) : k + 1;
        const long long kym = (iy == 0) ? k + N - a.Nx : k - a.Nx;
        const long long kyp = (iy == a.Ny - 1) ? k - (N - a.Nx) : k + a.Nx;
        const cplx<double>* st = a.st[n];
        const cplx<double>* xv = x + (size_t)n * N;
        // four FMAs per term: FP64 issue, not HBM, bounds this kernel on this part
        cplx<double> acc = cmul(st[k], xv[k]);
        cmac<false>(acc, st[N + k], xv[kxm]);
        cmac<false>(acc, st[2 * N + k], xv[kxp]);
        cmac<false>(acc, st[3 * N + k], xv[kym]);
        cmac<false>(acc, st[4 * N + k], xv[kyp]);
        const cplx<double> d = deps[k];
        const double c = a.half_w2eps0[n];
        if (n + 1 < a.K) acc = cadd(acc, cmul(cmk(c * d.re, -c * d.im), xv[N + k]));
        if (n > 0) acc = cadd(acc, cmul(cmk(c * d.re, c * d.im), xv[k - N]));
        if (b) {
            const cplx<double> bv = b[(size_t)n * N + k];
            acc = csub(bv, acc);
            bb = bv.re * bv.re + bv.im * bv.im;
        }
        rr = acc.re * acc.re + acc.im * acc.im;
        r[(size_t)n * N + k] = acc;
    }
    if (!part) return;
    __shared__ double s_rr[32], s_bb[32];
    for (int o = 16; o > 0; o >>= 1) {
        rr += __shfl_down_sync(0xffffffffu, rr, o);
        bb += __shfl_down_sync(0xffffffffu, bb, o);
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) { s_rr[w] = rr; s_bb[w] = bb; }
    __syncthreads();
    if (w == 0) {
        const int nw = blockDim.x >> 5;
        rr = l < nw ? s_rr[l] : 0.0;
        bb = l < nw ? s_bb[l] : 0.0;
        for (int o = 16; o > 0; o >>= 1) {
            rr += __shfl_down_sync(0xffffffffu, rr, o);
            bb += __shfl_down_sync(0xffffffffu, bb, o);
        }
        if (l == 0) {
            double* p = part + ((size_t)n * gridDim.x + blockIdx.x) * 2;
            p[0] = rr;
            p[1] = bb;
        }
    }
}

// ---------------------------------------------------------------------------
// χ³ systems of the nonlinear driven solve (src/solver/nonlinear.jl:92-129).
// mode 1 (Born): r = b − (A + diag d1) x on one N-vector;
// mode 2 (Newton on the stacked unknown [x1; x2]):
//   r1 = b1 − (A x1 + d1⊙x1 + d2⊙x2),  r2 = b2 − (conj(A) x2 + conj(d2)⊙x1 + conj(d1)⊙x2).
// Grid (blocks, 1 or 2 halves); partial sums of |r|², |b|² per half.
// ---------------------------------------------------------------------------
__global__ void residual_nl_kernel(int Nx, int Ny, int mode, const cplx<double>* __restrict__ st,
                                   const cplx<double>* __restrict__ d1, const cplx<double>* __restrict__ d2,
                                   const cplx<double>* __restrict__ x, const cplx<double>* __restrict__ b,
                                   cplx<double>* __restrict__ r, double* __restrict__ part) {
    const long long N = (long long)Nx * Ny;
    const int half = blockIdx.y;
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double rr = 0.0, bb = 0.0;
    if (k < N) {
        const int ix = (int)(k % Nx), iy = (int)(k / Nx);
        const long long kxm = (ix == 0) ? k + Nx - 1 : k - 1;
        const long long kxp = (ix == Nx - 1) ? k - (Nx - 1) : k + 1;
        const long long kym = (iy == 0) ? k + N - Nx : k - Nx;
        const long long kyp = (iy == Ny - 1) ? k - (N - Nx) : k + Nx;
        const cplx<double>* xs = x + (size_t)half * N;
        const double cj = half ? -1.0 : 1.0;   // conjugate the coefficients in the second half
        auto c = [&](cplx<double> v) { return cmk(v.re, cj * v.im); };
        cplx<double> acc = cmul(c(st[k]), xs[k]);
        acc = cadd(acc, cmul(c(st[N + k]), xs[kxm]));
        acc = cadd(acc, cmul(c(st[2 * N + k]), xs[kxp]));
        acc = cadd(acc, cmul(c(st[3 * N + k]), xs[kym]));
        acc = cadd(acc, cmul(c(st[4 * N + k]), xs[kyp]));
        acc = cadd(acc, cmul(c(d1[k]), xs[k]));
        if (mode == 2) acc = cadd(acc, cmul(c(d2[k]), x[(size_t)(1 - half) * N + k]));
        if (b) {
            const cplx<double> bv = b[(size_t)half * N + k];
            acc = csub(bv, acc);
            bb = bv.re * bv.re + bv.im * bv.im;
        }
        rr = acc.re * acc.re + acc.im * acc.im;
        r[(size_t)half * N + k] = acc;
    }
    if (!part) return;
    __shared__ double s_rr[32], s_bb[32];
    for (int o = 16; o > 0; o >>= 1) {
        rr += __shfl_down_sync(0xffffffffu, rr, o);
        bb += __shfl_down_sync(0xffffffffu, bb, o);
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) { s_rr[w] = rr; s_bb[w] = bb; }
    __syncthreads();
    if (w == 0) {
        const int nw = blockDim.x >> 5;
        rr = l < nw ? s_rr[l] : 0.0;
        bb = l < nw ? s_bb[l] : 0.0;
        for (int o = 16; o > 0; o >>= 1) {
            rr += __shfl_down_sync(0xffffffffu, rr, o);
            bb += __shfl_down_sync(0xffffffffu, bb, o);
        }
        if (l == 0) {
            double* p = part + ((size_t)half * gridDim.x + blockIdx.x) * 2;
            p[0] = rr;
            p[1] = bb;
        }
    }
}

// χ³ diagonals from the field e (coeff = ω²ϵ₀·3χ/L₀, nonlinear.jl:71):
// mode 1: d1 = coeff|e|²;  mode 2 (Newton Jacobian): d1 = 2coeff|e|², d2 = coeff·e².
__global__ void chi3_diag_kernel(long long N, int mode, const double* __restrict__ coeff,
                                 const cplx<double>* __restrict__ e, cplx<double>* __restrict__ d1,
                                 cplx<double>* __restrict__ d2) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= N) return;
    const cplx<double> v = e[k];
    const double c = coeff[k], m2 = v.re * v.re + v.im * v.im;
    if (mode == 1) {
        d1[k] = cmk(c * m2, 0.0);
    } else {
        d1[k] = cmk(2.0 * c * m2, 0.0);
        d2[k] = cmk(c * (v.re * v.re - v.im * v.im), c * 2.0 * v.re * v.im);
    }
}

// out = conj(in)  (n values; in may equal out)
__global__ void vconj_kernel(long long n, const cplx<double>* in, cplx<double>* out) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) out[k] = cmk(in[k].re, -in[k].im);
}

// y += alpha·x  (n values)
__global__ void vaxpy_kernel(long long n, double alpha, const cplx<double>* __restrict__ x,
                             cplx<double>* __restrict__ y) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) y[k] = cmk(y[k].re + alpha * x[k].re, y[k].im + alpha * x[k].im);
}

// out[rhs*nvals + v] = Σ_blocks part[rhs][block][v]   (fixed order: deterministic)
// grid: (nrhs, any number ≤ nvals), block 256
__global__ void reduce_partials_kernel(const double* __restrict__ part, int nblocks, int nvals,
                                       double* __restrict__ out) {
    int rhs = blockIdx.x;
    __shared__ double s[32];
    // values spread over grid y (one value per block when gridDim.y == nvals)
    for (int v = blockIdx.y; v < nvals; v += gridDim.y) {
        double acc = 0.0;
        for (int i = threadIdx.x; i < nblocks; i += blockDim.x)
            acc += part[((size_t)rhs * nblocks + i) * nvals + v];
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        int w = threadIdx.x >> 5, l = threadIdx.x & 31;
        if (l == 0) s[w] = acc;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0;
            for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += s[i];
            out[rhs * nvals + v] = t;
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Field recovery (FP64), following the reference's expression order:
//   REC_TM_DRIVEN  hx = c_x·(δyb ez), hy = c_y·(δxb ez)        driven.jl:40-41
//   REC_TM_EIGEN   hx = c_x·(δyf ez), hy = c_y·(δxf ez)        eigen.jl:90-91
//   REC_TE_DRIVEN  ex = (c·Tϵyi)(δyb hz), ey = (c·Tϵxi)(-δxb hz) driven.jl:50-51
//   REC_TE_EIGEN   ex = (c·Tϵx⁻¹)(δyb hz), ey = (c·Tϵy⁻¹)(-δxb hz) eigen.jl:108-109
// TM: the scalar multiplies the matrix entries before the product (Julia
// evaluates coef*δ first), c_x = -1/1im/ω/μ₀, c_y = 1/1im/ω/μ₀.
// TE: c = 1/1im/ω.  Coefficients are per right-hand side (complex ω for eigen).
// ---------------------------------------------------------------------------
__global__ void recover_kernel(RecoverArgs a, const cplx<double>* __restrict__ sf,
                               const cplx<double>* __restrict__ eps, const cplx<double>* __restrict__ f,
                               const cplx<double>* __restrict__ coef, cplx<double>* __restrict__ g1,
                               cplx<double>* __restrict__ g2) {
    long long N = (long long)a.Nx * a.Ny;
    int rhs = blockIdx.y;
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= N) return;
    int ix = (int)(k % a.Nx), iy = (int)(k / a.Nx);
    const int tot = 2 * a.Nx + 2 * a.Ny;
    const cplx<double>* inv = sf + tot;
    const cplx<double>* fv = f + (size_t)rhs * N;
    cplx<double> c1 = coef[2 * rhs], c2 = coef[2 * rhs + 1];
    cplx<double> v = fv[k];
    if (a.mode == REC_TM_DRIVEN || a.mode == REC_TE_DRIVEN || a.mode == REC_TE_EIGEN) {
        // backward differences: (δb v)_k = s_k/dh (v_k - v_{k-1})
        long long kym = (iy == 0) ? k + N - a.Nx : k - a.Nx;
        long long kxm = (ix == 0) ? k + a.Nx - 1 : k - 1;
        cplx<double> ey = cscale_rn(inv[2 * a.Nx + a.Ny + iy], a.idy);   // syb/dy
        cplx<double> ex = cscale_rn(inv[a.Nx + ix], a.idx);              // sxb/dx
        if (a.mode == REC_TM_DRIVEN) {
            cplx<double> e1 = cmul_rn(c1, ey), e2 = cmul_rn(c2, ex);
            g1[(size_t)rhs * N + k] = cadd_rn(cmul_rn(e1, v), cneg(cmul_rn(e1, fv[kym])));
            g2[(size_t)rhs * N + k] = cadd_rn(cmul_rn(e2, v), cneg(cmul_rn(e2, fv[kxm])));
        } else {
            // TE: d1 = δyb v, d2 = -(δxb v)
            cplx<double> d1 = cadd_rn(cmul_rn(ey, v), cneg(cmul_rn(ey, fv[kym])));
            cplx<double> d2 = cadd_rn(cmul_rn(cneg(ex), v), cmul_rn(ex, fv[kxm]));
            bool drv = (a.mode == REC_TE_DRIVEN);
            cplx<double> t1 = eps_avg_inv(eps, ix, iy, a.Nx, a.Ny, !drv, a.eps0n);  // driven: Tϵyi, eigen: Tϵx⁻¹
            cplx<double> t2 = eps_avg_inv(eps, ix, iy, a.Nx, a.Ny, drv, a.eps0n);   // driven: Tϵxi, eigen: Tϵy⁻¹
            g1[(size_t)rhs * N + k] = cmul_rn(cmul_rn(c1, t1), d1);
            g2[(size_t)rhs * N + k] = cmul_rn(cmul_rn(c1, t2), d2);
        }
    } else {
        // REC_TM_EIGEN: forward differences (δf v)_k = s_k/dh (v_{k+1} - v_k)
        long long kyp = (iy == a.Ny - 1) ? k - (N - a.Nx) : k + a.Nx;
        long long kxp = (ix == a.Nx - 1) ? k - (a.Nx - 1) : k + 1;
        cplx<double> ey = cscale_rn(inv[2 * a.Nx + iy], a.idy);   // syf/dy
        cplx<double> ex = cscale_rn(inv[ix], a.idx);              // sxf/dx
        cplx<double> e1 = cmul_rn(c1, ey), e2 = cmul_rn(c2, ex);
        g1[(size_t)rhs * N + k] = cadd_rn(cneg(cmul_rn(e1, v)), cmul_rn(e1, fv[kyp]));
        g2[(size_t)rhs * N + k] = cadd_rn(cneg(cmul_rn(e2, v)), cmul_rn(e2, fv[kxp]));
    }
}

// ---------------------------------------------------------------------------
// Layout conversion between the natural FP64 layout (x fastest, nrhs stacked)
// and the node-planar layout of the factor sweeps:
//   vec[((node*nrhs + rhs)*2 + plane)*ld + i]
// node j / in-block index i map to (ix, iy) = (i, j), or (j, i) when the
// blocks run along x (transposed layout, b = Ny).
// ---------------------------------------------------------------------------
template <typename T>
__global__ void to_nodes_kernel(NodeMap m, int nrhs, const cplx<double>* __restrict__ in, double scale,
                                T* __restrict__ out) {
    long long N = (long long)m.Nx * m.Ny;
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int rhs = blockIdx.y;
    if (t >= N) return;
    // t enumerates (node, i) with i fastest for coalesced node-planar writes
    int i = (int)(t % m.b), j = (int)(t / m.b);
    long long k = m.transposed ? (long long)j + (long long)m.Nx * i : (long long)i + (long long)m.Nx * j;
    cplx<double> v = in[(size_t)rhs * N + k];
    T* o = out + ((size_t)j * nrhs + rhs) * 2 * m.ld;
    o[i] = (T)(v.re * scale);
    o[m.ld + i] = (T)(v.im * scale);
}

template <typename T>
__global__ void from_nodes_kernel(NodeMap m, int nrhs, const T* __restrict__ in, double scale, int accumulate,
                                  cplx<double>* __restrict__ out) {
    long long N = (long long)m.Nx * m.Ny;
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int rhs = blockIdx.y;
    if (t >= N) return;
    int i = (int)(t % m.b), j = (int)(t / m.b);
    long long k = m.transposed ? (long long)j + (long long)m.Nx * i : (long long)i + (long long)m.Nx * j;
    const T* s = in + ((size_t)j * nrhs + rhs) * 2 * m.ld;
    cplx<double> v = cmk((double)s[i] * scale, (double)s[m.ld + i] * scale);
    if (accumulate) v = cadd(v, out[(size_t)rhs * N + k]);
    out[(size_t)rhs * N + k] = v;
}

template <typename T>
void launch_to_nodes(dim3 grid, cudaStream_t s, NodeMap m, int nrhs, const cplx<double>* in, double scale, T* out) {
    to_nodes_kernel<T><<<grid, 256, 0, s>>>(m, nrhs, in, scale, out);
}
template <typename T>
void launch_from_nodes(dim3 grid, cudaStream_t s, NodeMap m, int nrhs, const T* in, double scale, int accumulate,
                       cplx<double>* out) {
    from_nodes_kernel<T><<<grid, 256, 0, s>>>(m, nrhs, in, scale, accumulate, out);
}
template void launch_to_nodes<float>(dim3, cudaStream_t, NodeMap, int, const cplx<double>*, double, float*);
template void launch_to_nodes<double>(dim3, cudaStream_t, NodeMap, int, const cplx<double>*, double, double*);
template void launch_from_nodes<float>(dim3, cudaStream_t, NodeMap, int, const float*, double, int, cplx<double>*);
template void launch_from_nodes<double>(dim3, cudaStream_t, NodeMap, int, const double*, double, int,
                                        cplx<double>*);

// ---------------------------------------------------------------------------
// Small FP64 vector kernels for the Krylov refinement (natural layout).
// ---------------------------------------------------------------------------
// y[rhs] = x[rhs] * s[rhs]  (complex scalar per rhs), or y = a*x + y with axpy.
__global__ void vscale_kernel(long long N, const cplx<double>* __restrict__ x, const cplx<double>* __restrict__ s,
                              cplx<double>* __restrict__ y) {
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int rhs = blockIdx.y;
    if (k >= N) return;
    y[(size_t)rhs * N + k] = cmul(s[rhs], x[(size_t)rhs * N + k]);
}

template <bool kSub>
__device__ __forceinline__ cplx<double> vcombine_elem(const cplx<double>* __restrict__ V, long long vstride,
                                                      const cplx<double>* __restrict__ c, int nvec, size_t o,
                                                      cplx<double> acc) {
    // the loads of four vectors are issued before their products (the sum keeps its order)
    int j = 0;
    for (; j + 4 <= nvec; j += 4) {
        cplx<double> v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) v[u] = V[(j + u) * vstride + o];
#pragma unroll
        for (int u = 0; u < 4; ++u) cmac<kSub>(acc, c[j + u], v[u]);
    }
    for (; j < nvec; ++j) cmac<kSub>(acc, c[j], V[j * vstride + o]);
    return acc;
}

// y[rhs] += sign Σ_j c[rhs*ldc + j] * V_j[rhs]   (V_j = V + j*vstride, sign = ±1)
__global__ void vcombine_kernel(long long N, int nvec, const cplx<double>* __restrict__ V, long long vstride,
                                const cplx<double>* __restrict__ c, int ldc, double sign,
                                cplx<double>* __restrict__ y) {
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int rhs = blockIdx.y;
    if (k >= N) return;
    const size_t o = (size_t)rhs * N + k;
    const cplx<double>* cr = c + (size_t)rhs * ldc;
    y[o] = sign < 0 ? vcombine_elem<true>(V, vstride, cr, nvec, o, y[o])
                    : vcombine_elem<false>(V, vstride, cr, nvec, o, y[o]);
}

// part[rhs][block][j] = Σ_k conj(V_j[rhs][k]) * w[rhs][k]  for j < nvec (eight vectors per pass)
__global__ void vdots_kernel(long long N, int nvec, const cplx<double>* __restrict__ V, long long vstride,
                             const cplx<double>* __restrict__ w, double* __restrict__ part) {
    int rhs = blockIdx.y;
    __shared__ double s[2][64][9];
    double acc_re[8], acc_im[8];
    int nw = blockDim.x >> 5, wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int j0 = 0; j0 < nvec; j0 += 8) {
        int nj = min(8, nvec - j0);
        for (int j = 0; j < 8; ++j) { acc_re[j] = 0; acc_im[j] = 0; }
        for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < N;
             k += (long long)gridDim.x * blockDim.x) {
            cplx<double> wv = w[(size_t)rhs * N + k];
            for (int j = 0; j < nj; ++j) {
                cplx<double> v = V[(j0 + j) * vstride + (size_t)rhs * N + k];
                // conj(v)·w in four FMAs
                acc_re[j] = fma(v.re, wv.re, acc_re[j]);
                acc_re[j] = fma(v.im, wv.im, acc_re[j]);
                acc_im[j] = fma(v.re, wv.im, acc_im[j]);
                acc_im[j] = fma(-v.im, wv.re, acc_im[j]);
            }
        }
        for (int j = 0; j < nj; ++j)
            for (int o = 16; o > 0; o >>= 1) {
                acc_re[j] += __shfl_down_sync(0xffffffffu, acc_re[j], o);
                acc_im[j] += __shfl_down_sync(0xffffffffu, acc_im[j], o);
            }
        if (lane == 0)
            for (int j = 0; j < nj; ++j) { s[0][wid][j] = acc_re[j]; s[1][wid][j] = acc_im[j]; }
        __syncthreads();
        if (threadIdx.x < nj) {
            double re = 0, im = 0;
            for (int i = 0; i < nw; ++i) { re += s[0][i][threadIdx.x]; im += s[1][i][threadIdx.x]; }
            size_t o = ((size_t)rhs * gridDim.x + blockIdx.x) * (2 * nvec) + 2 * (j0 + threadIdx.x);
            part[o] = re;
            part[o + 1] = im;
        }
        __syncthreads();
    }
}

// y[rhs] = x[rhs] / ‖x[rhs]‖ with ‖x‖² read from nrm[2*rhs] (0 where ‖x‖ ≤ 1e-300)
// (x may be y: each thread reads its element before writing it)
__global__ void vnormalize_kernel(long long N, const cplx<double>* x, const double* __restrict__ nrm,
                                  cplx<double>* y) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int rhs = blockIdx.y;
    // one FP64 square root and division per block (both are long FP64 sequences)
    __shared__ double sc;
    if (threadIdx.x == 0) {
        const double hn = sqrt(fmax(0.0, nrm[2 * rhs]));
        sc = hn > 1e-300 ? 1.0 / hn : 0.0;
    }
    __syncthreads();
    if (k >= N) return;
    const cplx<double> v = x[(size_t)rhs * N + k];
    y[(size_t)rhs * N + k] = cmk(sc * v.re, sc * v.im);
}

// Adjoint helpers (TM): v = P⁻¹ g  or  v = P g with P_k = s_xf[ix]·s_yf[iy]
// (the unstretched s-factors; P·A is complex symmetric).  mode 0: multiply by
// P⁻¹, mode 1: multiply by P.
__global__ void pscale_kernel(int Nx, int Ny, const cplx<double>* __restrict__ sf, int mode,
                              const cplx<double>* __restrict__ in, cplx<double>* __restrict__ out) {
    long long N = (long long)Nx * Ny;
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= N) return;
    int ix = (int)(k % Nx), iy = (int)(k / Nx);
    const int tot = 2 * Nx + 2 * Ny;
    cplx<double> p = mode ? cmul(sf[ix], sf[2 * Nx + iy]) : cmul(sf[tot + ix], sf[tot + 2 * Nx + iy]);
    out[k] = cmul(p, in[k]);
}

// grad_k = -2 Re(conj(s) ω²ϵ₀ λ_k E_k);  s = mᵀE supplied by the host.
__global__ void adjoint_grad_kernel(long long N, cplx<double> coef, const cplx<double>* __restrict__ lam,
                                    const cplx<double>* __restrict__ E, double* __restrict__ grad) {
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= N) return;
    cplx<double> t = cmul(coef, cmul(lam[k], E[k]));
    grad[k] = -2.0 * t.re;
}

// part[block][0..1] = Σ m_k E_k (no conjugation)
__global__ void vdotu_kernel(long long N, const cplx<double>* __restrict__ m, const cplx<double>* __restrict__ E,
                             double* __restrict__ part) {
    double re = 0, im = 0;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < N;
         k += (long long)gridDim.x * blockDim.x) {
        cplx<double> p = cmul(m[k], E[k]);
        re += p.re; im += p.im;
    }
    for (int o = 16; o > 0; o >>= 1) {
        re += __shfl_down_sync(0xffffffffu, re, o);
        im += __shfl_down_sync(0xffffffffu, im, o);
    }
    __shared__ double s[2][32];
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) { s[0][w] = re; s[1][w] = im; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0, b = 0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) { a += s[0][i]; b += s[1][i]; }
        part[blockIdx.x * 2] = a;
        part[blockIdx.x * 2 + 1] = b;
    }
}

// First invalid entries of a staged host input of n complex values (interleaved):
// first[0] = lowest double index of a NaN or ±inf, first[1] (when zeros) = lowest
// complex index whose real and imaginary parts are both zero.  first[] starts at
// ~0ull; a thread only writes when it finds something, so valid input costs one
// read of the data.  grid-stride, any grid.
__global__ void validate_kernel(const double2* __restrict__ x, long long n, int zeros, unsigned long long* first) {
    unsigned long long bad = ~0ull, zero = ~0ull;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
        const double2 v = x[c];
        if (!isfinite(v.x) && (unsigned long long)(2 * c) < bad) bad = 2 * c;
        else if (!isfinite(v.y) && (unsigned long long)(2 * c + 1) < bad) bad = 2 * c + 1;
        if (zeros && v.x == 0.0 && v.y == 0.0 && (unsigned long long)c < zero) zero = c;
    }
    if (bad != ~0ull) atomicMin(&first[0], bad);
    if (zero != ~0ull) atomicMin(&first[1], zero);
}
void launch_validate(cudaStream_t s, int nsm, const double* x, long long n, int zeros, unsigned long long* first) {
    cudaMemsetAsync(first, 0xFF, 2 * sizeof(unsigned long long), s);
    const long long want = (n + 255) / 256;
    const int grid = (int)std::max(1LL, std::min(want, 4LL * std::max(1, nsm)));
    validate_kernel<<<grid, 256, 0, s>>>(reinterpret_cast<const double2*>(x), n, zeros, first);
}
