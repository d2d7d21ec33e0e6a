// Block construction and dense block inversion for the cyclic-reduction
// factorization.
//
// With unknowns grouped into n "nodes" (grid lines) of b unknowns each, the
// 5-point operator is block-cyclic-tridiagonal: node j couples to itself
// through a cyclic tridiagonal D_j and to its ring neighbours j∓1 through
// diagonal matrices L_j, U_j (the periodic ±(N-1) corners of src/grid.jl:164-177
// close both the in-line and the node ring).
#include "common.cuh"
#include "kernels.cuh"

template <typename T>
__device__ __forceinline__ cplx<double> st_at(const cplx<double>* st, const NodeMap& m, int plane, int node, int i) {
    long long N = (long long)m.Nx * m.Ny;
    return st[plane * N + m.nat(node, i)];
}

template <typename T>
__device__ __forceinline__ void store_elem(const Pool<T>& P, T* base, int r, int c, cplx<T> v, int trans) {
    long long off = trans ? (long long)c * P.ld + r : (long long)r * P.ld + c;
    long long pe = P.plane_elems();
    base[off] = v.re;
    base[pe + off] = v.im;
    if (P.planes == 4) {
        base[2 * pe + off] = (T)tf32_lo((float)v.re);
        base[3 * pe + off] = (T)tf32_lo((float)v.im);
    }
}

// ---------------------------------------------------------------------------
// Dense D_k (scaled) for nodes eliminated in the first step: cyclic tridiagonal.
// grid: (ceil(b*b/256), nnodes)
// ---------------------------------------------------------------------------
template <typename T>
__global__ void build_tridiag_kernel(NodeMap m, const cplx<double>* st, double scale, Pool<T> D,
                                     const int* nodes) {
    int node = nodes[blockIdx.y];
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    int b = m.b;
    if (t >= (long long)b * b) return;
    int r = (int)(t / b), c = (int)(t % b);
    cplx<double> v = cmk(0.0, 0.0);
    if (c == r) v = st_at<T>(st, m, 0, node, r);
    if (c == (r + b - 1) % b) v = cadd(v, st_at<T>(st, m, m.p_inprev(), node, r));
    if (c == (r + 1) % b) v = cadd(v, st_at<T>(st, m, m.p_innext(), node, r));
    T* base = D.slot(node);
    store_elem<T>(D, base, r, c, cmk((T)(v.re * scale), (T)(v.im * scale)), 0);
}

// ---------------------------------------------------------------------------
// First reduction step, survivors s (diagonal couplings l, u at level 0):
//   D_s  = tri_s - [prev elim] diag(l_s) G_prev diag(u_prev) - [next elim] diag(u_s) G_next diag(l_next)
//   U_s' = next elim ? -diag(u_s) G_next diag(u_next) : diag(u_s)
//   L_s' = prev elim ? -diag(l_s) G_prev diag(l_prev) : diag(l_s)
// 32x32 tiles, block (32, 8); transposed stores go through shared memory.
// grid: (ceil(b/32), ceil(b/32), njobs)
// ---------------------------------------------------------------------------
template <typename T>
__global__ void level1_combine_kernel(NodeMap m, const cplx<double>* st, double scale, Pool<T> D,
                                      Pool<T> C, const L1Job* jobs) {
    __shared__ T tU[2][32][33], tL[2][32][33];
    const L1Job J = jobs[blockIdx.z];
    int b = m.b;
    int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    int tx = threadIdx.x, ty = threadIdx.y;
    const T* Gp = D.slot(J.prev);
    const T* Gn = D.slot(J.next);
    long long pe = D.plane_elems();
    T* Ds = D.slot(J.s);
    int c = c0 + tx;
    cplx<double> lc_next = cmk(0.0, 0.0), uc_next = cmk(0.0, 0.0), uc_prev = cmk(0.0, 0.0),
                 lc_prev = cmk(0.0, 0.0);
    if (c < b) {
        if (J.next_elim) {
            lc_next = cscale(st_at<T>(st, m, m.p_cprev(), J.next, c), scale);
            uc_next = cscale(st_at<T>(st, m, m.p_cnext(), J.next, c), scale);
        }
        if (J.prev_elim) {
            uc_prev = cscale(st_at<T>(st, m, m.p_cnext(), J.prev, c), scale);
            lc_prev = cscale(st_at<T>(st, m, m.p_cprev(), J.prev, c), scale);
        }
    }
    for (int q = 0; q < 4; ++q) {
        int rl = ty + 8 * q;
        int r = r0 + rl;
        cplx<double> dv = cmk(0.0, 0.0), uv = cmk(0.0, 0.0), lv = cmk(0.0, 0.0);
        bool ok = (r < b && c < b);
        if (ok) {
            cplx<double> ls = cscale(st_at<T>(st, m, m.p_cprev(), J.s, r), scale);
            cplx<double> us = cscale(st_at<T>(st, m, m.p_cnext(), J.s, r), scale);
            if (c == r) dv = st_at<T>(st, m, 0, J.s, r);
            if (c == (r + b - 1) % b) dv = cadd(dv, st_at<T>(st, m, m.p_inprev(), J.s, r));
            if (c == (r + 1) % b) dv = cadd(dv, st_at<T>(st, m, m.p_innext(), J.s, r));
            dv = cscale(dv, scale);
            if (J.prev_elim) {
                long long o = (long long)r * D.ld + c;
                cplx<double> g = cmk((double)Gp[o], (double)Gp[pe + o]);
                dv = csub(dv, cmul(cmul(ls, g), uc_prev));
                lv = cneg(cmul(cmul(ls, g), lc_prev));
            } else if (c == r) {
                lv = ls;
            }
            if (J.next_elim) {
                long long o = (long long)r * D.ld + c;
                cplx<double> g = cmk((double)Gn[o], (double)Gn[pe + o]);
                dv = csub(dv, cmul(cmul(us, g), lc_next));
                uv = cneg(cmul(cmul(us, g), uc_next));
            } else if (c == r) {
                uv = us;
            }
            store_elem<T>(D, Ds, r, c, cmk((T)dv.re, (T)dv.im), 0);
        }
        if (!J.u_trans) { if (ok) store_elem<T>(C, C.slot(J.u_slot), r, c, cmk((T)uv.re, (T)uv.im), 0); }
        else { tU[0][rl][tx] = (T)uv.re; tU[1][rl][tx] = (T)uv.im; }
        if (!J.l_trans) { if (ok) store_elem<T>(C, C.slot(J.l_slot), r, c, cmk((T)lv.re, (T)lv.im), 0); }
        else { tL[0][rl][tx] = (T)lv.re; tL[1][rl][tx] = (T)lv.im; }
    }
    if (J.u_trans || J.l_trans) {
        __syncthreads();
        // transposed store: element (r, c) -> position (c, r); thread writes row c0+ty*4+q, col r0+tx
        for (int q = 0; q < 4; ++q) {
            int cl = ty + 8 * q;
            int cc = c0 + cl, rr = r0 + tx;
            if (cc < b && rr < b) {
                if (J.u_trans)
                    store_elem<T>(C, C.slot(J.u_slot), cc, rr, cmk(tU[0][tx][cl], tU[1][tx][cl]), 0);
                if (J.l_trans)
                    store_elem<T>(C, C.slot(J.l_slot), cc, rr, cmk(tL[0][tx][cl], tL[1][tx][cl]), 0);
            }
        }
    }
}

template <typename T>
__global__ void perm_init_kernel(int* perm, int b) {
    int job = blockIdx.y;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < b; i += gridDim.x * blockDim.x)
        perm[(size_t)job * b + i] = i;
}

// ---------------------------------------------------------------------------
// Blocked in-place Gauss-Jordan inversion with partial pivoting, panel step.
//
// For the panel of columns [c0, c0+w) of each matrix M (b x b) the kernel
//  1. loads the panel M[:, c0:c0+w) into shared memory and runs w column
//     steps of in-place Gauss-Jordan on it: pivot = largest |re|+|im| among
//     the rows not yet used as pivots, row swap, pivot row scaled by 1/p with
//     the pivot entry replaced by 1/p, every other row i updated by
//     -M[i,j]·(scaled pivot row) with its pivot-column entry set to -M[i,j]/p.
//     The result G (b x w) holds the panel's block transformation;
//  2. applies the same row swaps to the full rows of M and records them in perm;
//  3. writes Rᵀ: the (swapped) panel rows M[c0:c0+w, :] transposed, with the
//     panel columns replaced by the identity.
// The rank-w update M = mask(M) + G·R is then one TN GEMM (gemm_*_kernel with
// mask [c0, c0+w)).  After the last panel M holds (P M₀)⁻¹, and
// gj_unpermute_kernel restores M₀⁻¹.  The in-place Gauss-Jordan scheme is the
// textbook one (e.g. G. W. Stewart, Matrix Algorithms I, §3.1).
// grid: njobs, block 512, dynamic smem (2*b*NB + 2*b)*sizeof(T)
// ---------------------------------------------------------------------------
template <typename T, int NB>
__global__ void __launch_bounds__(512) gj_panel_kernel(Pool<T> M, const int* slots, Pool<T> GP, Pool<T> RP,
                                                       int* perm, int c0, unsigned* err) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* pre = reinterpret_cast<T*>(smem_raw);
    const int b = M.rows;
    T* pim = pre + (size_t)b * NB;
    T* fre = pim + (size_t)b * NB;
    T* fim = fre + b;
    __shared__ T rowre[NB], rowim[NB];
    __shared__ int pivs[NB];
    __shared__ T redv[32];
    __shared__ int redi[32];
    __shared__ int s_piv;

    const int tid = threadIdx.x, nt = blockDim.x;
    const int job = blockIdx.x;
    const int slot = slots[job];
    T* Mre = M.slot(slot);
    T* Mim = Mre + M.plane_elems();
    const int ld = M.ld;
    const int w = min(NB, b - c0);

    for (int idx = tid; idx < b * NB; idx += nt) {
        int i = idx / NB, jj = idx % NB;
        T vr = 0, vi = 0;
        if (jj < w) { vr = Mre[(size_t)i * ld + c0 + jj]; vi = Mim[(size_t)i * ld + c0 + jj]; }
        pre[idx] = vr; pim[idx] = vi;
    }
    __syncthreads();

    for (int jj = 0; jj < w; ++jj) {
        const int r0 = c0 + jj;
        T best = (T)-1; int bi = b;
        for (int i = r0 + tid; i < b; i += nt) {
            T v = fabs(pre[i * NB + jj]) + fabs(pim[i * NB + jj]);
            if (v > best) { best = v; bi = i; }
        }
        for (int o = 16; o > 0; o >>= 1) {
            T ov = __shfl_down_sync(0xffffffffu, best, o);
            int oi = __shfl_down_sync(0xffffffffu, bi, o);
            if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
        }
        if ((tid & 31) == 0) { redv[tid >> 5] = best; redi[tid >> 5] = bi; }
        __syncthreads();
        if (tid < 32) {
            int nw = nt >> 5;
            best = tid < nw ? redv[tid] : (T)-1;
            bi = tid < nw ? redi[tid] : b;
            for (int o = 16; o > 0; o >>= 1) {
                T ov = __shfl_down_sync(0xffffffffu, best, o);
                int oi = __shfl_down_sync(0xffffffffu, bi, o);
                if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
            }
            if (tid == 0) {
                if (!(best > (T)0) || bi >= b || !isfinite((double)best)) {
                    dev_error(err, FDFD_DEVERR_SINGULAR);
                    bi = r0;
                }
                s_piv = bi;
                pivs[jj] = bi;
            }
        }
        __syncthreads();
        const int piv = s_piv;
        if (piv != r0 && tid < NB) {
            T a = pre[r0 * NB + tid]; pre[r0 * NB + tid] = pre[piv * NB + tid]; pre[piv * NB + tid] = a;
            T c = pim[r0 * NB + tid]; pim[r0 * NB + tid] = pim[piv * NB + tid]; pim[piv * NB + tid] = c;
        }
        __syncthreads();
        cplx<T> p = cmk(pre[r0 * NB + jj], pim[r0 * NB + jj]);
        cplx<T> inv = (p.re == (T)0 && p.im == (T)0) ? cmk((T)0, (T)0) : cinv(p);
        for (int i = tid; i < b; i += nt) { fre[i] = pre[i * NB + jj]; fim[i] = pim[i * NB + jj]; }
        if (tid < NB) {
            cplx<T> v = cmk((T)0, (T)0);
            if (tid < w) v = (tid == jj) ? inv : cmul(cmk(pre[r0 * NB + tid], pim[r0 * NB + tid]), inv);
            rowre[tid] = v.re; rowim[tid] = v.im;
        }
        __syncthreads();
        for (int idx = tid; idx < b * NB; idx += nt) {
            int i = idx / NB, j2 = idx % NB;
            if (j2 >= w) continue;
            if (i == r0) {
                pre[idx] = rowre[j2]; pim[idx] = rowim[j2];
            } else {
                cplx<T> f = cmk(fre[i], fim[i]);
                cplx<T> nv;
                if (j2 == jj) nv = cneg(cmul(f, inv));
                else nv = csub(cmk(pre[idx], pim[idx]), cmul(f, cmk(rowre[j2], rowim[j2])));
                pre[idx] = nv.re; pim[idx] = nv.im;
            }
        }
        __syncthreads();
    }

    // 1. G panel (b x GP.cols, zero padded)
    {
        T* g = GP.slot(job);
        const int gc = GP.cols;
        for (int idx = tid; idx < b * gc; idx += nt) {
            int i = idx / gc, k = idx % gc;
            cplx<T> v = cmk((T)0, (T)0);
            if (k < w) v = cmk(pre[i * NB + k], pim[i * NB + k]);
            store_elem<T>(GP, g, i, k, v, 0);
        }
    }
    // 2. row swaps on the full matrix, in order
    for (int jj = 0; jj < w; ++jj) {
        int r0 = c0 + jj, piv = pivs[jj];
        if (piv != r0) {
            for (int c = tid; c < b; c += nt) {
                T a = Mre[(size_t)r0 * ld + c]; Mre[(size_t)r0 * ld + c] = Mre[(size_t)piv * ld + c];
                Mre[(size_t)piv * ld + c] = a;
                T d = Mim[(size_t)r0 * ld + c]; Mim[(size_t)r0 * ld + c] = Mim[(size_t)piv * ld + c];
                Mim[(size_t)piv * ld + c] = d;
            }
            if (tid == 0) {
                int* pp = perm + (size_t)job * b;
                int t = pp[r0]; pp[r0] = pp[piv]; pp[piv] = t;
            }
        }
        __syncthreads();
    }
    // 3. Rᵀ (b x RP.cols): RT[c][k] = M[c0+k][c], identity on the panel columns
    {
        T* rt = RP.slot(job);
        const int rc = RP.cols;
        for (int idx = tid; idx < b * rc; idx += nt) {
            int k = idx / b, c = idx % b;    // c fastest: coalesced reads of M rows
            cplx<T> v = cmk((T)0, (T)0);
            if (k < w) {
                if (c >= c0 && c < c0 + w) v = cmk((T)((c - c0) == k ? 1 : 0), (T)0);
                else v = cmk(Mre[(size_t)(c0 + k) * ld + c], Mim[(size_t)(c0 + k) * ld + c]);
            }
            store_elem<T>(RP, rt, c, k, v, 0);
        }
    }
}

// M[:, perm[j]] = M[:, j] per row (in place via shared memory); rewrites lo planes.
// grid: (ceil(b/rows_per_block), njobs), block 256
template <typename T>
__global__ void gj_unpermute_kernel(Pool<T> M, const int* slots, const int* perm) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int b = M.rows;
    T* rre = reinterpret_cast<T*>(smem_raw);
    T* rim = rre + b;
    int job = blockIdx.y;
    T* base = M.slot(slots[job]);
    long long pe = M.plane_elems();
    const int* pp = perm + (size_t)job * b;
    const int rows_per = 8;
    for (int rr = 0; rr < rows_per; ++rr) {
        int r = blockIdx.x * rows_per + rr;
        if (r >= b) break;
        for (int j = threadIdx.x; j < b; j += blockDim.x) {
            rre[j] = base[(size_t)r * M.ld + j];
            rim[j] = base[pe + (size_t)r * M.ld + j];
        }
        __syncthreads();
        for (int j = threadIdx.x; j < b; j += blockDim.x) {
            int dst = pp[j];
            store_elem<T>(M, base, r, dst, cmk(rre[j], rim[j]), 0);
        }
        __syncthreads();
    }
}

// dst = P[s1] + P[s2] elementwise (same form), jobs (dst, s1, s2); grid (ceil(b*b/256), njobs)
template <typename T>
__global__ void madd_kernel(Pool<T> P, const int3* jobs) {
    int3 J = jobs[blockIdx.y];
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)P.rows * P.cols) return;
    int r = (int)(t / P.cols), c = (int)(t % P.cols);
    long long o = (long long)r * P.ld + c, pe = P.plane_elems();
    const T* a = P.slot(J.y);
    const T* bb = P.slot(J.z);
    store_elem<T>(P, P.slot(J.x), r, c, cmk(a[o] + bb[o], a[pe + o] + bb[pe + o]), 0);
}

// Dp[dst] = S[src] or S[src]ᵀ; jobs (dst, src, trans); grid (ceil(b/32), ceil(b/32), njobs), block (32, 8)
template <typename T>
__global__ void mcopy_kernel(Pool<T> S, Pool<T> Dp, const int3* jobs) {
    __shared__ T t[2][32][33];
    int3 J = jobs[blockIdx.z];
    int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    int tx = threadIdx.x, ty = threadIdx.y;
    const T* s = S.slot(J.y);
    long long pe = S.plane_elems();
    T* d = Dp.slot(J.x);
    for (int q = 0; q < 4; ++q) {
        int r = r0 + ty + 8 * q, c = c0 + tx;
        T vr = 0, vi = 0;
        if (r < S.rows && c < S.cols) { vr = s[(long long)r * S.ld + c]; vi = s[pe + (long long)r * S.ld + c]; }
        if (!J.z) { if (r < S.rows && c < S.cols) store_elem<T>(Dp, d, r, c, cmk(vr, vi), 0); }
        else { t[0][ty + 8 * q][tx] = vr; t[1][ty + 8 * q][tx] = vi; }
    }
    if (J.z) {
        __syncthreads();
        for (int q = 0; q < 4; ++q) {
            int cl = ty + 8 * q;
            int cc = c0 + cl, rr = r0 + tx;
            if (cc < S.cols && rr < S.rows) store_elem<T>(Dp, d, cc, rr, cmk(t[0][tx][cl], t[1][tx][cl]), 0);
        }
    }
}

// ---------------------------------------------------------------------------
// Host launchers
// ---------------------------------------------------------------------------
template <typename T>
void launch_build_tridiag(cudaStream_t s, int njobs, NodeMap m, const cplx<double>* st, double scale, Pool<T> D,
                          const int* nodes) {
    build_tridiag_kernel<T><<<dim3(ceil_div((long long)m.b * m.b, 256), njobs), 256, 0, s>>>(m, st, scale, D, nodes);
}
template <typename T>
void launch_level1_combine(cudaStream_t s, int njobs, NodeMap m, const cplx<double>* st, double scale, Pool<T> D,
                           Pool<T> C, const L1Job* jobs) {
    level1_combine_kernel<T><<<dim3(ceil_div(m.b, 32), ceil_div(m.b, 32), njobs), dim3(32, 8), 0, s>>>(
        m, st, scale, D, C, jobs);
}
void launch_perm_init(cudaStream_t s, int njobs, int* perm, int b) {
    perm_init_kernel<int><<<dim3(ceil_div(b, 256), njobs), 256, 0, s>>>(perm, b);
}
template <typename T, int NB>
static int gj_panel_nb(cudaStream_t s, int njobs, Pool<T> M, const int* slots, Pool<T> GP, Pool<T> RP, int* perm,
                       int c0, unsigned* err) {
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(gj_panel_kernel<T, NB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             220 * 1024);
        if (e != cudaSuccess) return (int)e;
        attr = true;
    }
    size_t smem = ((size_t)2 * M.rows * NB + 2 * M.rows) * sizeof(T);
    gj_panel_kernel<T, NB><<<njobs, 512, smem, s>>>(M, slots, GP, RP, perm, c0, err);
    return (int)cudaGetLastError();
}
template <typename T>
int launch_gj_panel(cudaStream_t s, int nb, int njobs, Pool<T> M, const int* slots, Pool<T> GP, Pool<T> RP,
                    int* perm, int c0, unsigned* err) {
    switch (nb) {
        case 32: return gj_panel_nb<T, 32>(s, njobs, M, slots, GP, RP, perm, c0, err);
        case 16: return gj_panel_nb<T, 16>(s, njobs, M, slots, GP, RP, perm, c0, err);
        case 8: return gj_panel_nb<T, 8>(s, njobs, M, slots, GP, RP, perm, c0, err);
        default: return (int)cudaErrorInvalidValue;
    }
}
template <typename T>
void launch_gj_unpermute(cudaStream_t s, int njobs, Pool<T> M, const int* slots, const int* perm) {
    gj_unpermute_kernel<T><<<dim3(ceil_div(M.rows, 8), njobs), 256, 2 * M.rows * sizeof(T), s>>>(M, slots, perm);
}
template <typename T>
void launch_madd(cudaStream_t s, int njobs, Pool<T> P, const int3* jobs) {
    madd_kernel<T><<<dim3(ceil_div((long long)P.rows * P.cols, 256), njobs), 256, 0, s>>>(P, jobs);
}
template <typename T>
void launch_mcopy(cudaStream_t s, int njobs, Pool<T> S, Pool<T> Dp, const int3* jobs) {
    mcopy_kernel<T><<<dim3(ceil_div(S.cols, 32), ceil_div(S.rows, 32), njobs), dim3(32, 8), 0, s>>>(S, Dp, jobs);
}

#define INST(T)                                                                                              \
    template void launch_build_tridiag<T>(cudaStream_t, int, NodeMap, const cplx<double>*, double, Pool<T>,   \
                                          const int*);                                                       \
    template void launch_level1_combine<T>(cudaStream_t, int, NodeMap, const cplx<double>*, double, Pool<T>,  \
                                           Pool<T>, const L1Job*);                                           \
    template int launch_gj_panel<T>(cudaStream_t, int, int, Pool<T>, const int*, Pool<T>, Pool<T>, int*, int, \
                                    unsigned*);                                                              \
    template void launch_gj_unpermute<T>(cudaStream_t, int, Pool<T>, const int*, const int*);                \
    template void launch_madd<T>(cudaStream_t, int, Pool<T>, const int3*);                                    \
    template void launch_mcopy<T>(cudaStream_t, int, Pool<T>, Pool<T>, const int3*);
INST(float)
INST(double)
