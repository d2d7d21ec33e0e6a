// Block construction and dense block inversion for the cyclic-reduction
// factorization.
//
// With unknowns grouped into n "nodes" (grid lines) of b unknowns each, the
// 5-point operator is block-cyclic-tridiagonal: node j couples to itself
// through a cyclic tridiagonal D_j and to its ring neighbours j∓1 through
// diagonal matrices L_j, U_j (the periodic ±(N-1) corners of src/grid.jl:138-151
// close both the in-line and the node ring).
#include "common.cuh"
#include "kernels.cuh"
#include <algorithm>

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
// Tiles of L1_TR = 16 rows x 128 columns, block 256: warp w takes rows w, w+8,
// each lane 4 consecutive columns, so block loads and row-major stores are
// 16-byte vectors and the per-row stencil factors are loaded once per lane.
// Transposed stores are staged in shared memory and written as 16-element
// transposed row segments, two per warp instruction.  The short tile keeps the
// staging at 34 KB, so five CTAs share an SM (the kernel waits on memory:
// resident warps are what keeps HBM busy).  Shared-memory layouts keep a warp's
// accesses on distinct banks: the per-column factors are stored lane-major
// (column 4·lane + e at e·32 + lane), and staged column c starts at c·17 + c/32
// (the skew spreads the 4·lane column stride over all 32 banks).
// grid: (ceil(b/128), ceil(b/L1_TR), njobs), dynamic smem level1_combine_smem<T>()
// ---------------------------------------------------------------------------
template <typename T> struct Vec16;
template <> struct Vec16<float> { typedef float4 type; };
template <> struct Vec16<double> { typedef double2 type; };

constexpr int L1_TR = 16;                       // tile rows
constexpr int L1_PS = 128 * (L1_TR + 1) + 4;    // staging plane stride (elements), skew included
template <typename T>
constexpr size_t level1_combine_smem() { return (size_t)2 * 2 * L1_PS * sizeof(T) + 4 * 128 * 2 * sizeof(T); }

// The five stencil planes of every node in the factor precision, scaled, contiguous
// in the in-line index: tab[(node·5 + plane)·b + i] = (T)(st · scale), converted
// once per factorization (FP64 issue is scarce, and a transposed node map strides
// st by Nx).  grid: (ceil(b/256), n), block 256
template <typename T>
__global__ void stencil_table_kernel(NodeMap m, const cplx<double>* st, double scale, cplx<T>* tab) {
    const int node = blockIdx.y, i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.b) return;
#pragma unroll
    for (int p = 0; p < 5; ++p) {
        const cplx<double> v = st_at<T>(st, m, p, node, i);
        tab[((size_t)node * 5 + p) * m.b + i] = cmk((T)(v.re * scale), (T)(v.im * scale));
    }
}

template <typename T>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 5 : 1) level1_combine_kernel(NodeMap m, const cplx<T>* tab,
                                                             Pool<T> D, Pool<T> C, const L1Job* jobs) {
    constexpr int CPL = 4;                    // columns per lane
    constexpr int VW = 16 / sizeof(T);
    constexpr int NVL = CPL / VW;             // 16-byte vectors per lane and plane
    typedef typename Vec16<T>::type VT;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int SR = L1_TR + 1;            // staging row stride
    T* tU = reinterpret_cast<T*>(smem_raw);  // [plane][tile column][tile row], plane stride L1_PS
    T* tL = tU + 2 * L1_PS;
    auto sidx = [](int c, int r) { return c * SR + (c >> 5) + r; };   // staged element (tile column c, row r)
    const L1Job J = jobs[blockIdx.z];
    const int b = m.b;
    const int c0 = blockIdx.x * 128, r0 = blockIdx.y * L1_TR;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int cl0 = lane * CPL;              // first tile column of this lane
    const int cb0 = c0 + cl0;                // its matrix column
    // distinct slots: no element is reached through two of these pointers
    const T* __restrict__ Gp = D.slot(J.prev);
    const T* __restrict__ Gn = D.slot(J.next);
    const long long pe = D.plane_elems();
    T* __restrict__ Ds = D.slot(J.s);
    T* __restrict__ Us = C.slot(J.u_slot);
    T* __restrict__ Ls = C.slot(J.l_slot);
    const long long cpe = C.plane_elems();
    // scaled stencil values in the factor precision (stencil_table_kernel)
    auto tv = [&](int plane, int node, int i) { return tab[((size_t)node * 5 + plane) * b + i]; };
    const cplx<T> z = cmk((T)0, (T)0);
    // per-column coupling factors of the neighbours, shared by the tile's rows:
    // [0] l_next, [1] u_next, [2] u_prev, [3] l_prev for the 128 tile columns,
    // tile column 4·lane + e at e·32 + lane
    cplx<T>* fac = reinterpret_cast<cplx<T>*>(tL + 2 * L1_PS);
    for (int t = threadIdx.x; t < 4 * 128; t += 256) {
        const int k = t / 128, cl = t % 128, c = c0 + cl;
        cplx<T> v = z;
        if (c < b) {
            if (k < 2 && J.next_elim) v = tv(k == 0 ? m.p_cprev() : m.p_cnext(), J.next, c);
            if (k >= 2 && J.prev_elim) v = tv(k == 2 ? m.p_cnext() : m.p_cprev(), J.prev, c);
        }
        fac[k * 128 + (cl % CPL) * 32 + cl / CPL] = v;
    }
    __syncthreads();
    const bool full = cb0 + CPL <= b;        // all four columns inside the matrix
#pragma unroll
    for (int q = 0; q < L1_TR / 8; ++q) {
        const int rl = warp + 8 * q;
        const int r = r0 + rl;
        if (r >= b || cb0 >= b) {
            // nothing to compute; the transposed staging of this element stays unused
            continue;
        }
        const cplx<T> ls = tv(m.p_cprev(), J.s, r);
        const cplx<T> us = tv(m.p_cnext(), J.s, r);
        // the cyclic tridiagonal row of D_s: three entries, converted once per row
        // (b >= 3, so no two of them share a column)
        const cplx<T> t_d = tv(0, J.s, r);
        const cplx<T> t_l = tv(m.p_inprev(), J.s, r);
        const cplx<T> t_u = tv(m.p_innext(), J.s, r);
        const int c_l = r == 0 ? b - 1 : r - 1, c_u = r == b - 1 ? 0 : r + 1;
        T gpr[CPL], gpi[CPL], gnr[CPL], gni[CPL];
        const long long o = (long long)r * D.ld + cb0;   // cb0 < b <= ld, cb0 % 4 == 0: vectors stay in the row
#pragma unroll
        for (int v = 0; v < NVL; ++v) {
            VT a = {}, c = {}, d = {}, f = {};
            if (J.prev_elim) {
                a = reinterpret_cast<const VT*>(Gp + o)[v];
                c = reinterpret_cast<const VT*>(Gp + pe + o)[v];
            }
            if (J.next_elim) {
                d = reinterpret_cast<const VT*>(Gn + o)[v];
                f = reinterpret_cast<const VT*>(Gn + pe + o)[v];
            }
#pragma unroll
            for (int e = 0; e < VW; ++e) {
                gpr[v * VW + e] = reinterpret_cast<const T*>(&a)[e];
                gpi[v * VW + e] = reinterpret_cast<const T*>(&c)[e];
                gnr[v * VW + e] = reinterpret_cast<const T*>(&d)[e];
                gni[v * VW + e] = reinterpret_cast<const T*>(&f)[e];
            }
        }
        T dr[CPL], di[CPL], ur[CPL], ui[CPL], lr[CPL], li[CPL];
#pragma unroll
        for (int e = 0; e < CPL; ++e) {
            const int c = cb0 + e;
            cplx<T> dv = c == r ? t_d : (c == c_l ? t_l : (c == c_u ? t_u : z));
            cplx<T> uv = z, lv = z;
            if (J.prev_elim) {
                const cplx<T> lg = cmul(ls, cmk(gpr[e], gpi[e]));
                dv = csub(dv, cmul(lg, fac[2 * 128 + e * 32 + lane]));
                lv = cneg(cmul(lg, fac[3 * 128 + e * 32 + lane]));
            } else if (c == r) {
                lv = ls;
            }
            if (J.next_elim) {
                const cplx<T> ug = cmul(us, cmk(gnr[e], gni[e]));
                dv = csub(dv, cmul(ug, fac[e * 32 + lane]));
                uv = cneg(cmul(ug, fac[128 + e * 32 + lane]));
            } else if (c == r) {
                uv = us;
            }
            dr[e] = dv.re; di[e] = dv.im; ur[e] = uv.re; ui[e] = uv.im; lr[e] = lv.re; li[e] = lv.im;
        }
        auto put_row = [&](T* base, long long ppe, const T* xr, const T* xi) {
            const long long ob = (long long)r * C.ld + cb0;
            if (full) {
#pragma unroll
                for (int v = 0; v < NVL; ++v) {
                    VT a, c;
#pragma unroll
                    for (int e = 0; e < VW; ++e) {
                        reinterpret_cast<T*>(&a)[e] = xr[v * VW + e];
                        reinterpret_cast<T*>(&c)[e] = xi[v * VW + e];
                    }
                    reinterpret_cast<VT*>(base + ob)[v] = a;
                    reinterpret_cast<VT*>(base + ppe + ob)[v] = c;
                }
            } else {
#pragma unroll
                for (int e = 0; e < CPL; ++e) {
                    if (cb0 + e < b) {
                        base[ob + e] = xr[e];
                        base[ppe + ob + e] = xi[e];
                    }
                }
            }
        };
        put_row(Ds, pe, dr, di);
        if (!J.u_trans) put_row(Us, cpe, ur, ui);
        else {
#pragma unroll
            for (int e = 0; e < CPL; ++e) {
                tU[sidx(cl0 + e, rl)] = ur[e];
                tU[L1_PS + sidx(cl0 + e, rl)] = ui[e];
            }
        }
        if (!J.l_trans) put_row(Ls, cpe, lr, li);
        else {
#pragma unroll
            for (int e = 0; e < CPL; ++e) {
                tL[sidx(cl0 + e, rl)] = lr[e];
                tL[L1_PS + sidx(cl0 + e, rl)] = li[e];
            }
        }
    }
    if (J.u_trans || J.l_trans) {
        __syncthreads();
        // transposed store: element (r, c) -> position (c, r); a warp instruction
        // writes two transposed row segments (tile columns cl, cl+1), lane % 16 =
        // tile row
        const int tr = lane % L1_TR;
        const int rr = r0 + tr;
        for (int cl = 2 * warp + lane / L1_TR; cl < 128; cl += 16) {
            const int cc = c0 + cl;
            if (cc >= b || rr >= b) continue;
            if (J.u_trans) store_elem<T>(C, Us, cc, rr, cmk(tU[sidx(cl, tr)], tU[L1_PS + sidx(cl, tr)]), 0);
            if (J.l_trans) store_elem<T>(C, Ls, cc, rr, cmk(tL[sidx(cl, tr)], tL[L1_PS + sidx(cl, tr)]), 0);
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
// Blocked Gauss-Jordan inversion with partial pivoting, panel step.
//
// For the panel of columns [c0, c0+w) of each matrix M (b x b) the kernel
//  1. loads the panel M[:, c0:c0+w) into registers and runs w column steps of
//     in-place Gauss-Jordan on it: pivot = largest |re|+|im| among the rows not
//     yet used as pivots (ties: lowest row), row exchange, pivot row scaled by
//     1/p with the pivot entry replaced by 1/p, every other row i updated by
//     -M[i,j]·(scaled pivot row) with its pivot-column entry set to -M[i,j]/p.
//     The result G (b x w) holds the panel's block transformation;
//  2. composes the panel's row exchanges into rowsrc (row r of the exchanged
//     matrix is row rowsrc[r] of M) and into perm; no row of M moves.
// gj_rt_kernel then writes Rᵀ: the exchanged panel rows M[rowsrc[c0:c0+w], :]
// transposed, with the panel columns replaced by the identity.
// The rank-w update M' = mask(M[rowsrc]) + G·R is then one TN GEMM
// (gemm_*_kernel with mask [c0, c0+w) reading its β term through rowsrc into
// a second buffer).  After the last panel M holds (P M₀)⁻¹, and
// gj_unpermute_kernel restores M₀⁻¹.  The Gauss-Jordan scheme is the textbook
// one (e.g. G. W. Stewart, Matrix Algorithms I, §3.1).
//
// Register tiling: the b x NB panel is cut into NB/C column blocks of 128
// threads each (4 warps, so a warp never straddles two blocks); thread rg of
// column block cb holds rows rg*R .. rg*R+R-1, columns cb*C .. cb*C+C-1.  A
// column step needs the pivot row only in the thread's C columns and the
// pivot column only in its R rows, which keeps the shared-memory traffic per
// step near b·(C+R) elements instead of b·NB.
// grid: njobs, block 512; requires b <= 128*R.
// ---------------------------------------------------------------------------
// Pivot search key of a candidate row: the FP32 bit pattern of |re|+|im| with
// its low 11 bits replaced by 2047 - (physical row).  Non-negative floats
// order like their bit patterns, so one unsigned max selects the largest
// magnitude; magnitudes that agree to 2^-12 relative go to the lowest physical
// row.  NaN sorts above +inf, so a NaN entry is picked and reported as
// singular.  Every candidate key is >= 1024, above the 0 of a non-candidate.
__device__ __forceinline__ unsigned pivot_key(float mag, int phys) {
    return (__float_as_uint(mag) & 0xFFFFF800u) | (unsigned)(2047 - phys);
}
__device__ __forceinline__ int pivot_key_row(unsigned key) { return 2047 - (int)(key & 0x7FFu); }

// 1/z = conj(z)/|z|² with z first scaled by a power of two (exact), so that
// |z|² neither overflows nor underflows; one reciprocal instead of the three
// divisions of Smith's algorithm.  z must be finite and non-zero.
template <typename T> __device__ __forceinline__ cplx<T> cinv_pow2(cplx<T> z) {
    int e;
    frexp(fmax(fabs(z.re), fabs(z.im)), &e);
    const T a = ldexp(z.re, -e), b = ldexp(z.im, -e);
    const T r = (T)1 / (a * a + b * b);
    return cmk(ldexp(a * r, -e), ldexp(-b * r, -e));
}

// dynamic shared memory of gj_panel_kernel (elements of T): the larger of the
// G staging tile (128 rows x NB+4, re and im) and the double-buffered pivot
// column (2 x 2 planes x 128*R)
template <int NB, int R>
__host__ __device__ constexpr size_t gj_panel_smem_elems() {
    return (size_t)2 * (128 * (NB + 4) > 2 * 128 * R ? 128 * (NB + 4) : 2 * 128 * R);
}


template <typename T, int NB, int R, int C>
__global__ void __launch_bounds__(512, 1) gj_panel_kernel(Pool<T> M, const int* slots, Pool<T> GP, int* perm,
                                                          int* rowsrc, int c0, unsigned* err) {
    constexpr int NT = 512;
    constexpr int NCB = NB / C;                        // column blocks
    constexpr int TPB = NT / NCB;                      // threads per column block
    constexpr int WPB = TPB / 32;                      // warps per column block
    constexpr int ROWS = TPB * R;                      // rows the block covers
    constexpr int VW = 16 / sizeof(T);                 // elements per 16-byte vector
    typedef typename Vec16<T>::type VT;
    static_assert(NCB * TPB == NT && TPB % 32 == 0 && C % VW == 0 && R % VW == 0, "panel tiling");
    __shared__ __align__(16) T prow_r[R][NB], prow_i[R][NB];  // the pivot row's row group
    __shared__ unsigned cand_key[WPB];
    __shared__ cplx<T> cand_p[WPB], cand_inv[WPB];      // each warp's candidate pivot and its inverse
    __shared__ int lrow_st[R];                         // logical rows of the pivot row's group
    __shared__ int rsm[ROWS];                          // composed row exchanges
    __shared__ cplx<T> alpha_s[ROWS];                  // deferred pivot-row scale factors
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* buf = reinterpret_cast<T*>(smem_raw);           // pivot column / G staging / Rᵀ transpose tile

    const int b = M.rows;
    const int tid = threadIdx.x;
    const int cb = tid / TPB, rg = tid % TPB;          // column block (warp-uniform), row group
    const int lane = tid & 31, wic = rg >> 5;          // warp index within the column block
    const int job = blockIdx.x;
    const T* Mre = M.slot(slots[job]);
    const T* Mim = Mre + M.plane_elems();
    const int ld = M.ld;
    const int w = min(NB, b - c0);

    // No data moves between threads: a row exchange only swaps the logical row
    // numbers (lrow) of the two physical rows, and a pivot row is not scaled in
    // place: its holders keep the unscaled row with 1 in the pivot column and
    // the factor 1/p goes to alpha_s (the later eliminations are linear in the
    // row, so the true row is alpha times the stored one throughout).
    T vr[R][C], vi[R][C];
    int lrow[R];
#pragma unroll
    for (int j = 0; j < R; ++j) {
        const int i = rg * R + j;
        lrow[j] = i < b ? i : INT_MAX;
        if (cb == 0) alpha_s[i] = cmk((T)1, (T)0);
#pragma unroll
        for (int v = 0; v < C / VW; ++v) {
            const int col = cb * C + v * VW;
            VT a = {}, c = {};
            // c0 + NB <= ld (ld is a multiple of 32 and of NB): the vector stays in the row
            if (i < b && col < w) {
                a = *reinterpret_cast<const VT*>(Mre + (size_t)i * ld + c0 + col);
                c = *reinterpret_cast<const VT*>(Mim + (size_t)i * ld + c0 + col);
            }
#pragma unroll
            for (int e = 0; e < VW; ++e) {
                const bool ok = i < b && col + e < w;
                vr[j][v * VW + e] = ok ? reinterpret_cast<const T*>(&a)[e] : (T)0;
                vi[j][v * VW + e] = ok ? reinterpret_cast<const T*>(&c)[e] : (T)0;
            }
        }
    }

    // Column step jj = g*C + sp (sp static): column block g holds the pivot
    // column.  Candidates are the logical rows >= r0, compared by pivot_key:
    // one 32-bit max-reduction per warp and one per block select the pivot.
#pragma unroll 1
    for (int g = 0; g * C < w; ++g) {
#pragma unroll
        for (int sp = 0; sp < C; ++sp) {
            const int jj = g * C + sp;
            if (jj < w) {   // uniform
            const int r0 = c0 + jj;
            T* cs_r = buf + (size_t)((jj & 1) * 2) * ROWS;   // pivot column, double-buffered
            T* cs_i = cs_r + ROWS;
            // A: column block g publishes the pivot column and its warps' candidates
            if (cb == g) {
                // each thread also inverts its own best candidate, so the winner's
                // 1/p is ready when the block has chosen (off the step's critical path)
                unsigned key = 0;
                T cvr = (T)1, cvi = (T)0;
#pragma unroll
                for (int j = 0; j < R; ++j)
                    if (lrow[j] >= r0 && lrow[j] < b) {
                        const unsigned k = pivot_key((float)(fabs(vr[j][sp]) + fabs(vi[j][sp])), rg * R + j);
                        if (k > key) { key = k; cvr = vr[j][sp]; cvi = vi[j][sp]; }
                    }
                const cplx<T> cinv_c = cinv_pow2(cmk(cvr, cvi));
#pragma unroll
                for (int v = 0; v < R / VW; ++v) {
                    VT a, c;
#pragma unroll
                    for (int e = 0; e < VW; ++e) {
                        reinterpret_cast<T*>(&a)[e] = vr[v * VW + e][sp];
                        reinterpret_cast<T*>(&c)[e] = vi[v * VW + e][sp];
                    }
                    reinterpret_cast<VT*>(cs_r + rg * R)[v] = a;
                    reinterpret_cast<VT*>(cs_i + rg * R)[v] = c;
                }
                const unsigned wkey = __reduce_max_sync(0xffffffffu, key);
                if (lane == 0) cand_key[wic] = wkey;
                if (key != 0u && key == wkey) {        // keys are unique: one lane per warp
                    cand_p[wic] = cmk(cvr, cvi);
                    cand_inv[wic] = cinv_c;
                }
            }
            __syncthreads();
            // B: block winner (every warp computes it; the holder of logical row r0
            // is always a candidate, so the winner is a real row); the threads of
            // the pivot row's group publish its rows and their logical numbers
            // (all R rows are staged: selecting one in registers would index the
            // register array at run time)
            const unsigned gkey = __reduce_max_sync(0xffffffffu, lane < WPB ? cand_key[lane] : 0u);
            const int pphys = pivot_key_row(gkey);     // physical row of the pivot
            const cplx<T> p = cand_p[(pphys / R) >> 5];
            const cplx<T> pinv = cand_inv[(pphys / R) >> 5];
            if (pphys / R == rg) {
#pragma unroll
                for (int j = 0; j < R; ++j) {
#pragma unroll
                    for (int v = 0; v < C / VW; ++v) {
                        VT a, c;
#pragma unroll
                        for (int e = 0; e < VW; ++e) {
                            reinterpret_cast<T*>(&a)[e] = vr[j][v * VW + e];
                            reinterpret_cast<T*>(&c)[e] = vi[j][v * VW + e];
                        }
                        reinterpret_cast<VT*>(&prow_r[j][cb * C])[v] = a;
                        reinterpret_cast<VT*>(&prow_i[j][cb * C])[v] = c;
                    }
                    if (cb == 0) lrow_st[j] = lrow[j];
                }
            }
            __syncthreads();
            const T* pr_r = prow_r[pphys % R];
            const T* pr_i = prow_i[pphys % R];
            const int pl = lrow_st[pphys % R];         // logical row of the pivot
            // C: every element: v -= (v[jj]/p)·(pivot row), pivot column <- -v[jj]/p;
            // the pivot row itself: f = 0 (unchanged), pivot column <- 1, alpha <- 1/p
            const bool bad = !(fabs(p.re) + fabs(p.im) > (T)0) || !isfinite(p.re) || !isfinite(p.im);
            if (bad && tid == 0) dev_error(err, FDFD_DEVERR_SINGULAR);
            const cplx<T> inv = bad ? cmk((T)0, (T)0) : pinv;
            T xr[C], xi[C];
#pragma unroll
            for (int v = 0; v < C / VW; ++v) {
                const VT a = reinterpret_cast<const VT*>(pr_r + cb * C)[v];
                const VT c = reinterpret_cast<const VT*>(pr_i + cb * C)[v];
#pragma unroll
                for (int e = 0; e < VW; ++e) {
                    xr[v * VW + e] = reinterpret_cast<const T*>(&a)[e];
                    xi[v * VW + e] = reinterpret_cast<const T*>(&c)[e];
                }
            }
            cplx<T> f[R];
            bool isp[R];
#pragma unroll
            for (int v = 0; v < R / VW; ++v) {
                const VT a = reinterpret_cast<const VT*>(cs_r + rg * R)[v];
                const VT c = reinterpret_cast<const VT*>(cs_i + rg * R)[v];
#pragma unroll
                for (int e = 0; e < VW; ++e) {
                    const int j = v * VW + e;
                    isp[j] = (lrow[j] == pl);
                    const cplx<T> fi = cmul(cmk(reinterpret_cast<const T*>(&a)[e], reinterpret_cast<const T*>(&c)[e]),
                                            inv);
                    f[j] = isp[j] ? cmk((T)0, (T)0) : fi;
                }
            }
            if constexpr (sizeof(T) == 4 && C % 2 == 0) {
                // packed FP32 FMAs (two lanes per instruction, each lane an IEEE fma:
                // the same results as the scalar form below)
#pragma unroll
                for (int j = 0; j < R; ++j) {
                    const float2 fi = make_float2(f[j].im, f[j].im), nfr = make_float2(-f[j].re, -f[j].re);
                    const float2 nfi = make_float2(-f[j].im, -f[j].im);
#pragma unroll
                    for (int k = 0; k < C; k += 2) {
                        const float2 x_r = make_float2(xr[k], xr[k + 1]), x_i = make_float2(xi[k], xi[k + 1]);
                        float2 a = make_float2(vr[j][k], vr[j][k + 1]), c = make_float2(vi[j][k], vi[j][k + 1]);
                        a = __ffma2_rn(nfr, x_r, __ffma2_rn(fi, x_i, a));
                        c = __ffma2_rn(nfr, x_i, __ffma2_rn(nfi, x_r, c));
                        vr[j][k] = a.x; vr[j][k + 1] = a.y;
                        vi[j][k] = c.x; vi[j][k + 1] = c.y;
                    }
                }
            } else {
#pragma unroll
                for (int j = 0; j < R; ++j)
#pragma unroll
                    for (int k = 0; k < C; ++k) {
                        vr[j][k] = fma(-f[j].re, xr[k], fma(f[j].im, xi[k], vr[j][k]));
                        vi[j][k] = fma(-f[j].re, xi[k], fma(-f[j].im, xr[k], vi[j][k]));
                    }
            }
#pragma unroll
            for (int j = 0; j < R; ++j) {
                if (cb == g) {
                    vr[j][sp] = isp[j] ? (T)1 : -f[j].re;
                    vi[j][sp] = isp[j] ? (T)0 : -f[j].im;
                }
                if (cb == 0 && isp[j]) alpha_s[rg * R + j] = inv;
                // exchange of logical rows r0 and pl between their holders
                lrow[j] = (lrow[j] == r0) ? pl : (isp[j] ? r0 : lrow[j]);
            }
            }
        }
    }
    __syncthreads();
    // apply the deferred pivot-row scale factors
#pragma unroll
    for (int j = 0; j < R; ++j) {
        const cplx<T> al = alpha_s[rg * R + j];
#pragma unroll
        for (int k = 0; k < C; ++k) {
            const cplx<T> x = cmul(al, cmk(vr[j][k], vi[j][k]));
            vr[j][k] = x.re;
            vi[j][k] = x.im;
        }
    }

    // 1. G panel (b x GP.cols, zero padded).  Rows
    //    are staged by logical row, 128 at a time, in shared memory (row stride
    //    NB+4 keeps 16-byte accesses conflict-free) and written as whole 16-byte
    //    vectors of consecutive columns, so each warp store covers full rows.
    {
        T* gp = GP.slot(job);
        const long long pe = GP.plane_elems();
        constexpr int SR = NB + 4;
        const int gv = GP.cols / VW;                   // vectors per G row (GP.cols % VW == 0)
        for (int ch = 0; ch < b; ch += 128) {
            __syncthreads();
#pragma unroll
            for (int j = 0; j < R; ++j) {
                const int L = lrow[j];                 // G row L is the row of logical row L
                if (L >= ch && L < ch + 128 && L < b) {
                    T* sr = buf + (size_t)(L - ch) * SR + cb * C;
                    T* si = buf + (size_t)128 * SR + (size_t)(L - ch) * SR + cb * C;
#pragma unroll
                    for (int v = 0; v < C / VW; ++v) {
                        VT a, c;
#pragma unroll
                        for (int e = 0; e < VW; ++e) {
                            reinterpret_cast<T*>(&a)[e] = vr[j][v * VW + e];
                            reinterpret_cast<T*>(&c)[e] = vi[j][v * VW + e];
                        }
                        reinterpret_cast<VT*>(sr)[v] = a;
                        reinterpret_cast<VT*>(si)[v] = c;
                    }
                }
            }
            __syncthreads();
            const int nr = min(128, b - ch);
            for (int idx = tid; idx < nr * gv; idx += NT) {
                const int rl = idx / gv, v = idx % gv;
                VT a = {}, c = {};
                if (v < NB / VW) {
                    a = reinterpret_cast<const VT*>(buf + (size_t)rl * SR)[v];
                    c = reinterpret_cast<const VT*>(buf + (size_t)128 * SR + (size_t)rl * SR)[v];
                }
                const long long o = (long long)(ch + rl) * GP.ld + v * VW;
                *reinterpret_cast<VT*>(gp + o) = a;
                *reinterpret_cast<VT*>(gp + pe + o) = c;
                if (GP.planes == 4) {   // pre-split tensor-core operand: TF32 residual planes
                    VT al, cl;
#pragma unroll
                    for (int e = 0; e < VW; ++e) {
                        reinterpret_cast<T*>(&al)[e] = (T)tf32_lo((float)reinterpret_cast<const T*>(&a)[e]);
                        reinterpret_cast<T*>(&cl)[e] = (T)tf32_lo((float)reinterpret_cast<const T*>(&c)[e]);
                    }
                    *reinterpret_cast<VT*>(gp + 2 * pe + o) = al;
                    *reinterpret_cast<VT*>(gp + 3 * pe + o) = cl;
                }
            }
        }
    }
    // 2. the panel's row exchanges, composed: row r of the exchanged matrix is
    //    row rsm[r] of M, the physical row that holds logical row r (the GEMM
    //    reads through this map, no rows move here)
    if (cb == 0) {
#pragma unroll
        for (int j = 0; j < R; ++j)
            if (lrow[j] < b) rsm[lrow[j]] = rg * R + j;
    }
    __syncthreads();
    {
        int* rs = rowsrc + (size_t)job * b;
        int* pp = perm + (size_t)job * b;
        constexpr int PPT = ROWS / NT;                 // rows per thread here (ROWS is a multiple of NT)
        int pv[PPT];
#pragma unroll
        for (int t = 0; t < PPT; ++t) {
            const int i = tid + t * NT;
            if (i < b) pv[t] = pp[rsm[i]];
        }
        __syncthreads();   // every old perm entry is read before any is overwritten
#pragma unroll
        for (int t = 0; t < PPT; ++t) {
            const int i = tid + t * NT;
            if (i < b) { pp[i] = pv[t]; rs[i] = rsm[i]; }
        }
    }
}

// Rᵀ of a panel (b x RP.cols): RT[c][k] = (row c0+k after the panel's exchanges)[c],
// the identity on the panel columns, read through rowsrc (row r of the exchanged
// matrix is row rowsrc[r] of M).  A separate launch from the panel kernel: the
// rows it reads outside the panel are written by the previous panel's wide
// update, which the look-ahead runs concurrently with this panel's column steps.
// One CTA per 128 columns and matrix; the tile is staged through shared memory so
// reads and writes coalesce.  grid: (ceil(b/128), njobs), block 512
template <typename T, int NB, int TW = 128>
__global__ void __launch_bounds__(512) gj_rt_kernel(Pool<T> M, const int* slots, Pool<T> RP, const int* rowsrc,
                                                    int c0, int rcw) {
    constexpr int NT = 512;
    constexpr int IT = NB * TW / NT;               // loads per thread
    static_assert((NB * TW) % NT == 0, "tile split");
    __shared__ T buf[2 * NB * (TW + 1)];
    const int b = M.rows, tid = threadIdx.x, job = blockIdx.y;
    const int cb = blockIdx.x * TW, cw = min(TW, b - cb);
    const int w = min(NB, b - c0);
    const T* Mre = M.slot(slots[job]);
    const T* Mim = Mre + M.plane_elems();
    const int ld = M.ld;
    const int* rs = rowsrc + (size_t)job * b;
    T* rt = RP.slot(job);
    const int rc = rcw;     // RT columns written (zero beyond the panel)
    const long long pe = RP.plane_elems();
    T la[IT], lb[IT];
#pragma unroll
    for (int u = 0; u < IT; ++u) {
        const int idx = tid + u * NT;
        const int k = idx / TW, c = idx % TW;
        const int cc = cb + c;
        la[u] = 0; lb[u] = 0;
        if (k < w && c < cw) {
            if (cc >= c0 && cc < c0 + w) la[u] = (T)((cc - c0) == k ? 1 : 0);
            else {
                const int sr = rs[c0 + k];
                la[u] = Mre[(size_t)sr * ld + cc];
                lb[u] = Mim[(size_t)sr * ld + cc];
            }
        }
    }
#pragma unroll
    for (int u = 0; u < IT; ++u) {
        const int idx = tid + u * NT;
        const int k = idx / TW, c = idx % TW;
        buf[2 * (k * (TW + 1) + c)] = la[u];
        buf[2 * (k * (TW + 1) + c) + 1] = lb[u];
    }
    __syncthreads();
    for (int idx = tid; idx < cw * rc; idx += NT) {
        const int c = idx / rc, k = idx % rc;
        T a = 0, d = 0;
        if (k < NB) { a = buf[2 * (k * (TW + 1) + c)]; d = buf[2 * (k * (TW + 1) + c) + 1]; }
        const long long o = (long long)(cb + c) * RP.ld + k;
        rt[o] = a;
        rt[pe + o] = d;
        if (RP.planes == 4) {   // pre-split tensor-core operand
            rt[2 * pe + o] = (T)tf32_lo((float)a);
            rt[3 * pe + o] = (T)tf32_lo((float)d);
        }
    }
}

// Gauss-Jordan panel step, lane-quad form (b <= 128*R, 16-byte vectors of NB/4
// columns).  The four lanes 4q..4q+3 of a warp share rows: lane c of the quad
// holds columns [c*C, c*C+C) (C = NB/4) of the quad's R rows (rows
// R*(8*warp + q) .. +R-1; R = 4 for b <= 512, 8 up to 1024, with the narrower
// panel there).  Every row therefore lives inside one warp, which
// gives a column step one block-wide barrier: the warp's best candidate row is
// published whole by its quad before the barrier; after it, every thread takes
// the largest of the 16 warp keys (the key names the physical row, hence the
// warp), reads its C columns of the winning row (shared memory) and gets the
// pivot-column values of its rows from the quad lane that holds that column
// (shuffles).  The arithmetic is that of
// gj_panel_kernel (same pivot keys, same reciprocal, same fma sequence,
// deferred pivot-row scale), so both forms give identical results.  Candidate
// slots alternate by step parity.  grid: njobs, block 512; requires b <= 128*R.
template <typename T, int NB, int R>
__global__ void __launch_bounds__(512, 1) gj_panel_quad_kernel(Pool<T> M, const int* slots, Pool<T> GP, int* perm,
                                                               int* rowsrc, int c0, unsigned* err, GjFuse fz) {
    constexpr int NT = 512, NW = NT / 32, C = NB / 4;
    constexpr int VW = 16 / sizeof(T);
    static_assert(C % VW == 0 && (R & (R - 1)) == 0, "quad tiling");
    typedef typename Vec16<T>::type VT;
    __shared__ __align__(16) T cand_row[2][NW][2 * NB];   // [parity][warp][re | im]
    __shared__ __align__(16) unsigned cand_key[2][NW];
    __shared__ cplx<T> cand_inv[2][NW];
    __shared__ int cand_lrow[2][NW];
    __shared__ int rsm[128 * R];                      // composed row exchanges, every row of the block
    const int b = M.rows;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const int qc = lane & 3;                         // column block of this lane
    const int qbase = lane & ~3;                     // first lane of the quad
    const int row0 = (warp * 8 + (lane >> 2)) * R;   // first of the quad's rows
    const int job = blockIdx.x;
    const T* Mre = M.slot(slots[job]);
    const T* Mim = Mre + M.plane_elems();
    const int ld = M.ld;
    const int w = min(NB, b - c0);
    T vr[R][C], vi[R][C];
    int lrow[R];
    cplx<T> alpha[R];                                // deferred pivot-row scales
#pragma unroll
    for (int j = 0; j < R; ++j) {
        const int i = row0 + j;
        lrow[j] = i < b ? i : INT_MAX;
        alpha[j] = cmk((T)1, (T)0);
#pragma unroll
        for (int v = 0; v < C / VW; ++v) {
            const int col = qc * C + v * VW;
            VT a = {}, c = {};
            if (i < b && col < w) {   // c0 + NB <= ld: the vector stays in the row
                a = *reinterpret_cast<const VT*>(Mre + (size_t)i * ld + c0 + col);
                c = *reinterpret_cast<const VT*>(Mim + (size_t)i * ld + c0 + col);
            }
#pragma unroll
            for (int e = 0; e < VW; ++e) {
                const bool ok = i < b && col + e < w;
                vr[j][v * VW + e] = ok ? reinterpret_cast<const T*>(&a)[e] : (T)0;
                vi[j][v * VW + e] = ok ? reinterpret_cast<const T*>(&c)[e] : (T)0;
            }
        }
    }
#pragma unroll 1
    for (int g = 0; g * C < w; ++g) {
#pragma unroll
        for (int sp = 0; sp < C; ++sp) {
            const int jj = g * C + sp;
            if (jj < w) {   // uniform
                const int r0 = c0 + jj;
                const int par = jj & 1;
                // A: keys of the rows held by the pivot column's lanes; warp maximum.
                // The key encodes the physical row, so the winning quad and row follow
                // from the maximum directly; the quad publishes the row, and its lane
                // in the pivot column adds the reciprocal of the pivot.
                unsigned key = 0;
                if (qc == g) {
#pragma unroll
                    for (int j = 0; j < R; ++j)
                        if (lrow[j] >= r0 && lrow[j] < b)
                            key = max(key, pivot_key((float)(fabs(vr[j][sp]) + fabs(vi[j][sp])), row0 + j));
                }
                const unsigned wkey = __reduce_max_sync(0xffffffffu, key);
                if (wkey != 0u) {
                    const int wphys = pivot_key_row(wkey);
                    const int wq = (wphys / R) & 7, jsel = wphys & (R - 1);
                    if ((lane >> 2) == wq) {
                        T* cr = cand_row[par][warp];
#pragma unroll
                        for (int j = 0; j < R; ++j) {
                            if (j == jsel) {
#pragma unroll
                                for (int v = 0; v < C / VW; ++v) {
                                    VT a, c;
#pragma unroll
                                    for (int e = 0; e < VW; ++e) {
                                        reinterpret_cast<T*>(&a)[e] = vr[j][v * VW + e];
                                        reinterpret_cast<T*>(&c)[e] = vi[j][v * VW + e];
                                    }
                                    reinterpret_cast<VT*>(cr + qc * C)[v] = a;
                                    reinterpret_cast<VT*>(cr + NB + qc * C)[v] = c;
                                }
                                if (qc == g) {
                                    cand_inv[par][warp] = cinv_pow2(cmk(vr[j][sp], vi[j][sp]));
                                    cand_lrow[par][warp] = lrow[j];
                                }
                            }
                        }
                    }
                }
                if (lane == 0) cand_key[par][warp] = wkey;
                __syncthreads();
                // B: the winner among the warp candidates (the holder of logical row r0
                // is always a candidate, so there is one)
                unsigned gkey = 0u;
#pragma unroll
                for (int q = 0; q < NW / 4; ++q) {
                    const uint4 kv = reinterpret_cast<const uint4*>(cand_key[par])[q];
                    gkey = max(gkey, max(max(kv.x, kv.y), max(kv.z, kv.w)));
                }
                const int ww = pivot_key_row(gkey) / (8 * R);   // a warp holds 8*R consecutive physical rows
                const T* pr = cand_row[par][ww];
                const int pl = cand_lrow[par][ww];
                const cplx<T> p = cmk(pr[jj], pr[NB + jj]);
                const bool bad = !(fabs(p.re) + fabs(p.im) > (T)0) || !isfinite(p.re) || !isfinite(p.im);
                if (bad && t == 0) dev_error(err, FDFD_DEVERR_SINGULAR);
                const cplx<T> inv = bad ? cmk((T)0, (T)0) : cand_inv[par][ww];
                // C: the pivot-column values of this lane's rows (held by quad lane g)
                cplx<T> f[R];
                bool isp[R];
#pragma unroll
                for (int j = 0; j < R; ++j) {
                    const T cr_ = __shfl_sync(0xffffffffu, vr[j][sp], qbase + g);
                    const T ci_ = __shfl_sync(0xffffffffu, vi[j][sp], qbase + g);
                    isp[j] = lrow[j] == pl;
                    const cplx<T> fi = cmul(cmk(cr_, ci_), inv);
                    f[j] = isp[j] ? cmk((T)0, (T)0) : fi;
                }
                T xr[C], xi[C];
#pragma unroll
                for (int v = 0; v < C / VW; ++v) {
                    const VT a = reinterpret_cast<const VT*>(pr + qc * C)[v];
                    const VT c = reinterpret_cast<const VT*>(pr + NB + qc * C)[v];
#pragma unroll
                    for (int e = 0; e < VW; ++e) {
                        xr[v * VW + e] = reinterpret_cast<const T*>(&a)[e];
                        xi[v * VW + e] = reinterpret_cast<const T*>(&c)[e];
                    }
                }
                if constexpr (sizeof(T) == 4 && C % 2 == 0) {
#pragma unroll
                    for (int j = 0; j < R; ++j) {
                        const float2 fim = make_float2(f[j].im, f[j].im), nfr = make_float2(-f[j].re, -f[j].re);
                        const float2 nfi = make_float2(-f[j].im, -f[j].im);
#pragma unroll
                        for (int k = 0; k < C; k += 2) {
                            const float2 x_r = make_float2(xr[k], xr[k + 1]), x_i = make_float2(xi[k], xi[k + 1]);
                            float2 a = make_float2(vr[j][k], vr[j][k + 1]), c = make_float2(vi[j][k], vi[j][k + 1]);
                            a = __ffma2_rn(nfr, x_r, __ffma2_rn(fim, x_i, a));
                            c = __ffma2_rn(nfr, x_i, __ffma2_rn(nfi, x_r, c));
                            vr[j][k] = a.x; vr[j][k + 1] = a.y;
                            vi[j][k] = c.x; vi[j][k + 1] = c.y;
                        }
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < R; ++j)
#pragma unroll
                        for (int k = 0; k < C; ++k) {
                            vr[j][k] = fma(-f[j].re, xr[k], fma(f[j].im, xi[k], vr[j][k]));
                            vi[j][k] = fma(-f[j].re, xi[k], fma(-f[j].im, xr[k], vi[j][k]));
                        }
                }
#pragma unroll
                for (int j = 0; j < R; ++j) {
                    if (qc == g) {
                        vr[j][sp] = isp[j] ? (T)1 : -f[j].re;
                        vi[j][sp] = isp[j] ? (T)0 : -f[j].im;
                    }
                    if (isp[j]) alpha[j] = inv;
                    // exchange of logical rows r0 and pl between their holders
                    lrow[j] = (lrow[j] == r0) ? pl : (isp[j] ? r0 : lrow[j]);
                }
            }
        }
    }
    // apply the deferred pivot-row scales
#pragma unroll
    for (int j = 0; j < R; ++j)
#pragma unroll
        for (int k = 0; k < C; ++k) {
            const cplx<T> x = cmul(alpha[j], cmk(vr[j][k], vi[j][k]));
            vr[j][k] = x.re;
            vi[j][k] = x.im;
        }
    // the panel's row exchanges, composed (row r of the exchanged matrix is row
    // rsm[r] of M); the perm gather is issued before the G stores so that its
    // latency overlaps them
    if (qc == 0) {
#pragma unroll
        for (int j = 0; j < R; ++j)
            if (lrow[j] < b) rsm[lrow[j]] = row0 + j;
    }
    __syncthreads();
    int* rs = rowsrc + (size_t)job * b;
    int* pp = perm + (size_t)job * b;
    constexpr int PPT = 128 * R / NT;                // rows per thread in the bookkeeping
    static_assert(128 * R % NT == 0, "rows per thread");
    int rsv[PPT], pv[PPT];
#pragma unroll
    for (int u = 0; u < PPT; ++u) {
        const int i = t + u * NT;
        rsv[u] = i < b ? rsm[i] : 0;
        pv[u] = i < b ? pp[rsv[u]] : 0;
    }
    // G (b x NB; the update reads K = NB columns): row j of this lane goes to G row
    // lrow[j], columns [qc*C, qc*C+C) as whole 16-byte vectors.  Fused super-panels
    // (fz.fused): the columns start at fz.gcol0 and the row is the super-panel's
    // input row of this physical row (fz.tot_in, identity when null).
    const int* tin = fz.tot_in ? fz.tot_in + (size_t)job * b : nullptr;
    {
        T* gp = GP.slot(job);
        const long long pe = GP.plane_elems();
#pragma unroll
        for (int j = 0; j < R; ++j) {
            if (lrow[j] >= b) continue;
            const int grow = fz.fused ? (tin ? tin[row0 + j] : row0 + j) : lrow[j];
            const long long o = (long long)grow * GP.ld + fz.gcol0;
#pragma unroll
            for (int v = 0; v < C / VW; ++v) {
                VT a, c;
#pragma unroll
                for (int e = 0; e < VW; ++e) {
                    reinterpret_cast<T*>(&a)[e] = vr[j][v * VW + e];
                    reinterpret_cast<T*>(&c)[e] = vi[j][v * VW + e];
                }
                const int col = qc * C + v * VW;
                *reinterpret_cast<VT*>(gp + o + col) = a;
                *reinterpret_cast<VT*>(gp + pe + o + col) = c;
                if (GP.planes == 4) {   // pre-split tensor-core operand: TF32 residual planes
                    VT al, cl;
#pragma unroll
                    for (int e = 0; e < VW; ++e) {
                        reinterpret_cast<T*>(&al)[e] = (T)tf32_lo((float)reinterpret_cast<const T*>(&a)[e]);
                        reinterpret_cast<T*>(&cl)[e] = (T)tf32_lo((float)reinterpret_cast<const T*>(&c)[e]);
                    }
                    *reinterpret_cast<VT*>(gp + 2 * pe + o + col) = al;
                    *reinterpret_cast<VT*>(gp + 3 * pe + o + col) = cl;
                }
            }
        }
    }
    // fused: rowsrc becomes the composed map tot_out[r] = tot_in[rsm[r]] (row of the
    // super-panel's input matrix that lands at logical row r)
    if (tin) {
#pragma unroll
        for (int u = 0; u < PPT; ++u) {
            const int i = t + u * NT;
            if (i < b) rsv[u] = tin[rsv[u]];
        }
    }
    __syncthreads();   // every old perm (and tot_in) entry is read before any is overwritten
#pragma unroll
    for (int u = 0; u < PPT; ++u) {
        const int i = t + u * NT;
        if (i < b) {
            pp[i] = pv[u];
            rs[i] = rsv[u];
            if (fz.fused) {
                fz.inv_out[(size_t)job * b + rsv[u]] = i;
                rsm[i] = rsv[u];
            }
        }
    }
    if (fz.fused && fz.gcol0 > 0) {
        // The earlier sub-panels' G columns of this panel's pivot rows (input rows
        // tot_out[c0 .. c0+w)): copied to gsub for the pivot-row product, then zeroed
        // (rows of this panel's pivots take no earlier update).
        __syncthreads();
        T* gp = GP.slot(job);
        const long long pe = GP.plane_elems();
        T* gs = static_cast<T*>(fz.gsub) + (size_t)job * 2 * NB * GP.cols;
        const int n = w * fz.gcol0;
        for (int idx = t; idx < n; idx += NT) {
            const int jj = idx / fz.gcol0, c = idx % fz.gcol0;
            const long long o = (long long)rsm[c0 + jj] * GP.ld + c;
            gs[(size_t)jj * GP.cols + c] = gp[o];
            gs[(size_t)(NB + jj) * GP.cols + c] = gp[pe + o];
            for (int pl2 = 0; pl2 < GP.planes; ++pl2) gp[pl2 * pe + o] = (T)0;
        }
    }
}

// Gauss-Jordan panel step, row form: thread t holds the R physical rows t·R ..
// t·R + R - 1 in all NB columns of the panel (registers), so the pivot column of
// a step is in every thread's own registers and the per-row bookkeeping (pivot
// key, exchange tracking, deferred scale) runs once per row.  The panel comes in
// and G goes out through shared memory (rows padded by 16 bytes, so a warp's
// row reads are conflict-free), with whole 16-byte vectors of consecutive
// columns per lane in global memory.  Steps run in groups of GS = min(8, NB):
// the GS steps of a group are unrolled and the register columns rotate by GS
// after each group, so the columns of the current group always sit in
// registers 0 .. GS-1 (static indices) while the code stays one group long.
// The step loop is software-pipelined: step s's pivot search runs
// before step s-1's rank-1 update of the bulk columns, so the FMA work of one
// step overlaps the latency chain (warp maximum, publication, block wait,
// broadcast read) of the next.  Iteration s:
//   1. column s and the bookkeeping (exchange, deferred scale, the Gauss-Jordan
//      column s-1) take step s-1's transformation;
//   2. warp maximum of the pivot keys of column s;
//   3. the owning lane publishes its row, still lacking step s-1 in the columns
//      other than s and s-1, with its step s-1 factor; the warp's lanes then
//      apply step s-1 to it, one column per lane, with the fma sequence the
//      owner applies to its registers, so the published row is the row the
//      sequential order would publish; the warp's key; one mbarrier arrival;
//   4. step s-1 on this thread's other columns (pivot row streamed from shared
//      memory);
//   5. bounded wait for every warp's arrival; the winner of step s and the
//      factors of this thread's rows.
// Iteration w (the panel width) only applies step w-1 (after the loop when w = NB).  Every element sees the
// operations of gj_panel_quad_kernel in the same order with the same pivots, so
// both forms give identical results.  Published rows rotate through three
// slots: a step's pivot row is read until step s+1's update, and its slot is
// written again at step s+3, after every warp has arrived at s+2.  A wait that
// runs past wait_ns sets FDFD_DEVERR_TIMEOUT (the results are then void).
// grid: njobs, block ceil(b / R / 32)·32 <= 512 threads, dynamic shared memory
// gj_panel_row_smem<T, NB>(block · R).
template <typename T, int NB> __host__ __device__ constexpr int gj_row_stride() { return NB * (int)sizeof(T) + 16; }
template <typename T, int NB> __host__ __device__ constexpr size_t gj_panel_row_smem(int rows) {
    return (size_t)2 * rows * gj_row_stride<T, NB>();
}

template <typename T, int NB, int R>
__global__ void __launch_bounds__(512, 1) gj_panel_row_kernel(Pool<T> M, const int* slots, Pool<T> GP, int* perm,
                                                              int* rowsrc, int c0, unsigned* err, uint64_t wait_ns) {
    constexpr int NWM = 16, VW = 16 / sizeof(T), NS = 3;
    constexpr int RSB = gj_row_stride<T, NB>();           // staging row stride, bytes
    constexpr int CPR = NB / VW;                          // 16-byte vectors per row and plane
    constexpr int GS = NB < 8 ? NB : 8, NG = NB / GS;     // steps per group, groups
    static_assert(NB % VW == 0 && NB <= 32, "row tiling");
    typedef typename Vec16<T>::type VT;
    extern __shared__ __align__(16) unsigned char stage[];  // [plane][row] x RSB bytes
    __shared__ __align__(16) T cand_row[NS][NWM][2 * NB];   // [slot][warp][re | im]
    __shared__ __align__(16) unsigned cand_key[NS][NWM];
    __shared__ cplx<T> cand_inv[NS][NWM];
    __shared__ int cand_lrow[NS][NWM];
    __shared__ cplx<T> cand_f[NWM];                         // step s-1 factor of the warp's published row
    __shared__ __align__(8) uint64_t bar;
    __shared__ int rsm[512 * R];                            // composed row exchanges, every row of the block
    const int b = M.rows, NT = blockDim.x, NW = NT / 32, NR = NT * R;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const int row0 = t * R;
    const int job = blockIdx.x;
    const T* Mre = M.slot(slots[job]);
    const T* Mim = Mre + M.plane_elems();
    const int ld = M.ld;
    const int w = min(NB, b - c0);
    const uint32_t bar_a = smem_u32(&bar);
    auto srow = [&](int plane, int r) { return reinterpret_cast<T*>(stage + ((size_t)plane * NR + r) * RSB); };
    if (t < NS * NWM) cand_key[t / NWM][t % NWM] = 0u;     // warps beyond the block never publish
    if (t == 0) mbar_init(bar_a, NW);
    // the panel, coalesced: consecutive threads take consecutive vectors of a row
    for (int idx = t; idx < 2 * b * CPR; idx += NT) {
        const int plane = idx / (b * CPR), rem = idx - plane * b * CPR;
        const int r = rem / CPR, col = (rem % CPR) * VW;
        VT a = {};
        if (col < w) {   // c0 + NB <= ld: the vector stays in the row
            a = *reinterpret_cast<const VT*>((plane ? Mim : Mre) + (size_t)r * ld + c0 + col);
#pragma unroll
            for (int e = 0; e < VW; ++e)
                if (col + e >= w) reinterpret_cast<T*>(&a)[e] = (T)0;
        }
        reinterpret_cast<VT*>(srow(plane, r))[col / VW] = a;
    }
    __syncthreads();
    T vr[R][NB], vi[R][NB];
    int lrow[R];
    cplx<T> alpha[R];                                       // deferred pivot-row scales
#pragma unroll
    for (int j = 0; j < R; ++j) {
        const int i = row0 + j;
        lrow[j] = i < b ? i : INT_MAX;
        alpha[j] = cmk((T)1, (T)0);
#pragma unroll
        for (int v = 0; v < CPR; ++v) {
            VT a = {}, c = {};
            if (i < b) {
                a = reinterpret_cast<const VT*>(srow(0, i))[v];
                c = reinterpret_cast<const VT*>(srow(1, i))[v];
            }
#pragma unroll
            for (int e = 0; e < VW; ++e) {
                vr[j][v * VW + e] = reinterpret_cast<const T*>(&a)[e];
                vi[j][v * VW + e] = reinterpret_cast<const T*>(&c)[e];
            }
        }
    }
    // the previous step: its pivot row (shared memory), reciprocal, logical row and
    // this thread's factors
    const T* xp = cand_row[0][0];
    cplx<T> inv_p = cmk((T)0, (T)0);
    int pl_p = -1;
    cplx<T> f[R];
    bool isp[R];
#pragma unroll
    for (int j = 0; j < R; ++j) { f[j] = cmk((T)0, (T)0); isp[j] = false; }
    bool timed_out = false;
    // step s-1's transformation of element (j, k)
    auto upd = [&](int j, int k, T xr_, T xi_) {
        vr[j][k] = fma(-f[j].re, xr_, fma(f[j].im, xi_, vr[j][k]));
        vi[j][k] = fma(-f[j].re, xi_, fma(-f[j].im, xr_, vi[j][k]));
    };
    // one step of the pipeline; register column sp holds column s = g·GS + sp, and
    // register (sp + NB - 1) % NB column s - 1 (the registers rotate by GS per group)
    auto step = [&](const int g, const int sp, const bool last) {
        const int s = g * GS + sp;
        const int rprev = (sp + NB - 1) % NB;
        const bool prev = s > 0 && s - 1 < w;   // step s-1 to apply (uniform)
        const bool cur = !last && s < w;        // step s to search (uniform)
        const int slot = s % NS;
        const int cbase = g * GS;               // absolute column of register 0
        // 1. column s and the bookkeeping through step s-1
        if (prev) {
            if (!last) {
                const T xs_r = xp[s], xs_i = xp[NB + s];
#pragma unroll
                for (int j = 0; j < R; ++j) upd(j, sp, xs_r, xs_i);
            }
            const int rp = c0 + s - 1;
#pragma unroll
            for (int j = 0; j < R; ++j) {
                vr[j][rprev] = isp[j] ? (T)1 : -f[j].re;
                vi[j][rprev] = isp[j] ? (T)0 : -f[j].im;
                if (isp[j]) alpha[j] = inv_p;
                lrow[j] = (lrow[j] == rp) ? pl_p : (isp[j] ? rp : lrow[j]);
            }
        }
        if (cur) {
            // 2. pivot keys of column s
            const int r0 = c0 + s;
            unsigned key = 0;
#pragma unroll
            for (int j = 0; j < R; ++j)
                if (lrow[j] >= r0 && lrow[j] < b)
                    key = max(key, pivot_key((float)(fabs(vr[j][sp]) + fabs(vi[j][sp])), row0 + j));
            const unsigned wkey = __reduce_max_sync(0xffffffffu, key);
            // 3. publication (register k is column (cbase + k) mod NB)
            T* crow = cand_row[slot][warp];
            if (wkey != 0u) {
                const int wphys = pivot_key_row(wkey);
                if (lane == (wphys / R) % 32) {
                    const int jsel = wphys % R;
#pragma unroll
                    for (int j = 0; j < R; ++j) {
                        if (j == jsel) {
#pragma unroll
                            for (int v = 0; v < CPR; ++v) {
                                VT a, c;
#pragma unroll
                                for (int e = 0; e < VW; ++e) {
                                    reinterpret_cast<T*>(&a)[e] = vr[j][v * VW + e];
                                    reinterpret_cast<T*>(&c)[e] = vi[j][v * VW + e];
                                }
                                const int col = (cbase + v * VW) % NB;
                                *reinterpret_cast<VT*>(crow + col) = a;
                                *reinterpret_cast<VT*>(crow + NB + col) = c;
                            }
                            cand_inv[slot][warp] = cinv_pow2(cmk(vr[j][sp], vi[j][sp]));
                            cand_lrow[slot][warp] = lrow[j];
                            if (s > 0) cand_f[warp] = f[j];
                        }
                    }
                }
                if (s > 0) {
                    __syncwarp();
                    if (lane < NB && lane != s && lane != s - 1) {
                        const cplx<T> fw = cand_f[warp];
                        const T xr_ = xp[lane], xi_ = xp[NB + lane];
                        const T a = crow[lane], c = crow[NB + lane];
                        crow[lane] = fma(-fw.re, xr_, fma(fw.im, xi_, a));
                        crow[NB + lane] = fma(-fw.re, xi_, fma(-fw.im, xr_, c));
                    }
                }
            }
            if (lane == 0) cand_key[slot][warp] = wkey;
            __syncwarp();
            if (lane == 0) mbar_arrive(bar_a);
        }
        // 4. step s-1 on the other columns
        if (prev) {
#pragma unroll
            for (int v = 0; v < CPR; ++v) {
                const int col = (cbase + v * VW) % NB;
                const VT a = *reinterpret_cast<const VT*>(xp + col);
                const VT c = *reinterpret_cast<const VT*>(xp + NB + col);
                const T* ar = reinterpret_cast<const T*>(&a);
                const T* ci = reinterpret_cast<const T*>(&c);
#pragma unroll
                for (int e = 0; e < VW; e += 2) {
                    const int k = v * VW + e;
                    const bool u0 = (last || k != sp) && k != rprev;
                    const bool u1 = (last || k + 1 != sp) && k + 1 != rprev;
                    if constexpr (sizeof(T) == 4) {
                        if (u0 && u1) {   // both columns: paired FP32 fmas, same operations per element
                            const float2 x_r = make_float2(ar[e], ar[e + 1]), x_i = make_float2(ci[e], ci[e + 1]);
#pragma unroll
                            for (int j = 0; j < R; ++j) {
                                const float2 fim = make_float2(f[j].im, f[j].im);
                                const float2 nfr = make_float2(-f[j].re, -f[j].re);
                                const float2 nfi = make_float2(-f[j].im, -f[j].im);
                                float2 a2 = make_float2(vr[j][k], vr[j][k + 1]);
                                float2 c2 = make_float2(vi[j][k], vi[j][k + 1]);
                                a2 = __ffma2_rn(nfr, x_r, __ffma2_rn(fim, x_i, a2));
                                c2 = __ffma2_rn(nfr, x_i, __ffma2_rn(nfi, x_r, c2));
                                vr[j][k] = a2.x; vr[j][k + 1] = a2.y;
                                vi[j][k] = c2.x; vi[j][k + 1] = c2.y;
                            }
                            continue;
                        }
                    }
#pragma unroll
                    for (int j = 0; j < R; ++j) {
                        if (u0) upd(j, k, ar[e], ci[e]);
                        if (u1) upd(j, k + 1, ar[e + 1], ci[e + 1]);
                    }
                }
            }
        }
        if (cur) {
            // 5. every warp's candidate; the winner of step s
            if (!mbar_wait_spin(bar_a, (uint32_t)(s & 1), wait_ns) && !timed_out) {
                timed_out = true;
                dev_error(err, FDFD_DEVERR_TIMEOUT);
            }
            unsigned gkey = 0u;
#pragma unroll
            for (int q = 0; q < NWM / 4; ++q) {
                const uint4 kv = reinterpret_cast<const uint4*>(cand_key[slot])[q];
                gkey = max(gkey, max(max(kv.x, kv.y), max(kv.z, kv.w)));
            }
            const int ww = min(pivot_key_row(gkey) / (32 * R), NWM - 1);   // a warp holds 32*R consecutive rows
            xp = cand_row[slot][ww];
            pl_p = cand_lrow[slot][ww];
            const cplx<T> p = cmk(xp[s], xp[NB + s]);
            const bool bad = !(fabs(p.re) + fabs(p.im) > (T)0) || !isfinite(p.re) || !isfinite(p.im);
            if (bad && t == 0) dev_error(err, FDFD_DEVERR_SINGULAR);
            inv_p = bad ? cmk((T)0, (T)0) : cand_inv[slot][ww];
#pragma unroll
            for (int j = 0; j < R; ++j) {
                isp[j] = lrow[j] == pl_p;
                const cplx<T> fi = cmul(cmk(vr[j][sp], vi[j][sp]), inv_p);
                f[j] = isp[j] ? cmk((T)0, (T)0) : fi;
            }
        }
    };
#pragma unroll 1
    for (int g = 0; g < NG; ++g) {
#pragma unroll
        for (int sp = 0; sp < GS; ++sp) step(g, sp, false);
        if constexpr (NG > 1) {
            // rotate the register columns by GS: the next group's columns to 0 .. GS-1
#pragma unroll
            for (int j = 0; j < R; ++j)
#pragma unroll
                for (int c = 0; c < GS; ++c) {   // GS cycles of length NG: one value in flight
                    const T tr = vr[j][c], ti = vi[j][c];
#pragma unroll
                    for (int q = 0; q + 1 < NG; ++q) {
                        vr[j][c + q * GS] = vr[j][c + (q + 1) * GS];
                        vi[j][c + q * GS] = vi[j][c + (q + 1) * GS];
                    }
                    vr[j][c + (NG - 1) * GS] = tr;
                    vi[j][c + (NG - 1) * GS] = ti;
                }
        }
    }
    // the registers are back in column order; a full panel's last step is still to apply
    if (w == NB) step(NG, 0, true);
    // deferred pivot-row scales; the rows of G staged in logical order
#pragma unroll
    for (int j = 0; j < R; ++j) {
        if (lrow[j] >= b) continue;
        rsm[lrow[j]] = row0 + j;
#pragma unroll
        for (int v = 0; v < CPR; ++v) {
            VT a, c;
#pragma unroll
            for (int e = 0; e < VW; ++e) {
                const cplx<T> x = cmul(alpha[j], cmk(vr[j][v * VW + e], vi[j][v * VW + e]));
                reinterpret_cast<T*>(&a)[e] = x.re;
                reinterpret_cast<T*>(&c)[e] = x.im;
            }
            reinterpret_cast<VT*>(srow(0, lrow[j]))[v] = a;
            reinterpret_cast<VT*>(srow(1, lrow[j]))[v] = c;
        }
    }
    __syncthreads();
    int* rs = rowsrc + (size_t)job * b;
    int* pp = perm + (size_t)job * b;
    int rsv[R], pv[R];
#pragma unroll
    for (int u = 0; u < R; ++u) {
        const int i = t + u * NT;
        rsv[u] = i < b ? rsm[i] : 0;
        pv[u] = i < b ? pp[rsv[u]] : 0;
    }
    // G (b x NB; the update reads K = NB columns), coalesced
    {
        T* gp = GP.slot(job);
        const long long pe = GP.plane_elems();
        for (int idx = t; idx < b * CPR; idx += NT) {
            const int r = idx / CPR, v = idx % CPR;
            const VT a = reinterpret_cast<const VT*>(srow(0, r))[v];
            const VT c = reinterpret_cast<const VT*>(srow(1, r))[v];
            const long long o = (long long)r * GP.ld + v * VW;
            *reinterpret_cast<VT*>(gp + o) = a;
            *reinterpret_cast<VT*>(gp + pe + o) = c;
            if (GP.planes == 4) {   // pre-split tensor-core operand: TF32 residual planes
                VT al, cl;
#pragma unroll
                for (int e = 0; e < VW; ++e) {
                    reinterpret_cast<T*>(&al)[e] = (T)tf32_lo((float)reinterpret_cast<const T*>(&a)[e]);
                    reinterpret_cast<T*>(&cl)[e] = (T)tf32_lo((float)reinterpret_cast<const T*>(&c)[e]);
                }
                *reinterpret_cast<VT*>(gp + 2 * pe + o) = al;
                *reinterpret_cast<VT*>(gp + 3 * pe + o) = cl;
            }
        }
    }
    __syncthreads();   // every old perm entry is read before any is overwritten
#pragma unroll
    for (int u = 0; u < R; ++u) {
        const int i = t + u * NT;
        if (i < b) {
            pp[i] = pv[u];
            rs[i] = rsv[u];
        }
    }
}

// Gauss-Jordan panel step, cluster form, for levels with few matrices: the b x NB
// panel of one matrix is split by rows over the CL CTAs of a thread-block cluster
// (CL = 2, 4 or 8), so a level with n matrices keeps n·CL SMs busy instead of n.
// CTA rank cr holds the physical rows [cr·RPC, cr·RPC + RPC) (RPC = NT/4 · R);
// inside a CTA the layout is that of gj_panel_quad_kernel (lane quads share R
// rows, lane c of a quad holds columns [c·C, c·C + C)).  A column step: every warp
// publishes its best candidate row in its own CTA's shared memory and its key in
// the key table of every CTA of the cluster; one cluster barrier (release /
// acquire, so the published rows are visible cluster-wide); every thread takes
// the largest of the CL·NW keys and reads its C columns of the winning row, the
// reciprocal of the pivot and the pivot's logical row from the owning CTA through
// the cluster's shared-memory window.  Candidate slots alternate by step parity:
// the slot written at step j was last read at step j-2, before the barrier of
// step j-1.  Pivot keys, the reciprocal and the fma sequence are those of the quad
// kernel, so both forms give identical results.  grid: njobs·CL, block NT;
// requires b <= CL·RPC.
template <int CL> __device__ __forceinline__ void cluster_barrier() {
    if constexpr (CL > 1)
        asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
    else
        __syncthreads();
}
template <typename P> __device__ __forceinline__ P* cluster_peer(P* p, unsigned rank) {
    return static_cast<P*>(__cluster_map_shared_rank((void*)p, rank));
}

template <typename T, int NB, int R, int NT, int CL>
__global__ void __cluster_dims__(CL, 1, 1) __launch_bounds__(NT)
    gj_panel_cl_kernel(Pool<T> M, const int* slots, Pool<T> GP, int* perm, int* rowsrc, int c0, unsigned* err) {
    constexpr int NW = NT / 32, C = NB / 4, RPC = NT / 4 * R;
    constexpr int VW = 16 / sizeof(T);
    constexpr int NK = CL * NW;                       // keys per step, cluster-wide
    static_assert(C % VW == 0 && (R & (R - 1)) == 0 && NK % 4 == 0 && NT % 32 == 0, "cluster panel tiling");
    typedef typename Vec16<T>::type VT;
    __shared__ __align__(16) T cand_row[2][NW][2 * NB];   // [parity][warp][re | im]
    __shared__ __align__(16) unsigned cand_key[2][NK];    // [parity][rank * NW + warp]
    __shared__ cplx<T> cand_inv[2][NW];
    __shared__ int cand_lrow[2][NW];
    __shared__ int rsm[CL * RPC];                          // composed row exchanges, every row of the matrix
    const int b = M.rows;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const int qc = lane & 3;                         // column block of this lane
    const int qbase = lane & ~3;                     // first lane of the quad
    unsigned cr;
    asm("mov.u32 %0, %%cluster_ctarank;" : "=r"(cr));
    const int rbase = (int)cr * RPC;                 // first physical row of this CTA
    const int row0 = rbase + (warp * 8 + (lane >> 2)) * R;
    const int job = blockIdx.x / CL;
    const T* Mre = M.slot(slots[job]);
    const T* Mim = Mre + M.plane_elems();
    const int ld = M.ld;
    const int w = min(NB, b - c0);
    T vr[R][C], vi[R][C];
    int lrow[R];
    cplx<T> alpha[R];                                // deferred pivot-row scales
#pragma unroll
    for (int j = 0; j < R; ++j) {
        const int i = row0 + j;
        lrow[j] = i < b ? i : INT_MAX;
        alpha[j] = cmk((T)1, (T)0);
#pragma unroll
        for (int v = 0; v < C / VW; ++v) {
            const int col = qc * C + v * VW;
            VT a = {}, c = {};
            if (i < b && col < w) {   // c0 + NB <= ld: the vector stays in the row
                a = *reinterpret_cast<const VT*>(Mre + (size_t)i * ld + c0 + col);
                c = *reinterpret_cast<const VT*>(Mim + (size_t)i * ld + c0 + col);
            }
#pragma unroll
            for (int e = 0; e < VW; ++e) {
                const bool ok = i < b && col + e < w;
                vr[j][v * VW + e] = ok ? reinterpret_cast<const T*>(&a)[e] : (T)0;
                vi[j][v * VW + e] = ok ? reinterpret_cast<const T*>(&c)[e] : (T)0;
            }
        }
    }
    // every CTA of the cluster runs before its shared memory is written remotely
    cluster_barrier<CL>();
#pragma unroll 1
    for (int g = 0; g * C < w; ++g) {
#pragma unroll
        for (int sp = 0; sp < C; ++sp) {
            const int jj = g * C + sp;
            if (jj < w) {   // uniform
                const int r0 = c0 + jj;
                const int par = jj & 1;
                unsigned key = 0;
                if (qc == g) {
#pragma unroll
                    for (int j = 0; j < R; ++j)
                        if (lrow[j] >= r0 && lrow[j] < b)
                            key = max(key, pivot_key((float)(fabs(vr[j][sp]) + fabs(vi[j][sp])), row0 + j));
                }
                const unsigned wkey = __reduce_max_sync(0xffffffffu, key);
                if (wkey != 0u) {
                    const int wphys = pivot_key_row(wkey) - rbase;
                    const int wq = (wphys / R) & 7, jsel = wphys & (R - 1);
                    if ((lane >> 2) == wq) {
                        T* crow = cand_row[par][warp];
#pragma unroll
                        for (int j = 0; j < R; ++j) {
                            if (j == jsel) {
#pragma unroll
                                for (int v = 0; v < C / VW; ++v) {
                                    VT a, c;
#pragma unroll
                                    for (int e = 0; e < VW; ++e) {
                                        reinterpret_cast<T*>(&a)[e] = vr[j][v * VW + e];
                                        reinterpret_cast<T*>(&c)[e] = vi[j][v * VW + e];
                                    }
                                    reinterpret_cast<VT*>(crow + qc * C)[v] = a;
                                    reinterpret_cast<VT*>(crow + NB + qc * C)[v] = c;
                                }
                                if (qc == g) {
                                    cand_inv[par][warp] = cinv_pow2(cmk(vr[j][sp], vi[j][sp]));
                                    cand_lrow[par][warp] = lrow[j];
                                }
                            }
                        }
                    }
                }
                // the warp's key into the key table of every CTA (lane d writes CTA d's)
                if (lane < CL) *cluster_peer(&cand_key[par][cr * NW + warp], (unsigned)lane) = wkey;
                cluster_barrier<CL>();
                unsigned gkey = 0u;
#pragma unroll
                for (int q = 0; q < NK / 4; ++q) {
                    const uint4 kv = reinterpret_cast<const uint4*>(cand_key[par])[q];
                    gkey = max(gkey, max(max(kv.x, kv.y), max(kv.z, kv.w)));
                }
                const int wrow = pivot_key_row(gkey);
                // CTA holding the pivot row and its warp (wrow < b whenever a key is set: the
                // holder of logical row r0 always is a candidate; the clamps only bound the ranks)
                const unsigned wc = (unsigned)min(wrow / RPC, CL - 1);
                const int ww = min((wrow - (int)wc * RPC) / (8 * R), NW - 1);
                const T* pr = cluster_peer(cand_row[par][ww], wc);
                const int pl = *cluster_peer(&cand_lrow[par][ww], wc);
                const cplx<T> p = cmk(pr[jj], pr[NB + jj]);
                const bool bad = !(fabs(p.re) + fabs(p.im) > (T)0) || !isfinite(p.re) || !isfinite(p.im);
                if (bad && t == 0 && cr == 0) dev_error(err, FDFD_DEVERR_SINGULAR);
                const cplx<T> inv = bad ? cmk((T)0, (T)0) : *cluster_peer(&cand_inv[par][ww], wc);
                cplx<T> f[R];
                bool isp[R];
#pragma unroll
                for (int j = 0; j < R; ++j) {
                    const T cr_ = __shfl_sync(0xffffffffu, vr[j][sp], qbase + g);
                    const T ci_ = __shfl_sync(0xffffffffu, vi[j][sp], qbase + g);
                    isp[j] = lrow[j] == pl;
                    const cplx<T> fi = cmul(cmk(cr_, ci_), inv);
                    f[j] = isp[j] ? cmk((T)0, (T)0) : fi;
                }
                T xr[C], xi[C];
#pragma unroll
                for (int v = 0; v < C / VW; ++v) {
                    const VT a = reinterpret_cast<const VT*>(pr + qc * C)[v];
                    const VT c = reinterpret_cast<const VT*>(pr + NB + qc * C)[v];
#pragma unroll
                    for (int e = 0; e < VW; ++e) {
                        xr[v * VW + e] = reinterpret_cast<const T*>(&a)[e];
                        xi[v * VW + e] = reinterpret_cast<const T*>(&c)[e];
                    }
                }
                if constexpr (sizeof(T) == 4 && C % 2 == 0) {
#pragma unroll
                    for (int j = 0; j < R; ++j) {
                        const float2 fim = make_float2(f[j].im, f[j].im), nfr = make_float2(-f[j].re, -f[j].re);
                        const float2 nfi = make_float2(-f[j].im, -f[j].im);
#pragma unroll
                        for (int k = 0; k < C; k += 2) {
                            const float2 x_r = make_float2(xr[k], xr[k + 1]), x_i = make_float2(xi[k], xi[k + 1]);
                            float2 a = make_float2(vr[j][k], vr[j][k + 1]), c = make_float2(vi[j][k], vi[j][k + 1]);
                            a = __ffma2_rn(nfr, x_r, __ffma2_rn(fim, x_i, a));
                            c = __ffma2_rn(nfr, x_i, __ffma2_rn(nfi, x_r, c));
                            vr[j][k] = a.x; vr[j][k + 1] = a.y;
                            vi[j][k] = c.x; vi[j][k + 1] = c.y;
                        }
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < R; ++j)
#pragma unroll
                        for (int k = 0; k < C; ++k) {
                            vr[j][k] = fma(-f[j].re, xr[k], fma(f[j].im, xi[k], vr[j][k]));
                            vi[j][k] = fma(-f[j].re, xi[k], fma(-f[j].im, xr[k], vi[j][k]));
                        }
                }
#pragma unroll
                for (int j = 0; j < R; ++j) {
                    if (qc == g) {
                        vr[j][sp] = isp[j] ? (T)1 : -f[j].re;
                        vi[j][sp] = isp[j] ? (T)0 : -f[j].im;
                    }
                    if (isp[j]) alpha[j] = inv;
                    lrow[j] = (lrow[j] == r0) ? pl : (isp[j] ? r0 : lrow[j]);
                }
            }
        }
    }
#pragma unroll
    for (int j = 0; j < R; ++j)
#pragma unroll
        for (int k = 0; k < C; ++k) {
            const cplx<T> x = cmul(alpha[j], cmk(vr[j][k], vi[j][k]));
            vr[j][k] = x.re;
            vi[j][k] = x.im;
        }
    // the composed row exchanges into every CTA's table (row r of the exchanged
    // matrix is row rsm[r] of M); the barrier also ends the last step's remote reads
    for (int d = qc; d < CL; d += 4) {   // the quad's lanes share the stores to the CL tables
#pragma unroll
        for (int j = 0; j < R; ++j)
            if (lrow[j] < b) *cluster_peer(&rsm[lrow[j]], (unsigned)d) = row0 + j;
    }
    cluster_barrier<CL>();
    int* rs = rowsrc + (size_t)job * b;
    int* pp = perm + (size_t)job * b;
    constexpr int PPT = (RPC + NT - 1) / NT;         // bookkeeping rows per thread (this CTA's slice)
    const int iend = min(b, rbase + RPC);
    int rsv[PPT], pv[PPT];
#pragma unroll
    for (int u = 0; u < PPT; ++u) {
        const int i = rbase + t + u * NT;
        rsv[u] = i < iend ? rsm[i] : 0;
        pv[u] = i < iend ? pp[rsv[u]] : 0;
    }
    {
        T* gp = GP.slot(job);
        const long long pe = GP.plane_elems();
#pragma unroll
        for (int j = 0; j < R; ++j) {
            if (lrow[j] >= b) continue;
            const long long o = (long long)lrow[j] * GP.ld;
#pragma unroll
            for (int v = 0; v < C / VW; ++v) {
                VT a, c;
#pragma unroll
                for (int e = 0; e < VW; ++e) {
                    reinterpret_cast<T*>(&a)[e] = vr[j][v * VW + e];
                    reinterpret_cast<T*>(&c)[e] = vi[j][v * VW + e];
                }
                const int col = qc * C + v * VW;
                *reinterpret_cast<VT*>(gp + o + col) = a;
                *reinterpret_cast<VT*>(gp + pe + o + col) = c;
                if (GP.planes == 4) {   // pre-split tensor-core operand: TF32 residual planes
                    VT al, cl;
#pragma unroll
                    for (int e = 0; e < VW; ++e) {
                        reinterpret_cast<T*>(&al)[e] = (T)tf32_lo((float)reinterpret_cast<const T*>(&a)[e]);
                        reinterpret_cast<T*>(&cl)[e] = (T)tf32_lo((float)reinterpret_cast<const T*>(&c)[e]);
                    }
                    *reinterpret_cast<VT*>(gp + 2 * pe + o + col) = al;
                    *reinterpret_cast<VT*>(gp + 3 * pe + o + col) = cl;
                }
            }
        }
    }
    cluster_barrier<CL>();   // every old perm entry is read, cluster-wide, before any is overwritten
#pragma unroll
    for (int u = 0; u < PPT; ++u) {
        const int i = rbase + t + u * NT;
        if (i < iend) {
            pp[i] = pv[u];
            rs[i] = rsv[u];
        }
    }
}

// Dst[r][perm[j]] = Src[r][j] per row (through shared memory, so Src may be Dst).
// grid: (ceil(b/8), njobs), block 256
template <typename T>
__global__ void gj_unpermute_kernel(Pool<T> Src, const int* sslots, Pool<T> Dst, const int* dslots,
                                    const int* perm) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int b = Src.rows;
    T* rre = reinterpret_cast<T*>(smem_raw);
    T* rim = rre + b;
    const int job = blockIdx.y;
    const T* sb = Src.slot(sslots[job]);
    T* db = Dst.slot(dslots[job]);
    const long long spe = Src.plane_elems();
    const int* pp = perm + (size_t)job * b;
    const int rows_per = 8;
    for (int rr = 0; rr < rows_per; ++rr) {
        const int r = blockIdx.x * rows_per + rr;
        if (r >= b) break;
        for (int j = threadIdx.x; j < b; j += blockDim.x) {
            rre[j] = sb[(size_t)r * Src.ld + j];
            rim[j] = sb[spe + (size_t)r * Src.ld + j];
        }
        __syncthreads();
        for (int j = threadIdx.x; j < b; j += blockDim.x) store_elem<T>(Dst, db, r, pp[j], cmk(rre[j], rim[j]), 0);
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
// Inverse of the cyclic tridiagonal blocks of the first reduction step, O(b²).
//
// D_k = T0 + a0·e_0·e_{b-1}ᵀ + cN·e_{b-1}·e_0ᵀ with T0 tridiagonal (the in-line
// neighbours without the periodic wrap) and the two corner terms of the wrap.
// With Z = T0⁻¹ the Sherman-Morrison-Woodbury identity gives
//     D_k⁻¹ = Z − [z0, zN] · W,   W = S⁻¹ [a0·Z[b−1,:] ; cN·Z[0,:]],
//     S = I + [[a0 z0[b−1], a0 zN[b−1]], [cN z0[0], cN zN[0]]],
// z0 = Z[:,0], zN = Z[:,b−1].  Two kernels:
//  * tri_factor_kernel, a warp per node, all in shared memory: lane 0 factors T0 with partial
//    pivoting by the recurrences of LAPACK's xGTTRF (row interchanges between
//    neighbours, a second superdiagonal du2); lanes 0-3 then solve for the two
//    columns z0, zN (xGTTRS recurrences) and the two rows Z[0,:], Z[b−1,:]
//    (the transposed recurrences, solving T0ᵀ x = e); all lanes form W.
//  * tri_columns_kernel, a thread per column j: Z[:,j] by the forward and
//    backward recurrences (the forward one starts at row j−1: rows above are
//    zero), the Woodbury correction applied as each row is finished, and the
//    column of G = D_k⁻¹ written once (re and im: these inverses are never GEMM operands).
// Factor workspace per node (cplx<T>): [dl | du | du2 | dinv | z0 | zN | w0 | w1],
// b entries each; ipiv: b ints per node.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(32) tri_factor_kernel(NodeMap m, const cplx<double>* st, double scale,
                                                        const int* nodes, cplx<T>* fac, int* piv, unsigned* err) {
    // everything runs out of shared memory: the serial recurrences then wait on
    // shared-memory latency, not on global loads.  Layout (cplx<T>, b each):
    // dl, du, du2, dinv, z0, zN, w0, w1, then ipiv (b ints)
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int b = m.b;
    cplx<T>* dl = reinterpret_cast<cplx<T>*>(smem_raw);
    cplx<T>* du = dl + b;
    cplx<T>* du2 = du + b;
    cplx<T>* dinv = du2 + b;
    cplx<T>* z0 = dinv + b;
    cplx<T>* zN = z0 + b;
    cplx<T>* w0 = zN + b;
    cplx<T>* w1 = w0 + b;
    int* ipiv = reinterpret_cast<int*>(w1 + b);
    const int job = blockIdx.x;
    const int lane = threadIdx.x;
    const int node = nodes[job];
    auto coef = [&](int plane, int i) {
        const cplx<double> v = cscale(st_at<T>(st, m, plane, node, i), scale);
        return cmk((T)v.re, (T)v.im);
    };
    const cplx<T> z = cmk((T)0, (T)0);
    // T0 into shared memory: diagonal (in dinv), sub-diagonal T0[i+1][i] (in dl),
    // super-diagonal T0[i][i+1] (in du)
    for (int i = lane; i < b; i += 32) {
        dinv[i] = coef(0, i);
        dl[i] = i + 1 < b ? coef(m.p_inprev(), i + 1) : z;
        du[i] = i + 1 < b ? coef(m.p_innext(), i) : z;
        du2[i] = z;
    }
    __syncwarp();
    if (lane == 0) {
        // xGTTRF recurrences; the diagonal is replaced by the reciprocals of its final entries
        int bad = 0;
        cplx<T> d = dinv[0];
        for (int i = 0; i + 1 < b; ++i) {
            cplx<T> lo = dl[i];
            cplx<T> dn = dinv[i + 1];
            const cplx<T> upper = du[i];
            int ip = i;
            if (cabs1(d) >= cabs1(lo)) {
                cplx<T> fact = z;
                if (cabs1(d) > (T)0) {
                    fact = cmul(lo, cinv_pow2(d));
                    dn = csub(dn, cmul(fact, upper));
                }
                lo = fact;
            } else {
                const cplx<T> fact = cmul(d, cinv_pow2(lo));
                d = lo;
                du[i] = dn;
                dn = csub(upper, cmul(fact, dn));
                if (i + 2 < b) {
                    du2[i] = du[i + 1];
                    du[i + 1] = cneg(cmul(fact, du[i + 1]));
                }
                lo = fact;
                ip = i + 1;
            }
            if (!(cabs1(d) > (T)0) || !isfinite((double)cabs1(d))) { bad = 1; d = cmk((T)1, (T)0); }
            dl[i] = lo;
            dinv[i] = cinv_pow2(d);
            ipiv[i] = ip;
            d = dn;
        }
        if (!(cabs1(d) > (T)0) || !isfinite((double)cabs1(d))) { bad = 1; d = cmk((T)1, (T)0); }
        dl[b - 1] = z;
        du[b - 1] = z;
        dinv[b - 1] = cinv_pow2(d);
        ipiv[b - 1] = b - 1;
        if (bad) dev_error(err, FDFD_DEVERR_SINGULAR);
    }
    __syncwarp();
    // two columns (lanes 0, 1: T0 x = e_0, e_{b-1}) and two rows (lanes 2, 3:
    // T0ᵀ x = e_0, e_{b-1}); results in z0, zN, w1 (row 0), w0 (row b-1)
    for (int i = lane; i < b; i += 32) {
        z0[i] = cmk((T)(i == 0 ? 1 : 0), (T)0);
        zN[i] = cmk((T)(i == b - 1 ? 1 : 0), (T)0);
        w1[i] = z0[i];
        w0[i] = zN[i];
    }
    __syncwarp();
    if (lane < 4) {
        cplx<T>* x = lane == 0 ? z0 : (lane == 1 ? zN : (lane == 2 ? w1 : w0));
        if (lane < 2) {
            // L y = e (interchanges between neighbours), then U x = y
            for (int i = 0; i + 1 < b; ++i) {
                if (ipiv[i] == i) {
                    x[i + 1] = csub(x[i + 1], cmul(dl[i], x[i]));
                } else {
                    const cplx<T> t = x[i];
                    x[i] = x[i + 1];
                    x[i + 1] = csub(t, cmul(dl[i], x[i]));
                }
            }
            cplx<T> x1 = cmul(x[b - 1], dinv[b - 1]), x2 = z;
            x[b - 1] = x1;
            for (int i = b - 2; i >= 0; --i) {
                const cplx<T> xi = cmul(csub(csub(x[i], cmul(du[i], x1)), cmul(du2[i], x2)), dinv[i]);
                x[i] = xi;
                x2 = x1;
                x1 = xi;
            }
        } else {
            // Uᵀ y = e, then Lᵀ x = y (interchanges applied in reverse)
            cplx<T> y1 = cmul(x[0], dinv[0]), y2 = z;   // y[i-1], y[i-2]
            x[0] = y1;
            for (int i = 1; i < b; ++i) {
                cplx<T> yi = csub(x[i], cmul(du[i - 1], y1));
                if (i >= 2) yi = csub(yi, cmul(du2[i - 2], y2));
                yi = cmul(yi, dinv[i]);
                x[i] = yi;
                y2 = y1;
                y1 = yi;
            }
            for (int i = b - 2; i >= 0; --i) {
                if (ipiv[i] == i) {
                    x[i] = csub(x[i], cmul(dl[i], x[i + 1]));
                } else {
                    const cplx<T> t = x[i + 1];
                    x[i + 1] = csub(x[i], cmul(dl[i], t));
                    x[i] = t;
                }
            }
        }
    }
    __syncwarp();
    // W = S⁻¹ [a0·Z[b−1,:]; cN·Z[0,:]] (w0 holds Z[b−1,:], w1 holds Z[0,:])
    const cplx<T> a0 = coef(m.p_inprev(), 0);        // D[0][b-1]
    const cplx<T> cN = coef(m.p_innext(), b - 1);    // D[b-1][0]
    const cplx<T> one = cmk((T)1, (T)0);
    const cplx<T> s00 = cadd(one, cmul(a0, z0[b - 1]));
    const cplx<T> s01 = cmul(a0, zN[b - 1]);
    const cplx<T> s10 = cmul(cN, z0[0]);
    const cplx<T> s11 = cadd(one, cmul(cN, zN[0]));
    const cplx<T> det = csub(cmul(s00, s11), cmul(s01, s10));
    const bool dbad = !(cabs1(det) > (T)0) || !isfinite((double)cabs1(det));
    if (dbad && lane == 0) dev_error(err, FDFD_DEVERR_SINGULAR);
    const cplx<T> id = dbad ? z : cinv_pow2(det);
    const cplx<T> i00 = cmul(s11, id), i01 = cneg(cmul(s01, id));
    const cplx<T> i10 = cneg(cmul(s10, id)), i11 = cmul(s00, id);
    __syncwarp();
    for (int j = lane; j < b; j += 32) {
        const cplx<T> v0 = cmul(a0, w0[j]), v1 = cmul(cN, w1[j]);
        w0[j] = cadd(cmul(i00, v0), cmul(i01, v1));
        w1[j] = cadd(cmul(i10, v0), cmul(i11, v1));
    }
    __syncwarp();
    // the node's factors to global memory (coalesced)
    cplx<T>* f = fac + (size_t)job * 8 * b;
    for (int i = lane; i < 8 * b; i += 32) f[i] = dl[i];
    for (int i = lane; i < b; i += 32) piv[(size_t)job * b + i] = ipiv[i];
}

// G[:, j] = Z[:, j] − z0·w0[j] − zN·w1[j] with Z[:, j] = T0⁻¹ e_j; the factor
// arrays of the node are staged in shared memory (read by every thread in the
// same order).  grid: (ceil(b/128), njobs), block 128,
// dynamic smem 6*b*sizeof(cplx<T>) + b*sizeof(int)
template <typename T>
__global__ void __launch_bounds__(128) tri_columns_kernel(int b, Pool<T> D, const int* nodes, const cplx<T>* fac,
                                                          const int* piv) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cplx<T>* s_dl = reinterpret_cast<cplx<T>*>(smem_raw);
    cplx<T>* s_du = s_dl + b;
    cplx<T>* s_du2 = s_du + b;
    cplx<T>* s_dinv = s_du2 + b;
    cplx<T>* s_z0 = s_dinv + b;
    cplx<T>* s_zN = s_z0 + b;
    int* s_piv = reinterpret_cast<int*>(s_zN + b);
    const int job = blockIdx.y;
    const cplx<T>* f = fac + (size_t)job * 8 * b;
    for (int i = threadIdx.x; i < 6 * b; i += blockDim.x) s_dl[i] = f[i];
    for (int i = threadIdx.x; i < b; i += blockDim.x) s_piv[i] = piv[(size_t)job * b + i];
    __syncthreads();
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= b) return;
    const cplx<T> w0 = f[6 * b + j], w1 = f[7 * b + j];
    T* Gre = D.slot(nodes[job]);
    const long long pe = D.plane_elems();
    T* Gim = Gre + pe;
    const int ld = D.ld;
    // rows above j-1 of L⁻¹ e_j are zero.  The forward recurrence starts at the
    // same row for the whole warp (its first column's j-1): a lane whose unit
    // entry comes later carries zeros until then, and the warp's stores of a
    // row stay one coalesced segment.
    const int jw = j & ~31;
    const int i0 = jw > 0 ? jw - 1 : 0;
    // forward: y = L⁻¹ e_j, rows i0 .. b-2 stored in G (as scratch)
    cplx<T> cur = cmk((T)(j == i0 ? 1 : 0), (T)0);
    for (int i = i0; i + 1 < b; ++i) {
        cplx<T> nxt = cmk((T)(i + 1 == j ? 1 : 0), (T)0);
        cplx<T> yi;
        if (s_piv[i] == i) {
            yi = cur;
            nxt = csub(nxt, cmul(s_dl[i], cur));
        } else {
            yi = nxt;
            nxt = csub(cur, cmul(s_dl[i], nxt));
        }
        Gre[(size_t)i * ld + j] = yi.re;
        Gim[(size_t)i * ld + j] = yi.im;
        cur = nxt;
    }
    // backward: x = U⁻¹ y, each finished row corrected and written with all planes
    auto put = [&](int r, cplx<T> x) {
        const cplx<T> g = csub(csub(x, cmul(s_z0[r], w0)), cmul(s_zN[r], w1));
        store_elem<T>(D, Gre, r, j, g, 0);
    };
    cplx<T> x1 = cmul(cur, s_dinv[b - 1]);     // x[b-1]
    put(b - 1, x1);
    cplx<T> x2 = cmk((T)0, (T)0);             // x[i+2]
    int i = b - 2;
    while (i >= 0) {
        const int n8 = min(8, i + 1);
        cplx<T> yv[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int r = i - u;
            yv[u] = cmk((T)0, (T)0);
            if (u < n8 && r >= i0) yv[u] = cmk(Gre[(size_t)r * ld + j], Gim[(size_t)r * ld + j]);
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            if (u < n8) {
                const int r = i - u;
                const cplx<T> sr = csub(csub(yv[u], cmul(s_du[r], x1)), cmul(s_du2[r], x2));
                const cplx<T> xr = cmul(sr, s_dinv[r]);
                put(r, xr);
                x2 = x1;
                x1 = xr;
            }
        }
        i -= n8;
    }
}

// ---------------------------------------------------------------------------
// Host launchers
// ---------------------------------------------------------------------------
template <typename T>
void launch_tri_inverse(cudaStream_t s, int njobs, NodeMap m, const cplx<double>* st, double scale, Pool<T> D,
                        const int* nodes, cplx<T>* fac, int* piv, unsigned* err) {
    // both kernels opt in once (thread-safe static initialisation) to the shared memory of
    // the largest block, b = 1024: above 48 KB they must opt in
    static const bool opted = [] {
        const size_t mx = 8 * (size_t)1024 * sizeof(cplx<T>) + (size_t)1024 * sizeof(int);
        return cudaFuncSetAttribute(tri_factor_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mx) ==
                   cudaSuccess &&
               cudaFuncSetAttribute(tri_columns_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mx) ==
                   cudaSuccess;
    }();
    (void)opted;
    const size_t fsmem = 8 * (size_t)m.b * sizeof(cplx<T>) + (size_t)m.b * sizeof(int);
    tri_factor_kernel<T><<<njobs, 32, fsmem, s>>>(m, st, scale, nodes, fac, piv, err);
    const size_t smem = 6 * (size_t)m.b * sizeof(cplx<T>) + (size_t)m.b * sizeof(int);
    tri_columns_kernel<T><<<dim3(ceil_div(m.b, 128), njobs), 128, smem, s>>>(m.b, D, nodes, fac, piv);
}
template <typename T>
void launch_build_tridiag(cudaStream_t s, int njobs, NodeMap m, const cplx<double>* st, double scale, Pool<T> D,
                          const int* nodes) {
    build_tridiag_kernel<T><<<dim3(ceil_div((long long)m.b * m.b, 256), njobs), 256, 0, s>>>(m, st, scale, D, nodes);
}
template <typename T>
void launch_level1_combine(cudaStream_t s, int njobs, NodeMap m, const cplx<double>* st, double scale, Pool<T> D,
                           Pool<T> C, const L1Job* jobs, cplx<T>* tab) {
    stencil_table_kernel<T><<<dim3(ceil_div(m.b, 256), m.n), 256, 0, s>>>(m, st, scale, tab);
    const size_t smem = level1_combine_smem<T>();
    static const cudaError_t attr =
        cudaFuncSetAttribute(level1_combine_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    (void)attr;
    level1_combine_kernel<T><<<dim3(ceil_div(m.b, 128), ceil_div(m.b, L1_TR), njobs), 256, smem, s>>>(m, tab, D, C,
                                                                                                     jobs);
}
void launch_perm_init(cudaStream_t s, int njobs, int* perm, int b) {
    perm_init_kernel<int><<<dim3(ceil_div(b, 256), njobs), 256, 0, s>>>(perm, b);
}
template <typename T, int NB, int R, int C>
static int gj_panel_launch(cudaStream_t s, int njobs, Pool<T> M, const int* slots, Pool<T> GP, int* perm,
                           int* rowsrc, int c0, unsigned* err) {
    const size_t smem = gj_panel_smem_elems<NB, R>() * sizeof(T);
    static const cudaError_t attr =
        cudaFuncSetAttribute(gj_panel_kernel<T, NB, R, C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (attr != cudaSuccess) return (int)attr;
    gj_panel_kernel<T, NB, R, C><<<njobs, 512, smem, s>>>(M, slots, GP, perm, rowsrc, c0, err);
    return (int)cudaGetLastError();
}

// cluster form with CL CTAs per matrix, R = 4 rows per lane quad: NT = bmax / CL
// threads for matrices of up to bmax rows
template <typename T, int NB, int R>
static int gj_panel_row_launch(cudaStream_t s, int njobs, Pool<T> M, const int* slots, Pool<T> GP, int* perm,
                               int* rowsrc, int c0, unsigned* err, uint64_t wait_ns) {
    const int nt = ceil_div(M.rows, 32 * R) * 32;
    if (nt > 512) return (int)cudaErrorInvalidValue;
    static const cudaError_t attr = cudaFuncSetAttribute(gj_panel_row_kernel<T, NB, R>,
                                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                         (int)gj_panel_row_smem<T, NB>(512 * R));
    if (attr != cudaSuccess) return (int)attr;
    gj_panel_row_kernel<T, NB, R><<<njobs, nt, gj_panel_row_smem<T, NB>(nt * R), s>>>(M, slots, GP, perm, rowsrc,
                                                                                     c0, err, wait_ns);
    return (int)cudaGetLastError();
}

template <typename T, int NB, int CL, int BMAX>
static int gj_panel_cl_launch(cudaStream_t s, int njobs, Pool<T> M, const int* slots, Pool<T> GP, int* perm,
                              int* rowsrc, int c0, unsigned* err) {
    constexpr int NT = BMAX / CL;
    gj_panel_cl_kernel<T, NB, 4, NT, CL><<<njobs * CL, NT, 0, s>>>(M, slots, GP, perm, rowsrc, c0, err);
    return (int)cudaGetLastError();
}

template <typename T>
int launch_gj_panel(cudaStream_t s, int nb, int njobs, Pool<T> M, const int* slots, Pool<T> GP, int* perm,
                    int* rowsrc, int c0, unsigned* err, GjFuse fz, int cl, int form, uint64_t wait_ns) {
    const bool two = M.rows > 512;
    if (M.rows > 1024) return (int)cudaErrorInvalidValue;
    if (form == 1 && cl <= 1 && !fz.fused) {
        // row form: panel widths as in the other forms, one row per thread up to 512 rows
        constexpr int NBS = sizeof(T) == 4 ? 32 : 16, NBT = NBS / 2;
        if (!two && nb == NBS) return gj_panel_row_launch<T, NBS, 1>(s, njobs, M, slots, GP, perm, rowsrc, c0, err, wait_ns);
        if (two && nb == NBT) return gj_panel_row_launch<T, NBT, 2>(s, njobs, M, slots, GP, perm, rowsrc, c0, err, wait_ns);
        return (int)cudaErrorInvalidValue;
    }
    if (cl > 1 && !fz.fused) {
        // panel widths as in the single-CTA forms: 32 / 16 (FP32), 16 / 8 (FP64)
        constexpr int NBS = sizeof(T) == 4 ? 32 : 16, NBT = NBS / 2;
        if (!two && nb == NBS) {
            if (cl == 2) return gj_panel_cl_launch<T, NBS, 2, 512>(s, njobs, M, slots, GP, perm, rowsrc, c0, err);
            if (cl == 4) return gj_panel_cl_launch<T, NBS, 4, 512>(s, njobs, M, slots, GP, perm, rowsrc, c0, err);
            if (cl == 8) return gj_panel_cl_launch<T, NBS, 8, 512>(s, njobs, M, slots, GP, perm, rowsrc, c0, err);
        }
        if (two && nb == NBT) {
            if (cl == 2) return gj_panel_cl_launch<T, NBT, 2, 1024>(s, njobs, M, slots, GP, perm, rowsrc, c0, err);
            if (cl == 4) return gj_panel_cl_launch<T, NBT, 4, 1024>(s, njobs, M, slots, GP, perm, rowsrc, c0, err);
            if (cl == 8) return gj_panel_cl_launch<T, NBT, 8, 1024>(s, njobs, M, slots, GP, perm, rowsrc, c0, err);
        }
        return (int)cudaErrorInvalidValue;
    }
    // lane-quad form: one barrier per column step; four rows per quad up to b = 512,
    // eight (with the half-width panel) up to 1024 in FP32
    constexpr int NB1 = sizeof(T) == 4 ? 32 : 16;
    if (!two && nb == NB1) {
        gj_panel_quad_kernel<T, NB1, 4><<<njobs, 512, 0, s>>>(M, slots, GP, perm, rowsrc, c0, err, fz);
        return (int)cudaGetLastError();
    }
    if constexpr (sizeof(T) == 4) {
        if (two && nb == 16) {
            gj_panel_quad_kernel<T, 16, 8><<<njobs, 512, 0, s>>>(M, slots, GP, perm, rowsrc, c0, err, fz);
            return (int)cudaGetLastError();
        }
    } else {
        // FP64 with eight rows per quad would spill (its per-row scale factors alone take 32
        // registers): the 2-D tiled kernel keeps those in shared memory
        if (fz.fused) return (int)cudaErrorInvalidValue;   // fused super-panels: lane-quad kernels only
        if (two && nb == 8) return gj_panel_launch<T, 8, 8, 2>(s, njobs, M, slots, GP, perm, rowsrc, c0, err);
    }
    return (int)cudaErrorInvalidValue;
}
template <typename T>
int launch_gj_rt(cudaStream_t s, int nb, int njobs, Pool<T> M, const int* slots, Pool<T> RP, const int* rowsrc,
                 int c0, int rcw) {
    const dim3 grid(ceil_div(M.rows, 128), njobs);
    if (rcw <= 0 || rcw > RP.cols) rcw = RP.cols;
    // a few matrices: 32-column tiles, four times the CTAs for the latency-bound gather
    static const int nsm = [] {
        int d = 0, n = 0;
        cudaGetDevice(&d);
        return cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, d) == cudaSuccess && n > 0 ? n : 1;
    }();
    if (nb == 32 && (long long)ceil_div(M.rows, 32) * njobs <= 2LL * nsm) {
        gj_rt_kernel<T, 32, 32><<<dim3(ceil_div(M.rows, 32), njobs), 512, 0, s>>>(M, slots, RP, rowsrc, c0, rcw);
        return (int)cudaGetLastError();
    }
    if (nb == 32) gj_rt_kernel<T, 32><<<grid, 512, 0, s>>>(M, slots, RP, rowsrc, c0, rcw);
    else if (nb == 16) gj_rt_kernel<T, 16><<<grid, 512, 0, s>>>(M, slots, RP, rowsrc, c0, rcw);
    else if (nb == 8) gj_rt_kernel<T, 8><<<grid, 512, 0, s>>>(M, slots, RP, rowsrc, c0, rcw);
    else return (int)cudaErrorInvalidValue;
    return (int)cudaGetLastError();
}

// Pivot rows of sub-panel s >= 1 of a fused super-panel, transposed into RP
// columns [kp, kp + NB) with kp = s·NB:
//   RT[n][kp + k] = δ(n − c0, k)                                    n in the panel's columns,
//                 = [n ∉ [c0q, c0)]·M0[tot[c0 + k]][n] + Σ_{t<kp} gsub[k][t]·RT[n][t]   otherwise,
// for k < w (zero beyond), M0 the super-panel's input matrix (it starts at column
// c0q), gsub the earlier G columns of the panel's pivot rows (written by the panel
// kernel).  The sum applies the earlier sub-panels' update to the pivot rows only,
// so the super-panel's single update is the only pass over the matrix.  The
// earlier RT columns of the panel's own columns, RT[n ∈ [c0, c0+w)][t < kp], are
// then zeroed.  FP32 CUDA-core FMAs: a small correction of b x NB x kp per matrix.
// grid: (ceil(b/64), njobs), block 256, dynamic smem gj_rs_smem<NB>(kp)
template <int NB>
__host__ __device__ constexpr size_t gj_rs_smem_elems(int kp) {
    // G transposed [t][NB] (re, im), RT tile [64][kp + 1] (re, im), β tile [NB][64] (re, im)
    return (size_t)2 * NB * kp + (size_t)2 * 64 * (kp + 1) + (size_t)2 * NB * 64;
}
template <typename T, int NB>
__global__ void __launch_bounds__(256) gj_rs_kernel(Pool<T> M, const int* slots, Pool<T> RP, const int* tot,
                                                    const T* gsub, int kp, int c0, int c0q) {
    constexpr int TN = 64, NT = 256;
    constexpr int KG = NB / 4;                       // groups of four k per n pair
    constexpr int NPT = TN * KG / NT;                // n values per thread (2 for NB = 32, 1 for 16)
    static_assert(NPT >= 1 && TN * KG % NT == 0, "rs tiling");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int KP = kp + 1;
    T* gtr = reinterpret_cast<T*>(smem_raw);         // [t][NB]
    T* gti = gtr + NB * kp;
    T* rre = gti + NB * kp;                          // [n][KP]
    T* rim = rre + TN * KP;
    T* bre = rim + TN * KP;                          // [k][TN]
    T* bim = bre + NB * TN;
    const int b = M.rows, job = blockIdx.y, n0 = blockIdx.x * TN, tid = threadIdx.x;
    const int w = min(NB, b - c0);
    const T* gs = gsub + (size_t)job * 2 * NB * RP.cols;
    T* rt = RP.slot(job);
    const long long pe = RP.plane_elems();
    const T* Mre = M.slot(slots[job]);
    const T* Mim = Mre + M.plane_elems();
    const int* tj = tot + (size_t)job * b;
    for (int idx = tid; idx < NB * kp; idx += NT) {
        const int k = idx / kp, t = idx % kp;
        gtr[t * NB + k] = gs[(size_t)k * RP.cols + t];
        gti[t * NB + k] = gs[(size_t)(NB + k) * RP.cols + t];
    }
    for (int idx = tid; idx < TN * kp; idx += NT) {
        const int nn = idx / kp, t = idx % kp, n = n0 + nn;
        const long long o = (long long)n * RP.ld + t;
        rre[nn * KP + t] = n < b ? rt[o] : (T)0;
        rim[nn * KP + t] = n < b ? rt[pe + o] : (T)0;
    }
    // β rows of M0 (the pivot rows before the super-panel), coalesced along n
    for (int idx = tid; idx < NB * TN; idx += NT) {
        const int k = idx / TN, nn = idx % TN, n = n0 + nn;
        T a = 0, d = 0;
        if (k < w && n < b && !(n >= c0q && n < c0 + w)) {
            const long long o = (long long)tj[c0 + k] * M.ld + n;
            a = Mre[o];
            d = Mim[o];
        }
        bre[k * TN + nn] = a;
        bim[k * TN + nn] = d;
    }
    __syncthreads();
    // thread: four consecutive k (one 16-byte G load per plane and t) for NPT values of n
    const int kg = tid % KG, k0 = 4 * kg;
    int nl[NPT];
    T ar[NPT][4], ai[NPT][4];
#pragma unroll
    for (int u = 0; u < NPT; ++u) {
        nl[u] = tid / KG + u * (NT / KG);
#pragma unroll
        for (int e = 0; e < 4; ++e) { ar[u][e] = bre[(k0 + e) * TN + nl[u]]; ai[u][e] = bim[(k0 + e) * TN + nl[u]]; }
    }
    for (int t = 0; t < kp; ++t) {
        const float4 gr4 = *reinterpret_cast<const float4*>(gtr + t * NB + k0);
        const float4 gi4 = *reinterpret_cast<const float4*>(gti + t * NB + k0);
        const T gr[4] = {gr4.x, gr4.y, gr4.z, gr4.w}, gi[4] = {gi4.x, gi4.y, gi4.z, gi4.w};
#pragma unroll
        for (int u = 0; u < NPT; ++u) {
            const T xr = rre[nl[u] * KP + t], xi = rim[nl[u] * KP + t];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                ar[u][e] = fma(gr[e], xr, fma(-gi[e], xi, ar[u][e]));
                ai[u][e] = fma(gr[e], xi, fma(gi[e], xr, ai[u][e]));
            }
        }
    }
#pragma unroll
    for (int u = 0; u < NPT; ++u) {
        const int n = n0 + nl[u];
        if (n >= b) continue;
        const bool own = n >= c0 && n < c0 + w;   // the panel's own columns: identity
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int k = k0 + e;
            T ore = 0, oim = 0;
            if (k < w) {
                if (own) ore = (T)(n - c0 == k ? 1 : 0);
                else { ore = ar[u][e]; oim = ai[u][e]; }
            }
            const long long o = (long long)n * RP.ld + kp + k;
            rt[o] = ore;
            rt[pe + o] = oim;
            if (RP.planes == 4) {
                rt[2 * pe + o] = (T)tf32_lo((float)ore);
                rt[3 * pe + o] = (T)tf32_lo((float)oim);
            }
        }
    }
    // the panel's own rows take no earlier update: zero their earlier RT columns
    const int z0 = max(c0, n0), z1 = min(c0 + w, min(n0 + TN, b));
    for (int idx = tid; idx < (z1 > z0 ? (z1 - z0) * kp : 0); idx += NT) {
        const int n = z0 + idx / kp, t = idx % kp;
        const long long o = (long long)n * RP.ld + t;
        for (int pl = 0; pl < RP.planes; ++pl) rt[pl * pe + o] = (T)0;
    }
}

template <typename T>
int launch_gj_rs(cudaStream_t s, int nb, int njobs, Pool<T> M, const int* slots, Pool<T> RP, const int* tot,
                 const T* gsub, int kp, int c0, int c0q) {
    if (kp <= 0 || kp + nb > RP.cols) return (int)cudaErrorInvalidValue;
    const dim3 grid(ceil_div(M.rows, 64), njobs);
    if (nb == 32) {
        const size_t smem = gj_rs_smem_elems<32>(kp) * sizeof(T);
        static const cudaError_t attr = cudaFuncSetAttribute(
            gj_rs_kernel<T, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(gj_rs_smem_elems<32>(128) * sizeof(T)));
        if (attr != cudaSuccess) return (int)attr;
        gj_rs_kernel<T, 32><<<grid, 256, smem, s>>>(M, slots, RP, tot, gsub, kp, c0, c0q);
    } else if (nb == 16) {
        const size_t smem = gj_rs_smem_elems<16>(kp) * sizeof(T);
        static const cudaError_t attr = cudaFuncSetAttribute(
            gj_rs_kernel<T, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(gj_rs_smem_elems<16>(128) * sizeof(T)));
        if (attr != cudaSuccess) return (int)attr;
        gj_rs_kernel<T, 16><<<grid, 256, smem, s>>>(M, slots, RP, tot, gsub, kp, c0, c0q);
    } else {
        return (int)cudaErrorInvalidValue;
    }
    return (int)cudaGetLastError();
}
template <typename T>
void launch_gj_unpermute(cudaStream_t s, int njobs, Pool<T> Src, const int* sslots, Pool<T> Dst,
                         const int* dslots, const int* perm) {
    gj_unpermute_kernel<T><<<dim3(ceil_div(Src.rows, 8), njobs), 256, 2 * Src.rows * sizeof(T), s>>>(
        Src, sslots, Dst, dslots, perm);
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
                                           Pool<T>, const L1Job*, cplx<T>*);                                 \
    template int launch_gj_panel<T>(cudaStream_t, int, int, Pool<T>, const int*, Pool<T>, int*, int*, int,    \
                                    unsigned*, GjFuse, int, int, uint64_t);                                  \
    template int launch_gj_rt<T>(cudaStream_t, int, int, Pool<T>, const int*, Pool<T>, const int*, int, int); \
    template void launch_gj_unpermute<T>(cudaStream_t, int, Pool<T>, const int*, Pool<T>, const int*,        \
                                         const int*);                                                       \
    template void launch_madd<T>(cudaStream_t, int, Pool<T>, const int3*);                                    \
    template void launch_mcopy<T>(cudaStream_t, int, Pool<T>, Pool<T>, const int3*);                         \
    template void launch_tri_inverse<T>(cudaStream_t, int, NodeMap, const cplx<double>*, double, Pool<T>,    \
                                        const int*, cplx<T>*, int*, unsigned*);
INST(float)
INST(double)
// fused super-panels run on the FP32 tensor-core path only
template int launch_gj_rs<float>(cudaStream_t, int, int, Pool<float>, const int*, Pool<float>, const int*,
                                 const float*, int, int, int);
