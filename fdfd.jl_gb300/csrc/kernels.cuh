// Kernel argument structs and declarations shared by the library's .cu files.
#pragma once
#include "common.cuh"

enum { OP_TM_DRIVEN = 0, OP_TE_DRIVEN = 1, OP_TM_EIGEN = 2, OP_TE_EIGEN = 3, OP_TM_SIDEBAND = 4 };
enum { REC_TM_DRIVEN = 0, REC_TE_DRIVEN = 1, REC_TM_EIGEN = 2, REC_TE_EIGEN = 3 };

struct SFactorArgs { int Nx, Ny, Npx, Npy; double dx, dy, omega, eps0n, eta0, m, lnR; };
struct StencilArgs { int Nx, Ny, op; double idx, idy, imu0, eps0n, omega2, omega2mu0, sigma_re, sigma_im; };
struct RecoverArgs { int Nx, Ny, mode; double idx, idy, eps0n; };

// Mapping between natural unknowns and (node, in-block index).
struct NodeMap {
    int Nx, Ny;
    int b, n, ld;        // block size, block count, vector/matrix leading dimension
    int transposed;      // 0: node = iy, i = ix (b = Nx); 1: node = ix, i = iy (b = Ny)
    __host__ __device__ long long nat(int node, int i) const {
        return transposed ? (long long)node + (long long)Nx * i : (long long)i + (long long)Nx * node;
    }
    // stencil planes [self, x-1, x+1, y-1, y+1]: in-line prev/next and coupling prev/next
    __host__ __device__ int p_inprev() const { return transposed ? 3 : 1; }
    __host__ __device__ int p_innext() const { return transposed ? 4 : 2; }
    __host__ __device__ int p_cprev() const { return transposed ? 1 : 3; }
    __host__ __device__ int p_cnext() const { return transposed ? 2 : 4; }
};

// ---- assemble.cu -----------------------------------------------------------
// assembly arguments are read from device memory (a captured factorization is
// replayed for another frequency by rewriting them)
struct AssembleArgs { SFactorArgs sf; StencilArgs st; };
__global__ void sfactor_kernel(const SFactorArgs* a, cplx<double>* out);
__global__ void stencil_kernel(const StencilArgs* a, const cplx<double>* eps, const cplx<double>* sf, cplx<double>* st);
// first[0]: lowest double index of a non-finite entry of x (n complex values), first[1]
// (zeros != 0): lowest complex index with a zero value; ~0ull where there is none
void launch_validate(cudaStream_t s, int nsm, const double* x, long long n, int zeros, unsigned long long* first);
__global__ void residual_kernel(int Nx, int Ny, int nrhs, const cplx<double>* st, const cplx<double>* x,
                                const cplx<double>* b, cplx<double>* r, double* part);
// Coupled sideband system of a modulated device: K = 2s+1 stencils (one per
// sideband, each an OP_TM_SIDEBAND operator) and the couplings
// ½ωₙ²ϵ₀ conj(Δϵ) (to sideband n+1) and ½ωₙ²ϵ₀ Δϵ (to n-1).
#define MF_MAX_K 33
struct MfResidualArgs {
    int Nx, Ny, K;
    const cplx<double>* st[MF_MAX_K];
    double half_w2eps0[MF_MAX_K];   // ½ ωₙ² ϵ₀L₀
};
__global__ void residual_mf_kernel(MfResidualArgs a, const cplx<double>* deps, const cplx<double>* x,
                                   const cplx<double>* b, cplx<double>* r, double* part);
__global__ void residual_nl_kernel(int Nx, int Ny, int mode, const cplx<double>* st, const cplx<double>* d1,
                                   const cplx<double>* d2, const cplx<double>* x, const cplx<double>* b,
                                   cplx<double>* r, double* part);
__global__ void chi3_diag_kernel(long long N, int mode, const double* coeff, const cplx<double>* e,
                                 cplx<double>* d1, cplx<double>* d2);
__global__ void vconj_kernel(long long n, const cplx<double>* in, cplx<double>* out);
__global__ void vaxpy_kernel(long long n, double alpha, const cplx<double>* x, cplx<double>* y);
__global__ void reduce_partials_kernel(const double* part, int nblocks, int nvals, double* out);
__global__ void recover_kernel(RecoverArgs a, const cplx<double>* sf, const cplx<double>* eps,
                               const cplx<double>* f, const cplx<double>* coef, cplx<double>* g1,
                               cplx<double>* g2);
template <typename T>
void launch_to_nodes(dim3 grid, cudaStream_t s, NodeMap m, int nrhs, const cplx<double>* in, double scale, T* out);
template <typename T>
void launch_from_nodes(dim3 grid, cudaStream_t s, NodeMap m, int nrhs, const T* in, double scale, int accumulate,
                       cplx<double>* out);
__global__ void vscale_kernel(long long N, const cplx<double>* x, const cplx<double>* s, cplx<double>* y);
__global__ void vcombine_kernel(long long N, int nvec, const cplx<double>* V, long long vstride,
                                const cplx<double>* c, int ldc, double sign, cplx<double>* y);
__global__ void vdots_kernel(long long N, int nvec, const cplx<double>* V, long long vstride,
                             const cplx<double>* w, double* part);
__global__ void vnormalize_kernel(long long N, const cplx<double>* x, const double* nrm, cplx<double>* y);
__global__ void pscale_kernel(int Nx, int Ny, const cplx<double>* sf, int mode, const cplx<double>* in,
                              cplx<double>* out);
__global__ void adjoint_grad_kernel(long long N, cplx<double> coef, const cplx<double>* lam,
                                    const cplx<double>* E, double* grad);
__global__ void vdotu_kernel(long long N, const cplx<double>* m, const cplx<double>* E, double* part);

// ---- blocks.cu ----------------------------------------------------------------
struct L1Job {                 // survivor of the first reduction step
    int s, prev, next;         // node and its ring neighbours
    int prev_elim, next_elim;  // neighbour eliminated in this step
    int u_slot, l_slot;        // coupling-pool slots of the new U, L
    int u_trans, l_trans;      // store transposed (node eliminated next step)
};

// Host launchers (each kernel template is instantiated in its own translation unit).
template <typename T>
void launch_build_tridiag(cudaStream_t s, int njobs, NodeMap m, const cplx<double>* st, double scale, Pool<T> D,
                          const int* nodes);
// (tab: workspace of 5·b·n cplx<T>, the scaled stencil table of every node, written first)
template <typename T>
void launch_level1_combine(cudaStream_t s, int njobs, NodeMap m, const cplx<double>* st, double scale, Pool<T> D,
                           Pool<T> C, const L1Job* jobs, cplx<T>* tab);
void launch_perm_init(cudaStream_t s, int njobs, int* perm, int b);
// D[node] = (cyclic tridiagonal block of node)⁻¹ in O(b²) (first reduction step);
// fac: 8*b cplx<T> and piv: b ints of workspace per job
template <typename T>
void launch_tri_inverse(cudaStream_t s, int njobs, NodeMap m, const cplx<double>* st, double scale, Pool<T> D,
                        const int* nodes, cplx<T>* fac, int* piv, unsigned* err);
// Fused super-panels of the Gauss-Jordan inversion (FP32 tensor-core path):
// several consecutive panels share one rank-(panels x nb) update of the matrix.
// Their G columns are kept in the row order of the super-panel's input matrix
// M0, so no earlier column is ever permuted; rowsrc carries the composed map
// tot[r] (row of M0 that lands at logical row r) and inv_out its inverse.
struct GjFuse {
    int fused;             // 0: single-panel form (the fields below unused)
    int gcol0;             // first GP column of this panel (sub-panel index x nb)
    const int* tot_in;     // composed map before this panel (per job b), null: identity
    int* inv_out;          // per job b: inv_out[tot_out[r]] = r
    void* gsub;            // per job 2 x nb x GP.cols: earlier G columns of the pivot rows (re | im)
};

// Gauss-Jordan panel step with panel width nb on the matrices M[slots[job]]
// (returns a cudaError_t value).  Writes the panel transformation to GP,
// updates perm and writes rowsrc[job][r], the row of M that lands at row r
// after this panel's interchanges (fused: of the super-panel's input matrix).
// cl = 2, 4 or 8 splits each matrix's panel over a cluster of cl CTAs (not with
// fused super-panels), 0 or 1 runs one CTA per matrix: in the lane-quad form
// (form 0) or the pipelined row form (form 1, not with fused super-panels; its
// block waits end after wait_ns with FDFD_DEVERR_TIMEOUT).
template <typename T>
int launch_gj_panel(cudaStream_t s, int nb, int njobs, Pool<T> M, const int* slots, Pool<T> GP, int* perm,
                    int* rowsrc, int c0, unsigned* err, GjFuse fz, int cl, int form, uint64_t wait_ns);
// The panel's transposed pivot rows (identity on the panel columns) into RP
// columns [0, rcw) (zero beyond the panel; rcw <= 0: all of RP.cols), read
// from M through rowsrc; M must hold the rows after the previous update.
template <typename T>
int launch_gj_rt(cudaStream_t s, int nb, int njobs, Pool<T> M, const int* slots, Pool<T> RP, const int* rowsrc,
                 int c0, int rcw);
// Pivot rows of a later sub-panel of a fused super-panel into RP columns
// [kp, kp+nb): M0's rows through tot (masked on the super-panel's earlier
// columns [c0q, c0)) plus the earlier sub-panels' update of those rows (gsub
// times RP columns [0, kp)); identity on the panel's columns [c0, c0+nb), whose
// earlier RP columns are zeroed.  nb = 16 or 32.  Returns a cudaError_t value.
template <typename T>
int launch_gj_rs(cudaStream_t s, int nb, int njobs, Pool<T> M, const int* slots, Pool<T> RP, const int* tot,
                 const T* gsub, int kp, int c0, int c0q);
// Dst[dslots[job]][r][perm[j]] = Src[sslots[job]][r][j] (Src may equal Dst)
template <typename T>
void launch_gj_unpermute(cudaStream_t s, int njobs, Pool<T> Src, const int* sslots, Pool<T> Dst,
                         const int* dslots, const int* perm);
// C[dst] = A[s1] + A[s2] (same storage form)
template <typename T>
void launch_madd(cudaStream_t s, int njobs, Pool<T> P, const int3* jobs);
// dst = src (optionally transposed) between pools
template <typename T>
void launch_mcopy(cudaStream_t s, int njobs, Pool<T> S, Pool<T> Dp, const int3* jobs);

// ---- modes.cu -------------------------------------------------------------------
// One guided-mode job: the 1-D slice of n cells starting at natural index k0,
// step `stride`, cell size dh, polarization pol (1 TM, 2 TE), shift σ =
// (ω n_eff/c₀)²; its unit vector goes to vecs[out_off .. out_off+n).
#define FDFD_MODE_MAX_POINTS 1023
struct ModeJob {
    int pol, n;
    long long k0, stride;
    double dh, omega, sig_re, sig_im;
    int out_off, pad;
};
size_t mode_smem_bytes(int nmax);
// beta[job] = √λ, vecs: unit eigenvectors, iters[job]: inverse-iteration steps
// (negative: no convergence).  Returns a cudaError_t value.
int launch_modes(cudaStream_t s, int njobs, int nmax, const ModeJob* jobs, const cplx<double>* eps, double eps0n,
                 double mu0n, cplx<double>* beta, cplx<double>* vecs, int* iters, unsigned* err);
// src[w] += |v| of the jobs job_start[w] .. job_start[w+1]-1 (nw frequencies, N cells each)
void launch_mode_src(cudaStream_t s, int nw, const ModeJob* jobs, const int* job_start, const cplx<double>* vecs,
                     long long N, cplx<double>* src);

// ---- flux.cu --------------------------------------------------------------------
// Poynting flux Sx, Sy per cell (flux.jl:15-29); pol 1 TM (Ez, Hx, Hy), 2 TE (Hz, Ex, Ey)
void launch_poynting(cudaStream_t s, int Nx, int Ny, int pol, const cplx<double>* f1, const cplx<double>* f2,
                     const cplx<double>* f3, double* Sx, double* Sy);
// x̂-normal line integrals (flux.jl:37-57): lines (xind, iy0, iy1), out[l] (one block per line)
void launch_flux_lines(cudaStream_t s, int nlines, int Nx, int pol, double dy, const int3* lines,
                       const cplx<double>* f1, const cplx<double>* f3, double* out);

// ---- gemm_simt.cu / gemm_tc.cu --------------------------------------------
// Batched complex "TN" GEMM on planar pools:
//   C[dst(m)][n] = beta(dst(m),n)·Cin[src(m)][n] + alpha·Σ_k A[m][k]·B[n][k]
// with A, B, C row-major slots; beta(m,n) = beta unless m or n lies in
// [mask_c0, mask_c0 + mask_w), where it is 0; c_trans stores Cᵀ instead.
// Cin is C itself (src(m) = m) unless Cin.base is set; then src(m) =
// row_src[job*M + m] when row_src is set.
template <typename T> struct GemmArgs {
    Pool<T> A, B, C;
    Pool<T> Cin;
    const int* cin_slot;
    const int* row_src;
    const int* a_slot; const int* b_slot; const int* c_slot;
    int M, N, K;
    T alpha; int beta;
    int mask_c0, mask_w;
    // tensor-core kernel only: the product covers matrix columns [n_off, n_off + N)
    // (B rows likewise); columns [skip_c0, skip_c0 + skip_w) are neither read nor written
    int n_off, skip_c0, skip_w;
    int c_trans;
    const int* c_trans_arr;   // per-job override of c_trans (device, may be null)
    // tensor-core kernel only (N-form C, Cin set): when set, A row m is output row
    // row_dst[job*M + m] (the β term is read from Cin row m, and the row mask tests
    // the output row) -- the fused Gauss-Jordan updates, whose G rows stay in the
    // order of the super-panel's input matrix
    const int* row_dst;
    unsigned* err;
    // tensor-core kernel only: limit of each pipeline wait in ns of %globaltimer
    // (0: FDFD_WAIT_LIMIT_NS); the drain waits before exit always take the full limit
    unsigned long long wait_ns;
    // tensor-core kernel only, split-K partial products: ksplit > 1 runs grid z = jobs x
    // ksplit, CTA z taking job z / ksplit over K columns [(z % ksplit)·kslice, +kslice) and
    // writing its raw product to C slot c_slot[z] (alpha 1, beta 0, N form, no windows)
    int ksplit = 0, kslice = 0;
};
template <typename T>
void launch_gemm_simt(cudaStream_t s, int njobs, const GemmArgs<T>& g);

// ---- sweep.cu -------------------------------------------------------------------
// y[job] = y0[job] + alpha·(op(M1)·v1 + op(M2)·v2) on node-planar vectors,
// op = identity (N-form storage) or the stored transpose (T-form storage).
#define GEMV_SHAPE_REGISTER_RULE 100
template <typename T> struct GemvArgs {
    Pool<T> P1, P2;
    const T* V1; const T* V2;
    const T* Y0; T* Y;
    const int4* jobs;   // (m1_slot, v1_node, m2_slot, v2_node), -1 = absent
    const int2* yjobs;  // (y_node, y0_node), y0_node -1 = zero
    int b, ld, nrhs;    // nrhs: right-hand sides handled by this launch (<= 8)
    int rtot, r0;       // right-hand sides stored per node, first one handled
    T alpha;
    int rpw, og;        // launch shape, set by launch_gemv: rows per warp (N form),
                        // lanes per output group (T form)
    int nsm;            // streaming multiprocessors of the device (launch shape)
    int shape;          // launch shape chosen by the caller (autotuner): rpw in {1, 2, 4} (N form, register
                        // loads), -2, -4 or -8 (N form, bulk-copy pipeline with that many rows per warp),
                        // og in {8, 16, 32} (T form); 0: launch_gemv's rule
    int nmat;           // most factor blocks one job references (1 or 2)
    // (a positive shape outside {1, 2, 4} selects the N form's register loads with launch_gemv's rule)
    unsigned* err;      // device error word (a bulk-copy wait that runs out sets FDFD_DEVERR_TIMEOUT)
};
// TR = 1: matrices stored transposed.  Returns a cudaError_t value.
template <typename T>
int launch_gemv(cudaStream_t s, int tr, int njobs, const GemvArgs<T>& g);
// right-hand sides one launch_gemv call may take for block size b
template <typename T>
int gemv_max_rhs(int b);
// Y[node] = Y0[node] + alpha·D_node⁻¹ V[node] for the first reduction step's
// nodes jobs[0..njobs) from their tridiagonal factor workspaces (fac, piv as
// written by launch_tri_inverse, workspace j for jobs[j]).  Y0 may be null or
// equal to Y.  Returns a cudaError_t value.
template <typename T>
int launch_tri_apply(cudaStream_t s, int b, int ld, int njobs, int nrhs, const int* jobs, const cplx<T>* fac,
                     const int* piv, const T* V, const T* Y0, T* Y, T alpha);
// r[s] -= u_s ⊙ z[next] + l_s ⊙ z[prev]  (first reduction step, diagonal couplings)
// mode 0: survivors update r from eliminated neighbours (jobs: L1Job-like int4 (s, prev, next, flags))
// mode 1: eliminated k: w[k] = l_k ⊙ x[prev] + u_k ⊙ x[next]
// (l, u: the scaled coupling planes of the factorization's stencil table)
template <typename T>
void launch_diag_sweep(cudaStream_t s, int njobs, NodeMap m, const cplx<T>* tab, int nrhs, const int4* jobs,
                       int mode, const T* src, T* dst);
