/*
 * libfdfd_cuda — GB300 (sm_103a) solve path for 2-D FDFD problems.
 *
 * C ABI for the drop-in replacement of the FDFD.jl solve path.  The reference
 * has no FFI; its backend seam is `dolinearsolve(A, b, sym)`
 * (src/solver/solver.jl:4-41), which sees only a CSC matrix.  This library
 * sits one level up and replaces, per frequency, the assembly, the linear
 * solve and the field recovery of
 *   solve(d::Device, pol)                       src/solver/driven.jl:4-59
 *   eigenfrequency(d, pol, nev; which)          src/solver/eigen.jl:69-115
 * so that Julia's `solve`/`eigenfrequency` can `ccall` it when
 * ENV["FDFD_SOLVER"] == "cuda".
 *
 * Array conventions (all entry points): complex arrays are interleaved
 * {re, im} doubles (Julia ComplexF64 / C `double _Complex`), Nx*Ny values per
 * field, x fastest (Julia column-major `A[:]`, driven.jl:21).  Host arrays
 * belong to the caller and are only read/written during the call.  Every call
 * blocks until its results are in the caller's arrays.  A handle is used by one
 * thread at a time; distinct handles are independent.
 *
 * Status codes: every entry point returns FDFD_OK or one of the errors below
 * and leaves a message retrievable with fdfd_last_error().
 */
#ifndef FDFD_CUDA_H
#define FDFD_CUDA_H

#ifdef __cplusplus
extern "C" {
#endif

#define FDFD_OK         0
#define FDFD_EINVAL     1  /* bad argument (sizes, NaN/Inf input, call order) */
#define FDFD_ENOMEM     2  /* device or pinned-host allocation failed        */
#define FDFD_ESINGULAR  3  /* zero or non-finite pivot in a block inversion   */
#define FDFD_ENOCONV    4  /* refinement hit its iteration cap above tol      */
#define FDFD_ETIMEOUT   5  /* a bounded device-side wait gave up              */
#define FDFD_ECUDA      6  /* CUDA runtime/driver error                       */

#define FDFD_TM 1          /* src/types.jl:20 (@enum Polarization TM=1 TE=2) */
#define FDFD_TE 2

#define FDFD_PREC_FP64  0  /* complex FP64 factorization and sweeps          */
#define FDFD_PREC_MIXED 1  /* complex FP32 storage, 3xTF32 tcgen05 products,
                              FP64 residual and refinement                   */

#define FDFD_REFINE_GMRES   0  /* flexible GMRES in FP64, factor as preconditioner */
#define FDFD_REFINE_CLASSIC 1  /* x += M^-1 (b - A x)                              */

#define FDFD_X 1           /* src/types.jl:18 (@enum Direction x̂=1 ŷ=2) */
#define FDFD_Y 2

#define FDFD_CHI3_NEWTON 1 /* src/solver/nonlinear.jl:5 (IterativeMethodGN=1 IterativeMethodB=2) */
#define FDFD_CHI3_BORN   2

/* eigfreq selection, as Arpack's `which` (src/solver/eigen.jl:69,86,104) in
 * shift-invert mode: it ranks θ = 1/(λ-σ), the eigenvalues of (A - σI)⁻¹ */
#define FDFD_WHICH_LM 0    /* largest |θ|: eigenvalues of A nearest sigma (:LM)     */
#define FDFD_WHICH_LR 1    /* largest real part of θ (:LR)                          */
#define FDFD_WHICH_SM 2    /* smallest |θ|: farthest from sigma (:SM)               */
#define FDFD_WHICH_SR 3    /* smallest real part of θ (:SR)                         */
#define FDFD_WHICH_LI 4    /* largest imaginary part of θ (:LI)                     */
#define FDFD_WHICH_SI 5    /* smallest imaginary part of θ (:SI)                    */

typedef struct fdfd_handle fdfd_handle;

/* Per-call statistics, filled by the solve/adjoint/eigen entry points. */
typedef struct {
    int    iterations;       /* preconditioner applications (factor solves)         */
    int    nrhs;             /* right-hand sides in the call                         */
    double rel_residual;     /* max over RHS of ||b - A x|| / ||b|| (FP64)           */
    double t_assemble_ms;    /* stencil + block assembly                             */
    double t_factor_ms;      /* block cyclic reduction factorization                 */
    double t_solve_ms;       /* refinement loop incl. factor solves and residuals    */
    double t_recover_ms;     /* H (TM) / E (TE) recovery and copies out              */
    double t_total_ms;       /* wall time of the call                                */
    double factor_flops;     /* algorithmic real flops of the last factorization     */
    int    block;            /* dense block size b = min(Nx, Ny)                     */
    int    nblocks;          /* number of blocks n = max(Nx, Ny)                     */
    int    levels;           /* cyclic-reduction elimination steps                   */
    int    tc_gemm;          /* 1 when the tcgen05 3xTF32 GEMM ran                   */
    long long device_bytes;  /* device memory held by the handle                     */
    long long gpu_launches;  /* kernels this library launched during the call        */
    int    factor_precision; /* FDFD_PREC_* of the factor the refinement finished with */
    int    fp64_fallback;    /* 1 when that factor is an FP64 re-factorization of an
                                FDFD_PREC_MIXED handle (fdfd_set_fallback); its time
                                counts in t_solve_ms                               */
} fdfd_stats;

/* Version string of the library. */
const char* fdfd_version(void);

/* Create a handle for an Nx x Ny grid (Grid, src/grid.jl:7-33) with Npx/Npy
 * PML cells per side, cell sizes dx, dy in units of L0 metres (grid.jl:68-74),
 * PML grading m and ln(R) (create_sfactor, src/pml.jl:1-31; the reference
 * hard-wires m=3.5, lnR=-12 because S_create does not forward them,
 * pml.jl:35-38), polarization FDFD_TM/FDFD_TE and precision FDFD_PREC_*.
 * Requires Nx, Ny >= 3. */
int  fdfd_create(fdfd_handle** h, int Nx, int Ny, int Npx, int Npy, double dx,
                 double dy, double L0, double pml_m, double pml_lnR, int pol,
                 int precision);
void fdfd_destroy(fdfd_handle* h);
const char* fdfd_last_error(const fdfd_handle* h);

/* Refinement stopping rule: ||b - A x||/||b|| <= tol within max_iter factor
 * solves (FDFD_REFINE_GMRES restarts its Krylov basis every m solves, m from
 * fdfd_set_restart). */
int  fdfd_set_refinement(fdfd_handle* h, double tol, int max_iter, int mode);

/* Basis length m of the restarted FGMRES refinement (0: automatic, the
 * default).  The refinement holds 2m+1 FP64 vectors per right-hand side. */
int  fdfd_set_restart(fdfd_handle* h, int m);

/* FP64 fallback of an FDFD_PREC_MIXED handle (on by default).  When the
 * refinement preconditioned by the FP32 factor is projected to miss tol
 * within max_iter solves (measured rate per restart cycle), or stops above
 * tol, the handle factors the same operator in FP64 and refines again; the
 * FP64 factor then serves the following solves until the next factorization.
 * Off: the call returns FDFD_ENOCONV instead.  No effect on FP64 handles. */
int  fdfd_set_fallback(fdfd_handle* h, int on);

/* Watchdog of the tensor-core GEMM (no counterpart in the reference, whose
 * solvers have no device waits).  Every pipeline wait of that kernel
 * (mbarrier, on TMA copies and MMAs) gives up after ns nanoseconds of
 * %globaltimer; the CTA then records the timeout, lets its own copies and
 * MMAs in flight finish (those waits keep the default limit), frees its
 * tensor memory and exits, and the call returns FDFD_ETIMEOUT with the
 * context still usable.  ns <= 0 restores the default, 2 s.  A limit far
 * below a kernel's run time makes every factorization time out: a
 * failure-path check, not a tuning knob. */
int  fdfd_set_wait_limit(fdfd_handle* h, long long ns);

/* Device-memory budget of the handle in bytes (no counterpart in the
 * reference; 0, the default, means no limit).  An allocation that would take
 * the handle's device memory above the budget fails with FDFD_ENOMEM and the
 * sizes in the message, as a failed cudaMalloc does. */
int  fdfd_set_device_budget(fdfd_handle* h, long long bytes);

/* Checkpointing of block factors to host memory (no counterpart in the
 * reference, whose sparse factors live in host memory).  mode 0 (default):
 * engaged at the first factorization when the resident factor storage would
 * not fit the handle's device budget (fdfd_set_device_budget) or, without a
 * budget, 95% of the device's free memory, while the checkpointed storage
 * does; 1: always (before the first factorization); -1: never.  Engaged, the
 * coupling blocks of each reduction step and its X blocks move to pinned host
 * memory as soon as the factorization no longer needs them (one copy per
 * step), and every solve sweep copies them back step by step: the device holds
 * about 3n instead of 4n blocks of b x b (n = max(Nx, Ny), b = min(Nx, Ny)),
 * at the price of host-link traffic in every sweep.  Results are identical to
 * the resident layout.  Engaged mode lasts for the handle's lifetime.
 * fdfd_checkpoint_info: engaged flag, pinned host bytes held, bytes copied
 * between device and host so far. */
int  fdfd_set_checkpoint(fdfd_handle* h, int mode);
int  fdfd_checkpoint_info(const fdfd_handle* h, int* active, long long* host_bytes,
                          long long* copied_bytes);

/* Relative permittivity ϵᵣ (Device.ϵᵣ, src/device.jl:19-25), Nx*Ny complex.
 * Rejects NaN/Inf and complex zeros (FDFD_EINVAL, with the first such index in
 * fdfd_last_error); the check runs on the device after the copy, and a
 * rejected ϵᵣ leaves the handle's permittivity and factorization unchanged.
 * Otherwise invalidates any existing factorization. */
int  fdfd_set_eps(fdfd_handle* h, const double* eps_r);

/* Assemble the driven operator of solve() at angular frequency omega (SI
 * rad/s) and factor it:  TM A = δxf μ₀⁻¹ δxb + δyf μ₀⁻¹ δyb + ω² Tϵ,
 * TE A = δxf Tϵxi δxb + δyf Tϵyi δyb + ω² μ₀ I  (driven.jl:21-45). */
int  fdfd_factor(fdfd_handle* h, double omega);

/* Driven solve with the current factorization for nrhs current sources
 * (Device.src, b = iω·src, driven.jl:36,46), each Nx*Ny complex, stacked.
 * A source with a NaN/Inf entry is rejected (FDFD_EINVAL) before any solve work
 * (checked on the device after the copy).
 * Outputs (each nrhs*Nx*Ny complex, any may be NULL):
 *   TM: f1 = Ez, f2 = Hx, f3 = Hy  (driven.jl:38-42)
 *   TE: f1 = Hz, f2 = Ex, f3 = Ey  (driven.jl:48-53)
 * Replaces dolinearsolve (solver.jl:4-41) plus the recovery SpMVs. */
int  fdfd_solve(fdfd_handle* h, const double* src, int nrhs, double* f1,
                double* f2, double* f3, fdfd_stats* stats);

/* As fdfd_solve, but every array is a DEVICE pointer (cudaMalloc'd by the
 * caller, same layout).  Used to time the solve with inputs resident in HBM. */
int  fdfd_solve_device(fdfd_handle* h, const double* d_src, int nrhs,
                       double* d_f1, double* d_f2, double* d_f3,
                       fdfd_stats* stats);

/* Adjoint gradient of J = |Σ_k m_k Ez_k|² with respect to real ϵᵣ for the
 * current factorization of a TM driven operator (fdfd_factor on an FDFD_TM
 * handle; a TE handle is FDFD_EINVAL) and one source (no counterpart in the reference,
 * which has no gradient code).  Solves A E = iω·src and Aᵀ λ = m by reusing
 * the forward factors (P·A is complex symmetric for the diagonal PML scaling
 * P, so Aᵀ = P A P⁻¹), then dJ/dϵᵣ_k = -2 Re(conj(mᵀE)·ω²ϵ₀·λ_k·E_k).
 * Outputs: J (scalar), grad (Nx*Ny doubles), ez (Nx*Ny complex, may be NULL). */
int  fdfd_adjoint(fdfd_handle* h, const double* src, const double* mvec,
                  double* J, double* grad, double* ez, fdfd_stats* stats);

/* Vector-Jacobian product of the TM solve with respect to real ϵᵣ (no
 * counterpart in the reference; the pullback of a ChainRulesCore.rrule on
 * solve): E = A⁻¹(iω·src), λ = A⁻ᵀ g with g (Nx*Ny complex) the conjugated
 * cotangent of Ez (ChainRules convention: dL = Re(Σ conj(ΔEz)·dEz), so
 * g = conj(ΔEz)), and grad_k = -Re(ω²ϵ₀·λ_k·E_k) = dL/dϵᵣ_k.  Same
 * factorization reuse and requirements as fdfd_adjoint, which is this
 * product for g = 2·conj(mᵀE)·m. */
int  fdfd_adjoint_vjp(fdfd_handle* h, const double* src, const double* g,
                      double* grad, double* ez, fdfd_stats* stats);

/* Shift-invert eigenfrequencies (eigenfrequency, src/solver/eigen.jl:69-115):
 * with the PML frozen at omega0, TM finds eigenpairs of
 * A = Tϵᵣ⁻¹(δxf δxb + δyf δyb) nearest σ = -ω₀²μ₀ϵ₀, TE of
 * A = δxf Tϵx⁻¹ δxb + δyf Tϵy⁻¹ δyb nearest σ = -ω₀²μ₀, by Arnoldi on
 * (A - σI)⁻¹ (classical Gram-Schmidt with re-orthogonalisation, explicit
 * restarts from the wanted Ritz vectors) with this library's factorization
 * and refinement for every operator application; converged when every wanted
 * Ritz pair has |h_{k+1,k}·s_k| <= tol·|θ| (tol <= 0 selects 1e-10).  Outputs:
 * omega (nev complex: sqrt(-λ/(μ₀ϵ₀)) TM, sqrt(-λ/μ₀) TE), lambda (nev
 * complex eigenvalues of A, may be NULL), fields (nev*3*Nx*Ny complex:
 * per mode f1,f2,f3 as in fdfd_solve but with the eigen.jl recovery, may be
 * NULL). */
int  fdfd_eigfreq(fdfd_handle* h, double omega0, int nev, int which,
                  double tol, double* omega, double* lambda, double* fields,
                  fdfd_stats* stats);

/* A mode source (Mode, src/device.jl:5-11): polarization, slice normal
 * (FDFD_X: the slice runs along y at column ix; FDFD_Y: along x at row iy),
 * centre cell (0-based: coord2ind(grid, Mode.pt) - 1), slice width in L0
 * units and the effective-index guess n_eff. */
typedef struct {
    int    pol;
    int    normal;
    int    ix, iy;
    double width;
    double neff_re, neff_im;
} fdfd_mode;

/* Guided mode of a grid slice: get_modes with nmodes = 1 (src/device.jl:124-149)
 * and the 1-D eigenmode it calls (src/solver/eigen.jl:6-29).  The slice has
 * round(width/dh) cells, made odd (*npts), of the handle's ϵᵣ; the periodic
 * 1-D operator A = ω²μ₀Tϵ + δxf δxb (TM) or ω²μ₀Tϵ + Tϵ δxf Tϵxinv δxb (TE)
 * gives the eigenpair nearest (ω n_eff/c₀)², found by shift-invert
 * iteration on the GPU.  beta: 1 complex (√λ, principal branch); vec: *npts
 * complex values (cap = its capacity), unit 2-norm, largest entry real and
 * positive.  A slice leaving the grid, or of fewer than 3 or more than 1023
 * cells, is FDFD_EINVAL. */
int  fdfd_get_mode(fdfd_handle* h, double omega, const fdfd_mode* mode, int cap,
                   double* beta, double* vec, int* npts);

/* Mode sources for nw frequencies (driven.jl:15-19 with setup_mode!,
 * device.jl:118-121): src (nw*Nx*Ny complex, host) is overwritten with, per
 * frequency, the sum over the nmodes modes of normalize(abs.(v)) on each
 * mode's slice.  All nw*nmodes mode problems run in one launch (a warp each).
 * Like the reference's solve loop, callers pass pol = FDFD_TM for sources. */
int  fdfd_mode_sources(fdfd_handle* h, int nw, const double* omegas, int nmodes,
                       const fdfd_mode* modes, double* src);

/* Poynting flux of a field (poynting, src/flux.jl:15-29) on the handle's grid:
 * f1, f2, f3 = (Ez, Hx, Hy) for FDFD_TM or (Hz, Ex, Ey) for FDFD_TE, Nx*Ny
 * complex each (host); Sx, Sy: Nx*Ny doubles.  TM: Sx = -½Re(avgx(Ez) Hy*),
 * Sy = ½Re(avgy(Ez) Hx*); TE: Sx = ½Re(Ey avgx(Hz)*), Sy = -½Re(Ex avgy(Hz)*),
 * avg the periodic grid_average (grid.jl:157-162).  The reference's TE branch
 * reads fields a FieldTE lacks (flux.jl:26-27); the averaged Hz is used. */
int  fdfd_poynting(fdfd_handle* h, int pol, const double* f1, const double* f2,
                   const double* f3, double* Sx, double* Sy);
/* The same on device pointers (e.g. the outputs of fdfd_solve_device), with
 * no host copies. */
int  fdfd_poynting_device(fdfd_handle* h, int pol, const double* d_f1, const double* d_f2,
                          const double* d_f3, double* d_Sx, double* d_Sy);

/* flux_surface_integral(field, center, width, normal) (src/flux.jl:37-66) for
 * nlines lines (x̂ normal): lines holds (xind, iy0, iy1) per line, 0-based:
 * the column of center.x and the rows whose centres lie in
 * [center.y - width, center.y + width].  flux[l] = Σ -½Re(½(f1[xind]+f1[xind+1])
 * f3[xind]*)·dy, f1/f3 = Ez/Hy (TM) or Hz/Ey (TE; the reference's TE branch
 * names an undefined `pt` and reads :Hy, flux.jl:49,54 — the column of center
 * and :Ey are used).  FDFD_Y is FDFD_EINVAL, as in the reference. */
int  fdfd_flux_integral(fdfd_handle* h, int pol, const double* f1, const double* f3,
                        int normal, int nlines, const int* lines, double* flux);

/* χ³ nonlinear TM solve, solve(d::χ3Device, method) (src/solver/nonlinear.jl:36-129)
 * for the handle's factored TM operator A (fdfd_factor) and one source:
 * the linear field, then
 *   FDFD_CHI3_BORN:   e ← (A + diag(c|e|²))⁻¹ b until ||Δe||/||e|| <= tol,
 *   FDFD_CHI3_NEWTON: Newton on [e; conj e] with J = [A + 2c|e|², c e²;
 *                     conj(c e²), conj(A + 2c|e|²)] until ||δ||/||[e; conj e]|| <= tol,
 * c = ω²ϵ₀·3χ/L₀ (chi: Nx*Ny real), at most maxit steps (the reference uses
 * tol 1e-12, 50).  Each linear system is refined by FGMRES to a decade below
 * tol, preconditioned by the factor of A (Newton: by blockdiag(A⁻¹, conj(A)⁻¹)
 * through one two-right-hand-side sweep), so the factorization is reused by
 * every step.  Outputs Ez, Hx, Hy (driven recovery, may be NULL), the step
 * errors err_hist[0..*nerr-1] (err_hist[0] = 1 as the reference's history;
 * capacity maxit+1).  FDFD_ENOCONV when tol is not reached.  The reference's
 * Born step misplaces a parenthesis in its solve call (nonlinear.jl:97); its
 * evident intent is implemented. */
int  fdfd_chi3_solve(fdfd_handle* h, const double* chi, const double* src, int method,
                     double tol, int maxit, double* f1, double* f2, double* f3,
                     double* err_hist, int* nerr, fdfd_stats* stats);

/* Modulated device (multi-frequency FDFD): replaces solve(d::ModulatedDevice)
 * (src/solver/modulation.jl:35-119, TM only as the reference).  The handle
 * holds K = 2*nsidebands+1 sideband operators
 *   Aₙ = Sxb δxb μ₀⁻¹ Sxf δxf + Syb δyb μ₀⁻¹ Syf δyf + ωₙ² ϵ₀ϵᵣ,  ωₙ = ω + nΩ,
 * n = -s..s, with the PML at ω (shared_pml != 0, the reference default) or at
 * ωₙ, coupled by ½ωₙ² ϵ₀ conj(Δϵᵣ) to sideband n+1 and ½ωₙ² ϵ₀ Δϵᵣ to n-1
 * (modulation.jl:93-101).  The coupled system is refined in FP64 (FGMRES) to
 * the handle's tol, preconditioned by the K sideband factorizations, which
 * are solved concurrently.  fdfd_set_eps, fdfd_set_refinement,
 * fdfd_set_restart, fdfd_set_fallback, fdfd_apply (nrhs 1, K*Nx*Ny values,
 * sideband-major) and fdfd_destroy accept the handle; fdfd_factor,
 * fdfd_solve, fdfd_adjoint and fdfd_eigfreq reject it (FDFD_EINVAL).
 * nsidebands in [0, 16]. */
int  fdfd_mf_create(fdfd_handle** h, int Nx, int Ny, int Npx, int Npy, double dx,
                    double dy, double L0, double pml_m, double pml_lnR,
                    int nsidebands, int shared_pml, int precision);

/* Modulation amplitude Δϵᵣ (ModulatedDevice.Δϵᵣ, setup_Δϵᵣ!,
 * modulation.jl:7,28-32), Nx*Ny complex; zero after fdfd_mf_create. */
int  fdfd_mf_set_deps(fdfd_handle* h, const double* deps_r);

/* Assemble and factor the K sideband operators for carrier ω and modulation
 * frequency Ω (ModulatedDevice.ω, .Ω); every ωₙ must be positive. */
int  fdfd_mf_factor(fdfd_handle* h, double omega, double Omega);

/* One source (Nx*Ny complex): b = iω·src in the centre sideband
 * (modulation.jl:67-69).  Outputs (each may be NULL) hold K*Nx*Ny complex
 * values, sideband n = -s..s in order: Ez and the forward-difference
 * H = (-Syf δyf Ez, Sxf δxf Ez)/(iωₙμ₀) (modulation.jl:108-114).  Stats:
 * iterations are applications of the block preconditioner. */
int  fdfd_mf_solve(fdfd_handle* h, const double* src, double* ez, double* hx,
                   double* hy, fdfd_stats* stats);

/* Batched factorizations in one CUDA graph (no counterpart in the reference,
 * whose solve loop re-assembles and re-factors each frequency in turn,
 * src/solver/driven.jl:11-55).  A batch groups n existing driven handles
 * (TM or TE, any grid sizes and precisions; not modulated devices; each handle
 * in at most one batch).  fdfd_batch_factor(B, omegas, status) assembles and
 * factors every handle at its omegas[i] (SI rad/s) with the permittivity last
 * given to fdfd_set_eps: the first call does so handle by handle and then
 * captures the device work of all of them as the parallel branches of one
 * CUDA graph; every later call is one cudaGraphLaunch of that graph (the
 * handles' factorizations run concurrently on the GPU).  status[i] (may be
 * NULL) receives each handle's code; the call returns the first error.  The
 * handles are then factored as after fdfd_factor (fdfd_solve, fdfd_adjoint on
 * each).  The handles must outlive the batch and not profile
 * (fdfd_set_profiling) while batched; a handle may belong to several batches
 * used one at a time; its power-of-two operator scaling is the one of the
 * first call.  fdfd_batch_stats: kernels captured
 * in the graph, graph launches so far, device time of the last launch (ms). */
typedef struct fdfd_batch fdfd_batch;
int  fdfd_batch_create(fdfd_batch** B, int n, fdfd_handle* const* handles);
int  fdfd_batch_factor(fdfd_batch* B, const double* omegas, int* status);
int  fdfd_batch_stats(const fdfd_batch* B, long long* kernels,
                      long long* graph_launches, double* last_ms);
const char* fdfd_batch_last_error(const fdfd_batch* B);
void fdfd_batch_destroy(fdfd_batch* B);

/* Autotuner of the launch shapes (no counterpart in the reference).  Times,
 * on the handle's own storage and job lists, every tensor-core GEMM shape of
 * its factorization (tile width 64, 128 or 256 columns) and every sweep product
 * of its plan for 1 and for the largest right-hand-side count per launch (rows
 * per warp 1/2/4, or output-group width 8/16/32 for the transposed form), and
 * keeps the fastest for the handle's later factorizations, solves and batch
 * graphs.  It overwrites the factor storage (call it before fdfd_factor, or
 * factor again after it).  fdfd_get_tuning copies the record of the choices
 * (one line per shape with each candidate's time) into buf (cap bytes, NUL
 * terminated) and returns its full length (-1 on bad arguments). */
int  fdfd_autotune(fdfd_handle* h);
int  fdfd_get_tuning(const fdfd_handle* h, char* buf, int cap);

/* Debug/parity: copy the assembled FP64 5-point stencil of the last factored
 * operator to the host: 5*Nx*Ny complex, planes [self, x-1, x+1, y-1, y+1]
 * (periodic neighbours, unscaled, reference units). */
int  fdfd_get_stencil(fdfd_handle* h, double* out);

/* Matrix-free product y = A x with the assembled FP64 operator (host arrays,
 * nrhs stacked vectors). */
int  fdfd_apply(fdfd_handle* h, const double* x, int nrhs, double* y);

/* Per-kernel-class timing (no counterpart in the reference; it only logs wall
 * time, src/solver/solver.jl:5,38).  While profiling is on, the library
 * brackets each launch of the classes below with CUDA events on its stream
 * and accumulates device time and algorithmic work (flops for GEMMs, bytes
 * for the HBM-bound kernels).  fdfd_set_profiling(h, 1) resets the totals. */
typedef struct {
    double ms[8];            /* device time per class                           */
    double work[8];          /* flops (classes 0, 1) or bytes (the others)       */
    long long launches[8];   /* launches per class                              */
} fdfd_profile;
#define FDFD_PROF_GEMM_TC   0  /* tcgen05 3xTF32 Schur-update GEMMs (flops, 8MNK) */
#define FDFD_PROF_GEMM_SIMT 1  /* CUDA-core Schur-update GEMMs (flops)            */
#define FDFD_PROF_GJ_PANEL  2  /* Gauss-Jordan panel steps                        */
#define FDFD_PROF_SWEEP     3  /* solve sweeps: block GEMV (factor bytes read)    */
#define FDFD_PROF_RESIDUAL  4  /* FP64 stencil residual / product (bytes)         */
#define FDFD_PROF_OTHER     5  /* assembly, layout, Krylov vector kernels         */
#define FDFD_PROF_GJ_UPDATE 6  /* Gauss-Jordan rank-panel updates, either GEMM    */
                               /* (bytes: each matrix read and written once)      */
#define FDFD_PROF_LEVEL1    7  /* first reduction step: O(b^2) inverses and Schur */
                               /* updates (bytes of the blocks written)           */
int  fdfd_set_profiling(fdfd_handle* h, int on);
int  fdfd_get_profile(fdfd_handle* h, fdfd_profile* out);

/* Allocation-free residual: r = b - A x (or r = A x when b is NULL) and, per
 * right-hand side, norms[2k] = ||r_k||², norms[2k+1] = ||b_k||², for nrhs
 * stacked FP64 vectors.  No counterpart in the reference.  It exists for
 * callers that may not let a library call cudaMalloc/cudaFree: runtimes that
 * own all device memory through their own pool (CUDA.jl, PyTorch's caching
 * allocator, fixed-budget servers) and code that cannot take the device-wide
 * synchronisation those calls may imply.  Every pointer is a caller-owned
 * DEVICE pointer: stencil is the 5*Nx*Ny complex operator in the layout of
 * fdfd_get_stencil, x/b/r hold nrhs*Nx*Ny complex values, norms 2*nrhs
 * doubles.  stream is a cudaStream_t (NULL = default stream); the call
 * returns after the stream has finished its work.  Scratch: a fixed 1 MiB
 * device array of the library (block partial sums).  It is created when the
 * library's module loads on a device (with CUDA's default lazy loading, at the
 * first use there, which may allocate and synchronise once) and is held by
 * every GPU that loads it until exit; a caller that must never see an
 * allocation makes one warm-up call per device first.  Sizes with
 * ceil(Nx*Ny/256)*nrhs > 65536, or nrhs > 65535, are rejected with
 * FDFD_EINVAL.  The first call on a device resolves that array's device
 * address (cudaGetSymbolAddress) and should come before any stream capture;
 * the address is cached for the device's primary context and must not
 * outlive a cudaDeviceReset.  All calls share the array, so calls that
 * overlap on the GPU (other streams or threads) race; serialise them. */
int  fdfd_residual_noalloc(int Nx, int Ny, int nrhs, const double* stencil,
                           const double* x, const double* b, double* r,
                           double* norms, void* stream);

/* Test entry (no counterpart in the reference): eigenvalues w (n complex) and
 * unit eigenvectors V (n x n complex, row-major, column i for w[i]) of the
 * complex upper Hessenberg matrix H (n x n row-major interleaved): the
 * Ritz-pair solver of fdfd_eigfreq.  Host only. */
int  fdfd_debug_hessenberg_eig(int n, const double* H, double* w, double* V);

/* Kernel test entry (no counterpart in the reference): C = A·Bᵀ for complex
 * row-major interleaved host matrices A (M x K), B (N x K), C (M x N), through
 * the library's block GEMM: precision FDFD_PREC_FP64 (CUDA-core FP64) or
 * FDFD_PREC_MIXED (FP32 storage; use_tc = 1 selects the tcgen05 3xTF32
 * kernel with the library's tile choice, 64, 128 or 256 that kernel with
 * 128 x use_tc tiles, 129 its 128 x 128 tile sized for two CTAs per SM, 0
 * the CUDA-core FP32 kernel; a negative use_tc passes
 * the operands pre-split, as the Gauss-Jordan panel buffers are).  *ms (may
 * be NULL) receives the kernel time in milliseconds. */
int  fdfd_debug_gemm(int M, int N, int K, const double* A, const double* B,
                     double* C, int precision, int use_tc, double* ms);

#ifdef __cplusplus
}
#endif
#endif /* FDFD_CUDA_H */
