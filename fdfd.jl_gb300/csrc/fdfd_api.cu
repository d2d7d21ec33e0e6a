// libfdfd_cuda: handle, block cyclic reduction plan, factorization driver,
// sweeps, FP64 refinement and the C ABI declared in include/fdfd_cuda.h.
//
// Method.  With the unknowns of a grid line ("node", b = min(Nx, Ny) unknowns)
// grouped together, the FDFD operator is block-cyclic-tridiagonal over the
// n = max(Nx, Ny) nodes.  It is factored by block cyclic reduction: each step
// eliminates every other node of the current ring,
//     G_k = D_k⁻¹ (blocked Gauss-Jordan with partial pivoting),
//     X_L = G_k L_k,  X_R = G_k U_k,
//     D_p -= U_p X_L,  U_p' = -U_p X_R,  D_q -= L_q X_R,  L_q' = -L_q X_L,
// for k with ring neighbours p (previous) and q (next), until two nodes
// remain; they are merged and solved directly.  The first step has diagonal
// couplings and costs O(b²) per node beyond the inversions; every later step
// is dense complex GEMM work, batched over the eliminated nodes.
//
// The solve sweeps the steps forward (z_k = G_k r_k; r_p -= U_p z_k;
// r_q -= L_q z_k) and backward (x_k = z_k - X_L x_p - X_R x_q).
// FDFD_PREC_FP64 runs all of it in complex FP64; FDFD_PREC_MIXED stores the
// factors in complex FP32, forms the products with 3xTF32 tcgen05 MMAs, and
// recovers FP64 accuracy with flexible GMRES (or classic refinement) whose
// residuals b - A x and updates are FP64.
#include "fdfd_cuda.h"
#include "kernels.cuh"
#include "gemm_tc.cuh"
#include "hessenberg_eig.hpp"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <map>
#include <tuple>
#include <unordered_map>
#include <vector>

#define FDFD_VERSION_STR "fdfd_cuda 0.1.0 (sm_103a)"


namespace {

constexpr double kEPS0 = 8.85418782e-12;   // src/types.jl:6
constexpr double kMU0 = 1.25663706e-6;     // src/types.jl:7

typedef std::complex<double> zd;

struct StepPlan {
    std::vector<int> elim, eprev, enext;          // eliminated nodes and ring neighbours
    std::vector<int> surv, sprev, snext;          // survivors (ring order) and neighbours
    std::vector<char> sprev_elim, snext_elim;
};

template <typename T> struct DevArr {
    T* p = nullptr;
    size_t n = 0;
};

// all device-side integer job arrays of a plan live in one allocation
struct JobBlob {
    std::vector<unsigned char> host;
    size_t add(const void* src, size_t bytes) {
        size_t off = (host.size() + 15) & ~size_t(15);
        host.resize(off + bytes);
        if (bytes) memcpy(host.data() + off, src, bytes);
        return off;
    }
};

struct StepJobs {     // offsets into the job blob
    size_t elim = 0, l1 = 0, fwd1 = 0, fwd1y = 0, dswf = 0, dswb = 0, bwd1 = 0, bwd1y = 0;
    size_t xt_a = 0, xt_b = 0, xt_c = 0;
    size_t dp_a = 0, dp_b = 0, dp_c = 0, dq_a = 0, dq_b = 0, dq_c = 0;
    size_t cp_a = 0, cp_b = 0, cp_c = 0, cp_t = 0;
    size_t cpy = 0;
    size_t f2 = 0, f2y = 0, bw = 0, bwy = 0;
    size_t iota = 0;
    int ne = 0, ns = 0, nl1 = 0, ncp = 0, ncpy = 0, nf2 = 0;
    int nf2b = 0;         // coupling blocks the forward survivor jobs (f2) reference
};

template <typename T> struct FactorStore {
    Pool<T> D, C, X, GP, RP;
    Pool<T> Tg;                 // Gauss-Jordan ping-pong buffer (re, im planes)
    T* rv = nullptr; T* xv = nullptr; T* wv = nullptr;
    int vec_nrhs = 0;
    int* perm = nullptr;
    int* rowsrc = nullptr;      // per-panel composed row exchanges (two sets, panel parity)
    int* inv = nullptr;         // fused super-panels: inverse of the composed map (two sets)
    T* gsub = nullptr;          // fused super-panels: earlier G columns of a panel's pivot rows
    int* gj_slots = nullptr;    // 0 .. 2*max_ne-1: GP/RP slot lists of both parities
    cplx<T>* trifac = nullptr;  // first-step tridiagonal factors (8*b per node)
    int* tripiv = nullptr;      // and their interchanges (b per node)
    cplx<T>* sttab = nullptr;   // scaled stencil planes of every node in the factor precision (5*b per node)
    Pool<T> Wk;                 // split-K partial products (FP32 tensor-core path)
    int* wk_iota = nullptr;     // 0 .. Wk.count-1
    bool tc_ok = false;
    TcMaps tc;       // TMA descriptors (FP32 only)
    bool complete = false;   // every pool above allocated
    T* hC = nullptr;         // checkpoint mode: pinned host copies of every coupling ring ...
    T* hX = nullptr;         // ... and of every level's X blocks (original slot numbering)
};

}  // namespace

// Modulated device (multi-frequency FDFD, modulation.jl): K = 2s+1 sideband
// operators, each factored by its own handle, coupled through Δϵ.
struct MfState {
    int s = 0, K = 1;
    bool shared_pml = true;
    double omega = 0, Omega = 0;
    std::vector<double> wn;              // ωₙ = ω + nΩ, n = -s..s
    std::vector<fdfd_handle*> sub;       // one handle per sideband (its own stream)
    cplx<double>* deps = nullptr;        // Δϵᵣ (Nx*Ny, device)
    cudaEvent_t ev_in = nullptr;
    std::vector<cudaEvent_t> ev_out;
};

struct fdfd_handle {
    // problem
    int Nx, Ny, Npx, Npy, pol, precision;
    int num_sms = 1;             // streaming multiprocessors of the device (launch shapes)
    double dx, dy, L0, pml_m, pml_lnR;
    double tol = 1e-10;
    int max_iter = 40;
    int refine_mode = FDFD_REFINE_GMRES;
    int fact_prec = FDFD_PREC_FP64;  // precision of the current factor
    bool fallback = true;            // MIXED: re-factor in FP64 when the refinement would not converge
    int restart = 0;                 // FGMRES basis length (0: automatic)
    int nsb = 1;                     // Krylov vector length in units of Nx*Ny (K for a modulated device)
    long long kr_vlen = 0;           // vector length the Krylov workspace was sized for
    bool warm_start = false;         // next refine() starts from h->kx instead of 0 (consumed)
    // χ³ solve (nonlinear.jl): 0 off, 1 Born operator A + diag d1, 2 Newton's stacked system
    int nl_mode = 0;
    cplx<double>* nl_d1 = nullptr;
    cplx<double>* nl_d2 = nullptr;
    cplx<double>* nl_tmp = nullptr;  // 2N: conjugated preconditioner input (Newton)
    MfState* mf = nullptr;           // modulated device state (fdfd_mf_create), else null
    double mf_factor_ms = 0;         // wall time of the last fdfd_mf_factor
    unsigned char* mode_buf = nullptr;   // guided-mode scratch (jobs, vectors, sources)
    size_t mode_cap = 0;
    bool fell_back = false;          // the current factor is such an FP64 re-factorization
    NodeMap map;
    // state
    bool eps_set = false, factored = false;
    int op = OP_TM_DRIVEN;
    double omega = 0;            // frequency of the factored operator
    zd sigma = 0;                // eigen shift of the factored operator
    double scale = 1;            // factorization scaling of A
    std::string err;
    cudaStream_t stream = nullptr;
    cudaStream_t stream2 = nullptr;   // Gauss-Jordan look-ahead: the wide part of each panel update
    cudaEvent_t ev_panel = nullptr, ev_wide = nullptr;
    cudaEvent_t ev[8];
    long long launches = 0;
    long long dev_bytes = 0;
    long long dev_budget = 0;            // device bytes the handle may hold (0: no limit)
    AssembleArgs hargs;                  // assembly arguments (host copy) ...
    AssembleArgs* dargs = nullptr;       // ... and the device block the assembly kernels read
    std::unordered_map<void*, size_t> alloc_bytes;   // live dev_alloc buffers and their sizes
    unsigned long long wait_ns = 0;      // pipeline wait limit of the tensor-core GEMM (0: default)
    // FP64 device buffers (natural layout)
    cplx<double>* eps = nullptr;     // Nx*Ny
    cplx<double>* eps_stage = nullptr;   // fdfd_set_eps: the new ϵᵣ, validated before it replaces eps
    unsigned long long* vflags = nullptr;     // validate_kernel's first invalid entries (device) ...
    unsigned long long* vflags_h = nullptr;   // ... and their pinned host copy
    cplx<double>* sf = nullptr;      // 2*(2Nx+2Ny)
    cplx<double>* st = nullptr;      // 5*Nx*Ny
    unsigned* derr = nullptr;        // device error word
    double* part = nullptr;          // reduction partials
    double* red = nullptr;           // reduced values
    int part_blocks = 0;
    size_t part_cap = 0, red_cap = 0;
    // Krylov workspace (FP64 natural), sized for kr_nrhs right-hand sides
    cplx<double>* kb = nullptr;      // right-hand sides
    cplx<double>* kx = nullptr;      // solutions
    cplx<double>* kr = nullptr;      // residuals
    cplx<double>* kV = nullptr;      // (m+1) basis vectors
    cplx<double>* kZ = nullptr;      // m preconditioned vectors
    cplx<double>* kc = nullptr;      // small coefficient array
    cplx<double>* io = nullptr;      // staging for the host API (source + 3 fields)
    size_t io_cap = 0;
    int kr_nrhs = 0, kr_m = 0;
    // plan
    std::vector<StepPlan> steps;
    int fin_a = -1, fin_c = -1;
    std::vector<std::vector<int>> Lslot, Uslot;     // [e][node], e = 1..E
    std::vector<int> XL, XR;                        // [node]
    int Xf = -1, C01 = -1, C10 = -1;
    int nCslots = 0, nXslots = 0, max_ne = 0;
    // per ring e: first coupling slot and slot count; per level e >= 2: first X slot and count
    // (the plan's own numbering, kept as the host layout of checkpoint mode)
    std::vector<int> cring0, cringn, xlev0, xlevn;
    // checkpoint mode: coupling rings alternate between two device buffers and every level's X
    // blocks share one device window; completed rings and levels live in pinned host memory
    int ckpt_mode = 0;           // 0 automatic (when the resident factor storage does not fit), 1 on, -1 off
    bool ckpt = false;           // engaged (the slot tables are remapped to the windows)
    int ckpt_nA = 0;             // slots of the odd-ring coupling buffer (the even one follows)
    int orig_nC = 0, orig_nX = 0;   // slot counts of the resident layout
    long long host_bytes = 0, ckpt_copied = 0;
    std::vector<StepJobs> sj;
    size_t fin_mrg = 0, fin_c_slot = 0, fin_a_slot = 0, fin_xt_a = 0, fin_xt_b = 0, fin_xt_c = 0,
           fin_da_a = 0, fin_da_b = 0, fin_da_c = 0, fin_g1 = 0, fin_g1y = 0, fin_ra = 0, fin_ray = 0,
           fin_g0 = 0, fin_g0y = 0, fin_bx = 0, fin_bxy = 0, fin_iota = 0;
    unsigned char* djobs = nullptr;
    // factor storage
    FactorStore<float> f32;
    FactorStore<double> f64;
    double last_factor_flops = 0;
    int tc_used = 0;
    bool use_tc = true;
    bool level1_gj = false;     // invert first-step blocks by Gauss-Jordan instead of the O(b²) kernel
    bool tri_sweep = true;      // first-step sweep products through the tridiagonal factors, not the dense inverses
    // fdfd_factor through a captured CUDA graph: a second consecutive factorization at the same ω
    // captures the assembly and factorization; later ones at that ω replay it (ϵᵣ and the new
    // assembly arguments are read from device memory).  cfg_gen counts the changes a captured
    // graph depends on (storage, launch shapes, wait limit, checkpoint mode, budget).
    bool graph_factor = true;      // FDFD_FACTOR_GRAPH=0: plain launches only
    cudaGraph_t fgraph = nullptr;
    cudaGraphExec_t fgexec = nullptr;
    double fg_omega = 0, fg_scale = 0, last_plain_omega = -1;
    long long fg_kernels = 0;
    unsigned fg_gen = 0, cfg_gen = 1;
    // the preconditioner's sweep (node vectors rv -> xv) as a graph per factor precision, keyed by
    // the right-hand-side count, the vector buffer and cfg_gen; replayed by every FGMRES iteration
    cudaGraph_t sg_graph[2] = {nullptr, nullptr};
    cudaGraphExec_t sg_exec[2] = {nullptr, nullptr};
    int sg_nrhs[2] = {0, 0};
    const void* sg_rv[2] = {nullptr, nullptr};
    unsigned sg_gen[2] = {0, 0};
    long long sg_kernels[2] = {0, 0};
    bool splitk = true;            // split-K for tensor-core products whose tiles fill less than half the
                                   // SMs (FDFD_SPLITK=0: off)
    bool gemv_bulk = false;        // untuned N-form sweep products through the bulk-copy pipeline where it
                                   // fits (FDFD_GEMV_BULK=1), else register loads; the autotuner times both
    bool gj_presplit = true;       // FP32 panel buffers G, Rᵀ stored with their TF32 residual planes
                                   // (FDFD_GJ_PRESPLIT=0: two planes, split inside the GEMM)
    int gj_form = 0;               // one-CTA Gauss-Jordan panel: 0 lane-quad form, 1 pipelined row form
                                   // (FDFD_GJ_FORM)
    int gj_cl = -2;                // CTAs per matrix of the Gauss-Jordan panel (-2, the default: clusters of 8
                                   // for the deep levels, where eight CTAs per matrix fit in half of the SMs,
                                   // else one; 1: always one; 2/4/8: always that cluster; -1: the largest
                                   // cluster the level's matrix count fits; FDFD_GJ_CL)
    int gj_fused_k = 0;            // FP32 tensor-core Gauss-Jordan: columns of the panels that share one
                                   // update (0: one update per panel, the default; FDFD_GJ_FUSED_K)
    int gj_fused_min = 1;          // ... for batches of at least this many matrices
    // autotuner (fdfd_autotune): tile width per tensor-core GEMM shape (M, N, K, jobs, pre-split
    // operands) and launch shape per sweep product (form, jobs, right-hand sides per launch)
    std::map<std::tuple<int, int, int, int, int>, int> tune_gemm;
    std::map<std::tuple<int, int, int, int>, int> tune_gemv;   // (form, jobs, blocks per job, rhs) -> shape
    std::string tune_log;
    int force_bn = 0, force_shape = 0;   // set while the autotuner times a candidate
    // profiling (CUDA events around launches on the handle's stream)
    struct ProfRec { int cls, e0, e1; double work; };
    bool prof_on = false;
    std::vector<cudaEvent_t> evpool;
    std::vector<int> evfree;
    std::vector<ProfRec> recs;
    fdfd_profile prof_tot;
};

namespace {

// length of one refinement vector (unknowns of the solved system)
long long vlen(const fdfd_handle* h) { return (long long)h->Nx * h->Ny * h->nsb; }

// index of the first NaN/Inf in x[0..n), or -1.  Input validation runs on every
// host-buffer call, so each 4096-value chunk is first tested by a branch-free
// exponent test (vectorised by the compiler) and searched only if it fails.
long long first_nonfinite(const double* x, long long n) {
    constexpr uint64_t kExp = 0x7ff0000000000000ull;
    for (long long c = 0; c < n; c += 4096) {
        const long long e = std::min(n, c + 4096);
        uint64_t bad = 0;
        for (long long k = c; k < e; ++k) {
            uint64_t u;
            memcpy(&u, x + k, sizeof u);
            bad |= (uint64_t)((u & kExp) == kExp);
        }
        if (bad)
            for (long long k = c; k < e; ++k)
                if (!std::isfinite(x[k])) return k;
    }
    return -1;
}

int set_err(fdfd_handle* h, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (h) h->err = buf;
    return code;
}

#define CK(call)                                                                                    \
    do {                                                                                            \
        cudaError_t e_ = (call);                                                                    \
        if (e_ != cudaSuccess)                                                                      \
            return set_err(h, e_ == cudaErrorMemoryAllocation ? FDFD_ENOMEM : FDFD_ECUDA,           \
                           "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
    } while (0)

#define RET(x)                  \
    do {                        \
        int r_ = (x);           \
        if (r_ != FDFD_OK) return r_; \
    } while (0)

#define LAUNCH(kernel, grid, block, smem, ...)                                  \
    do {                                                                        \
        kernel<<<(grid), (block), (smem), h->stream>>>(__VA_ARGS__);            \
        h->launches++;                                                          \
    } while (0)

int check_launch(fdfd_handle* h, const char* where) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_err(h, FDFD_ECUDA, "kernel launch failed in %s: %s", where, cudaGetErrorString(e));
    return FDFD_OK;
}

int dev_alloc(fdfd_handle* h, void** p, size_t bytes) {
    if (bytes == 0) bytes = 16;
    if (h->dev_budget > 0 && h->dev_bytes + (long long)bytes > h->dev_budget) {
        *p = nullptr;
        return set_err(h, FDFD_ENOMEM, "device budget of %lld bytes exceeded: %lld held, %zu more requested",
                       h->dev_budget, h->dev_bytes, bytes);
    }
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        return set_err(h, FDFD_ENOMEM, "cudaMalloc(%zu bytes) failed: %s", bytes, cudaGetErrorString(e));
    }
    h->dev_bytes += (long long)bytes;
    h->alloc_bytes[*p] = bytes;
    return FDFD_OK;
}

// first invalid entries of n complex values already on the device (on the handle's
// stream, which it synchronises): *bad = lowest double index of a NaN/inf, *zero (may
// be null) = lowest complex index of a zero; -1 where there is none
int validate_device(fdfd_handle* h, const double* dx, long long n, bool zeros, long long* bad, long long* zero) {
    if (!h->vflags) RET(dev_alloc(h, (void**)&h->vflags, 2 * sizeof(unsigned long long)));
    if (!h->vflags_h && cudaMallocHost((void**)&h->vflags_h, 2 * sizeof(unsigned long long)) != cudaSuccess) {
        h->vflags_h = nullptr;
        return set_err(h, FDFD_ENOMEM, "pinned host allocation failed");
    }
    launch_validate(h->stream, h->num_sms, dx, n, zeros ? 1 : 0, h->vflags);
    h->launches++;
    CK(cudaMemcpyAsync(h->vflags_h, h->vflags, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    *bad = h->vflags_h[0] == ~0ull ? -1 : (long long)h->vflags_h[0];
    if (zero) *zero = (zeros && h->vflags_h[1] != ~0ull) ? (long long)h->vflags_h[1] : -1;
    return FDFD_OK;
}


// frees a dev_alloc'd buffer and returns its bytes to the handle's count
void dev_free(fdfd_handle* h, void* p) {
    if (!p) return;
    auto it = h->alloc_bytes.find(p);
    if (it != h->alloc_bytes.end()) {
        h->dev_bytes -= (long long)it->second;
        h->alloc_bytes.erase(it);
    }
    cudaFree(p);
}

// ---- profiling -------------------------------------------------------------
int prof_event(fdfd_handle* h) {
    if (h->evfree.empty()) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) return -1;
        h->evpool.push_back(e);
        return (int)h->evpool.size() - 1;
    }
    int i = h->evfree.back();
    h->evfree.pop_back();
    return i;
}
// returns the start event index (or -1 when profiling is off)
int prof_begin(fdfd_handle* h) {
    if (!h->prof_on) return -1;
    int e = prof_event(h);
    if (e >= 0) cudaEventRecord(h->evpool[e], h->stream);
    return e;
}
void prof_end(fdfd_handle* h, int e0, int cls, double work) {
    if (e0 < 0) return;
    int e1 = prof_event(h);
    if (e1 < 0) return;
    cudaEventRecord(h->evpool[e1], h->stream);
    h->recs.push_back({cls, e0, e1, work});
}
void prof_collect(fdfd_handle* h) {
    if (h->recs.empty()) return;
    cudaStreamSynchronize(h->stream);
    for (auto& r : h->recs) {
        float ms = 0;
        cudaEventElapsedTime(&ms, h->evpool[r.e0], h->evpool[r.e1]);
        h->prof_tot.ms[r.cls] += ms;
        h->prof_tot.work[r.cls] += r.work;
        h->prof_tot.launches[r.cls] += 1;
        h->evfree.push_back(r.e0);
        h->evfree.push_back(r.e1);
    }
    h->recs.clear();
}

// poll the device error word (synchronises the stream)
int check_device(fdfd_handle* h, const char* where) {
    unsigned e = 0;
    CK(cudaMemcpyAsync(&e, h->derr, sizeof e, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    if (e) {
        CK(cudaMemsetAsync(h->derr, 0, sizeof(unsigned), h->stream));
        if (e & FDFD_DEVERR_TIMEOUT)
            return set_err(h, FDFD_ETIMEOUT, "%s: a bounded device wait timed out", where);
        if (e & FDFD_DEVERR_SINGULAR)
            return set_err(h, FDFD_ESINGULAR, "%s: zero or non-finite pivot in a block inversion", where);
        return set_err(h, FDFD_ECUDA, "%s: device error 0x%x", where, e);
    }
    return FDFD_OK;
}

// ---------------------------------------------------------------------------
// Plan: ring sequence of the cyclic reduction, slot assignment, job arrays.
// ---------------------------------------------------------------------------
void build_plan(fdfd_handle* h) {
    const int n = h->map.n;
    h->steps.clear();
    std::vector<int> ring(n);
    for (int j = 0; j < n; ++j) ring[j] = j;
    std::vector<std::vector<int>> rings;
    rings.push_back(ring);
    while ((int)ring.size() > 2) {
        int m = (int)ring.size();
        StepPlan sp;
        std::vector<char> is_elim(m, 0);
        for (int pos = 1; pos < m; pos += 2) is_elim[pos] = 1;
        for (int pos = 1; pos < m; pos += 2) {
            sp.elim.push_back(ring[pos]);
            sp.eprev.push_back(ring[pos - 1]);
            sp.enext.push_back(ring[(pos + 1) % m]);
        }
        std::vector<int> next;
        for (int pos = 0; pos < m; pos += 2) {
            sp.surv.push_back(ring[pos]);
            int pp = (pos - 1 + m) % m, pn = (pos + 1) % m;
            sp.sprev.push_back(ring[pp]);
            sp.snext.push_back(ring[pn]);
            sp.sprev_elim.push_back(is_elim[pp]);
            sp.snext_elim.push_back(is_elim[pn]);
            next.push_back(ring[pos]);
        }
        h->steps.push_back(sp);
        ring = next;
        rings.push_back(ring);
    }
    h->fin_a = ring[0];
    h->fin_c = ring[1];
    const int E = (int)h->steps.size();   // rings[1..E] carry dense couplings
    // coupling slots
    h->Lslot.assign(E + 1, std::vector<int>(n, -1));
    h->Uslot.assign(E + 1, std::vector<int>(n, -1));
    int cs = 0;
    h->cring0.assign(E + 1, 0);
    h->cringn.assign(E + 1, 0);
    for (int e = 1; e <= E; ++e) {
        h->cring0[e] = cs;
        for (int s : rings[e]) { h->Lslot[e][s] = cs++; h->Uslot[e][s] = cs++; }
        h->cringn[e] = cs - h->cring0[e];
    }
    h->C01 = cs++;
    h->C10 = cs++;
    h->nCslots = cs;
    h->XL.assign(n, -1);
    h->XR.assign(n, -1);
    int xs = 0;
    h->max_ne = 1;
    h->xlev0.assign(E + 1, 0);
    h->xlevn.assign(E + 1, 0);
    for (int e = 1; e <= E; ++e) {
        const StepPlan& sp = h->steps[e - 1];
        h->max_ne = std::max(h->max_ne, (int)sp.elim.size());
        h->xlev0[e] = xs;
        if (e >= 2)
            for (int k : sp.elim) { h->XL[k] = xs++; h->XR[k] = xs++; }
        h->xlevn[e] = xs - h->xlev0[e];
    }
    h->Xf = xs++;
    h->nXslots = xs;
}

// storage form of node s's couplings in ring e: transposed iff s is eliminated next
bool coupling_trans(const fdfd_handle* h, int e, int s) {
    const int E = (int)h->steps.size();
    if (e == E) return s == h->fin_c;
    const StepPlan& nx = h->steps[e];   // step e+1
    return std::find(nx.elim.begin(), nx.elim.end(), s) != nx.elim.end();
}

void build_jobs(fdfd_handle* h, JobBlob& B) {
    const int E = (int)h->steps.size();
    h->sj.assign(E + 1, StepJobs());
    for (int e = 1; e <= E; ++e) {
        const StepPlan& sp = h->steps[e - 1];
        StepJobs& J = h->sj[e];
        const int ne = (int)sp.elim.size(), ns = (int)sp.surv.size();
        J.ne = ne; J.ns = ns;
        J.elim = B.add(sp.elim.data(), ne * sizeof(int));
        std::vector<int> iota(ne);
        for (int i = 0; i < ne; ++i) iota[i] = i;
        J.iota = B.add(iota.data(), ne * sizeof(int));
        // forward F1: z_k = G_k r_k
        std::vector<int4> f1(ne);
        std::vector<int2> f1y(ne);
        for (int i = 0; i < ne; ++i) { f1[i] = make_int4(sp.elim[i], sp.elim[i], -1, -1); f1y[i] = make_int2(sp.elim[i], -1); }
        J.fwd1 = B.add(f1.data(), ne * sizeof(int4));
        J.fwd1y = B.add(f1y.data(), ne * sizeof(int2));
        if (e == 1) {
            std::vector<L1Job> l1(ns);
            std::vector<int4> dswf, dswb(ne), b1(ne);
            std::vector<int2> b1y(ne);
            for (int i = 0; i < ns; ++i) {
                int s = sp.surv[i];
                L1Job j;
                j.s = s; j.prev = sp.sprev[i]; j.next = sp.snext[i];
                j.prev_elim = sp.sprev_elim[i]; j.next_elim = sp.snext_elim[i];
                j.u_slot = h->Uslot[1][s]; j.l_slot = h->Lslot[1][s];
                j.u_trans = j.l_trans = coupling_trans(h, 1, s) ? 1 : 0;
                l1[i] = j;
                int flags = (sp.sprev_elim[i] ? 1 : 0) | (sp.snext_elim[i] ? 2 : 0);
                if (flags) dswf.push_back(make_int4(s, sp.sprev[i], sp.snext[i], flags));
            }
            for (int i = 0; i < ne; ++i) {
                dswb[i] = make_int4(sp.elim[i], sp.eprev[i], sp.enext[i], 3);
                b1[i] = make_int4(sp.elim[i], sp.elim[i], -1, -1);     // G_k · w_k
                b1y[i] = make_int2(sp.elim[i], sp.elim[i]);
            }
            J.l1 = B.add(l1.data(), ns * sizeof(L1Job));
            J.nl1 = ns;
            J.dswf = B.add(dswf.data(), dswf.size() * sizeof(int4));
            J.nf2 = (int)dswf.size();
            J.dswb = B.add(dswb.data(), ne * sizeof(int4));
            J.bwd1 = B.add(b1.data(), ne * sizeof(int4));
            J.bwd1y = B.add(b1y.data(), ne * sizeof(int2));
        } else {
            std::vector<int> xa(2 * ne), xb(2 * ne), xc(2 * ne);
            std::vector<int> dpa(ne), dpb(ne), dpc(ne), dqa(ne), dqb(ne), dqc(ne);
            std::vector<int> cpa(2 * ne), cpb(2 * ne), cpc(2 * ne), cpt(2 * ne);
            std::vector<int4> bw(ne);
            std::vector<int2> bwy(ne);
            for (int i = 0; i < ne; ++i) {
                int k = sp.elim[i], p = sp.eprev[i], q = sp.enext[i];
                xa[i] = h->Lslot[e - 1][k]; xb[i] = k; xc[i] = h->XL[k];
                xa[ne + i] = h->Uslot[e - 1][k]; xb[ne + i] = k; xc[ne + i] = h->XR[k];
                dpa[i] = h->Uslot[e - 1][p]; dpb[i] = h->XL[k]; dpc[i] = p;
                dqa[i] = h->Lslot[e - 1][q]; dqb[i] = h->XR[k]; dqc[i] = q;
                cpa[i] = h->Uslot[e - 1][p]; cpb[i] = h->XR[k]; cpc[i] = h->Uslot[e][p];
                cpt[i] = coupling_trans(h, e, p) ? 1 : 0;
                cpa[ne + i] = h->Lslot[e - 1][q]; cpb[ne + i] = h->XL[k]; cpc[ne + i] = h->Lslot[e][q];
                cpt[ne + i] = coupling_trans(h, e, q) ? 1 : 0;
                bw[i] = make_int4(h->XL[k], p, h->XR[k], q);
                bwy[i] = make_int2(k, k);
            }
            J.xt_a = B.add(xa.data(), 2 * ne * sizeof(int));
            J.xt_b = B.add(xb.data(), 2 * ne * sizeof(int));
            J.xt_c = B.add(xc.data(), 2 * ne * sizeof(int));
            J.dp_a = B.add(dpa.data(), ne * sizeof(int)); J.dp_b = B.add(dpb.data(), ne * sizeof(int));
            J.dp_c = B.add(dpc.data(), ne * sizeof(int));
            J.dq_a = B.add(dqa.data(), ne * sizeof(int)); J.dq_b = B.add(dqb.data(), ne * sizeof(int));
            J.dq_c = B.add(dqc.data(), ne * sizeof(int));
            J.cp_a = B.add(cpa.data(), 2 * ne * sizeof(int)); J.cp_b = B.add(cpb.data(), 2 * ne * sizeof(int));
            J.cp_c = B.add(cpc.data(), 2 * ne * sizeof(int)); J.cp_t = B.add(cpt.data(), 2 * ne * sizeof(int));
            J.ncp = 2 * ne;
            // couplings that cross no eliminated node: copied (transposed if the form changes)
            std::vector<int3> cpy;
            std::vector<int4> f2;
            std::vector<int2> f2y;
            for (int i = 0; i < ns; ++i) {
                int s = sp.surv[i];
                int tr = coupling_trans(h, e, s) ? 1 : 0;
                if (!sp.snext_elim[i]) cpy.push_back(make_int3(h->Uslot[e][s], h->Uslot[e - 1][s], tr));
                if (!sp.sprev_elim[i]) cpy.push_back(make_int3(h->Lslot[e][s], h->Lslot[e - 1][s], tr));
                if (sp.snext_elim[i] || sp.sprev_elim[i]) {
                    f2.push_back(make_int4(sp.snext_elim[i] ? h->Uslot[e - 1][s] : -1, sp.snext[i],
                                           sp.sprev_elim[i] ? h->Lslot[e - 1][s] : -1, sp.sprev[i]));
                    f2y.push_back(make_int2(s, s));
                    J.nf2b += (sp.snext_elim[i] ? 1 : 0) + (sp.sprev_elim[i] ? 1 : 0);
                }
            }
            J.cpy = B.add(cpy.data(), cpy.size() * sizeof(int3));
            J.ncpy = (int)cpy.size();
            J.f2 = B.add(f2.data(), f2.size() * sizeof(int4));
            J.f2y = B.add(f2y.data(), f2y.size() * sizeof(int2));
            J.nf2 = (int)f2.size();
            J.bw = B.add(bw.data(), ne * sizeof(int4));
            J.bwy = B.add(bwy.data(), ne * sizeof(int2));
        }
    }
    // final two nodes
    const int a = h->fin_a, c = h->fin_c;
    int3 mrg[2] = {make_int3(h->C01, h->Uslot[E][a], h->Lslot[E][a]),
                   make_int3(h->C10, h->Uslot[E][c], h->Lslot[E][c])};
    h->fin_mrg = B.add(mrg, sizeof mrg);
    h->fin_c_slot = B.add(&c, sizeof(int));
    h->fin_a_slot = B.add(&a, sizeof(int));
    int zero = 0;
    h->fin_iota = B.add(&zero, sizeof(int));
    h->fin_xt_a = B.add(&h->C10, sizeof(int));
    h->fin_xt_b = B.add(&c, sizeof(int));
    h->fin_xt_c = B.add(&h->Xf, sizeof(int));
    h->fin_da_a = B.add(&h->C01, sizeof(int));
    h->fin_da_b = B.add(&h->Xf, sizeof(int));
    h->fin_da_c = B.add(&a, sizeof(int));
    int4 g1 = make_int4(c, c, -1, -1); int2 g1y = make_int2(c, -1);
    int4 ra = make_int4(h->C01, c, -1, -1); int2 ray = make_int2(a, a);
    int4 g0 = make_int4(a, a, -1, -1); int2 g0y = make_int2(a, -1);
    int4 bx = make_int4(h->Xf, a, -1, -1); int2 bxy = make_int2(c, c);
    h->fin_g1 = B.add(&g1, sizeof g1); h->fin_g1y = B.add(&g1y, sizeof g1y);
    h->fin_ra = B.add(&ra, sizeof ra); h->fin_ray = B.add(&ray, sizeof ray);
    h->fin_g0 = B.add(&g0, sizeof g0); h->fin_g0y = B.add(&g0y, sizeof g0y);
    h->fin_bx = B.add(&bx, sizeof bx); h->fin_bxy = B.add(&bxy, sizeof bxy);
}

template <typename U> U* J(fdfd_handle* h, size_t off) { return reinterpret_cast<U*>(h->djobs + off); }

// ---------------------------------------------------------------------------
// Factor storage
// ---------------------------------------------------------------------------
template <typename T> FactorStore<T>& store(fdfd_handle* h);
template <> FactorStore<float>& store<float>(fdfd_handle* h) { return h->f32; }
template <> FactorStore<double>& store<double>(fdfd_handle* h) { return h->f64; }

// Gauss-Jordan panel width: the panel lives in registers, one (b <= 512) or two
// (b <= 1024) rows per thread of a 512-thread block.
template <typename T> int panel_nb(int b) {
    if (sizeof(T) == 4) return b <= 512 ? 32 : 16;
    return b <= 512 ? 16 : 8;
}

template <typename T> int alloc_pool(fdfd_handle* h, Pool<T>& P, int rows, int cols, int ld, int planes,
                                     long long count) {
    P.rows = rows; P.cols = cols; P.ld = ld; P.planes = planes; P.count = count;
    size_t bytes = (size_t)P.slot_elems() * count * sizeof(T);
    void* p = nullptr;
    RET(dev_alloc(h, &p, bytes));
    P.base = (T*)p;
    return FDFD_OK;
}

template <typename T> void free_store(fdfd_handle* h, FactorStore<T>& F) {
    h->cfg_gen++;   // a captured factorization addresses this storage
    void* bufs[] = {F.D.base, F.C.base, F.X.base, F.GP.base, F.RP.base, F.Tg.base, F.rv, F.xv, F.wv,
                    F.perm, F.rowsrc, F.inv, F.gsub, F.gj_slots, F.trifac, F.tripiv, F.sttab, F.Wk.base,
                    F.wk_iota};
    for (void* p : bufs) dev_free(h, p);
    if (F.hC || F.hX) {
        const long long se = F.C.slot_elems();
        h->host_bytes -= (long long)sizeof(T) * se * ((F.hC ? h->orig_nC - 2 : 0) + (F.hX ? h->orig_nX - 1 : 0));
    }
    if (F.hC) cudaFreeHost(F.hC);
    if (F.hX) cudaFreeHost(F.hX);
    F = FactorStore<T>();
}

// ---------------------------------------------------------------------------
// Checkpoint mode: block factors beyond HBM.  Resident, the factor storage is
// n D blocks, about 2n coupling blocks (two per survivor of every ring) and
// about n X blocks.  The couplings of ring e are written at step e and read at
// step e+1; the X blocks of step e are read only within step e; after that both
// serve only the solve sweeps.  In checkpoint mode the rings alternate between
// two device buffers (odd and even e) and all steps' X blocks share one device
// window; when step e ends, its X blocks and ring e-1 are copied to pinned host
// memory (one cudaMemcpyAsync each, in the plan's slot order), and each sweep
// copies them back step by step before the products that read them.  The device
// then holds n + ~1.5n + ~n/2 blocks instead of ~4n; the sweeps move the
// couplings and X blocks over the host link every time.
// ---------------------------------------------------------------------------
int restart_len(const fdfd_handle* h, int nrhs);

// K slices of a tensor-core product with bcols-wide tiles: a product whose tiles fill less
// than half of the SMs is split along K (at most 8 slices of at least 64 columns, at most
// SPLITK_SLOTS partial products per launch) so that its CTAs cover the GPU; 1 = no split
constexpr int SPLITK_SLOTS = 64;
static int splitk_of(const fdfd_handle* h, int M, int N, int K, int njobs, int bcols) {
    if (!h->splitk || K < 256) return 1;
    const long long tiles = (long long)ceil_div(M, 128) * ceil_div(N, bcols) * njobs;
    if (2 * tiles > h->num_sms) return 1;
    int ks = (int)std::min<long long>(8, h->num_sms / tiles);
    ks = std::min(ks, K / 64);
    while (ks > 1 && (long long)njobs * ks > SPLITK_SLOTS) --ks;
    return ks < 2 ? 1 : ks;
}

// device bytes the factorization and a one-source solve will add, resident and in
// checkpoint mode: D, C and X blocks, the Gauss-Jordan and first-step work space,
// the sweep vectors and the FP64 Krylov basis (estimates of the later allocations)
template <typename T> void factor_bytes(const fdfd_handle* h, double* resident, double* windowed) {
    const int b = h->map.b, n = h->map.n, ld = h->map.ld;
    const double sb = (double)b * ld * 2 * sizeof(T);
    int nA = 0, nB = 0, nXw = 0, gj_max = 1;
    for (int e = 1; e < (int)h->cringn.size(); ++e) {
        if (e & 1) nA = std::max(nA, h->cringn[e]);
        else nB = std::max(nB, h->cringn[e]);
        nXw = std::max(nXw, h->xlevn[e]);
        if (e >= 2 && e < (int)h->sj.size()) gj_max = std::max(gj_max, h->sj[e].ne);
    }
    const int nC = h->ckpt ? h->orig_nC : h->nCslots, nX = h->ckpt ? h->orig_nX : h->nXslots;
    const double N = (double)h->Nx * h->Ny;
    const double wk = (sizeof(T) == 4 && h->use_tc && h->splitk && b >= 256) ? sb * SPLITK_SLOTS : 0.0;   // split-K
    const double work = wk + sb * gj_max + 2.0 * 2 * h->max_ne * b * 32 * 4 * sizeof(T) + 3.0 * h->max_ne * b * 4 +
                        (double)n * 14 * b * sizeof(cplx<T>) + 3.0 * n * 2 * ld * sizeof(T) +
                        (2.0 * restart_len(h, 1) + 4) * N * sizeof(cplx<double>);
    *resident = sb * (n + nC + nX) + work;
    *windowed = sb * (n + nA + nB + 2 + nXw + 1) + work;
}

// remaps the coupling and X slot tables onto the device windows and rebuilds the job lists
int ckpt_engage(fdfd_handle* h) {
    h->cfg_gen++;
    const int E = (int)h->steps.size();
    int nA = 0, nB = 0, nXw = 0;
    for (int e = 1; e <= E; ++e) {
        if (e & 1) nA = std::max(nA, h->cringn[e]);
        else nB = std::max(nB, h->cringn[e]);
        nXw = std::max(nXw, h->xlevn[e]);
    }
    h->orig_nC = h->nCslots;
    h->orig_nX = h->nXslots;
    for (int e = 1; e <= E; ++e) {
        const int base = (e & 1) ? 0 : nA;
        for (int& v : h->Lslot[e]) if (v >= 0) v = v - h->cring0[e] + base;
        for (int& v : h->Uslot[e]) if (v >= 0) v = v - h->cring0[e] + base;
        if (e >= 2)
            for (int k : h->steps[e - 1].elim) { h->XL[k] -= h->xlev0[e]; h->XR[k] -= h->xlev0[e]; }
    }
    h->C01 = nA + nB;
    h->C10 = nA + nB + 1;
    h->nCslots = nA + nB + 2;
    h->Xf = nXw;
    h->nXslots = nXw + 1;
    h->ckpt_nA = nA;
    JobBlob B;
    build_jobs(h, B);
    CK(cudaMemcpy(h->djobs, B.host.data(), B.host.size(), cudaMemcpyHostToDevice));
    h->ckpt = true;
    return FDFD_OK;
}

// device buffer of ring e's couplings in checkpoint mode
template <typename T> T* ckpt_ring_dev(fdfd_handle* h, int e) {
    FactorStore<T>& F = store<T>(h);
    return F.C.slot((e & 1) ? 0 : h->ckpt_nA);
}

// end of step e: its X blocks and ring e-1 to the host
template <typename T> int ckpt_offload(fdfd_handle* h, int e) {
    if (!h->ckpt || e < 2) return FDFD_OK;
    FactorStore<T>& F = store<T>(h);
    const size_t se = (size_t)F.C.slot_elems();
    if (h->xlevn[e]) {
        const size_t bytes = se * h->xlevn[e] * sizeof(T);
        CK(cudaMemcpyAsync(F.hX + se * h->xlev0[e], F.X.slot(0), bytes, cudaMemcpyDeviceToHost, h->stream));
        h->ckpt_copied += (long long)bytes;
    }
    if (h->cringn[e - 1]) {
        const size_t bytes = se * h->cringn[e - 1] * sizeof(T);
        CK(cudaMemcpyAsync(F.hC + se * h->cring0[e - 1], ckpt_ring_dev<T>(h, e - 1), bytes, cudaMemcpyDeviceToHost,
                           h->stream));
        h->ckpt_copied += (long long)bytes;
    }
    return FDFD_OK;
}

// sweeps: ring e back to its device buffer, or step e's X blocks back to the window
template <typename T> int ckpt_reload_ring(fdfd_handle* h, int e) {
    if (!h->ckpt || !h->cringn[e]) return FDFD_OK;
    FactorStore<T>& F = store<T>(h);
    const size_t se = (size_t)F.C.slot_elems(), bytes = se * h->cringn[e] * sizeof(T);
    CK(cudaMemcpyAsync(ckpt_ring_dev<T>(h, e), F.hC + se * h->cring0[e], bytes, cudaMemcpyHostToDevice, h->stream));
    h->ckpt_copied += (long long)bytes;
    return FDFD_OK;
}
template <typename T> int ckpt_reload_x(fdfd_handle* h, int e) {
    if (!h->ckpt || !h->xlevn[e]) return FDFD_OK;
    FactorStore<T>& F = store<T>(h);
    const size_t se = (size_t)F.C.slot_elems(), bytes = se * h->xlevn[e] * sizeof(T);
    CK(cudaMemcpyAsync(F.X.slot(0), F.hX + se * h->xlev0[e], bytes, cudaMemcpyHostToDevice, h->stream));
    h->ckpt_copied += (long long)bytes;
    return FDFD_OK;
}

template <typename T> int alloc_factor_pools(fdfd_handle* h);

// factor storage of precision T: all of it, or (on failure) none of it
template <typename T> int alloc_factor(fdfd_handle* h) {
    FactorStore<T>& F = store<T>(h);
    if (F.complete) return FDFD_OK;
    const int rc = alloc_factor_pools<T>(h);
    if (rc != FDFD_OK) {
        free_store(h, F);
        return rc;
    }
    F.complete = true;
    return FDFD_OK;
}

template <typename T> int alloc_factor_pools(fdfd_handle* h) {
    FactorStore<T>& F = store<T>(h);
    const int b = h->map.b, n = h->map.n, ld = h->map.ld;
    // checkpoint mode: forced, or automatic when the resident storage would not fit what is
    // left of the device budget (or of the device's free memory) but the windowed one does
    if (!h->ckpt && h->ckpt_mode >= 0 && h->steps.size() >= 2) {
        double resident = 0, windowed = 0;
        factor_bytes<T>(h, &resident, &windowed);
        double avail = 0;
        if (h->dev_budget > 0) {
            avail = (double)(h->dev_budget - h->dev_bytes);
        } else {
            size_t fr = 0, tot = 0;
            if (cudaMemGetInfo(&fr, &tot) == cudaSuccess) avail = 0.95 * (double)fr;
            else cudaGetLastError();
        }
        if (h->ckpt_mode == 1 || (avail > 0 && resident > avail && windowed < avail)) RET(ckpt_engage(h));
    }
    const int planes = 2;   // re, im (the tensor-core GEMM forms the TF32 residuals itself)
    // panel buffer width: one panel, or (fused super-panels, FP32 tensor-core path) the
    // gj_fused_k columns of the panels that share one update
    const bool fused = sizeof(T) == 4 && h->use_tc && h->gj_fused_k > panel_nb<T>(b);
    const int pc = fused ? (h->gj_fused_k + 31) / 32 * 32 : (sizeof(T) == 4 ? 32 : panel_nb<T>(b));
    RET(alloc_pool<T>(h, F.D, b, b, ld, planes, n));
    RET(alloc_pool<T>(h, F.C, b, b, ld, planes, h->nCslots));
    RET(alloc_pool<T>(h, F.X, b, b, ld, planes, h->nXslots));
    // the panel buffers are short-K tensor-core operands: stored pre-split (re, im, re_lo, im_lo),
    // unless gj_presplit is off (the GEMM then forms the residual planes itself)
    const int pplanes = (sizeof(T) == 4 && h->gj_presplit) ? 4 : 2;
    // two sets (panel parity) so that a panel can run while the previous panel's update reads the other set
    RET(alloc_pool<T>(h, F.GP, b, pc, pc, pplanes, 2 * h->max_ne));
    RET(alloc_pool<T>(h, F.RP, b, pc, pc, pplanes, 2 * h->max_ne));
    // split-K work space: the most slices any Schur product of the plan can take
    if (sizeof(T) == 4 && h->use_tc && h->splitk) {
        long long wk = 0;
        auto need = [&](int nj) {
            for (int bc : {64, 128, 256}) {
                const int ks = splitk_of(h, b, b, b, nj, bc);
                if (ks > 1) wk = std::max(wk, (long long)nj * ks);
            }
        };
        for (int e = 2; e < (int)h->sj.size(); ++e) {
            need(2 * h->sj[e].ne);
            need(h->sj[e].ne);
            need(h->sj[e].ncp);
        }
        need(1);
        if (wk > 1) {
            RET(alloc_pool<T>(h, F.Wk, b, b, ld, 2, wk));
            std::vector<int> io(wk);
            for (long long i = 0; i < wk; ++i) io[i] = (int)i;
            RET(dev_alloc(h, (void**)&F.wk_iota, io.size() * sizeof(int)));
            CK(cudaMemcpy(F.wk_iota, io.data(), io.size() * sizeof(int), cudaMemcpyHostToDevice));
        }
    }
    {
        std::vector<int> sl(2 * h->max_ne);
        for (int i = 0; i < 2 * h->max_ne; ++i) sl[i] = i;
        RET(dev_alloc(h, (void**)&F.gj_slots, sl.size() * sizeof(int)));
        CK(cudaMemcpy(F.gj_slots, sl.data(), sl.size() * sizeof(int), cudaMemcpyHostToDevice));
    }
    RET(dev_alloc(h, (void**)&F.perm, (size_t)h->max_ne * b * sizeof(int)));
    RET(dev_alloc(h, (void**)&F.rowsrc, (size_t)2 * h->max_ne * b * sizeof(int)));
    if (fused) {
        RET(dev_alloc(h, (void**)&F.inv, (size_t)2 * h->max_ne * b * sizeof(int)));
        RET(dev_alloc(h, (void**)&F.gsub, (size_t)h->max_ne * 2 * panel_nb<T>(b) * pc * sizeof(T)));
    }
    // largest Gauss-Jordan batch: the eliminated nodes of steps >= 2 (and of step 1
    // when it inverts by Gauss-Jordan), or the final pair's single matrices
    int gj_max = 1;
    for (int e = 1; e < (int)h->sj.size(); ++e)
        if (e >= 2 || h->level1_gj) gj_max = std::max(gj_max, h->sj[e].ne);
    RET(alloc_pool<T>(h, F.Tg, b, b, ld, 2, gj_max));
    if (h->sj.size() > 1 && !h->level1_gj) {
        const size_t n1 = (size_t)std::max(1, h->sj[1].ne);
        RET(dev_alloc(h, (void**)&F.trifac, n1 * 8 * b * sizeof(cplx<T>)));
        RET(dev_alloc(h, (void**)&F.tripiv, n1 * b * sizeof(int)));
    }
    if (h->sj.size() > 1) RET(dev_alloc(h, (void**)&F.sttab, (size_t)h->map.n * 5 * b * sizeof(cplx<T>)));
    if (h->ckpt) {
        const size_t se = (size_t)F.C.slot_elems() * sizeof(T);
        const size_t bc = se * (h->orig_nC - 2), bx = se * (h->orig_nX - 1);
        if (cudaHostAlloc((void**)&F.hC, std::max<size_t>(bc, 16), cudaHostAllocDefault) != cudaSuccess) {
            cudaGetLastError();
            F.hC = nullptr;
            return set_err(h, FDFD_ENOMEM, "pinned host memory for the checkpointed couplings (%zu bytes) failed", bc);
        }
        h->host_bytes += (long long)bc;
        if (cudaHostAlloc((void**)&F.hX, std::max<size_t>(bx, 16), cudaHostAllocDefault) != cudaSuccess) {
            cudaGetLastError();
            F.hX = nullptr;
            return set_err(h, FDFD_ENOMEM, "pinned host memory for the checkpointed X blocks (%zu bytes) failed", bx);
        }
        h->host_bytes += (long long)bx;
    }
    if (sizeof(T) == 4 && h->use_tc) {
        F.tc_ok = tc_make_maps(reinterpret_cast<Pool<float>*>(&F.D), reinterpret_cast<Pool<float>*>(&F.C),
                               reinterpret_cast<Pool<float>*>(&F.X), reinterpret_cast<Pool<float>*>(&F.GP),
                               reinterpret_cast<Pool<float>*>(&F.RP), &F.tc);
    }
    return FDFD_OK;
}

template <typename T> int alloc_vectors(fdfd_handle* h, int nrhs) {
    FactorStore<T>& F = store<T>(h);
    if (F.vec_nrhs >= nrhs) return FDFD_OK;
    dev_free(h, F.rv); dev_free(h, F.xv); dev_free(h, F.wv);
    F.rv = F.xv = F.wv = nullptr;
    F.vec_nrhs = 0;   // stays 0 unless all three allocations succeed
    size_t bytes = (size_t)h->map.n * nrhs * 2 * h->map.ld * sizeof(T);
    RET(dev_alloc(h, (void**)&F.rv, bytes));
    RET(dev_alloc(h, (void**)&F.xv, bytes));
    RET(dev_alloc(h, (void**)&F.wv, bytes));
    CK(cudaMemsetAsync(F.rv, 0, bytes, h->stream));
    CK(cudaMemsetAsync(F.xv, 0, bytes, h->stream));
    CK(cudaMemsetAsync(F.wv, 0, bytes, h->stream));
    F.vec_nrhs = nrhs;
    return FDFD_OK;
}

// ---------------------------------------------------------------------------
// GEMM dispatch
// ---------------------------------------------------------------------------
enum PoolId { P_D = 0, P_C = 1, P_X = 2, P_GP = 3, P_RP = 4, P_TG = 5 };

template <typename T> Pool<T>& pool_of(FactorStore<T>& F, int id) {
    switch (id) {
        case P_D: return F.D;
        case P_C: return F.C;
        case P_X: return F.X;
        case P_GP: return F.GP;
        case P_TG: return F.Tg;
        default: return F.RP;
    }
}

template <typename T>
int gemm(fdfd_handle* h, int pa, int pb, int pc, const int* a_slot, const int* b_slot, const int* c_slot,
         const int* c_trans_arr, int c_trans, int njobs, int M, int N, int K, T alpha, int beta, int mask_c0,
         int mask_w, int pcin = -1, const int* cin_slot = nullptr,
         const int* row_src = nullptr, int prof_cls = -1, double prof_work = 0.0, cudaStream_t stream = nullptr,
         int n_off = 0, int skip_c0 = 0, int skip_w = 0, int a_pool_slot0 = 0, const int* row_dst = nullptr) {
    if (njobs == 0) return FDFD_OK;
    FactorStore<T>& F = store<T>(h);
    if (!stream) stream = h->stream;
    GemmArgs<T> g;
    g.A = pool_of(F, pa); g.B = pool_of(F, pb); g.C = pool_of(F, pc);
    g.a_slot = a_slot; g.b_slot = b_slot; g.c_slot = c_slot;
    g.Cin = pcin >= 0 ? pool_of(F, pcin) : Pool<T>();
    g.cin_slot = cin_slot; g.row_src = row_src;
    g.M = M; g.N = N; g.K = K; g.alpha = alpha; g.beta = beta;
    g.mask_c0 = mask_c0; g.mask_w = mask_w; g.c_trans = c_trans;
    g.n_off = n_off; g.skip_c0 = skip_c0; g.skip_w = skip_w;
    g.c_trans_arr = nullptr;
    g.row_dst = row_dst;
    g.err = h->derr;
    g.wait_ns = h->wait_ns;
    const double flops = 8.0 * M * N * K * njobs;
    int ev = prof_begin(h);
    if (sizeof(T) == 4 && F.tc_ok) {
        int bn = h->force_bn;
        if (!bn) {
            auto it = h->tune_gemm.find(std::make_tuple(M, N, K, njobs, (int)(g.A.planes == 4)));
            if (it != h->tune_gemm.end()) bn = it->second;
        }
        // split-K (deterministic): partial products into the Wk slots, then their ordered sum
        // with the α, β and storage form of the product
        const int bne = (bn == 64 || bn == 128 || bn == 256 || bn == TC_BN128_TWO) ? bn
                                                                                   : tc_pick_bn(M, N, K, njobs, h->num_sms);
        int ks = (F.Wk.base && mask_w == 0 && n_off == 0 && skip_w == 0 && !row_dst && !row_src && pcin < 0 &&
                  g.A.planes == 2)
                     ? splitk_of(h, M, N, K, njobs, bne == TC_BN128_TWO ? 128 : bne)
                     : 1;
        int rc = 0;
        if constexpr (sizeof(T) != 4) ks = 1;   // (the tensor-core path is FP32 only)
        else if (ks > 1) {
            GemmArgs<T> pg = g;
            pg.kslice = ceil_div(K, ks * 8) * 8;
            ks = ceil_div(K, pg.kslice);
            pg.ksplit = ks;
            pg.C = F.Wk;
            pg.c_slot = F.wk_iota;
            pg.alpha = (T)1;
            pg.beta = 0;
            pg.c_trans = 0;
            if ((long long)njobs * ks > F.Wk.count || M > F.Wk.rows || N > F.Wk.cols) ks = 1;
            else {
                rc = tc_gemm_launch(reinterpret_cast<GemmArgs<float>*>(&pg), nullptr, pa, pb, njobs, &F.tc,
                                    h->num_sms, stream, bn);
                if (rc == 0)
                    rc = tc_splitk_sum(F.Wk, ks, g.C, c_slot, c_trans_arr, c_trans, njobs, M, N, (float)alpha, beta,
                                       stream);
                h->launches++;
            }
        }
        if (ks <= 1)
            rc = tc_gemm_launch(reinterpret_cast<GemmArgs<float>*>(&g), c_trans_arr, pa, pb, njobs, &F.tc,
                                h->num_sms, stream, bn);
        if (rc != 0) return set_err(h, FDFD_ECUDA, "tcgen05 GEMM launch failed (%d)", rc);
        prof_end(h, ev, prof_cls >= 0 ? prof_cls : FDFD_PROF_GEMM_TC, prof_cls >= 0 ? prof_work : flops);
        h->launches++;
        h->tc_used = 1;
        return check_launch(h, "gemm_tc");
    }
    if (n_off || skip_w || row_dst) return set_err(h, FDFD_EINVAL, "column windows need the tensor-core GEMM");
    g.c_trans_arr = c_trans_arr;
    launch_gemm_simt<T>(stream, njobs, g);
    prof_end(h, ev, prof_cls >= 0 ? prof_cls : FDFD_PROF_GEMM_SIMT, prof_cls >= 0 ? prof_work : flops);
    h->launches++;
    return check_launch(h, "gemm_simt");
}

// ---------------------------------------------------------------------------
// Gauss-Jordan inversion of D-pool slots (batched)
// ---------------------------------------------------------------------------
int gj_invert_fused(fdfd_handle* h, const int* d_slots, const int* d_iota, int njobs);

// block-wait limit of the kernels with bounded waits (the handle's, else 2 s)
static uint64_t wait_limit(const fdfd_handle* h) { return h->wait_ns ? h->wait_ns : FDFD_WAIT_LIMIT_NS; }

// CTAs per matrix of the Gauss-Jordan panel: a level with few matrices spreads each
// panel over a cluster of CTAs, as many as keep every cluster resident at once
static int gj_cluster(const fdfd_handle* h, int njobs) {
    if (h->gj_cl == 1 || h->gj_cl == 2 || h->gj_cl == 4 || h->gj_cl == 8) return h->gj_cl > 1 ? h->gj_cl : 0;
    if (h->gj_cl == -2)   // deep levels only: eight CTAs per matrix within half of the SMs
        return (long long)njobs * 8 * 2 <= h->num_sms ? 8 : 0;
    for (int cl : {8, 4, 2})
        if ((long long)njobs * cl <= h->num_sms) return cl;
    return 0;
}

template <typename T> int gj_invert(fdfd_handle* h, const int* d_slots, const int* d_iota, int njobs) {
    if (njobs == 0) return FDFD_OK;
    FactorStore<T>& F = store<T>(h);
    if constexpr (sizeof(T) == 4)
        if (F.tc_ok && F.inv && njobs >= h->gj_fused_min) return gj_invert_fused(h, d_slots, d_iota, njobs);
    const int b = h->map.b;
    const int nb = panel_nb<T>(b);
    if (njobs > F.Tg.count) return set_err(h, FDFD_EINVAL, "Gauss-Jordan batch %d exceeds %lld", njobs, F.Tg.count);
    launch_perm_init(h->stream, njobs, F.perm, b);
    h->launches++;
    // The matrices alternate between the D slots and the ping-pong buffer: each
    // panel's update reads the current buffer through the panel's row exchanges
    // and writes the other one.
    //
    // Look-ahead (FP32 tensor-core path, not while profiling): the update of
    // panel p is split into the next panel's columns (on the main stream, so
    // panel p+1 can start right away) and all other columns (on a second
    // stream, overlapping panel p+1).  The panel buffers, rowsrc and their slot
    // lists alternate by panel parity, so panel p+1 never overwrites what the
    // wide update of panel p reads; the wide update of panel p must finish before
    // the narrow update of panel p+1 writes into the buffer it reads.
    const bool overlap = sizeof(T) == 4 && F.tc_ok && !h->prof_on && h->stream2;
    const int npan = ceil_div(b, nb);
    int cur = P_D, alt = P_TG;
    const int* cur_slots = d_slots;
    const int* alt_slots = d_iota;
    bool wide_pending = false;
    for (int p = 0; p < npan; ++p) {
        const int c0 = p * nb, w = std::min(nb, b - c0);
        const int par = overlap ? (p & 1) : 0;
        Pool<T> GPp = F.GP, RPp = F.RP;
        GPp.base += (size_t)par * h->max_ne * F.GP.slot_elems();
        RPp.base += (size_t)par * h->max_ne * F.RP.slot_elems();
        int* rs = F.rowsrc + (size_t)par * h->max_ne * b;
        const int* pslots = F.gj_slots + par * h->max_ne;   // GP/RP slots of this parity
        int ev = prof_begin(h);
        int e = launch_gj_panel<T>(h->stream, nb, njobs, pool_of(F, cur), cur_slots, GPp, F.perm, rs, c0, h->derr,
                                   GjFuse{}, gj_cluster(h, njobs), h->gj_form, wait_limit(h));
        h->launches++;
        if (e) return set_err(h, FDFD_ECUDA, "gj_panel launch failed: %s", cudaGetErrorString((cudaError_t)e));
        // Rᵀ reads the pivot rows in full: the previous panel's wide update, which ran
        // concurrently with this panel's column steps, must have finished
        if (wide_pending) {
            CK(cudaStreamWaitEvent(h->stream, h->ev_wide, 0));
            wide_pending = false;
        }
        e = launch_gj_rt<T>(h->stream, nb, njobs, pool_of(F, cur), cur_slots, RPp, rs, c0, nb);
        prof_end(h, ev, FDFD_PROF_GJ_PANEL, 0.0);
        h->launches++;
        if (e) return set_err(h, FDFD_ECUDA, "gj_rt launch failed: %s", cudaGetErrorString((cudaError_t)e));
        const double ubytes = 4.0 * sizeof(T) * (double)b * b * njobs;
        if (overlap && p + 1 < npan) {
            const int c1 = c0 + nb, w1 = std::min(nb, b - c1);
            CK(cudaEventRecord(h->ev_panel, h->stream));
            RET(gemm<T>(h, P_GP, P_RP, alt, pslots, pslots, alt_slots, nullptr, 0, njobs, b, w1, nb, (T)1, 1,
                        c0, w, cur, cur_slots, rs, FDFD_PROF_GJ_UPDATE, ubytes * w1 / b, h->stream, c1));
            CK(cudaStreamWaitEvent(h->stream2, h->ev_panel, 0));
            RET(gemm<T>(h, P_GP, P_RP, alt, pslots, pslots, alt_slots, nullptr, 0, njobs, b, b, nb, (T)1, 1,
                        c0, w, cur, cur_slots, rs, FDFD_PROF_GJ_UPDATE, ubytes * (b - w1) / b, h->stream2, 0, c1,
                        w1));
            CK(cudaEventRecord(h->ev_wide, h->stream2));
            wide_pending = true;
        } else {
            RET(gemm<T>(h, P_GP, P_RP, alt, pslots, pslots, alt_slots, nullptr, 0, njobs, b, b, nb, (T)1, 1,
                        c0, w, cur, cur_slots, rs, FDFD_PROF_GJ_UPDATE, ubytes));
        }
        std::swap(cur, alt);
        std::swap(cur_slots, alt_slots);
    }
    if (wide_pending) CK(cudaStreamWaitEvent(h->stream, h->ev_wide, 0));
    launch_gj_unpermute<T>(h->stream, njobs, pool_of(F, cur), cur_slots, F.D, d_slots, F.perm);
    h->launches++;
    return check_launch(h, "gj_unpermute");
}

// Fused super-panels (FP32 tensor-core path, FDFD_GJ_FUSED_K = 64 or 128; off by
// default: on the 800 x 480 workload K = 64 saved 0.7 ms of the 26.7 ms factor but
// its rounding took FGMRES from 8 to 9 iterations, +1.3 ms).  The S = K / nb panels of
// a super-panel share one rank-(S·nb) update of the matrix, so each matrix is
// read and written once per super-panel instead of once per panel.  With M0 the
// super-panel's input matrix, P the composed row exchanges of its panels so far
// and J their columns, the matrix after them is
//     M = mask_J(P M0) + P·Ĝ·R,
// where Ĝ holds the panels' G columns in M0's row order (each panel writes its
// rows there, so no earlier column is ever permuted; its pivot rows' earlier
// columns are zeroed) and R their pivot rows.  A later panel's pivot rows are
// formed from M0 and the earlier G and R (gj_rs), the next panel's columns by a
// narrow product (K = panels so far × nb), and the rest of the matrix by one
// wide product at the end; both GEMMs scatter the rows of Ĝ·R to their logical
// places (row_dst = P's inverse) and read β from M0 directly.  Look-ahead (not
// while profiling): the wide product runs on the second stream, overlapping the
// next super-panel's first panel; the panel buffers and maps alternate by
// super-panel parity.
int gj_invert_fused(fdfd_handle* h, const int* d_slots, const int* d_iota, int njobs) {
    FactorStore<float>& F = h->f32;
    const int b = h->map.b;
    const int nb = panel_nb<float>(b);
    const int S = F.GP.cols / nb;
    if (njobs > F.Tg.count) return set_err(h, FDFD_EINVAL, "Gauss-Jordan batch %d exceeds %lld", njobs, F.Tg.count);
    launch_perm_init(h->stream, njobs, F.perm, b);
    h->launches++;
    const bool overlap = !h->prof_on && h->stream2;
    const int npan = ceil_div(b, nb), nsup = ceil_div(npan, S);
    int cur = P_D, alt = P_TG;
    const int* cur_slots = d_slots;
    const int* alt_slots = d_iota;
    bool wide_pending = false;
    const double ubytes = 4.0 * sizeof(float) * (double)b * b * njobs;   // each matrix read and written once
    for (int q = 0; q < nsup; ++q) {
        const int par = overlap ? (q & 1) : 0;
        Pool<float> GPq = F.GP, RPq = F.RP;
        GPq.base += (size_t)par * h->max_ne * F.GP.slot_elems();
        RPq.base += (size_t)par * h->max_ne * F.RP.slot_elems();
        int* tot = F.rowsrc + (size_t)par * h->max_ne * b;
        int* inv = F.inv + (size_t)par * h->max_ne * b;
        const int* pslots = F.gj_slots + par * h->max_ne;   // GP/RP slots of this parity
        const int p0 = q * S, pans = std::min(S, npan - p0), c0q = p0 * nb;
        for (int si = 0; si < pans; ++si) {
            const int c0 = (p0 + si) * nb, kp = si * nb, K = kp + nb;
            GjFuse fz;
            fz.fused = 1;
            fz.gcol0 = kp;
            fz.tot_in = si == 0 ? nullptr : tot;
            fz.inv_out = inv;
            fz.gsub = F.gsub;
            // the panel reads its columns of the matrix after the previous panels: the
            // super-panel's input for the first, the narrow product's output after that
            int ev = prof_begin(h);
            int e = launch_gj_panel<float>(h->stream, nb, njobs, pool_of(F, si == 0 ? cur : alt),
                                           si == 0 ? cur_slots : alt_slots, GPq, F.perm, tot, c0, h->derr, fz, 0, 0,
                                           wait_limit(h));
            h->launches++;
            if (e) return set_err(h, FDFD_ECUDA, "gj_panel launch failed: %s", cudaGetErrorString((cudaError_t)e));
            if (si == 0) {
                // pivot rows in full: the previous super-panel's wide product must have finished
                if (wide_pending) {
                    CK(cudaStreamWaitEvent(h->stream, h->ev_wide, 0));
                    wide_pending = false;
                }
                e = launch_gj_rt<float>(h->stream, nb, njobs, pool_of(F, cur), cur_slots, RPq, tot, c0, nb);
            } else {
                e = launch_gj_rs<float>(h->stream, nb, njobs, pool_of(F, cur), cur_slots, RPq, tot, F.gsub, kp, c0,
                                        c0q);
            }
            prof_end(h, ev, FDFD_PROF_GJ_PANEL, 0.0);
            h->launches++;
            if (e) return set_err(h, FDFD_ECUDA, "gj pivot-row launch failed: %s", cudaGetErrorString((cudaError_t)e));
            const bool last = si == pans - 1;
            const int c1 = c0 + nb, w1 = std::min(nb, b - c1);
            const bool has_next = c1 < b;
            if (has_next && (!last || overlap)) {
                // the next panel's columns, on the main stream
                RET(gemm<float>(h, P_GP, P_RP, alt, pslots, pslots, alt_slots, nullptr, 0, njobs, b, w1, K, 1.0f, 1,
                                c0q, K, cur, cur_slots, nullptr, FDFD_PROF_GJ_UPDATE, ubytes * w1 / b, h->stream, c1,
                                0, 0, 0, inv));
            }
            if (last) {
                if (has_next && overlap) {
                    // every other column on the second stream, overlapping the next panel
                    CK(cudaEventRecord(h->ev_panel, h->stream));
                    CK(cudaStreamWaitEvent(h->stream2, h->ev_panel, 0));
                    RET(gemm<float>(h, P_GP, P_RP, alt, pslots, pslots, alt_slots, nullptr, 0, njobs, b, b, K, 1.0f, 1,
                                    c0q, K, cur, cur_slots, nullptr, FDFD_PROF_GJ_UPDATE, ubytes * (b - w1) / b,
                                    h->stream2, 0, c1, w1, 0, inv));
                    CK(cudaEventRecord(h->ev_wide, h->stream2));
                    wide_pending = true;
                } else {
                    RET(gemm<float>(h, P_GP, P_RP, alt, pslots, pslots, alt_slots, nullptr, 0, njobs, b, b, K, 1.0f, 1,
                                    c0q, K, cur, cur_slots, nullptr, FDFD_PROF_GJ_UPDATE, ubytes, h->stream, 0, 0, 0,
                                    0, inv));
                }
            }
        }
        std::swap(cur, alt);
        std::swap(cur_slots, alt_slots);
    }
    if (wide_pending) CK(cudaStreamWaitEvent(h->stream, h->ev_wide, 0));
    launch_gj_unpermute<float>(h->stream, njobs, pool_of(F, cur), cur_slots, F.D, d_slots, F.perm);
    h->launches++;
    return check_launch(h, "gj_unpermute");
}

// ---------------------------------------------------------------------------
// Factorization
// ---------------------------------------------------------------------------
template <typename T> int factor_impl(fdfd_handle* h) {
    RET(alloc_factor<T>(h));
    FactorStore<T>& F = store<T>(h);
    const int b = h->map.b;
    const int E = (int)h->steps.size();
    double flops = 0;
    const double b3 = (double)b * b * b;
    for (int e = 1; e <= E; ++e) {
        const StepJobs& S = h->sj[e];
        const int ne = S.ne;
        if (e == 1) {
            if (h->level1_gj) {
                launch_build_tridiag<T>(h->stream, ne, h->map, h->st, h->scale, F.D, J<int>(h, S.elim));
                h->launches++;
                RET(check_launch(h, "build_tridiag"));
                RET(gj_invert<T>(h, J<int>(h, S.elim), J<int>(h, S.iota), ne));
                flops += 8.0 * b3 * ne;
            } else {
                int ev = prof_begin(h);
                launch_tri_inverse<T>(h->stream, ne, h->map, h->st, h->scale, F.D, J<int>(h, S.elim), F.trifac,
                                      F.tripiv, h->derr);
                prof_end(h, ev, FDFD_PROF_LEVEL1, 2.0 * sizeof(T) * b * b * ne);
                h->launches += 2;
                RET(check_launch(h, "tri_inverse"));
            }
            // bytes: two inverses read (re, im), D written (re, im), both couplings written (all planes)
            int ev1 = prof_begin(h);
            launch_level1_combine<T>(h->stream, S.nl1, h->map, h->st, h->scale, F.D, F.C, J<L1Job>(h, S.l1),
                                     F.sttab);
            prof_end(h, ev1, FDFD_PROF_LEVEL1, (6.0 + 2.0 * F.C.planes) * sizeof(T) * b * b * S.nl1);
            h->launches += 2;
            RET(check_launch(h, "level1_combine"));
        } else {
            RET(gj_invert<T>(h, J<int>(h, S.elim), J<int>(h, S.iota), ne));
            // Xᵀ = [Lᵀ; Uᵀ] Gᵀ
            RET(gemm<T>(h, P_C, P_D, P_X, J<int>(h, S.xt_a), J<int>(h, S.xt_b), J<int>(h, S.xt_c), nullptr, 0,
                        2 * ne, b, b, b, (T)1, 0, 0, 0));
            // D_p -= U_p X_L ; D_q -= L_q X_R
            RET(gemm<T>(h, P_C, P_X, P_D, J<int>(h, S.dp_a), J<int>(h, S.dp_b), J<int>(h, S.dp_c), nullptr, 0,
                        ne, b, b, b, (T)-1, 1, 0, 0));
            RET(gemm<T>(h, P_C, P_X, P_D, J<int>(h, S.dq_a), J<int>(h, S.dq_b), J<int>(h, S.dq_c), nullptr, 0,
                        ne, b, b, b, (T)-1, 1, 0, 0));
            // new couplings U_p' = -U_p X_R, L_q' = -L_q X_L (storage form per node)
            RET(gemm<T>(h, P_C, P_X, P_C, J<int>(h, S.cp_a), J<int>(h, S.cp_b), J<int>(h, S.cp_c),
                        J<int>(h, S.cp_t), 0, S.ncp, b, b, b, (T)-1, 0, 0, 0));
            if (S.ncpy) {
                launch_mcopy<T>(h->stream, S.ncpy, F.C, F.C, J<int3>(h, S.cpy));
                h->launches++;
                RET(check_launch(h, "mcopy"));
            }
            flops += 8.0 * b3 * ne * 7;   // inversion + 2 (Xᵀ) + 4 (updates)
        }
        RET(ckpt_offload<T>(h, e));
    }
    // final pair (a, c)
    launch_madd<T>(h->stream, 2, F.C, J<int3>(h, h->fin_mrg));
    h->launches++;
    RET(check_launch(h, "madd"));
    RET(gj_invert<T>(h, J<int>(h, h->fin_c_slot), J<int>(h, h->fin_iota), 1));
    RET(gemm<T>(h, P_C, P_D, P_X, J<int>(h, h->fin_xt_a), J<int>(h, h->fin_xt_b), J<int>(h, h->fin_xt_c), nullptr,
                0, 1, b, b, b, (T)1, 0, 0, 0));
    RET(gemm<T>(h, P_C, P_X, P_D, J<int>(h, h->fin_da_a), J<int>(h, h->fin_da_b), J<int>(h, h->fin_da_c), nullptr,
                0, 1, b, b, b, (T)-1, 1, 0, 0));
    RET(gj_invert<T>(h, J<int>(h, h->fin_a_slot), J<int>(h, h->fin_iota), 1));
    flops += 8.0 * b3 * 4;
    h->last_factor_flops = flops;
    return FDFD_OK;
}

// ---------------------------------------------------------------------------
// Solve sweeps: F.rv holds the (scaled) right-hand sides in node layout on
// entry; F.xv holds the solution on exit.
// ---------------------------------------------------------------------------
// nblk: factor blocks the njobs jobs reference (a job's second block may be absent)
template <typename T> int gemv(fdfd_handle* h, int tr, int p1, int p2, const T* V1, const T* V2, const T* Y0, T* Y,
                               const int4* jobs, const int2* yjobs, int njobs, int nblk, int nrhs, T alpha) {
    if (njobs == 0) return FDFD_OK;
    FactorStore<T>& F = store<T>(h);
    const int b = h->map.b;
    const int rmax = gemv_max_rhs<T>(b);
    for (int r0 = 0; r0 < nrhs; r0 += rmax) {
        GemvArgs<T> g;
        g.P1 = pool_of(F, p1); g.P2 = pool_of(F, p2);
        g.V1 = V1; g.V2 = V2; g.Y0 = Y0; g.Y = Y;
        g.jobs = jobs; g.yjobs = yjobs;
        g.b = b; g.ld = h->map.ld; g.nrhs = std::min(rmax, nrhs - r0); g.rtot = nrhs; g.r0 = r0;
        g.alpha = alpha;
        g.nsm = h->num_sms;
        g.nmat = nblk > njobs ? 2 : 1;
        g.err = h->derr;
        g.shape = h->force_shape;
        if (!g.shape) {
            auto it = h->tune_gemv.find(std::make_tuple(tr, njobs, g.nmat, g.nrhs));
            if (it != h->tune_gemv.end()) g.shape = it->second;
        }
        if (!tr && g.shape == 0 && !h->gemv_bulk) g.shape = GEMV_SHAPE_REGISTER_RULE;
        int ev = prof_begin(h);
        int e = launch_gemv<T>(h->stream, tr, njobs, g);
        // algorithmic bytes: every referenced block (re + im planes) read once; per job and
        // right-hand side the input vectors of its blocks, y0 and y (each b complex values)
        prof_end(h, ev, FDFD_PROF_SWEEP,
                 (double)nblk * 2.0 * b * b * sizeof(T) + (double)(nblk + 2 * njobs) * g.nrhs * 2.0 * b * sizeof(T));
        h->launches++;
        if (e) return set_err(h, FDFD_ECUDA, "gemv launch failed: %s", cudaGetErrorString((cudaError_t)e));
    }
    return FDFD_OK;
}

// First-step products through the tridiagonal factors (launch_tri_apply):
// Y = Y0 + alpha·D_k⁻¹ V for the step's eliminated nodes
template <typename T> int tri_apply(fdfd_handle* h, const T* V, const T* Y0, T* Y, int nrhs, T alpha) {
    FactorStore<T>& F = store<T>(h);
    const StepJobs& S = h->sj[1];
    const int b = h->map.b;
    int ev = prof_begin(h);
    int e = launch_tri_apply<T>(h->stream, b, h->map.ld, S.ne, nrhs, J<int>(h, S.elim), F.trifac, F.tripiv, V, Y0, Y,
                                alpha);
    // factor workspace (8b complex + b pivots) per node; per node and right-hand side V read,
    // Y written (and Y0 read) once
    prof_end(h, ev, FDFD_PROF_SWEEP,
             (double)S.ne * (8.0 * b * sizeof(cplx<T>) + 4.0 * b + (2.0 + (Y0 ? 1 : 0)) * nrhs * 2.0 * b * sizeof(T)));
    h->launches++;
    if (e) return set_err(h, FDFD_ECUDA, "tri_apply launch failed: %s", cudaGetErrorString((cudaError_t)e));
    return FDFD_OK;
}

template <typename T> int sweep_impl(fdfd_handle* h, int nrhs) {
    FactorStore<T>& F = store<T>(h);
    const int E = (int)h->steps.size();
    const bool tri1 = F.trifac && !h->level1_gj && h->tri_sweep;
    // forward
    for (int e = 1; e <= E; ++e) {
        const StepJobs& S = h->sj[e];
        if (e == 1 && tri1) {
            RET(tri_apply<T>(h, F.rv, nullptr, F.xv, nrhs, (T)1));
        } else {
            RET(gemv<T>(h, 0, P_D, P_D, F.rv, F.rv, nullptr, F.xv, J<int4>(h, S.fwd1), J<int2>(h, S.fwd1y), S.ne, S.ne,
                        nrhs, (T)1));
        }
        if (e == 1) {
            if (S.nf2) {
                launch_diag_sweep<T>(h->stream, S.nf2, h->map, F.sttab, nrhs, J<int4>(h, S.dswf), 0,
                                     (const T*)F.xv, F.rv);
                h->launches++;
            }
        } else {
            RET(ckpt_reload_ring<T>(h, e - 1));
            RET(gemv<T>(h, 0, P_C, P_C, F.xv, F.xv, F.rv, F.rv, J<int4>(h, S.f2), J<int2>(h, S.f2y), S.nf2, S.nf2b, nrhs,
                        (T)-1));
        }
    }
    // final pair
    RET(gemv<T>(h, 0, P_D, P_D, F.rv, F.rv, nullptr, F.xv, J<int4>(h, h->fin_g1), J<int2>(h, h->fin_g1y), 1, 1, nrhs,
                (T)1));
    RET(gemv<T>(h, 0, P_C, P_C, F.xv, F.xv, F.rv, F.rv, J<int4>(h, h->fin_ra), J<int2>(h, h->fin_ray), 1, 1, nrhs,
                (T)-1));
    RET(gemv<T>(h, 0, P_D, P_D, F.rv, F.rv, nullptr, F.xv, J<int4>(h, h->fin_g0), J<int2>(h, h->fin_g0y), 1, 1, nrhs,
                (T)1));
    RET(gemv<T>(h, 1, P_X, P_X, F.xv, F.xv, F.xv, F.xv, J<int4>(h, h->fin_bx), J<int2>(h, h->fin_bxy), 1, 1, nrhs,
                (T)-1));
    // backward
    for (int e = E; e >= 1; --e) {
        const StepJobs& S = h->sj[e];
        if (e == 1) {
            launch_diag_sweep<T>(h->stream, S.ne, h->map, F.sttab, nrhs, J<int4>(h, S.dswb), 1,
                                 (const T*)F.xv, F.wv);
            h->launches++;
            if (tri1) {
                RET(tri_apply<T>(h, F.wv, F.xv, F.xv, nrhs, (T)-1));
            } else {
                RET(gemv<T>(h, 0, P_D, P_D, F.wv, F.wv, F.xv, F.xv, J<int4>(h, S.bwd1), J<int2>(h, S.bwd1y), S.ne, S.ne,
                            nrhs, (T)-1));
            }
        } else {
            RET(ckpt_reload_x<T>(h, e));
            RET(gemv<T>(h, 1, P_X, P_X, F.xv, F.xv, F.xv, F.xv, J<int4>(h, S.bw), J<int2>(h, S.bwy), S.ne, 2 * S.ne, nrhs,
                        (T)-1));
        }
    }
    return check_launch(h, "sweep");
}

// the sweep through this handle's graph for (T, nrhs, vector buffer, cfg_gen): captured on the first
// use of that key (without running), then launched; plain launches while profiling, in checkpoint
// mode (host copies), with graphs off, or when the capture fails
template <typename T> int sweep_graph(fdfd_handle* h, int nrhs) {
    const int ti = sizeof(T) == 4 ? 0 : 1;
    FactorStore<T>& F = store<T>(h);
    if (!h->graph_factor || h->prof_on || h->ckpt || h->ckpt_mode == 1) return sweep_impl<T>(h, nrhs);
    if (!(h->sg_exec[ti] && h->sg_nrhs[ti] == nrhs && h->sg_rv[ti] == (const void*)F.rv &&
          h->sg_gen[ti] == h->cfg_gen)) {
        if (h->sg_exec[ti]) { cudaGraphExecDestroy(h->sg_exec[ti]); h->sg_exec[ti] = nullptr; }
        if (h->sg_graph[ti]) { cudaGraphDestroy(h->sg_graph[ti]); h->sg_graph[ti] = nullptr; }
        if (cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            cudaGetLastError();
            return sweep_impl<T>(h, nrhs);
        }
        const long long l0 = h->launches;
        const int rc = sweep_impl<T>(h, nrhs);
        cudaGraph_t g = nullptr;
        const cudaError_t ee = cudaStreamEndCapture(h->stream, &g);
        const long long kernels = h->launches - l0;
        h->launches = l0;
        if (rc != FDFD_OK || ee != cudaSuccess || !g || cudaGraphInstantiate(&h->sg_exec[ti], g, 0) != cudaSuccess) {
            cudaGetLastError();
            if (g) cudaGraphDestroy(g);
            h->sg_exec[ti] = nullptr;
            h->err.clear();
            return sweep_impl<T>(h, nrhs);
        }
        h->sg_graph[ti] = g;
        h->sg_nrhs[ti] = nrhs;
        h->sg_rv[ti] = (const void*)F.rv;
        h->sg_gen[ti] = h->cfg_gen;
        h->sg_kernels[ti] = kernels;
    }
    if (cudaGraphLaunch(h->sg_exec[ti], h->stream) != cudaSuccess) {
        cudaGetLastError();
        return set_err(h, FDFD_ECUDA, "cudaGraphLaunch of the sweep failed");
    }
    h->launches += h->sg_kernels[ti];
    return FDFD_OK;
}

// preconditioner: out = (scale·A)⁻¹ (scale·in) = A⁻¹ in  (FP64 natural layout, nrhs vectors)
template <typename T> int precond_impl(fdfd_handle* h, const cplx<double>* in, cplx<double>* out, int nrhs) {
    RET(alloc_vectors<T>(h, nrhs));
    FactorStore<T>& F = store<T>(h);
    long long N = (long long)h->Nx * h->Ny;
    dim3 grid(ceil_div(N, 256), nrhs);
    launch_to_nodes<T>(grid, h->stream, h->map, nrhs, in, h->scale, F.rv);
    h->launches++;
    RET(sweep_graph<T>(h, nrhs));
    launch_from_nodes<T>(grid, h->stream, h->map, nrhs, (const T*)F.xv, 1.0, 0, out);
    h->launches++;
    return check_launch(h, "precond");
}

int precond(fdfd_handle* h, const cplx<double>* in, cplx<double>* out, int nrhs);

// modulated device: block-diagonal preconditioner, sideband n solved by its
// own factor on its own stream (the K sweeps run concurrently)
int precond_mf(fdfd_handle* h, const cplx<double>* in, cplx<double>* out) {
    MfState& M = *h->mf;
    const long long N = (long long)h->Nx * h->Ny;
    CK(cudaEventRecord(M.ev_in, h->stream));
    for (int n = 0; n < M.K; ++n) {
        fdfd_handle* s = M.sub[n];
        CK(cudaStreamWaitEvent(s->stream, M.ev_in, 0));
        const long long l0 = s->launches;
        int rc = precond(s, in + (size_t)n * N, out + (size_t)n * N, 1);
        h->launches += s->launches - l0;
        if (rc != FDFD_OK) return set_err(h, rc, "sideband %d: %s", n, s->err.c_str());
        CK(cudaEventRecord(M.ev_out[n], s->stream));
    }
    for (int n = 0; n < M.K; ++n) CK(cudaStreamWaitEvent(h->stream, M.ev_out[n], 0));
    return FDFD_OK;
}

int precond(fdfd_handle* h, const cplx<double>* in, cplx<double>* out, int nrhs) {
    if (h->mf) return precond_mf(h, in, out);
    if (h->nl_mode == 2) {
        // Newton's stacked system: blockdiag(A⁻¹, conj(A)⁻¹), conj(A)⁻¹v = conj(A⁻¹ conj(v)),
        // both halves through one two-right-hand-side sweep
        const long long N = (long long)h->Nx * h->Ny;
        CK(cudaMemcpyAsync(h->nl_tmp, in, N * sizeof(cplx<double>), cudaMemcpyDeviceToDevice, h->stream));
        LAUNCH(vconj_kernel, ceil_div(N, 256), 256, 0, N, in + N, h->nl_tmp + N);
        int rc = h->fact_prec == FDFD_PREC_FP64 ? precond_impl<double>(h, h->nl_tmp, out, 2)
                                                : precond_impl<float>(h, h->nl_tmp, out, 2);
        if (rc != FDFD_OK) return rc;
        LAUNCH(vconj_kernel, ceil_div(N, 256), 256, 0, N, out + N, out + N);
        return check_launch(h, "precond");
    }
    return h->fact_prec == FDFD_PREC_FP64 ? precond_impl<double>(h, in, out, nrhs)
                                          : precond_impl<float>(h, in, out, nrhs);
}

// ---------------------------------------------------------------------------
// Reductions and Krylov refinement (FP64, natural layout)
// ---------------------------------------------------------------------------
int ensure_part(fdfd_handle* h, size_t doubles) {
    if (h->part_cap >= doubles) return FDFD_OK;
    dev_free(h, h->part);
    h->part = nullptr;
    h->part_cap = 0;
    RET(dev_alloc(h, (void**)&h->part, doubles * sizeof(double)));
    h->part_cap = doubles;
    return FDFD_OK;
}
int ensure_red(fdfd_handle* h, size_t doubles) {
    if (h->red_cap >= doubles) return FDFD_OK;
    dev_free(h, h->red);
    h->red = nullptr;
    h->red_cap = 0;
    RET(dev_alloc(h, (void**)&h->red, doubles * sizeof(double)));
    h->red_cap = doubles;
    return FDFD_OK;
}

// r = b - A x (b may be null: r = A x); optionally ||r||², ||b||² per rhs to host
int residual_mf(fdfd_handle* h, const cplx<double>* x, const cplx<double>* b, cplx<double>* r,
                std::vector<double>* norms) {
    const MfState& M = *h->mf;
    const long long N = (long long)h->Nx * h->Ny;
    const int nb = ceil_div(N, 256);
    RET(ensure_part(h, (size_t)M.K * nb * 2));
    RET(ensure_red(h, (size_t)M.K * 2));
    MfResidualArgs a;
    a.Nx = h->Nx; a.Ny = h->Ny; a.K = M.K;
    for (int n = 0; n < M.K; ++n) {
        a.st[n] = M.sub[n]->st;
        a.half_w2eps0[n] = 0.5 * M.wn[n] * M.wn[n] * (kEPS0 * h->L0);
    }
    int ev = prof_begin(h);
    LAUNCH(residual_mf_kernel, dim3(nb, M.K), 256, 0, a, M.deps, x, b, r, norms ? h->part : nullptr);
    prof_end(h, ev, FDFD_PROF_RESIDUAL, (double)N * M.K * (96.0 + 16.0 * (b ? 3 : 2)));
    if (norms) {
        LAUNCH(reduce_partials_kernel, M.K, 256, 0, h->part, nb, 2, h->red);
        std::vector<double> per(2 * M.K);
        CK(cudaMemcpyAsync(per.data(), h->red, per.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        norms->assign(2, 0.0);
        for (int n = 0; n < M.K; ++n) {
            (*norms)[0] += per[2 * n];
            (*norms)[1] += per[2 * n + 1];
        }
    }
    return check_launch(h, "residual");
}

// χ³ operators (nl_mode 1: A + diag d1; 2: Newton's stacked system), nrhs = 1
int residual_nl(fdfd_handle* h, const cplx<double>* x, const cplx<double>* b, cplx<double>* r,
                std::vector<double>* norms) {
    const long long N = (long long)h->Nx * h->Ny;
    const int nb = ceil_div(N, 256), halves = h->nl_mode == 2 ? 2 : 1;
    RET(ensure_part(h, (size_t)halves * nb * 2));
    RET(ensure_red(h, (size_t)halves * 2));
    int ev = prof_begin(h);
    LAUNCH(residual_nl_kernel, dim3(nb, halves), 256, 0, h->Nx, h->Ny, h->nl_mode, h->st, h->nl_d1, h->nl_d2, x, b,
           r, norms ? h->part : nullptr);
    prof_end(h, ev, FDFD_PROF_RESIDUAL, (double)N * halves * (112.0 + 16.0 * (b ? 3 : 2)));
    if (norms) {
        LAUNCH(reduce_partials_kernel, halves, 256, 0, h->part, nb, 2, h->red);
        std::vector<double> per(2 * halves);
        CK(cudaMemcpyAsync(per.data(), h->red, per.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        norms->assign(2, 0.0);
        for (int i = 0; i < halves; ++i) {
            (*norms)[0] += per[2 * i];
            (*norms)[1] += per[2 * i + 1];
        }
    }
    return check_launch(h, "residual");
}

int residual(fdfd_handle* h, const cplx<double>* x, const cplx<double>* b, cplx<double>* r, int nrhs,
             std::vector<double>* norms) {
    if (h->mf) return residual_mf(h, x, b, r, norms);   // nrhs = 1
    if (h->nl_mode) return residual_nl(h, x, b, r, norms);   // nrhs = 1
    long long N = (long long)h->Nx * h->Ny;
    int nb = ceil_div(N, 256);
    RET(ensure_part(h, (size_t)nrhs * nb * 2));
    RET(ensure_red(h, (size_t)nrhs * 2));
    int ev = prof_begin(h);
    LAUNCH(residual_kernel, dim3(nb, nrhs), 256, 0, h->Nx, h->Ny, nrhs, h->st, x, b, r, norms ? h->part : nullptr);
    // algorithmic bytes per unknown: 5 stencil coefficients (80 B), x, r and b (16 B each)
    prof_end(h, ev, FDFD_PROF_RESIDUAL, (double)N * nrhs * (80.0 + 16.0 * (b ? 3 : 2)));
    if (norms) {
        LAUNCH(reduce_partials_kernel, dim3(nrhs, 2), 256, 0, h->part, nb, 2, h->red);
        norms->resize(2 * nrhs);
        CK(cudaMemcpyAsync(norms->data(), h->red, 2 * nrhs * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
    }
    return check_launch(h, "residual");
}

// out[rhs*nvec + j] = V_jᴴ w  (complex)
int dots(fdfd_handle* h, const cplx<double>* V, long long vstride, int nvec, const cplx<double>* w, int nrhs,
         std::vector<zd>& out) {
    long long N = vlen(h);
    const int nb = 4 * h->num_sms;   // four blocks per SM: enough loads in flight for HBM
    RET(ensure_part(h, (size_t)nrhs * nb * 2 * nvec));
    RET(ensure_red(h, (size_t)nrhs * 2 * nvec));
    LAUNCH(vdots_kernel, dim3(nb, nrhs), 256, 0, N, nvec, V, vstride, w, h->part);
    LAUNCH(reduce_partials_kernel, dim3(nrhs, 2 * nvec), 256, 0, h->part, nb, 2 * nvec, h->red);
    std::vector<double> tmp(2 * nvec * nrhs);
    CK(cudaMemcpyAsync(tmp.data(), h->red, tmp.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    out.resize(nvec * nrhs);
    for (int i = 0; i < nvec * nrhs; ++i) out[i] = zd(tmp[2 * i], tmp[2 * i + 1]);
    return check_launch(h, "dots");
}

// y[rhs] += sign Σ_j c[rhs][j] V_j[rhs]
int combine(fdfd_handle* h, const cplx<double>* V, long long vstride, int nvec, const std::vector<zd>& c, int nrhs,
            double sign, cplx<double>* y) {
    long long N = vlen(h);
    CK(cudaMemcpyAsync(h->kc, c.data(), c.size() * sizeof(zd), cudaMemcpyHostToDevice, h->stream));
    LAUNCH(vcombine_kernel, dim3(ceil_div(N, 256), nrhs), 256, 0, N, nvec, V, vstride, h->kc, nvec, sign, y);
    return check_launch(h, "combine");
}

// One Arnoldi orthogonalisation on the device: two classical Gram-Schmidt
// passes of w against V_0..V_{nvec-1}, then w /= ‖w‖:
//   h1 = Vᴴw, w -= V h1, h2 = Vᴴw, w -= V h2, nn = ‖w‖², w /= √nn.
// The coefficients stay on the device between the passes, and one read-back
// returns h1, h2 (out[rhs*nvec + j]) and nn (per rhs) for the Hessenberg column.
int arnoldi_orth(fdfd_handle* h, const cplx<double>* V, long long vstride, int nvec, cplx<double>* w, int nrhs,
                 std::vector<zd>& h1, std::vector<zd>& h2, std::vector<double>& nn) {
    long long N = vlen(h);
    const int nb = 4 * h->num_sms;
    const size_t nc = (size_t)nrhs * 2 * nvec;   // doubles per coefficient set
    RET(ensure_part(h, (size_t)nrhs * nb * 2 * nvec));
    RET(ensure_red(h, 2 * nc + 2 * (size_t)nrhs));
    double* r1 = h->red;
    double* r2 = h->red + nc;
    double* r3 = h->red + 2 * nc;
    LAUNCH(vdots_kernel, dim3(nb, nrhs), 256, 0, N, nvec, V, vstride, w, h->part);
    LAUNCH(reduce_partials_kernel, dim3(nrhs, 2 * nvec), 256, 0, h->part, nb, 2 * nvec, r1);
    const dim3 ge(ceil_div(N, 256), nrhs);
    LAUNCH(vcombine_kernel, ge, 256, 0, N, nvec, V, vstride, reinterpret_cast<const cplx<double>*>(r1), nvec,
           -1.0, w);
    LAUNCH(vdots_kernel, dim3(nb, nrhs), 256, 0, N, nvec, V, vstride, w, h->part);
    LAUNCH(reduce_partials_kernel, dim3(nrhs, 2 * nvec), 256, 0, h->part, nb, 2 * nvec, r2);
    LAUNCH(vcombine_kernel, ge, 256, 0, N, nvec, V, vstride, reinterpret_cast<const cplx<double>*>(r2), nvec,
           -1.0, w);
    LAUNCH(vdots_kernel, dim3(nb, nrhs), 256, 0, N, 1, w, 0, w, h->part);
    LAUNCH(reduce_partials_kernel, dim3(nrhs, 2), 256, 0, h->part, nb, 2, r3);
    LAUNCH(vnormalize_kernel, dim3(ceil_div(N, 256), nrhs), 256, 0, N, w, r3, w);
    std::vector<double> tmp(2 * nc + 2 * (size_t)nrhs);
    CK(cudaMemcpyAsync(tmp.data(), h->red, tmp.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    const size_t nv = (size_t)nrhs * nvec;
    h1.resize(nv);
    h2.resize(nv);
    nn.resize(nrhs);
    for (size_t i = 0; i < nv; ++i) {
        h1[i] = zd(tmp[2 * i], tmp[2 * i + 1]);
        h2[i] = zd(tmp[nc + 2 * i], tmp[nc + 2 * i + 1]);
    }
    for (int r = 0; r < nrhs; ++r) nn[r] = tmp[2 * nc + 2 * r];
    return check_launch(h, "arnoldi");
}

int scale_vec(fdfd_handle* h, const cplx<double>* x, const std::vector<zd>& s, int nrhs, cplx<double>* y) {
    long long N = vlen(h);
    CK(cudaMemcpyAsync(h->kc, s.data(), nrhs * sizeof(zd), cudaMemcpyHostToDevice, h->stream));
    LAUNCH(vscale_kernel, dim3(ceil_div(N, 256), nrhs), 256, 0, N, x, h->kc, y);
    return check_launch(h, "scale");
}

// FGMRES basis length: the handle's setting, else the iteration budget up to
// 80 solves while the 2m+1 basis vectors fit in 8 GiB, at least 20.  Slowly
// converging FP32-preconditioned problems (strong resonances at 1024²) stall
// under restarts every 20 solves and converge unrestarted within ~60.
int restart_len(const fdfd_handle* h, int nrhs) {
    if (h->restart > 0) return h->restart;
    const double vec = (double)vlen(h) * nrhs * sizeof(cplx<double>);
    const int cap = (int)((8.0 * (1ull << 30) / vec - 1) / 2);
    return std::max(20, std::min(std::min(h->max_iter, 80), cap));
}

int ensure_krylov(fdfd_handle* h, int nrhs, int m) {
    if (h->kr_nrhs >= nrhs && h->kr_m >= m && h->kr_vlen == vlen(h)) return FDFD_OK;
    dev_free(h, h->kb); dev_free(h, h->kx); dev_free(h, h->kr); dev_free(h, h->kV); dev_free(h, h->kZ); dev_free(h, h->kc);
    h->kb = h->kx = h->kr = h->kV = h->kZ = h->kc = nullptr;
    h->kr_nrhs = h->kr_m = 0;   // stay 0 unless every allocation succeeds
    h->kr_vlen = 0;
    long long N = vlen(h);
    size_t v = (size_t)N * nrhs * sizeof(cplx<double>);
    RET(dev_alloc(h, (void**)&h->kb, v));
    RET(dev_alloc(h, (void**)&h->kx, v));
    RET(dev_alloc(h, (void**)&h->kr, v));
    RET(dev_alloc(h, (void**)&h->kV, v * (m + 1)));
    RET(dev_alloc(h, (void**)&h->kZ, v * m));
    // coefficients: 2(m+2) per rhs for the refinement, 2 per sideband for the recovery
    RET(dev_alloc(h, (void**)&h->kc, ((size_t)nrhs * (m + 2) * 2 + 2 * MF_MAX_K) * sizeof(cplx<double>)));
    h->kr_nrhs = nrhs;
    h->kr_m = m;
    h->kr_vlen = vlen(h);
    return FDFD_OK;
}

// Solve A x = b (h->kb, nrhs vectors) into h->kx to ||b - A x||/||b|| <= tol.
// GMRES mode: restarted flexible GMRES (Saad 1993) with classical Gram-Schmidt
// and one re-orthogonalisation, right-preconditioned by the factorization.
// give_up: stop as soon as the residual reduction measured over the last
// update projects past max_iter solves (the caller then re-factors).
int refine(fdfd_handle* h, int nrhs, int* iters, double* relres, bool give_up) {
    long long N = vlen(h);
    // the caller sized the workspace (ensure_krylov) before filling h->kb
    if (h->kr_nrhs < nrhs || h->kr_m < 1) return set_err(h, FDFD_EINVAL, "Krylov workspace not allocated");
    const int m = std::min(restart_len(h, nrhs), h->kr_m);
    const size_t vs = (size_t)N * nrhs;   // stride between basis vectors
    if (!h->warm_start) CK(cudaMemsetAsync(h->kx, 0, vs * sizeof(cplx<double>), h->stream));
    h->warm_start = false;
    std::vector<double> nrm;
    RET(residual(h, h->kx, h->kb, h->kr, nrhs, &nrm));
    std::vector<double> bnorm(nrhs), rel(nrhs);
    for (int r = 0; r < nrhs; ++r) {
        bnorm[r] = std::sqrt(nrm[2 * r + 1]);
        if (bnorm[r] == 0) bnorm[r] = 1;
        rel[r] = std::sqrt(nrm[2 * r]) / bnorm[r];
    }
    int it = 0;
    auto maxrel = [&]() { return *std::max_element(rel.begin(), rel.end()); };
    // log-linear projection of the solves still needed from the reduction
    // r0 -> r1 over `used` solves
    auto hopeless = [&](double r0, double r1, int used) {
        if (!give_up || r1 <= h->tol || used < 1) return false;
        if (!(r1 < r0)) return true;
        const double per = std::log(r1 / r0) / used;
        return it + std::log(h->tol / r1) / per > h->max_iter;
    };
    if (h->refine_mode == FDFD_REFINE_CLASSIC) {
        while (maxrel() > h->tol && it < h->max_iter) {
            const double r0 = maxrel();
            RET(precond(h, h->kr, h->kZ, nrhs));
            ++it;
            std::vector<zd> one(nrhs, zd(1, 0));
            RET(combine(h, h->kZ, 0, 1, one, nrhs, 1.0, h->kx));
            RET(residual(h, h->kx, h->kb, h->kr, nrhs, &nrm));
            for (int r = 0; r < nrhs; ++r) rel[r] = std::sqrt(nrm[2 * r]) / bnorm[r];
            if (it >= 3 && hopeless(r0, maxrel(), 1)) break;
        }
    } else {
        while (maxrel() > h->tol && it < h->max_iter) {
            const double r0 = maxrel();
            // start a cycle from the current residual
            std::vector<double> beta(nrhs);
            std::vector<zd> inv(nrhs);
            for (int r = 0; r < nrhs; ++r) {
                beta[r] = rel[r] * bnorm[r];
                inv[r] = beta[r] > 0 ? zd(1.0 / beta[r], 0) : zd(0, 0);
            }
            RET(scale_vec(h, h->kr, inv, nrhs, h->kV));
            std::vector<std::vector<zd>> H(nrhs, std::vector<zd>((m + 1) * m, 0));
            std::vector<std::vector<zd>> cs(nrhs, std::vector<zd>(m)), sn(nrhs, std::vector<zd>(m));
            std::vector<std::vector<zd>> gvec(nrhs, std::vector<zd>(m + 1, 0));
            for (int r = 0; r < nrhs; ++r) gvec[r][0] = beta[r];
            std::vector<char> done(nrhs, 0);
            int j = 0;
            for (; j < m && it < h->max_iter; ++j) {
                cplx<double>* Vj = h->kV + j * vs;
                cplx<double>* Vn = h->kV + (j + 1) * vs;
                cplx<double>* Zj = h->kZ + j * vs;
                RET(precond(h, Vj, Zj, nrhs));
                ++it;
                RET(residual(h, Zj, nullptr, Vn, nrhs, nullptr));   // Vn = A Zj
                // Vn ⟂ V_0..V_j, normalised (the device applies 1/hn, or 0 where hn ≤ 1e-300)
                std::vector<zd> hc, hc2;
                std::vector<double> nn;
                RET(arnoldi_orth(h, h->kV, vs, j + 1, Vn, nrhs, hc, hc2, nn));
                bool all = true;
                for (int r = 0; r < nrhs; ++r) {
                    std::vector<zd>& Hr = H[r];
                    for (int i = 0; i <= j; ++i) Hr[i * m + j] = hc[r * (j + 1) + i] + hc2[r * (j + 1) + i];
                    double hn = std::sqrt(std::max(0.0, nn[r]));
                    Hr[(j + 1) * m + j] = hn;
                    // apply previous Givens rotations
                    for (int i = 0; i < j; ++i) {
                        zd a = Hr[i * m + j], bb = Hr[(i + 1) * m + j];
                        Hr[i * m + j] = std::conj(cs[r][i]) * a + std::conj(sn[r][i]) * bb;
                        Hr[(i + 1) * m + j] = -sn[r][i] * a + cs[r][i] * bb;
                    }
                    zd a = Hr[j * m + j], bb = Hr[(j + 1) * m + j];
                    double den = std::sqrt(std::norm(a) + std::norm(bb));
                    if (den == 0) { cs[r][j] = 1; sn[r][j] = 0; }
                    else { cs[r][j] = a / den; sn[r][j] = bb / den; }
                    Hr[j * m + j] = std::conj(cs[r][j]) * a + std::conj(sn[r][j]) * bb;
                    Hr[(j + 1) * m + j] = 0;
                    zd g0 = gvec[r][j];
                    gvec[r][j] = std::conj(cs[r][j]) * g0;
                    gvec[r][j + 1] = -sn[r][j] * g0;
                    double est = std::abs(gvec[r][j + 1]) / bnorm[r];
                    if (est <= 0.5 * h->tol || hn <= 1e-300 * bnorm[r]) done[r] = 1;
                    if (!done[r]) all = false;
                }
                if (all) { ++j; break; }
            }
            // x += Z y  with H y = g (upper triangular, j columns)
            int k = j;
            std::vector<zd> coef((size_t)nrhs * k);
            for (int r = 0; r < nrhs; ++r) {
                std::vector<zd> y(k);
                for (int i = k - 1; i >= 0; --i) {
                    zd s = gvec[r][i];
                    for (int l = i + 1; l < k; ++l) s -= H[r][i * m + l] * y[l];
                    zd d = H[r][i * m + i];
                    y[i] = std::abs(d) > 0 ? s / d : zd(0, 0);
                }
                for (int i = 0; i < k; ++i) coef[(size_t)r * k + i] = y[i];
            }
            if (k > 0) RET(combine(h, h->kZ, vs, k, coef, nrhs, 1.0, h->kx));
            RET(residual(h, h->kx, h->kb, h->kr, nrhs, &nrm));
            for (int r = 0; r < nrhs; ++r) rel[r] = std::sqrt(nrm[2 * r]) / bnorm[r];
            if (hopeless(r0, maxrel(), k)) break;
        }
    }
    *iters = it;
    *relres = maxrel();
    return FDFD_OK;
}

// ---------------------------------------------------------------------------
// Assembly + factorization of the operator `op`
// ---------------------------------------------------------------------------
// the operator's assembly arguments, copied to the handle's device argument block on `s`
int assemble_args(fdfd_handle* h, int op, double omega_pml, zd sigma, double omega_drv, cudaStream_t s) {
    SFactorArgs& sa = h->hargs.sf;
    sa.Nx = h->Nx; sa.Ny = h->Ny; sa.Npx = h->Npx; sa.Npy = h->Npy;
    sa.dx = h->dx; sa.dy = h->dy; sa.omega = omega_pml; sa.eps0n = kEPS0 * h->L0;
    sa.eta0 = std::sqrt(kMU0 / kEPS0); sa.m = h->pml_m; sa.lnR = h->pml_lnR;
    StencilArgs& a = h->hargs.st;
    a.Nx = h->Nx; a.Ny = h->Ny; a.op = op;
    a.idx = 1.0 / h->dx; a.idy = 1.0 / h->dy;
    a.imu0 = 1.0 / (kMU0 * h->L0);
    a.eps0n = kEPS0 * h->L0;
    a.omega2 = omega_drv * omega_drv;
    a.omega2mu0 = omega_drv * omega_drv * (kMU0 * h->L0);
    a.sigma_re = sigma.real(); a.sigma_im = sigma.imag();
    CK(cudaMemcpyAsync(h->dargs, &h->hargs, sizeof(AssembleArgs), cudaMemcpyHostToDevice, s));
    return FDFD_OK;
}

// the assembly kernels (device arguments), on the handle's stream
int assemble_kernels(fdfd_handle* h) {
    int tot = 2 * h->Nx + 2 * h->Ny;
    LAUNCH(sfactor_kernel, ceil_div(tot, 128), 128, 0, &h->dargs->sf, h->sf);
    long long N = (long long)h->Nx * h->Ny;
    LAUNCH(stencil_kernel, ceil_div(N, 256), 256, 0, &h->dargs->st, h->eps, h->sf, h->st);
    return check_launch(h, "assemble");
}

int assemble(fdfd_handle* h, int op, double omega_pml, zd sigma, double omega_drv) {
    RET(assemble_args(h, op, omega_pml, sigma, omega_drv, h->stream));
    RET(assemble_kernels(h));
    long long N = (long long)h->Nx * h->Ny;
    // factorization scale: power of two nearest 1/Σ|off-diagonal| at the grid centre
    long long kc = h->Nx / 2 + (long long)h->Nx * (h->Ny / 2);
    cplx<double> c[5];
    for (int p = 0; p < 5; ++p)
        CK(cudaMemcpyAsync(&c[p], h->st + p * N + kc, sizeof(cplx<double>), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    double s = 0;
    for (int p = 1; p < 5; ++p) s += std::hypot(c[p].re, c[p].im);
    if (!(s > 0) || !std::isfinite(s)) return set_err(h, FDFD_EINVAL, "degenerate operator (zero couplings)");
    h->scale = std::ldexp(1.0, -(int)std::lround(std::log2(s)));
    h->op = op;
    return FDFD_OK;
}

// factors the assembled operator in precision `prec` (FDFD_PREC_*; -1: the handle's)
int factor_op(fdfd_handle* h, int prec = -1);

// modulated device: assemble and factor the K sideband operators
// (modulation.jl:79-92; PML at ω when shared, else at ωₙ)
int factor_mf(fdfd_handle* h, int prec) {
    MfState& M = *h->mf;
    h->factored = false;
    for (int n = 0; n < M.K; ++n) {
        fdfd_handle* s = M.sub[n];
        const long long l0 = s->launches;
        int rc = assemble(s, OP_TM_SIDEBAND, M.shared_pml ? M.omega : M.wn[n], zd(0, 0), M.wn[n]);
        if (rc == FDFD_OK) rc = factor_op(s, prec);
        h->launches += s->launches - l0;
        if (rc != FDFD_OK) return set_err(h, rc, "sideband %d: %s", n, s->err.c_str());
    }
    h->fact_prec = prec;
    h->fell_back = prec != h->precision;
    h->op = OP_TM_SIDEBAND;
    h->factored = true;
    return FDFD_OK;
}

int factor_op(fdfd_handle* h, int prec) {
    if (prec < 0) prec = h->precision;
    if (h->mf) return factor_mf(h, prec);
    h->factored = false;
    int rc = prec == FDFD_PREC_FP64 ? factor_impl<double>(h) : factor_impl<float>(h);
    if (rc != FDFD_OK) return rc;
    RET(check_device(h, "factor"));
    h->fact_prec = prec;
    h->fell_back = prec != h->precision;
    h->factored = true;
    return FDFD_OK;
}

// refine() and, for a MIXED handle whose FP32-preconditioned refinement
// stalls, an FP64 factorization of the same operator followed by a second
// refinement (the first one's iterations count towards *iters).
int refine_fb(fdfd_handle* h, int nrhs, int* iters, double* relres) {
    const bool can = h->fallback && h->fact_prec == FDFD_PREC_MIXED;
    RET(refine(h, nrhs, iters, relres, can));
    if (!can || *relres <= h->tol) return FDFD_OK;
    RET(factor_op(h, FDFD_PREC_FP64));
    int it2 = 0;
    RET(refine(h, nrhs, &it2, relres, false));
    *iters += it2;
    return FDFD_OK;
}

double elapsed_ms(cudaEvent_t a, cudaEvent_t b) {
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    return ms;
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

const char* fdfd_version(void) { return FDFD_VERSION_STR; }

const char* fdfd_last_error(const fdfd_handle* h) { return h ? h->err.c_str() : "null handle"; }

int fdfd_create(fdfd_handle** out, int Nx, int Ny, int Npx, int Npy, double dx, double dy, double L0, double pml_m,
                double pml_lnR, int pol, int precision) {
    if (!out) return FDFD_EINVAL;
    *out = nullptr;
    if (Nx < 3 || Ny < 3 || Npx < 0 || Npy < 0 || 2 * Npx > Nx || 2 * Npy > Ny) return FDFD_EINVAL;
    if (!(dx > 0) || !(dy > 0) || !(L0 > 0) || !std::isfinite(pml_m) || !std::isfinite(pml_lnR)) return FDFD_EINVAL;
    if (pol != FDFD_TM && pol != FDFD_TE) return FDFD_EINVAL;
    if (precision != FDFD_PREC_FP64 && precision != FDFD_PREC_MIXED) return FDFD_EINVAL;
    if (std::min(Nx, Ny) > 1024) return FDFD_EINVAL;   // dense block size limit of the panel kernel
    fdfd_handle* h = new fdfd_handle();
    h->Nx = Nx; h->Ny = Ny; h->Npx = Npx; h->Npy = Npy;
    h->dx = dx; h->dy = dy; h->L0 = L0; h->pml_m = pml_m; h->pml_lnR = pml_lnR;
    h->pol = pol; h->precision = precision;
    const char* env = getenv("FDFD_DISABLE_TC");
    if (env && env[0] == '1') h->use_tc = false;
    const char* env1 = getenv("FDFD_LEVEL1_GJ");
    if (env1 && env1[0] == '1') h->level1_gj = true;
    const char* env2 = getenv("FDFD_DENSE_L1_SWEEP");
    if (env2 && env2[0] == '1') h->tri_sweep = false;
    if (const char* e = getenv("FDFD_GJ_FUSED_K")) h->gj_fused_k = std::max(0, atoi(e));
    if (const char* e = getenv("FDFD_GJ_CL")) h->gj_cl = atoi(e);
    if (const char* e = getenv("FDFD_GJ_FORM")) h->gj_form = atoi(e) == 1 ? 1 : 0;
    if (const char* e = getenv("FDFD_GJ_PRESPLIT")) h->gj_presplit = atoi(e) != 0;
    if (const char* e = getenv("FDFD_GEMV_BULK")) h->gemv_bulk = atoi(e) != 0;
    if (const char* e = getenv("FDFD_SPLITK")) h->splitk = atoi(e) != 0;
    if (const char* e = getenv("FDFD_FACTOR_GRAPH")) h->graph_factor = atoi(e) != 0;
    if (const char* e = getenv("FDFD_GJ_FUSED_MIN")) h->gj_fused_min = std::max(1, atoi(e));
    NodeMap& m = h->map;
    m.Nx = Nx; m.Ny = Ny;
    m.transposed = Nx > Ny ? 1 : 0;
    m.b = m.transposed ? Ny : Nx;
    m.n = m.transposed ? Nx : Ny;
    m.ld = (m.b + 31) / 32 * 32;
    auto fail = [&](int rc) {
        fdfd_destroy(h);
        return rc;
    };
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        delete h;
        return FDFD_ECUDA;
    }
    for (auto& e : h->ev) cudaEventCreate(&e);
    if (cudaStreamCreateWithFlags(&h->stream2, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ev_panel, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ev_wide, cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        return fail(FDFD_ECUDA);
    }
    {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || h->num_sms < 1)
            h->num_sms = 1;
    }
    long long N = (long long)Nx * Ny;
    int rc;
    if ((rc = dev_alloc(h, (void**)&h->eps, N * sizeof(cplx<double>)))) return fail(rc);
    if ((rc = dev_alloc(h, (void**)&h->sf, 2 * (2 * Nx + 2 * Ny) * sizeof(cplx<double>)))) return fail(rc);
    if ((rc = dev_alloc(h, (void**)&h->st, 5 * N * sizeof(cplx<double>)))) return fail(rc);
    if ((rc = dev_alloc(h, (void**)&h->derr, sizeof(unsigned)))) return fail(rc);
    if ((rc = dev_alloc(h, (void**)&h->dargs, sizeof(AssembleArgs)))) return fail(rc);
    cudaMemsetAsync(h->derr, 0, sizeof(unsigned), h->stream);
    build_plan(h);
    JobBlob B;
    build_jobs(h, B);
    if ((rc = dev_alloc(h, (void**)&h->djobs, B.host.size()))) return fail(rc);
    if (cudaMemcpy(h->djobs, B.host.data(), B.host.size(), cudaMemcpyHostToDevice) != cudaSuccess) return fail(FDFD_ECUDA);
    *out = h;
    return FDFD_OK;
}

void fdfd_destroy(fdfd_handle* h) {
    if (!h) return;
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->fgexec) cudaGraphExecDestroy(h->fgexec);
    if (h->fgraph) cudaGraphDestroy(h->fgraph);
    for (int i = 0; i < 2; ++i) {
        if (h->sg_exec[i]) cudaGraphExecDestroy(h->sg_exec[i]);
        if (h->sg_graph[i]) cudaGraphDestroy(h->sg_graph[i]);
    }
    if (h->mf) {
        for (fdfd_handle* s : h->mf->sub) fdfd_destroy(s);
        dev_free(h, h->mf->deps);
        if (h->mf->ev_in) cudaEventDestroy(h->mf->ev_in);
        for (auto& e : h->mf->ev_out) if (e) cudaEventDestroy(e);
        delete h->mf;
        h->mf = nullptr;
    }
    void* bufs[] = {h->eps, h->sf, h->st, h->derr, h->dargs, h->part, h->red, h->kb, h->kx, h->kr, h->kV, h->kZ,
                    h->kc, h->io, h->djobs, h->mode_buf, h->nl_d1, h->eps_stage, h->vflags};
    for (void* p : bufs) dev_free(h, p);
    if (h->vflags_h) cudaFreeHost(h->vflags_h);
    free_store(h, h->f32);
    free_store(h, h->f64);
    for (auto& e : h->ev) if (e) cudaEventDestroy(e);
    for (auto& e : h->evpool) cudaEventDestroy(e);
    if (h->stream) cudaStreamDestroy(h->stream);
    if (h->stream2) cudaStreamDestroy(h->stream2);
    if (h->ev_panel) cudaEventDestroy(h->ev_panel);
    if (h->ev_wide) cudaEventDestroy(h->ev_wide);
    delete h;
}

int fdfd_set_refinement(fdfd_handle* h, double tol, int max_iter, int mode) {
    if (!h) return FDFD_EINVAL;
    if (!(tol > 0) || max_iter < 1 || (mode != FDFD_REFINE_GMRES && mode != FDFD_REFINE_CLASSIC))
        return set_err(h, FDFD_EINVAL, "invalid refinement settings");
    h->tol = tol; h->max_iter = max_iter; h->refine_mode = mode;
    return FDFD_OK;
}

int fdfd_set_restart(fdfd_handle* h, int m) {
    if (!h) return FDFD_EINVAL;
    if (m < 0 || m > 512) return set_err(h, FDFD_EINVAL, "restart length must be in [0, 512]");
    h->restart = m;
    return FDFD_OK;
}

int fdfd_set_fallback(fdfd_handle* h, int on) {
    if (!h) return FDFD_EINVAL;
    h->fallback = on != 0;
    return FDFD_OK;
}

int fdfd_set_wait_limit(fdfd_handle* h, long long ns) {
    if (!h) return FDFD_EINVAL;
    if (h->mf)
        for (fdfd_handle* s : h->mf->sub) s->wait_ns = ns > 0 ? (unsigned long long)ns : 0ull;
    h->wait_ns = ns > 0 ? (unsigned long long)ns : 0ull;
    h->cfg_gen++;
    return FDFD_OK;
}

int fdfd_set_checkpoint(fdfd_handle* h, int mode) {
    if (!h || mode < -1 || mode > 1) return FDFD_EINVAL;
    if (h->mf) {
        for (fdfd_handle* s : h->mf->sub) RET(fdfd_set_checkpoint(s, mode));
        h->ckpt_mode = mode;
        return FDFD_OK;
    }
    if (h->ckpt && mode < 0) return set_err(h, FDFD_EINVAL, "checkpoint mode is engaged for the handle's lifetime");
    if (!h->ckpt && mode == 1 && (h->f32.complete || h->f64.complete))
        return set_err(h, FDFD_EINVAL, "fdfd_set_checkpoint(1) must come before the first factorization");
    h->ckpt_mode = mode;
    h->cfg_gen++;
    return FDFD_OK;
}

int fdfd_checkpoint_info(const fdfd_handle* h, int* active, long long* host_bytes, long long* copied_bytes) {
    if (!h) return FDFD_EINVAL;
    if (active) *active = h->ckpt ? 1 : 0;
    if (host_bytes) *host_bytes = h->host_bytes;
    if (copied_bytes) *copied_bytes = h->ckpt_copied;
    return FDFD_OK;
}

int fdfd_set_device_budget(fdfd_handle* h, long long bytes) {
    if (!h || bytes < 0) return FDFD_EINVAL;
    if (h->mf)
        for (fdfd_handle* s : h->mf->sub) s->dev_budget = bytes;
    h->dev_budget = bytes;
    h->cfg_gen++;
    return FDFD_OK;
}

int fdfd_set_eps(fdfd_handle* h, const double* eps_r) {
    if (!h || !eps_r) return h ? set_err(h, FDFD_EINVAL, "eps_r is NULL") : FDFD_EINVAL;
    long long N = (long long)h->Nx * h->Ny;
    // staged and validated on the device (one read at HBM speed instead of two host scans);
    // a rejected ϵᵣ leaves the handle's permittivity as it was
    if (!h->eps_stage) RET(dev_alloc(h, (void**)&h->eps_stage, N * sizeof(cplx<double>)));
    CK(cudaMemcpyAsync(h->eps_stage, eps_r, N * sizeof(cplx<double>), cudaMemcpyHostToDevice, h->stream));
    long long kbad = -1, kzero = -1;
    RET(validate_device(h, reinterpret_cast<const double*>(h->eps_stage), N, true, &kbad, &kzero));
    if (kbad >= 0) return set_err(h, FDFD_EINVAL, "eps_r has a non-finite entry at %lld", kbad / 2);
    if (kzero >= 0) return set_err(h, FDFD_EINVAL, "eps_r is zero at %lld", kzero);
    CK(cudaMemcpyAsync(h->eps, h->eps_stage, N * sizeof(cplx<double>), cudaMemcpyDeviceToDevice, h->stream));
    if (h->mf)
        for (fdfd_handle* s : h->mf->sub) {
            CK(cudaMemcpyAsync(s->eps, h->eps, N * sizeof(cplx<double>), cudaMemcpyDeviceToDevice, h->stream));
            s->eps_set = true;
            s->factored = false;
        }
    CK(cudaStreamSynchronize(h->stream));
    h->eps_set = true;
    h->factored = false;
    return FDFD_OK;
}

}  // extern "C"

namespace {

int factor_work(fdfd_handle* h);

// the ordinary driven factorization: assembly (with its scale), then the factorization
int factor_plain(fdfd_handle* h, double omega) {
    h->launches = 0;
    h->factored = false;
    cudaEventRecord(h->ev[0], h->stream);
    RET(assemble(h, h->pol == FDFD_TM ? OP_TM_DRIVEN : OP_TE_DRIVEN, omega, zd(0, 0), omega));
    cudaEventRecord(h->ev[1], h->stream);
    RET(factor_op(h));
    cudaEventRecord(h->ev[2], h->stream);
    h->omega = omega;
    return FDFD_OK;
}

// capture of the work factor_plain just did (assembly kernels reading their arguments from
// device memory, then the factorization) as this handle's graph; nothing runs
int factor_capture(fdfd_handle* h, double omega) {
    if (h->fgexec) { cudaGraphExecDestroy(h->fgexec); h->fgexec = nullptr; }
    if (h->fgraph) { cudaGraphDestroy(h->fgraph); h->fgraph = nullptr; }
    const long long l0 = h->launches;
    if (cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        return FDFD_OK;   // no graph: the plain path stays in use
    }
    int rc = factor_work(h);
    cudaGraph_t g = nullptr;
    const cudaError_t ee = cudaStreamEndCapture(h->stream, &g);
    const long long kernels = h->launches - l0;
    h->launches = l0;
    if (rc == FDFD_OK && ee == cudaSuccess && g && cudaGraphInstantiate(&h->fgexec, g, 0) == cudaSuccess) {
        h->fgraph = g;
        h->fg_omega = omega;
        h->fg_scale = h->scale;
        h->fg_kernels = kernels;
        h->fg_gen = h->cfg_gen;
        return FDFD_OK;
    }
    cudaGetLastError();
    if (g) cudaGraphDestroy(g);
    h->fgexec = nullptr;
    h->err.clear();
    return FDFD_OK;   // capture is an optimisation: its failure leaves the plain path
}

// replay: the assembly arguments for ω (device memory, on the handle's stream), then the graph
int factor_replay(fdfd_handle* h, double omega) {
    const int op = h->pol == FDFD_TM ? OP_TM_DRIVEN : OP_TE_DRIVEN;
    h->launches = 0;
    h->factored = false;
    cudaEventRecord(h->ev[0], h->stream);
    RET(assemble_args(h, op, omega, zd(0, 0), omega, h->stream));
    cudaEventRecord(h->ev[1], h->stream);
    if (cudaGraphLaunch(h->fgexec, h->stream) != cudaSuccess) {
        cudaGetLastError();
        return set_err(h, FDFD_ECUDA, "cudaGraphLaunch of the factorization failed");
    }
    cudaEventRecord(h->ev[2], h->stream);
    h->launches = h->fg_kernels;
    h->scale = h->fg_scale;   // the scale the captured work was built with
    h->op = op;
    RET(check_device(h, "factor"));
    h->fact_prec = h->precision;
    h->fell_back = false;
    h->factored = true;
    h->omega = omega;
    return FDFD_OK;
}

}  // namespace

extern "C" {

int fdfd_factor(fdfd_handle* h, double omega) {
    if (!h) return FDFD_EINVAL;
    if (h->mf) return set_err(h, FDFD_EINVAL, "modulated device: use fdfd_mf_factor");
    if (!h->eps_set) return set_err(h, FDFD_EINVAL, "fdfd_set_eps must be called before fdfd_factor");
    if (!(omega > 0) || !std::isfinite(omega)) return set_err(h, FDFD_EINVAL, "omega must be positive and finite");
    // (not while profiling, whose per-launch events need plain launches, nor in checkpoint
    // mode, whose host copies are left to the plain path)
    const bool graphable = h->graph_factor && !h->prof_on && !h->ckpt && h->ckpt_mode != 1;
    if (graphable && h->fgexec && h->fg_gen == h->cfg_gen && h->fg_omega == omega) return factor_replay(h, omega);
    RET(factor_plain(h, omega));
    // a second consecutive factorization at this ω: capture it for the next ones
    if (graphable && h->fact_prec == h->precision && h->last_plain_omega == omega) RET(factor_capture(h, omega));
    h->last_plain_omega = omega;
    return FDFD_OK;
}

}  // extern "C"

namespace {

// driven solve on device buffers: src (nrhs natural vectors) -> fields
int solve_core(fdfd_handle* h, const cplx<double>* d_src, int nrhs, cplx<double>* f1, cplx<double>* f2,
               cplx<double>* f3, fdfd_stats* st) {
    if (h->mf) return set_err(h, FDFD_EINVAL, "modulated device: use fdfd_mf_solve");
    if (!h->factored || (h->op != OP_TM_DRIVEN && h->op != OP_TE_DRIVEN))
        return set_err(h, FDFD_EINVAL, "fdfd_factor must be called before the solve");
    long long N = (long long)h->Nx * h->Ny;
    RET(ensure_krylov(h, nrhs, restart_len(h, nrhs)));
    cudaEventRecord(h->ev[3], h->stream);
    // b = iω·src   (driven.jl:36,46)
    std::vector<zd> iw(nrhs, zd(0, h->omega));
    RET(scale_vec(h, d_src, iw, nrhs, h->kb));
    int iters = 0;
    double rel = 0;
    RET(refine_fb(h, nrhs, &iters, &rel));
    cudaEventRecord(h->ev[4], h->stream);
    RET(check_device(h, "solve"));
    if (f1) CK(cudaMemcpyAsync(f1, h->kx, N * nrhs * sizeof(cplx<double>), cudaMemcpyDeviceToDevice, h->stream));
    if (f2 || f3) {
        // coefficients per rhs (driven.jl:40-41, 199-200)
        std::vector<zd> coef(2 * nrhs);
        const double w = h->omega, mu0 = kMU0 * h->L0;
        for (int r = 0; r < nrhs; ++r) {
            if (h->pol == FDFD_TM) {
                coef[2 * r] = zd(-0.0, (1.0 / w) / mu0);      // -1/1im/ω/μ₀
                coef[2 * r + 1] = zd(0.0, (-1.0 / w) / mu0);  //  1/1im/ω/μ₀
            } else {
                coef[2 * r] = zd(0.0, -1.0 / w);              //  1/1im/ω
                coef[2 * r + 1] = coef[2 * r];
            }
        }
        CK(cudaMemcpyAsync(h->kc, coef.data(), coef.size() * sizeof(zd), cudaMemcpyHostToDevice, h->stream));
        RecoverArgs ra;
        ra.Nx = h->Nx; ra.Ny = h->Ny; ra.mode = h->pol == FDFD_TM ? REC_TM_DRIVEN : REC_TE_DRIVEN;
        ra.idx = 1.0 / h->dx; ra.idy = 1.0 / h->dy; ra.eps0n = kEPS0 * h->L0;
        cplx<double>* g1 = f2 ? f2 : h->kr;
        cplx<double>* g2 = f3 ? f3 : h->kr;
        LAUNCH(recover_kernel, dim3(ceil_div(N, 256), nrhs), 256, 0, ra, h->sf, h->eps, h->kx, h->kc, g1, g2);
        RET(check_launch(h, "recover"));
    }
    cudaEventRecord(h->ev[5], h->stream);
    CK(cudaStreamSynchronize(h->stream));
    if (st) {
        st->iterations = iters;
        st->nrhs = nrhs;
        st->rel_residual = rel;
        st->t_assemble_ms = elapsed_ms(h->ev[0], h->ev[1]);
        st->t_factor_ms = elapsed_ms(h->ev[1], h->ev[2]);
        st->t_solve_ms = elapsed_ms(h->ev[3], h->ev[4]);
        st->t_recover_ms = elapsed_ms(h->ev[4], h->ev[5]);
        st->factor_flops = h->last_factor_flops;
        st->block = h->map.b;
        st->nblocks = h->map.n;
        st->levels = (int)h->steps.size() + 1;
        st->tc_gemm = h->tc_used;
        st->factor_precision = h->fact_prec;
        st->fp64_fallback = h->fell_back;
        st->device_bytes = h->dev_bytes;
        st->gpu_launches = h->launches;
    }
    if (!(rel <= h->tol))
        return set_err(h, FDFD_ENOCONV, "refinement stopped at relative residual %.3e > tol %.1e after %d iterations",
                       rel, h->tol, iters);
    return FDFD_OK;
}

}  // namespace

extern "C" {

int fdfd_solve_device(fdfd_handle* h, const double* d_src, int nrhs, double* d_f1, double* d_f2, double* d_f3,
                      fdfd_stats* stats) {
    if (!h) return FDFD_EINVAL;
    if (!d_src || nrhs < 1) return set_err(h, FDFD_EINVAL, "invalid source arguments");
    auto t0 = std::chrono::steady_clock::now();
    int rc = solve_core(h, (const cplx<double>*)d_src, nrhs, (cplx<double>*)d_f1, (cplx<double>*)d_f2,
                        (cplx<double>*)d_f3, stats);
    if (stats) stats->t_total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return rc;
}

int fdfd_solve(fdfd_handle* h, const double* src, int nrhs, double* f1, double* f2, double* f3, fdfd_stats* stats) {
    if (!h) return FDFD_EINVAL;
    if (!src || nrhs < 1) return set_err(h, FDFD_EINVAL, "invalid source arguments");
    auto t0 = std::chrono::steady_clock::now();
    long long N = (long long)h->Nx * h->Ny;
    size_t bytes = (size_t)N * nrhs * sizeof(cplx<double>);
    // staging: [src | f1 | f2 | f3], kept by the handle between calls
    if (h->io_cap < 4 * bytes) {
        dev_free(h, h->io);
        h->io = nullptr;
        h->io_cap = 0;
        RET(dev_alloc(h, (void**)&h->io, 4 * bytes));
        h->io_cap = 4 * bytes;
    }
    cplx<double>* io = h->io;
    cplx<double>* dsrc = io;
    cplx<double>* d1 = f1 ? io + N * nrhs : nullptr;
    cplx<double>* d2 = f2 ? io + 2 * N * nrhs : nullptr;
    cplx<double>* d3 = f3 ? io + 3 * N * nrhs : nullptr;
    int rc = FDFD_OK;
    if (cudaMemcpyAsync(dsrc, src, bytes, cudaMemcpyHostToDevice, h->stream) != cudaSuccess)
        rc = set_err(h, FDFD_ECUDA, "copy of src failed");
    if (rc == FDFD_OK) {   // validated on the device, before any solve work
        long long kbad = -1;
        rc = validate_device(h, reinterpret_cast<const double*>(dsrc), N * nrhs, false, &kbad, nullptr);
        if (rc == FDFD_OK && kbad >= 0) rc = set_err(h, FDFD_EINVAL, "src has a non-finite entry");
    }
    if (rc == FDFD_OK) rc = solve_core(h, dsrc, nrhs, d1, d2, d3, stats);
    if (rc == FDFD_OK || rc == FDFD_ENOCONV) {
        if (f1) cudaMemcpyAsync(f1, d1, bytes, cudaMemcpyDeviceToHost, h->stream);
        if (f2) cudaMemcpyAsync(f2, d2, bytes, cudaMemcpyDeviceToHost, h->stream);
        if (f3) cudaMemcpyAsync(f3, d3, bytes, cudaMemcpyDeviceToHost, h->stream);
        if (cudaStreamSynchronize(h->stream) != cudaSuccess) rc = set_err(h, FDFD_ECUDA, "copy of fields failed");
    }
    if (stats) stats->t_total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return rc;
}

// ---- modulated device (multi-frequency FDFD), modulation.jl -----------------
// ---- batched factorizations in one CUDA graph ------------------------------
// Many frequencies, or independent problems of uneven sizes, each on its own
// handle: their assemblies and factorizations become the parallel branches of one
// captured graph, so a batch is one cudaGraphLaunch and the GPU runs the
// factorizations side by side (the deep, few-matrix levels of one leave most of
// the GPU to the others).  The first fdfd_batch_factor factors every handle the
// ordinary way (allocating its storage and fixing its scaling), then captures the
// work; later calls rewrite each handle's assembly arguments (frequency) and
// replay the graph.  The captured work is the factorization only: solves run on
// each handle afterwards (they are ordered after the graph on the handle's stream).
}  // extern "C"

struct fdfd_batch {
    std::vector<fdfd_handle*> hs;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_done = nullptr, ev_t0 = nullptr, ev_t1 = nullptr;
    std::vector<cudaEvent_t> ev_join, ev_in;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    long long kernels = 0;        // kernel launches captured in the graph
    std::vector<long long> hkernels;   // ... per handle
    long long graph_launches = 0; // cudaGraphLaunch calls
    double last_ms = 0;           // device time of the last graph launch
    std::string err;
};

namespace {

int batch_err(fdfd_batch* B, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    B->err = buf;
    return code;
}

// the device work of one handle's driven factorization (assembly kernels from the
// device argument block, then the block cyclic reduction), on its stream
int factor_work(fdfd_handle* h) {
    RET(assemble_kernels(h));
    return h->precision == FDFD_PREC_FP64 ? factor_impl<double>(h) : factor_impl<float>(h);
}

int batch_capture(fdfd_batch* B) {
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(B->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        return batch_err(B, FDFD_ECUDA, "cudaStreamBeginCapture failed");
    }
    int rc = FDFD_OK;
    long long k0 = 0;
    for (fdfd_handle* h : B->hs) k0 += h->launches;
    B->hkernels.assign(B->hs.size(), 0);
    if (cudaEventRecord(B->ev_fork, B->stream) != cudaSuccess) rc = FDFD_ECUDA;
    for (size_t i = 0; i < B->hs.size() && rc == FDFD_OK; ++i) {
        fdfd_handle* h = B->hs[i];
        if (cudaStreamWaitEvent(h->stream, B->ev_fork, 0) != cudaSuccess) { rc = FDFD_ECUDA; break; }
        const long long l0 = h->launches;
        rc = factor_work(h);
        B->hkernels[i] = h->launches - l0;
        if (rc != FDFD_OK) { B->err = h->err; break; }
        if (cudaEventRecord(B->ev_join[i], h->stream) != cudaSuccess ||
            cudaStreamWaitEvent(B->stream, B->ev_join[i], 0) != cudaSuccess)
            rc = FDFD_ECUDA;
    }
    const cudaError_t ee = cudaStreamEndCapture(B->stream, &g);
    if (rc == FDFD_OK && (ee != cudaSuccess || !g)) rc = FDFD_ECUDA;
    long long k1 = 0;
    for (fdfd_handle* h : B->hs) k1 += h->launches;
    if (rc == FDFD_OK && cudaGraphInstantiate(&B->exec, g, 0) != cudaSuccess) rc = FDFD_ECUDA;
    if (rc != FDFD_OK) {
        cudaGetLastError();
        if (g) cudaGraphDestroy(g);
        B->exec = nullptr;
        if (B->err.empty()) B->err = "graph capture of the batch factorization failed";
        return rc;
    }
    B->graph = g;
    B->kernels = k1 - k0;
    return FDFD_OK;
}

}  // namespace

extern "C" {

int fdfd_batch_create(fdfd_batch** out, int n, fdfd_handle* const* handles) {
    if (!out || n < 1 || !handles) return FDFD_EINVAL;
    *out = nullptr;
    for (int i = 0; i < n; ++i) {
        if (!handles[i] || handles[i]->mf) return FDFD_EINVAL;
        for (int j = 0; j < i; ++j)
            if (handles[j] == handles[i]) return FDFD_EINVAL;
    }
    fdfd_batch* B = new fdfd_batch();
    B->hs.assign(handles, handles + n);
    bool ok = cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking) == cudaSuccess &&
              cudaEventCreateWithFlags(&B->ev_fork, cudaEventDisableTiming) == cudaSuccess &&
              cudaEventCreateWithFlags(&B->ev_done, cudaEventDisableTiming) == cudaSuccess &&
              cudaEventCreate(&B->ev_t0) == cudaSuccess && cudaEventCreate(&B->ev_t1) == cudaSuccess;
    B->ev_join.assign(n, nullptr);
    B->ev_in.assign(n, nullptr);
    for (int i = 0; i < n && ok; ++i)
        ok = cudaEventCreateWithFlags(&B->ev_join[i], cudaEventDisableTiming) == cudaSuccess &&
             cudaEventCreateWithFlags(&B->ev_in[i], cudaEventDisableTiming) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        fdfd_batch_destroy(B);
        return FDFD_ECUDA;
    }
    *out = B;
    return FDFD_OK;
}

void fdfd_batch_destroy(fdfd_batch* B) {
    if (!B) return;
    if (B->stream) cudaStreamSynchronize(B->stream);
    if (B->exec) cudaGraphExecDestroy(B->exec);
    if (B->graph) cudaGraphDestroy(B->graph);
    for (cudaEvent_t e : B->ev_join) if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : B->ev_in) if (e) cudaEventDestroy(e);
    cudaEvent_t evs[] = {B->ev_fork, B->ev_done, B->ev_t0, B->ev_t1};
    for (cudaEvent_t e : evs) if (e) cudaEventDestroy(e);
    if (B->stream) cudaStreamDestroy(B->stream);
    delete B;
}

const char* fdfd_batch_last_error(const fdfd_batch* B) { return B ? B->err.c_str() : "null batch"; }

int fdfd_batch_factor(fdfd_batch* B, const double* omegas, int* status) {
    if (!B) return FDFD_EINVAL;
    if (!omegas) return batch_err(B, FDFD_EINVAL, "fdfd_batch_factor: NULL omegas");
    const int n = (int)B->hs.size();
    for (int i = 0; i < n; ++i) {
        fdfd_handle* h = B->hs[i];
        if (!(omegas[i] > 0) || !std::isfinite(omegas[i]))
            return batch_err(B, FDFD_EINVAL, "fdfd_batch_factor: omega[%d] must be positive and finite", i);
        if (!h->eps_set) return batch_err(B, FDFD_EINVAL, "fdfd_batch_factor: handle %d has no permittivity", i);
        if (h->prof_on) return batch_err(B, FDFD_EINVAL, "fdfd_batch_factor: handle %d is profiling", i);
    }
    int first = FDFD_OK;
    if (!B->exec) {
        // the ordinary factorizations: storage, scaling, and this call's results
        for (int i = 0; i < n; ++i) {
            const int rc = B->hs[i]->eps_set ? factor_plain(B->hs[i], omegas[i]) : FDFD_EINVAL;
            if (status) status[i] = rc;
            if (rc != FDFD_OK && first == FDFD_OK) {
                first = rc;
                B->err = B->hs[i]->err;
            }
        }
        if (first != FDFD_OK) return first;
        for (int i = 0; i < n; ++i)
            if (B->hs[i]->fact_prec != B->hs[i]->precision) return batch_err(B, FDFD_EINVAL, "handle %d: mixed factor unavailable", i);
        return batch_capture(B);
    }
    // replay: new assembly arguments on the batch stream, after each handle's own
    // pending work (its permittivity copy)
    for (int i = 0; i < n; ++i) {
        fdfd_handle* h = B->hs[i];
        const int op = h->pol == FDFD_TM ? OP_TM_DRIVEN : OP_TE_DRIVEN;
        h->launches = 0;
        h->factored = false;
        if (cudaEventRecord(B->ev_in[i], h->stream) != cudaSuccess ||
            cudaStreamWaitEvent(B->stream, B->ev_in[i], 0) != cudaSuccess)
            return batch_err(B, FDFD_ECUDA, "batch: stream ordering failed");
        const int rc = assemble_args(h, op, omegas[i], zd(0, 0), omegas[i], B->stream);
        if (rc != FDFD_OK) return batch_err(B, rc, "%s", h->err.c_str());
    }
    if (cudaEventRecord(B->ev_t0, B->stream) != cudaSuccess || cudaGraphLaunch(B->exec, B->stream) != cudaSuccess ||
        cudaEventRecord(B->ev_t1, B->stream) != cudaSuccess || cudaEventRecord(B->ev_done, B->stream) != cudaSuccess) {
        cudaGetLastError();
        return batch_err(B, FDFD_ECUDA, "cudaGraphLaunch of the batch factorization failed");
    }
    B->graph_launches++;
    for (int i = 0; i < n; ++i)
        if (cudaStreamWaitEvent(B->hs[i]->stream, B->ev_done, 0) != cudaSuccess)
            return batch_err(B, FDFD_ECUDA, "batch: stream ordering failed");
    if (cudaStreamSynchronize(B->stream) != cudaSuccess) {
        cudaGetLastError();
        return batch_err(B, FDFD_ECUDA, "batch factorization failed on the device");
    }
    float ms = 0;
    cudaEventElapsedTime(&ms, B->ev_t0, B->ev_t1);
    B->last_ms = ms;
    for (int i = 0; i < n; ++i) {
        fdfd_handle* h = B->hs[i];
        int rc = check_device(h, "batch factor");
        if (rc == FDFD_OK) {
            h->launches = B->hkernels[i];
            h->op = h->pol == FDFD_TM ? OP_TM_DRIVEN : OP_TE_DRIVEN;
            h->omega = omegas[i];
            h->fact_prec = h->precision;
            h->fell_back = false;
            h->factored = true;
        }
        if (status) status[i] = rc;
        if (rc != FDFD_OK && first == FDFD_OK) {
            first = rc;
            B->err = h->err;
        }
    }
    return first;
}

int fdfd_batch_stats(const fdfd_batch* B, long long* kernels, long long* graph_launches, double* last_ms) {
    if (!B) return FDFD_EINVAL;
    if (kernels) *kernels = B->kernels;
    if (graph_launches) *graph_launches = B->graph_launches;
    if (last_ms) *last_ms = B->last_ms;
    return FDFD_OK;
}

int fdfd_mf_create(fdfd_handle** out, int Nx, int Ny, int Npx, int Npy, double dx, double dy, double L0,
                   double pml_m, double pml_lnR, int nsidebands, int shared_pml, int precision) {
    if (!out) return FDFD_EINVAL;
    *out = nullptr;
    if (nsidebands < 0 || 2 * nsidebands + 1 > MF_MAX_K) return FDFD_EINVAL;
    fdfd_handle* h = nullptr;
    int rc = fdfd_create(&h, Nx, Ny, Npx, Npy, dx, dy, L0, pml_m, pml_lnR, FDFD_TM, precision);
    if (rc != FDFD_OK) return rc;
    MfState* M = new MfState();
    h->mf = M;
    M->s = nsidebands;
    M->K = 2 * nsidebands + 1;
    M->shared_pml = shared_pml != 0;
    h->nsb = M->K;
    auto fail = [&](int code) {
        fdfd_destroy(h);
        return code;
    };
    for (int n = 0; n < M->K; ++n) {
        fdfd_handle* s = nullptr;
        rc = fdfd_create(&s, Nx, Ny, Npx, Npy, dx, dy, L0, pml_m, pml_lnR, FDFD_TM, precision);
        if (rc != FDFD_OK) return fail(rc);
        M->sub.push_back(s);
    }
    M->ev_out.assign(M->K, nullptr);
    if (cudaEventCreateWithFlags(&M->ev_in, cudaEventDisableTiming) != cudaSuccess) return fail(FDFD_ECUDA);
    for (auto& e : M->ev_out)
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return fail(FDFD_ECUDA);
    const long long N = (long long)Nx * Ny;
    rc = dev_alloc(h, (void**)&M->deps, N * sizeof(cplx<double>));
    if (rc != FDFD_OK) return fail(rc);
    if (cudaMemset(M->deps, 0, N * sizeof(cplx<double>)) != cudaSuccess) return fail(FDFD_ECUDA);
    *out = h;
    return FDFD_OK;
}

int fdfd_mf_set_deps(fdfd_handle* h, const double* deps_r) {
    if (!h) return FDFD_EINVAL;
    if (!h->mf) return set_err(h, FDFD_EINVAL, "not a modulated device handle (fdfd_mf_create)");
    if (!deps_r) return set_err(h, FDFD_EINVAL, "deps_r is NULL");
    const long long N = (long long)h->Nx * h->Ny;
    if (const long long k = first_nonfinite(deps_r, 2 * N); k >= 0)
        return set_err(h, FDFD_EINVAL, "deps_r has a non-finite entry at %lld", k / 2);
    CK(cudaMemcpyAsync(h->mf->deps, deps_r, N * sizeof(cplx<double>), cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return FDFD_OK;
}

int fdfd_mf_factor(fdfd_handle* h, double omega, double Omega) {
    if (!h) return FDFD_EINVAL;
    if (!h->mf) return set_err(h, FDFD_EINVAL, "not a modulated device handle (fdfd_mf_create)");
    if (!h->eps_set) return set_err(h, FDFD_EINVAL, "fdfd_set_eps must be called before fdfd_mf_factor");
    if (!(omega > 0) || !std::isfinite(omega) || !std::isfinite(Omega))
        return set_err(h, FDFD_EINVAL, "omega must be positive and finite, Omega finite");
    MfState& M = *h->mf;
    M.omega = omega;
    M.Omega = Omega;
    M.wn.resize(M.K);
    for (int j = 0; j < M.K; ++j) {
        M.wn[j] = omega + Omega * (j - M.s);   // modulation.jl:49
        if (!(M.wn[j] > 0))
            return set_err(h, FDFD_EINVAL, "sideband frequency omega + %d*Omega = %g is not positive", j - M.s, M.wn[j]);
    }
    h->launches = 0;
    h->factored = false;
    auto t0 = std::chrono::steady_clock::now();
    RET(factor_op(h));
    h->mf_factor_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    h->omega = omega;
    return FDFD_OK;
}

int fdfd_mf_solve(fdfd_handle* h, const double* src, double* ez, double* hx, double* hy, fdfd_stats* stats) {
    if (!h) return FDFD_EINVAL;
    if (!h->mf) return set_err(h, FDFD_EINVAL, "not a modulated device handle (fdfd_mf_create)");
    if (!src) return set_err(h, FDFD_EINVAL, "src is NULL");
    if (!h->factored) return set_err(h, FDFD_EINVAL, "fdfd_mf_factor must be called before fdfd_mf_solve");
    auto t0 = std::chrono::steady_clock::now();
    MfState& M = *h->mf;
    const long long N = (long long)h->Nx * h->Ny;
    if (first_nonfinite(src, 2 * N) >= 0) return set_err(h, FDFD_EINVAL, "src has a non-finite entry");
    const size_t bytes = (size_t)N * M.K * sizeof(cplx<double>);
    if (h->io_cap < 4 * bytes) {
        dev_free(h, h->io);
        h->io = nullptr;
        h->io_cap = 0;
        RET(dev_alloc(h, (void**)&h->io, 4 * bytes));
        h->io_cap = 4 * bytes;
    }
    cplx<double>* d_src = h->io;
    cplx<double>* d_hx = h->io + N * M.K;
    cplx<double>* d_hy = h->io + 2 * N * M.K;
    RET(ensure_krylov(h, 1, restart_len(h, 1)));
    CK(cudaMemcpyAsync(d_src, src, N * sizeof(cplx<double>), cudaMemcpyHostToDevice, h->stream));
    cudaEventRecord(h->ev[3], h->stream);
    // b = iω·src in the centre sideband, zero elsewhere (modulation.jl:67-69)
    CK(cudaMemsetAsync(h->kb, 0, bytes, h->stream));
    const zd iw(0, M.omega);
    CK(cudaMemcpyAsync(h->kc, &iw, sizeof(zd), cudaMemcpyHostToDevice, h->stream));
    LAUNCH(vscale_kernel, dim3(ceil_div(N, 256), 1), 256, 0, N, d_src, h->kc, h->kb + (size_t)M.s * N);
    int iters = 0;
    double rel = 0;
    RET(refine_fb(h, 1, &iters, &rel));
    cudaEventRecord(h->ev[4], h->stream);
    // H per sideband with forward differences (modulation.jl:112-113)
    std::vector<zd> coef(2 * M.K);
    const double mu0 = kMU0 * h->L0;
    for (int j = 0; j < M.K; ++j) {
        coef[2 * j] = zd(-0.0, (1.0 / M.wn[j]) / mu0);       // -1/1im/ωₙ/μ₀
        coef[2 * j + 1] = zd(0.0, (-1.0 / M.wn[j]) / mu0);   //  1/1im/ωₙ/μ₀
    }
    CK(cudaMemcpyAsync(h->kc, coef.data(), coef.size() * sizeof(zd), cudaMemcpyHostToDevice, h->stream));
    RecoverArgs ra;
    ra.Nx = h->Nx; ra.Ny = h->Ny; ra.mode = REC_TM_EIGEN;
    ra.idx = 1.0 / h->dx; ra.idy = 1.0 / h->dy; ra.eps0n = kEPS0 * h->L0;
    for (int j = 0; j < M.K; ++j)
        LAUNCH(recover_kernel, dim3(ceil_div(N, 256), 1), 256, 0, ra, M.sub[j]->sf, M.sub[j]->eps,
               h->kx + (size_t)j * N, h->kc + 2 * j, d_hx + (size_t)j * N, d_hy + (size_t)j * N);
    RET(check_launch(h, "recover"));
    cudaEventRecord(h->ev[5], h->stream);
    int rc = FDFD_OK;
    if (ez && cudaMemcpyAsync(ez, h->kx, bytes, cudaMemcpyDeviceToHost, h->stream) != cudaSuccess) rc = FDFD_ECUDA;
    if (hx && cudaMemcpyAsync(hx, d_hx, bytes, cudaMemcpyDeviceToHost, h->stream) != cudaSuccess) rc = FDFD_ECUDA;
    if (hy && cudaMemcpyAsync(hy, d_hy, bytes, cudaMemcpyDeviceToHost, h->stream) != cudaSuccess) rc = FDFD_ECUDA;
    if (cudaStreamSynchronize(h->stream) != cudaSuccess) rc = FDFD_ECUDA;
    if (rc != FDFD_OK) return set_err(h, rc, "copy of fields failed");
    RET(check_device(h, "mf_solve"));
    if (stats) {
        fdfd_handle* s0 = M.sub[0];
        double flops = 0;
        long long bytes_all = h->dev_bytes;
        for (fdfd_handle* s : M.sub) {
            flops += s->last_factor_flops;
            bytes_all += s->dev_bytes;
        }
        stats->iterations = iters;
        stats->nrhs = 1;
        stats->rel_residual = rel;
        stats->t_assemble_ms = 0;
        stats->t_factor_ms = h->mf_factor_ms;
        stats->t_solve_ms = elapsed_ms(h->ev[3], h->ev[4]);
        stats->t_recover_ms = elapsed_ms(h->ev[4], h->ev[5]);
        stats->factor_flops = flops;
        stats->block = s0->map.b;
        stats->nblocks = s0->map.n;
        stats->levels = (int)s0->steps.size() + 1;
        stats->tc_gemm = s0->tc_used;
        stats->device_bytes = bytes_all;
        stats->gpu_launches = h->launches;
        stats->factor_precision = h->fact_prec;
        stats->fp64_fallback = h->fell_back;
        stats->t_total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
    if (!(rel <= h->tol))
        return set_err(h, FDFD_ENOCONV, "refinement stopped at relative residual %.3e > tol %.1e after %d iterations",
                       rel, h->tol, iters);
    return FDFD_OK;
}

// ---- guided modes and mode sources (get_modes, setup_mode!, eigenmode) ------
namespace {

// slice of one Mode (device.jl:124-142): srcpoints = round(width/dh), made odd,
// centred on (ix, iy) across the slice normal; shift σ = (ω n_eff/c₀)² (eigen.jl:23-25)
int mode_job(fdfd_handle* h, const fdfd_mode* md, double omega, ModeJob* J) {
    if (!md) return set_err(h, FDFD_EINVAL, "mode is NULL");
    if (md->normal != FDFD_X && md->normal != FDFD_Y) return set_err(h, FDFD_EINVAL, "mode normal must be FDFD_X or FDFD_Y");
    if (md->pol != FDFD_TM && md->pol != FDFD_TE) return set_err(h, FDFD_EINVAL, "mode polarization must be TM or TE");
    if (!(md->width > 0) || !std::isfinite(md->width) || !std::isfinite(md->neff_re) || !std::isfinite(md->neff_im))
        return set_err(h, FDFD_EINVAL, "mode width must be positive, n_eff finite");
    if (!(omega > 0) || !std::isfinite(omega)) return set_err(h, FDFD_EINVAL, "omega must be positive and finite");
    if (md->ix < 0 || md->ix >= h->Nx || md->iy < 0 || md->iy >= h->Ny)
        return set_err(h, FDFD_EINVAL, "mode centre (%d, %d) outside the grid", md->ix, md->iy);
    const bool xn = md->normal == FDFD_X;
    const double dh = xn ? h->dy : h->dx;
    long long pts = (long long)std::nearbyint(md->width / dh);   // round half to even, as Julia's round
    if (pts % 2 == 0) pts += 1;
    const long long M = (pts - 1) / 2;
    if (pts < 3 || pts > FDFD_MODE_MAX_POINTS)
        return set_err(h, FDFD_EINVAL, "mode slice of %lld cells (3..%d)", pts, FDFD_MODE_MAX_POINTS);
    const int c = xn ? md->iy : md->ix, lim = xn ? h->Ny : h->Nx;
    if (c - M < 0 || c + M >= lim) return set_err(h, FDFD_EINVAL, "mode slice leaves the grid");
    J->pol = md->pol;
    J->n = (int)pts;
    J->k0 = xn ? md->ix + (long long)h->Nx * (c - M) : (c - M) + (long long)h->Nx * md->iy;
    J->stride = xn ? h->Nx : 1;
    J->dh = dh;
    J->omega = omega;
    const double k = omega / (std::sqrt(1.0 / kEPS0 / kMU0) / h->L0);
    const zd sb = zd(k * md->neff_re, k * md->neff_im);
    const zd sg = sb * sb;
    J->sig_re = sg.real();
    J->sig_im = sg.imag();
    J->out_off = 0;
    J->pad = 0;
    return FDFD_OK;
}

// solves the jobs (one per (frequency, mode)); optionally builds nw source arrays
int run_modes(fdfd_handle* h, std::vector<ModeJob>& jobs, const std::vector<int>& job_start, bool want_src,
              std::vector<zd>* beta, std::vector<zd>* vecs, double* src_host) {
    if (!h->eps_set) return set_err(h, FDFD_EINVAL, "fdfd_set_eps must be called before the mode solve");
    const int nj = (int)jobs.size();
    const int nw = (int)job_start.size() - 1;
    int tot = 0, nmax = 0;
    for (ModeJob& J : jobs) {
        J.out_off = tot;
        tot += J.n;
        nmax = std::max(nmax, J.n);
    }
    const long long N = (long long)h->Nx * h->Ny;
    auto al = [](size_t b) { return (b + 255) / 256 * 256; };
    const size_t o_jobs = 0, o_start = al(o_jobs + nj * sizeof(ModeJob)), o_beta = al(o_start + (nw + 1) * sizeof(int)),
                 o_it = al(o_beta + nj * sizeof(zd)), o_vec = al(o_it + nj * sizeof(int)),
                 o_src = al(o_vec + (size_t)tot * sizeof(zd)),
                 need = o_src + (want_src ? (size_t)nw * N * sizeof(zd) : 0);
    if (h->mode_cap < need) {
        dev_free(h, h->mode_buf);
        h->mode_buf = nullptr;
        h->mode_cap = 0;
        RET(dev_alloc(h, (void**)&h->mode_buf, need));
        h->mode_cap = need;
    }
    unsigned char* B = h->mode_buf;
    CK(cudaMemcpyAsync(B + o_jobs, jobs.data(), nj * sizeof(ModeJob), cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(B + o_start, job_start.data(), (nw + 1) * sizeof(int), cudaMemcpyHostToDevice, h->stream));
    int rc = launch_modes(h->stream, nj, nmax, (const ModeJob*)(B + o_jobs), h->eps, kEPS0 * h->L0, kMU0 * h->L0,
                          (cplx<double>*)(B + o_beta), (cplx<double>*)(B + o_vec), (int*)(B + o_it), h->derr);
    h->launches++;
    if (rc != 0) return set_err(h, FDFD_ECUDA, "mode kernel launch: %s", cudaGetErrorString((cudaError_t)rc));
    if (want_src) {
        CK(cudaMemsetAsync(B + o_src, 0, (size_t)nw * N * sizeof(zd), h->stream));
        launch_mode_src(h->stream, nw, (const ModeJob*)(B + o_jobs), (const int*)(B + o_start),
                        (const cplx<double>*)(B + o_vec), N, (cplx<double>*)(B + o_src));
        h->launches++;
        RET(check_launch(h, "mode sources"));
        CK(cudaMemcpyAsync(src_host, B + o_src, (size_t)nw * N * sizeof(zd), cudaMemcpyDeviceToHost, h->stream));
    }
    std::vector<int> its(nj);
    CK(cudaMemcpyAsync(its.data(), B + o_it, nj * sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    if (beta) {
        beta->resize(nj);
        CK(cudaMemcpyAsync(beta->data(), B + o_beta, nj * sizeof(zd), cudaMemcpyDeviceToHost, h->stream));
    }
    if (vecs) {
        vecs->resize(tot);
        CK(cudaMemcpyAsync(vecs->data(), B + o_vec, (size_t)tot * sizeof(zd), cudaMemcpyDeviceToHost, h->stream));
    }
    RET(check_device(h, "mode solve"));   // synchronises
    for (int j = 0; j < nj; ++j)
        if (its[j] < 0)
            return set_err(h, FDFD_ENOCONV, "mode job %d: inverse iteration did not converge in %d steps", j, -its[j]);
    return FDFD_OK;
}

}  // namespace

int fdfd_get_mode(fdfd_handle* h, double omega, const fdfd_mode* mode, int cap, double* beta, double* vec,
                  int* npts) {
    if (!h) return FDFD_EINVAL;
    if (!beta || !vec || !npts) return set_err(h, FDFD_EINVAL, "fdfd_get_mode: NULL argument");
    std::vector<ModeJob> jobs(1);
    RET(mode_job(h, mode, omega, &jobs[0]));
    *npts = jobs[0].n;
    if (cap < jobs[0].n) return set_err(h, FDFD_EINVAL, "vec holds %d values, the slice has %d", cap, jobs[0].n);
    std::vector<zd> b, v;
    RET(run_modes(h, jobs, std::vector<int>{0, 1}, false, &b, &v, nullptr));
    beta[0] = b[0].real();
    beta[1] = b[0].imag();
    memcpy(vec, v.data(), v.size() * sizeof(zd));
    return FDFD_OK;
}

int fdfd_mode_sources(fdfd_handle* h, int nw, const double* omegas, int nmodes, const fdfd_mode* modes, double* src) {
    if (!h) return FDFD_EINVAL;
    if (nw < 1 || nmodes < 1 || !omegas || !modes || !src)
        return set_err(h, FDFD_EINVAL, "fdfd_mode_sources: invalid arguments");
    std::vector<ModeJob> jobs((size_t)nw * nmodes);
    std::vector<int> start(nw + 1);
    for (int w = 0; w < nw; ++w) {
        start[w] = w * nmodes;
        for (int m = 0; m < nmodes; ++m) RET(mode_job(h, &modes[m], omegas[w], &jobs[(size_t)w * nmodes + m]));
    }
    start[nw] = nw * nmodes;
    return run_modes(h, jobs, start, true, nullptr, nullptr, src);
}

// ---- Poynting flux (src/flux.jl) ------------------------------------------------
int fdfd_poynting_device(fdfd_handle* h, int pol, const double* d_f1, const double* d_f2, const double* d_f3,
                         double* d_Sx, double* d_Sy) {
    if (!h) return FDFD_EINVAL;
    if (pol != FDFD_TM && pol != FDFD_TE) return set_err(h, FDFD_EINVAL, "pol must be FDFD_TM or FDFD_TE");
    if (!d_f1 || !d_f2 || !d_f3 || !d_Sx || !d_Sy) return set_err(h, FDFD_EINVAL, "fdfd_poynting: NULL argument");
    launch_poynting(h->stream, h->Nx, h->Ny, pol, (const cplx<double>*)d_f1, (const cplx<double>*)d_f2,
                    (const cplx<double>*)d_f3, d_Sx, d_Sy);
    h->launches++;
    RET(check_launch(h, "poynting"));
    CK(cudaStreamSynchronize(h->stream));
    return FDFD_OK;
}

int fdfd_poynting(fdfd_handle* h, int pol, const double* f1, const double* f2, const double* f3, double* Sx,
                  double* Sy) {
    if (!h) return FDFD_EINVAL;
    if (!f1 || !f2 || !f3 || !Sx || !Sy) return set_err(h, FDFD_EINVAL, "fdfd_poynting: NULL argument");
    const long long N = (long long)h->Nx * h->Ny;
    const size_t fb = (size_t)N * sizeof(cplx<double>), sb = (size_t)N * sizeof(double);
    if (h->io_cap < 3 * fb + 2 * sb) {
        dev_free(h, h->io);
        h->io = nullptr;
        h->io_cap = 0;
        RET(dev_alloc(h, (void**)&h->io, 3 * fb + 2 * sb));
        h->io_cap = 3 * fb + 2 * sb;
    }
    unsigned char* B = reinterpret_cast<unsigned char*>(h->io);
    CK(cudaMemcpyAsync(B, f1, fb, cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(B + fb, f2, fb, cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(B + 2 * fb, f3, fb, cudaMemcpyHostToDevice, h->stream));
    double* dS = reinterpret_cast<double*>(B + 3 * fb);
    RET(fdfd_poynting_device(h, pol, (const double*)B, (const double*)(B + fb), (const double*)(B + 2 * fb), dS,
                             dS + N));
    CK(cudaMemcpyAsync(Sx, dS, sb, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(Sy, dS + N, sb, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return FDFD_OK;
}

int fdfd_flux_integral(fdfd_handle* h, int pol, const double* f1, const double* f3, int normal, int nlines,
                       const int* lines, double* flux) {
    if (!h) return FDFD_EINVAL;
    if (pol != FDFD_TM && pol != FDFD_TE) return set_err(h, FDFD_EINVAL, "pol must be FDFD_TM or FDFD_TE");
    if (normal == FDFD_Y)   // flux.jl:59-66
        return set_err(h, FDFD_EINVAL, "%s normal %s calculation not yet implemented", "y",
                       pol == FDFD_TM ? "TM" : "TE");
    if (normal != FDFD_X) return set_err(h, FDFD_EINVAL, "normal must be FDFD_X or FDFD_Y");
    if (!f1 || !f3 || !lines || !flux || nlines < 1) return set_err(h, FDFD_EINVAL, "fdfd_flux_integral: bad argument");
    for (int l = 0; l < nlines; ++l) {
        const int x = lines[3 * l], y0 = lines[3 * l + 1], y1 = lines[3 * l + 2];
        if (x < 0 || x + 1 >= h->Nx || y0 < 0 || y1 >= h->Ny || y0 > y1)
            return set_err(h, FDFD_EINVAL, "flux line %d (column %d, rows %d..%d) outside the grid", l, x, y0, y1);
    }
    const long long N = (long long)h->Nx * h->Ny;
    const size_t fb = (size_t)N * sizeof(cplx<double>);
    const size_t need = 2 * fb + (size_t)nlines * (sizeof(int3) + sizeof(double)) + 64;
    if (h->io_cap < need) {
        dev_free(h, h->io);
        h->io = nullptr;
        h->io_cap = 0;
        RET(dev_alloc(h, (void**)&h->io, need));
        h->io_cap = need;
    }
    unsigned char* B = reinterpret_cast<unsigned char*>(h->io);
    int3* dl = reinterpret_cast<int3*>(B + 2 * fb);
    double* dout = reinterpret_cast<double*>(B + ((2 * fb + (size_t)nlines * sizeof(int3) + 15) / 16 * 16));
    CK(cudaMemcpyAsync(B, f1, fb, cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(B + fb, f3, fb, cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(dl, lines, (size_t)nlines * sizeof(int3), cudaMemcpyHostToDevice, h->stream));
    launch_flux_lines(h->stream, nlines, h->Nx, pol, h->dy, dl, (const cplx<double>*)B,
                      (const cplx<double>*)(B + fb), dout);
    h->launches++;
    RET(check_launch(h, "flux lines"));
    CK(cudaMemcpyAsync(flux, dout, (size_t)nlines * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return FDFD_OK;
}

// ---- χ³ nonlinear driven solve (src/solver/nonlinear.jl) -------------------------
namespace {

double vnorm(fdfd_handle* h, const cplx<double>* x, long long n) {
    const int nb = h->num_sms;   // one partial per SM
    if (ensure_part(h, (size_t)nb * 2) != FDFD_OK || ensure_red(h, 2) != FDFD_OK) return NAN;
    vdots_kernel<<<dim3(nb, 1), 256, 0, h->stream>>>(n, 1, x, 0, x, h->part);
    reduce_partials_kernel<<<1, 256, 0, h->stream>>>(h->part, nb, 2, h->red);
    h->launches += 2;
    double v[2] = {0, 0};
    if (cudaMemcpyAsync(v, h->red, sizeof v, cudaMemcpyDeviceToHost, h->stream) != cudaSuccess ||
        cudaStreamSynchronize(h->stream) != cudaSuccess)
        return NAN;
    return std::sqrt(std::max(v[0], 0.0));
}

// restores the handle's single-system state on every exit of fdfd_chi3_solve
struct NlGuard {
    fdfd_handle* h;
    double tol;
    ~NlGuard() {
        h->nl_mode = 0;
        h->nsb = 1;
        h->tol = tol;
        h->warm_start = false;
    }
};

}  // namespace

int fdfd_chi3_solve(fdfd_handle* h, const double* chi, const double* src, int method, double tol, int maxit,
                    double* f1, double* f2, double* f3, double* err_hist, int* nerr, fdfd_stats* stats) {
    if (!h) return FDFD_EINVAL;
    if (h->mf) return set_err(h, FDFD_EINVAL, "fdfd_chi3_solve: not defined for a modulated device");
    if (!h->factored || h->op != OP_TM_DRIVEN)
        return set_err(h, FDFD_EINVAL, "fdfd_chi3_solve needs a factored TM driven operator (fdfd_factor, FDFD_TM)");
    if (!chi || !src) return set_err(h, FDFD_EINVAL, "fdfd_chi3_solve: NULL argument");
    if (method != FDFD_CHI3_NEWTON && method != FDFD_CHI3_BORN)
        return set_err(h, FDFD_EINVAL, "method must be FDFD_CHI3_NEWTON or FDFD_CHI3_BORN");
    if (!(tol > 0) || maxit < 0) return set_err(h, FDFD_EINVAL, "tol must be positive, maxit >= 0");
    const long long N = (long long)h->Nx * h->Ny;
    if (const long long k = first_nonfinite(chi, N); k >= 0)
        return set_err(h, FDFD_EINVAL, "chi has a non-finite entry at %lld", k);
    if (first_nonfinite(src, 2 * N) >= 0) return set_err(h, FDFD_EINVAL, "src has a non-finite entry");
    auto t0 = std::chrono::steady_clock::now();
    const size_t vb = (size_t)N * sizeof(cplx<double>);
    // scratch: d1 | d2 | tmp (2N) | Z (2N) | B (N) | coeff (N doubles)
    if (!h->nl_d1) {
        RET(dev_alloc(h, (void**)&h->nl_d1, 8 * vb + (size_t)N * sizeof(double)));
        h->nl_d2 = h->nl_d1 + N;
        h->nl_tmp = h->nl_d2 + N;
    }
    cplx<double>* Z = h->nl_tmp + 2 * N;
    cplx<double>* B = Z + 2 * N;
    double* dco = reinterpret_cast<double*>(B + N);
    if (h->io_cap < 4 * vb) {
        dev_free(h, h->io);
        h->io = nullptr;
        h->io_cap = 0;
        RET(dev_alloc(h, (void**)&h->io, 4 * vb));
        h->io_cap = 4 * vb;
    }
    cplx<double>* d_src = h->io;
    // coeff = ω²ϵ₀·3χ/L₀ (nonlinear.jl:71, ϵ₀ normalised)
    std::vector<double> coeff(N);
    const double w = h->omega;
    for (long long k = 0; k < N; ++k) coeff[k] = w * w * (kEPS0 * h->L0) * 3 * chi[k] / h->L0;
    CK(cudaMemcpyAsync(dco, coeff.data(), N * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(d_src, src, vb, cudaMemcpyHostToDevice, h->stream));
    NlGuard guard{h, h->tol};
    // inner linear solves a decade below the nonlinear tolerance (the reference solves them directly)
    h->tol = std::max(std::min(h->tol, 0.1 * tol), 1e-14);
    h->nl_mode = 0;
    h->nsb = 1;
    cudaEventRecord(h->ev[3], h->stream);
    RET(ensure_krylov(h, 1, restart_len(h, 1)));
    RET(scale_vec(h, d_src, std::vector<zd>(1, zd(0, w)), 1, h->kb));   // b = iω·src
    CK(cudaMemcpyAsync(B, h->kb, vb, cudaMemcpyDeviceToDevice, h->stream));
    int iters = 0, it = 0;
    double rel = 0;
    RET(refine_fb(h, 1, &it, &rel));   // linear solve (nonlinear.jl:66-69)
    iters += it;
    CK(cudaMemcpyAsync(Z, h->kx, vb, cudaMemcpyDeviceToDevice, h->stream));
    std::vector<double> errs(1, 1.0);
    const int nb = ceil_div(N, 256);
    if (method == FDFD_CHI3_BORN) {
        // _doborn (nonlinear.jl:92-106)
        for (int i = 1; errs.back() > tol && i <= maxit; ++i) {
            LAUNCH(chi3_diag_kernel, nb, 256, 0, N, 1, dco, Z, h->nl_d1, h->nl_d2);
            h->nl_mode = 1;
            h->warm_start = true;   // kx holds the previous iterate
            RET(refine_fb(h, 1, &it, &rel));
            iters += it;
            CK(cudaMemcpyAsync(h->nl_tmp, h->kx, vb, cudaMemcpyDeviceToDevice, h->stream));
            LAUNCH(vaxpy_kernel, nb, 256, 0, N, -1.0, Z, h->nl_tmp);
            const double nz = vnorm(h, Z, N), nd = vnorm(h, h->nl_tmp, N);
            CK(cudaMemcpyAsync(Z, h->kx, vb, cudaMemcpyDeviceToDevice, h->stream));
            errs.push_back(nd / nz);
        }
    } else {
        // _donewton (nonlinear.jl:108-129) on [e; conj(e)]: J δ = [F; conj F], e ← e − δ.  With
        // r = b − (A + diag(coeff|e|²)) e = −F the system is solved for δ' = −δ and e += δ'.
        LAUNCH(vconj_kernel, nb, 256, 0, N, Z, Z + N);
        h->nsb = 2;
        RET(ensure_krylov(h, 1, restart_len(h, 1)));
        for (int i = 1; errs.back() > tol && i <= maxit; ++i) {
            LAUNCH(chi3_diag_kernel, nb, 256, 0, N, 1, dco, Z, h->nl_d1, h->nl_d2);
            LAUNCH(residual_nl_kernel, dim3(nb, 1), 256, 0, h->Nx, h->Ny, 1, h->st, h->nl_d1, h->nl_d2, Z, B, h->kb,
                   nullptr);
            LAUNCH(vconj_kernel, nb, 256, 0, N, h->kb, h->kb + N);
            LAUNCH(chi3_diag_kernel, nb, 256, 0, N, 2, dco, Z, h->nl_d1, h->nl_d2);
            h->nl_mode = 2;
            RET(refine_fb(h, 1, &it, &rel));
            iters += it;
            const double nz = vnorm(h, Z, 2 * N), nd = vnorm(h, h->kx, 2 * N);
            LAUNCH(vaxpy_kernel, ceil_div(2 * N, 256), 256, 0, 2 * N, 1.0, h->kx, Z);
            errs.push_back(nd / nz);
        }
    }
    RET(check_launch(h, "chi3"));
    cudaEventRecord(h->ev[4], h->stream);
    // H recovery (nonlinear.jl:82-83): the driven TM recovery of the final field
    std::vector<zd> coef(2);
    const double mu0 = kMU0 * h->L0;
    coef[0] = zd(-0.0, (1.0 / w) / mu0);
    coef[1] = zd(0.0, (-1.0 / w) / mu0);
    CK(cudaMemcpyAsync(h->kc, coef.data(), 2 * sizeof(zd), cudaMemcpyHostToDevice, h->stream));
    RecoverArgs ra;
    ra.Nx = h->Nx; ra.Ny = h->Ny; ra.mode = REC_TM_DRIVEN;
    ra.idx = 1.0 / h->dx; ra.idy = 1.0 / h->dy; ra.eps0n = kEPS0 * h->L0;
    LAUNCH(recover_kernel, dim3(nb, 1), 256, 0, ra, h->sf, h->eps, Z, h->kc, h->io + N, h->io + 2 * N);
    RET(check_launch(h, "recover"));
    if (f1) CK(cudaMemcpyAsync(f1, Z, vb, cudaMemcpyDeviceToHost, h->stream));
    if (f2) CK(cudaMemcpyAsync(f2, h->io + N, vb, cudaMemcpyDeviceToHost, h->stream));
    if (f3) CK(cudaMemcpyAsync(f3, h->io + 2 * N, vb, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    RET(check_device(h, "chi3"));
    if (err_hist)
        for (size_t i = 0; i < errs.size() && i <= (size_t)maxit; ++i) err_hist[i] = errs[i];
    if (nerr) *nerr = (int)errs.size();
    if (stats) {
        stats->iterations = iters;
        stats->nrhs = 1;
        stats->rel_residual = rel;
        stats->t_assemble_ms = elapsed_ms(h->ev[0], h->ev[1]);
        stats->t_factor_ms = elapsed_ms(h->ev[1], h->ev[2]);
        stats->t_solve_ms = elapsed_ms(h->ev[3], h->ev[4]);
        stats->t_recover_ms = 0;
        stats->factor_flops = h->last_factor_flops;
        stats->block = h->map.b;
        stats->nblocks = h->map.n;
        stats->levels = (int)h->steps.size() + 1;
        stats->tc_gemm = h->tc_used;
        stats->device_bytes = h->dev_bytes;
        stats->gpu_launches = h->launches;
        stats->factor_precision = h->fact_prec;
        stats->fp64_fallback = h->fell_back;
        stats->t_total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
    if (errs.back() > tol)
        return set_err(h, FDFD_ENOCONV, "chi3 %s iteration stopped at step error %.3e > tol %.1e after %d steps",
                       method == FDFD_CHI3_BORN ? "Born" : "Newton", errs.back(), tol, (int)errs.size() - 1);
    return FDFD_OK;
}

}  // extern "C"

namespace {

// device time (ms) of fn() on the handle's stream: one untimed run, then the mean of three
template <typename F> int time_launch(fdfd_handle* h, F fn, double* ms) {
    RET(fn());
    CK(cudaEventRecord(h->ev[5], h->stream));
    for (int r = 0; r < 3; ++r) RET(fn());
    CK(cudaEventRecord(h->ev[6], h->stream));
    CK(cudaEventSynchronize(h->ev[6]));
    float t = 0;
    CK(cudaEventElapsedTime(&t, h->ev[5], h->ev[6]));
    *ms = t / 3.0;
    return FDFD_OK;
}

// zeroes a pool (so that the candidates run on finite data)
template <typename T> int zero_pool(fdfd_handle* h, const Pool<T>& P) {
    if (P.base) CK(cudaMemsetAsync(P.base, 0, (size_t)P.slot_elems() * P.count * sizeof(T), h->stream));
    return FDFD_OK;
}

// The autotuner: every tensor-core GEMM shape of the factorization and every
// sweep product of the plan is timed with each candidate launch shape, on the
// handle's own storage and job lists (zeroed first, row maps the identity), and
// the fastest is recorded for the handle's later launches.
template <typename T> int autotune_impl(fdfd_handle* h) {
    RET(alloc_factor<T>(h));
    const int nrhs_max = std::min(8, gemv_max_rhs<T>(h->map.b));
    RET(alloc_vectors<T>(h, nrhs_max));
    FactorStore<T>& F = store<T>(h);
    const int b = h->map.b, E = (int)h->steps.size();
    RET(zero_pool<T>(h, F.D)); RET(zero_pool<T>(h, F.C)); RET(zero_pool<T>(h, F.X));
    RET(zero_pool<T>(h, F.GP)); RET(zero_pool<T>(h, F.RP)); RET(zero_pool<T>(h, F.Tg));
    launch_perm_init(h->stream, 2 * h->max_ne, F.rowsrc, b);   // in-range rows for the β gathers
    h->launches++;
    h->tune_gemm.clear();
    h->tune_gemv.clear();
    std::string log;
    char line[256];
    const bool prof = h->prof_on;
    h->prof_on = false;
    // ---- tensor-core GEMM tile widths
    if (sizeof(T) == 4 && F.tc_ok) {
        auto tune = [&](int M, int N, int K, int njobs, int presplit, const char* role, auto launch) -> int {
            const auto key = std::make_tuple(M, N, K, njobs, presplit);
            if (njobs == 0 || h->tune_gemm.count(key)) return FDFD_OK;
            int best = 0;
            double tbest = 1e30;
            std::string cand;
            for (int bn : {64, 128, TC_BN128_TWO, 256}) {
                if ((bn == 256 && N <= 128) || (bn != 64 && N <= 64)) continue;   // no wider than the product
                h->force_bn = bn;
                double ms = 0;
                const int rc = time_launch(h, launch, &ms);
                h->force_bn = 0;
                RET(rc);
                snprintf(line, sizeof line, " %s:%.4f", tc_tile_name(bn), ms);
                cand += line;
                if (ms < tbest) { tbest = ms; best = bn; }
            }
            h->tune_gemm[key] = best;
            snprintf(line, sizeof line, "gemm %-10s M=%d N=%d K=%d jobs=%d -> BN=%s  (ms%s)\n", role, M, N, K, njobs,
                     tc_tile_name(best), cand.c_str());
            log += line;
            return FDFD_OK;
        };
        const int nb = panel_nb<T>(b);
        for (int e = 2; e <= E; ++e) {
            const StepJobs& S = h->sj[e];
            const int ne = S.ne;
            RET(tune(b, b, b, 2 * ne, 0, "schur-2n", [&] {
                return gemm<T>(h, P_C, P_D, P_X, J<int>(h, S.xt_a), J<int>(h, S.xt_b), J<int>(h, S.xt_c), nullptr, 0,
                               2 * ne, b, b, b, (T)1, 0, 0, 0);
            }));
            RET(tune(b, b, b, ne, 0, "schur-n", [&] {
                return gemm<T>(h, P_C, P_X, P_D, J<int>(h, S.dp_a), J<int>(h, S.dp_b), J<int>(h, S.dp_c), nullptr, 0,
                               ne, b, b, b, (T)-1, 1, 0, 0);
            }));
            const int w1 = std::min(nb, b - nb);
            RET(tune(b, w1, nb, ne, 1, "gj-narrow", [&] {
                return gemm<T>(h, P_GP, P_RP, P_TG, F.gj_slots, F.gj_slots, J<int>(h, S.iota), nullptr, 0, ne, b, w1,
                               nb, (T)1, 1, 0, nb, P_D, J<int>(h, S.elim), F.rowsrc, -1, 0.0, h->stream, nb);
            }));
            RET(tune(b, b, nb, ne, 1, "gj-wide", [&] {
                return gemm<T>(h, P_GP, P_RP, P_TG, F.gj_slots, F.gj_slots, J<int>(h, S.iota), nullptr, 0, ne, b, b,
                               nb, (T)1, 1, 0, nb, P_D, J<int>(h, S.elim), F.rowsrc, -1, 0.0, h->stream, 0, nb, w1);
            }));
        }
        // the final pair's single-matrix products
        RET(tune(b, b, b, 1, 0, "schur-1", [&] {
            return gemm<T>(h, P_C, P_D, P_X, J<int>(h, h->fin_xt_a), J<int>(h, h->fin_xt_b), J<int>(h, h->fin_xt_c),
                           nullptr, 0, 1, b, b, b, (T)1, 0, 0, 0);
        }));
    }
    // ---- sweep product launch shapes
    auto tune_v = [&](int tr, int p1, int p2, const T* V1, const T* V2, const T* Y0, T* Y, const int4* jobs,
                      const int2* yjobs, int njobs, int nblk, int nrhs, const char* role) -> int {
        const auto key = std::make_tuple(tr, njobs, nblk > njobs ? 2 : 1, nrhs);
        if (njobs == 0 || h->tune_gemv.count(key)) return FDFD_OK;
        int best = 0;
        double tbest = 1e30;
        std::string cand;
        const int cands[2][6] = {{1, 2, 4, -2, -4, -8}, {8, 16, 32, 0, 0, 0}};
        for (int c : cands[tr]) {
            if (c == 0) continue;
            h->force_shape = c;
            double ms = 0;
            const int rc = time_launch(h, [&] { return gemv<T>(h, tr, p1, p2, V1, V2, Y0, Y, jobs, yjobs, njobs,
                                                               nblk, nrhs, (T)1); }, &ms);
            h->force_shape = 0;
            RET(rc);
            snprintf(line, sizeof line, " %d:%.4f", c, ms);
            cand += line;
            if (ms < tbest) { tbest = ms; best = c; }
        }
        h->tune_gemv[key] = best;
        snprintf(line, sizeof line, "gemv %-10s %s jobs=%d rhs=%d -> %s=%d  (ms%s)\n", role, tr ? "T" : "N", njobs,
                 nrhs, tr ? "og" : "rpw", best, cand.c_str());
        log += line;
        return FDFD_OK;
    };
    CK(cudaMemsetAsync(F.rv, 0, (size_t)h->map.n * F.vec_nrhs * 2 * h->map.ld * sizeof(T), h->stream));
    CK(cudaMemsetAsync(F.xv, 0, (size_t)h->map.n * F.vec_nrhs * 2 * h->map.ld * sizeof(T), h->stream));
    const int rhs_set[2] = {1, nrhs_max};
    for (int nr : rhs_set) {
        for (int e = 1; e <= E; ++e) {
            const StepJobs& S = h->sj[e];
            if (e == 1 && !(F.trifac && h->tri_sweep && !h->level1_gj))
                RET(tune_v(0, P_D, P_D, F.rv, F.rv, nullptr, F.xv, J<int4>(h, S.fwd1), J<int2>(h, S.fwd1y), S.ne, S.ne,
                           nr, "inverse"));
            if (e >= 2) {
                RET(tune_v(0, P_D, P_D, F.rv, F.rv, nullptr, F.xv, J<int4>(h, S.fwd1), J<int2>(h, S.fwd1y), S.ne, S.ne,
                           nr, "inverse"));
                RET(tune_v(0, P_C, P_C, F.xv, F.xv, F.rv, F.rv, J<int4>(h, S.f2), J<int2>(h, S.f2y), S.nf2, S.nf2b,
                           nr, "coupling"));
                RET(tune_v(1, P_X, P_X, F.xv, F.xv, F.xv, F.xv, J<int4>(h, S.bw), J<int2>(h, S.bwy), S.ne, 2 * S.ne,
                           nr, "back"));
            }
        }
        RET(tune_v(0, P_D, P_D, F.rv, F.rv, nullptr, F.xv, J<int4>(h, h->fin_g1), J<int2>(h, h->fin_g1y), 1, 1, nr,
                   "inverse"));
        RET(tune_v(1, P_X, P_X, F.xv, F.xv, F.xv, F.xv, J<int4>(h, h->fin_bx), J<int2>(h, h->fin_bxy), 1, 1, nr,
                   "back"));
    }
    h->prof_on = prof;
    CK(cudaStreamSynchronize(h->stream));
    RET(check_device(h, "autotune"));
    h->tune_log = log;
    h->factored = false;   // the factor storage now holds the candidates' output
    return FDFD_OK;
}

}  // namespace

extern "C" {

int fdfd_autotune(fdfd_handle* h) {
    if (!h) return FDFD_EINVAL;
    if (h->mf) return set_err(h, FDFD_EINVAL, "fdfd_autotune: tune the sideband handles of a modulated device");
    h->cfg_gen++;   // new launch shapes
    return h->precision == FDFD_PREC_FP64 ? autotune_impl<double>(h) : autotune_impl<float>(h);
}

int fdfd_get_tuning(const fdfd_handle* h, char* buf, int cap) {
    if (!h || cap < 0 || (cap > 0 && !buf)) return -1;
    const int n = (int)h->tune_log.size();
    if (cap > 0) {
        const int m = std::min(n, cap - 1);
        memcpy(buf, h->tune_log.data(), (size_t)m);
        buf[m] = 0;
    }
    return n;
}

int fdfd_set_profiling(fdfd_handle* h, int on) {
    if (!h) return FDFD_EINVAL;
    prof_collect(h);
    h->prof_on = on != 0;
    memset(&h->prof_tot, 0, sizeof h->prof_tot);
    return FDFD_OK;
}

int fdfd_get_profile(fdfd_handle* h, fdfd_profile* out) {
    if (!h || !out) return FDFD_EINVAL;
    prof_collect(h);
    *out = h->prof_tot;
    return FDFD_OK;
}

int fdfd_get_stencil(fdfd_handle* h, double* out) {
    if (!h || !out) return FDFD_EINVAL;
    if (!h->factored) return set_err(h, FDFD_EINVAL, "no assembled operator");
    if (h->mf) return set_err(h, FDFD_EINVAL, "modulated device: one stencil per sideband, none exported");
    long long N = (long long)h->Nx * h->Ny;
    CK(cudaMemcpyAsync(out, h->st, 5 * N * sizeof(cplx<double>), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return FDFD_OK;
}

int fdfd_apply(fdfd_handle* h, const double* x, int nrhs, double* y) {
    if (!h || !x || !y || nrhs < 1) return FDFD_EINVAL;
    if (!h->factored) return set_err(h, FDFD_EINVAL, "no assembled operator");
    if (h->mf && nrhs != 1) return set_err(h, FDFD_EINVAL, "modulated device: nrhs must be 1");
    long long N = vlen(h);
    size_t bytes = (size_t)N * nrhs * sizeof(cplx<double>);
    cplx<double>* buf = nullptr;
    RET(dev_alloc(h, (void**)&buf, 2 * bytes));
    int rc = FDFD_OK;
    if (cudaMemcpyAsync(buf, x, bytes, cudaMemcpyHostToDevice, h->stream) != cudaSuccess) rc = FDFD_ECUDA;
    if (rc == FDFD_OK) rc = residual(h, buf, nullptr, buf + N * nrhs, nrhs, nullptr);
    if (rc == FDFD_OK && cudaMemcpyAsync(y, buf + N * nrhs, bytes, cudaMemcpyDeviceToHost, h->stream) != cudaSuccess)
        rc = FDFD_ECUDA;
    cudaStreamSynchronize(h->stream);
    dev_free(h, buf);
    return rc == FDFD_ECUDA ? set_err(h, rc, "fdfd_apply copy failed") : rc;
}

}  // extern "C"

namespace {

// Shared core of fdfd_adjoint (objective form: g = m, the gradient of J = |mᵀE|²)
// and fdfd_adjoint_vjp (g is the caller's cotangent, grad_k = -Re(ω²ϵ₀ λ_k E_k)).
int adjoint_core(fdfd_handle* h, const double* src, const double* mvec, bool objective, double* J, double* grad,
                 double* ez, fdfd_stats* stats) {
    const char* fn = objective ? "fdfd_adjoint" : "fdfd_adjoint_vjp";
    if (!h) return FDFD_EINVAL;
    if (h->mf) return set_err(h, FDFD_EINVAL, "%s: not defined for a modulated device", fn);
    if (!src || !mvec || (objective && !J) || !grad) return set_err(h, FDFD_EINVAL, "%s: NULL argument", fn);
    if (!h->factored || h->op != OP_TM_DRIVEN)
        return set_err(h, FDFD_EINVAL, "%s needs a factored TM driven operator (fdfd_factor, FDFD_TM)", fn);
    auto t0 = std::chrono::steady_clock::now();
    const long long N = (long long)h->Nx * h->Ny;
    if (first_nonfinite(src, 2 * N) >= 0 || first_nonfinite(mvec, 2 * N) >= 0)
        return set_err(h, FDFD_EINVAL, "%s: non-finite input", fn);
    const size_t bytes = (size_t)N * sizeof(cplx<double>);
    RET(ensure_krylov(h, 2, restart_len(h, 2)));
    if (h->io_cap < 4 * bytes) {
        dev_free(h, h->io);
        h->io = nullptr;
        h->io_cap = 0;
        RET(dev_alloc(h, (void**)&h->io, 4 * bytes));
        h->io_cap = 4 * bytes;
    }
    cplx<double>* d_src = h->io;
    cplx<double>* d_m = h->io + N;
    cplx<double>* d_lam = h->io + 2 * N;
    double* d_grad = reinterpret_cast<double*>(h->io + 3 * N);
    CK(cudaMemcpyAsync(d_src, src, bytes, cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(d_m, mvec, bytes, cudaMemcpyHostToDevice, h->stream));
    cudaEventRecord(h->ev[3], h->stream);
    // right-hand sides: E solves A E = iω·src; μ solves A μ = P⁻¹ m, so that
    // λ = P μ solves Aᵀ λ = m (P·A is complex symmetric for P = diag(s_xf s_yf)).
    std::vector<zd> iw(1, zd(0, h->omega));
    RET(scale_vec(h, d_src, iw, 1, h->kb));
    const int nb = ceil_div(N, 256);
    LAUNCH(pscale_kernel, nb, 256, 0, h->Nx, h->Ny, h->sf, 0, d_m, h->kb + N);
    int iters = 0;
    double rel = 0;
    RET(refine_fb(h, 2, &iters, &rel));
    LAUNCH(pscale_kernel, nb, 256, 0, h->Nx, h->Ny, h->sf, 1, h->kx + N, d_lam);
    zd s(0, 0);
    const double w2e0 = h->omega * h->omega * kEPS0 * h->L0;
    zd coef(0.5 * w2e0, 0.0);   // vjp: grad_k = -2 Re(½ω²ϵ₀·λ_k·E_k)
    if (objective) {
        // s = mᵀE (no conjugation), reduced on the host from per-block partials
        const int nparts = h->num_sms;   // one partial per SM
        RET(ensure_part(h, 2 * (size_t)nparts));
        LAUNCH(vdotu_kernel, nparts, 256, 0, N, d_m, h->kx, h->part);
        std::vector<double> part(2 * (size_t)nparts);
        CK(cudaMemcpyAsync(part.data(), h->part, part.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        for (int i = 0; i < nparts; ++i) s += zd(part[2 * i], part[2 * i + 1]);
        // dJ/dϵᵣ_k = -2 Re(conj(s)·ω²ϵ₀·λ_k·E_k)
        coef = std::conj(s) * w2e0;
    }
    cplx<double> c;
    c.re = coef.real();
    c.im = coef.imag();
    LAUNCH(adjoint_grad_kernel, nb, 256, 0, N, c, d_lam, h->kx, d_grad);
    RET(check_launch(h, "adjoint"));
    CK(cudaMemcpyAsync(grad, d_grad, N * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    if (ez) CK(cudaMemcpyAsync(ez, h->kx, bytes, cudaMemcpyDeviceToHost, h->stream));
    cudaEventRecord(h->ev[4], h->stream);
    CK(cudaStreamSynchronize(h->stream));
    RET(check_device(h, "adjoint"));
    if (J) *J = std::norm(s);
    if (stats) {
        stats->iterations = iters;
        stats->nrhs = 2;
        stats->rel_residual = rel;
        stats->t_assemble_ms = elapsed_ms(h->ev[0], h->ev[1]);
        stats->t_factor_ms = elapsed_ms(h->ev[1], h->ev[2]);
        stats->t_solve_ms = elapsed_ms(h->ev[3], h->ev[4]);
        stats->t_recover_ms = 0;
        stats->factor_flops = h->last_factor_flops;
        stats->block = h->map.b;
        stats->nblocks = h->map.n;
        stats->levels = (int)h->steps.size() + 1;
        stats->tc_gemm = h->tc_used;
        stats->factor_precision = h->fact_prec;
        stats->fp64_fallback = h->fell_back;
        stats->device_bytes = h->dev_bytes;
        stats->gpu_launches = h->launches;
        stats->t_total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
    if (!(rel <= h->tol))
        return set_err(h, FDFD_ENOCONV, "adjoint refinement stopped at relative residual %.3e > tol %.1e", rel,
                       h->tol);
    return FDFD_OK;
}

}  // namespace

extern "C" {

int fdfd_adjoint(fdfd_handle* h, const double* src, const double* mvec, double* J, double* grad, double* ez,
                 fdfd_stats* stats) {
    return adjoint_core(h, src, mvec, true, J, grad, ez, stats);
}

int fdfd_adjoint_vjp(fdfd_handle* h, const double* src, const double* g, double* grad, double* ez,
                     fdfd_stats* stats) {
    return adjoint_core(h, src, g, false, nullptr, grad, ez, stats);
}

int fdfd_eigfreq(fdfd_handle* h, double omega0, int nev, int which, double tol, double* omega, double* lambda,
                 double* fields, fdfd_stats* stats) {
    if (!h) return FDFD_EINVAL;
    if (h->mf) return set_err(h, FDFD_EINVAL, "fdfd_eigfreq: not defined for a modulated device");
    const long long N = (long long)h->Nx * h->Ny;
    if (!h->eps_set) return set_err(h, FDFD_EINVAL, "fdfd_set_eps must be called before fdfd_eigfreq");
    if (!(omega0 > 0) || nev < 1 || nev > 64 || nev >= N - 1 || !omega)
        return set_err(h, FDFD_EINVAL, "fdfd_eigfreq: invalid arguments");
    if (which < FDFD_WHICH_LM || which > FDFD_WHICH_SI)
        return set_err(h, FDFD_EINVAL, "fdfd_eigfreq: which must be one of FDFD_WHICH_LM/LR/SM/SR/LI/SI");
    if (!(tol > 0)) tol = 1e-10;
    auto t0 = std::chrono::steady_clock::now();
    h->launches = 0;
    const double eps0 = kEPS0 * h->L0, mu0 = kMU0 * h->L0;
    // eigen.jl:86 (TM) and :104 (TE): shift σ = -ω₀²μ₀ϵ₀ resp. -ω₀²μ₀, PML frozen at ω₀
    const zd sigma = h->pol == FDFD_TM ? zd(-omega0 * omega0 * mu0 * eps0, 0) : zd(-omega0 * omega0 * mu0, 0);
    cudaEventRecord(h->ev[0], h->stream);
    h->factored = false;
    RET(assemble(h, h->pol == FDFD_TM ? OP_TM_EIGEN : OP_TE_EIGEN, omega0, sigma, 0.0));
    cudaEventRecord(h->ev[1], h->stream);
    RET(factor_op(h));
    cudaEventRecord(h->ev[2], h->stream);
    h->omega = omega0;
    h->sigma = sigma;

    // Arnoldi basis (m+1 vectors) on the device
    const int m = (int)std::min<long long>(N - 1, std::max(2 * nev + 24, 48));
    RET(ensure_krylov(h, 2, restart_len(h, 2)));
    cplx<double>* V = nullptr;
    const size_t vbytes = (size_t)N * sizeof(cplx<double>);
    RET(dev_alloc(h, (void**)&V, vbytes * (m + 1)));
    struct Free {
        fdfd_handle* h; void* p; size_t b;
        ~Free() { dev_free(h, p); }
    } free_v{h, V, vbytes * (m + 1)};
    // deterministic start vector (splitmix64 hash of the index), unit norm
    {
        std::vector<zd> v0(N);
        double nn = 0;
        for (long long k = 0; k < N; ++k) {
            uint64_t x = (uint64_t)k * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull;
            x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
            x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
            x ^= x >> 31;
            v0[k] = zd((double)(x >> 11) / 9007199254740992.0 - 0.5, 0);
            nn += std::norm(v0[k]);
        }
        for (auto& v : v0) v /= std::sqrt(nn);
        CK(cudaMemcpyAsync(V, v0.data(), vbytes, cudaMemcpyHostToDevice, h->stream));
    }
    cudaEventRecord(h->ev[3], h->stream);
    // ARPACK's `which` in shift-invert mode ranks the eigenvalues θ = 1/(λ - σ) of the operator
    auto before = [which](const zd& a, const zd& b) {
        switch (which) {
            case FDFD_WHICH_LR: return a.real() > b.real();
            case FDFD_WHICH_SM: return std::abs(a) < std::abs(b);
            case FDFD_WHICH_SR: return a.real() < b.real();
            case FDFD_WHICH_LI: return a.imag() > b.imag();
            case FDFD_WHICH_SI: return a.imag() < b.imag();
            default: return std::abs(a) > std::abs(b);
        }
    };
    std::vector<zd> Hm((size_t)(m + 1) * m, zd(0, 0));
    std::vector<zd> theta, S;
    std::vector<int> pick;
    int iters = 0, restarts = 0, k = 0;
    bool converged = false;
    double worst = 0;
    auto select = [&](int kk) {
        // Ritz pairs of the kk x kk Hessenberg matrix, the nev wanted ones first
        std::vector<zd> Hk((size_t)kk * kk);
        for (int i = 0; i < kk; ++i)
            for (int j = 0; j < kk; ++j) Hk[(size_t)i * kk + j] = Hm[(size_t)i * m + j];
        if (!hess::eig(kk, Hk, theta, S)) return false;
        std::vector<int> idx(kk);
        for (int i = 0; i < kk; ++i) idx[i] = i;
        std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return before(theta[a], theta[b]); });
        pick.assign(idx.begin(), idx.begin() + std::min(nev, kk));
        return true;
    };
    while (!converged && restarts < 8) {
        k = 0;
        for (int j = 0; j < m; ++j) {
            // w = (A - σI)⁻¹ v_j, refined to the handle's tolerance
            CK(cudaMemcpyAsync(h->kb, V + (size_t)j * N, vbytes, cudaMemcpyDeviceToDevice, h->stream));
            int it = 0;
            double rr = 0;
            RET(refine_fb(h, 1, &it, &rr));
            iters += it;
            cplx<double>* w = V + (size_t)(j + 1) * N;
            CK(cudaMemcpyAsync(w, h->kx, vbytes, cudaMemcpyDeviceToDevice, h->stream));
            std::vector<zd> hc, hc2, nn;
            RET(dots(h, V, N, j + 1, w, 1, hc));
            RET(combine(h, V, N, j + 1, hc, 1, -1.0, w));
            RET(dots(h, V, N, j + 1, w, 1, hc2));
            RET(combine(h, V, N, j + 1, hc2, 1, -1.0, w));
            RET(dots(h, w, 0, 1, w, 1, nn));
            for (int i = 0; i <= j; ++i) Hm[(size_t)i * m + j] = hc[i] + hc2[i];
            const double hn = std::sqrt(std::max(0.0, nn[0].real()));
            Hm[(size_t)(j + 1) * m + j] = hn;
            k = j + 1;
            std::vector<zd> sc(1, hn > 0 ? zd(1.0 / hn, 0) : zd(0, 0));
            RET(scale_vec(h, w, sc, 1, w));
            if (hn == 0 || ((k >= nev + 2) && (k % 4 == 0 || k == m))) {
                if (!select(k)) return set_err(h, FDFD_ENOCONV, "Hessenberg QR did not converge");
                worst = 0;
                for (int i : pick) {
                    const double res = hn * std::abs(S[(size_t)(k - 1) * k + i]);
                    worst = std::max(worst, res / std::max(std::abs(theta[i]), 1e-300));
                }
                if ((int)pick.size() == nev && worst <= tol) { converged = true; break; }
                if (hn == 0) break;
            }
        }
        if (!converged) {
            // explicit restart from the sum of the wanted Ritz vectors
            if (!select(k)) return set_err(h, FDFD_ENOCONV, "Hessenberg QR did not converge");
            std::vector<zd> c(k, zd(0, 0));
            for (int i : pick)
                for (int r = 0; r < k; ++r) c[r] += S[(size_t)r * k + i];
            CK(cudaMemsetAsync(h->kr, 0, vbytes, h->stream));
            RET(combine(h, V, N, k, c, 1, 1.0, h->kr));
            std::vector<zd> nn;
            RET(dots(h, h->kr, 0, 1, h->kr, 1, nn));
            std::vector<zd> sc(1, zd(1.0 / std::sqrt(std::max(nn[0].real(), 1e-300)), 0));
            RET(scale_vec(h, h->kr, sc, 1, V));
            ++restarts;
        }
    }
    cudaEventRecord(h->ev[4], h->stream);
    // eigenvalues of A (λ = σ + 1/θ), eigenfrequencies, Ritz vectors and fields
    std::vector<zd> lam(nev), om(nev);
    std::vector<int> order(pick);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return before(theta[a], theta[b]); });
    for (int q = 0; q < nev; ++q) {
        const zd th = theta[order[q]];
        lam[q] = sigma + 1.0 / th;
        om[q] = h->pol == FDFD_TM ? std::sqrt(-lam[q] / mu0 / eps0) : std::sqrt(-lam[q] / mu0);   // eigen.jl:87,105
        omega[2 * q] = om[q].real();
        omega[2 * q + 1] = om[q].imag();
        if (lambda) { lambda[2 * q] = lam[q].real(); lambda[2 * q + 1] = lam[q].imag(); }
    }
    if (fields) {
        for (int q = 0; q < nev; ++q) {
            std::vector<zd> c(k);
            for (int r = 0; r < k; ++r) c[r] = S[(size_t)r * k + order[q]];
            cplx<double>* y = h->kx;
            CK(cudaMemsetAsync(y, 0, vbytes, h->stream));
            RET(combine(h, V, N, k, c, 1, 1.0, y));
            // unit norm, largest component real positive
            std::vector<zd> host(N);
            CK(cudaMemcpyAsync(host.data(), y, vbytes, cudaMemcpyDeviceToHost, h->stream));
            CK(cudaStreamSynchronize(h->stream));
            double nn = 0;
            long long imax = 0;
            for (long long i = 0; i < N; ++i) {
                nn += std::norm(host[i]);
                if (std::abs(host[i]) > std::abs(host[imax])) imax = i;
            }
            const zd ph = std::abs(host[imax]) > 0 ? std::conj(host[imax]) / std::abs(host[imax]) : zd(1, 0);
            const zd sc = ph / std::sqrt(nn);
            for (auto& v : host) v *= sc;
            double* f1 = fields + (size_t)q * 3 * 2 * N;
            memcpy(f1, host.data(), vbytes);
            CK(cudaMemcpyAsync(y, host.data(), vbytes, cudaMemcpyHostToDevice, h->stream));
            // eigen.jl:90-91 (TM, forward differences) / :108-109 (TE)
            std::vector<zd> coef(2);
            if (h->pol == FDFD_TM) {
                coef[0] = zd(-0.0, 1.0) / om[q] / mu0;    // -1/1im/ω/μ₀
                coef[1] = zd(0.0, -1.0) / om[q] / mu0;    //  1/1im/ω/μ₀
            } else {
                coef[0] = zd(0.0, -1.0) / om[q];          //  1/1im/ω
                coef[1] = coef[0];
            }
            CK(cudaMemcpyAsync(h->kc, coef.data(), 2 * sizeof(zd), cudaMemcpyHostToDevice, h->stream));
            RecoverArgs ra;
            ra.Nx = h->Nx; ra.Ny = h->Ny; ra.mode = h->pol == FDFD_TM ? REC_TM_EIGEN : REC_TE_EIGEN;
            ra.idx = 1.0 / h->dx; ra.idy = 1.0 / h->dy; ra.eps0n = eps0;
            LAUNCH(recover_kernel, dim3(ceil_div(N, 256), 1), 256, 0, ra, h->sf, h->eps, y, h->kc, h->kr,
                   h->kr + N);
            RET(check_launch(h, "eigen recover"));
            CK(cudaMemcpyAsync(f1 + 2 * N, h->kr, 2 * vbytes, cudaMemcpyDeviceToHost, h->stream));
        }
    }
    CK(cudaStreamSynchronize(h->stream));
    RET(check_device(h, "eigfreq"));
    if (stats) {
        stats->iterations = iters;
        stats->nrhs = nev;
        stats->rel_residual = worst;
        stats->t_assemble_ms = elapsed_ms(h->ev[0], h->ev[1]);
        stats->t_factor_ms = elapsed_ms(h->ev[1], h->ev[2]);
        stats->t_solve_ms = elapsed_ms(h->ev[3], h->ev[4]);
        stats->t_recover_ms = 0;
        stats->factor_flops = h->last_factor_flops;
        stats->block = h->map.b;
        stats->nblocks = h->map.n;
        stats->levels = (int)h->steps.size() + 1;
        stats->tc_gemm = h->tc_used;
        stats->factor_precision = h->fact_prec;
        stats->fp64_fallback = h->fell_back;
        stats->device_bytes = h->dev_bytes;
        stats->gpu_launches = h->launches;
        stats->t_total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
    if (!converged)
        return set_err(h, FDFD_ENOCONV, "Arnoldi: wanted Ritz pairs not converged (worst residual %.2e)", worst);
    return FDFD_OK;
}

// Test entry: eigen-decomposition of a small complex upper Hessenberg matrix
// (host only, the Ritz-pair solver of fdfd_eigfreq).
int fdfd_debug_hessenberg_eig(int n, const double* H, double* w, double* V) {
    if (n < 1 || !H || !w || !V) return FDFD_EINVAL;
    std::vector<zd> Hm((size_t)n * n), ww, VV;
    for (size_t i = 0; i < Hm.size(); ++i) Hm[i] = zd(H[2 * i], H[2 * i + 1]);
    if (!hess::eig(n, Hm, ww, VV)) return FDFD_ENOCONV;
    for (int i = 0; i < n; ++i) { w[2 * i] = ww[i].real(); w[2 * i + 1] = ww[i].imag(); }
    for (size_t i = 0; i < VV.size(); ++i) { V[2 * i] = VV[i].real(); V[2 * i + 1] = VV[i].imag(); }
    return FDFD_OK;
}

}  // extern "C"

namespace {

template <typename T>
int debug_gemm_impl(int M, int N, int K, const double* A, const double* B, double* C, int use_tc, double* ms) {
    // use_tc < 0: the operands as pre-split four-plane pools (the panel-buffer form)
    const int planes = (sizeof(T) == 4 && use_tc < 0) ? 4 : 2;
    use_tc = use_tc < 0 ? -use_tc : use_tc;
    Pool<T> PA, PB, PC;
    auto setp = [&](Pool<T>& P, int rows, int cols, int np) {
        P.rows = rows; P.cols = cols; P.ld = (cols + 31) / 32 * 32; P.planes = np; P.count = 1;
    };
    setp(PA, M, K, planes); setp(PB, N, K, planes); setp(PC, M, N, 2);
    auto upload = [&](Pool<T>& P, const double* src) -> int {
        std::vector<T> host((size_t)P.slot_elems(), (T)0);
        long long pe = P.plane_elems();
        for (int r = 0; r < P.rows; ++r)
            for (int c = 0; c < P.cols; ++c) {
                double re = src[2 * ((size_t)r * P.cols + c)], im = src[2 * ((size_t)r * P.cols + c) + 1];
                size_t o = (size_t)r * P.ld + c;
                host[o] = (T)re;
                host[pe + o] = (T)im;
                if (P.planes == 4) {   // TF32 residuals: x minus x with the low 13 mantissa bits cleared
                    float fr = (float)re, fi = (float)im;
                    uint32_t ur, ui;
                    memcpy(&ur, &fr, 4); memcpy(&ui, &fi, 4);
                    ur &= 0xffffe000u; ui &= 0xffffe000u;
                    float hr, hi;
                    memcpy(&hr, &ur, 4); memcpy(&hi, &ui, 4);
                    host[2 * pe + o] = (T)(fr - hr);
                    host[3 * pe + o] = (T)(fi - hi);
                }
            }
        if (cudaMalloc(&P.base, host.size() * sizeof(T)) != cudaSuccess) return FDFD_ENOMEM;
        if (cudaMemcpy(P.base, host.data(), host.size() * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess)
            return FDFD_ECUDA;
        return FDFD_OK;
    };
    int rc = upload(PA, A);
    if (rc == FDFD_OK) rc = upload(PB, B);
    std::vector<double> zeros((size_t)2 * M * N, 0.0);
    if (rc == FDFD_OK) rc = upload(PC, zeros.data());
    int* slots = nullptr;
    unsigned* derr = nullptr;
    if (rc == FDFD_OK && cudaMalloc(&slots, sizeof(int)) != cudaSuccess) rc = FDFD_ENOMEM;
    if (rc == FDFD_OK && cudaMalloc(&derr, sizeof(unsigned)) != cudaSuccess) rc = FDFD_ENOMEM;
    if (rc == FDFD_OK) {
        cudaMemset(slots, 0, sizeof(int));
        cudaMemset(derr, 0, sizeof(unsigned));
    }
    if (rc == FDFD_OK) {
        GemmArgs<T> g;
        g.A = PA; g.B = PB; g.C = PC;
        g.a_slot = g.b_slot = g.c_slot = slots;
        g.Cin = Pool<T>(); g.cin_slot = nullptr; g.row_src = nullptr;
        g.M = M; g.N = N; g.K = K; g.alpha = (T)1; g.beta = 0; g.mask_c0 = 0; g.mask_w = 0;
        g.c_trans = 0; g.c_trans_arr = nullptr; g.row_dst = nullptr; g.err = derr; g.wait_ns = 0;
        g.n_off = 0; g.skip_c0 = 0; g.skip_w = 0;
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0); cudaEventCreate(&e1);
        if (sizeof(T) == 4 && use_tc) {
            CUtensorMap ma[3], mb[3];
            const Pool<float>* fa = reinterpret_cast<const Pool<float>*>(&PA);
            const Pool<float>* fb = reinterpret_cast<const Pool<float>*>(&PB);
            if (!tc_make_map(*fa, &ma[0], &ma[1], &ma[2]) || !tc_make_map(*fb, &mb[0], &mb[1], &mb[2]))
                rc = FDFD_ECUDA;
            int dev = 0, sms = 0;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            const int bn = (use_tc == 64 || use_tc == 128 || use_tc == 256 || use_tc == TC_BN128_TWO)
                               ? use_tc
                               : tc_pick_bn(M, N, K, 1, sms);
            const int bi = bn == 256 ? 1 : ((bn == 128 || bn == TC_BN128_TWO) ? 0 : 2);
            if (rc == FDFD_OK) {
                cudaEventRecord(e0);
                if (tc_gemm_launch_maps(reinterpret_cast<GemmArgs<float>*>(&g), nullptr, &ma[0], &mb[bi], bn, 1, 0) !=
                    0)
                    rc = FDFD_ECUDA;
                cudaEventRecord(e1);
            }
        } else {
            cudaEventRecord(e0);
            launch_gemm_simt<T>(0, 1, g);
            cudaEventRecord(e1);
        }
        if (cudaDeviceSynchronize() != cudaSuccess) rc = FDFD_ECUDA;
        float t = 0;
        cudaEventElapsedTime(&t, e0, e1);
        if (ms) *ms = t;
        cudaEventDestroy(e0); cudaEventDestroy(e1);
        unsigned e = 0;
        cudaMemcpy(&e, derr, sizeof e, cudaMemcpyDeviceToHost);
        if (rc == FDFD_OK && e) rc = (e & FDFD_DEVERR_TIMEOUT) ? FDFD_ETIMEOUT : FDFD_ECUDA;
    }
    if (rc == FDFD_OK) {
        std::vector<T> host((size_t)PC.slot_elems());
        cudaMemcpy(host.data(), PC.base, host.size() * sizeof(T), cudaMemcpyDeviceToHost);
        long long pe = PC.plane_elems();
        for (int r = 0; r < M; ++r)
            for (int c = 0; c < N; ++c) {
                C[2 * ((size_t)r * N + c)] = host[(size_t)r * PC.ld + c];
                C[2 * ((size_t)r * N + c) + 1] = host[pe + (size_t)r * PC.ld + c];
            }
    }
    cudaFree(PA.base); cudaFree(PB.base); cudaFree(PC.base); cudaFree(slots); cudaFree(derr);
    return rc;
}

}  // namespace

extern "C" {

// Test entry point: C = A·Bᵀ (complex, A: M x K, B: N x K, C: M x N, row-major
// interleaved host arrays) through the library's GEMM kernels: precision
// FDFD_PREC_FP64 (SIMT FP64) or FDFD_PREC_MIXED (FP32 storage; use_tc selects
// the tcgen05 3xTF32 kernel or the SIMT FP32 kernel).  *ms receives the kernel
// time.  No counterpart in the reference.
int fdfd_debug_gemm(int M, int N, int K, const double* A, const double* B, double* C, int precision, int use_tc,
                    double* ms) {
    if (M < 1 || N < 1 || K < 1 || !A || !B || !C) return FDFD_EINVAL;
    if (precision == FDFD_PREC_FP64) return debug_gemm_impl<double>(M, N, K, A, B, C, 0, ms);
    return debug_gemm_impl<float>(M, N, K, A, B, C, use_tc, ms);
}

}  // extern "C"
