// Batched complex TN GEMM on the sm_103a tensor cores: tcgen05.mma kind::tf32
// with 3xTF32 split precision, TMA-staged operands, accumulators in TMEM.
//
//   C[m][n] = beta(m,n)·Cin[src(m)][n] + alpha·Σ_k A[m][k]·B[n][k]      (complex)
//
// over matrix columns n in [n_off, n_off + N) without [skip_c0, skip_c0 + skip_w)
//
// Operands are FP32 planar pools.  The tensor core reads only the top 19 bits
// of an FP32 operand, so the raw plane serves as the "hi" term; with the TF32
// residual lo = x - (x with the low 13 mantissa bits cleared)
//   a·b ≈ hi(a)·hi(b) + hi(a)·lo(b) + lo(a)·hi(b)
// recovers close to FP32 accuracy (the split of Markidis et al., 2018, as used
// for 3xTF32 GEMMs).  Two operand forms: pools of two planes (re, im; the
// factor blocks), whose lo planes are formed in shared memory as each stage
// lands, so TMA moves half the bytes; and pools of four planes (re, im, re_lo,
// im_lo; the small Gauss-Jordan panel buffers), loaded pre-split so that a
// short-K product has no conversion on its critical path.  A and B of one
// launch have the same form.  Each complex product is four real products (the im·im
// term through the instruction's negate-A bit), so one K-step issues 12 MMAs
// into two TMEM accumulators (real and imaginary, BN columns each).
//
// CTA tile 128 x BN (complex outputs, BN = 256, 128 or 64: the launcher takes
// the widest tile that still fills the GPU, so small batches get more CTAs),
// K-step 8 (one 32-byte swizzle row per operand row), 4-stage TMA pipeline,
// 64 + 32*NEPI threads:
//   warp 0      TMA producer (one elected lane): the planes of A and B
//   warp 1      TMEM allocator and MMA issuer (one elected lane)
//   warps 2..    during the K loop (two-plane operands): write the lo planes of
//               each landed stage (bar_full -> bar_conv); then the epilogue:
//               tcgen05.ld -> registers -> global (N- or T-form).  4 warps, or 8
//               for BN >= 128 (two per TMEM lane quarter, one per column half)
// Every mbarrier wait is bounded (2 s of %globaltimer); on timeout the CTA sets
// FDFD_DEVERR_TIMEOUT, drains its own TMA copies (bounded), frees TMEM and exits.
#include "gemm_tc.cuh"

namespace {

constexpr int BM = 128, BK = 8;
constexpr int A_PLANE_BYTES = BM * BK * 4;                  // 4 KB
// TWO = 1: a 128-column tile sized so that two CTAs share an SM (three pipeline
// stages, one epilogue warp per TMEM lane quarter), so one CTA's epilogue overlaps
// the other's MMAs; an autotuner candidate beside the one-CTA tiles.
template <int BN, int TWO = 0> struct TcTile {
    static constexpr int STAGES = TWO ? 3 : 4;
    // epilogue warps: two per TMEM lane quarter (each takes half the columns),
    // one at BN = 64 and in the two-CTA form (two CTAs share an SM there)
    static constexpr int NEPI = (BN >= 128 && !TWO) ? 8 : 4;
    static constexpr int THREADS = 64 + 32 * NEPI;
    static constexpr int MIN_BLOCKS = (BN <= 64 || TWO) ? 2 : 1;
    static constexpr int B_PLANE_BYTES = BN * BK * 4;
    static constexpr int STAGE_BYTES = 4 * A_PLANE_BYTES + 4 * B_PLANE_BYTES;
    static constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024;   // + alignment slack
    static constexpr uint32_t TMEM_COLS = 2 * BN;                     // re and im accumulators
    // the epilogue stages NEPI warps x 2 x 32 x 36 floats in the idle pipeline buffers
    static_assert(STAGES * STAGE_BYTES >= NEPI * 2 * 32 * 36 * 4, "epilogue staging");
    static_assert(MIN_BLOCKS * (SMEM_BYTES + 1024) <= 227 * 1024, "shared memory per SM");
};

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2,
                                            uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(bar)
        : "memory");
}

// bulk prefetch of a global range into L2 (16-byte aligned address, size a multiple of 16)
__device__ __forceinline__ void l2_prefetch(const void* src, uint32_t bytes) {
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(reinterpret_cast<uint64_t>(src)), "r"(bytes)
                 : "memory");
}

// tcgen05 shared-memory matrix descriptor, K-major, 32-byte swizzle:
// start address >> 4 (bits 0-13), leading byte offset >> 4 (16-29, unused for
// swizzled K-major), stride byte offset >> 4 (32-45: 8 rows x 32 B = 256 B
// between 8-row groups), descriptor version 1 (bits 46-47), swizzle mode
// 6 = 32-byte (bits 61-63).
__device__ __forceinline__ uint64_t sdesc_sw32(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFF);
    d |= (uint64_t)1 << 16;
    d |= (uint64_t)(256 >> 4) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)6 << 61;
    return d;
}

// instruction descriptor, kind::tf32: D=F32 (bits 4-5 = 1), A=B=TF32 (bits 7-9,
// 10-12 = 2), negate A (bit 13), both K-major (bits 15,16 = 0), N>>3 (17-22),
// M>>4 (24-28).
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N, int negA) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)negA << 13) | ((uint32_t)(N >> 3) << 17) |
           ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accum) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accum));
}

__device__ __forceinline__ void mma_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&v)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
          "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
          "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
        : "r"(taddr));
}

struct TcParams {
    GemmArgs<float> g;
};

template <int BN, int TWO>
__global__ void __launch_bounds__(TcTile<BN, TWO>::THREADS, TcTile<BN, TWO>::MIN_BLOCKS)
    gemm_tc_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
                   const TcParams P) {
    constexpr int STAGES = TcTile<BN, TWO>::STAGES;
    constexpr int B_PLANE_BYTES = TcTile<BN, TWO>::B_PLANE_BYTES;
    constexpr int STAGE_BYTES = TcTile<BN, TWO>::STAGE_BYTES;
    constexpr uint32_t TMEM_COLS = TcTile<BN, TWO>::TMEM_COLS;
    constexpr int NEPI = TcTile<BN, TWO>::NEPI;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bar_full[STAGES], bar_conv[STAGES], bar_empty[STAGES], bar_acc;
    __shared__ uint32_t tmem_base_slot;
    __shared__ int s_abort;

    const GemmArgs<float>& g = P.g;
    const uint64_t wait_ns = g.wait_ns ? g.wait_ns : FDFD_WAIT_LIMIT_NS;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // split-K: CTA z works on job z / ksplit over one slice of K and writes its own C slot
    const int ks = g.ksplit > 1 ? g.ksplit : 1;
    const int job = blockIdx.z / ks;
    const int cjob = ks > 1 ? (int)blockIdx.z : job;     // index into c_slot
    const int kbeg = ks > 1 ? (int)(blockIdx.z % ks) * g.kslice : 0;
    const int klen = ks > 1 ? min(g.kslice, g.K - kbeg) : g.K;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    const int nk = (klen + BK - 1) / BK;
    const bool presplit = g.A.planes == 4;             // operand form (A and B alike)
    const int np = presplit ? 4 : 2;                   // planes loaded by TMA
    unsigned char* smem = reinterpret_cast<unsigned char*>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    const uint32_t sbase = smem_u32(smem);

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(smem_u32(&bar_full[s]), 1);
            mbar_init(smem_u32(&bar_conv[s]), 32 * NEPI);   // every epilogue thread converts
            mbar_init(smem_u32(&bar_empty[s]), 1);
        }
        mbar_init(smem_u32(&bar_acc), 1);
        s_abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(&tmem_base_slot)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_base_slot;

    if (warp == 0) {
        if (lane == 0) {
            const int aslot = g.a_slot[job], bslot = g.b_slot[job];
            int issued = 0;
            bool ok = true;
            for (int kt = 0; kt < nk; ++kt) {
                const int s = kt % STAGES;
                if (kt >= STAGES) {
                    if (!mbar_wait(smem_u32(&bar_empty[s]), ((kt / STAGES) - 1) & 1, wait_ns)) { ok = false; break; }
                }
                const uint32_t bar = smem_u32(&bar_full[s]);
                mbar_expect_tx(bar, np * (A_PLANE_BYTES + B_PLANE_BYTES));
                const uint32_t st = sbase + s * STAGE_BYTES;
                const int k0 = kbeg + kt * BK;
                for (int p = 0; p < np; ++p)
                    tma_load_3d(st + p * A_PLANE_BYTES, &mapA, k0, m0, aslot * np + p, bar);
                for (int p = 0; p < np; ++p)
                    tma_load_3d(st + 4 * A_PLANE_BYTES + p * B_PLANE_BYTES, &mapB, k0, n0 + g.n_off, bslot * np + p, bar);
                issued = kt + 1;
            }
            if (!ok) {
                dev_error(g.err, FDFD_DEVERR_TIMEOUT);
                atomicExch(&s_abort, 1);
            }
            // drain this CTA's copies in flight (bounded)
            for (int kt = (issued > STAGES ? issued - STAGES : 0); kt < issued; ++kt)
                if (!mbar_wait(smem_u32(&bar_full[kt % STAGES]), (kt / STAGES) & 1, FDFD_WAIT_LIMIT_NS)) {
                    dev_error(g.err, FDFD_DEVERR_TIMEOUT);
                    break;
                }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            bool ok = true;
            const uint32_t acc_re = tmem, acc_im = tmem + BN;
            const uint32_t id_pos = idesc_tf32(BM, BN, 0), id_neg = idesc_tf32(BM, BN, 1);
            for (int kt = 0; kt < nk; ++kt) {
                const int s = kt % STAGES;
                if (!mbar_wait(smem_u32(presplit ? &bar_full[s] : &bar_conv[s]), (kt / STAGES) & 1, wait_ns)) {
                    ok = false;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t st = sbase + s * STAGE_BYTES;
                uint64_t a[4], b[4];
                for (int p = 0; p < 4; ++p) {
                    a[p] = sdesc_sw32(st + p * A_PLANE_BYTES);
                    b[p] = sdesc_sw32(st + 4 * A_PLANE_BYTES + p * B_PLANE_BYTES);
                }
                const uint32_t first = (kt > 0) ? 1u : 0u;
                // planes: 0 re, 1 im, 2 re_lo, 3 im_lo
                mma_tf32(acc_re, a[0], b[0], id_pos, first);   // re·re
                mma_tf32(acc_re, a[0], b[2], id_pos, 1);
                mma_tf32(acc_re, a[2], b[0], id_pos, 1);
                mma_tf32(acc_re, a[1], b[1], id_neg, 1);       // -im·im
                mma_tf32(acc_re, a[1], b[3], id_neg, 1);
                mma_tf32(acc_re, a[3], b[1], id_neg, 1);
                mma_tf32(acc_im, a[0], b[1], id_pos, first);   // re·im
                mma_tf32(acc_im, a[0], b[3], id_pos, 1);
                mma_tf32(acc_im, a[2], b[1], id_pos, 1);
                mma_tf32(acc_im, a[1], b[0], id_pos, 1);       // im·re
                mma_tf32(acc_im, a[1], b[2], id_pos, 1);
                mma_tf32(acc_im, a[3], b[0], id_pos, 1);
                mma_commit(smem_u32(&bar_empty[s]));
            }
            if (!ok) {
                dev_error(g.err, FDFD_DEVERR_TIMEOUT);
                atomicExch(&s_abort, 1);
            }
            mma_commit(smem_u32(&bar_acc));
        }
    } else {
        // epilogue warps 2..5; TMEM lane quarter = warp % 4
        const int q = warp & 3;
        const int part = (warp - 2) >> 2;              // column part of this warp (NEPI / 4 parts)
        constexpr int PARTS = NEPI / 4, PCOLS = BN / PARTS;
        // A short-K product (the Gauss-Jordan rank-panel update) is bound by its β read:
        // each lane pulls its β row (re, im) into L2 while the MMAs run.  Rows are
        // ld-padded, so the range [n0, min(n0 + BN, ld)) is 16-byte aligned and sized.
        if (g.beta && nk <= STAGES && !(g.c_trans_arr ? g.c_trans_arr[job] : g.c_trans)) {
            const bool sep = g.Cin.base != nullptr;
            const float* Ci = sep ? g.Cin.slot(g.cin_slot[job]) : g.C.slot(g.c_slot[cjob]);
            const long long cipe = sep ? g.Cin.plane_elems() : g.C.plane_elems();
            const int cild = sep ? g.Cin.ld : g.C.ld;
            const int* rsrc = (sep && g.row_src) ? g.row_src + (long long)job * g.M : nullptr;
            const int r = m0 + q * 32 + lane;
            const int nlo = n0 + g.n_off + part * PCOLS;
            const int ncols = min(min(PCOLS, cild - nlo), g.n_off + g.N - nlo);
            const int rd = (g.row_dst && r < g.M) ? g.row_dst[(long long)job * g.M + r] : r;   // output row
            const bool mrow = (rd >= g.mask_c0 && rd < g.mask_c0 + g.mask_w);
            if (r < g.M && !mrow && ncols > 0) {
                const float* src = Ci + (long long)(rsrc ? rsrc[r] : r) * cild + nlo;
                l2_prefetch(src, (uint32_t)ncols * 4u);
                l2_prefetch(src + cipe, (uint32_t)ncols * 4u);
            }
        }
        // warps 2..5: first the TF32 residual planes of every landed stage
        // (two-plane operands).  The lo planes have the layout of the raw
        // planes, so the split is elementwise at equal offsets, whatever the swizzle.
        if (!presplit) {
            const int ct = threadIdx.x - 64;                    // 0 .. 32*NEPI-1
            constexpr int NV4 = (2 * A_PLANE_BYTES + 2 * B_PLANE_BYTES) / 16;   // float4s per stage
            bool okc = true;
            for (int kt = 0; kt < nk; ++kt) {
                const int s = kt % STAGES;
                if (*(volatile int*)&s_abort) { okc = false; break; }
                if (!mbar_wait(smem_u32(&bar_full[s]), (kt / STAGES) & 1, wait_ns)) { okc = false; break; }
                unsigned char* st = smem + s * STAGE_BYTES;
                for (int v = ct; v < NV4; v += 32 * NEPI) {
                    // A re, A im | B re, B im; each lo plane sits two planes after its raw plane
                    const int off = v < 2 * A_PLANE_BYTES / 16 ? v * 16 : 4 * A_PLANE_BYTES + (v * 16 - 2 * A_PLANE_BYTES);
                    const int lo_off = off + (v < 2 * A_PLANE_BYTES / 16 ? 2 * A_PLANE_BYTES : 2 * B_PLANE_BYTES);
                    const float4 x = *reinterpret_cast<const float4*>(st + off);
                    *reinterpret_cast<float4*>(st + lo_off) = make_float4(tf32_lo(x.x), tf32_lo(x.y), tf32_lo(x.z),
                                                                          tf32_lo(x.w));
                }
                // make the generic-proxy stores visible to the tensor core (async proxy)
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&bar_conv[s])) : "memory");
            }
            if (!okc) {
                dev_error(g.err, FDFD_DEVERR_TIMEOUT);
                atomicExch(&s_abort, 1);
            }
        }
        // the accumulator barrier also drains the MMAs in flight: full limit
        const bool ok_l = mbar_wait(smem_u32(&bar_acc), 0, FDFD_WAIT_LIMIT_NS);
        const bool ok = __all_sync(0xffffffffu, ok_l);
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const int abort = __shfl_sync(0xffffffffu, *(volatile int*)&s_abort, 0);
        if (!ok) {
            if (lane == 0) dev_error(g.err, FDFD_DEVERR_TIMEOUT);
        } else if (!abort) {
            const int row0 = m0 + q * 32;
            const int row = row0 + lane;
            const int ctr = g.c_trans_arr ? g.c_trans_arr[job] : g.c_trans;
            float* C = g.C.slot(g.c_slot[cjob]);
            const long long pe = g.C.plane_elems();
            const long long ld = g.C.ld;
            // β term source: C itself, or row row_src[m] of Cin
            const bool sep = g.Cin.base != nullptr;
            const float* Ci = sep ? g.Cin.slot(g.cin_slot[job]) : C;
            const long long cipe = sep ? g.Cin.plane_elems() : pe;
            const long long cild = sep ? (long long)g.Cin.ld : ld;
            const int* rsrc = (sep && g.row_src) ? g.row_src + (long long)job * g.M : nullptr;
            const int* rdst = g.row_dst ? g.row_dst + (long long)job * g.M : nullptr;
            const uint32_t lane_off = (uint32_t)(q * 32) << 16;
            // per-warp staging tile (the pipeline buffers are idle once the accumulator is final)
            float* stg = reinterpret_cast<float*>(smem) + (warp - 2) * (2 * 32 * 36);
            // β-source row offsets and output rows of the 8 rows this lane handles in the
            // row-major epilogue
            long long srow[8];
            int drow[8];
#pragma unroll
            for (int it = 0; it < 8; ++it) {
                const int r = row0 + 4 * it + (lane >> 3);
                srow[it] = (long long)(rsrc && r < g.M ? rsrc[r] : r) * cild;
                drow[it] = (rdst && r < g.M) ? rdst[r] : r;
            }
            for (int ch = part * (PCOLS / 32); ch < (part + 1) * (PCOLS / 32); ++ch) {
                const int nb = n0 + ch * 32;
                if (nb >= g.N) break;
                uint32_t vr[32], vi[32];
                tmem_ld32(tmem + lane_off + ch * 32, vr);
                tmem_ld32(tmem + lane_off + BN + ch * 32, vi);
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                if (ctr) {
                    // transposed store: lanes (rows) are contiguous in Cᵀ -> coalesced per column
                    if (row < g.M) {
#pragma unroll
                        for (int j = 0; j < 32; ++j) {
                            const int n = nb + j;
                            if (n >= g.N) break;
                            const int na = n + g.n_off;      // matrix column
                            if (na >= g.skip_c0 && na < g.skip_c0 + g.skip_w) continue;
                            const float xr = g.alpha * __uint_as_float(vr[j]);
                            const float xi = g.alpha * __uint_as_float(vi[j]);
                            const long long off = (long long)na * ld + row;
                            C[off] = xr;
                            C[pe + off] = xi;
                        }
                    }
                } else {
                    // Row-major store through shared memory.  The 32x32 sub-tile is staged
                    // (row stride 36 floats keeps float4 rows 16-byte aligned and the staging
                    // writes conflict-free), then read back as float4: 8 lanes cover one
                    // 128-byte row segment, 4 rows per instruction, and every C load of the
                    // sub-tile is issued before the first store.
#pragma unroll
                    for (int q4 = 0; q4 < 8; ++q4) {
                        *reinterpret_cast<float4*>(&stg[lane * 36 + 4 * q4]) =
                            make_float4(__uint_as_float(vr[4 * q4]), __uint_as_float(vr[4 * q4 + 1]),
                                        __uint_as_float(vr[4 * q4 + 2]), __uint_as_float(vr[4 * q4 + 3]));
                        *reinterpret_cast<float4*>(&stg[32 * 36 + lane * 36 + 4 * q4]) =
                            make_float4(__uint_as_float(vi[4 * q4]), __uint_as_float(vi[4 * q4 + 1]),
                                        __uint_as_float(vi[4 * q4 + 2]), __uint_as_float(vi[4 * q4 + 3]));
                    }
                    __syncwarp();
                    const int sub = lane >> 3, cq = lane & 7;
                    const int n = nb + 4 * cq;
                    const int na = n + g.n_off;          // matrix column of the group
                    // a group touching the skipped columns takes the per-element path
                    const bool skipg = na + 3 >= g.skip_c0 && na < g.skip_c0 + g.skip_w;
                    const bool full4 = (n + 3 < g.N) && !skipg;
                    float4 cre[8], cim[8];
#pragma unroll
                    for (int it = 0; it < 8; ++it) {
                        const int r = row0 + 4 * it + sub;
                        cre[it] = make_float4(0.f, 0.f, 0.f, 0.f);
                        cim[it] = cre[it];
                        const bool mrow = (drow[it] >= g.mask_c0 && drow[it] < g.mask_c0 + g.mask_w);
                        if (g.beta && r < g.M && !mrow) {
                            const long long off = srow[it] + na;
                            if (full4) {
                                cre[it] = __ldcg(reinterpret_cast<const float4*>(Ci + off));
                                cim[it] = __ldcg(reinterpret_cast<const float4*>(Ci + cipe + off));
                            } else {
                                float* a = reinterpret_cast<float*>(&cre[it]);
                                float* c = reinterpret_cast<float*>(&cim[it]);
                                for (int e = 0; e < 4; ++e)
                                    if (n + e < g.N && !(na + e >= g.skip_c0 && na + e < g.skip_c0 + g.skip_w)) {
                                        a[e] = __ldcg(Ci + off + e);
                                        c[e] = __ldcg(Ci + cipe + off + e);
                                    }
                            }
                        }
                    }
#pragma unroll
                    for (int it = 0; it < 8; ++it) {
                        const int rl = 4 * it + sub;
                        const int r = row0 + rl;
                        if (r >= g.M) continue;
                        const int rd = drow[it];
                        const bool mrow = (rd >= g.mask_c0 && rd < g.mask_c0 + g.mask_w);
                        const float4 sr = *reinterpret_cast<const float4*>(&stg[rl * 36 + 4 * cq]);
                        const float4 si = *reinterpret_cast<const float4*>(&stg[32 * 36 + rl * 36 + 4 * cq]);
                        const float* srp = reinterpret_cast<const float*>(&sr);
                        const float* sip = reinterpret_cast<const float*>(&si);
                        const float* crp = reinterpret_cast<const float*>(&cre[it]);
                        const float* cip = reinterpret_cast<const float*>(&cim[it]);
                        float xr[4], xi[4];
#pragma unroll
                        for (int e = 0; e < 4; ++e) {
                            const int col = na + e;
                            const bool keep = g.beta && !(mrow || (col >= g.mask_c0 && col < g.mask_c0 + g.mask_w));
                            xr[e] = g.alpha * srp[e] + (keep ? crp[e] : 0.f);
                            xi[e] = g.alpha * sip[e] + (keep ? cip[e] : 0.f);
                        }
                        const long long off = (long long)rd * ld + na;
                        if (full4) {
                            *reinterpret_cast<float4*>(C + off) = make_float4(xr[0], xr[1], xr[2], xr[3]);
                            *reinterpret_cast<float4*>(C + pe + off) = make_float4(xi[0], xi[1], xi[2], xi[3]);
                        } else {
                            for (int e = 0; e < 4; ++e)
                                if (n + e < g.N && !(na + e >= g.skip_c0 && na + e < g.skip_c0 + g.skip_w)) {
                                    C[off + e] = xr[e];
                                    C[pe + off + e] = xi[e];
                                }
                        }
                    }
                    __syncwarp();
                }
            }
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    }
    __syncthreads();
    if (warp == 1) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS)
                     : "memory");
    }
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn get_encode() {
    static const EncodeTiledFn fn = [] {   // thread-safe static initialisation
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            return (EncodeTiledFn)p;
        cudaGetLastError();
        return (EncodeTiledFn) nullptr;
    }();
    return fn;
}

bool encode_pool(const Pool<float>& P, int box_rows, CUtensorMap* out) {
    EncodeTiledFn enc = get_encode();
    if (!enc || !P.base) return false;
    cuuint64_t dims[3] = {(cuuint64_t)P.cols, (cuuint64_t)P.rows, (cuuint64_t)(P.count * P.planes)};
    cuuint64_t strides[2] = {(cuuint64_t)P.ld * 4, (cuuint64_t)P.rows * P.ld * 4};
    cuuint32_t box[3] = {(cuuint32_t)BK, (cuuint32_t)box_rows, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = enc(out, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, (void*)P.base, dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_32B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

}  // namespace

bool tc_make_map(const Pool<float>& P, CUtensorMap* box128, CUtensorMap* box256, CUtensorMap* box64) {
    if ((P.planes != 2 && P.planes != 4) || (P.ld % 4) != 0) return false;
    return encode_pool(P, 128, box128) && encode_pool(P, 256, box256) && encode_pool(P, 64, box64);
}

bool tc_make_maps(const Pool<float>* D, const Pool<float>* C, const Pool<float>* X, const Pool<float>* GP,
                  const Pool<float>* RP, TcMaps* out) {
    const Pool<float>* pools[5] = {D, C, X, GP, RP};
    for (int i = 0; i < 5; ++i)
        if (!tc_make_map(*pools[i], &out->map[i][0], &out->map[i][1], &out->map[i][2])) return false;
    return true;
}

namespace {
template <int BN, int TWO = 0>
int tc_launch_bn(const GemmArgs<float>* g, const int* c_trans_arr, const CUtensorMap* mapA, const CUtensorMap* mapB,
                 int njobs, cudaStream_t stream) {
    typedef TcTile<BN, TWO> Tile;
    static const cudaError_t attr =
        cudaFuncSetAttribute(gemm_tc_kernel<BN, TWO>, cudaFuncAttributeMaxDynamicSharedMemorySize, Tile::SMEM_BYTES);
    if (attr != cudaSuccess) return (int)attr;
    TcParams P;
    P.g = *g;
    if (c_trans_arr) P.g.c_trans_arr = c_trans_arr;
    dim3 grid((g->N + BN - 1) / BN, (g->M + BM - 1) / BM, njobs * (g->ksplit > 1 ? g->ksplit : 1));
    gemm_tc_kernel<BN, TWO><<<grid, Tile::THREADS, Tile::SMEM_BYTES, stream>>>(*mapA, *mapB, P);
    return (int)cudaGetLastError();
}
}  // namespace

// Split-K sum: C[c_slot[job]] = alpha·Σ_{s<ks} W[job·ks + s] (+ C itself when beta), the
// slices added in order (deterministic); stored transposed (Cᵀ) when trans, through a
// 32 x 32 shared tile so both the reads and the writes coalesce.
// grid (ceil(N/32), ceil(M/32), njobs), block (32, 8)
__global__ void splitk_sum_kernel(Pool<float> W, int ks, Pool<float> Cp, const int* c_slot, const int* c_trans_arr,
                                  int c_trans, int M, int N, float alpha, int beta) {
    __shared__ float t[2][32][33];
    const int job = blockIdx.z;
    const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const long long wpe = W.plane_elems(), cpe = Cp.plane_elems();
    float* C = Cp.slot(c_slot[job]);
    const int tr = c_trans_arr ? c_trans_arr[job] : c_trans;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int r = r0 + ty + 8 * q, c = c0 + tx;
        float sr = 0.f, si = 0.f;
        if (r < M && c < N) {
            for (int s = 0; s < ks; ++s) {
                const float* w = W.slot((long long)job * ks + s) + (long long)r * W.ld + c;
                sr += w[0];
                si += w[wpe];
            }
            sr *= alpha;
            si *= alpha;
            if (!tr) {
                const long long o = (long long)r * Cp.ld + c;
                if (beta) { sr += C[o]; si += C[cpe + o]; }
                C[o] = sr;
                C[cpe + o] = si;
            }
        }
        t[0][ty + 8 * q][tx] = sr;
        t[1][ty + 8 * q][tx] = si;
    }
    if (!tr) return;   // uniform per block
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int cl = ty + 8 * q;
        const int cc = c0 + cl, rr = r0 + tx;
        if (cc < N && rr < M) {
            const long long o = (long long)cc * Cp.ld + rr;
            C[o] = t[0][tx][cl];
            C[cpe + o] = t[1][tx][cl];
        }
    }
}

int tc_splitk_sum(const Pool<float>& W, int ks, const Pool<float>& C, const int* c_slot, const int* c_trans_arr,
                  int c_trans, int njobs, int M, int N, float alpha, int beta, cudaStream_t stream) {
    splitk_sum_kernel<<<dim3((N + 31) / 32, (M + 31) / 32, njobs), dim3(32, 8), 0, stream>>>(
        W, ks, C, c_slot, c_trans_arr, c_trans, M, N, alpha, beta);
    return (int)cudaGetLastError();
}

int tc_gemm_launch_maps(const GemmArgs<float>* g, const int* c_trans_arr, const CUtensorMap* mapA,
                        const CUtensorMap* mapB, int bn, int njobs, cudaStream_t stream) {
    switch (bn) {
        case 256: return tc_launch_bn<256>(g, c_trans_arr, mapA, mapB, njobs, stream);
        case 128: return tc_launch_bn<128>(g, c_trans_arr, mapA, mapB, njobs, stream);
        case TC_BN128_TWO: return tc_launch_bn<128, 1>(g, c_trans_arr, mapA, mapB, njobs, stream);
        case 64: return tc_launch_bn<64>(g, c_trans_arr, mapA, mapB, njobs, stream);
        default: return (int)cudaErrorInvalidValue;
    }
}

int tc_pick_bn(int M, int N, int K, int njobs, int num_sms) {
    const long long mt = (M + BM - 1) / BM;
    auto tiles = [&](int bn) { return mt * ((N + bn - 1) / bn) * njobs; };
    // no wider than the product (a narrow column window would idle most of a wide tile)
    if (N > 128 && tiles(256) >= num_sms) return 256;
    if (N > 64 && tiles(128) >= num_sms) return 128;
    return 64;
}
