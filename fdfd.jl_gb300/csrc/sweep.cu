// Forward/backward sweeps of the cyclic-reduction solve: batched complex
// matrix-vector products (1..8 right-hand sides) on node-planar vectors.
// They stream every factor block once per sweep, so they are HBM-bound; both
// kernels issue all of a thread's 16-byte loads for a row (or a group of rows)
// before the first FMA so that enough bytes are in flight per SM.
#include <algorithm>

#include "common.cuh"
#include "kernels.cuh"

namespace {

template <typename T> struct V16;
template <> struct V16<float> { typedef float4 type; };
template <> struct V16<double> { typedef double2 type; };

template <typename T> __device__ __forceinline__ typename V16<T>::type ld16(const T* p) {
    return __ldcs(reinterpret_cast<const typename V16<T>::type*>(p));
}
template <typename T> __device__ __forceinline__ typename V16<T>::type zero16() {
    typename V16<T>::type v;
    T* e = reinterpret_cast<T*>(&v);
#pragma unroll
    for (int i = 0; i < (int)(16 / sizeof(T)); ++i) e[i] = 0;
    return v;
}

// stage the (up to two) input vectors of a job into shared memory, zero padded:
// sv[((t*R + r)*2 + plane)*bpad + i]
template <typename T>
__device__ void stage_vectors(const GemvArgs<T>& g, const int mslot[2], const int vnode[2], T* sv, int R, int bpad) {
    const T* V[2] = {g.V1, g.V2};
    for (int t = 0; t < 2; ++t) {
        if (mslot[t] < 0) continue;
        const T* v = V[t] + ((size_t)vnode[t] * g.rtot + g.r0) * 2 * g.ld;
        for (int rp = 0; rp < 2 * R; ++rp) {   // (right-hand side, plane) = (rp / 2, rp % 2)
            const T* src = v + (size_t)rp * g.ld;
            T* dst = sv + ((size_t)t * 2 * R + rp) * bpad;
            const bool live = rp / 2 < g.nrhs;
            for (int i = threadIdx.x; i < bpad; i += blockDim.x) dst[i] = (live && i < g.b) ? src[i] : (T)0;
        }
    }
}

}  // namespace

// N-form (row-major blocks): warp per row, lanes over 16-byte column groups.
// grid: (ceil(b/(8*rpw)), njobs), block 256 (8 warps x rpw rows)
template <typename T, int R>
__global__ void __launch_bounds__(256) gemv_n_kernel(GemvArgs<T> g) {
    constexpr int VW = 16 / sizeof(T);
    constexpr int CW = 32 * VW;       // columns per warp-wide load
    constexpr int GRP = 4;            // column chunks whose loads are issued together
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* sv = reinterpret_cast<T*>(smem_raw);
    const int b = g.b;
    const int nch = (b + CW - 1) / CW;
    const int bpad = nch * CW;
    const int4 J = g.jobs[blockIdx.y];
    const int2 Y = g.yjobs[blockIdx.y];
    const int mslot[2] = {J.x, J.z}, vnode[2] = {J.y, J.w};
    stage_vectors<T>(g, mslot, vnode, sv, R, bpad);
    __syncthreads();
    T* y = g.Y + ((size_t)Y.x * g.rtot + g.r0) * 2 * g.ld;
    const T* y0 = Y.y >= 0 ? g.Y0 + ((size_t)Y.y * g.rtot + g.r0) * 2 * g.ld : nullptr;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int rpw = g.rpw;
    for (int q = 0; q < rpw; ++q) {
        const int row = (blockIdx.x * 8 + warp) * rpw + q;
        if (row >= b) break;
        T ar[R], ai[R];
#pragma unroll
        for (int r = 0; r < R; ++r) { ar[r] = 0; ai[r] = 0; }
        for (int t = 0; t < 2; ++t) {
            if (mslot[t] < 0) continue;
            const Pool<T>& P = t ? g.P2 : g.P1;
            const T* Mr = P.slot(mslot[t]) + (size_t)row * P.ld;
            const T* Mi = Mr + P.plane_elems();
            const T* vt = sv + (size_t)t * R * 2 * bpad;
            for (int c0 = 0; c0 < nch; c0 += GRP) {
                typename V16<T>::type mr[GRP], mi[GRP];
#pragma unroll
                for (int u = 0; u < GRP; ++u) {
                    const int c = (c0 + u) * CW + lane * VW;
                    if (c0 + u < nch && c < b) { mr[u] = ld16<T>(Mr + c); mi[u] = ld16<T>(Mi + c); }
                    else { mr[u] = zero16<T>(); mi[u] = zero16<T>(); }
                }
#pragma unroll
                for (int u = 0; u < GRP; ++u) {
                    const int c = (c0 + u) * CW + lane * VW;
                    const T* er = reinterpret_cast<const T*>(&mr[u]);
                    const T* ei = reinterpret_cast<const T*>(&mi[u]);
                    // the 16-byte vector is inside the row, in its padding, or (b not a multiple
                    // of VW) straddles b: its entries at b and beyond are zeroed, and the input
                    // vector's padding is zero, so they add nothing
                    if (c < b) {
                        if (c + VW > b) {
#pragma unroll
                            for (int e = 0; e < VW; ++e)
                                if (c + e >= b) {
                                    reinterpret_cast<T*>(&mr[u])[e] = 0;
                                    reinterpret_cast<T*>(&mi[u])[e] = 0;
                                }
                        }
#pragma unroll
                        for (int r = 0; r < R; ++r) {
                            const typename V16<T>::type v_r =
                                *reinterpret_cast<const typename V16<T>::type*>(vt + (r * 2) * bpad + c);
                            const typename V16<T>::type v_i =
                                *reinterpret_cast<const typename V16<T>::type*>(vt + (r * 2 + 1) * bpad + c);
                            const T* xr = reinterpret_cast<const T*>(&v_r);
                            const T* xi = reinterpret_cast<const T*>(&v_i);
#pragma unroll
                            for (int e = 0; e < VW; ++e) {
                                ar[r] = fma(er[e], xr[e], ar[r]); ar[r] = fma(-ei[e], xi[e], ar[r]);
                                ai[r] = fma(er[e], xi[e], ai[r]); ai[r] = fma(ei[e], xr[e], ai[r]);
                            }
                        }
                    }
                }
            }
        }
#pragma unroll
        for (int r = 0; r < R; ++r)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                ar[r] += __shfl_down_sync(0xffffffffu, ar[r], o);
                ai[r] += __shfl_down_sync(0xffffffffu, ai[r], o);
            }
        if (lane == 0) {
#pragma unroll
            for (int r = 0; r < R; ++r) {
                if (r >= g.nrhs) break;
                T br = 0, bi = 0;
                if (y0) { br = y0[(r * 2) * g.ld + row]; bi = y0[(r * 2 + 1) * g.ld + row]; }
                y[(r * 2) * g.ld + row] = br + g.alpha * ar[r];
                y[(r * 2 + 1) * g.ld + row] = bi + g.alpha * ai[r];
            }
        }
    }
}

// N-form product fed by bulk copies: each warp owns rows row_base .. row_base+RW-1
// and streams them (both planes of every block of the job) into a private ring of
// shared-memory slots with cp.async.bulk, one mbarrier per slot, so the bytes in
// flight are bounded by shared memory rather than by registers.  The warp then
// works like gemv_n_kernel on a row (lanes over 16-byte column vectors, the same
// per-lane order of the fmas and the same shuffle reduction), so both kernels give
// identical results.  Slot s is refilled with row k + nslot once the warp has
// finished row k (a __syncwarp, then a proxy fence orders the generic reads before
// the asynchronous write).  Every slot wait is bounded (FDFD_WAIT_LIMIT_NS); a wait
// that runs out sets FDFD_DEVERR_TIMEOUT and the warp waits (bounded) for the copies
// it has issued before it leaves.
// grid: (ceil(b/(8*RW)), njobs), block 256, dynamic shared memory
// gemv_nb_smem<T, R>(b) + 8 * ring_bytes; ring_bytes a multiple of 16 holding at
// least one slot of two blocks (4 row planes of ceil16(b·sizeof(T)) bytes).
template <typename T, int R>
__host__ __device__ constexpr size_t gemv_nb_smem(int b) {
    return ((size_t)2 * R * 2 * ((b + 32 * (16 / sizeof(T)) - 1) / (32 * (16 / sizeof(T))) * 32 * (16 / sizeof(T))) *
                sizeof(T) + 127) / 128 * 128;
}

template <typename T, int R>
__global__ void __launch_bounds__(256) gemv_nb_kernel(GemvArgs<T> g, int RW, int ring_bytes) {
    constexpr int VW = 16 / sizeof(T);
    constexpr int CW = 32 * VW;
    constexpr int MAXS = 8;
    typedef typename V16<T>::type VT;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bars[8][MAXS];
    T* sv = reinterpret_cast<T*>(smem_raw);
    const int b = g.b;
    const int nch = (b + CW - 1) / CW;
    const int bpad = nch * CW;
    const int4 J = g.jobs[blockIdx.y];
    const int2 Y = g.yjobs[blockIdx.y];
    const int mslot[2] = {J.x, J.z}, vnode[2] = {J.y, J.w};
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int rb = (b * (int)sizeof(T) + 15) & ~15;     // bytes copied per row and plane
    const int nm = (mslot[0] >= 0 ? 1 : 0) + (mslot[1] >= 0 ? 1 : 0);
    const int slot_bytes = (nm > 0 ? nm : 1) * 2 * rb;
    const int nslot = min(MAXS, ring_bytes / slot_bytes);   // >= 1 by the launcher's sizing
    unsigned char* ring = smem_raw + gemv_nb_smem<T, R>(b) + (size_t)warp * ring_bytes;
    if (lane == 0)
        for (int q = 0; q < nslot; ++q) mbar_init(smem_u32(&bars[warp][q]), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    stage_vectors<T>(g, mslot, vnode, sv, R, bpad);
    __syncthreads();
    const int row_base = (blockIdx.x * 8 + warp) * RW;
    const int nrows = max(0, min(RW, b - row_base));
    // lane 0: the planes of row row_base + k of every block of the job into slot k % nslot
    auto issue = [&](int k) {
        const int q = k % nslot, row = row_base + k;
        const uint32_t bar = smem_u32(&bars[warp][q]);
        const uint32_t dst = smem_u32(ring + (size_t)q * slot_bytes);
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(nm * 2 * rb)
                     : "memory");
        int m = 0;
        for (int t = 0; t < 2; ++t) {
            if (mslot[t] < 0) continue;
            const Pool<T>& P = t ? g.P2 : g.P1;
            const T* src = P.slot(mslot[t]) + (size_t)row * P.ld;
#pragma unroll
            for (int pl = 0; pl < 2; ++pl)
                asm volatile(
                    "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                        dst + (uint32_t)((2 * m + pl) * rb)),
                    "l"(src + pl * P.plane_elems()), "r"(rb), "r"(bar)
                    : "memory");
            ++m;
        }
    };
    if (lane == 0 && nm > 0)
        for (int k = 0; k < min(nslot, nrows); ++k) issue(k);
    T* y = g.Y + ((size_t)Y.x * g.rtot + g.r0) * 2 * g.ld;
    const T* y0 = Y.y >= 0 ? g.Y0 + ((size_t)Y.y * g.rtot + g.r0) * 2 * g.ld : nullptr;
    int k = 0;
    bool ok = true;
    for (; k < nrows; ++k) {
        const int q = k % nslot, row = row_base + k;
        if (nm > 0) {   // a job without blocks only writes y0 (or zero)
            const bool okl = mbar_wait(smem_u32(&bars[warp][q]), (uint32_t)((k / nslot) & 1), FDFD_WAIT_LIMIT_NS);
            if (!__all_sync(0xffffffffu, okl)) {
                ok = false;
                break;
            }
        }
        const unsigned char* slot = ring + (size_t)q * slot_bytes;
        T ar[R], ai[R];
#pragma unroll
        for (int r = 0; r < R; ++r) { ar[r] = 0; ai[r] = 0; }
        int m = 0;
        for (int t = 0; t < 2; ++t) {
            if (mslot[t] < 0) continue;
            const T* Mr = reinterpret_cast<const T*>(slot + (size_t)(2 * m) * rb);
            const T* Mi = reinterpret_cast<const T*>(slot + (size_t)(2 * m + 1) * rb);
            const T* vt = sv + (size_t)t * R * 2 * bpad;
            ++m;
            for (int ch = 0; ch < nch; ++ch) {
                const int c = ch * CW + lane * VW;
                if (c >= b) continue;
                VT mr = *reinterpret_cast<const VT*>(Mr + c), mi = *reinterpret_cast<const VT*>(Mi + c);
                if (c + VW > b) {   // b not a multiple of VW: entries at b and beyond add nothing
#pragma unroll
                    for (int e = 0; e < VW; ++e)
                        if (c + e >= b) {
                            reinterpret_cast<T*>(&mr)[e] = 0;
                            reinterpret_cast<T*>(&mi)[e] = 0;
                        }
                }
                const T* er = reinterpret_cast<const T*>(&mr);
                const T* ei = reinterpret_cast<const T*>(&mi);
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const VT v_r = *reinterpret_cast<const VT*>(vt + (r * 2) * bpad + c);
                    const VT v_i = *reinterpret_cast<const VT*>(vt + (r * 2 + 1) * bpad + c);
                    const T* xr = reinterpret_cast<const T*>(&v_r);
                    const T* xi = reinterpret_cast<const T*>(&v_i);
#pragma unroll
                    for (int e = 0; e < VW; ++e) {
                        ar[r] = fma(er[e], xr[e], ar[r]); ar[r] = fma(-ei[e], xi[e], ar[r]);
                        ai[r] = fma(er[e], xi[e], ai[r]); ai[r] = fma(ei[e], xr[e], ai[r]);
                    }
                }
            }
        }
#pragma unroll
        for (int r = 0; r < R; ++r)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                ar[r] += __shfl_down_sync(0xffffffffu, ar[r], o);
                ai[r] += __shfl_down_sync(0xffffffffu, ai[r], o);
            }
        if (lane == 0) {
#pragma unroll
            for (int r = 0; r < R; ++r) {
                if (r >= g.nrhs) break;
                T br = 0, bi = 0;
                if (y0) { br = y0[(r * 2) * g.ld + row]; bi = y0[(r * 2 + 1) * g.ld + row]; }
                y[(r * 2) * g.ld + row] = br + g.alpha * ar[r];
                y[(r * 2 + 1) * g.ld + row] = bi + g.alpha * ai[r];
            }
        }
        __syncwarp();   // every lane is done with slot q
        if (lane == 0 && nm > 0 && k + nslot < nrows) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            issue(k + nslot);
        }
    }
    if (!ok) {
        // row k's wait ran out: report it, then let this warp's issued copies land
        if (lane == 0) dev_error(g.err, FDFD_DEVERR_TIMEOUT);
        const int issued = min(nrows, k + nslot);
        for (int kk = k; kk < issued; ++kk)
            (void)mbar_wait(smem_u32(&bars[warp][kk % nslot]), (uint32_t)((kk / nslot) & 1), FDFD_WAIT_LIMIT_NS);
    }
}

// Stored-transpose form (row-major Mᵀ): y[i] = Σ_j Mᵀ[j][i] v[j].  A lane owns
// VW consecutive outputs (one 16-byte load per row j); a group of og lanes
// covers og*VW outputs, the 8*(32/og) lane groups of the block split the j
// range, and the partial sums are reduced through shared memory.
// grid: (ceil(b/(og*VW)), njobs), block 256
template <typename T, int R>
__global__ void __launch_bounds__(256) gemv_t_kernel(GemvArgs<T> g) {
    constexpr int VW = 16 / sizeof(T);
    constexpr int U = 4;              // rows j whose loads are issued together
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int b = g.b;
    const int bpad = (b + 31) / 32 * 32;
    T* sv = reinterpret_cast<T*>(smem_raw);
    T* red = sv + (size_t)2 * R * 2 * bpad;          // [group][out][r][re|im]
    const int4 J = g.jobs[blockIdx.y];
    const int2 Y = g.yjobs[blockIdx.y];
    const int mslot[2] = {J.x, J.z}, vnode[2] = {J.y, J.w};
    stage_vectors<T>(g, mslot, vnode, sv, R, bpad);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int og = g.og, ngrp = 32 / og;          // lanes per output group, groups per warp
    const int grp = lane / og, sub = lane % og;
    const int nout = og * VW;                     // outputs of this block
    const int pid = warp * ngrp + grp;            // partial-sum index, 0 .. 8*ngrp-1
    const int rstride = 8 * ngrp;                 // j stride between a group's rows
    const int i0 = blockIdx.x * nout + sub * VW;
    T ar[VW][R], ai[VW][R];
#pragma unroll
    for (int e = 0; e < VW; ++e)
#pragma unroll
        for (int r = 0; r < R; ++r) { ar[e][r] = 0; ai[e][r] = 0; }
    if (i0 < b) {
        for (int t = 0; t < 2; ++t) {
            if (mslot[t] < 0) continue;
            const Pool<T>& P = t ? g.P2 : g.P1;
            const T* Mr = P.slot(mslot[t]) + i0;
            const T* Mi = Mr + P.plane_elems();
            const T* vt = sv + (size_t)t * R * 2 * bpad;
            for (int j0 = pid; j0 < b; j0 += rstride * U) {
                typename V16<T>::type mr[U], mi[U];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const int j = j0 + rstride * u;
                    if (j < b) {
                        mr[u] = ld16<T>(Mr + (size_t)j * P.ld);
                        mi[u] = ld16<T>(Mi + (size_t)j * P.ld);
                    } else {
                        mr[u] = zero16<T>(); mi[u] = zero16<T>();
                    }
                }
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const int j = j0 + rstride * u;
                    if (j < b) {
                        const T* er = reinterpret_cast<const T*>(&mr[u]);
                        const T* ei = reinterpret_cast<const T*>(&mi[u]);
#pragma unroll
                        for (int r = 0; r < R; ++r) {
                            const T vr = vt[(r * 2) * bpad + j], vi = vt[(r * 2 + 1) * bpad + j];
#pragma unroll
                            for (int e = 0; e < VW; ++e) {
                                ar[e][r] = fma(er[e], vr, ar[e][r]); ar[e][r] = fma(-ei[e], vi, ar[e][r]);
                                ai[e][r] = fma(er[e], vi, ai[e][r]); ai[e][r] = fma(ei[e], vr, ai[e][r]);
                            }
                        }
                    }
                }
            }
        }
    }
    // cross-group reduction
#pragma unroll
    for (int e = 0; e < VW; ++e)
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const size_t o = (((size_t)pid * nout + sub * VW + e) * R + r) * 2;
            red[o] = ar[e][r];
            red[o + 1] = ai[e][r];
        }
    __syncthreads();
    T* y = g.Y + ((size_t)Y.x * g.rtot + g.r0) * 2 * g.ld;
    const T* y0 = Y.y >= 0 ? g.Y0 + ((size_t)Y.y * g.rtot + g.r0) * 2 * g.ld : nullptr;
    for (int idx = threadIdx.x; idx < nout * g.nrhs; idx += blockDim.x) {
        const int out = idx % nout, r = idx / nout;
        const int i = blockIdx.x * nout + out;
        if (i >= b) continue;
        T sr = 0, si = 0;
        for (int w = 0; w < rstride; ++w) {
            const size_t o = (((size_t)w * nout + out) * R + r) * 2;
            sr += red[o];
            si += red[o + 1];
        }
        T br = 0, bi = 0;
        if (y0) { br = y0[(r * 2) * g.ld + i]; bi = y0[(r * 2 + 1) * g.ld + i]; }
        y[(r * 2) * g.ld + i] = br + g.alpha * sr;
        y[(r * 2 + 1) * g.ld + i] = bi + g.alpha * si;
    }
}

// First reduction step with diagonal couplings (scaled stencil values).
// jobs: (node, prev, next, flags) with flags bit0 = prev participates, bit1 = next participates.
// mode 0: dst[node] -= u_node ⊙ src[next] + l_node ⊙ src[prev]   (forward, survivors)
// mode 1: dst[node]  = l_node ⊙ src[prev] + u_node ⊙ src[next]   (backward, eliminated)
// grid: (ceil(b/256), njobs), block 256
template <typename T>
__global__ void diag_sweep_kernel(NodeMap m, const cplx<T>* tab, int nrhs, const int4* jobs, int mode, const T* src,
                                  T* dst) {
    const int4 J = jobs[blockIdx.y];
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.b) return;
    // the node's scaled couplings from the factorization's stencil table (contiguous in i)
    const cplx<T> l = tab[((size_t)J.x * 5 + m.p_cprev()) * m.b + i];
    const cplx<T> u = tab[((size_t)J.x * 5 + m.p_cnext()) * m.b + i];
    const int ld = m.ld;
    for (int r = 0; r < nrhs; ++r) {
        cplx<T> acc = cmk((T)0, (T)0);
        if (J.w & 1) {
            const T* s = src + ((size_t)J.y * nrhs + r) * 2 * ld;
            acc = cadd(acc, cmul(l, cmk(s[i], s[ld + i])));
        }
        if (J.w & 2) {
            const T* s = src + ((size_t)J.z * nrhs + r) * 2 * ld;
            acc = cadd(acc, cmul(u, cmk(s[i], s[ld + i])));
        }
        T* d = dst + ((size_t)J.x * nrhs + r) * 2 * ld;
        if (mode == 0) {
            d[i] -= acc.re;
            d[ld + i] -= acc.im;
        } else {
            d[i] = acc.re;
            d[ld + i] = acc.im;
        }
    }
}

// First-step sweep products y = y0 + alpha·D_k⁻¹ v without the dense inverse:
// D_k = T0 + corners (the first reduction step's cyclic tridiagonal block) is
// applied through its stored factorization (tri_factor_kernel's workspace:
// the xGTTRF factors of T0 and the Sherman-Morrison-Woodbury terms),
//     D_k⁻¹ v = T0⁻¹ v − z0 (w0·v) − zN (w1·v),
// with the xGTTRS recurrences for T0⁻¹.  That reads 8b complex factor values
// per node instead of the b² of the dense inverse.
//
// One warp per node, the node's factors in shared memory.  Both recurrences
// are affine in their carried state, so the warp runs them as scans: each
// lane composes the maps of a contiguous chunk of steps, a shuffle scan of the
// 32 composed maps gives every lane the state entering its chunk, and the
// lanes replay their chunks.  Forward (L y = P v, interchanges between
// neighbours): the state is the pending entry s, and step i maps
//     no interchange:  y_i = s,       s ← −l_i s + v_{i+1}
//     interchange:     y_i = v_{i+1}, s ← s − l_i v_{i+1}
// with y_{b−1} the final state.  Backward (U x = y): the state is
// (x_i, x_{i+1}), and step i (from b−2 down to 0) maps it by
//     x_i = dinv_i (y_i − du_i x_{i+1} − du2_i x_{i+2}),
// a 2 x 2 complex matrix and a 2-vector.  The chain of one right-hand side
// is then about 2·b/32 steps per lane plus two 5-round scans instead of 2·b
// dependent steps on one lane.  The multipliers l_i of a partially pivoted
// factorization are at most one in magnitude, so the composed forward maps
// stay bounded.  The Woodbury dots come from a warp reduction over v.
// jobs[j] = node of factor workspace j; grid: njobs, block 32,
// dynamic smem 10b cplx<T> + b ints
template <typename T>
__device__ __forceinline__ cplx<T> shfl_up_c(cplx<T> z, int d) {
    return cmk(__shfl_up_sync(0xffffffffu, z.re, d), __shfl_up_sync(0xffffffffu, z.im, d));
}
template <typename T>
__device__ __forceinline__ cplx<T> shfl_idx_c(cplx<T> z, int src) {
    return cmk(__shfl_sync(0xffffffffu, z.re, src), __shfl_sync(0xffffffffu, z.im, src));
}
template <typename T>
__device__ __forceinline__ cplx<T> shfl_xor_c(cplx<T> z, int m) {
    return cmk(__shfl_xor_sync(0xffffffffu, z.re, m), __shfl_xor_sync(0xffffffffu, z.im, m));
}

template <typename T>
__global__ void __launch_bounds__(32) tri_apply_kernel(int b, int ld, int nrhs, int rc, const int* jobs,
                                                       const cplx<T>* __restrict__ fac, const int* __restrict__ piv,
                                                       const T* V, const T* Y0, T* Y, T alpha) {
    (void)rc;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cplx<T>* sf = reinterpret_cast<cplx<T>*>(smem_raw);      // dl du du2 dinv z0 zN w0 w1
    cplx<T>* sv = sf + 8 * (size_t)b;                          // v of the current right-hand side
    cplx<T>* sy = sv + b;                                      // y, then the output
    int* sp = reinterpret_cast<int*>(sy + b);
    const int j = blockIdx.x, lane = threadIdx.x;
    const int node = jobs[j];
    const cplx<T>* f = fac + (size_t)j * 8 * b;
    for (int i = lane; i < 8 * b; i += 32) sf[i] = f[i];
    for (int i = lane; i < b; i += 32) sp[i] = piv[(size_t)j * b + i];
    const cplx<T>* dl = sf;
    const cplx<T>* du = sf + b;
    const cplx<T>* du2 = sf + 2 * b;
    const cplx<T>* dinv = sf + 3 * b;
    const cplx<T>* z0 = sf + 4 * b;
    const cplx<T>* zN = sf + 5 * b;
    const cplx<T>* w0 = sf + 6 * b;
    const cplx<T>* w1 = sf + 7 * b;
    const cplx<T> one = cmk((T)1, (T)0), zero = cmk((T)0, (T)0);
    const int steps = b - 1;                      // both recurrences have b − 1 steps
    const int ch = (steps + 31) / 32;
    const int k0 = min(steps, lane * ch), k1 = min(steps, k0 + ch);
    for (int r = 0; r < nrhs; ++r) {
        const size_t vo = ((size_t)node * nrhs + r) * 2 * ld;
        const T* v = V + vo;
        __syncwarp();
        for (int i = lane; i < b; i += 32) sv[i] = cmk(v[i], v[ld + i]);
        __syncwarp();
        // Woodbury dots with the original v
        cplx<T> c0 = zero, c1 = zero;
        for (int i = lane; i < b; i += 32) {
            c0 = cadd(c0, cmul(w0[i], sv[i]));
            c1 = cadd(c1, cmul(w1[i], sv[i]));
        }
#pragma unroll
        for (int m = 16; m > 0; m >>= 1) {
            c0 = cadd(c0, shfl_xor_c(c0, m));
            c1 = cadd(c1, shfl_xor_c(c1, m));
        }
        // ---- forward: compose this lane's maps s ← a s + c
        cplx<T> A = one, C = zero;
        for (int i = k0; i < k1; ++i) {
            const cplx<T> xn = sv[i + 1];
            const bool keep = sp[i] == i;
            const cplx<T> a = keep ? cneg(dl[i]) : one;
            const cplx<T> c = keep ? xn : cneg(cmul(dl[i], xn));
            A = cmul(a, A);
            C = cadd(cmul(a, C), c);
        }
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const cplx<T> Ap = shfl_up_c(A, d), Cp = shfl_up_c(C, d);
            if (lane >= d) {
                C = cadd(cmul(A, Cp), C);
                A = cmul(A, Ap);
            }
        }
        const cplx<T> v0 = sv[0];
        {
            const cplx<T> Ae = shfl_up_c(A, 1), Ce = shfl_up_c(C, 1);
            const cplx<T> last = cadd(cmul(shfl_idx_c(A, 31), v0), shfl_idx_c(C, 31));
            cplx<T> st = lane == 0 ? v0 : cadd(cmul(Ae, v0), Ce);
            for (int i = k0; i < k1; ++i) {
                const cplx<T> xn = sv[i + 1];
                if (sp[i] == i) {
                    sy[i] = st;
                    st = csub(xn, cmul(dl[i], st));
                } else {
                    sy[i] = xn;
                    st = csub(st, cmul(dl[i], xn));
                }
            }
            if (lane == 0) sy[b - 1] = last;
        }
        __syncwarp();
        // ---- backward: compose this lane's maps (x_i, x_{i+1}) ← M (x_{i+1}, x_{i+2}) + t, i = b−2−k
        cplx<T> m00 = one, m01 = zero, m10 = zero, m11 = one, t0 = zero, t1 = zero;
        for (int k = k0; k < k1; ++k) {
            const int i = b - 2 - k;
            const cplx<T> g = dinv[i];
            const cplx<T> p = cneg(cmul(g, du[i])), q = cneg(cmul(g, du2[i]));   // row 0 of the step's matrix
            const cplx<T> u = cmul(g, sy[i]);
            // step ∘ current: [[p, q], [1, 0]]·M and [[p, q], [1, 0]]·t + (u, 0)
            const cplx<T> n00 = cadd(cmul(p, m00), cmul(q, m10)), n01 = cadd(cmul(p, m01), cmul(q, m11));
            const cplx<T> nt0 = cadd(cadd(cmul(p, t0), cmul(q, t1)), u);
            m10 = m00; m11 = m01; t1 = t0;
            m00 = n00; m01 = n01; t0 = nt0;
        }
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const cplx<T> a00 = shfl_up_c(m00, d), a01 = shfl_up_c(m01, d), a10 = shfl_up_c(m10, d),
                          a11 = shfl_up_c(m11, d), s0 = shfl_up_c(t0, d), s1 = shfl_up_c(t1, d);
            if (lane >= d) {
                // this lane's maps after the earlier lanes': M·A and M·s + t
                const cplx<T> n00 = cadd(cmul(m00, a00), cmul(m01, a10)), n01 = cadd(cmul(m00, a01), cmul(m01, a11));
                const cplx<T> n10 = cadd(cmul(m10, a00), cmul(m11, a10)), n11 = cadd(cmul(m10, a01), cmul(m11, a11));
                const cplx<T> nt0 = cadd(cadd(cmul(m00, s0), cmul(m01, s1)), t0);
                const cplx<T> nt1 = cadd(cadd(cmul(m10, s0), cmul(m11, s1)), t1);
                m00 = n00; m01 = n01; m10 = n10; m11 = n11; t0 = nt0; t1 = nt1;
            }
        }
        {
            const cplx<T> e00 = shfl_up_c(m00, 1), e01 = shfl_up_c(m01, 1), e10 = shfl_up_c(m10, 1),
                          e11 = shfl_up_c(m11, 1), f0 = shfl_up_c(t0, 1), f1 = shfl_up_c(t1, 1);
            const cplx<T> xl = cmul(sy[b - 1], dinv[b - 1]);      // state (x_{b−1}, 0) entering step b−2
            cplx<T> x0 = xl, x1 = zero;
            if (lane > 0) {
                x0 = cadd(cmul(e00, xl), f0);
                x1 = cadd(cmul(e10, xl), f1);
                (void)e01; (void)e11;
            }
            __syncwarp();
            for (int k = k0; k < k1; ++k) {
                const int i = b - 2 - k;
                const cplx<T> xv = cmul(csub(csub(sy[i], cmul(du[i], x0)), cmul(du2[i], x1)), dinv[i]);
                sy[i] = csub(csub(xv, cmul(z0[i], c0)), cmul(zN[i], c1));
                x1 = x0;
                x0 = xv;
            }
            if (lane == 0) sy[b - 1] = csub(csub(xl, cmul(z0[b - 1], c0)), cmul(zN[b - 1], c1));
        }
        __syncwarp();
        const T* y0 = Y0 ? Y0 + vo : nullptr;
        T* y = Y + vo;
        for (int i = lane; i < b; i += 32) {
            const cplx<T> g = sy[i];
            T o_r = alpha * g.re, o_i = alpha * g.im;
            if (y0) { o_r += y0[i]; o_i += y0[ld + i]; }
            y[i] = o_r;
            y[ld + i] = o_i;
        }
    }
}

namespace {
template <typename T, int R>
size_t gemv_smem(int tr, int b) {
    constexpr int VW = 16 / sizeof(T);
    if (tr) {
        const int bpad = (b + 31) / 32 * 32;
        return ((size_t)2 * R * 2 * bpad + (size_t)8 * 32 * VW * R * 2) * sizeof(T);
    }
    const int bpad = ceil_div(b, 32 * VW) * 32 * VW;
    return (size_t)2 * R * 2 * bpad * sizeof(T);
}

template <typename T, int R>
int gemv_launch_r(cudaStream_t s, int tr, int njobs, const GemvArgs<T>& g) {
    constexpr int VW = 16 / sizeof(T);
    static const cudaError_t attr = [] {   // thread-safe static initialisation
        cudaError_t e = cudaFuncSetAttribute(gemv_n_kernel<T, R>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             200 * 1024);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(gemv_t_kernel<T, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        return e;
    }();
    if (attr != cudaSuccess) return (int)attr;
    const size_t smem = gemv_smem<T, R>(tr, g.b);
    // Launch shape: the widest per-block tile that still gives about four blocks
    // per SM.  Small batches (the deep reduction levels) get narrow tiles, so
    // their few blocks are still spread over the whole GPU.
    const long long want = 4LL * (g.nsm > 0 ? g.nsm : 1);
    GemvArgs<T> a = g;
    if (tr) {
        a.og = 32;
        while (a.og > 8 && (long long)ceil_div(g.b, a.og * VW) * njobs < want) a.og >>= 1;
        if (g.shape == 8 || g.shape == 16 || g.shape == 32) a.og = g.shape;
        gemv_t_kernel<T, R><<<dim3(ceil_div(g.b, a.og * VW), njobs), 256, smem, s>>>(a);
    } else if (g.shape <= 0) {
        // bulk-copy pipeline: per warp a ring of three slots of the launch's blocks per job
        // (at least two slots, and one slot of two blocks), inside 200 KB of shared memory
        static const cudaError_t attr_nb = cudaFuncSetAttribute(
            gemv_nb_kernel<T, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        if (attr_nb != cudaSuccess) return (int)attr_nb;
        const size_t rb = (size_t)(g.b * (int)sizeof(T) + 15) / 16 * 16;
        const size_t svb = gemv_nb_smem<T, R>(g.b);
        const size_t nmx = g.nmat > 1 ? 2 : 1;
        size_t ring = 3 * nmx * 2 * rb;
        if (svb + 8 * ring > 200 * 1024) ring = (200 * 1024 - std::min<size_t>(svb, 200 * 1024)) / 8 / 16 * 16;
        if (ring >= 2 * nmx * 2 * rb && ring >= 4 * rb) {
            int rw = 8;
            while (rw > 1 && (long long)ceil_div(g.b, 8 * rw) * njobs < 2 * want / 4) rw >>= 1;
            if (g.shape == -2 || g.shape == -4 || g.shape == -8) rw = -g.shape;
            gemv_nb_kernel<T, R><<<dim3(ceil_div(g.b, 8 * rw), njobs), 256, svb + 8 * ring, s>>>(a, rw, (int)ring);
            return (int)cudaGetLastError();
        }
        a.rpw = 4;
        while (a.rpw > 1 && (long long)ceil_div(g.b, 8 * a.rpw) * njobs < want) a.rpw >>= 1;
        gemv_n_kernel<T, R><<<dim3(ceil_div(g.b, 8 * a.rpw), njobs), 256, smem, s>>>(a);
    } else {
        a.rpw = 4;
        while (a.rpw > 1 && (long long)ceil_div(g.b, 8 * a.rpw) * njobs < want) a.rpw >>= 1;
        if (g.shape == 1 || g.shape == 2 || g.shape == 4) a.rpw = g.shape;
        gemv_n_kernel<T, R><<<dim3(ceil_div(g.b, 8 * a.rpw), njobs), 256, smem, s>>>(a);
    }
    return (int)cudaGetLastError();
}
}  // namespace

// g.nrhs must not exceed gemv_max_rhs<T>(b).
template <typename T>
int launch_gemv(cudaStream_t s, int tr, int njobs, const GemvArgs<T>& g) {
    if (g.nrhs <= 1) return gemv_launch_r<T, 1>(s, tr, njobs, g);
    if (g.nrhs <= 2) return gemv_launch_r<T, 2>(s, tr, njobs, g);
    if (g.nrhs <= 4) return gemv_launch_r<T, 4>(s, tr, njobs, g);
    return gemv_launch_r<T, 8>(s, tr, njobs, g);
}

// largest right-hand-side count (8, 4, 2 or 1) whose shared memory fits both forms
template <typename T>
int gemv_max_rhs(int b) {
    if (gemv_smem<T, 8>(1, b) <= 200 * 1024) return 8;
    if (gemv_smem<T, 4>(1, b) <= 200 * 1024) return 4;
    if (gemv_smem<T, 2>(1, b) <= 200 * 1024) return 2;
    return 1;
}

template <typename T>
void launch_diag_sweep(cudaStream_t s, int njobs, NodeMap m, const cplx<T>* tab, int nrhs, const int4* jobs,
                       int mode, const T* src, T* dst) {
    diag_sweep_kernel<T><<<dim3(ceil_div(m.b, 256), njobs), 256, 0, s>>>(m, tab, nrhs, jobs, mode, src, dst);
}
template <typename T>
int launch_tri_apply(cudaStream_t s, int b, int ld, int njobs, int nrhs, const int* jobs, const cplx<T>* fac,
                     const int* piv, const T* V, const T* Y0, T* Y, T alpha) {
    if (njobs == 0 || nrhs == 0) return 0;
    const size_t smem = 10 * (size_t)b * sizeof(cplx<T>) + (size_t)b * sizeof(int);
    if (smem > 200 * 1024) return (int)cudaErrorInvalidValue;
    static const cudaError_t attr = cudaFuncSetAttribute(tri_apply_kernel<T>,
                                                         cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    if (attr != cudaSuccess) return (int)attr;
    tri_apply_kernel<T><<<njobs, 32, smem, s>>>(b, ld, nrhs, 1, jobs, fac, piv, V, Y0, Y, alpha);
    return (int)cudaGetLastError();
}
template int launch_tri_apply<float>(cudaStream_t, int, int, int, int, const int*, const cplx<float>*, const int*,
                                     const float*, const float*, float*, float);
template int launch_tri_apply<double>(cudaStream_t, int, int, int, int, const int*, const cplx<double>*, const int*,
                                      const double*, const double*, double*, double);
template int launch_gemv<float>(cudaStream_t, int, int, const GemvArgs<float>&);
template int launch_gemv<double>(cudaStream_t, int, int, const GemvArgs<double>&);
template int gemv_max_rhs<float>(int);
template int gemv_max_rhs<double>(int);
template void launch_diag_sweep<float>(cudaStream_t, int, NodeMap, const cplx<float>*, int, const int4*,
                                       int, const float*, float*);
template void launch_diag_sweep<double>(cudaStream_t, int, NodeMap, const cplx<double>*, int, const int4*,
                                        int, const double*, double*);
