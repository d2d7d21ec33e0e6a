// Forward/backward sweeps of the cyclic-reduction solve: batched complex
// matrix-vector products (1..8 right-hand sides) on node-planar vectors.
// These are HBM-bound: every factor matrix is streamed once per sweep.
#include "common.cuh"
#include "kernels.cuh"

#define GEMV_MAXR 8

// TR = 0: matrices stored N-form (row-major), warp per row, lanes over columns.
// TR = 1: matrices stored as their transpose (row-major Mᵀ): thread per output
//         row i reads column i of the stored array, coalesced across threads.
// grid: (ceil(b/32), njobs), block 256 (8 warps); dynamic smem 2 terms x b x nrhs complex.
template <typename T, int TR>
__global__ void __launch_bounds__(256) gemv_kernel(GemvArgs<T> g) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* sv = reinterpret_cast<T*>(smem_raw);        // [term][rhs][plane][b]
    const int b = g.b, ld = g.ld, R = g.nrhs;
    const int4 J = g.jobs[blockIdx.y];
    const int2 Y = g.yjobs[blockIdx.y];
    const int tid = threadIdx.x;
    const int mslot[2] = {J.x, J.z}, vnode[2] = {J.y, J.w};
    const T* V[2] = {g.V1, g.V2};
    // stage the input vectors
    for (int t = 0; t < 2; ++t) {
        if (mslot[t] < 0) continue;
        const T* v = V[t] + ((size_t)vnode[t] * g.rtot + g.r0) * 2 * ld;
        for (int idx = tid; idx < R * 2 * b; idx += blockDim.x) {
            int r = idx / (2 * b), rem = idx % (2 * b), p = rem / b, i = rem % b;
            sv[((size_t)t * R + r) * 2 * b + p * b + i] = v[((size_t)r * 2 + p) * ld + i];
        }
    }
    __syncthreads();
    T* y = g.Y + ((size_t)Y.x * g.rtot + g.r0) * 2 * ld;
    const T* y0 = Y.y >= 0 ? g.Y0 + ((size_t)Y.y * g.rtot + g.r0) * 2 * ld : nullptr;
    if (TR == 0) {
        const int warp = tid >> 5, lane = tid & 31;
        for (int q = 0; q < 4; ++q) {
            int row = blockIdx.x * 32 + warp * 4 + q;
            if (row >= b) break;
            T ar[GEMV_MAXR], ai[GEMV_MAXR];
#pragma unroll
            for (int r = 0; r < GEMV_MAXR; ++r) { ar[r] = 0; ai[r] = 0; }
            for (int t = 0; t < 2; ++t) {
                if (mslot[t] < 0) continue;
                const Pool<T>& P = t ? g.P2 : g.P1;
                const T* Mr = P.slot(mslot[t]) + (size_t)row * P.ld;
                const T* Mi = Mr + P.plane_elems();
                const T* vt = sv + (size_t)t * R * 2 * b;
                for (int j = lane; j < b; j += 32) {
                    T mr = Mr[j], mi = Mi[j];
#pragma unroll
                    for (int r = 0; r < GEMV_MAXR; ++r) {
                        if (r >= R) break;
                        T vr = vt[(r * 2) * b + j], vi = vt[(r * 2 + 1) * b + j];
                        ar[r] = fma(mr, vr, ar[r]); ar[r] = fma(-mi, vi, ar[r]);
                        ai[r] = fma(mr, vi, ai[r]); ai[r] = fma(mi, vr, ai[r]);
                    }
                }
            }
#pragma unroll
            for (int r = 0; r < GEMV_MAXR; ++r) {
                if (r >= R) break;
                for (int o = 16; o > 0; o >>= 1) {
                    ar[r] += __shfl_down_sync(0xffffffffu, ar[r], o);
                    ai[r] += __shfl_down_sync(0xffffffffu, ai[r], o);
                }
            }
            if (lane == 0) {
                for (int r = 0; r < R; ++r) {
                    T br = 0, bi = 0;
                    if (y0) { br = y0[(r * 2) * ld + row]; bi = y0[(r * 2 + 1) * ld + row]; }
                    y[(r * 2) * ld + row] = br + g.alpha * ar[r];
                    y[(r * 2 + 1) * ld + row] = bi + g.alpha * ai[r];
                }
            }
        }
    } else {
        // 256 threads: 32 output rows x 8 j-groups, reduced through shared memory
        __shared__ T red[2][8][32][GEMV_MAXR];
        const int il = tid & 31, jg = tid >> 5;
        const int row = blockIdx.x * 32 + il;
        T ar[GEMV_MAXR], ai[GEMV_MAXR];
#pragma unroll
        for (int r = 0; r < GEMV_MAXR; ++r) { ar[r] = 0; ai[r] = 0; }
        if (row < b) {
            for (int t = 0; t < 2; ++t) {
                if (mslot[t] < 0) continue;
                const Pool<T>& P = t ? g.P2 : g.P1;
                const T* Mr = P.slot(mslot[t]);
                const T* Mi = Mr + P.plane_elems();
                const T* vt = sv + (size_t)t * R * 2 * b;
                for (int j = jg; j < b; j += 8) {
                    T mr = Mr[(size_t)j * P.ld + row], mi = Mi[(size_t)j * P.ld + row];
#pragma unroll
                    for (int r = 0; r < GEMV_MAXR; ++r) {
                        if (r >= R) break;
                        T vr = vt[(r * 2) * b + j], vi = vt[(r * 2 + 1) * b + j];
                        ar[r] = fma(mr, vr, ar[r]); ar[r] = fma(-mi, vi, ar[r]);
                        ai[r] = fma(mr, vi, ai[r]); ai[r] = fma(mi, vr, ai[r]);
                    }
                }
            }
        }
#pragma unroll
        for (int r = 0; r < GEMV_MAXR; ++r) { red[0][jg][il][r] = ar[r]; red[1][jg][il][r] = ai[r]; }
        __syncthreads();
        if (jg == 0 && row < b) {
            for (int r = 0; r < R; ++r) {
                T sr = 0, si = 0;
                for (int q = 0; q < 8; ++q) { sr += red[0][q][il][r]; si += red[1][q][il][r]; }
                T br = 0, bi = 0;
                if (y0) { br = y0[(r * 2) * ld + row]; bi = y0[(r * 2 + 1) * ld + row]; }
                y[(r * 2) * ld + row] = br + g.alpha * sr;
                y[(r * 2 + 1) * ld + row] = bi + g.alpha * si;
            }
        }
    }
}

// First reduction step with diagonal couplings (scaled stencil values).
// jobs: (node, prev, next, flags) with flags bit0 = prev participates, bit1 = next participates.
// mode 0: dst[node] -= u_node ⊙ src[next] + l_node ⊙ src[prev]   (forward, survivors)
// mode 1: dst[node]  = l_node ⊙ src[prev] + u_node ⊙ src[next]   (backward, eliminated)
// grid: (ceil(b/256), njobs), block 256
template <typename T>
__global__ void diag_sweep_kernel(NodeMap m, const cplx<double>* st, double scale, int nrhs, const int4* jobs,
                                  int mode, const T* src, T* dst) {
    const int4 J = jobs[blockIdx.y];
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.b) return;
    long long N = (long long)m.Nx * m.Ny;
    long long k = m.nat(J.x, i);
    cplx<double> l = cscale(st[m.p_cprev() * N + k], scale);
    cplx<double> u = cscale(st[m.p_cnext() * N + k], scale);
    const int ld = m.ld;
    for (int r = 0; r < nrhs; ++r) {
        cplx<double> acc = cmk(0.0, 0.0);
        if (J.w & 1) {
            const T* s = src + ((size_t)J.y * nrhs + r) * 2 * ld;
            acc = cadd(acc, cmul(l, cmk((double)s[i], (double)s[ld + i])));
        }
        if (J.w & 2) {
            const T* s = src + ((size_t)J.z * nrhs + r) * 2 * ld;
            acc = cadd(acc, cmul(u, cmk((double)s[i], (double)s[ld + i])));
        }
        T* d = dst + ((size_t)J.x * nrhs + r) * 2 * ld;
        if (mode == 0) {
            d[i] = (T)((double)d[i] - acc.re);
            d[ld + i] = (T)((double)d[ld + i] - acc.im);
        } else {
            d[i] = (T)acc.re;
            d[ld + i] = (T)acc.im;
        }
    }
}

template <typename T>
int launch_gemv(cudaStream_t s, int tr, int njobs, const GemvArgs<T>& g) {
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(gemv_kernel<T, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             160 * 1024);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(gemv_kernel<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024);
        if (e != cudaSuccess) return (int)e;
        attr = true;
    }
    size_t smem = (size_t)2 * g.nrhs * 2 * g.b * sizeof(T);
    dim3 grid(ceil_div(g.b, 32), njobs);
    if (tr) gemv_kernel<T, 1><<<grid, 256, smem, s>>>(g);
    else gemv_kernel<T, 0><<<grid, 256, smem, s>>>(g);
    return (int)cudaGetLastError();
}
template <typename T>
void launch_diag_sweep(cudaStream_t s, int njobs, NodeMap m, const cplx<double>* st, double scale, int nrhs,
                       const int4* jobs, int mode, const T* src, T* dst) {
    diag_sweep_kernel<T><<<dim3(ceil_div(m.b, 256), njobs), 256, 0, s>>>(m, st, scale, nrhs, jobs, mode, src, dst);
}
template int launch_gemv<float>(cudaStream_t, int, int, const GemvArgs<float>&);
template int launch_gemv<double>(cudaStream_t, int, int, const GemvArgs<double>&);
template void launch_diag_sweep<float>(cudaStream_t, int, NodeMap, const cplx<double>*, double, int, const int4*,
                                       int, const float*, float*);
template void launch_diag_sweep<double>(cudaStream_t, int, NodeMap, const cplx<double>*, double, int, const int4*,
                                        int, const double*, double*);
