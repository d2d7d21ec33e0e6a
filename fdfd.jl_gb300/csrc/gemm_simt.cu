// Batched complex TN GEMM on CUDA cores (FP64 factorization path, and the FP32
// path's reference implementation).  Register-tiled: 64x64 output tile per
// CTA, 256 threads, 4x4 complex accumulators per thread, K staged through
// shared memory in steps of 16.
#include "common.cuh"
#include "kernels.cuh"

template <typename T>
__global__ void __launch_bounds__(256) gemm_simt_kernel(GemmArgs<T> g) {
    constexpr int BM = 64, BN = 64, BK = 16;
    __shared__ T As[2][BK][BM + 4];
    __shared__ T Bs[2][BK][BN + 4];
    const int job = blockIdx.z;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    const T* A = g.A.slot(g.a_slot[job]);
    const T* B = g.B.slot(g.b_slot[job]);
    T* C = g.C.slot(g.c_slot[job]);
    const long long ape = g.A.plane_elems(), bpe = g.B.plane_elems(), cpe = g.C.plane_elems();
    const int tid = threadIdx.x;
    const int tx = tid % 16, ty = tid / 16;
    T accr[4][4], acci[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) { accr[i][j] = 0; acci[i][j] = 0; }

    // loader mapping: 256 threads x 4 elements = 64 rows x 16 k
    const int lrow = tid / 4, lk = (tid % 4) * 4;
    for (int k0 = 0; k0 < g.K; k0 += BK) {
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            int k = k0 + lk + e;
            int am = m0 + lrow, bn = n0 + lrow;
            T ar = 0, ai = 0, br = 0, bi = 0;
            if (am < g.M && k < g.K) {
                ar = A[(long long)am * g.A.ld + k];
                ai = A[ape + (long long)am * g.A.ld + k];
            }
            if (bn < g.N && k < g.K) {
                br = B[(long long)bn * g.B.ld + k];
                bi = B[bpe + (long long)bn * g.B.ld + k];
            }
            As[0][lk + e][lrow] = ar; As[1][lk + e][lrow] = ai;
            Bs[0][lk + e][lrow] = br; Bs[1][lk + e][lrow] = bi;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
            T ar[4], ai[4], br[4], bi[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                ar[i] = As[0][kk][ty * 4 + i]; ai[i] = As[1][kk][ty * 4 + i];
                br[i] = Bs[0][kk][tx * 4 + i]; bi[i] = Bs[1][kk][tx * 4 + i];
            }
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    accr[i][j] = fma(ar[i], br[j], accr[i][j]);
                    accr[i][j] = fma(-ai[i], bi[j], accr[i][j]);
                    acci[i][j] = fma(ar[i], bi[j], acci[i][j]);
                    acci[i][j] = fma(ai[i], br[j], acci[i][j]);
                }
        }
        __syncthreads();
    }
    // epilogue
    const int ctr = g.c_trans_arr ? g.c_trans_arr[job] : g.c_trans;
    // β term source: C itself, or row row_src[m] of Cin (N-form only)
    const bool sep = g.Cin.base != nullptr;
    const T* Ci = sep ? g.Cin.slot(g.cin_slot[job]) : C;
    const long long cipe = sep ? g.Cin.plane_elems() : cpe;
    const long long cild = sep ? (long long)g.Cin.ld : (long long)g.C.ld;
    const int* rsrc = (sep && g.row_src) ? g.row_src + (long long)job * g.M : nullptr;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        int m = m0 + ty * 4 + i;
        if (m >= g.M) continue;
        bool mrow = (m >= g.mask_c0 && m < g.mask_c0 + g.mask_w);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            int n = n0 + tx * 4 + j;
            if (n >= g.N) continue;
            T vr = g.alpha * accr[i][j], vi = g.alpha * acci[i][j];
            bool masked = mrow || (n >= g.mask_c0 && n < g.mask_c0 + g.mask_w);
            long long off = ctr ? (long long)n * g.C.ld + m : (long long)m * g.C.ld + n;
            if (g.beta && !masked) {
                const long long io = ctr ? off : (long long)(rsrc ? rsrc[m] : m) * cild + n;
                vr += Ci[io];
                vi += Ci[cipe + io];
            }
            C[off] = vr;
            C[cpe + off] = vi;
        }
    }
}

template <typename T>
void launch_gemm_simt(cudaStream_t s, int njobs, const GemmArgs<T>& g) {
    gemm_simt_kernel<T><<<dim3(ceil_div(g.N, 64), ceil_div(g.M, 64), njobs), 256, 0, s>>>(g);
}
template void launch_gemm_simt<float>(cudaStream_t, int, const GemmArgs<float>&);
template void launch_gemm_simt<double>(cudaStream_t, int, const GemmArgs<double>&);
