// tcgen05 3xTF32 complex GEMM (FP32 factor path): host interface.
#pragma once
#include <cuda.h>
#include "kernels.cuh"

// TMA descriptors of the five FP32 pools (D, C, X, GP, RP), each with a
// 128-row box (A operand tiles and BN = 128 B tiles), a 256-row and a 64-row
// box (B operand tiles of the other widths).
struct TcMaps {
    CUtensorMap map[5][3];
};

// Encodes the three descriptors of one pool; false if cuTensorMapEncodeTiled rejects one.
bool tc_make_map(const Pool<float>& P, CUtensorMap* box128, CUtensorMap* box256, CUtensorMap* box64);

// Encodes the descriptors of the five pools; false if any is refused (the
// SIMT GEMM is used then).
bool tc_make_maps(const Pool<float>* D, const Pool<float>* C, const Pool<float>* X, const Pool<float>* GP,
                  const Pool<float>* RP, TcMaps* out);

// C[c_slot[job]] = alpha·Σ_{s<ks} W[job·ks + s] (+ beta·C), N form or transposed per job:
// the second phase of a split-K product (returns a cudaError_t value)
int tc_splitk_sum(const Pool<float>& W, int ks, const Pool<float>& C, const int* c_slot, const int* c_trans_arr,
                  int c_trans, int njobs, int M, int N, float alpha, int beta, cudaStream_t stream);

// tile code of the 128-column tile sized for two CTAs per SM (three pipeline
// stages, four epilogue warps): its B tiles use the 128-row box
#define TC_BN128_TWO 129

inline const char* tc_tile_name(int bn) {
    return bn == 256 ? "256" : bn == 128 ? "128" : bn == TC_BN128_TWO ? "128x2" : bn == 64 ? "64" : "?";
}

// Launches the batched TN GEMM of `g` on the tensor cores with 128 x bn tiles
// (bn = 256, 128, TC_BN128_TWO or 64), A tiles read through `mapA` (128-row
// box) and B tiles through `mapB` (bn-row box).  c_trans_arr (device, per job, may be null)
// overrides g->c_trans.  Returns 0 or a cudaError_t value.
int tc_gemm_launch_maps(const GemmArgs<float>* g, const int* c_trans_arr, const CUtensorMap* mapA,
                        const CUtensorMap* mapB, int bn, int njobs, cudaStream_t stream);

// Tile width for a launch: the widest tile (256, 128 or 64 columns, no wider
// than the product needs) whose tile count still covers num_sms.
int tc_pick_bn(int M, int N, int K, int njobs, int num_sms);

// bn > 0 forces the tile (the autotuner's choice), 0 takes tc_pick_bn's
inline int tc_gemm_launch(const GemmArgs<float>* g, const int* c_trans_arr, int pa, int pb, int njobs,
                          const TcMaps* maps, int num_sms, cudaStream_t stream, int bn = 0) {
    if (bn != 64 && bn != 128 && bn != 256 && bn != TC_BN128_TWO)
        bn = tc_pick_bn(g->M, g->N, g->K, njobs, num_sms);
    const int bi = bn == 256 ? 1 : ((bn == 128 || bn == TC_BN128_TWO) ? 0 : 2);
    return tc_gemm_launch_maps(g, c_trans_arr, &maps->map[pa][0], &maps->map[pb][bi], bn, njobs, stream);
}
