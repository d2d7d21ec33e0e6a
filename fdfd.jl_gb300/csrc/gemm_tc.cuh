// tcgen05 3xTF32 complex GEMM (FP32 factor path): host interface.
#pragma once
#include <cuda.h>
#include "kernels.cuh"

// TMA descriptors of the five FP32 pools (D, C, X, GP, RP), each with a
// 128-row box (A operand tiles) and a 256-row box (B operand tiles).
struct TcMaps {
    CUtensorMap map[5][2];
};

// Encodes the two descriptors of one pool; false if the driver refuses.
bool tc_make_map(const Pool<float>& P, CUtensorMap* box128, CUtensorMap* box256);

// Encodes the descriptors of the five pools; false if any is refused (the
// SIMT GEMM is used then).
bool tc_make_maps(const Pool<float>* D, const Pool<float>* C, const Pool<float>* X, const Pool<float>* GP,
                  const Pool<float>* RP, TcMaps* out);

// Launches the batched TN GEMM of `g` on the tensor cores with A tiles read
// through `mapA` (128-row box) and B tiles through `mapB` (256-row box).
// c_trans_arr (device, per job, may be null) overrides g->c_trans.
// Returns 0 or a cudaError_t value.
int tc_gemm_launch_maps(const GemmArgs<float>* g, const int* c_trans_arr, const CUtensorMap* mapA,
                        const CUtensorMap* mapB, int njobs, cudaStream_t stream);

inline int tc_gemm_launch(const GemmArgs<float>* g, const int* c_trans_arr, int pa, int pb, int njobs,
                          const TcMaps* maps, cudaStream_t stream) {
    return tc_gemm_launch_maps(g, c_trans_arr, &maps->map[pa][0], &maps->map[pb][1], njobs, stream);
}
