// TMA-pipelined mixed stage kernel: host-side interface (stage_tma.cu).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include "kernels.cuh"

// Tensor maps of the three FP32 stage buffers (halo and plain boxes) and of the two FP32
// copies of F_n (parity pair). Encoded once per integrator after the buffers exist.
struct TmaStage32 {
  CUtensorMap halo[33][3];  // indexed by tile height (8, 16, 24, 32) and buffer
  CUtensorMap plain[33][3];
  CUtensorMap f0[33][2];
  bool ok = false;
};

constexpr int TMA_STAGE32_NVARIANTS = 6;
const char* tma_stage32_variant_name(int variant);
bool tma_stage32_supported(long long nx, long long ny);
bool tma_stage32_prepare(TmaStage32* t, float* const D[3], float* const Ff[2], long long nx, long long ny);
// d_{j-1} = D[im1], d_{j-2} = D[im2] (im2 < 0: none, stage 2), F_0 = Ff[if0]
bool tma_stage32_launch(const TmaStage32* t, int variant, int num_sms, const ProbDev& P, const StageArgs* A, int im1,
                        int im2, int if0, float* out, int* err, cudaStream_t st);
