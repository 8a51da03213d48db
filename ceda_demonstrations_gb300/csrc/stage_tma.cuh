// TMA-pipelined mixed stage kernel: host-side interface (stage_tma.cu).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include "kernels.cuh"

constexpr int TMA_FUSED_NTILES = 6; // fused-stage tile configurations

// Tensor maps of the three FP32 stage buffers (halo and plain boxes) and of the two FP32
// copies of F_n (parity pair). Encoded once per integrator after the buffers exist.
struct TmaStage32 {
  CUtensorMap halo[33][4];  // indexed by tile height (8, 16, 24, 32) and buffer
  CUtensorMap plain[33][4];
  CUtensorMap f0[33][2];
  bool ok = false;
  bool have[4] = {false, false, false, false}; // maps encoded for buffer b
  // fused stages: 128 x (TH+8) boxes of the four stage buffers and of F_n, per tile configuration
  CUtensorMap fz[TMA_FUSED_NTILES][4];
  CUtensorMap fzf[TMA_FUSED_NTILES][2];
  bool fz_ok = false;
};

constexpr int TMA_STAGE32_NVARIANTS = 6;
const char* tma_stage32_variant_name(int variant);
bool tma_stage32_supported(long long nx, long long ny);
// a 2-D FP32 tensor map of an nx x ny row-major buffer with box_w x box_h boxes
bool tma_encode_f32_2d(CUtensorMap* m, const float* base, long long nx, long long ny, int box_w, int box_h);
// encodes the maps of every stage buffer D[0..3] that is allocated (D[3]: fused stages only)
bool tma_stage32_prepare(TmaStage32* t, float* const D[4], float* const Ff[2], long long nx, long long ny);
// d_{j-1} = D[im1], d_{j-2} = D[im2] (im2 < 0: none, stage 2), F_0 = Ff[if0]
bool tma_stage32_launch(const TmaStage32* t, int variant, int num_sms, const ProbDev& P, const StageArgs* A, int im1,
                        int im2, int if0, float* out, int* err, cudaStream_t st);

// Fused stages j .. j+ks-1 (2 <= ks <= 4) in one launch: A = the StageArgs of stage j (ks
// consecutive entries), d_{j-1} = D[im1], d_{j-2} = D[im2] (im2 < 0: j = 2), F_0 = Ff[if0];
// writes d_{j+ks-2} to o2 and d_{j+ks-1} to o1 (neither may be an input buffer). Tile
// configuration ti in [0, TMA_FUSED_NTILES).
int tma_fused_tile_rows(int ti);
const char* tma_fused_config_name(int ti);
bool tma_fused_prepare(TmaStage32* t, float* const D[4], float* const Ff[2], long long nx, long long ny);
bool tma_fused_launch(const TmaStage32* t, int ti, int ks, int num_sms, const ProbDev& P, const StageArgs* A, int im1,
                      int im2, int if0, float* o2, float* o1, int* err, cudaStream_t st);
