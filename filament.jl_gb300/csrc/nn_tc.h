// nn_tc.h -- inference path of the learned plasma surrogate (nn_tc.cu):
// channel-last activations, the two 64 -> 64 layers as tcgen05 implicit
// GEMMs.  A plan holds the buffers of one set of rows and the TMA maps over
// them.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <cuda_bf16.h>

struct NnRowsPlan {
  const __nv_bfloat16* x0;   // [rows][3][T] network inputs
  __nv_bfloat16* a1;         // [rows][T][64] hidden activations (channel-last)
  __nv_bfloat16* a2;
  float* out;                // [rows][T]
  int T, maxrows;
  const int* count;          // device row count (NULL: maxrows)
  const int* stop;           // device flag: non-zero skips the launches (or NULL)
  int* err;                  // set to 1 when a bounded wait gave up
  CUtensorMap map_a1, map_a2;   // 3-D maps {64, T, rows}, box {64, 128, 1}
  int sms;                   // persistent grid size of the tensor-core layers
};

// maps and grid of a plan whose buffers are set; returns 0 on success
int nn_plan_init(NnRowsPlan* p);

// weights of one 64 -> 64 layer: W[k][co][ci] BF16 and its TMA map
// {64, 9 * 64}, box {64, 64}
int nn_weight_map(CUtensorMap* m, const __nv_bfloat16* wt);

cudaError_t nn_launch_l0_cl(const __nv_bfloat16* x, const __nv_bfloat16* w, const float* bias, __nv_bfloat16* y,
                            int T, int maxrows, const int* count, const int* stop, cudaStream_t st);
cudaError_t nn_launch_l3_cl(const __nv_bfloat16* y, const __nv_bfloat16* w, const float* bias, float* out, int T,
                            int maxrows, const int* count, const int* stop, cudaStream_t st);
cudaError_t nn_launch_conv_tc(const CUtensorMap& tx, const CUtensorMap& tw, const float* bias, __nv_bfloat16* out,
                              const NnRowsPlan& p, cudaStream_t st);

struct fil_nn;
// the four layers over the rows of the plan (layer 0 and 3 on CUDA cores,
// 1 and 2 on the tensor cores); surrogate.cu
cudaError_t nn_infer(const fil_nn* n, const NnRowsPlan& p, cudaStream_t st);
