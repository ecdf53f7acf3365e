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
  float* part;               // [rows][9][T] layer-3 partial sums (nn_out_at)
  int T, maxrows;
  const int* count;          // device row count (NULL: maxrows)
  const int* stop;           // device flag: non-zero skips the launches (or NULL)
  int* err;                  // set to 1 when a bounded wait gave up
  // the tiles to run: the first *tcount entries of tlist (row * T/128 +
  // tile), in any order; NULL: every tile of the rows
  const int* tlist;
  const int* tcount;
  CUtensorMap map_a1, map_a2;   // 3-D maps {64, T, rows}, box {64, 136, 1} (a tile with its halo)
  int sms;                   // persistent grid size of the tensor-core layers
};

// maps and grid of a plan whose buffers are set; returns 0 on success
int nn_plan_init(NnRowsPlan* p);

// weights of one 64 -> 64 layer: W[k][co][ci] BF16 and its TMA map
// {64, 9 * 64}, box {64, 64}
int nn_weight_map(CUtensorMap* m, const __nv_bfloat16* wt);
// layer 1 (part == NULL: activations into out; with x0, w0, b0 layer 0 is
// computed inside the kernel from the inputs x0 and tx is unused) or layer 2
// with layer 3 applied in the epilogue (partial sums into part)
cudaError_t nn_launch_conv_tc(const CUtensorMap& tx, const CUtensorMap& tw, const float* bias, __nv_bfloat16* out,
                              const __nv_bfloat16* w3, float* part, const NnRowsPlan& p, cudaStream_t st,
                              const __nv_bfloat16* x0 = nullptr, const __nv_bfloat16* w0 = nullptr,
                              const float* b0 = nullptr);
// out [rows][T] from the partial sums [rows][9][T]
cudaError_t nn_launch_out(const float* part, const float* b3, float* out, int T, int rows, cudaStream_t st);

// network output at t of one row from its layer-3 partial sums P [9][T]:
// b3 + sum_k P_k[t + k - 4] (terms outside [0, T) are zero padding)
__device__ __forceinline__ float nn_out_at(const float* __restrict__ P, float b3, int t, int T) {
  float s = b3;
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    const int u = t + k - 4;
    if (u >= 0 && u < T) s += __ldg(&P[(size_t)k * T + u]);
  }
  return s;
}

struct fil_nn;
// the network over the rows of the plan: layers 0 and 1 in one tensor-core
// kernel (layer 0 through an im2col tile into layer 1's operand), layer 2 on
// the tensor cores with layer 3 in its epilogue, leaving the partial sums in
// p.part; surrogate.cu
cudaError_t nn_infer(const fil_nn* n, const NnRowsPlan& p, cudaStream_t st);
// device pointer to the output layer's bias (the b3 of nn_out_at)
const float* nn_out_bias(const fil_nn* n);
