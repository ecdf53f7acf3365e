// tc_params.h -- launch parameters of the tensor-core Hankel GEMM
// (kernel in dht_tc.cuh), shared with the host code.
#pragma once
#include <cuda_runtime.h>

struct DevCtl;

struct TcGemmParams {
  float* out;
  int ldo;                // leading dimension of out (floats)
  int K;                  // contraction length, multiple of 64
  int mode;               // 1 transposed store; 2 row-major store (+ guard pending);
                          // 3 row-major store
  const float* qa;        // [M] row scales of A (powers of two)
  const float* qb;        // [K/64][ldqb] chunk scales of B (powers of two)
  int ldqb;
  DevCtl* ctl;            // NULL: no controller (dz = dz_fixed)
  float dz_fixed;
  int* err;               // set to 1 on a timed-out wait
};
