// dht_tc.cu -- launch wrapper of the tcgen05 Hankel GEMM (dht_tc.cuh).
#include "launch.h"
#include "dht_tc.cuh"

cudaError_t launch_dht_tc(const CUtensorMap& a0, const CUtensorMap& a1, const CUtensorMap& a2,
                          const CUtensorMap& b, const TcGemmParams& p, int M, int N, cudaStream_t st) {
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_dht_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM_BYTES);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  dim3 grid(N / TC_BN, M / TC_BM);
  k_dht_tc<<<grid, TC_THREADS, TC_SMEM_BYTES, st>>>(a0, a1, a2, b, p);
  return cudaGetLastError();
}
