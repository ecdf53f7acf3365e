// dht_tc.cu -- launch wrapper of the tcgen05 Hankel GEMM (dht_tc2.cuh).
#include "launch.h"
#include "dht_tc2.cuh"

cudaError_t launch_dht_tc2(const CUtensorMap& th, const CUtensorMap& tm, const CUtensorMap& tl,
                           const CUtensorMap& b, const TcGemmParams& p, int M, int N, cudaStream_t st) {
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_dht_tc2, cudaFuncAttributeMaxDynamicSharedMemorySize, T2_SMEM_BYTES);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  dim3 grid(N / T2_BN, M / T2_BM);
  k_dht_tc2<<<grid, T2_THREADS, T2_SMEM_BYTES, st>>>(th, tm, tl, b, p);
  return cudaGetLastError();
}
