// dht_tc.cu -- launch wrappers of the tensor-core Hankel GEMM and its
// operand slicer (dht_tc.cuh).
#include "launch.h"
#include "dht_tc.cuh"

cudaError_t launch_dht_tc(const CUtensorMap (&a)[3], const CUtensorMap (&b)[3], const TcGemmParams& p, int M,
                          int N, cudaStream_t st) {
  // set on every launch (a host call, legal under stream capture): the
  // attribute belongs to the current device's context
  cudaError_t e = cudaFuncSetAttribute(k_dht_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM_BYTES);
  if (e != cudaSuccess) return e;
  if (M % TC_BM || N % TC_BN || p.K % TC_CHUNK) return cudaErrorInvalidValue;
  dim3 grid(N / TC_BN, M / TC_BM);
  k_dht_tc<<<grid, TC_THREADS, TC_SMEM_BYTES, st>>>(a[0], a[1], a[2], b[0], b[1], b[2], p);
  return cudaGetLastError();
}

cudaError_t launch_slice(const float* B, void* const (&s)[3], float* qb, int N, int K, const DevCtl* ctl,
                         cudaStream_t st) {
  if (K % TC_CHUNK) return cudaErrorInvalidValue;
  const int nch = K / TC_CHUNK;
  __half2 *s0 = (__half2*)s[0], *s1 = (__half2*)s[1], *s2 = (__half2*)s[2];
  if (nch % 4 == 0) k_slice<4><<<(N * (nch / 4) + 7) / 8, 256, 0, st>>>(B, s0, s1, s2, qb, N, K, ctl);
  else if (nch % 2 == 0) k_slice<2><<<(N * (nch / 2) + 7) / 8, 256, 0, st>>>(B, s0, s1, s2, qb, N, K, ctl);
  else k_slice<1><<<(N * nch + 7) / 8, 256, 0, st>>>(B, s0, s1, s2, qb, N, K, ctl);
  return cudaGetLastError();
}

cudaError_t launch_slice_prop(const float* W, const float2* kz, const float* gd, void* const (&s)[3], float* qb, int nh,
                              int K, const DevCtl* ctl, cudaStream_t st) {
  if (K % TC_CHUNK) return cudaErrorInvalidValue;
  const int nch = K / TC_CHUNK;
  __half2 *s0 = (__half2*)s[0], *s1 = (__half2*)s[1], *s2 = (__half2*)s[2];
  if (nch % 2 == 0)
    k_slice_prop<2, false><<<(nh * (nch / 2) + 7) / 8, 256, 0, st>>>(W, kz, gd, s0, s1, s2, qb, nh, K, ctl, 0.f);
  else
    k_slice_prop<1, false><<<(nh * nch + 7) / 8, 256, 0, st>>>(W, kz, gd, s0, s1, s2, qb, nh, K, ctl, 0.f);
  return cudaGetLastError();
}

cudaError_t launch_slice_mul(const float* W, const float2* f, void* const (&s)[3], float* qb, int nh, int K,
                             const DevCtl* ctl, cudaStream_t st) {
  if (K % TC_CHUNK) return cudaErrorInvalidValue;
  const int nch = K / TC_CHUNK;
  __half2 *s0 = (__half2*)s[0], *s1 = (__half2*)s[1], *s2 = (__half2*)s[2];
  if (nch % 2 == 0)
    k_slice_prop<2, true><<<(nh * (nch / 2) + 7) / 8, 256, 0, st>>>(W, f, nullptr, s0, s1, s2, qb, nh, K, ctl, 0.f);
  else
    k_slice_prop<1, true><<<(nh * nch + 7) / 8, 256, 0, st>>>(W, f, nullptr, s0, s1, s2, qb, nh, K, ctl, 0.f);
  return cudaGetLastError();
}
