// common.cuh -- complex arithmetic and small helpers shared by the kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define FIL_DEV __device__ __forceinline__
#define FIL_HD __host__ __device__ __forceinline__

template <typename R> struct C2T;
template <> struct C2T<float> { typedef float2 type; };
template <> struct C2T<double> { typedef double2 type; };

template <typename R> FIL_HD typename C2T<R>::type mk(R x, R y) {
  typename C2T<R>::type c;
  c.x = x;
  c.y = y;
  return c;
}
FIL_HD float2 operator+(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
FIL_HD float2 operator-(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
FIL_HD float2 operator*(float s, float2 a) { return make_float2(s * a.x, s * a.y); }
FIL_HD double2 operator+(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
FIL_HD double2 operator-(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
FIL_HD double2 operator*(double s, double2 a) { return make_double2(s * a.x, s * a.y); }

template <typename C> FIL_HD C cmul(C a, C b) {
  C r;
  r.x = a.x * b.x - a.y * b.y;
  r.y = a.x * b.y + a.y * b.x;
  return r;
}
// a * conj(b)
template <typename C> FIL_HD C cmulc(C a, C b) {
  C r;
  r.x = a.x * b.x + a.y * b.y;
  r.y = a.y * b.x - a.x * b.y;
  return r;
}
template <typename C> FIL_HD C cconj(C a) {
  a.y = -a.y;
  return a;
}
// multiply by i
template <typename C> FIL_HD C cmuli(C a) {
  C r;
  r.x = -a.y;
  r.y = a.x;
  return r;
}
template <typename C> FIL_HD decltype(C().x) cabs2(C a) { return a.x * a.x + a.y * a.y; }

// padded shared-memory index: one spare element every 16 keeps the strided
// Stockham stores of 8- and 16-byte elements free of bank conflicts.
FIL_HD int pad16(int i) { return i + (i >> 4); }

// atomic max for non-negative floats/doubles through their bit patterns
FIL_DEV void atomic_max_nonneg(unsigned int* addr, float v) {
  atomicMax(addr, __float_as_uint(v));
}
FIL_DEV void atomic_max_nonneg(unsigned long long* addr, double v) {
  atomicMax(addr, (unsigned long long)__double_as_longlong(v));
}

template <typename R> struct MaxBits;
template <> struct MaxBits<float> { typedef unsigned int type; };
template <> struct MaxBits<double> { typedef unsigned long long type; };

// block-wide reductions (blockDim.x a multiple of 32, <= 1024)
template <typename T> FIL_DEV T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
template <typename T> FIL_DEV T warp_max(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
// scratch: >= 32 elements of T in shared memory
template <typename T> FIL_DEV T block_sum(T v, T* scratch) {
  v = warp_sum(v);
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __syncthreads();
  if (lane == 0) scratch[w] = v;
  __syncthreads();
  T r = (threadIdx.x < nw) ? scratch[threadIdx.x] : T(0);
  if (w == 0) r = warp_sum(r);
  if (threadIdx.x == 0) scratch[0] = r;
  __syncthreads();
  r = scratch[0];
  __syncthreads();
  return r;
}
template <typename T> FIL_DEV T block_max(T v, T* scratch) {
  v = warp_max(v);
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __syncthreads();
  if (lane == 0) scratch[w] = v;
  __syncthreads();
  T r = (threadIdx.x < nw) ? scratch[threadIdx.x] : T(0);
  if (w == 0) r = warp_max(r);
  if (threadIdx.x == 0) scratch[0] = r;
  __syncthreads();
  r = scratch[0];
  __syncthreads();
  return r;
}
