// fft.cuh -- block-level Stockham FFT of one row held in shared memory.
//
// N = 2^L points, N/16 threads, 16 elements per thread.  Passes: one
// radix-(2^(L mod 4)) pass (if L is not a multiple of 4) followed by radix-16
// passes; each pass loads all of a thread's elements into registers, syncs,
// and stores them in Stockham (auto-sorted) order, so the transform is
// in place and the output is in natural order.  Twiddles come from a table
// tw[m] = exp(-2 pi i m / N) computed in FP64 on the host.
//
// SIGN = -1: X_k = sum_n x_n exp(-2 pi i k n / N)  (FFTW fft, w -> t here)
// SIGN = +1: X_k = sum_n x_n exp(+2 pi i k n / N)  (unscaled; the caller
//            applies 1/N where it wants FFTW's ifft, t -> w here).
#pragma once
#include "common.cuh"

namespace filfft {

template <typename C, int SIGN> FIL_DEV C mul_si(C b) {  // SIGN * i * b
  C r;
  if (SIGN < 0) { r.x = b.y; r.y = -b.x; }
  else { r.x = -b.y; r.y = b.x; }
  return r;
}

template <typename C, int SIGN> FIL_DEV void dft2(C* v) {
  C a = v[0], b = v[1];
  v[0] = a + b;
  v[1] = a - b;
}

template <typename C, int SIGN> FIL_DEV void dft4(C* v) {
  C a0 = v[0] + v[2], a1 = v[0] - v[2], b0 = v[1] + v[3], b1 = mul_si<C, SIGN>(v[1] - v[3]);
  v[0] = a0 + b0;
  v[2] = a0 - b0;
  v[1] = a1 + b1;
  v[3] = a1 - b1;
}

template <typename C, int SIGN> FIL_DEV void dft8(C* v) {
  typedef decltype(C().x) R;
  const R h = (R)0.70710678118654752440;
  C e[4] = {v[0], v[2], v[4], v[6]};
  C o[4] = {v[1], v[3], v[5], v[7]};
  dft4<C, SIGN>(e);
  dft4<C, SIGN>(o);
  // W8^k = exp(SIGN 2 pi i k / 8)
  C w1 = mk<R>(h, SIGN * h), w3 = mk<R>(-h, SIGN * h);
  C t0 = o[0], t1 = cmul(o[1], w1), t2 = mul_si<C, SIGN>(o[2]), t3 = cmul(o[3], w3);
  v[0] = e[0] + t0; v[4] = e[0] - t0;
  v[1] = e[1] + t1; v[5] = e[1] - t1;
  v[2] = e[2] + t2; v[6] = e[2] - t2;
  v[3] = e[3] + t3; v[7] = e[3] - t3;
}

template <typename C, int SIGN> FIL_DEV void dft16(C* v) {
  typedef decltype(C().x) R;
  // cos(k pi/8), sin(k pi/8), k = 0..7
  const R c1 = (R)0.92387953251128675613, s1 = (R)0.38268343236508977173;
  const R c2 = (R)0.70710678118654752440;
  C e[8], o[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) { e[i] = v[2 * i]; o[i] = v[2 * i + 1]; }
  dft8<C, SIGN>(e);
  dft8<C, SIGN>(o);
  C t[8];
  t[0] = o[0];
  t[1] = cmul(o[1], mk<R>(c1, SIGN * s1));
  t[2] = cmul(o[2], mk<R>(c2, SIGN * c2));
  t[3] = cmul(o[3], mk<R>(s1, SIGN * c1));
  t[4] = mul_si<C, SIGN>(o[4]);
  t[5] = cmul(o[5], mk<R>(-s1, SIGN * c1));
  t[6] = cmul(o[6], mk<R>(-c2, SIGN * c2));
  t[7] = cmul(o[7], mk<R>(-c1, SIGN * s1));
#pragma unroll
  for (int k = 0; k < 8; ++k) { v[k] = e[k] + t[k]; v[k + 8] = e[k] - t[k]; }
}

template <typename C, int RD, int SIGN> FIL_DEV void dft(C* v) {
  if constexpr (RD == 2) dft2<C, SIGN>(v);
  else if constexpr (RD == 4) dft4<C, SIGN>(v);
  else if constexpr (RD == 8) dft8<C, SIGN>(v);
  else dft16<C, SIGN>(v);
}

template <typename C, int N, int RD, int NS, int SIGN>
FIL_DEV void pass(C* s, const C* __restrict__ tw) {
  constexpr int T = N / 16;
  constexpr int NB = N / RD;
  constexpr int Q = NB / T;
  C v[Q][RD];
  const int tid = threadIdx.x;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int b = tid + q * T;
#pragma unroll
    for (int r = 0; r < RD; ++r) v[q][r] = s[pad16(b + r * NB)];
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int b = tid + q * T;
    const int k = b % NS;
    if constexpr (NS > 1) {
#pragma unroll
      for (int r = 1; r < RD; ++r) {
        C w = __ldg(&tw[(k * r) * (N / (NS * RD))]);
        if (SIGN > 0) w = cconj(w);
        v[q][r] = cmul(v[q][r], w);
      }
    }
    dft<C, RD, SIGN>(v[q]);
    const int o = (b / NS) * NS * RD + k;
#pragma unroll
    for (int r = 0; r < RD; ++r) s[pad16(o + r * NS)] = v[q][r];
  }
  __syncthreads();
}

template <typename C, int N, int NS, int SIGN>
FIL_DEV void passes16(C* s, const C* __restrict__ tw) {
  if constexpr (NS < N) {
    pass<C, N, 16, NS, SIGN>(s, tw);
    passes16<C, N, NS * 16, SIGN>(s, tw);
  }
}

__host__ __device__ constexpr int ilog2(int n) { return n <= 1 ? 0 : 1 + ilog2(n / 2); }

// In-place FFT of s[pad16(0..N-1)] by the first N/16 threads of the block
// (blockDim.x must equal N/16).  Synchronises on entry and exit.
template <typename C, int N, int SIGN>
FIL_DEV void block_fft(C* s, const C* __restrict__ tw) {
  static_assert(N >= 256 && (N & (N - 1)) == 0, "N must be a power of two >= 256");
  constexpr int L = ilog2(N);
  constexpr int R0 = 1 << (L % 4);
  __syncthreads();
  if constexpr (R0 > 1) {
    pass<C, N, R0, 1, SIGN>(s, tw);
    passes16<C, N, R0, SIGN>(s, tw);
  } else {
    passes16<C, N, 1, SIGN>(s, tw);
  }
}

}  // namespace filfft
