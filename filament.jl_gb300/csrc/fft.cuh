// fft.cuh -- block-level Stockham FFT of one row held in shared memory.
//
// N = 2^L points (N >= 16), N/16 threads, 16 elements per thread.  Passes: one
// radix-(2^(L mod 4)) pass (if L is not a multiple of 4) followed by radix-16
// passes; each pass loads all of a thread's elements into registers, syncs,
// and stores them in Stockham (auto-sorted) order, so the transform is
// in place and the output is in natural order.  Twiddles come from a table
// computed in FP64 on the host and laid out per pass: the radix-16 pass of
// stride NS reads tp[(r - 1) NS + k] = exp(-2 pi i k r / (16 NS)), r = 1..15,
// k < NS, so the lanes of a warp (consecutive k) read consecutive entries;
// the pass tables follow each other in pass order.  (One table indexed by
// k r N / (16 NS) scatters a warp's reads over up to 32 cache lines, which
// made the transform 2.4 times slower.)
//
// sign -1: X_k = sum_n x_n exp(-2 pi i k n / N)  (FFTW fft, w -> t here)
// sign +1: X_k = sum_n x_n exp(+2 pi i k n / N)  (unscaled; the caller
//          applies 1/N where it wants FFTW's ifft, t -> w here).
#pragma once
#include "common.cuh"

namespace filfft {

// The direction is an argument sg = -1 / +1 of the working precision: call
// sites with a literal sign are specialised by the compiler when the
// transform is inlined; a run-time sign gives one copy of the code for both
// directions (the row kernel's stage loop, where code size matters).

template <typename C> FIL_DEV C mul_si(C b, decltype(C().x) sg) {  // sg * i * b
  C r;
  r.x = -sg * b.y;
  r.y = sg * b.x;
  return r;
}

template <typename C> FIL_DEV void dft2(C* v) {
  C a = v[0], b = v[1];
  v[0] = a + b;
  v[1] = a - b;
}

template <typename C> FIL_DEV void dft4(C* v, decltype(C().x) sg) {
  C a0 = v[0] + v[2], a1 = v[0] - v[2], b0 = v[1] + v[3], b1 = mul_si<C>(v[1] - v[3], sg);
  v[0] = a0 + b0;
  v[2] = a0 - b0;
  v[1] = a1 + b1;
  v[3] = a1 - b1;
}

// Multiplication by exp(sg i K pi/8), K = 1, 2, 3.  In single precision
// the constants are applied as head + remainder: the nearest FP32 values of
// cos(pi/8), sin(pi/8) and sqrt(2)/2 all lie below the true values
// (|w|^2 - 1 = -5.7e-8 and -3.4e-8), which would shrink the field by ~2e-8
// per butterfly and, over six radix-16 passes per time<->frequency round
// trip, damp the energy by ~1.5e-7 every z-step.  The split form keeps the
// rotation's magnitude exact to ~2^-48.
template <int K> FIL_DEV float2 rot8(float2 v, float sg) {
  // K=1: (c1, s1), K=2: (c2, c2), K=3: (s1, c1); head + remainder
  const float c1h = 0.92387950420379638671875f, c1l = 2.8307490243e-08f;
  const float s1h = 0.3826834261417388916015625f, s1l = 6.2233508e-09f;
  const float c2h = 0.707106769084930419921875f, c2l = 1.2101617e-08f;
  float ch, cl, sh, sl;
  if (K == 1) { ch = c1h; cl = c1l; sh = s1h; sl = s1l; }
  else if (K == 2) { ch = c2h; cl = c2l; sh = c2h; sl = c2l; }
  else { ch = s1h; cl = s1l; sh = c1h; sl = c1l; }
  // re = x c - sg y s, im = y c + sg x s
  const float ys = fmaf(v.y, sh, v.y * sl), xs = fmaf(v.x, sh, v.x * sl);
  const float re = fmaf(v.x, ch, fmaf(v.x, cl, -sg * ys));
  const float im = fmaf(v.y, ch, fmaf(v.y, cl, sg * xs));
  return make_float2(re, im);
}
template <int K> FIL_DEV double2 rot8(double2 v, double sg) {
  const double c1 = 0.92387953251128675613, s1 = 0.38268343236508977173, c2 = 0.70710678118654752440;
  double c, s;
  if (K == 1) { c = c1; s = s1; }
  else if (K == 2) { c = c2; s = c2; }
  else { c = s1; s = c1; }
  return make_double2(v.x * c - sg * v.y * s, v.y * c + sg * v.x * s);
}

template <typename C> FIL_DEV void dft8(C* v, decltype(C().x) sg) {
  C e[4] = {v[0], v[2], v[4], v[6]};
  C o[4] = {v[1], v[3], v[5], v[7]};
  dft4<C>(e, sg);
  dft4<C>(o, sg);
  // W8^1 = exp(sg i pi/4), W8^2 = sg i, W8^3 = sg i W8^1
  C t0 = o[0], t1 = rot8<2>(o[1], sg), t2 = mul_si<C>(o[2], sg), t3 = mul_si<C>(rot8<2>(o[3], sg), sg);
  v[0] = e[0] + t0; v[4] = e[0] - t0;
  v[1] = e[1] + t1; v[5] = e[1] - t1;
  v[2] = e[2] + t2; v[6] = e[2] - t2;
  v[3] = e[3] + t3; v[7] = e[3] - t3;
}

template <typename C> FIL_DEV void dft16(C* v, decltype(C().x) sg) {
  C e[8], o[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) { e[i] = v[2 * i]; o[i] = v[2 * i + 1]; }
  dft8<C>(e, sg);
  dft8<C>(o, sg);
  // W16^k = exp(sg i k pi/8); W16^(k+4) = sg i W16^k
  C t[8];
  t[0] = o[0];
  t[1] = rot8<1>(o[1], sg);
  t[2] = rot8<2>(o[2], sg);
  t[3] = rot8<3>(o[3], sg);
  t[4] = mul_si<C>(o[4], sg);
  t[5] = mul_si<C>(rot8<1>(o[5], sg), sg);
  t[6] = mul_si<C>(rot8<2>(o[6], sg), sg);
  t[7] = mul_si<C>(rot8<3>(o[7], sg), sg);
#pragma unroll
  for (int k = 0; k < 8; ++k) { v[k] = e[k] + t[k]; v[k + 8] = e[k] - t[k]; }
}

template <typename C, int RD> FIL_DEV void dft(C* v, decltype(C().x) sg) {
  if constexpr (RD == 2) dft2<C>(v);
  else if constexpr (RD == 4) dft4<C>(v, sg);
  else if constexpr (RD == 8) dft8<C>(v, sg);
  else dft16<C>(v, sg);
}

// One Stockham pass.  Padded indices are formed once per butterfly group:
// pad16(b + r NB) = pad16(b) + r (NB + NB/16) when NB is a multiple of 16,
// and the output run o + r NS likewise (NS a multiple of 16), or, for
// NS = 1 with RD = 16, o = 16 b and pad16(o + r) = o + b + r.
template <typename C, int N, int RD, int NS>
FIL_DEV void pass(C* s, const C* __restrict__ tp, int tid, decltype(C().x) sg) {
  constexpr int T = N / 16;
  constexpr int NB = N / RD;
  constexpr int Q = NB / T;
  C v[Q][RD];
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int b = tid + q * T;
    if constexpr (NB % 16 == 0) {
      const int pb = pad16(b);
#pragma unroll
      for (int r = 0; r < RD; ++r) v[q][r] = s[pb + r * (NB + NB / 16)];
    } else {
#pragma unroll
      for (int r = 0; r < RD; ++r) v[q][r] = s[pad16(b + r * NB)];
    }
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const int b = tid + q * T;
    const int k = b % NS;
    if constexpr (NS > 1) {
#pragma unroll
      for (int r = 1; r < RD; ++r) {
        C w = __ldg(&tp[(r - 1) * NS + k]);
        w.y = -sg * w.y;          // conjugate for sg = +1
        v[q][r] = cmul(v[q][r], w);
      }
    }
    dft<C, RD>(v[q], sg);
    const int o = (b / NS) * NS * RD + k;
    if constexpr (NS % 16 == 0) {
      const int po = pad16(o);
#pragma unroll
      for (int r = 0; r < RD; ++r) s[po + r * (NS + NS / 16)] = v[q][r];
    } else if constexpr (NS == 1 && RD == 16) {
      const int po = o + b;
#pragma unroll
      for (int r = 0; r < RD; ++r) s[po + r] = v[q][r];
    } else {
#pragma unroll
      for (int r = 0; r < RD; ++r) s[pad16(o + r * NS)] = v[q][r];
    }
  }
  __syncthreads();
}

template <typename C, int N, int NS>
FIL_DEV void passes16(C* s, const C* __restrict__ tp, int tid, decltype(C().x) sg) {
  if constexpr (NS < N) {
    pass<C, N, 16, NS>(s, tp, tid, sg);
    passes16<C, N, NS * 16>(s, tp + (NS > 1 ? 15 * NS : 0), tid, sg);
  }
}


__host__ __device__ constexpr int ilog2(int n) { return n <= 1 ? 0 : 1 + ilog2(n / 2); }

// In-place FFT of s[pad16(0..N-1)] by a group of N/16 threads; `tid` is the
// thread's index in its group; sg = -1: X_k = sum_n x_n exp(-2 pi i k n / N),
// sg = +1: the same with exp(+...), unscaled.  Several groups may run side
// by side on their own arrays: every thread of the block must call it (the
// passes synchronise the whole block), all with the same N and sign.
template <typename C, int N>
FIL_DEV void group_fft_sg(C* s, const C* __restrict__ tw, int tid, decltype(C().x) sg) {
  static_assert(N >= 16 && (N & (N - 1)) == 0, "N must be a power of two >= 16");
  constexpr int L = ilog2(N);
  constexpr int R0 = 1 << (L % 4);
  __syncthreads();
  if constexpr (R0 > 1) {
    pass<C, N, R0, 1>(s, tw, tid, sg);
    passes16<C, N, R0>(s, tw, tid, sg);
  } else {
    passes16<C, N, 1>(s, tw, tid, sg);
  }
}

template <typename C, int N, int SIGN>
FIL_DEV void group_fft(C* s, const C* __restrict__ tw, int tid) {
  group_fft_sg<C, N>(s, tw, tid, (decltype(C().x))SIGN);
}

// In-place FFT of s[pad16(0..N-1)] by the N/16 threads of the block.
template <typename C, int N, int SIGN>
FIL_DEV void block_fft(C* s, const C* __restrict__ tw) {
  group_fft<C, N, SIGN>(s, tw, threadIdx.x);
}

// The same with the direction given at run time (one copy of the code).
template <typename C, int N>
FIL_DEV void block_fft_sg(C* s, const C* __restrict__ tw, decltype(C().x) sg) {
  group_fft_sg<C, N>(s, tw, threadIdx.x, sg);
}

}  // namespace filfft
