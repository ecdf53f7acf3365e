// rowkernels.cu -- instantiations of the row and DHT kernels and the
// controller kernel, plus host-side launch wrappers used by api.cu.
#include <cstdio>

#include "launch.h"
#include "rowkernels.cuh"
#include "dht_simt.cuh"
#include "rowstep_launch.h"

// ---------------------------------------------------------------------------
// Controller (AdaptiveSteps.jl:96-107, Filament.jl:123-164): one block.
__global__ void k_control(DevCtl* c, const double* __restrict__ fluence, const double* __restrict__ w,
                          int nrows) {
  __shared__ double sc[32];
  if (c->done) return;
  double e = 0;
  for (int i = threadIdx.x; i < nrows; i += blockDim.x) e += fluence[i] * w[i];
  e = block_sum<double>(e, sc);
  if (threadIdx.x != 0) return;
  const double imax = __longlong_as_double((long long)c->imax_acc);
  const double rhomax = __longlong_as_double((long long)c->rhomax_acc);
  c->imax = imax;
  c->rhomax = rhomax;
  c->energy = e;
  c->imax_acc = 0;
  if (c->flags & FIL_FLAG_NAN) { c->done = 1; c->status = -3; return; }
  if (!c->first && imax > c->istop) { c->done = 1; c->status = 2; c->flags |= FIL_FLAG_ISTOP; return; }
  if (!(c->z < c->zmax)) { c->done = 1; c->status = 1; return; }
  if (c->run_steps >= c->nmax) { c->done = 1; c->status = 3; return; }
  double dz = c->dz0;
  if (c->nonlinearity) {
    if (imax > 0) dz = fmin(dz, c->phimax / (c->phik * imax));
    if (c->phip > 0 && rhomax > 0) dz = fmin(dz, c->phimax / (c->phip * rhomax));
  }
  if (c->clamp_last && c->z + dz > c->zmax) dz = c->zmax - c->z;
  if (c->nn_on) {
    // the step just taken was a check step: every row ran the ODE, rhomax is
    // its maximum
    if (c->nn_check) {
      const double diff = __longlong_as_double((long long)c->nn_diff_acc);
      const double err = rhomax > 0 ? diff / rhomax : (diff > 0 ? 1.0 : 0.0);
      c->nn_err = err;
      c->nn_err_max = fmax(c->nn_err_max, err);
      c->nn_checked += 1;
      c->nn_use = err <= c->nn_tol;
      if (!c->nn_use) c->nn_rejected += 1;
      c->nn_diff_acc = 0;
    }
    c->nn_check = (c->nn_steps % c->nn_every) == 0;
    c->nn_rows = (c->nn_use || c->nn_check) ? c->nn_count : 0;
    c->nn_tiles_run = (c->nn_use || c->nn_check) ? c->nn_tiles : 0;
    if (c->nn_use && !c->nn_check) {
      c->nn_used += 1;
      c->nn_rows_sum += c->nn_rows;
      c->nn_tiles_sum += c->nn_tiles;
    }
    c->nn_steps += 1;
  } else {
    c->nn_check = 0;
    c->nn_rows = 0;
    c->nn_tiles_run = 0;
  }
  c->nn_count = 0;
  c->nn_tiles = 0;
  c->z += dz;
  c->dz = dz;
  c->steps += 1;
  c->run_steps += 1;
  c->first = 0;
  c->rhomax_acc = 0;
}

// fil_step: latch the plasma maximum of the previous solve, set z and dz.
__global__ void k_setdz(DevCtl* c, double z, double dz) {
  c->done = 0;
  c->nn_check = 0;   // single steps solve the plasma equation
  c->nn_rows = 0;
  c->nn_count = 0;
  c->nn_tiles = c->nn_tiles_run = 0;
  c->rhomax = __longlong_as_double((long long)c->rhomax_acc);
  c->rhomax_acc = 0;
  c->z = z;
  c->dz = dz;
  c->steps += 1;
  c->first = 0;
}

// ---------------------------------------------------------------------------
template <typename R, int N> static size_t x_smem() {
  typedef typename C2T<R>::type C;
  return (N + N / 16) * sizeof(C) + 64 * sizeof(double);
}

template <typename R, int N>
static cudaError_t launch_rowstep_n(const RowParams<R>& P, int nc, int mode, cudaStream_t st) {
  const bool ram = P.has_raman != 0;
  if (P.tsit && mode == 0) {   // Tsitouras step kernels (nc <= 2, checked at fil_create)
    if (nc == 0)
      return ram ? launch_rowstep_t<R, N, 0, true, true>(P, mode, st) : launch_rowstep_t<R, N, 0, false, true>(P, mode, st);
    if (nc == 1)
      return ram ? launch_rowstep_t<R, N, 1, true, true>(P, mode, st) : launch_rowstep_t<R, N, 1, false, true>(P, mode, st);
    if (nc == 2)
      return ram ? launch_rowstep_t<R, N, 2, true, true>(P, mode, st) : launch_rowstep_t<R, N, 2, false, true>(P, mode, st);
    return cudaErrorInvalidValue;
  }
  if (nc == 0) return ram ? launch_rowstep_t<R, N, 0, true>(P, mode, st) : launch_rowstep_t<R, N, 0, false>(P, mode, st);
  if (nc == 1) return ram ? launch_rowstep_t<R, N, 1, true>(P, mode, st) : launch_rowstep_t<R, N, 1, false>(P, mode, st);
  if (nc == 2) return ram ? launch_rowstep_t<R, N, 2, true>(P, mode, st) : launch_rowstep_t<R, N, 2, false>(P, mode, st);
  if (ram) return cudaErrorInvalidValue;   // refused at fil_create
  return nc == 3 ? launch_rowstep_t<R, N, 3, false>(P, mode, st) : launch_rowstep_t<R, N, 4, false>(P, mode, st);
}

template <typename R>
cudaError_t launch_rowstep(const RowParams<R>& P, int n, int nc, int mode, cudaStream_t st) {
  switch (n) {
    case 512: return launch_rowstep_n<R, 512>(P, nc, mode, st);
    case 1024: return launch_rowstep_n<R, 1024>(P, nc, mode, st);
    case 2048: return launch_rowstep_n<R, 2048>(P, nc, mode, st);
    case 4096: return launch_rowstep_n<R, 4096>(P, nc, mode, st);
  }
  return cudaErrorInvalidValue;
}

template <typename R, int N>
static cudaError_t launch_rowstage_n(const RowParams<R>& P, int nc, cudaStream_t st) {
  const bool ram = P.has_raman != 0;
  if (nc == 0) return ram ? launch_rowstage_t<R, N, 0, true>(P, st) : launch_rowstage_t<R, N, 0, false>(P, st);
  if (nc == 1) return ram ? launch_rowstage_t<R, N, 1, true>(P, st) : launch_rowstage_t<R, N, 1, false>(P, st);
  if (nc == 2) return ram ? launch_rowstage_t<R, N, 2, true>(P, st) : launch_rowstage_t<R, N, 2, false>(P, st);
  return cudaErrorInvalidValue;   // refused at fil_create
}

template <typename R>
cudaError_t launch_rowstage(const RowParams<R>& P, int n, int nc, cudaStream_t st) {
  switch (n) {
    case 512: return launch_rowstage_n<R, 512>(P, nc, st);
    case 1024: return launch_rowstage_n<R, 1024>(P, nc, st);
    case 2048: return launch_rowstage_n<R, 2048>(P, nc, st);
    case 4096: return launch_rowstage_n<R, 4096>(P, nc, st);
  }
  return cudaErrorInvalidValue;
}

template <typename R>
cudaError_t launch_np_combine(const RowParams<R>& P, int nh, cudaStream_t st) {
  k_np_combine<R><<<P.nrows, 256, 0, st>>>(P, nh);
  return cudaGetLastError();
}

template <typename R, int N>
static cudaError_t launch_rowreduce_n(const RowParams<R>& P, double* fl, R* Iout, int check_done, cudaStream_t st) {
  size_t sm = x_smem<R, N>();
  cudaError_t e = cudaFuncSetAttribute(k_rowreduce<R, N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  k_rowreduce<R, N><<<P.nrows, N / 16, sm, st>>>(P, fl, Iout, check_done);
  return cudaGetLastError();
}
template <typename R>
cudaError_t launch_rowreduce(const RowParams<R>& P, int n, double* fl, R* Iout, int check_done, cudaStream_t st) {
  switch (n) {
    case 512: return launch_rowreduce_n<R, 512>(P, fl, Iout, check_done, st);
    case 1024: return launch_rowreduce_n<R, 1024>(P, fl, Iout, check_done, st);
    case 2048: return launch_rowreduce_n<R, 2048>(P, fl, Iout, check_done, st);
    case 4096: return launch_rowreduce_n<R, 4096>(P, fl, Iout, check_done, st);
  }
  return cudaErrorInvalidValue;
}
template <typename R>
cudaError_t launch_rowspec(const RowParams<R>& P, int n, R* out, cudaStream_t st) {
  size_t sm = 0;
  switch (n) {
#define FIL_ROWSPEC_CASE(NN)                                                                              \
  case NN: {                                                                                              \
    sm = x_smem<R, NN>();                                                                                 \
    cudaError_t e = cudaFuncSetAttribute(k_rowspec<R, NN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm); \
    if (e != cudaSuccess) return e;                                                                       \
    k_rowspec<R, NN><<<P.nrows, NN / 16, sm, st>>>(P, out);                                               \
    return cudaGetLastError();                                                                            \
  }
    FIL_ROWSPEC_CASE(512)
    FIL_ROWSPEC_CASE(1024)
    FIL_ROWSPEC_CASE(2048)
    FIL_ROWSPEC_CASE(4096)
#undef FIL_ROWSPEC_CASE
  }
  return cudaErrorInvalidValue;
}
template <typename R>
cudaError_t launch_colsum(const R* I, const double* w, double* power, int nrows, int nt, cudaStream_t st) {
  dim3 grid((nt + 255) / 256, (nrows + 63) / 64);
  k_colsum<R><<<grid, 256, 0, st>>>(I, w, power, nrows, nt);
  return cudaGetLastError();
}

template <typename R, int N>
static cudaError_t launch_field_in_n(const typename C2T<R>::type* E, typename C2T<R>::type* S,
                                     typename C2T<R>::type* U, int ld, const typename C2T<R>::type* tw,
                                     int analytic, int nrows, cudaStream_t st) {
  size_t sm = x_smem<R, N>();
  cudaError_t e = cudaFuncSetAttribute(k_field_in<R, N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  k_field_in<R, N><<<nrows, N / 16, sm, st>>>(E, S, U, ld, tw, analytic);
  return cudaGetLastError();
}
template <typename R>
cudaError_t launch_field_in(const typename C2T<R>::type* E, typename C2T<R>::type* S, typename C2T<R>::type* U,
                            int ld, const typename C2T<R>::type* tw, int analytic, int nrows, int n,
                            cudaStream_t st) {
  switch (n) {
    case 512: return launch_field_in_n<R, 512>(E, S, U, ld, tw, analytic, nrows, st);
    case 1024: return launch_field_in_n<R, 1024>(E, S, U, ld, tw, analytic, nrows, st);
    case 2048: return launch_field_in_n<R, 2048>(E, S, U, ld, tw, analytic, nrows, st);
    case 4096: return launch_field_in_n<R, 4096>(E, S, U, ld, tw, analytic, nrows, st);
  }
  return cudaErrorInvalidValue;
}

template <typename R, int N>
static cudaError_t launch_field_out_n(const RowParams<R>& P, typename C2T<R>::type* E, cudaStream_t st) {
  size_t sm = x_smem<R, N>();
  cudaError_t e = cudaFuncSetAttribute(k_field_out<R, N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  k_field_out<R, N><<<P.nrows, N / 16, sm, st>>>(P, E);
  return cudaGetLastError();
}
template <typename R>
cudaError_t launch_field_out(const RowParams<R>& P, int n, typename C2T<R>::type* E, cudaStream_t st) {
  switch (n) {
    case 512: return launch_field_out_n<R, 512>(P, E, st);
    case 1024: return launch_field_out_n<R, 1024>(P, E, st);
    case 2048: return launch_field_out_n<R, 2048>(P, E, st);
    case 4096: return launch_field_out_n<R, 4096>(P, E, st);
  }
  return cudaErrorInvalidValue;
}

template <typename R>
cudaError_t launch_dht_simt(const R* A, const R* B, R* C, int M, int N, int K, const PropParams<R>& pp,
                            DevCtl* ctl, int epi, cudaStream_t st) {
  dim3 grid(N / 128, M / 128);
  if (epi == 1) k_dht_simt<R, 1><<<grid, 256, 0, st>>>(A, B, C, M, N, K, pp, ctl);
  else if (epi == 2) k_dht_simt<R, 2><<<grid, 256, 0, st>>>(A, B, C, M, N, K, pp, ctl);
  else if (epi == 3) k_dht_simt<R, 3><<<grid, 256, 0, st>>>(A, B, C, M, N, K, pp, ctl);
  else k_dht_simt<R, 4><<<grid, 256, 0, st>>>(A, B, C, M, N, K, pp, ctl);
  return cudaGetLastError();
}

cudaError_t launch_control(DevCtl* c, const double* fl, const double* w, int nrows, cudaStream_t st) {
  k_control<<<1, 256, 0, st>>>(c, fl, w, nrows);
  return cudaGetLastError();
}
// Writes a buffer larger than L2 so the next step starts with a cold cache
// (benchmark timing only).
__global__ void k_flush(float4* buf, size_t n, float v) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    buf[i] = make_float4(v, v, v, v);
}
cudaError_t launch_flush(void* buf, size_t bytes, cudaStream_t st) {
  k_flush<<<152 * 8, 256, 0, st>>>((float4*)buf, bytes / sizeof(float4), 0.0f);
  return cudaGetLastError();
}

// Batched sweep: number of members whose controller has not raised done
// (one block; read by the host after a run of batch steps).
__global__ void k_batch_live(DevCtl* const* c, int n, int* live) {
  __shared__ int s_live;
  if (threadIdx.x == 0) s_live = 0;
  __syncthreads();
  int k = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) k += c[i]->done ? 0 : 1;
  if (k) atomicAdd(&s_live, k);
  __syncthreads();
  if (threadIdx.x == 0) *live = s_live;
}
cudaError_t launch_batch_live(DevCtl* const* c, int n, int* live, cudaStream_t st) {
  k_batch_live<<<1, 256, 0, st>>>(c, n, live);
  return cudaGetLastError();
}

cudaError_t launch_setdz(DevCtl* c, double z, double dz, cudaStream_t st) {
  k_setdz<<<1, 1, 0, st>>>(c, z, dz);
  return cudaGetLastError();
}

#define INST(R)                                                                                          \
  template cudaError_t launch_rowstep<R>(const RowParams<R>&, int, int, int, cudaStream_t);            \
  template cudaError_t launch_rowstage<R>(const RowParams<R>&, int, int, cudaStream_t);                \
  template cudaError_t launch_np_combine<R>(const RowParams<R>&, int, cudaStream_t);                   \
  template cudaError_t launch_rowreduce<R>(const RowParams<R>&, int, double*, R*, int, cudaStream_t);   \
  template cudaError_t launch_colsum<R>(const R*, const double*, double*, int, int, cudaStream_t);       \
  template cudaError_t launch_rowspec<R>(const RowParams<R>&, int, R*, cudaStream_t);                    \
  template cudaError_t launch_field_in<R>(const C2T<R>::type*, C2T<R>::type*, C2T<R>::type*, int,         \
                                          const C2T<R>::type*, int, int, int, cudaStream_t);             \
  template cudaError_t launch_field_out<R>(const RowParams<R>&, int, C2T<R>::type*, cudaStream_t);      \
  template cudaError_t launch_dht_simt<R>(const R*, const R*, R*, int, int, int, const PropParams<R>&,  \
                                          DevCtl*, int, cudaStream_t);
INST(float)
INST(double)
