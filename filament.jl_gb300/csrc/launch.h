// launch.h -- host-side launch wrappers shared by the translation units.
#pragma once
#include <cuda_runtime.h>

#include <cuda.h>
#include <string>

#include "common.cuh"

// sets the message that fil_last_error(NULL) returns
void fil_set_global_error(const std::string& m);

struct DevCtl;
template <typename R> struct RowParams;
template <typename R> struct PropParams;

template <typename R>
cudaError_t launch_rowstep(const RowParams<R>& P, int n, int nc, int mode, cudaStream_t st);
template <typename R>
cudaError_t launch_rowstage(const RowParams<R>& P, int n, int nc, cudaStream_t st);
template <typename R>
cudaError_t launch_np_combine(const RowParams<R>& P, int nh, cudaStream_t st);
template <typename R>
cudaError_t launch_rowreduce(const RowParams<R>& P, int n, double* fluence, R* Iout, int check_done,
                             cudaStream_t st);
template <typename R>
cudaError_t launch_colsum(const R* I, const double* w, double* power, int nrows, int nt, cudaStream_t st);
template <typename R>
cudaError_t launch_rowspec(const RowParams<R>& P, int n, R* out, cudaStream_t st);
template <typename R>
cudaError_t launch_field_in(const typename C2T<R>::type* E, typename C2T<R>::type* S, typename C2T<R>::type* U,
                            int ld, const typename C2T<R>::type* tw, int analytic, int nrows, int n,
                            cudaStream_t st);
template <typename R>
cudaError_t launch_field_out(const RowParams<R>& P, int n, typename C2T<R>::type* E, cudaStream_t st);
template <typename R>
cudaError_t launch_dht_simt(const R* A, const R* B, R* C, int M, int N, int K, const PropParams<R>& pp,
                            DevCtl* ctl, int epi, cudaStream_t st);
struct TcGemmParams;
cudaError_t launch_dht_tc(const CUtensorMap (&a)[3], const CUtensorMap (&b)[3], const TcGemmParams& p, int M,
                          int N, cudaStream_t st);
cudaError_t launch_slice(const float* B, void* const (&s)[3], float* qb, int N, int K, const DevCtl* ctl,
                         cudaStream_t st);
cudaError_t launch_slice_prop(const float* W, const float2* kz, const float* gd, void* const (&s)[3], float* qb, int nh,
                              int K, const DevCtl* ctl, cudaStream_t st);
// slices of the forward transform's output W [2 nh][K] times the complex
// factor f [nh][K] (non-paraxial prefactor)
cudaError_t launch_slice_mul(const float* W, const float2* f, void* const (&s)[3], float* qb, int nh, int K,
                             const DevCtl* ctl, cudaStream_t st);
cudaError_t launch_control(DevCtl* c, const double* fluence, const double* w, int nrows, cudaStream_t st);
// R geometry: one Hankel matrix-vector product (dht_vec.cu); mode 1 times
// the propagator, mode 2 times the field guard g_row
template <typename R>
cudaError_t launch_dht_vec(const R* M, const typename C2T<R>::type* in, typename C2T<R>::type* out, int n, int ldm,
                           const PropParams<R>& pp, const R* g_row, DevCtl* ctl, int mode, cudaStream_t st);
cudaError_t launch_flush(void* buf, size_t bytes, cudaStream_t st);
cudaError_t launch_setdz(DevCtl* c, double z, double dz, cudaStream_t st);
cudaError_t launch_batch_live(DevCtl* const* c, int n, int* live, cudaStream_t st);

// learned plasma surrogate (surrogate.cu): the network over the rows below
// *count (device value) of x0 [rows][3][T] (BF16) into out [rows][T];
// a1, a2: BF16 scratch [rows][64][T]; `stop` non-zero skips the launches
struct fil_nn;
int nn_time_points(const fil_nn* n);
cudaError_t nn_forward_rows(const fil_nn* n, const void* x0, void* a1, void* a2, float* out, int T, int maxrows,
                            const int* count, const int* stop, cudaStream_t st);

