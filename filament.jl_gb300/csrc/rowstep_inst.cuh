// rowstep_inst.cuh -- definition of the row-kernel launchers; included by
// the rowstep_*.cu translation units, each instantiating one share.
#pragma once
#include "rowstep_launch.h"

template <typename R, int N, int NC>
static size_t rowstep_smem() {
  typedef typename C2T<R>::type C;
  constexpr int NP = N + N / 16;
  return 2 * NP * sizeof(C) + 2 * NP * sizeof(R) + 32 * sizeof(R) + 32 * sizeof(Aff<R, (NC > 0 ? NC : 1)>) +
         sizeof(PlasmaSmem<R>);
}

template <typename R, int N, int NC, bool RAM, bool TS>
cudaError_t launch_rowstep_t(const RowParams<R>& P, int mode, cudaStream_t st) {
  size_t sm = rowstep_smem<R, N, NC>();
  cudaError_t e =
      cudaFuncSetAttribute(k_rowstep<R, N, NC, RAM, TS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  k_rowstep<R, N, NC, RAM, TS><<<P.nrows, N / 16, sm, st>>>(P, mode);
  return cudaGetLastError();
}

// the Tsitouras methods (up to two species)
#define FIL_ROWSTEP_INST_TS(R, RAM)                                                                      \
  template cudaError_t launch_rowstep_t<R, 512, 0, RAM, true>(const RowParams<R>&, int, cudaStream_t);  \
  template cudaError_t launch_rowstep_t<R, 512, 1, RAM, true>(const RowParams<R>&, int, cudaStream_t);  \
  template cudaError_t launch_rowstep_t<R, 512, 2, RAM, true>(const RowParams<R>&, int, cudaStream_t);  \
  template cudaError_t launch_rowstep_t<R, 1024, 0, RAM, true>(const RowParams<R>&, int, cudaStream_t); \
  template cudaError_t launch_rowstep_t<R, 1024, 1, RAM, true>(const RowParams<R>&, int, cudaStream_t); \
  template cudaError_t launch_rowstep_t<R, 1024, 2, RAM, true>(const RowParams<R>&, int, cudaStream_t); \
  template cudaError_t launch_rowstep_t<R, 2048, 0, RAM, true>(const RowParams<R>&, int, cudaStream_t); \
  template cudaError_t launch_rowstep_t<R, 2048, 1, RAM, true>(const RowParams<R>&, int, cudaStream_t); \
  template cudaError_t launch_rowstep_t<R, 2048, 2, RAM, true>(const RowParams<R>&, int, cudaStream_t); \
  template cudaError_t launch_rowstep_t<R, 4096, 0, RAM, true>(const RowParams<R>&, int, cudaStream_t); \
  template cudaError_t launch_rowstep_t<R, 4096, 1, RAM, true>(const RowParams<R>&, int, cudaStream_t); \
  template cudaError_t launch_rowstep_t<R, 4096, 2, RAM, true>(const RowParams<R>&, int, cudaStream_t);

// three and four ionising species (paraxial prefactor, no Raman channel)
#define FIL_ROWSTEP_INST_NC34(R)                                                                    \
  template cudaError_t launch_rowstep_t<R, 512, 3, false>(const RowParams<R>&, int, cudaStream_t);  \
  template cudaError_t launch_rowstep_t<R, 512, 4, false>(const RowParams<R>&, int, cudaStream_t);  \
  template cudaError_t launch_rowstep_t<R, 1024, 3, false>(const RowParams<R>&, int, cudaStream_t); \
  template cudaError_t launch_rowstep_t<R, 1024, 4, false>(const RowParams<R>&, int, cudaStream_t); \
  template cudaError_t launch_rowstep_t<R, 2048, 3, false>(const RowParams<R>&, int, cudaStream_t); \
  template cudaError_t launch_rowstep_t<R, 2048, 4, false>(const RowParams<R>&, int, cudaStream_t); \
  template cudaError_t launch_rowstep_t<R, 4096, 3, false>(const RowParams<R>&, int, cudaStream_t); \
  template cudaError_t launch_rowstep_t<R, 4096, 4, false>(const RowParams<R>&, int, cudaStream_t);

#define FIL_ROWSTEP_INST(R, RAM)                                                                   \
  template cudaError_t launch_rowstep_t<R, 512, 0, RAM>(const RowParams<R>&, int, cudaStream_t);  \
  template cudaError_t launch_rowstep_t<R, 512, 1, RAM>(const RowParams<R>&, int, cudaStream_t);  \
  template cudaError_t launch_rowstep_t<R, 512, 2, RAM>(const RowParams<R>&, int, cudaStream_t);  \
  template cudaError_t launch_rowstep_t<R, 1024, 0, RAM>(const RowParams<R>&, int, cudaStream_t); \
  template cudaError_t launch_rowstep_t<R, 1024, 1, RAM>(const RowParams<R>&, int, cudaStream_t); \
  template cudaError_t launch_rowstep_t<R, 1024, 2, RAM>(const RowParams<R>&, int, cudaStream_t); \
  template cudaError_t launch_rowstep_t<R, 2048, 0, RAM>(const RowParams<R>&, int, cudaStream_t); \
  template cudaError_t launch_rowstep_t<R, 2048, 1, RAM>(const RowParams<R>&, int, cudaStream_t); \
  template cudaError_t launch_rowstep_t<R, 2048, 2, RAM>(const RowParams<R>&, int, cudaStream_t); \
  template cudaError_t launch_rowstep_t<R, 4096, 0, RAM>(const RowParams<R>&, int, cudaStream_t); \
  template cudaError_t launch_rowstep_t<R, 4096, 1, RAM>(const RowParams<R>&, int, cudaStream_t); \
  template cudaError_t launch_rowstep_t<R, 4096, 2, RAM>(const RowParams<R>&, int, cudaStream_t);

template <typename R, int N>
static size_t rowstage_smem() {
  typedef typename C2T<R>::type C;
  constexpr int NP = N + N / 16;
  return 2 * NP * sizeof(C) + 2 * NP * sizeof(R);
}

template <typename R, int N, int NC, bool RAM>
cudaError_t launch_rowstage_t(const RowParams<R>& P, cudaStream_t st) {
  size_t sm = rowstage_smem<R, N>();
  cudaError_t e =
      cudaFuncSetAttribute(k_rowstage<R, N, NC, RAM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  k_rowstage<R, N, NC, RAM><<<P.nrows, N / 16, sm, st>>>(P);
  return cudaGetLastError();
}

#define FIL_ROWSTAGE_INST_N(R, N)                                                                 \
  template cudaError_t launch_rowstage_t<R, N, 0, false>(const RowParams<R>&, cudaStream_t);    \
  template cudaError_t launch_rowstage_t<R, N, 1, false>(const RowParams<R>&, cudaStream_t);    \
  template cudaError_t launch_rowstage_t<R, N, 2, false>(const RowParams<R>&, cudaStream_t);    \
  template cudaError_t launch_rowstage_t<R, N, 0, true>(const RowParams<R>&, cudaStream_t);     \
  template cudaError_t launch_rowstage_t<R, N, 1, true>(const RowParams<R>&, cudaStream_t);     \
  template cudaError_t launch_rowstage_t<R, N, 2, true>(const RowParams<R>&, cudaStream_t);
#define FIL_ROWSTAGE_INST(R)        \
  FIL_ROWSTAGE_INST_N(R, 512)       \
  FIL_ROWSTAGE_INST_N(R, 1024)      \
  FIL_ROWSTAGE_INST_N(R, 2048)      \
  FIL_ROWSTAGE_INST_N(R, 4096)
