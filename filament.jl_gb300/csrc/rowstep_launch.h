// rowstep_launch.h -- launchers of the fused row kernel, one per
// (precision, row length, species, Raman, Tsitouras); the instantiations are spread over
// the rowstep_*.cu translation units so that they compile in parallel.
#pragma once
#include "rowkernels.cuh"

template <typename R, int N, int NC, bool RAM, bool TS = false>
cudaError_t launch_rowstep_t(const RowParams<R>& P, int mode, cudaStream_t st);

// non-paraxial stage kernel (k_rowstage) of the same shapes
template <typename R, int N, int NC, bool RAM>
cudaError_t launch_rowstage_t(const RowParams<R>& P, cudaStream_t st);
