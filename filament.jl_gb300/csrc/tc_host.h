// tc_host.h -- host helpers for the tensor-core GEMMs: TMA tensor maps
// through the driver entry point (no link-time dependency on libcuda).
#pragma once
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

static inline PFN_cuTensorMapEncodeTiled_v12000 tc_encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
  }
  return fn;
}

// 2-D row-major tensor [outer][inner] of FP32 (elem 4) or FP16 (elem 2),
// box [box_outer][box_inner]; the swizzle span is the box row
// (box_inner * elem = 128 B: 128-byte swizzle, 64 B: 64-byte swizzle).
// Returns 0 on success.
static inline int tc_make_map(CUtensorMap* m, const void* base, int elem, unsigned long long inner,
                              unsigned long long outer, unsigned box_inner, unsigned box_outer) {
  PFN_cuTensorMapEncodeTiled_v12000 fn = tc_encode_fn();
  if (!fn) return -1;
  const unsigned row = box_inner * (unsigned)elem;
  CUtensorMapSwizzle sw;
  if (row == 128) sw = CU_TENSOR_MAP_SWIZZLE_128B;
  else if (row == 64) sw = CU_TENSOR_MAP_SWIZZLE_64B;
  else return -2;
  cuuint64_t dims[2] = {inner, outer};
  cuuint64_t strides[1] = {inner * (unsigned long long)elem};
  cuuint32_t box[2] = {box_inner, box_outer};
  cuuint32_t es[2] = {1, 1};
  CUtensorMapDataType dt = (elem == 4) ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16;
  CUresult r = fn(m, dt, 2, const_cast<void*>(base), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, sw,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? 0 : (int)r;
}

// BF16 tensor of rank 2 or 3 (dims[0] contiguous, dims[i] elements, packed
// rows), box `box`; 128-byte swizzle (the box row must be 128 B); elements
// outside the tensor read as zero.  Returns 0 on success.
static inline int tc_make_map_bf16(CUtensorMap* m, const void* base, int rank, const unsigned long long* dims,
                                   const unsigned* box) {
  PFN_cuTensorMapEncodeTiled_v12000 fn = tc_encode_fn();
  if (!fn) return -1;
  if (rank < 2 || rank > 3 || box[0] * 2 != 128) return -2;
  cuuint64_t d[3], s[2];
  cuuint32_t b[3], es[3] = {1, 1, 1};
  for (int i = 0; i < rank; ++i) {
    d[i] = dims[i];
    b[i] = box[i];
  }
  s[0] = dims[0] * 2ull;
  if (rank == 3) s[1] = dims[0] * dims[1] * 2ull;
  CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, (cuuint32_t)rank, const_cast<void*>(base), d, s, b, es,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? 0 : (int)r;
}
