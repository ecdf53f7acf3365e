// noalloc.cu -- the linear propagator of an RT z-step on caller-owned device
// buffers, without any device allocation.
//
// Some callers cannot allocate device memory at the point where they need
// the propagator: a host that pre-reserves all device memory and hands out
// fixed pools, a loop that must not pay for the device-wide synchronisation
// of cudaMalloc/cudaFree, or a caller that must not grow the process's
// memory footprint after start-up.  fil_hankel_propagate_noalloc serves them: the caller passes every
// input and the output; the one intermediate (the Hankel-transformed,
// propagated spectrum) lives in a file-scope __device__ array of fixed size
// that every GPU loading this library holds until the process exits.
#include <mutex>
#include <string>

#include <cuda.h>
#include <cudaTypedefs.h>

#include "../../include/filament_gb.h"
#include "launch.h"
#include "rowkernels.cuh"
#include "dht_simt.cuh"

// 4 Mi floats = 16 MiB: one [128-padded Nr][Nt] real view of the half
// spectrum up to Nr <= 1024, Nt <= 4096.
#define FIL_NOALLOC_MAX_FLOATS (4u << 20)
#define FIL_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) float g_noalloc_scratch[FIL_NOALLOC_MAX_FLOATS];
static __device__ DevCtl g_noalloc_ctl;

namespace {
std::mutex g_mu;
// per device: the device addresses of the two arrays and the unique ID of
// the context they were looked up in (a device reset, or the primary
// context torn down and created again, reloads the module, possibly at
// another address; the lookup is then redone)
float* g_scratch[FIL_NOALLOC_MAX_DEVICES];
DevCtl* g_ctl[FIL_NOALLOC_MAX_DEVICES];
unsigned long long g_ctx_id[FIL_NOALLOC_MAX_DEVICES];

// unique ID of the current context (0: none current, or the driver call is
// unavailable), through the driver entry points (no link-time libcuda)
unsigned long long current_context_id() {
  static PFN_cuCtxGetCurrent_v4000 get_cur = nullptr;
  static PFN_cuCtxGetId_v12000 get_id = nullptr;
  if (!get_cur || !get_id) {
    void* p = nullptr;
    void* q = nullptr;
    cudaDriverEntryPointQueryResult r1, r2;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 4000, cudaEnableDefault, &r1) != cudaSuccess ||
        r1 != cudaDriverEntryPointSuccess ||
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &q, 12000, cudaEnableDefault, &r2) != cudaSuccess ||
        r2 != cudaDriverEntryPointSuccess)
      return 0;
    get_cur = (PFN_cuCtxGetCurrent_v4000)p;
    get_id = (PFN_cuCtxGetId_v12000)q;
  }
  CUcontext c = nullptr;
  if (get_cur(&c) != CUDA_SUCCESS || !c) return 0;
  unsigned long long id = 0;
  if (get_id(c, &id) != CUDA_SUCCESS) return 0;
  return id;
}

// the message is read back with fil_last_error(NULL)
int noalloc_fail(int code, const std::string& m) {
  fil_set_global_error(m);
  return code;
}

__global__ void k_noalloc_arm(DevCtl* c, double dz) {
  c->done = 0;
  c->dz = dz;
}
}  // namespace

extern "C" int fil_hankel_propagate_noalloc(const float* m1, const float* m2, const float* kt2, const float* beta,
                                            const float* dfr, const float* kmax2, const float* wg, int kparaxial,
                                            const float* in, float* out, int mpad, int nh, double dz,
                                            void* stream) {
  if (!m1 || !m2 || !kt2 || !beta || !dfr || !in || !out) return noalloc_fail(FIL_ERR_ARG, "null pointer argument");
  if (mpad <= 0 || mpad % 128 != 0) return noalloc_fail(FIL_ERR_ARG, "mpad must be a positive multiple of 128");
  // mpad >= 128, so mpad * 2 nh >= 256 nh: a larger nh exceeds the array
  // (checked before any int arithmetic on nh)
  if (nh > (int)(FIL_NOALLOC_MAX_FLOATS / 256))
    return noalloc_fail(FIL_ERR_ARG, "nh = " + std::to_string(nh) + " exceeds the fixed scratch of " +
                                         std::to_string(FIL_NOALLOC_MAX_FLOATS) + " floats (16 MiB)");
  if (nh <= 0 || (2 * nh) % 128 != 0) return noalloc_fail(FIL_ERR_ARG, "2*nh must be a positive multiple of 128");
  const unsigned long long need = (unsigned long long)mpad * (2ull * (unsigned long long)nh);
  if (need > FIL_NOALLOC_MAX_FLOATS)
    return noalloc_fail(FIL_ERR_ARG, "mpad * 2 * nh = " + std::to_string(need) +
                                         " exceeds the fixed scratch of " + std::to_string(FIL_NOALLOC_MAX_FLOATS) +
                                         " floats (16 MiB)");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return noalloc_fail(FIL_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= FIL_NOALLOC_MAX_DEVICES) return noalloc_fail(FIL_ERR_ARG, "device index out of range");
  float* scratch;
  DevCtl* ctl;
  {
    // set-up per device, with that device current: the device addresses of
    // the static arrays (the host-side names are not device addresses);
    // done on the first call and again after the device's context changed
    std::lock_guard<std::mutex> lk(g_mu);
    const unsigned long long ctx = current_context_id();
    if (!g_scratch[dev] || ctx == 0 || ctx != g_ctx_id[dev]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess)
        return noalloc_fail(FIL_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
      void* q = nullptr;
      e = cudaGetSymbolAddress(&q, g_noalloc_ctl);
      if (e != cudaSuccess)
        return noalloc_fail(FIL_ERR_CUDA, std::string("cudaGetSymbolAddress(ctl): ") + cudaGetErrorString(e));
      g_scratch[dev] = (float*)p;
      g_ctl[dev] = (DevCtl*)q;
      // the lookup made the device's primary context current if none was
      g_ctx_id[dev] = current_context_id();
    }
    scratch = g_scratch[dev];
    ctl = g_ctl[dev];
  }
  cudaStream_t st = (cudaStream_t)stream;
  PropParams<float> pp;
  pp.kt2 = kt2;
  pp.beta = (const float2*)beta;
  pp.dfr = (const float2*)dfr;
  pp.kmax2 = kmax2;
  pp.wg = wg;
  pp.kparaxial = kparaxial;
  k_noalloc_arm<<<1, 1, 0, st>>>(ctl, dz);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = launch_dht_simt<float>(m1, in, scratch, mpad, 2 * nh, mpad, pp, ctl, 1, st);
  if (e == cudaSuccess) e = launch_dht_simt<float>(m2, scratch, out, mpad, 2 * nh, mpad, pp, ctl, 2, st);
  if (e != cudaSuccess) return noalloc_fail(FIL_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
  return FIL_OK;
}
