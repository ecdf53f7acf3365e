// surrogate.cu -- training and inference of the plasma surrogate network
// (surrogate.cuh): the fil_nn_* entry points of include/filament_gb.h.
//
// One training iteration on a batch of B rows of T points: gather the rows
// (features to BF16), four forward convolutions (BF16 activations kept for
// the backward pass), masked squared error of ln w, then per layer the weight
// gradient (FP32 atomics) and the input gradient (the convolution with the
// flipped, transposed kernel), back through tanh, and Adam on the FP32 master
// parameters followed by the BF16 repacking of every layer.
#include <cmath>
#include <cstdint>
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/filament_gb.h"
#include "launch.h"
#include "nn_tc.h"
#include "surrogate.cuh"

struct fil_nn {
  int T = 0, bmax = 0;
  float* p = nullptr;   // FP32 master parameters
  float* m = nullptr;
  float* v = nullptr;
  float* g = nullptr;   // gradients
  __nv_bfloat16* wf[NN_LAYERS] = {};   // [ci][k][co]
  __nv_bfloat16* wb[NN_LAYERS] = {};   // [co][k][ci], k flipped
  __nv_bfloat16* wt[NN_LAYERS] = {};   // [k][co][ci], layers 1 and 2 (tensor cores)
  CUtensorMap wmap[NN_LAYERS];         // TMA maps over wt
  __nv_bfloat16* act[NN_LAYERS] = {};   // x0, y0, y1, y2: [B][C][T]
  float* out = nullptr;                 // [B][T]
  float* gr[2] = {};    // FP32 gradients of the activations [B][64][T]
  float* tgt = nullptr;
  float* mask = nullptr;
  float* loss = nullptr;
  float* data_f = nullptr;   // training rows on the device
  float* data_t = nullptr;
  float* data_m = nullptr;
  int data_rows = 0;
  long step = 0;
  cudaStream_t st = nullptr;
  std::string err;
};

static std::string g_nn_err;

static int nn_fail(fil_nn* n, int code, const std::string& m) {
  if (n) n->err = m;
  g_nn_err = m;
  fil_set_global_error(m);
  return code;
}
#define NK(call)                                                          \
  do {                                                                    \
    cudaError_t e_ = (call);                                              \
    if (e_ != cudaSuccess) return nn_fail(n, FIL_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

static int nn_pack(fil_nn* n) {
  for (int l = 0; l < NN_LAYERS; ++l) {
    const int w = nn_wsize(l);
    k_nn_pack<<<(w + 255) / 256, 256, 0, n->st>>>(n->p, n->wf[l], n->wb[l], n->wt[l], l);
    NK(cudaGetLastError());
  }
  return 0;
}

// x0 <- features of rows idx (host list) of the device data set, or of the
// caller's device array
__global__ void k_nn_gather(const float* __restrict__ f, const int* __restrict__ idx, __nv_bfloat16* x0, int B,
                            int T) {
  const long i = blockIdx.x * 256L + threadIdx.x;
  if (i >= (long)B * NN_IN * T) return;
  const int b = (int)(i / ((long)NN_IN * T));
  const long r = idx ? idx[b] : b;
  x0[i] = __float2bfloat16_rn(f[r * NN_IN * (long)T + (i - (long)b * NN_IN * T)]);
}
__global__ void k_nn_gather_t(const float* __restrict__ t, const float* __restrict__ m, const int* __restrict__ idx,
                              float* to, float* mo, int B, int T) {
  const long i = blockIdx.x * 256L + threadIdx.x;
  if (i >= (long)B * T) return;
  const int b = (int)(i / T);
  const long r = idx ? idx[b] : b;
  to[i] = t[r * T + (i - (long)b * T)];
  mo[i] = m[r * T + (i - (long)b * T)];
}

// The four layers: x0 -> a1 -> a2 -> a3 -> out.  Rows below *count (device)
// or B; a3 may alias a1 (inference).
int nn_forward_dev(const fil_nn* n, const __nv_bfloat16* x0, __nv_bfloat16* a1, __nv_bfloat16* a2,
                   __nv_bfloat16* a3, float* out, int T, int B, const int* count, const int* stop,
                   cudaStream_t st) {
  const int gx64 = (T + 31) / 32, gx1 = (T + 127) / 128;
  // rows in flight: about eight 256-thread blocks per SM, at most B
  const int gy64 = count ? std::max(1, std::min(B, (152 * 8 + gx64 - 1) / gx64)) : B;
  const int gy1 = count ? std::max(1, std::min(B, (152 * 16 + gx1 - 1) / gx1)) : B;
  dim3 g64(gx64, gy64), g1(gx1, gy1);
  k_nn_conv<NN_IN, 64, 32, 8, 1><<<g64, 256, 0, st>>>(x0, n->wf[0], n->p + nn_poff(0) + nn_wsize(0), a1, T, B, count,
                                                  stop);
  k_nn_conv<64, 64, 32, 8, 1><<<g64, 256, 0, st>>>(a1, n->wf[1], n->p + nn_poff(1) + nn_wsize(1), a2, T, B, count,
                                                   stop);
  k_nn_conv<64, 64, 32, 8, 1><<<g64, 256, 0, st>>>(a2, n->wf[2], n->p + nn_poff(2) + nn_wsize(2), a3, T, B, count,
                                                   stop);
  k_nn_conv<64, 1, 128, 1, 0><<<g1, 128, 0, st>>>(a3, n->wf[3], n->p + nn_poff(3) + nn_wsize(3), out, T, B, count,
                                                  stop);
  return (int)cudaGetLastError();
}

int nn_time_points(const fil_nn* n) { return n->T; }

cudaError_t nn_infer(const fil_nn* n, const NnRowsPlan& p, cudaStream_t st) {
  cudaError_t e = nn_launch_conv_tc(p.map_a1, n->wmap[1], n->p + nn_poff(1) + nn_wsize(1), p.a2, nullptr, nullptr, p,
                                    st, p.x0, n->wf[0], n->p + nn_poff(0) + nn_wsize(0));
  if (e == cudaSuccess)
    e = nn_launch_conv_tc(p.map_a2, n->wmap[2], n->p + nn_poff(2) + nn_wsize(2), nullptr, n->wf[3], p.part, p, st);
  return e;
}

const float* nn_out_bias(const fil_nn* n) { return n->p + nn_poff(3) + nn_wsize(3); }

cudaError_t nn_forward_rows(const fil_nn* n, const void* x0, void* a1, void* a2, float* out, int T, int maxrows,
                            const int* count, const int* stop, cudaStream_t st) {
  return (cudaError_t)nn_forward_dev(n, (const __nv_bfloat16*)x0, (__nv_bfloat16*)a1, (__nv_bfloat16*)a2,
                                     (__nv_bfloat16*)a1, out, T, maxrows, count, stop, st);
}

static int nn_forward(fil_nn* n, int B) {
  NK((cudaError_t)nn_forward_dev(n, n->act[0], n->act[1], n->act[2], n->act[3], n->out, n->T, B, nullptr, nullptr,
                                 n->st));
  return 0;
}

// loss and gradients of the batch in act[0], tgt, mask
static int nn_backward(fil_nn* n, int B, float inv_count) {
  const int T = n->T;
  const long nb = (long)B * T, nb64 = nb * 64;
  NK(cudaMemsetAsync(n->g, 0, nn_nparams() * sizeof(float), n->st));
  NK(cudaMemsetAsync(n->loss, 0, sizeof(float), n->st));
  float* g3 = n->gr[1];   // [B][1][T]
  k_nn_loss<<<(unsigned)((nb + 255) / 256), 256, 0, n->st>>>(n->out, n->tgt, n->mask, g3, n->loss, nb, inv_count);
  dim3 g64((T + 31) / 32, B);
  // layer 3 (64 -> 1)
  k_nn_wgrad<64, 1, 1><<<dim3(1, 64), 256, 0, n->st>>>(n->act[3], g3, n->g + nn_poff(3), n->g + nn_poff(3) + nn_wsize(3),
                                                      B, T);
  float* d = n->gr[0];
  k_nn_conv<1, 64, 32, 8, 0><<<g64, 256, 0, n->st>>>(g3, n->wb[3], (const float*)nullptr, d, T, B, nullptr, nullptr);
  k_nn_tanh_bwd<<<(unsigned)((nb64 + 255) / 256), 256, 0, n->st>>>(d, n->act[3], d, nb64);
  // layers 2, 1 (64 -> 64): gradient of layer l's output in d; the input
  // gradient goes to the other buffer
  for (int l = 2; l >= 1; --l) {
    float* dn = (d == n->gr[0]) ? n->gr[1] : n->gr[0];
    k_nn_wgrad<64, 64, 8><<<dim3(8, 64), 256, 0, n->st>>>(n->act[l], d, n->g + nn_poff(l),
                                                          n->g + nn_poff(l) + nn_wsize(l), B, T);
    k_nn_conv<64, 64, 32, 8, 0><<<g64, 256, 0, n->st>>>(d, n->wb[l], (const float*)nullptr, dn, T, B, nullptr,
                                                        nullptr);
    k_nn_tanh_bwd<<<(unsigned)((nb64 + 255) / 256), 256, 0, n->st>>>(dn, n->act[l], dn, nb64);
    d = dn;
  }
  // layer 0 (2 -> 64)
  k_nn_wgrad<NN_IN, 64, 8><<<dim3(8, NN_IN), 256, 0, n->st>>>(n->act[0], d, n->g + nn_poff(0), n->g + nn_poff(0) + nn_wsize(0),
                                                      B, T);
  NK(cudaGetLastError());
  return 0;
}

static void nn_free(fil_nn* n) {
  void* bufs[] = {n->p, n->m, n->v, n->g, n->tgt, n->mask, n->loss, n->data_f, n->data_t, n->data_m,
                  n->gr[0], n->gr[1], n->out};
  for (void* b : bufs)
    if (b) cudaFree(b);
  for (int l = 0; l < NN_LAYERS; ++l) {
    if (n->wf[l]) cudaFree(n->wf[l]);
    if (n->wb[l]) cudaFree(n->wb[l]);
    if (n->wt[l]) cudaFree(n->wt[l]);
  }
  for (int l = 0; l < NN_LAYERS; ++l)
    if (n->act[l]) cudaFree(n->act[l]);
  if (n->st) cudaStreamDestroy(n->st);
}

// batch buffers for up to b rows
static int nn_reserve(fil_nn* n, int b) {
  if (b <= n->bmax) return 0;
  for (int l = 0; l < NN_LAYERS; ++l)
    if (n->act[l]) { cudaFree(n->act[l]); n->act[l] = nullptr; }
  if (n->out) { cudaFree(n->out); n->out = nullptr; }
  for (int i = 0; i < 2; ++i)
    if (n->gr[i]) { cudaFree(n->gr[i]); n->gr[i] = nullptr; }
  if (n->tgt) cudaFree(n->tgt);
  if (n->mask) cudaFree(n->mask);
  const size_t bt = (size_t)b * n->T;
  NK(cudaMalloc(&n->act[0], bt * NN_IN * sizeof(__nv_bfloat16)));
  for (int l = 1; l < NN_LAYERS; ++l) NK(cudaMalloc(&n->act[l], bt * NN_CH * sizeof(__nv_bfloat16)));
  NK(cudaMalloc(&n->out, bt * sizeof(float)));
  for (int i = 0; i < 2; ++i) NK(cudaMalloc(&n->gr[i], bt * NN_CH * sizeof(float)));
  NK(cudaMalloc(&n->tgt, bt * sizeof(float)));
  NK(cudaMalloc(&n->mask, bt * sizeof(float)));
  n->bmax = b;
  return 0;
}

extern "C" {

int fil_nn_nparams(void) { return nn_nparams(); }

const char* fil_nn_last_error(const fil_nn* n) { return n ? n->err.c_str() : g_nn_err.c_str(); }

int fil_nn_create(int nt, uint64_t seed, fil_nn** out) {
  fil_nn* n = nullptr;
  if (!out || nt < 16) return nn_fail(nullptr, FIL_ERR_ARG, "bad argument");
  *out = nullptr;
  n = new fil_nn();
  n->T = nt;
  int rc = 0;
  auto mk = [&](void** p, size_t bytes) -> int {
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) return nn_fail(n, FIL_ERR_CUDA, cudaGetErrorString(e));
    return 0;
  };
  const int np = nn_nparams();
  {
    const cudaError_t e = cudaStreamCreateWithFlags(&n->st, cudaStreamNonBlocking);
    if (e != cudaSuccess) rc = nn_fail(n, FIL_ERR_CUDA, std::string("cudaStreamCreateWithFlags: ") + cudaGetErrorString(e));
  }
  for (void** p : {(void**)&n->p, (void**)&n->m, (void**)&n->v, (void**)&n->g})
    if (!rc) rc = mk(p, np * sizeof(float));
  if (!rc) rc = mk((void**)&n->loss, sizeof(float));
  for (int l = 0; l < NN_LAYERS && !rc; ++l) {
    rc = mk((void**)&n->wf[l], nn_wsize(l) * sizeof(__nv_bfloat16));
    if (!rc) rc = mk((void**)&n->wb[l], nn_wsize(l) * sizeof(__nv_bfloat16));
    if (!rc && (l == 1 || l == 2)) {
      rc = mk((void**)&n->wt[l], nn_wsize(l) * sizeof(__nv_bfloat16));
      if (!rc && nn_weight_map(&n->wmap[l], n->wt[l])) rc = nn_fail(n, FIL_ERR_CUDA, "weight tensor map");
    }
  }
  if (rc) {
    nn_free(n);
    delete n;
    return rc;
  }
  // uniform initialisation +-sqrt(3 / fan_in) (unit variance through tanh),
  // biases zero; splitmix64 stream from the seed
  std::vector<float> h(np, 0.f);
  uint64_t s = seed ? seed : 0x9E3779B97F4A7C15ull;
  auto rnd = [&]() {
    s += 0x9E3779B97F4A7C15ull;
    uint64_t z = s;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
  };
  for (int l = 0; l < NN_LAYERS; ++l) {
    // the output layer starts near zero: an untrained network gives g ~ 0,
    // the closed form with first-order avalanche
    const double a = std::sqrt(3.0 / (nn_ci(l) * NN_K)) * (l == NN_LAYERS - 1 ? 1e-2 : 1.0);
    for (int i = 0; i < nn_wsize(l); ++i) h[nn_poff(l) + i] = (float)((2.0 * rnd() - 1.0) * a);
  }
  if (cudaMemcpy(n->p, h.data(), np * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemset(n->m, 0, np * sizeof(float)) != cudaSuccess || cudaMemset(n->v, 0, np * sizeof(float)) != cudaSuccess ||
      nn_pack(n) || cudaStreamSynchronize(n->st) != cudaSuccess) {
    nn_free(n);
    delete n;
    return nn_fail(nullptr, FIL_ERR_CUDA, "initialisation failed");
  }
  *out = n;
  return FIL_OK;
}

int fil_nn_destroy(fil_nn* n) {
  if (!n) return FIL_OK;
  nn_free(n);
  delete n;
  return FIL_OK;
}

int fil_nn_get_params(fil_nn* n, float* p) {
  if (!n || !p) return nn_fail(n, FIL_ERR_ARG, "null argument");
  NK(cudaMemcpyAsync(p, n->p, nn_nparams() * sizeof(float), cudaMemcpyDeviceToHost, n->st));
  NK(cudaStreamSynchronize(n->st));
  return FIL_OK;
}

int fil_nn_set_params(fil_nn* n, const float* p) {
  if (!n || !p) return nn_fail(n, FIL_ERR_ARG, "null argument");
  NK(cudaMemcpyAsync(n->p, p, nn_nparams() * sizeof(float), cudaMemcpyHostToDevice, n->st));
  int rc = nn_pack(n);
  if (rc) return rc;
  NK(cudaStreamSynchronize(n->st));
  return FIL_OK;
}

int fil_nn_forward(fil_nn* n, const float* feat, int b, float* out) {
  if (!n || !feat || !out || b < 1) return nn_fail(n, FIL_ERR_ARG, "bad argument");
  int rc = nn_reserve(n, b);
  if (rc) return rc;
  const size_t bt = (size_t)b * n->T;
  float* df = nullptr;
  NK(cudaMallocAsync((void**)&df, bt * NN_IN * sizeof(float), n->st));
  NK(cudaMemcpyAsync(df, feat, bt * NN_IN * sizeof(float), cudaMemcpyHostToDevice, n->st));
  k_nn_gather<<<(unsigned)((bt * NN_IN + 255) / 256), 256, 0, n->st>>>(df, nullptr, n->act[0], b, n->T);
  rc = nn_forward(n, b);
  if (rc) return rc;
  NK(cudaMemcpyAsync(out, n->out, bt * sizeof(float), cudaMemcpyDeviceToHost, n->st));
  NK(cudaFreeAsync(df, n->st));
  NK(cudaStreamSynchronize(n->st));
  return FIL_OK;
}

// The inference path the simulation runs (tensor-core layers 1 and 2,
// channel-last activations) on host features; nt a multiple of 128.
int fil_nn_infer(fil_nn* n, const float* feat, int b, float* out) {
  if (!n || !feat || !out || b < 1) return nn_fail(n, FIL_ERR_ARG, "bad argument");
  if (n->T % 128) return nn_fail(n, FIL_ERR_UNSUPPORTED, "tensor-core inference needs nt a multiple of 128");
  const size_t bt = (size_t)b * n->T;
  float* df = nullptr;
  NnRowsPlan pl;
  std::memset(&pl, 0, sizeof pl);
  void* buf = nullptr;
  const size_t bytes = bt * NN_IN * 2 + 2 * bt * 64 * 2 + 10 * bt * sizeof(float) + 256;
  NK(cudaMallocAsync(&buf, bytes, n->st));
  NK(cudaMallocAsync((void**)&df, bt * NN_IN * sizeof(float), n->st));
  uint8_t* q = (uint8_t*)buf;
  pl.a1 = (__nv_bfloat16*)q;
  pl.a2 = pl.a1 + bt * 64;
  pl.part = (float*)(pl.a2 + bt * 64);
  float* dout = pl.part + 9 * bt;
  __nv_bfloat16* x0 = (__nv_bfloat16*)(dout + bt);
  pl.x0 = x0;
  pl.err = (int*)(x0 + bt * NN_IN + 64);
  pl.T = n->T;
  pl.maxrows = b;
  if (nn_plan_init(&pl)) {
    cudaFreeAsync(df, n->st);
    cudaFreeAsync(buf, n->st);
    return nn_fail(n, FIL_ERR_CUDA, "tensor map of the activations");
  }
  NK(cudaMemsetAsync(pl.err, 0, sizeof(int), n->st));
  NK(cudaMemcpyAsync(df, feat, bt * NN_IN * sizeof(float), cudaMemcpyHostToDevice, n->st));
  k_nn_gather<<<(unsigned)((bt * NN_IN + 255) / 256), 256, 0, n->st>>>(df, nullptr, x0, b, n->T);
  NK(nn_infer(n, pl, n->st));
  NK(nn_launch_out(pl.part, nn_out_bias(n), dout, n->T, b, n->st));
  int e = 0;
  NK(cudaMemcpyAsync(out, dout, bt * sizeof(float), cudaMemcpyDeviceToHost, n->st));
  NK(cudaMemcpyAsync(&e, pl.err, sizeof(int), cudaMemcpyDeviceToHost, n->st));
  NK(cudaFreeAsync(df, n->st));
  NK(cudaFreeAsync(buf, n->st));
  NK(cudaStreamSynchronize(n->st));
  if (e) return nn_fail(n, FIL_ERR_TIMEOUT, "a tensor-core pipeline wait timed out");
  return FIL_OK;
}

int fil_nn_grad(fil_nn* n, const float* feat, const float* tgt, const float* mask, int b, float* grad, float* loss) {
  if (!n || !feat || !tgt || !mask || !grad || b < 1) return nn_fail(n, FIL_ERR_ARG, "bad argument");
  int rc = nn_reserve(n, b);
  if (rc) return rc;
  const size_t bt = (size_t)b * n->T;
  float* df = nullptr;
  NK(cudaMallocAsync((void**)&df, bt * NN_IN * sizeof(float), n->st));
  NK(cudaMemcpyAsync(df, feat, bt * NN_IN * sizeof(float), cudaMemcpyHostToDevice, n->st));
  NK(cudaMemcpyAsync(n->tgt, tgt, bt * sizeof(float), cudaMemcpyHostToDevice, n->st));
  NK(cudaMemcpyAsync(n->mask, mask, bt * sizeof(float), cudaMemcpyHostToDevice, n->st));
  k_nn_gather<<<(unsigned)((bt * NN_IN + 255) / 256), 256, 0, n->st>>>(df, nullptr, n->act[0], b, n->T);
  double cnt = 0;
  for (size_t i = 0; i < bt; ++i) cnt += mask[i];
  rc = nn_forward(n, b);
  if (!rc) rc = nn_backward(n, b, cnt > 0 ? (float)(1.0 / cnt) : 0.f);
  if (rc) return rc;
  NK(cudaMemcpyAsync(grad, n->g, nn_nparams() * sizeof(float), cudaMemcpyDeviceToHost, n->st));
  if (loss) NK(cudaMemcpyAsync(loss, n->loss, sizeof(float), cudaMemcpyDeviceToHost, n->st));
  NK(cudaFreeAsync(df, n->st));
  NK(cudaStreamSynchronize(n->st));
  return FIL_OK;
}

// Adam training on a data set of `rows` rows (features [rows][3][T], targets
// and masks [rows][T], host arrays), `iters` iterations of `batch` rows
// drawn with a seeded generator; loss_hist[iters] receives the batch losses.
int fil_nn_train(fil_nn* n, const float* feat, const float* tgt, const float* mask, int rows, int batch, int iters,
                 float lr, uint64_t seed, float* loss_hist) {
  if (!n || !feat || !tgt || !mask || rows < 1 || batch < 1 || iters < 0) return nn_fail(n, FIL_ERR_ARG, "bad argument");
  int rc = nn_reserve(n, batch);
  if (rc) return rc;
  const size_t T = n->T;
  if (n->data_f) { cudaFree(n->data_f); cudaFree(n->data_t); cudaFree(n->data_m); }
  NK(cudaMalloc(&n->data_f, rows * NN_IN * T * sizeof(float)));
  NK(cudaMalloc(&n->data_t, rows * T * sizeof(float)));
  NK(cudaMalloc(&n->data_m, rows * T * sizeof(float)));
  NK(cudaMemcpyAsync(n->data_f, feat, rows * NN_IN * T * sizeof(float), cudaMemcpyHostToDevice, n->st));
  NK(cudaMemcpyAsync(n->data_t, tgt, rows * T * sizeof(float), cudaMemcpyHostToDevice, n->st));
  NK(cudaMemcpyAsync(n->data_m, mask, rows * T * sizeof(float), cudaMemcpyHostToDevice, n->st));
  std::vector<double> rowcnt(rows, 0.0);
  for (int r = 0; r < rows; ++r)
    for (size_t t = 0; t < T; ++t) rowcnt[r] += mask[r * T + t];
  int* didx = nullptr;
  NK(cudaMalloc(&didx, (size_t)iters * batch * sizeof(int) + sizeof(int)));
  std::vector<int> idx((size_t)iters * batch);
  std::vector<float> invc(iters);
  uint64_t s = seed ? seed : 1;
  for (int it = 0; it < iters; ++it) {
    double c = 0;
    for (int q = 0; q < batch; ++q) {
      s ^= s << 13; s ^= s >> 7; s ^= s << 17;   // xorshift64
      const int r = (int)(s % (uint64_t)rows);
      idx[(size_t)it * batch + q] = r;
      c += rowcnt[r];
    }
    invc[it] = c > 0 ? (float)(1.0 / c) : 0.f;
  }
  NK(cudaMemcpyAsync(didx, idx.data(), idx.size() * sizeof(int), cudaMemcpyHostToDevice, n->st));
  const size_t bt = (size_t)batch * T;
  std::vector<float> lh(iters, 0.f);
  float* dloss = nullptr;
  NK(cudaMalloc(&dloss, (size_t)iters * sizeof(float) + sizeof(float)));
  for (int it = 0; it < iters; ++it) {
    const int* bi = didx + (size_t)it * batch;
    k_nn_gather<<<(unsigned)((bt * NN_IN + 255) / 256), 256, 0, n->st>>>(n->data_f, bi, n->act[0], batch, (int)T);
    k_nn_gather_t<<<(unsigned)((bt + 255) / 256), 256, 0, n->st>>>(n->data_t, n->data_m, bi, n->tgt, n->mask, batch,
                                                                   (int)T);
    rc = nn_forward(n, batch);
    if (!rc) rc = nn_backward(n, batch, invc[it]);
    if (rc) break;
    NK(cudaMemcpyAsync(dloss + it, n->loss, sizeof(float), cudaMemcpyDeviceToDevice, n->st));
    ++n->step;
    NnAdam a;
    a.lr = lr;
    a.b1 = 0.9f;
    a.b2 = 0.999f;
    a.eps = 1e-8f;
    a.c1 = (float)(1.0 - std::pow(0.9, (double)n->step));
    a.c2 = (float)(1.0 - std::pow(0.999, (double)n->step));
    const int np = nn_nparams();
    k_nn_adam<<<(np + 255) / 256, 256, 0, n->st>>>(n->p, n->m, n->v, n->g, np, a);
    rc = nn_pack(n);
    if (rc) break;
  }
  if (!rc && iters > 0) NK(cudaMemcpyAsync(lh.data(), dloss, iters * sizeof(float), cudaMemcpyDeviceToHost, n->st));
  cudaStreamSynchronize(n->st);
  cudaFree(didx);
  cudaFree(dloss);
  if (rc) return rc;
  if (loss_hist) std::memcpy(loss_hist, lh.data(), iters * sizeof(float));
  return FIL_OK;
}

}  // extern "C"
