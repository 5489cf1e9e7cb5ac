// MLP engine of the learned far-wake surrogate (see mlp.h): FP32 CUDA-core
// kernels for forward, backward and Adam, and the vlm_mlp_* C ABI.
//
// GEMM: C[M x N] = op(A)[M x K] op(B)[K x N] (+ bias, + tanh), 64 x 64 output
// tile per 256-thread block, 4 x 4 outputs per thread, K in steps of 16
// through shared memory.  Each output sums k = 0..K-1 in order, so results
// (and the batch reductions of the weight gradients, which are GEMMs over the
// batch) do not depend on the launch configuration.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/vlm.h"
#include "mlp.h"
#include "vlm_bs.h"

namespace vlm {

extern thread_local std::string g_err;

namespace {

#define MLP_CUDA(x)                                                                        \
  do {                                                                                     \
    cudaError_t e_ = (x);                                                                  \
    if (e_ != cudaSuccess) throw std::runtime_error(std::string("CUDA: ") + cudaGetErrorString(e_)); \
  } while (0)

enum { EPI_NONE = 0, EPI_BIAS = 1, EPI_BIAS_TANH = 2 };

template <bool TA, bool TB, int EPI>
__global__ void __launch_bounds__(256) k_gemm(int M, int N, int K, const float* __restrict__ A, int lda,
                                              const float* __restrict__ B, int ldb, float* __restrict__ C, int ldc,
                                              const float* __restrict__ bias) {
  __shared__ float As[16][64 + 4];
  __shared__ float Bs[16][64 + 4];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
  float acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
  for (int k0 = 0; k0 < K; k0 += 16) {
    for (int e = threadIdx.x; e < 1024; e += 256) {
      int mm, kk;
      if (TA) {
        mm = e & 63;
        kk = e >> 6;
      } else {
        kk = e & 15;
        mm = e >> 4;
      }
      const int gm = m0 + mm, gk = k0 + kk;
      float a = 0.f;
      if (gm < M && gk < K) a = TA ? A[(size_t)gk * lda + gm] : A[(size_t)gm * lda + gk];
      As[kk][mm] = a;
    }
    for (int e = threadIdx.x; e < 1024; e += 256) {
      int nn, kk;
      if (TB) {
        kk = e & 15;
        nn = e >> 4;
      } else {
        nn = e & 63;
        kk = e >> 6;
      }
      const int gn = n0 + nn, gk = k0 + kk;
      float b = 0.f;
      if (gn < N && gk < K) b = TB ? B[(size_t)gn * ldb + gk] : B[(size_t)gk * ldb + gn];
      Bs[kk][nn] = b;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 16; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int gm = m0 + ty * 4 + i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gn = n0 + tx * 4 + j;
      if (gn >= N) continue;
      float c = acc[i][j];
      if (EPI >= EPI_BIAS) c += bias[gn];
      if (EPI == EPI_BIAS_TANH) c = tanhf(c);
      C[(size_t)gm * ldc + gn] = c;
    }
  }
}

template <bool TA, bool TB, int EPI>
void gemm(cudaStream_t st, int M, int N, int K, const float* A, int lda, const float* B, int ldb, float* C, int ldc,
          const float* bias) {
  if (M <= 0 || N <= 0) return;
  dim3 grid((N + 63) / 64, (M + 63) / 64);
  count_launch();
  k_gemm<TA, TB, EPI><<<grid, 256, 0, st>>>(M, N, K, A, lda, B, ldb, C, ldc, bias);
}

// dH <- dH * (1 - H^2): gradient through tanh, in place
__global__ void k_tanh_back(float* __restrict__ dH, const float* __restrict__ H, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) {
    const float h = H[i];
    dH[i] = dH[i] * (1.f - h * h);
  }
}

// out[c] = sum over rows r (in order) of X[r * ld + c]
__global__ void k_colsum(const float* __restrict__ X, int rows, int cols, int ld, float* __restrict__ out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cols) return;
  float s = 0.f;
  for (int r = 0; r < rows; ++r) s += X[(size_t)r * ld + c];
  out[c] = s;
}

// dY = 2 (Y - T) / (rows x cols); per-block partial sums of (Y - T)^2
constexpr int kLossThreads = 256;
__global__ void k_mse(const float* __restrict__ Y, const float* __restrict__ T, int64_t n, float scale,
                      float* __restrict__ dY, float* __restrict__ part) {
  __shared__ float red[kLossThreads];
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  float e2 = 0.f;
  if (i < n) {
    const float e = Y[i] - T[i];
    dY[i] = 2.f * e * scale;
    e2 = e * e;
  }
  red[threadIdx.x] = e2;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}
__global__ void k_sum_parts(const float* __restrict__ part, int n, float scale, float* __restrict__ out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  float s = 0.f;
  for (int i = 0; i < n; ++i) s += part[i];
  out[0] = s * scale;
}

__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       int64_t n, float lr, float b1, float b2, float eps, float c1, float c2) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

uint64_t splitmix(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

}  // namespace

void MlpShape::finalize() {
  nparam = 0;
  maxw = 0;
  for (int l = 0; l < nl; ++l) {
    woff[l] = nparam;
    nparam += (int64_t)sz[l + 1] * sz[l];
    boff[l] = nparam;
    nparam += sz[l + 1];
  }
  for (int l = 0; l <= nl; ++l) maxw = std::max(maxw, sz[l]);
}

void Mlp::create(const std::vector<int>& sizes, uint64_t seed, cudaStream_t stream) {
  if (sizes.size() < 2 || (int)sizes.size() > kMlpMaxLayers + 1) throw std::invalid_argument("MLP needs 2..9 layer sizes");
  for (int s : sizes)
    if (s <= 0 || s > 4096) throw std::invalid_argument("MLP layer sizes must be in [1, 4096]");
  st = stream;
  sh.nl = (int)sizes.size() - 1;
  for (size_t i = 0; i < sizes.size(); ++i) sh.sz[i] = sizes[i];
  sh.finalize();
  // Glorot-uniform weights from a seeded generator, zero biases
  std::vector<float> h((size_t)sh.nparam, 0.f);
  uint64_t s = seed;
  for (int l = 0; l < sh.nl; ++l) {
    const double a = std::sqrt(6.0 / (sh.sz[l] + sh.sz[l + 1]));
    for (int64_t i = 0; i < (int64_t)sh.sz[l + 1] * sh.sz[l]; ++i) {
      const double u = (double)(splitmix(s) >> 11) * (1.0 / 9007199254740992.0);
      h[(size_t)(sh.woff[l] + i)] = (float)((2.0 * u - 1.0) * a);
    }
  }
  MLP_CUDA(cudaMalloc(&p, sizeof(float) * sh.nparam));
  MLP_CUDA(cudaMalloc(&g, sizeof(float) * sh.nparam));
  MLP_CUDA(cudaMalloc(&m, sizeof(float) * sh.nparam));
  MLP_CUDA(cudaMalloc(&v, sizeof(float) * sh.nparam));
  MLP_CUDA(cudaMalloc(&loss, sizeof(float) * 2));
  MLP_CUDA(cudaMemcpy(p, h.data(), sizeof(float) * sh.nparam, cudaMemcpyHostToDevice));
  MLP_CUDA(cudaMemset(g, 0, sizeof(float) * sh.nparam));
  MLP_CUDA(cudaMemset(m, 0, sizeof(float) * sh.nparam));
  MLP_CUDA(cudaMemset(v, 0, sizeof(float) * sh.nparam));
  adamStep = 0;
  tcFits = tc.plan(sh);
  if (tcFits) {
    MLP_CUDA(cudaMalloc(&tcImg, tc.imgBytes));
    MLP_CUDA(cudaMalloc(&tcErr, sizeof(int)));
    MLP_CUDA(cudaMemset(tcErr, 0, sizeof(int)));
  }
  useTc = tcFits;
  tcStale = true;
}

bool Mlp::setTensorCores(bool on) {
  if (on && !tcFits) return false;
  useTc = on;
  return true;
}

void Mlp::destroy() {
  for (float* q : {p, g, m, v, act, dact, loss, part})
    if (q) cudaFree(q);
  p = g = m = v = act = dact = loss = part = nullptr;
  if (tcImg) cudaFree(tcImg);
  if (tcErr) cudaFree(tcErr);
  tcImg = nullptr;
  tcErr = nullptr;
  cap = 0;
}

void Mlp::reserve(int batch) {
  if (batch <= cap) return;
  if (act) cudaFree(act);
  if (dact) cudaFree(dact);
  if (part) cudaFree(part);
  act = dact = part = nullptr;
  MLP_CUDA(cudaMalloc(&act, sizeof(float) * (size_t)(sh.nl + 1) * batch * sh.maxw));
  MLP_CUDA(cudaMalloc(&dact, sizeof(float) * (size_t)2 * batch * sh.maxw));
  MLP_CUDA(cudaMalloc(&part, sizeof(float) * (size_t)((int64_t)batch * sh.maxw / kLossThreads + 2)));
  cap = batch;
}

void Mlp::forward(const float* X, int n, float* Y) {
  if (useTc) {
    if (tcStale) {
      tc_pack(p, sh, tc, tcImg, st);
      tcStale = false;
    }
    tc_forward(tc, tcImg, X, n, Y, tcErr, st);
    return;
  }
  const int chunk = std::max(cap, 1);
  for (int r0 = 0; r0 < n; r0 += chunk) {
    const int rows = std::min(chunk, n - r0);
    const float* H = X + (size_t)r0 * sh.sz[0];
    for (int l = 0; l < sh.nl; ++l) {
      const int in = sh.sz[l], out = sh.sz[l + 1];
      const bool last = l == sh.nl - 1;
      float* Z = last ? Y + (size_t)r0 * out : act + (size_t)(l + 1) * cap * sh.maxw;
      if (last) gemm<false, true, EPI_BIAS>(st, rows, out, in, H, in, p + sh.woff[l], in, Z, out, p + sh.boff[l]);
      else gemm<false, true, EPI_BIAS_TANH>(st, rows, out, in, H, in, p + sh.woff[l], in, Z, out, p + sh.boff[l]);
      H = Z;
    }
  }
}

void Mlp::grad(const float* X, const float* T, int n) {
  reserve(n);
  // forward, keeping every layer's output (layer 0 = X)
  const float* Hs[kMlpMaxLayers + 1];
  Hs[0] = X;
  for (int l = 0; l < sh.nl; ++l) {
    const int in = sh.sz[l], out = sh.sz[l + 1];
    float* Z = act + (size_t)(l + 1) * cap * sh.maxw;
    if (l == sh.nl - 1) gemm<false, true, EPI_BIAS>(st, n, out, in, Hs[l], in, p + sh.woff[l], in, Z, out, p + sh.boff[l]);
    else gemm<false, true, EPI_BIAS_TANH>(st, n, out, in, Hs[l], in, p + sh.woff[l], in, Z, out, p + sh.boff[l]);
    Hs[l + 1] = Z;
  }
  // loss and dY
  const int out = sh.sz[sh.nl];
  const int64_t ny = (int64_t)n * out;
  float* dZ = dact;
  const int nb = (int)((ny + kLossThreads - 1) / kLossThreads);
  count_launch();
  k_mse<<<nb, kLossThreads, 0, st>>>(Hs[sh.nl], T, ny, 1.f / (float)ny, dZ, part);
  count_launch();
  k_sum_parts<<<1, 32, 0, st>>>(part, nb, 1.f / (float)ny, loss);
  // backward
  for (int l = sh.nl - 1; l >= 0; --l) {
    const int in = sh.sz[l], o = sh.sz[l + 1];
    if (l < sh.nl - 1) {
      const int64_t cnt = (int64_t)n * o;
      count_launch();
      k_tanh_back<<<(unsigned)((cnt + 255) / 256), 256, 0, st>>>(dZ, Hs[l + 1], cnt);
    }
    // dW = dZ^T H_prev, db = column sums of dZ
    gemm<true, false, EPI_NONE>(st, o, in, n, dZ, o, Hs[l], in, g + sh.woff[l], in, nullptr);
    count_launch();
    k_colsum<<<(o + 127) / 128, 128, 0, st>>>(dZ, n, o, o, g + sh.boff[l]);
    if (l > 0) {
      float* dH = (dZ == dact) ? dact + (size_t)cap * sh.maxw : dact;
      gemm<false, false, EPI_NONE>(st, n, in, o, dZ, o, p + sh.woff[l], in, dH, in, nullptr);
      dZ = dH;
    }
  }
}

void Mlp::adam(float lr, float b1, float b2, float eps) {
  ++adamStep;
  tcStale = true;
  const float c1 = 1.f - std::pow(b1, (float)adamStep), c2 = 1.f - std::pow(b2, (float)adamStep);
  count_launch();
  k_adam<<<(unsigned)((sh.nparam + 255) / 256), 256, 0, st>>>(p, g, m, v, sh.nparam, lr, b1, b2, eps, c1, c2);
}

}  // namespace vlm

// ---------------------------------------------------------------------------
// C ABI (no counterpart in the reference: the learned part of this engine)
using namespace vlm;

struct vlm_mlp {
  Mlp net;
  float* dX = nullptr;
  float* dT = nullptr;
  float* dY = nullptr;
  int64_t capX = 0, capT = 0, capY = 0;
  ~vlm_mlp() {
    net.destroy();
    for (float* q : {dX, dT, dY})
      if (q) cudaFree(q);
  }
};

template <class F>
static int mlp_guard(F f) {
  try {
    f();
    return VLM_OK;
  } catch (const std::invalid_argument& e) {
    g_err = e.what();
    return VLM_ERR_INVALID;
  } catch (const std::exception& e) {
    g_err = e.what();
    return VLM_ERR_CUDA;
  }
}

static void grow_dev(float** q, int64_t& cap, int64_t n) {
  if (n <= cap) return;
  if (*q) cudaFree(*q);
  *q = nullptr;
  MLP_CUDA(cudaMalloc(q, sizeof(float) * (size_t)n));
  cap = n;
}

extern "C" int vlm_mlp_create(const int* sizes, int nsizes, uint64_t seed, vlm_mlp** out) {
  if (!sizes || !out || nsizes < 2) return VLM_ERR_INVALID;
  return mlp_guard([&]() {
    vlm_mlp* h = new vlm_mlp();
    try {
      h->net.create(std::vector<int>(sizes, sizes + nsizes), seed, nullptr);
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
  });
}

extern "C" int vlm_mlp_destroy(vlm_mlp* h) {
  delete h;
  return VLM_OK;
}

extern "C" int64_t vlm_mlp_param_count(const vlm_mlp* h) { return h ? h->net.sh.nparam : -1; }

extern "C" int vlm_mlp_get_params(vlm_mlp* h, float* out) {
  if (!h || !out) return VLM_ERR_INVALID;
  return mlp_guard([&]() {
    MLP_CUDA(cudaMemcpy(out, h->net.p, sizeof(float) * h->net.sh.nparam, cudaMemcpyDeviceToHost));
  });
}

extern "C" int vlm_mlp_set_params(vlm_mlp* h, const float* in) {
  if (!h || !in) return VLM_ERR_INVALID;
  return mlp_guard([&]() {
    MLP_CUDA(cudaMemcpy(h->net.p, in, sizeof(float) * h->net.sh.nparam, cudaMemcpyHostToDevice));
    h->net.tcStale = true;
  });
}

extern "C" int vlm_mlp_set_inference(vlm_mlp* h, int mode) {
  if (!h || mode < 0 || mode > 1) return VLM_ERR_INVALID;
  if (!h->net.setTensorCores(mode == 1)) {
    g_err = "vlm_mlp_set_inference: the network does not fit the tensor-core kernel (a layer wider than 256)";
    return VLM_ERR_UNSUPPORTED;
  }
  return VLM_OK;
}

extern "C" int vlm_mlp_get_inference(const vlm_mlp* h) { return h ? (h->net.useTc ? 1 : 0) : -1; }

extern "C" int vlm_mlp_forward(vlm_mlp* h, const float* X, int64_t n, float* Y) {
  if (!h || n < 0 || (n > 0 && (!X || !Y)) || n > (1 << 28)) return VLM_ERR_INVALID;
  if (n == 0) return VLM_OK;
  return mlp_guard([&]() {
    const int in = h->net.sh.sz[0], out = h->net.sh.sz[h->net.sh.nl];
    grow_dev(&h->dX, h->capX, n * in);
    grow_dev(&h->dY, h->capY, n * out);
    h->net.reserve((int)std::min<int64_t>(n, 1 << 16));
    MLP_CUDA(cudaMemcpy(h->dX, X, sizeof(float) * n * in, cudaMemcpyHostToDevice));
    h->net.forward(h->dX, (int)n, h->dY);
    MLP_CUDA(cudaGetLastError());
    MLP_CUDA(cudaMemcpy(Y, h->dY, sizeof(float) * n * out, cudaMemcpyDeviceToHost));
    if (h->net.useTc) {
      int e = 0;
      MLP_CUDA(cudaMemcpy(&e, h->net.tcErr, sizeof(int), cudaMemcpyDeviceToHost));
      if (e) {
        MLP_CUDA(cudaMemset(h->net.tcErr, 0, sizeof(int)));
        throw std::runtime_error("tensor-core MLP: a bounded wait expired");
      }
    }
  });
}

extern "C" int vlm_mlp_gradient(vlm_mlp* h, const float* X, const float* T, int64_t n, float* grad, float* loss) {
  if (!h || !X || !T || !grad || n <= 0 || n > (1 << 22)) return VLM_ERR_INVALID;
  return mlp_guard([&]() {
    const int in = h->net.sh.sz[0], out = h->net.sh.sz[h->net.sh.nl];
    grow_dev(&h->dX, h->capX, n * in);
    grow_dev(&h->dT, h->capT, n * out);
    MLP_CUDA(cudaMemcpy(h->dX, X, sizeof(float) * n * in, cudaMemcpyHostToDevice));
    MLP_CUDA(cudaMemcpy(h->dT, T, sizeof(float) * n * out, cudaMemcpyHostToDevice));
    h->net.grad(h->dX, h->dT, (int)n);
    MLP_CUDA(cudaGetLastError());
    MLP_CUDA(cudaMemcpy(grad, h->net.g, sizeof(float) * h->net.sh.nparam, cudaMemcpyDeviceToHost));
    if (loss) MLP_CUDA(cudaMemcpy(loss, h->net.loss, sizeof(float), cudaMemcpyDeviceToHost));
  });
}

extern "C" int vlm_mlp_train(vlm_mlp* h, const float* X, const float* T, int64_t n, int batch, int iters, float lr,
                             float* final_loss) {
  if (!h || !X || !T || n <= 0 || batch <= 0 || iters < 0 || n > (1 << 26)) return VLM_ERR_INVALID;
  return mlp_guard([&]() {
    const int in = h->net.sh.sz[0], out = h->net.sh.sz[h->net.sh.nl];
    grow_dev(&h->dX, h->capX, n * in);
    grow_dev(&h->dT, h->capT, n * out);
    MLP_CUDA(cudaMemcpy(h->dX, X, sizeof(float) * n * in, cudaMemcpyHostToDevice));
    MLP_CUDA(cudaMemcpy(h->dT, T, sizeof(float) * n * out, cudaMemcpyHostToDevice));
    const int b = (int)std::min<int64_t>(batch, n);
    const int64_t nbatch = n / b;
    for (int it = 0; it < iters; ++it) {
      const int64_t k = it % std::max<int64_t>(nbatch, 1);  // consecutive batches of the (pre-shuffled) set
      h->net.grad(h->dX + (size_t)k * b * in, h->dT + (size_t)k * b * out, b);
      h->net.adam(lr);
    }
    MLP_CUDA(cudaGetLastError());
    if (final_loss) {
      MLP_CUDA(cudaStreamSynchronize(h->net.st));
      MLP_CUDA(cudaMemcpy(final_loss, h->net.loss, sizeof(float), cudaMemcpyDeviceToHost));
    }
  });
}
