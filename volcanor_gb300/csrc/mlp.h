// Multilayer perceptron engine of the learned far-wake surrogate: FP32
// parameters, tanh hidden layers, linear output, MSE loss, Adam; forward,
// backward and update are this library's own CUDA kernels (a tiled FP32 GEMM
// with fused bias / tanh epilogues, an elementwise tanh derivative, column
// sums and the Adam step).  Every reduction runs in a fixed order, so
// training is reproducible run to run.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

namespace vlm {

constexpr int kMlpMaxLayers = 8;

struct MlpShape {
  int nl = 0;                       // linear layers
  int sz[kMlpMaxLayers + 1] = {0};  // sz[0] inputs ... sz[nl] outputs
  // parameter offsets: W_l (sz[l+1] x sz[l], row major) then b_l (sz[l+1])
  int64_t woff[kMlpMaxLayers] = {0}, boff[kMlpMaxLayers] = {0};
  int64_t nparam = 0;
  int maxw = 0;  // widest layer
  void finalize();
};

struct Mlp {
  MlpShape sh;
  float* p = nullptr;      // parameters
  float* g = nullptr;      // gradient
  float* m = nullptr;      // Adam first moment
  float* v = nullptr;      // Adam second moment
  float* act = nullptr;    // activations of a batch: nl+1 blocks of [batch x maxw]
  float* dact = nullptr;   // two [batch x maxw] gradient buffers
  float* loss = nullptr;   // [2]: loss of the last batch, scratch
  float* part = nullptr;   // per-block loss partials
  int cap = 0;             // batch capacity of act / dact
  int64_t adamStep = 0;
  cudaStream_t st = nullptr;

  void create(const std::vector<int>& sizes, uint64_t seed, cudaStream_t stream);
  void destroy();
  void reserve(int batch);
  // Y[n x out] = f(X[n x in]) (device pointers); uses act for n <= cap rows at a time
  void forward(const float* X, int n, float* Y);
  // one gradient of MSE loss over the batch (X, T device pointers), into g; loss -> this->loss[0]
  void grad(const float* X, const float* T, int n);
  // Adam step with the gradient in g
  void adam(float lr, float b1 = 0.9f, float b2 = 0.999f, float eps = 1e-8f);
};

}  // namespace vlm
