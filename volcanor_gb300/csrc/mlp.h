// Multilayer perceptron engine of the learned far-wake surrogate: FP32
// parameters, tanh hidden layers, linear output, MSE loss, Adam; forward,
// backward and update are this library's own CUDA kernels (a tiled FP32 GEMM
// with fused bias / tanh epilogues, an elementwise tanh derivative, column
// sums and the Adam step; for inference also a fused tcgen05 kernel with
// BF16 operands, mlp_tc.cu).  Every reduction runs in a fixed order, so
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

// The network packed for the tensor-core forward pass (mlp_tc.cu): per
// layer N x K BF16 weights (N, K padded to multiples of 16) in the MMA's
// canonical K-major layout, then every layer's FP32 biases, in one image
// that the kernel copies to shared memory.
struct TcLayer {
  int N = 0, K = 0;
  uint32_t woff = 0, boff = 0;  // byte offsets of the weights and biases in the image
};
struct TcNet {
  int nl = 0, in = 0, out = 0, Kmax = 0;
  uint32_t imgBytes = 0, tmemCols = 0, smemBytes = 0;
  TcLayer L[kMlpMaxLayers];
  // Lays the image out for sh; false if the network does not fit the kernel
  // (a layer wider than 256 or more than 200 KiB of shared memory).
  bool plan(const MlpShape& sh);
};
// BF16 image of the parameters p (FP32, MlpShape layout) on stream st.
void tc_pack(const float* p, const MlpShape& sh, const TcNet& net, uint8_t* img, cudaStream_t st);
// Y[n x out] = f(X[n x in]) with the packed image; err receives 1 if a
// bounded wait of the kernel expired.
void tc_forward(const TcNet& net, const uint8_t* img, const float* X, int n, float* Y, int* err, cudaStream_t st);

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
  // tensor-core inference: the packed image, rebuilt before the first
  // forward pass after the parameters change
  TcNet tc;
  bool tcFits = false;     // the shape fits the tensor-core kernel
  bool useTc = false;      // forward() runs on the tensor cores
  bool tcStale = true;     // parameters changed since the last pack
  uint8_t* tcImg = nullptr;
  int* tcErr = nullptr;    // device word the kernel flags an expired wait in

  void create(const std::vector<int>& sizes, uint64_t seed, cudaStream_t stream);
  void destroy();
  void reserve(int batch);
  // Y[n x out] = f(X[n x in]) (device pointers): on the tensor cores when
  // useTc (BF16 operands, FP32 accumulation), else the FP32 GEMMs, which use
  // act for n <= cap rows at a time
  void forward(const float* X, int n, float* Y);
  // selects the tensor-core (true) or FP32 CUDA-core forward pass; false
  // if the tensor-core kernel cannot hold this network
  bool setTensorCores(bool on);
  // one gradient of MSE loss over the batch (X, T device pointers), into g; loss -> this->loss[0]
  void grad(const float* X, const float* T, int n);
  // Adam step with the gradient in g
  void adam(float lr, float b1 = 0.9f, float b2 = 0.999f, float eps = 1e-8f);
};

}  // namespace vlm
