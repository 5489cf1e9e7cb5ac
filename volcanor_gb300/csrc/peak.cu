// FP32 CUDA-core throughput probe: the denominator the N-body kernel's
// roofline fraction is quoted against, measured on the device at hand.
//
// Every thread runs kChains independent FMA chains (enough independent work
// to cover the FMA pipe's latency) for `iters` rounds; the grid is a whole
// number of waves over all SMs.  Nothing else is in the loop, so the issue
// rate is the FP32 FMA pipe's.  Work = 2 flop per FMA.
#include <cuda_runtime.h>

#include <string>

#include "../../include/vlm.h"
#include "vlm_bs.h"

namespace vlm {

extern thread_local std::string g_err;

namespace {

constexpr int kChains = 8;
constexpr int kPeakThreads = 256;

__global__ void __launch_bounds__(kPeakThreads) k_fma_chains(int iters, float seed, float* out) {
  float a[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) a[c] = seed + (float)(threadIdx.x + c);
  const float m = 1.0000001f, b = -1e-7f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 16; ++u)
#pragma unroll
      for (int c = 0; c < kChains; ++c) a[c] = fmaf(a[c], m, b);
  }
  float s = 0.f;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += a[c];
  // a store no compiler can drop (the host never reads a value of 0.5)
  if (s == 0.5f) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

}  // namespace vlm

using namespace vlm;

extern "C" int vlm_measure_fp32_peak(int device, int reps, double* tflops, double* ms_per_launch) {
  if (!tflops || !ms_per_launch || reps <= 0) {
    g_err = "vlm_measure_fp32_peak: null output or reps <= 0";
    return VLM_ERR_INVALID;
  }
  auto fail = [](cudaError_t e, const char* what) {
    g_err = std::string(what) + ": " + cudaGetErrorString(e);
    return VLM_ERR_CUDA;
  };
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return fail(e, "cudaSetDevice");
  int sms = 0, per = 0;
  e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) return fail(e, "cudaDeviceGetAttribute");
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_fma_chains, kPeakThreads, 0);
  if (e != cudaSuccess) return fail(e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
  const int blocks = sms * (per > 0 ? per : 1);
  const int iters = 4096;  // 4096 x 16 x 8 FMA per thread: ~2 ms per launch at full rate
  float* out = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = VLM_OK;
  do {
    if ((e = cudaMalloc(&out, sizeof(float) * (size_t)blocks * kPeakThreads)) != cudaSuccess) { rc = fail(e, "cudaMalloc"); break; }
    if ((e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking)) != cudaSuccess) { rc = fail(e, "cudaStreamCreate"); break; }
    if ((e = cudaEventCreate(&e0)) != cudaSuccess || (e = cudaEventCreate(&e1)) != cudaSuccess) { rc = fail(e, "cudaEventCreate"); break; }
    count_launch();
    k_fma_chains<<<blocks, kPeakThreads, 0, st>>>(iters, 1.0f, out);  // warm-up
    cudaEventRecord(e0, st);
    for (int r = 0; r < reps; ++r) {
      count_launch();
      k_fma_chains<<<blocks, kPeakThreads, 0, st>>>(iters, 1.0f + r, out);
    }
    cudaEventRecord(e1, st);
    if ((e = cudaEventSynchronize(e1)) != cudaSuccess) { rc = fail(e, "kernel"); break; }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    const double flop = 2.0 * (double)blocks * kPeakThreads * (double)iters * 16.0 * kChains;
    *ms_per_launch = ms / reps;
    *tflops = flop / (*ms_per_launch * 1e-3) / 1e12;
  } while (false);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st) cudaStreamDestroy(st);
  if (out) cudaFree(out);
  return rc;
}
