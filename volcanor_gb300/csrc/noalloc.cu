// vlm_biot_savart_rings_noalloc: the ring kernel without any device
// allocation, for callers that cannot allocate device memory.
//
// Some hosts of this path cannot call cudaMalloc at the moment they need a
// Biot-Savart sum: a solver that reserves all of its device memory once at
// start-up and must not grow afterwards, code running under a hard device
// memory cap, or a caller that cannot afford the implicit device-wide
// synchronisation an allocation or free may trigger.  This entry point takes
// all of its scratch from one fixed array compiled into the library, so it
// never allocates; the price is a fixed maximum problem size.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/vlm.h"
#include "vlm_bs.h"

namespace vlm {

extern thread_local std::string g_err;

namespace {

// Limits of the fixed scratch (see include/vlm.h).
constexpr int64_t kMaxRings = 16384;
constexpr int64_t kMaxPoints = 65536;
constexpr int64_t kMaxNear = 65536;
// Chunks of the FP32 sums (whose summation order is free): enough to fill the
// device when M is small; M x chunks partials must fit the part buffer.
constexpr int kMaxChunks = 256;

constexpr size_t align256(size_t b) { return (b + 255) & ~size_t(255); }
constexpr size_t kOffRec64 = 0;
constexpr size_t kOffRec32 = kOffRec64 + align256(kMaxRings * kRec64 * sizeof(double));
constexpr size_t kOffPart = kOffRec32 + align256(kMaxRings * kRec32 * sizeof(float));
constexpr size_t kOffNear = kOffPart + align256(kMaxPoints * 3 * sizeof(double));
constexpr size_t kNearBytes = near_scratch_bytes((int)kMaxPoints, (size_t)kMaxNear);  // near-field grid + pair list
constexpr size_t kOffNacc = kOffNear + align256(kNearBytes);
constexpr size_t kOffTables = kOffNacc + align256(kMaxPoints * 3 * sizeof(long long));
constexpr size_t kOffGroup = kOffTables + align256(kMaxChunks * sizeof(Chunk));
constexpr size_t kOffCtl = kOffGroup + align256(sizeof(Group));
constexpr size_t kScratchBytes = kOffCtl + 256;  // chunk table, group, control words

// One fixed scratch area per device that loads the library, held until exit.
// Every FP32 + FP64-near call clears the near-field accumulators it uses
// before its launch, so a call that failed half-way leaves nothing behind.
// In host code this name is only a stand-in for the device object: kernels
// get its device address from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_mu;
unsigned char* g_base[64] = {nullptr};

// The per-call chunk table, passed by value (2 KiB of kernel parameters).
struct ChunkList {
  int n;
  Chunk c[kMaxChunks];
};

// Writes the per-call tables into the scratch: the chunk table, one
// wing-kind group over all N rings, zeroed control words (error flag and
// near-pair count).
__global__ void k_noalloc_tables(unsigned char* base, ChunkList cl, int N) {
  Chunk* ch = reinterpret_cast<Chunk*>(base + kOffTables);
  for (int q = threadIdx.x; q < cl.n; q += blockDim.x) ch[q] = cl.c[q];
  if (threadIdx.x != 0) return;
  Group* g = reinterpret_cast<Group*>(base + kOffGroup);
  int* ctl = reinterpret_cast<int*>(base + kOffCtl);
  g->rec_begin = 0;
  g->rec_count = N;
  g->chunk_begin = 0;
  g->chunk_count = cl.n;
  g->kind = 0;
  g->blade = 0;
  g->pad[0] = g->pad[1] = 0;
  for (int k = 0; k < 4; ++k) ctl[k] = 0;
}

__global__ void k_zero(double* v, int64_t n) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) v[i] = 0.0;
}

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

}  // namespace

}  // namespace vlm

using namespace vlm;

extern "C" int vlm_biot_savart_rings_noalloc(const double* corners, const double* rvc, const double* gam, int64_t N,
                                             const double* P, int64_t M, double* V, int precision, void* stream) {
  if (precision < VLM_PREC_FP64 || precision > VLM_PREC_FP32_NEAR64) return fail(VLM_ERR_INVALID, "precision must be 0, 1 or 2");
  if (N < 0 || M < 0) return fail(VLM_ERR_INVALID, "N and M must not be negative");
  if (N > kMaxRings)
    return fail(VLM_ERR_INVALID, "vlm_biot_savart_rings_noalloc: N = " + std::to_string(N) + " rings exceeds the fixed scratch limit of " +
                                     std::to_string(kMaxRings));
  if (M > kMaxPoints)
    return fail(VLM_ERR_INVALID, "vlm_biot_savart_rings_noalloc: M = " + std::to_string(M) + " points exceeds the fixed scratch limit of " +
                                     std::to_string(kMaxPoints));
  if (M == 0) return VLM_OK;
  if ((N > 0 && (!corners || !rvc || !gam)) || !P || !V) return fail(VLM_ERR_INVALID, "null device pointer");
  cudaStream_t st = (cudaStream_t)stream;
  // the call waits for its stream (below), which a capturing stream cannot do
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  cudaError_t e = cudaStreamIsCapturing(st, &cap);
  if (e != cudaSuccess || cap != cudaStreamCaptureStatusNone)
    return fail(VLM_ERR_INVALID, "vlm_biot_savart_rings_noalloc cannot be called on a capturing stream");
  int dev = 0;
  e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(VLM_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= 64) return fail(VLM_ERR_CUDA, "device ordinal out of range");
  unsigned char* base = nullptr;
  {
    // set-up, once per device, with that device current: the device address
    // of the scratch array (the host-side symbol is not a device address)
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_base[dev]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p) return fail(VLM_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      g_base[dev] = static_cast<unsigned char*>(p);
    }
    base = g_base[dev];
  }
  double* rec64 = reinterpret_cast<double*>(base + kOffRec64);
  float* rec32 = reinterpret_cast<float*>(base + kOffRec32);
  double* part = reinterpret_cast<double*>(base + kOffPart);
  unsigned char* near = base + kOffNear;
  long long* nacc = reinterpret_cast<long long*>(base + kOffNacc);
  Chunk* chunks = reinterpret_cast<Chunk*>(base + kOffTables);
  Group* group = reinterpret_cast<Group*>(base + kOffGroup);
  int* ctl = reinterpret_cast<int*>(base + kOffCtl);

  // FP64: one chunk over all rings, the reference's summation order.  FP32:
  // the chunks that fill the device (plan_chunks32), at most kMaxPoints / M
  // so that the M x chunks partials and near-field accumulators fit.
  ChunkList cl{};
  cl.n = N > 0 ? 1 : 0;
  cl.c[0] = Chunk{0, (int32_t)N};
  if (N > 0 && precision != VLM_PREC_FP64) {
    Group hg{0, (int32_t)N, 0, 0, 0, 0, {0, 0}};
    const int capq = (int)std::min<int64_t>(kMaxChunks, kMaxPoints / M);
    const int nq = plan_chunks32(&hg, 1, (int)M, partial32_slots(), cl.c, capq);
    if (nq >= 1) {
      cl.n = nq;
    } else {
      cl.n = 1;
      cl.c[0] = Chunk{0, (int32_t)N};
    }
  }
  count_launch();
  k_noalloc_tables<<<1, 256, 0, st>>>(base, cl, (int)N);
  if (N > 0) {
    launch_rings_to_rec64(corners, rvc, gam, N, rec64, st);
    if (precision == VLM_PREC_FP64) {
      launch_partial64(rec64, chunks, 1, P, (int)M, part, st);
      launch_combine(part, (int)M, group, 1, 2, V, st);
    } else {
      const bool nearOn = precision == VLM_PREC_FP32_NEAR64;
      if (nearOn) {
        e = cudaMemsetAsync(nacc, 0, (size_t)M * cl.n * 3 * sizeof(long long), st);
        if (e != cudaSuccess) return fail(VLM_ERR_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
      }
      launch_pack32(rec64, (int)N, nearOn ? 4.0 : 0.0, rec32, st);
      launch_partial32(rec32, rec64, chunks, cl.n, (int)N, P, (int)M, part, ctl, nearOn ? near : nullptr, kNearBytes,
                       nacc, st);
      launch_combine_unordered(part, (int)M, group, 1, cl.n, 2, V, st);
    }
  } else {
    count_launch();
    k_zero<<<(unsigned)((3 * M + 255) / 256), 256, 0, st>>>(V, 3 * M);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail(VLM_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
  // the scratch is shared by every call on this device: finish this one
  // before returning, and read its error flag
  int flags[2] = {0, 0};
  e = cudaMemcpyAsync(flags, ctl, sizeof(flags), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return fail(VLM_ERR_CUDA, std::string("cudaStreamSynchronize: ") + cudaGetErrorString(e));
  if (flags[0] == 3) return fail(VLM_ERR_INVALID, "vlm_biot_savart_rings_noalloc: the near-field pair list overflowed (more than 65536 pairs)");
  if (flags[0] == 4) return fail(VLM_ERR_NONFINITE, "vlm_biot_savart_rings_noalloc: near-field velocity outside the fixed-point range");
  if (flags[0]) return fail(VLM_ERR_CUDA, "device wait limit expired in a Biot-Savart tile pipeline");
  return VLM_OK;
}
