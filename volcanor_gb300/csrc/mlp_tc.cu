// Tensor-core inference of the surrogate MLP on sm_103a: tcgen05.mma with
// BF16 operands in shared memory and FP32 accumulators in tensor memory
// (TMEM), all layers of the network fused in one kernel.
//
// One CTA of 128 threads owns a tile of 128 targets (the MMA's M = 128 =
// TMEM lanes; thread t holds row t).  The whole network's weights, packed
// once per parameter update into BF16 images in the MMA's canonical
// K-major layout (k_tc_pack), arrive in shared memory by one bulk copy and
// stay there while the CTA walks its tiles.  Per layer: one elected thread
// issues K/16 MMAs (D[128 x N] += A[128 x 16] B[16 x N]) and commits them to
// an mbarrier; after the wait every thread reads its row of D from TMEM
// (tcgen05.ld), adds the bias, applies tanh, rounds to BF16 and writes the
// row back into the A buffer as the next layer's input; the output layer
// writes Y.  Activations never leave the SM.
//
// Canonical K-major layout without swizzle (both operands): 8 x 8 BF16 core
// matrices of 128 contiguous bytes (8 rows of 16 bytes).  An operand of R
// rows and K columns is stored as K/16 slices of 16 columns; inside a slice
// the two core matrices of an 8-row group are adjacent (leading byte offset
// 128) and the 8-row groups follow each other (stride byte offset 256).
//
// Every wait is bounded: on expiry the CTA records an error, stops issuing
// work, waits (bounded) for its last commit and frees its TMEM.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <stdexcept>
#include <string>

#include "mlp.h"
#include "vlm_bs.h"

namespace vlm {

namespace {

constexpr int kTcRows = 128;
constexpr int kTcThreads = 128;
constexpr uint32_t kTcWaitLimit = 1u << 20;  // polls; with the back-off below, well under a second
constexpr uint32_t kSliceBytesA = kTcRows * 16 * 2;  // one 16-column slice of the A buffer

__device__ __forceinline__ uint32_t su32(const void* p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

// Bounded wait for the phase with the given parity (non-blocking polls,
// backing off after the first few); false if the limit expired.
__device__ __forceinline__ bool tc_wait(uint64_t* bar, uint32_t parity) {
  const uint32_t a = su32(bar);
  for (uint32_t i = 0; i < kTcWaitLimit; ++i) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    if (ok) return true;
    if (i >= 64) __nanosleep(128);
  }
  return false;
}

// Shared-memory matrix descriptor: start address, leading and stride byte
// offsets (all in 16-byte units), descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t tc_sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, M = 128, N = n.
__host__ __device__ constexpr uint32_t tc_idesc(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(kTcRows >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void tc_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(bar))
               : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 16 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
      "tcgen05.wait::ld.sync.aligned;\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);  // .x = a (low half), .y = b
  return *reinterpret_cast<const uint32_t*>(&h);
}

// Writes 16 values as the columns c0..c0+15 of row `row` of an operand in
// the canonical layout (slice c0/16: two core matrices, 16 bytes each).
__device__ __forceinline__ void put_row16(uint8_t* base, uint32_t slice_bytes, int row, int c0, const float (&v)[16]) {
  uint8_t* s = base + (size_t)(c0 >> 4) * slice_bytes + (row >> 3) * 256 + (row & 7) * 16;
  uint4 lo, hi;
  lo.x = pack_bf16(v[0], v[1]);
  lo.y = pack_bf16(v[2], v[3]);
  lo.z = pack_bf16(v[4], v[5]);
  lo.w = pack_bf16(v[6], v[7]);
  hi.x = pack_bf16(v[8], v[9]);
  hi.y = pack_bf16(v[10], v[11]);
  hi.z = pack_bf16(v[12], v[13]);
  hi.w = pack_bf16(v[14], v[15]);
  *reinterpret_cast<uint4*>(s) = lo;
  *reinterpret_cast<uint4*>(s + 128) = hi;
}

// FP32 parameters (W_l row major [out][in], then b_l) -> the BF16 weight
// images (zero padding) and FP32 biases of the packed network.
__global__ void k_tc_pack(const float* __restrict__ p, TcNet net, int64_t woff, int64_t boff, int l, int in, int out,
                          uint8_t* __restrict__ img) {
  const TcLayer& L = net.L[l];
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t nw = (int64_t)L.N * L.K;
  if (i < nw) {
    const int n = (int)(i / L.K), k = (int)(i % L.K);
    const float w = (n < out && k < in) ? p[woff + (int64_t)n * in + k] : 0.f;
    const int kk = k & 15;
    const size_t off = L.woff + (size_t)(k >> 4) * (L.N * 32) + (n >> 3) * 256 + (kk >> 3) * 128 + (n & 7) * 16 +
                       (kk & 7) * 2;
    *reinterpret_cast<__nv_bfloat16*>(img + off) = __float2bfloat16_rn(w);
  } else if (i < nw + L.N) {
    const int n = (int)(i - nw);
    reinterpret_cast<float*>(img + L.boff)[n] = n < out ? p[boff + n] : 0.f;
  }
}

__global__ void __launch_bounds__(kTcThreads, 1)
    k_mlp_tc(TcNet net, const uint8_t* __restrict__ img, const float* __restrict__ X, int n, float* __restrict__ Y,
             int* __restrict__ err) {
  extern __shared__ __align__(128) uint8_t sm[];
  uint8_t* sW = sm;
  uint8_t* sA = sm + net.imgBytes;
  uint64_t* bar = reinterpret_cast<uint64_t*>(sA + (size_t)(net.Kmax >> 4) * kSliceBytesA);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 2);
  const int tid = threadIdx.x, warp = tid >> 5;
  const int tiles = (n + kTcRows - 1) / kTcRows;

  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&bar[0])) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(&bar[1])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(tslot)),
                 "r"(net.tmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  // the packed network: one bulk copy (imgBytes is a multiple of 16)
  if (tid == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(&bar[0])), "r"(net.imgBytes)
                 : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(su32(sW)),
        "l"(img), "r"(net.imgBytes), "r"(su32(&bar[0]))
        : "memory");
  }
  bool ok = __syncthreads_and(tc_wait(&bar[0], 0)) != 0;
  uint32_t phase = 0;
  bool committed = false;  // a commit whose completion has not been waited for
  const uint32_t lane_base = (uint32_t)(32 * warp) << 16;

  for (int tile = blockIdx.x; ok && tile < tiles; tile += gridDim.x) {
    const int row = tile * kTcRows + tid;
    // layer 0 input: this thread's row of X, zero padded to K0 columns
    for (int c0 = 0; c0 < net.L[0].K; c0 += 16) {
      float v[16];
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const int c = c0 + j;
        v[j] = (row < n && c < net.in) ? X[(size_t)row * net.in + c] : 0.f;
      }
      put_row16(sA, kSliceBytesA, tid, c0, v);
    }
    for (int l = 0; ok && l < net.nl; ++l) {
      const TcLayer& L = net.L[l];
      // the A rows written by every thread become visible to the tensor core
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      tc_fence_before();
      __syncthreads();
      if (tid == 0) {
        tc_fence_after();
        const uint32_t a0 = su32(sA), b0 = su32(sW + L.woff);
        const uint32_t idesc = tc_idesc(L.N);
        for (int s = 0; s < (L.K >> 4); ++s)
          tc_mma(tmem, tc_sdesc(a0 + s * kSliceBytesA, 128, 256), tc_sdesc(b0 + s * (uint32_t)(L.N * 32), 128, 256),
                 idesc, s > 0 ? 1u : 0u);
        tc_commit(&bar[1]);
      }
      committed = true;
      ok = __syncthreads_and(tc_wait(&bar[1], phase)) != 0;
      if (!ok) break;
      committed = false;
      phase ^= 1u;
      tc_fence_after();
      const float* bias = reinterpret_cast<const float*>(sW + L.boff);
      const bool last = l == net.nl - 1;
      for (int c0 = 0; c0 < L.N; c0 += 16) {
        float v[16];
        tc_ld16(tmem + lane_base + (uint32_t)c0, v);
#pragma unroll
        for (int j = 0; j < 16; ++j) v[j] += bias[c0 + j];
        if (last) {
          if (row < n)
            for (int j = 0; j < 16; ++j)
              if (c0 + j < net.out) Y[(size_t)row * net.out + c0 + j] = v[j];
        } else {
#pragma unroll
          for (int j = 0; j < 16; ++j) v[j] = tanhf(v[j]);
          put_row16(sA, kSliceBytesA, tid, c0, v);
        }
      }
    }
  }
  if (!ok) {
    if (tid == 0) atomicExch(err, 1);
    // an MMA group may still be running: give it the bounded wait once more
    if (committed) tc_wait(&bar[1], phase);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(net.tmemCols) : "memory");
  }
}

}  // namespace

bool TcNet::plan(const MlpShape& sh) {
  *this = TcNet{};
  nl = sh.nl;
  in = sh.sz[0];
  out = sh.sz[sh.nl];
  uint32_t off = 0;
  int maxN = 0;
  Kmax = 0;
  for (int l = 0; l < sh.nl; ++l) {
    TcLayer& L = this->L[l];
    L.K = (sh.sz[l] + 15) / 16 * 16;
    L.N = std::max(16, (sh.sz[l + 1] + 15) / 16 * 16);
    if (L.N > 256 || L.K > 256) return false;
    L.woff = off;
    off += (uint32_t)L.N * L.K * 2;
    maxN = std::max(maxN, L.N);
    Kmax = std::max(Kmax, L.K);
  }
  // the next layer reads A with the previous layer's N columns
  for (int l = 1; l < sh.nl; ++l) Kmax = std::max(Kmax, this->L[l - 1].N);
  for (int l = 0; l < sh.nl; ++l) {
    this->L[l].boff = off;
    off += (uint32_t)this->L[l].N * 4;
  }
  imgBytes = (off + 15) / 16 * 16;
  tmemCols = 32;
  while ((int)tmemCols < maxN) tmemCols *= 2;
  smemBytes = imgBytes + (uint32_t)(Kmax / 16) * kSliceBytesA + 64;
  return smemBytes <= 200 * 1024;
}

void tc_pack(const float* p, const MlpShape& sh, const TcNet& net, uint8_t* img, cudaStream_t st) {
  for (int l = 0; l < net.nl; ++l) {
    const int64_t cnt = (int64_t)net.L[l].N * net.L[l].K + net.L[l].N;
    count_launch();
    k_tc_pack<<<(unsigned)((cnt + 255) / 256), 256, 0, st>>>(p, net, sh.woff[l], sh.boff[l], l, sh.sz[l],
                                                            sh.sz[l + 1], img);
  }
}

void tc_forward(const TcNet& net, const uint8_t* img, const float* X, int n, float* Y, int* err, cudaStream_t st) {
  if (n <= 0) return;
  static bool attr = false;  // the kernel's shared-memory limit, raised once per process
  if (!attr) {
    if (cudaFuncSetAttribute(k_mlp_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) != cudaSuccess)
      throw std::runtime_error("cudaFuncSetAttribute(k_mlp_tc)");
    attr = true;
  }
  const int tiles = (n + kTcRows - 1) / kTcRows;
  const int grid = std::min(tiles, 2 * device_sm_count());
  count_launch();
  k_mlp_tc<<<grid, kTcThreads, net.smemBytes, st>>>(net, img, X, n, Y, err);
}

}  // namespace vlm
