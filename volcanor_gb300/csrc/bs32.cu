// FP32 Biot-Savart N-body kernel with FP64 accumulation and an FP64
// near-field path, for sm_103a.  Compiled with -ftz=true.
//
// Layout: one block = 8 consumer warps (256 threads x 2 targets per thread)
// plus one producer warp, one chunk of source records.  Source records
// (48 floats, 192 B) stream through a 4-stage shared-memory ring filled by
// bulk asynchronous copies (cp.async.bulk) from the producer; FULL/EMPTY
// mbarriers hand stages between producer and consumers (every wait bounded),
// so consumer warps never wait for one another.  Each staged record is read
// with broadcast LDS.128 and evaluated for both targets of a thread.
//
// Per target and record: corner vectors r_k = P - c_k with rsqrt norms (c3's
// only when edge 2 or 3 carries circulation: a lattice-form interior ring has
// just edges 0 and 1), then per filament k -> j = k+1 the Vatistas n=2
// kernel (src/classdef.f90:476-503)
//   v = (r_k x r_j) w_k (e.r_k/|r_k| - e.r_j/|r_j|) / sqrt((rvc|e|)^4 + |r_k x r_j|^4)
// with e.r_j = e.r_k - |e|^2 and the source-only terms hoisted into the
// record, the weight w_k = gam/4pi folded into e.  A target on the filament
// line has r_k x r_j = 0 exactly, so its (finite) factor contributes exactly
// zero; the reference's eps^2 cut-off needs no separate test.  FP32 partial sums are promoted to
// the FP64 accumulator after every tile.
//
// Near field (VLM_PREC_FP32_NEAR64): the FP32 kernel sums every pair; the
// pairs within near_factor core radii of a filament segment -- where the
// FP32 cross product and Vatistas denominator lose digits -- are then
// corrected to FP64 outside the hot loop.  The targets are binned into a
// hashed uniform grid (cell size three times the mean near-zone radius); every
// near-zone filament, cut into pieces no longer than a cell, visits the
// cells around each piece and tests their targets, listing the near pairs
// (k_near_find).  For every listed pair k_near_fix recomputes the FP32
// kernel's own contribution bit for bit (same
// inline arithmetic, same FP32 inputs) and adds FP64 value - FP32
// contribution to order-independent fixed-point accumulators, which
// k_near_apply folds into the chunk partial sums.  The result equals summing
// the far pairs in FP32 and the near pairs in FP64, up to the FP32 rounding
// of the tile sums that held the near terms.
#include <stdint.h>

#include <algorithm>
#include <climits>
#include <atomic>

#include "vlm_bs.h"
#include "vlm_math.h"

namespace vlm {

namespace {

constexpr uint32_t kWaitLimit = 1u << 22;
constexpr float kS2Min = 1e-30f;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
// Bounded wait for the phase with the given parity; false if the limit expired.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t limit = kWaitLimit) {
  const uint32_t a = smem_u32(bar);
  for (uint32_t i = 0; i < limit; ++i) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

constexpr unsigned kFull = 0xffffffffu;

// Corner vector r = P - c and 1/|r| (|r|^2 + 1e-30: a target on a corner
// gets a finite 1/|r|, times r = 0).
__device__ __forceinline__ void corner_vector(float px, float py, float pz, float cx, float cy, float cz, float& rx,
                                              float& ry, float& rz, float& inv) {
  rx = px - cx;
  ry = py - cy;
  rz = pz - cz;
  inv = rsqrtf(fmaf(rx, rx, fmaf(ry, ry, fmaf(rz, rz, kS2Min))));
}

// The staged fields of one record that the filament evaluations read.
struct RecView {
  float ex[4], ey[4], ez[4], eev[4], a4v[4];
};
__device__ __forceinline__ void load_view(const float4* __restrict__ R4, RecView& v) {
  const float4 q3 = R4[3], q4 = R4[4], q5 = R4[5];  // weighted edges
  const float4 ee = R4[6], a4 = R4[7];
  v.ex[0] = q3.x, v.ex[1] = q3.w, v.ex[2] = q4.z, v.ex[3] = q5.y;
  v.ey[0] = q3.y, v.ey[1] = q4.x, v.ey[2] = q4.w, v.ey[3] = q5.z;
  v.ez[0] = q3.z, v.ez[1] = q4.y, v.ez[2] = q5.x, v.ez[3] = q5.w;
  v.eev[0] = ee.x, v.eev[1] = ee.y, v.eev[2] = ee.z, v.eev[3] = ee.w;
  v.a4v[0] = a4.x, v.a4v[1] = a4.y, v.a4v[2] = a4.z, v.a4v[3] = a4.w;
}

// FP32 velocity of filament K (c_K -> c_{K+1}) at one target, from the
// corner vectors (r, 1/|r|) of its two ends: the factor f and the cross
// product r_K x r_{K+1}; the contribution is f (kx, ky, kz).  The near-field
// correction recomputes exactly this (k_near_fix), so keep every operation
// explicit (no expression the compiler could contract differently).
struct Fil32 {
  float f, kx, ky, kz, c2, tt;
};
__device__ __forceinline__ Fil32 fil_terms(float ex, float ey, float ez, float eev, float a4, float rxk, float ryk,
                                           float rzk, float invk, float rxj, float ryj, float rzj, float invj) {
  Fil32 o;
  o.kx = fmaf(ryk, rzj, -rzk * ryj);
  o.ky = fmaf(rzk, rxj, -rxk * rzj);
  o.kz = fmaf(rxk, ryj, -ryk * rxj);
  o.c2 = fmaf(o.kx, o.kx, fmaf(o.ky, o.ky, o.kz * o.kz));
  // w (e.r_k/|r_k| - e.r_j/|r_j|) with the weight folded into e
  o.tt = fmaf(ex, rxk, fmaf(ey, ryk, ez * rzk));
  const float d = fmaf(o.tt, invk, -(o.tt - eev) * invj);
  o.f = d * rsqrtf(fmaf(o.c2, o.c2, a4));
  return o;
}

// Adds the FP32 velocity of filament K at one target.
template <int K>
__device__ __forceinline__ void fil_fp32(const RecView& v, float rxk, float ryk, float rzk, float invk, float rxj,
                                         float ryj, float rzj, float invj, float& ax, float& ay, float& az) {
  const Fil32 t = fil_terms(v.ex[K], v.ey[K], v.ez[K], v.eev[K], v.a4v[K], rxk, ryk, rzk, invk, rxj, ryj, rzj, invj);
  ax = fmaf(t.f, t.kx, ax);
  ay = fmaf(t.f, t.ky, ay);
  az = fmaf(t.f, t.kz, az);
}

// A whole ring (all four edges active): the four corner vectors r_k = P - c_k
// and 1/|r_k| (|r|^2 + 1e-30 as in corner_vector).
__device__ __forceinline__ void corner_vectors(float px, float py, float pz, const float (&cx)[4], const float (&cy)[4],
                                               const float (&cz)[4], float (&rx)[4], float (&ry)[4], float (&rz)[4],
                                               float (&inv)[4]) {
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    rx[k] = px - cx[k];
    ry[k] = py - cy[k];
    rz[k] = pz - cz[k];
    inv[k] = rsqrtf(fmaf(rx[k], rx[k], fmaf(ry[k], ry[k], fmaf(rz[k], rz[k], kS2Min))));
  }
}

// Adds the FP32 velocity of a whole ring at one target (corner vectors r_k
// and rsqrt norms given).
__device__ __forceinline__ void ring_fp32(const float4* __restrict__ R4, const float (&rx)[4], const float (&ry)[4],
                                          const float (&rz)[4], const float (&inv)[4], float& ax, float& ay,
                                          float& az) {
  RecView v;
  load_view(R4, v);
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int j = (k + 1) & 3;
    const Fil32 t = fil_terms(v.ex[k], v.ey[k], v.ez[k], v.eev[k], v.a4v[k], rx[k], ry[k], rz[k], inv[k], rx[j], ry[j],
                              rz[j], inv[j]);
    ax = fmaf(t.f, t.kx, ax);
    ay = fmaf(t.f, t.ky, ay);
    az = fmaf(t.f, t.kz, az);
  }
}

// Both targets of a thread, one lattice-form record, no near test: both
// targets' c0..c2 vectors first (more independent work in flight), edges 0
// and 1, then c3 and the border edges 2 / 3 where they carry circulation
// (uniform branches: every lane evaluates the same record).
template <int T>
__device__ __forceinline__ void rec_lat_pair(const float4* __restrict__ R4, const float (&cx)[4], const float (&cy)[4],
                                             const float (&cz)[4], const float (&px)[T], const float (&py)[T],
                                             const float (&pz)[T], float (&ax)[T], float (&ay)[T], float (&az)[T]) {
  RecView v;
  load_view(R4, v);
  float rx[T][4], ry[T][4], rz[T][4], inv[T][4];
#pragma unroll
  for (int u = 0; u < T; ++u)
#pragma unroll
    for (int k = 0; k < 3; ++k)
      corner_vector(px[u], py[u], pz[u], cx[k], cy[k], cz[k], rx[u][k], ry[u][k], rz[u][k], inv[u][k]);
#pragma unroll
  for (int u = 0; u < T; ++u) {
    fil_fp32<0>(v, rx[u][0], ry[u][0], rz[u][0], inv[u][0], rx[u][1], ry[u][1], rz[u][1], inv[u][1], ax[u], ay[u],
                az[u]);
    fil_fp32<1>(v, rx[u][1], ry[u][1], rz[u][1], inv[u][1], rx[u][2], ry[u][2], rz[u][2], inv[u][2], ax[u], ay[u],
                az[u]);
  }
  const bool t2 = v.a4v[2] >= 0.f, t3 = v.a4v[3] >= 0.f;
  if (t2 || t3) {
#pragma unroll
    for (int u = 0; u < T; ++u)
      corner_vector(px[u], py[u], pz[u], cx[3], cy[3], cz[3], rx[u][3], ry[u][3], rz[u][3], inv[u][3]);
    if (t2) {
#pragma unroll
      for (int u = 0; u < T; ++u)
        fil_fp32<2>(v, rx[u][2], ry[u][2], rz[u][2], inv[u][2], rx[u][3], ry[u][3], rz[u][3], inv[u][3], ax[u],
                    ay[u], az[u]);
    }
    if (t3) {
#pragma unroll
      for (int u = 0; u < T; ++u)
        fil_fp32<3>(v, rx[u][3], ry[u][3], rz[u][3], inv[u][3], rx[u][0], ry[u][0], rz[u][0], inv[u][0], ax[u],
                    ay[u], az[u]);
    }
  }
}

// ---- packed pairs of FP32 values (the sm_100 family's f32x2 instructions) --
// A thread with two targets evaluates every record for both at once: each
// add / mul / fma below is one instruction for the two lanes, each lane
// rounded exactly as the scalar instruction (.rn, .ftz as the unit's
// -ftz=true).  The scalar functions above are rewritten only where a
// negation would need its own instruction: -(a b) as (-a) b with the exactly
// negated corner vector c - P, -(t - e) as e - t; both exact, so every lane
// carries the scalar path's bits (k_near_fix recomputes those).
typedef unsigned long long f2;
__device__ __forceinline__ f2 f2pack(float a, float b) {
  f2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ f2 f2splat(float a) { return f2pack(a, a); }
__device__ __forceinline__ void f2unpack(f2 r, float& a, float& b) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r));
}
__device__ __forceinline__ f2 f2sub(f2 a, f2 b) {
  f2 d;
  asm("sub.rn.ftz.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f2 f2mul(f2 a, f2 b) {
  f2 d;
  asm("mul.rn.ftz.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f2 f2fma(f2 a, f2 b, f2 c) {
  f2 d;
  asm("fma.rn.ftz.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
__device__ __forceinline__ f2 f2rsqrt(f2 a) {
  float x, y;
  f2unpack(a, x, y);
  return f2pack(rsqrtf(x), rsqrtf(y));
}

// corner_vector for both targets: r = P - c, 1/|r|
__device__ __forceinline__ void corner_pair(f2 px, f2 py, f2 pz, float cx, float cy, float cz, f2& rx, f2& ry, f2& rz,
                                            f2& inv) {
  rx = f2sub(px, f2splat(cx));
  ry = f2sub(py, f2splat(cy));
  rz = f2sub(pz, f2splat(cz));
  inv = f2rsqrt(f2fma(rx, rx, f2fma(ry, ry, f2fma(rz, rz, f2splat(kS2Min)))));
}

// fil_fp32 for both targets; (cxk, cyk, czk) is corner K itself, whose
// negated corner vector c - P the cross product takes
template <int K>
__device__ __forceinline__ void fil_pair(const RecView& v, f2 px, f2 py, f2 pz, float cxk, float cyk, float czk,
                                         f2 rxk, f2 ryk, f2 rzk, f2 invk, f2 rxj, f2 ryj, f2 rzj, f2 invj, f2& ax,
                                         f2& ay, f2& az) {
  const f2 nrxk = f2sub(f2splat(cxk), px), nryk = f2sub(f2splat(cyk), py), nrzk = f2sub(f2splat(czk), pz);
  const f2 kx = f2fma(ryk, rzj, f2mul(nrzk, ryj));
  const f2 ky = f2fma(rzk, rxj, f2mul(nrxk, rzj));
  const f2 kz = f2fma(rxk, ryj, f2mul(nryk, rxj));
  const f2 c2 = f2fma(kx, kx, f2fma(ky, ky, f2mul(kz, kz)));
  const f2 tt = f2fma(f2splat(v.ex[K]), rxk, f2fma(f2splat(v.ey[K]), ryk, f2mul(f2splat(v.ez[K]), rzk)));
  const f2 d = f2fma(tt, invk, f2mul(f2sub(f2splat(v.eev[K]), tt), invj));
  const f2 f = f2mul(d, f2rsqrt(f2fma(c2, c2, f2splat(v.a4v[K]))));
  ax = f2fma(f, kx, ax);
  ay = f2fma(f, ky, ay);
  az = f2fma(f, kz, az);
}

// ring_fp32 for both targets (all four edges)
__device__ __forceinline__ void ring_pair(const float4* __restrict__ R4, const float (&cx)[4], const float (&cy)[4],
                                          const float (&cz)[4], f2 px, f2 py, f2 pz, f2& ax, f2& ay, f2& az) {
  RecView v;
  load_view(R4, v);
  f2 rx[4], ry[4], rz[4], inv[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) corner_pair(px, py, pz, cx[k], cy[k], cz[k], rx[k], ry[k], rz[k], inv[k]);
  fil_pair<0>(v, px, py, pz, cx[0], cy[0], cz[0], rx[0], ry[0], rz[0], inv[0], rx[1], ry[1], rz[1], inv[1], ax, ay, az);
  fil_pair<1>(v, px, py, pz, cx[1], cy[1], cz[1], rx[1], ry[1], rz[1], inv[1], rx[2], ry[2], rz[2], inv[2], ax, ay, az);
  fil_pair<2>(v, px, py, pz, cx[2], cy[2], cz[2], rx[2], ry[2], rz[2], inv[2], rx[3], ry[3], rz[3], inv[3], ax, ay, az);
  fil_pair<3>(v, px, py, pz, cx[3], cy[3], cz[3], rx[3], ry[3], rz[3], inv[3], rx[0], ry[0], rz[0], inv[0], ax, ay, az);
}

// rec_lat_pair<2> with packed pairs
__device__ __forceinline__ void rec_lat_packed(const float4* __restrict__ R4, const float (&cx)[4],
                                               const float (&cy)[4], const float (&cz)[4], f2 px, f2 py, f2 pz, f2& ax,
                                               f2& ay, f2& az) {
  RecView v;
  load_view(R4, v);
  f2 rx[4], ry[4], rz[4], inv[4];
#pragma unroll
  for (int k = 0; k < 3; ++k) corner_pair(px, py, pz, cx[k], cy[k], cz[k], rx[k], ry[k], rz[k], inv[k]);
  fil_pair<0>(v, px, py, pz, cx[0], cy[0], cz[0], rx[0], ry[0], rz[0], inv[0], rx[1], ry[1], rz[1], inv[1], ax, ay, az);
  fil_pair<1>(v, px, py, pz, cx[1], cy[1], cz[1], rx[1], ry[1], rz[1], inv[1], rx[2], ry[2], rz[2], inv[2], ax, ay, az);
  const bool t2 = v.a4v[2] >= 0.f, t3 = v.a4v[3] >= 0.f;
  if (t2 || t3) {
    corner_pair(px, py, pz, cx[3], cy[3], cz[3], rx[3], ry[3], rz[3], inv[3]);
    if (t2)
      fil_pair<2>(v, px, py, pz, cx[2], cy[2], cz[2], rx[2], ry[2], rz[2], inv[2], rx[3], ry[3], rz[3], inv[3], ax, ay,
                  az);
    if (t3)
      fil_pair<3>(v, px, py, pz, cx[3], cy[3], cz[3], rx[3], ry[3], rz[3], inv[3], rx[0], ry[0], rz[0], inv[0], ax, ay,
                  az);
  }
}

// One block = 8 consumer warps (256 threads x kTPT targets) + 1 producer
// warp.  The producer's lane 0 streams the chunk's records through kStages
// shared stages with bulk copies; consumers wait on a stage's FULL barrier,
// compute, and release it through its EMPTY barrier (one arrival per
// consumer warp).  Tile shapes (targets per thread, stages, resident blocks
// per SM) are template arguments; kPartial32Shapes lists the compiled ones,
// among which the case autotuner picks per evaluation.
constexpr int kTileW = 128;                 // records per stage (24 KB)
// evaluations with at most this many targets (and at most 2^22 record-target
// pairs) find their near pairs by testing every pair (k_near_find_small)
constexpr int kNearSmallTargets = 1024;
constexpr int kConsumerWarps = 8;
constexpr int kBlockW = (kConsumerWarps + 1) * 32;

// LAT: the records are in lattice form (edges 2 and 3 marked when they carry
// no circulation); otherwise every record is evaluated as a whole ring.
template <bool LAT, int kTPT, int kStages, int kMinBlocks>
__global__ void __launch_bounds__(kBlockW, kMinBlocks) k_partial32(const float* __restrict__ rec32,
                                                                  const Chunk* __restrict__ chunks,
                                                                  const double* __restrict__ P, int M,
                                                                  double* __restrict__ part, int* __restrict__ ctl) {
  constexpr int kTargetsPerBlock = kConsumerWarps * 32 * kTPT;
  extern __shared__ __align__(16) float stage[];  // [kStages][kTileW * kRec32]
  __shared__ __align__(8) uint64_t full[kStages];
  __shared__ __align__(8) uint64_t empty[kStages];
  const int q = blockIdx.y;
  const Chunk ch = chunks[q];
  const int tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;
  const int ntiles = (ch.rec_count + kTileW - 1) / kTileW;
  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], kConsumerWarps);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();  // the only block-wide barrier: roles split below

  if (warp == kConsumerWarps) {
    // ---- producer ----
    if (lane == 0) {
      int issued = 0;
      for (int t = 0; t < ntiles; ++t) {
        const int s = t % kStages;
        // a stage the consumers have not released may still be read: after an
        // expired wait no further copy is issued (the consumers' own bounded
        // waits for the missing tiles expire and they stop)
        if (t >= kStages && !mbar_wait(&empty[s], ((t / kStages) - 1) & 1)) {
          atomicExch(ctl, 1);
          break;
        }
        const int n = min(kTileW, ch.rec_count - t * kTileW);
        const uint32_t bytes = (uint32_t)n * kRec32 * 4u;
        mbar_expect_tx(&full[s], bytes);
        bulk_g2s(stage + s * kTileW * kRec32, rec32 + (size_t)(ch.rec_begin + t * kTileW) * kRec32, bytes, &full[s]);
        issued = t + 1;
      }
      // the block must not retire with a copy still writing its shared memory
      for (int t = max(0, issued - kStages); t < issued; ++t)
        if (!mbar_wait(&full[t % kStages], (t / kStages) & 1)) atomicExch(ctl, 2);
    }
    return;
  }

  // ---- consumers ----
  int mt[kTPT];
  bool valid[kTPT];
  float px[kTPT], py[kTPT], pz[kTPT];
  double acc64[kTPT][3];
#pragma unroll
  for (int u = 0; u < kTPT; ++u) {
    // runs of 256 targets per u: a warp's targets are two runs of 32
    // consecutive ones (measured 1-2 % faster than one run of 64)
    mt[u] = blockIdx.x * kTargetsPerBlock + u * (32 * kConsumerWarps) + tid;
    valid[u] = mt[u] < M;
    const int mm = valid[u] ? mt[u] : M - 1;
    px[u] = (float)P[3 * (size_t)mm];
    py[u] = (float)P[3 * (size_t)mm + 1];
    pz[u] = (float)P[3 * (size_t)mm + 2];
    acc64[u][0] = acc64[u][1] = acc64[u][2] = 0.0;
  }
  bool ok = true;
  for (int t = 0; t < ntiles; ++t) {
    const int s = t % kStages;
    // the warp goes on only if every lane saw the stage arrive; after one
    // expired wait it waits no more (ok is uniform across the warp)
    if (ok && !__all_sync(kFull, mbar_wait(&full[s], (t / kStages) & 1))) {
      ok = false;
      if (lane == 0) atomicExch(ctl, 1);
    }
    if (ok && kTPT == 2) {
      // both targets in packed pairs
      const int n = min(kTileW, ch.rec_count - t * kTileW);
      const float* tile = stage + s * kTileW * kRec32;
      const f2 PX = f2pack(px[0], px[kTPT - 1]), PY = f2pack(py[0], py[kTPT - 1]), PZ = f2pack(pz[0], pz[kTPT - 1]);
      f2 AX = 0ull, AY = 0ull, AZ = 0ull;  // +0.0f in both lanes
#pragma unroll 1
      for (int r = 0; r < n; ++r) {
        const float4* R4 = reinterpret_cast<const float4*>(tile + r * kRec32);
        const float4 q0 = R4[0], q1 = R4[1], q2 = R4[2];  // corners
        const float cx[4] = {q0.x, q0.w, q1.z, q2.y};
        const float cy[4] = {q0.y, q1.x, q1.w, q2.z};
        const float cz[4] = {q0.z, q1.y, q2.x, q2.w};
        if (!LAT) ring_pair(R4, cx, cy, cz, PX, PY, PZ, AX, AY, AZ);
        else rec_lat_packed(R4, cx, cy, cz, PX, PY, PZ, AX, AY, AZ);
      }
      float a0, a1;
      f2unpack(AX, a0, a1);
      acc64[0][0] += (double)a0;
      acc64[kTPT - 1][0] += (double)a1;
      f2unpack(AY, a0, a1);
      acc64[0][1] += (double)a0;
      acc64[kTPT - 1][1] += (double)a1;
      f2unpack(AZ, a0, a1);
      acc64[0][2] += (double)a0;
      acc64[kTPT - 1][2] += (double)a1;
    } else if (ok) {
      const int n = min(kTileW, ch.rec_count - t * kTileW);
      const float* tile = stage + s * kTileW * kRec32;
      float ax[kTPT], ay[kTPT], az[kTPT];
#pragma unroll
      for (int u = 0; u < kTPT; ++u) ax[u] = ay[u] = az[u] = 0.f;
#pragma unroll 1
      for (int r = 0; r < n; ++r) {
        const float4* R4 = reinterpret_cast<const float4*>(tile + r * kRec32);
        const float4 q0 = R4[0], q1 = R4[1], q2 = R4[2];  // corners
        const float cx[4] = {q0.x, q0.w, q1.z, q2.y};
        const float cy[4] = {q0.y, q1.x, q1.w, q2.z};
        const float cz[4] = {q0.z, q1.y, q2.x, q2.w};
        if (!LAT) {
          // both targets' corner vectors first: more independent work in flight
          float rx[kTPT][4], ry[kTPT][4], rz[kTPT][4], inv[kTPT][4];
#pragma unroll
          for (int u = 0; u < kTPT; ++u) corner_vectors(px[u], py[u], pz[u], cx, cy, cz, rx[u], ry[u], rz[u], inv[u]);
#pragma unroll
          for (int u = 0; u < kTPT; ++u) ring_fp32(R4, rx[u], ry[u], rz[u], inv[u], ax[u], ay[u], az[u]);
        } else {
          rec_lat_pair<kTPT>(R4, cx, cy, cz, px, py, pz, ax, ay, az);
        }
      }
#pragma unroll
      for (int u = 0; u < kTPT; ++u) {
        acc64[u][0] += (double)ax[u];
        acc64[u][1] += (double)ay[u];
        acc64[u][2] += (double)az[u];
      }
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[s]);
  }
#pragma unroll
  for (int u = 0; u < kTPT; ++u) {
    if (valid[u]) {
      double* o = part + ((size_t)q * M + mt[u]) * 3;
      o[0] = acc64[u][0];
      o[1] = acc64[u][1];
      o[2] = acc64[u][2];
    }
  }
}


// ---- near field: uniform grid over the targets, occupied cells hashed -----
// Scratch layout: grid_layout (vlm_bs.h).  A cell's key packs its three
// coordinates (21 bits each, offset by 2^20); kEmptyKey marks a free slot.
// Every target's cell is inserted by linear probing (atomicCAS); the slot's
// targets are then listed contiguously (count, scan, fill).  A lookup of a
// cell probes until it finds the key (the cell is occupied) or a free slot
// (it is not), so empty cells cost one or two reads and a slot holds the
// targets of one cell only.
constexpr unsigned long long kEmptyKey = ~0ull;
constexpr double kCellOverZone = 3.0;  // cell size / mean near-zone radius
constexpr int kCellBias = 1 << 20;

__device__ __forceinline__ unsigned long long cell_key(int ix, int iy, int iz) {
  return ((unsigned long long)(unsigned)(ix + kCellBias) & 0x1FFFFFull) |
         (((unsigned long long)(unsigned)(iy + kCellBias) & 0x1FFFFFull) << 21) |
         (((unsigned long long)(unsigned)(iz + kCellBias) & 0x1FFFFFull) << 42);
}
__device__ __forceinline__ unsigned cell_hash(int ix, int iy, int iz, int T) {
  return ((unsigned)ix * 73856093u ^ (unsigned)iy * 19349663u ^ (unsigned)iz * 83492791u) & (unsigned)(T - 1);
}
// saturating conversion, clamped to the key's 21-bit range
__device__ __forceinline__ int cell_of(float x, float invh) {
  return max(-kCellBias + 1, min(kCellBias - 2, __float2int_rd(x * invh)));
}
// the slot of cell (ix, iy, iz), or -1 if no target lies in it
__device__ __forceinline__ int cell_slot(const unsigned long long* __restrict__ key, int T, int ix, int iy, int iz) {
  const unsigned long long k = cell_key(ix, iy, iz);
  unsigned b = cell_hash(ix, iy, iz, T);
  for (int n = 0; n < T; ++n) {
    const unsigned long long v = key[b];
    if (v == k) return (int)b;
    if (v == kEmptyKey) return -1;
    b = (b + 1) & (unsigned)(T - 1);
  }
  return -1;
}

__global__ void k_grid_init(unsigned char* scratch, int T) {
  GridHdr* H = reinterpret_cast<GridHdr*>(scratch);
  H->zsum = 0.0;
  H->zcount = 0u;
  H->T = T;
  for (int a = 0; a < 3; ++a) {
    H->lo[a] = INT_MAX;
    H->hi[a] = INT_MIN;
  }
}

// a float's order-preserving int code (finite values) and back
__device__ __forceinline__ int ord_code(float f) {
  const int i = __float_as_int(f);
  return i >= 0 ? i : i ^ 0x7FFFFFFF;
}
__device__ __forceinline__ float ord_value(int c) { return __int_as_float(c >= 0 ? c : c ^ 0x7FFFFFFF); }

// Sum and count of the near-zone radii near_factor rvc_k = sqrt([32 + k]) /
// |e_k| of the active filaments (the cell size is twice their mean).
__global__ void k_zone_mean(const float* __restrict__ rec32, int nrec, unsigned char* __restrict__ scratch) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double z = 0.0;
  unsigned c = 0u;
  if (i < nrec) {
    const float* R = rec32 + (size_t)i * kRec32;
    for (int k = 0; k < 4; ++k) {
      const float thr = R[32 + k];
      if (!(thr >= 0.f)) continue;
      const int j = (k + 1) & 3;
      const float ex = R[3 * j] - R[3 * k], ey = R[3 * j + 1] - R[3 * k + 1], ez = R[3 * j + 2] - R[3 * k + 2];
      const float ee = fmaf(ex, ex, fmaf(ey, ey, ez * ez));
      if (!(ee > 0.f)) continue;
      z += sqrt((double)thr / (double)ee);
      ++c;
    }
  }
  // one atomic pair per warp
  for (int o = 16; o > 0; o >>= 1) {
    z += __shfl_down_sync(kFull, z, o);
    c += __shfl_down_sync(kFull, c, o);
  }
  if ((threadIdx.x & 31) == 0 && c) {
    GridHdr* H = reinterpret_cast<GridHdr*>(scratch);
    atomicAdd(&H->zsum, z);
    atomicAdd(&H->zcount, c);
  }
}

__device__ __forceinline__ float grid_h(const GridHdr* H) {
  return H->zcount ? (float)(kCellOverZone * H->zsum / (double)H->zcount) : 0.f;
}

// PASS 0: insert the target's cell key and count the target in its slot;
// PASS 1: write the target's FP32 position and index at its slot's cursor.
template <int PASS>
__global__ void k_tgrid_insert(const double* __restrict__ P, int M, unsigned char* __restrict__ scratch) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (PASS == 0) {
    // the targets' bounding box: one min and one max per axis and warp
    GridHdr* Hw = reinterpret_cast<GridHdr*>(scratch);
    for (int a = 0; a < 3; ++a) {
      const int c = m < M ? ord_code((float)P[3 * (size_t)m + a]) : 0;
      const int cmin = __reduce_min_sync(kFull, m < M ? c : INT_MAX);
      const int cmax = __reduce_max_sync(kFull, m < M ? c : INT_MIN);
      if ((threadIdx.x & 31) == 0 && cmin <= cmax) {
        atomicMin(&Hw->lo[a], cmin);
        atomicMax(&Hw->hi[a], cmax);
      }
    }
  }
  if (m >= M) return;
  const GridHdr* H = reinterpret_cast<const GridHdr*>(scratch);
  const float h = grid_h(H);
  if (!(h > 0.f)) return;
  const float invh = 1.f / h;
  const int T = H->T;
  const GridLayout L = grid_layout(M);
  unsigned long long* key = reinterpret_cast<unsigned long long*>(scratch + L.key);
  int* count = reinterpret_cast<int*>(scratch + L.count);
  const int ix = cell_of((float)P[3 * (size_t)m], invh), iy = cell_of((float)P[3 * (size_t)m + 1], invh),
            iz = cell_of((float)P[3 * (size_t)m + 2], invh);
  if (PASS == 0) {
    const unsigned long long k = cell_key(ix, iy, iz);
    unsigned b = cell_hash(ix, iy, iz, T);
    // T >= M >= occupied cells: a free slot always exists
    for (int n = 0; n < T; ++n) {
      const unsigned long long old = atomicCAS(key + b, kEmptyKey, k);
      if (old == kEmptyKey || old == k) {
        atomicAdd(count + b, 1);
        return;
      }
      b = (b + 1) & (unsigned)(T - 1);
    }
  } else {
    const int b = cell_slot(key, T, ix, iy, iz);
    const int slot = atomicAdd(count + b, 1);
    reinterpret_cast<float4*>(scratch + L.entry)[slot] =
        make_float4((float)P[3 * (size_t)m], (float)P[3 * (size_t)m + 1], (float)P[3 * (size_t)m + 2],
                    __int_as_float(m));
  }
}

// Exclusive scan of the slot counts into start[0..T]; the counts become the
// fill cursors (= start).  One block of 1024 threads: tiles of 1024 slots,
// each scanned with warp shuffles, carried from tile to tile.
__global__ void k_grid_scan(int M, unsigned char* __restrict__ scratch) {
  const GridLayout L = grid_layout(M);
  const int T = reinterpret_cast<const GridHdr*>(scratch)->T;
  int* count = reinterpret_cast<int*>(scratch + L.count);
  int* start = reinterpret_cast<int*>(scratch + L.start);
  __shared__ int wsum[32];
  __shared__ int carry;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < T; base += 1024) {
    const int i = base + threadIdx.x;
    const int c = i < T ? count[i] : 0;
    int x = c;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(kFull, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    if (warp == 0) {
      int w = wsum[lane];
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(kFull, w, o);
        if (lane >= o) w += y;
      }
      wsum[lane] = w;  // inclusive over warps
    }
    __syncthreads();
    const int excl = carry + (warp ? wsum[warp - 1] : 0) + x - c;
    if (i < T) {
      start[i] = excl;
      count[i] = excl;
    }
    __syncthreads();
    if (threadIdx.x == 0) carry += wsum[31];
    __syncthreads();
  }
  if (threadIdx.x == 0) start[T] = carry;
}

// FP64 filament velocity (src/classdef.f90:476-503: the Vatistas n=2 kernel
// with the eps^2 cut-off) written for speed on a part whose FP64 divide and
// square root are slow: three reciprocal square roots, no division.  Equal
// to the reference arithmetic to a few FP64 ulps.
__device__ __forceinline__ d3 fil_near64(d3 p, d3 a, d3 b, double rvc) {
  const d3 r1 = p - a, r2 = p - b, r0 = r1 - r2;
  const d3 c = cross3(r1, r2);
  const double c2 = dot3(c, c);
  if (!(c2 > kEps * kEps)) return zero3();
  const double d = dot3(r0, r1) * rsqrt(dot3(r1, r1)) - dot3(r0, r2) * rsqrt(dot3(r2, r2));
  const double s2 = (rvc * rvc) * dot3(r0, r0);
  return c * (d * rsqrt(s2 * s2 + c2 * c2) * kInv4Pi);
}

// Detection, one warp per filament (record r, edge k).  A filament with a near zone
// (radius z = near_factor rvc_k, from [32 + k]) is cut into np pieces no
// longer than a cell; the lanes take the cells of each piece's box (grown by
// 1.42 z, which holds the zone's cylinder and its extensions past the ends),
// skip cells whose centre is farther from the piece than sqrt(2) z + half a
// cell diagonal, look the rest up in the cell table, and then share out the
// targets of the cells found, 32 at a time.  A target is taken only by the
// piece that holds its projection on the filament, so every (target,
// filament) pair is tested once.  A near pair -- |r_k x r_j|^2 <
// (near_factor rvc |e|)^2 and the projection within the segment extended by
// near_factor rvc, on the FP32 kernel's own FP32 values -- is appended to the
// near list (one atomic per warp and batch; ctl[1] counts, ctl[0] = 3 if the
// list is full).
// Near pairs of an evaluation with few targets (the collocation points):
// every (record, target) pair gets k_near_find's test directly, one thread
// per pair -- the same pairs without building a grid of the targets or
// walking every filament through it.
__global__ void __launch_bounds__(256) k_near_find_small(const float* __restrict__ rec32, int nrec,
                                                         const Chunk* __restrict__ chunks, int nchunks,
                                                         const double* __restrict__ P, int M,
                                                         NearPair* __restrict__ near, int near_cap,
                                                         int* __restrict__ ctl) {
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  const bool live = t < (size_t)nrec * M;
  const int r = live ? (int)(t / M) : 0, m = live ? (int)(t % M) : 0;
  const float px = (float)P[3 * (size_t)m], py = (float)P[3 * (size_t)m + 1], pz = (float)P[3 * (size_t)m + 2];
  const float* R = rec32 + (size_t)r * kRec32;
  int q = 0;
  {
    int hi = nchunks - 1;
    while (q < hi) {
      const int mid = (q + hi + 1) >> 1;
      if (chunks[mid].rec_begin <= r) q = mid;
      else hi = mid - 1;
    }
  }
  for (int k = 0; k < 4; ++k) {
    bool isnear = false;
    const float thr = R[32 + k];
    if (live && thr >= 0.f) {
      const int j = (k + 1) & 3;
      const float ax = R[3 * k], ay = R[3 * k + 1], az = R[3 * k + 2];
      const float ex = R[3 * j] - ax, ey = R[3 * j + 1] - ay, ez = R[3 * j + 2] - az;
      const float eev = R[24 + k];
      const float ee = fmaf(ex, ex, fmaf(ey, ey, ez * ez));
      if (ee > 0.f && eev != 0.f) {
        const float len = sqrtf(ee);
        const float z = sqrtf(thr) / len;
        const float iee = 1.f / ee, z2 = z * z, tlo = -z * len, thi = fmaf(z, len, ee);
        const float dx = px - ax, dy = py - ay, dz = pz - az;
        const float tr = fmaf(dx, ex, fmaf(dy, ey, dz * ez));
        const float tn = tr * iee;
        const float qx = fmaf(-tn, ex, dx), qy = fmaf(-tn, ey, dy), qz = fmaf(-tn, ez, dz);
        isnear = fmaf(qx, qx, fmaf(qy, qy, qz * qz)) < z2 && tr > tlo && tr < thi;
      }
    }
    const unsigned mask = __ballot_sync(kFull, isnear);
    if (mask) {
      int base_slot = 0;
      if (lane == 0) base_slot = atomicAdd(ctl + 1, __popc(mask));
      base_slot = __shfl_sync(kFull, base_slot, 0);
      if (isnear) {
        const int slot = base_slot + __popc(mask & lt);
        if (slot < near_cap) {
          NearPair np_;
          np_.m = m;
          np_.q = q;
          np_.rec = r;
          np_.k = k;
          near[slot] = np_;
        } else {
          atomicExch(ctl, 3);
        }
      }
    }
  }
}

__global__ void __launch_bounds__(256, 4) k_near_find(const float* __restrict__ rec32, int nrec,
                                                   const Chunk* __restrict__ chunks, int nchunks,
                                                   const double* __restrict__ P, int M,
                                                   const unsigned char* __restrict__ scratch,
                                                   NearPair* __restrict__ near, int near_cap, int* __restrict__ ctl) {
  const size_t wid = (blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (wid >= (size_t)nrec * 4) return;  // whole warps leave together
  const int r = (int)(wid >> 2), k = (int)(wid & 3);
  const float* R = rec32 + (size_t)r * kRec32;
  const float thr = R[32 + k];
  if (!(thr >= 0.f)) return;
  const GridHdr* H = reinterpret_cast<const GridHdr*>(scratch);
  const float h = grid_h(H);
  if (!(h > 0.f)) return;
  const float invh = 1.f / h;
  const int T = H->T;
  const GridLayout L = grid_layout(M);
  const unsigned long long* key = reinterpret_cast<const unsigned long long*>(scratch + L.key);
  const int* start = reinterpret_cast<const int*>(scratch + L.start);
  const float4* entry = reinterpret_cast<const float4*>(scratch + L.entry);
  // the record's chunk (chunks are in record order)
  int q = 0;
  {
    int hi = nchunks - 1;
    while (q < hi) {
      const int mid = (q + hi + 1) >> 1;
      if (chunks[mid].rec_begin <= r) q = mid;
      else hi = mid - 1;
    }
  }
  const unsigned lt = (1u << lane) - 1u;
  {
    const int j = (k + 1) & 3;
    const float ax = R[3 * k], ay = R[3 * k + 1], az = R[3 * k + 2];
    const float bx = R[3 * j], by = R[3 * j + 1], bz = R[3 * j + 2];
    const float eev = R[24 + k];
    const float ex = bx - ax, ey = by - ay, ez = bz - az;
    const float ee = fmaf(ex, ex, fmaf(ey, ey, ez * ez));
    if (!(ee > 0.f) || !(eev != 0.f)) return;
    const float len = sqrtf(ee);
    const float z = sqrtf(thr) / len;
    // near zone: distance to the line < z, projection within the segment
    // extended by z at both ends (the FP32 kernel's own near test, in
    // distance form; which pairs are corrected is an accuracy choice, the
    // correction itself is exact)
    const float iee = 1.f / ee, z2 = z * z, tlo = -z * len, thi = fmaf(z, len, ee);
    const int np = max(1, min(4096, (int)ceilf(len * invh)));
    const float amax = fmaxf(fmaxf(fabsf(ax), fabsf(ay)), fabsf(az)) + len;
    const float grow = 1.42f * z * 1.0001f + 1e-6f + 4e-7f * amax;
    // a near zone wholly outside the targets' bounding box holds none of
    // them (the cells walked below lie within the segment's box +- grow)
    if (fmaxf(ax, bx) + grow < ord_value(H->lo[0]) || fminf(ax, bx) - grow > ord_value(H->hi[0]) ||
        fmaxf(ay, by) + grow < ord_value(H->lo[1]) || fminf(ay, by) - grow > ord_value(H->hi[1]) ||
        fmaxf(az, bz) + grow < ord_value(H->lo[2]) || fminf(az, bz) - grow > ord_value(H->hi[2]))
      return;
    const float reach = 1.4143f * z * 1.0001f + 0.8661f * h + 1e-6f + 4e-7f * amax;
    const float reach2 = reach * reach;
    for (int pc = 0; pc < np; ++pc) {
      const float t0 = (float)pc / np, t1 = (float)(pc + 1) / np;
      const float qx0 = fmaf(ex, t0, ax), qy0 = fmaf(ey, t0, ay), qz0 = fmaf(ez, t0, az);
      const float qx1 = fmaf(ex, t1, ax), qy1 = fmaf(ey, t1, ay), qz1 = fmaf(ez, t1, az);
      const float sx = qx1 - qx0, sy = qy1 - qy0, sz = qz1 - qz0;
      const float ss = fmaf(sx, sx, fmaf(sy, sy, sz * sz));
      const int x0 = cell_of(fminf(qx0, qx1) - grow, invh), x1 = cell_of(fmaxf(qx0, qx1) + grow, invh);
      const int y0 = cell_of(fminf(qy0, qy1) - grow, invh), y1 = cell_of(fmaxf(qy0, qy1) + grow, invh);
      const int z0 = cell_of(fminf(qz0, qz1) - grow, invh), z1 = cell_of(fmaxf(qz0, qz1) + grow, invh);
      const int nx = x1 - x0 + 1, ny = y1 - y0 + 1, nxy = nx * ny;
      const float inx = 1.f / (float)nx, inxy = 1.f / (float)nxy;
      // (a piece's box spans a few cells per axis unless a zone is far larger
      // than the mean; 2^31 cells would take hours, never an index overflow)
      const int ncell = (int)min((long long)nxy * (z1 - z0 + 1), (long long)INT_MAX - 32);
      for (int base = 0; base < ncell; base += 32) {
        // each lane one cell: culled by distance, then looked up
        const int ci = base + lane;
        int s0 = 0, cnt = 0;
        if (ci < ncell) {
          // exact for the small cell counts of a piece (ci < 2^22)
          const int iz = (int)(((float)ci + 0.5f) * inxy), rem = ci - iz * nxy;
          const int iy = (int)(((float)rem + 0.5f) * inx);
          const int cx = x0 + rem - iy * nx, cy = y0 + iy, cz = z0 + iz;
          const float gx = ((float)cx + 0.5f) * h - qx0, gy = ((float)cy + 0.5f) * h - qy0,
                      gz = ((float)cz + 0.5f) * h - qz0;
          const float tq = ss > 0.f ? fminf(fmaxf(fmaf(gx, sx, fmaf(gy, sy, gz * sz)) / ss, 0.f), 1.f) : 0.f;
          const float dx = fmaf(-tq, sx, gx), dy = fmaf(-tq, sy, gy), dz = fmaf(-tq, sz, gz);
          if (fmaf(dx, dx, fmaf(dy, dy, dz * dz)) <= reach2) {
            const int b = cell_slot(key, T, cx, cy, cz);
            if (b >= 0) {
              s0 = start[b];
              cnt = start[b + 1] - s0;
            }
          }
        }
        // the found cells' targets, shared out 32 at a time
        int incl = cnt;
        for (int o = 1; o < 32; o <<= 1) {
          const int y = __shfl_up_sync(kFull, incl, o);
          if (lane >= o) incl += y;
        }
        const int total = __shfl_sync(kFull, incl, 31);
        for (int tb = 0; tb < total; tb += 32) {
          const int idx = tb + lane;
          // the lane whose cell holds target idx: the first with incl > idx
          int own = 0;
          for (int step = 16; step >= 1; step >>= 1) {
            const int v = __shfl_sync(kFull, incl, own + step - 1);
            if (v <= idx) own += step;
          }
          own = min(own, 31);
          const int os0 = __shfl_sync(kFull, s0, own);
          const int oex = __shfl_sync(kFull, incl - cnt, own);
          bool isnear = false;
          int m = 0;
          if (idx < total) {
            const float4 e4 = entry[os0 + idx - oex];
            m = __float_as_int(e4.w);
            // projection on the filament and distance to its line
            const float dx = e4.x - ax, dy = e4.y - ay, dz = e4.z - az;
            const float tr = fmaf(dx, ex, fmaf(dy, ey, dz * ez));  // e.(p - a)
            const float tn = tr * iee;
            const float qx = fmaf(-tn, ex, dx), qy = fmaf(-tn, ey, dy), qz = fmaf(-tn, ez, dz);
            // the piece that holds the target's projection takes the pair
            const int piece = max(0, min(np - 1, __float2int_rd(tn * (float)np)));
            isnear = piece == pc && fmaf(qx, qx, fmaf(qy, qy, qz * qz)) < z2 && tr > tlo && tr < thi;
          }
          const unsigned mask = __ballot_sync(kFull, isnear);
          if (mask) {
            int base_slot = 0;
            if (lane == 0) base_slot = atomicAdd(ctl + 1, __popc(mask));
            base_slot = __shfl_sync(kFull, base_slot, 0);
            if (isnear) {
              const int slot = base_slot + __popc(mask & lt);
              if (slot < near_cap) {
                NearPair np_;
                np_.m = m;
                np_.q = q;
                np_.rec = r;
                np_.k = k;
                near[slot] = np_;
              } else {
                atomicExch(ctl, 3);
              }
            }
          }
        }
      }
    }
  }
}

// Correction, one thread per listed near pair: FP64 velocity x weight - the
// FP32 kernel's contribution f (r_k x r_j) (recomputed with the same FP32
// operations, the product taken exactly in FP64), added in fixed point to the
// accumulator of the target and the record's chunk (order-independent).
// ctl[0] = 4 flags a correction outside the fixed-point range.
__global__ void k_near_fix(const NearPair* __restrict__ near, int near_cap, const float* __restrict__ rec32,
                           const double* __restrict__ rec64, const double* __restrict__ ew,
                           const double* __restrict__ P, int M, unsigned long long* __restrict__ nacc,
                           int* __restrict__ ctl) {
  const int n = min(ctl[1], near_cap);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const NearPair np_ = near[i];
    const int r = np_.rec, k = np_.k, j = (k + 1) & 3, m = np_.m;
    const float* R = rec32 + (size_t)r * kRec32;
    const double* D = rec64 + (size_t)r * kRec64;
    const double p64x = P[3 * (size_t)m], p64y = P[3 * (size_t)m + 1], p64z = P[3 * (size_t)m + 2];
    const float px = (float)p64x, py = (float)p64y, pz = (float)p64z;  // as the FP32 kernel
    float rxk, ryk, rzk, invk, rxj, ryj, rzj, invj;
    corner_vector(px, py, pz, R[3 * k], R[3 * k + 1], R[3 * k + 2], rxk, ryk, rzk, invk);
    corner_vector(px, py, pz, R[3 * j], R[3 * j + 1], R[3 * j + 2], rxj, ryj, rzj, invj);
    const Fil32 t = fil_terms(R[12 + 3 * k], R[12 + 3 * k + 1], R[12 + 3 * k + 2], R[24 + k], R[28 + k], rxk, ryk, rzk,
                              invk, rxj, ryj, rzj, invj);
    const d3 p = mk3(p64x, p64y, p64z);
    d3 v64;
    if ((int)D[17] & REC_FIL) {
      v64 = fil_near64(p, mk3(D[0], D[1], D[2]), mk3(D[3], D[4], D[5]), D[12]);
    } else {
      v64 = fil_near64(p, mk3(D[3 * k], D[3 * k + 1], D[3 * k + 2]), mk3(D[3 * j], D[3 * j + 1], D[3 * j + 2]),
                       D[12 + k]);
    }
    v64 = v64 * (ew ? ew[4 * (size_t)r + k] : D[16]);
    const double c[3] = {v64.x - (double)t.f * (double)t.kx, v64.y - (double)t.f * (double)t.ky,
                         v64.z - (double)t.f * (double)t.kz};
    unsigned long long* o = nacc + ((size_t)np_.q * M + m) * 3;
    for (int a = 0; a < 3; ++a) {
      if (!(fabs(c[a]) < kNearMax)) {
        atomicExch(ctl, 4);
        continue;
      }
      atomicAdd(o + a, (unsigned long long)__double2ll_rn(c[a] * kNearScale));
    }
  }
}

__global__ void k_set_flag(int* ctl, int code) { atomicExch(ctl, code); }

// part += nacc / 2^44, and nacc back to zero for the next evaluation.
__global__ void k_near_apply(double* __restrict__ part, long long* __restrict__ nacc, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const long long a = nacc[i];
    if (a != 0) {
      part[i] += (double)a * (1.0 / kNearScale);
      nacc[i] = 0;
    }
  }
}

// Self-test of the bounded waits: one thread waits on an mbarrier that
// nothing arrives on, with a short limit; the wait must give up and report.
__global__ void k_wait_probe(uint32_t limit, int* out) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x != 0) return;
  mbar_init(&bar, 1);
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  out[0] = mbar_wait(&bar, 0, limit) ? 0 : 1;  // 1: the limit expired, as it must
}

// FP64 record -> FP32 record.  The edge vectors are differenced in FP64
// (nearby corners cancel) and rounded once; everything else is FP32 (the
// record is FP32; GB300's FP64 rate would make this kernel latency-bound).
// With edge weights ew (lattice form) edge k carries ew[k] and is active iff
// ew[k] != 0; without, every filament of a record carries its gam unless the
// record is skipped (|gam| <= eps with REC_SKIP), a single filament only its
// first.  Inactive edges 2 and 3 are marked for the kernel to skip.
__global__ void k_pack32(const double* __restrict__ rec64, int nrec, double near_factor, float* __restrict__ rec32,
                         const double* __restrict__ ew) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nrec) return;
  const double* R = rec64 + (size_t)i * kRec64;
  float* o = rec32 + (size_t)i * kRec32;
  const int flags = (int)R[17];
  const double g = R[16];
  const bool skipped = (flags & REC_SKIP) && !(fabs(g) > kEps);
  const bool fil = flags & REC_FIL;
  const double* EW = ew ? ew + 4 * (size_t)i : nullptr;
  // corner k (FP64) and core radius of filament k
  double cx[4], cy[4], cz[4];
  float rv[4];
  for (int k = 0; k < 4; ++k) {
    const int src = fil ? (k == 1 || k == 2 ? 1 : 0) : k;
    cx[k] = R[3 * src];
    cy[k] = R[3 * src + 1];
    cz[k] = R[3 * src + 2];
    rv[k] = fil ? (k == 0 ? (float)R[12] : 0.f) : (float)R[12 + k];
  }
  const float nf = (float)near_factor;
  const float w = (float)(g * kInv4Pi);
  for (int k = 0; k < 4; ++k) {
    const int j = (k + 1) & 3;
    const bool act = EW ? EW[k] != 0.0 : (!fil || k == 0) && !skipped;
    const float ex = (float)(cx[j] - cx[k]), ey = (float)(cy[j] - cy[k]), ez = (float)(cz[j] - cz[k]);
    const float ee = fmaf(ex, ex, fmaf(ey, ey, ez * ez));
    const float sk = rv[k] * sqrtf(ee);
    const float s2 = sk * sk;
    o[3 * k] = (float)cx[k];
    o[3 * k + 1] = (float)cy[k];
    o[3 * k + 2] = (float)cz[k];
    const float wk = act ? (EW ? (float)(EW[k] * kInv4Pi) : w) : 0.f;
    o[12 + 3 * k] = wk * ex;
    o[12 + 3 * k + 1] = wk * ey;
    o[12 + 3 * k + 2] = wk * ez;
    o[24 + k] = wk * ee;
    o[28 + k] = EW && k >= 2 && !act ? -1.f : fmaxf(s2 * s2, 1e-36f);
    const bool on = act && nf > 0.f;
    const float nfs = nf * sk;
    o[32 + k] = on ? nfs * nfs : -1.f;
    // -s < e.r1 < |e|^2 + s, multiplied by w_k
    const float blo = -nfs * wk, bhi = (ee + nfs) * wk;
    o[36 + k] = on ? fminf(blo, bhi) : 0.f;
    o[40 + k] = on ? fmaxf(blo, bhi) : 0.f;
  }
  o[44] = o[45] = o[46] = o[47] = 0.f;
}

}  // namespace

void launch_pack32(const double* rec64, int nrec, double near_factor, float* rec32, cudaStream_t s,
                   const double* ew) {
  if (nrec <= 0) return;
  count_launch();
  k_pack32<<<(nrec + 255) / 256, 256, 0, s>>>(rec64, nrec, near_factor, rec32, ew);
}

// The compiled tile shapes: {targets per thread, stages, blocks per SM}.
// Shape 0 = 2 targets per thread, 4 stages (96 KB), 2 blocks per SM: the
// most reuse of a staged record; shape 1 = 1 target per thread, 3 stages
// (72 KB), 3 blocks per SM: twice the target blocks and 1.5x the resident
// blocks, for evaluations whose grid would leave slots idle.
template <int V>
struct Shape32;
template <>
struct Shape32<0> {
  static constexpr int tpt = 2, stages = 4, minb = 2;
};
template <>
struct Shape32<1> {
  static constexpr int tpt = 1, stages = 3, minb = 3;
};
static_assert(kPartial32Shapes == 2, "shape table");

template <int V>
int shape_smem() {
  return Shape32<V>::stages * kTileW * kRec32 * (int)sizeof(float);
}

template <int V, bool LAT>
void set_smem_attr() {
  using S = Shape32<V>;
  cudaFuncSetAttribute(k_partial32<LAT, S::tpt, S::stages, S::minb>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       shape_smem<V>());
}

template <int V>
void launch_shape(bool lat, dim3 grid, const float* rec32, const Chunk* chunks, const double* P, int M, double* part,
                  int* ctl, cudaStream_t s) {
  using S = Shape32<V>;
  if (lat) k_partial32<true, S::tpt, S::stages, S::minb><<<grid, kBlockW, shape_smem<V>(), s>>>(rec32, chunks, P, M, part, ctl);
  else k_partial32<false, S::tpt, S::stages, S::minb><<<grid, kBlockW, shape_smem<V>(), s>>>(rec32, chunks, P, M, part, ctl);
}

// the dynamic shared-memory opt-in is per device; set it once on each
void ensure_smem_attrs() {
  static std::atomic<bool> attr[64];
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64 || !attr[dev].load(std::memory_order_acquire)) {
    set_smem_attr<0, false>();
    set_smem_attr<0, true>();
    set_smem_attr<1, false>();
    set_smem_attr<1, true>();
    if (dev >= 0 && dev < 64) attr[dev].store(true, std::memory_order_release);
  }
}

int partial32_targets_per_block(int shape) { return kConsumerWarps * 32 * (shape == 1 ? Shape32<1>::tpt : Shape32<0>::tpt); }

void launch_partial32(const float* rec32, const double* rec64, const Chunk* chunks, int nchunks, int nrec,
                      const double* P, int M, double* part, int* ctl, void* near_scratch, size_t near_bytes,
                      long long* nacc, cudaStream_t s, const double* ew, int shape, const NearOverlap* ov,
                      bool reuse_grid) {
  if (M <= 0 || nchunks <= 0) return;
  ensure_smem_attrs();
  const int tpb = partial32_targets_per_block(shape);
  dim3 grid((M + tpb - 1) / tpb, nchunks);
  const bool nearOn = near_scratch && nrec > 0;
  const size_t gridBytes = near_grid_bytes(M);
  if (nearOn && near_bytes < gridBytes + (size_t)kNearAlign) {
    count_launch();
    k_set_flag<<<1, 1, 0, s>>>(ctl, 3);
    return;
  }
  // With ov, the near-field detection and FP64 correction (which read only
  // the records and targets) run on ov->stream alongside the pair kernel;
  // the fold into the partial sums waits for both.
  cudaStream_t ns = s;
  if (nearOn && ov) {
    cudaEventRecord(ov->fork, s);
    cudaStreamWaitEvent(ov->stream, ov->fork, 0);
    ns = ov->stream;
  }
  count_launch();
  if (shape == 1) launch_shape<1>(ew != nullptr, grid, rec32, chunks, P, M, part, ctl, s);
  else launch_shape<0>(ew != nullptr, grid, rec32, chunks, P, M, part, ctl, s);
  if (!nearOn) return;
  // near field: targets binned in a grid, near pairs listed, FP64
  // corrections of the listed pairs, corrections folded into the partials
  unsigned char* g = static_cast<unsigned char*>(near_scratch);
  NearPair* list = reinterpret_cast<NearPair*>(g + gridBytes);
  const int cap = (int)std::min<size_t>((near_bytes - gridBytes) / sizeof(NearPair), (size_t)1 << 30);
  const GridLayout L = grid_layout(M);
  const int T = grid_buckets(M);
  const int sms = device_sm_count();
  if (M <= kNearSmallTargets && (size_t)nrec * M <= ((size_t)1 << 22)) {
    // few targets: every pair tested directly
    count_launches(2);
    k_near_find_small<<<(unsigned)(((size_t)nrec * M + 255) / 256), 256, 0, ns>>>(rec32, nrec, chunks, nchunks, P, M,
                                                                                   list, cap, ctl);
    k_near_fix<<<4 * sms, 128, 0, ns>>>(list, cap, rec32, rec64, ew, P, M,
                                        reinterpret_cast<unsigned long long*>(nacc), ctl);
    if (ns != s) {
      cudaEventRecord(ov->join, ns);
      cudaStreamWaitEvent(s, ov->join, 0);
    }
    const size_t n = (size_t)M * nchunks * 3;
    count_launch();
    k_near_apply<<<(unsigned)std::min<size_t>((n + 255) / 256, (size_t)8 * sms), 256, 0, s>>>(part, nacc, n);
    return;
  }
  if (!reuse_grid) {
    count_launches(5);
    k_grid_init<<<1, 1, 0, ns>>>(g, T);
    k_zone_mean<<<(nrec + 255) / 256, 256, 0, ns>>>(rec32, nrec, g);
    cudaMemsetAsync(g + L.key, 0xFF, (size_t)T * sizeof(unsigned long long), ns);
    cudaMemsetAsync(g + L.count, 0, (size_t)T * sizeof(int), ns);
    k_tgrid_insert<0><<<(M + 255) / 256, 256, 0, ns>>>(P, M, g);
    k_grid_scan<<<1, 1024, 0, ns>>>(M, g);
    k_tgrid_insert<1><<<(M + 255) / 256, 256, 0, ns>>>(P, M, g);
  }
  count_launches(2);
  k_near_find<<<(unsigned)(((size_t)nrec * 4 * 32 + 255) / 256), 256, 0, ns>>>(rec32, nrec, chunks, nchunks, P, M,
                                                                               g, list, cap, ctl);
  k_near_fix<<<4 * sms, 128, 0, ns>>>(list, cap, rec32, rec64, ew, P, M, reinterpret_cast<unsigned long long*>(nacc),
                                      ctl);
  if (ns != s) {
    cudaEventRecord(ov->join, ns);
    cudaStreamWaitEvent(s, ov->join, 0);
  }
  const size_t n = (size_t)M * nchunks * 3;
  count_launch();
  k_near_apply<<<(unsigned)std::min<size_t>((n + 255) / 256, (size_t)8 * sms), 256, 0, s>>>(part, nacc, n);
}

// A host without a usable device still plans (sizes are queried before any
// launch): it plans for a GB300's 152 SMs.
constexpr int kPlanSmsWithoutDevice = 152;

int device_sm_count() {
  static std::atomic<int> cache[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return kPlanSmsWithoutDevice;
  if (!cache[dev]) {
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
      return kPlanSmsWithoutDevice;
    cache[dev] = sms;
  }
  return cache[dev];
}

int partial32_slots(int shape) {
  static std::atomic<int> cache[64][kPartial32Shapes];
  int dev = 0;
  shape = shape == 1 ? 1 : 0;
  const int fallback = (shape == 1 ? Shape32<1>::minb : Shape32<0>::minb) * kPlanSmsWithoutDevice;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return fallback;
  if (!cache[dev][shape]) {
    int per = 0;
    ensure_smem_attrs();
    if (shape == 1) {
      using S = Shape32<1>;
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_partial32<true, S::tpt, S::stages, S::minb>, kBlockW,
                                                    shape_smem<1>());
    } else {
      using S = Shape32<0>;
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_partial32<true, S::tpt, S::stages, S::minb>, kBlockW,
                                                    shape_smem<0>());
    }
    cache[dev][shape] = device_sm_count() * std::max(1, per);
  }
  return cache[dev][shape];
}

int selftest_bounded_wait(uint32_t limit) {
  int* d = nullptr;
  if (cudaMalloc(&d, sizeof(int)) != cudaSuccess) return -1;
  int h = -1;
  count_launch();
  k_wait_probe<<<1, 32>>>(limit, d);
  cudaError_t e = cudaMemcpy(&h, d, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(d);
  return e == cudaSuccess ? h : -1;
}

}  // namespace vlm
