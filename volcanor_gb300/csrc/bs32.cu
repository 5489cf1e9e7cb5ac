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
// Near field: one compare per target and ring (distance to the record's
// centre against its reach) and a warp vote select the records some lane of
// the warp may be near; for those the warp evaluates the record with a per-
// filament near-zone test that leaves near filaments out of the FP32 sum and
// appends one (target, record, filament) entry per near filament to a list
// (staged per warp in shared memory).  k_near64 evaluates the list
// coherently in FP64 into order-independent fixed-point accumulators, and
// k_near_apply adds them to the chunk partial sums, so the result does not
// depend on the order of the list.
#include <stdint.h>

#include <algorithm>
#include <atomic>

#include "vlm_bs.h"
#include "vlm_math.h"

namespace vlm {

namespace {

constexpr int kTPT = 2;         // targets per thread
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

// Near-list entries are staged per warp in shared memory and written to the
// global list in batches, one atomic per batch (a single global counter
// shared by every warp would otherwise put its latency on every append).
constexpr int kNearStage = 128;  // entries staged per warp

// Writes the warp's staged entries to the global list.
__device__ __forceinline__ void near_flush(NearPair* __restrict__ stage, int& staged, int lane, int* __restrict__ ctl,
                                           NearPair* __restrict__ near, int near_cap) {
  if (staged == 0) return;
  int base = 0;
  if (lane == 0) base = atomicAdd(ctl + 1, staged);
  base = __shfl_sync(kFull, base, 0);
  __syncwarp();
  for (int i = lane; i < staged; i += 32) {
    if (base + i < near_cap) near[base + i] = stage[i];
    else atomicExch(ctl, 3);
  }
  __syncwarp();
  staged = 0;
}

// Appends one entry per near filament (bits of msk, at most 4) of this
// warp's lanes.  Slots come from one ballot per filament index, no shuffles:
// filament k of lane l goes to P_k + popc(ballot_k & lanes below l), P_k the
// entries of the filament indices below k.
__device__ __forceinline__ void near_append(unsigned msk, int m, int q, int rec, int lane, int* __restrict__ ctl,
                                            NearPair* __restrict__ near, int near_cap, NearPair* __restrict__ stage,
                                            int& staged) {
  if (!__ballot_sync(kFull, msk != 0u)) return;
  const unsigned lt = (1u << lane) - 1u;
  unsigned bk[4];
  int pk[4], total = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    bk[k] = __ballot_sync(kFull, (msk >> k) & 1u);
    pk[k] = total;
    total += __popc(bk[k]);
  }
  int base;
  NearPair* dst;
  if (total <= kNearStage) {
    if (staged + total > kNearStage) near_flush(stage, staged, lane, ctl, near, near_cap);
    base = staged;
    dst = stage;
  } else {
    // more than a stage holds (up to 32 lanes x 4 filaments): straight out
    int b0 = 0;
    if (lane == 0) b0 = atomicAdd(ctl + 1, total);
    base = __shfl_sync(kFull, b0, 0);
    dst = nullptr;
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    if ((msk >> k) & 1u) {
      const int slot = base + pk[k] + __popc(bk[k] & lt);
      NearPair np;
      np.m = m;
      np.q = q;
      np.rec = rec;
      np.k = k;
      if (dst) dst[slot] = np;
      else if (slot < near_cap) near[slot] = np;
      else atomicExch(ctl, 3);
    }
  }
  __syncwarp();
  if (dst) staged += total;
}

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

// Adds the FP32 velocity of filament K (c_K -> c_{K+1}) at one target, from
// the corner vectors (r, 1/|r|) of its two ends.  CHECK: also tests the
// filament against its near zone (record fields [32+K], [36+K], [40+K]); a
// near filament is left out and reported through the return value.
template <int K, bool CHECK>
__device__ __forceinline__ bool fil_fp32(const float4* __restrict__ R4, const RecView& v, float rxk, float ryk,
                                         float rzk, float invk, float rxj, float ryj, float rzj, float invj, float& ax,
                                         float& ay, float& az, bool mine) {
  const float kx = fmaf(ryk, rzj, -rzk * ryj);
  const float ky = fmaf(rzk, rxj, -rxk * rzj);
  const float kz = fmaf(rxk, ryj, -ryk * rxj);
  const float c2 = fmaf(kx, kx, fmaf(ky, ky, kz * kz));
  // w (e.r_k/|r_k| - e.r_j/|r_j|) with the weight folded into e
  const float tt = fmaf(v.ex[K], rxk, fmaf(v.ey[K], ryk, v.ez[K] * rzk));
  const float d = fmaf(tt, invk, -(tt - v.eev[K]) * invj);
  float f = d * rsqrtf(fmaf(c2, c2, v.a4v[K]));
  bool nr = false;
  if (CHECK) {
    const float thr = reinterpret_cast<const float*>(R4)[32 + K];
    const float lo = reinterpret_cast<const float*>(R4)[36 + K];
    const float hi = reinterpret_cast<const float*>(R4)[40 + K];
    // exact zeros (target on the filament line) stay in the FP32 sum; only
    // a target inside the record's sphere can flag (so that which pairs are
    // near does not depend on the other lanes of its warp)
    nr = mine && c2 < thr && c2 > kS2Min && tt > lo && tt < hi;
    f = nr ? 0.f : f;
  }
  ax = fmaf(f, kx, ax);
  ay = fmaf(f, ky, ay);
  az = fmaf(f, kz, az);
  return nr;
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
// and rsqrt norms given).  CHECK: also tests every filament against its near
// zone, leaves the near ones out and returns their bit mask.
template <bool CHECK>
__device__ __forceinline__ unsigned ring_fp32(const float4* __restrict__ R4, const float (&rx)[4], const float (&ry)[4],
                                              const float (&rz)[4], const float (&inv)[4], float& ax, float& ay,
                                              float& az, bool mine = false) {
  const float4 q3 = R4[3], q4 = R4[4], q5 = R4[5];  // weighted edges
  const float4 ee = R4[6], a4 = R4[7];
  const float ex[4] = {q3.x, q3.w, q4.z, q5.y};
  const float ey[4] = {q3.y, q4.x, q4.w, q5.z};
  const float ez[4] = {q3.z, q4.y, q5.x, q5.w};
  const float eev[4] = {ee.x, ee.y, ee.z, ee.w};
  const float a4v[4] = {a4.x, a4.y, a4.z, a4.w};
  float thr[4], lo[4], hi[4];
  if (CHECK) {
    const float4 t = R4[8], l = R4[9], h = R4[10];
    thr[0] = t.x, thr[1] = t.y, thr[2] = t.z, thr[3] = t.w;
    lo[0] = l.x, lo[1] = l.y, lo[2] = l.z, lo[3] = l.w;
    hi[0] = h.x, hi[1] = h.y, hi[2] = h.z, hi[3] = h.w;
  }
  unsigned msk = 0u;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int j = (k + 1) & 3;
    const float kx = fmaf(ry[k], rz[j], -rz[k] * ry[j]);
    const float ky = fmaf(rz[k], rx[j], -rx[k] * rz[j]);
    const float kz = fmaf(rx[k], ry[j], -ry[k] * rx[j]);
    const float c2 = fmaf(kx, kx, fmaf(ky, ky, kz * kz));
    // w (e.r_k/|r_k| - e.r_j/|r_j|) with the weight folded into e
    const float tt = fmaf(ex[k], rx[k], fmaf(ey[k], ry[k], ez[k] * rz[k]));
    const float d = fmaf(tt, inv[k], -(tt - eev[k]) * inv[j]);
    float f = d * rsqrtf(fmaf(c2, c2, a4v[k]));
    if (CHECK) {
      // exact zeros (target on the filament line) stay in the FP32 sum
      // only a target inside the record's sphere can flag (so that which
      // pairs are near does not depend on the other lanes of its warp)
      const bool nr = mine && c2 < thr[k] && c2 > kS2Min && tt > lo[k] && tt < hi[k];
      f = nr ? 0.f : f;
      msk |= nr ? (1u << k) : 0u;
    }
    ax = fmaf(f, kx, ax);
    ay = fmaf(f, ky, ay);
    az = fmaf(f, kz, az);
  }
  return msk;
}

// One lattice-form record at one target: corners c0..c2 and edges 0 and 1,
// then c3 and the border edges 2 / 3 only where they carry circulation
// (a whole ring takes all four).  CHECK: returns the mask of near filaments.
template <bool CHECK>
__device__ __forceinline__ unsigned rec_lat(const float4* __restrict__ R4, const RecView& v, const float (&cx)[4],
                                            const float (&cy)[4], const float (&cz)[4], float px, float py, float pz,
                                            float& ax, float& ay, float& az, bool mine = false) {
  float rx[4], ry[4], rz[4], inv[4];
#pragma unroll
  for (int k = 0; k < 3; ++k) corner_vector(px, py, pz, cx[k], cy[k], cz[k], rx[k], ry[k], rz[k], inv[k]);
  unsigned msk = 0u;
  if (fil_fp32<0, CHECK>(R4, v, rx[0], ry[0], rz[0], inv[0], rx[1], ry[1], rz[1], inv[1], ax, ay, az, mine)) msk |= 1u;
  if (fil_fp32<1, CHECK>(R4, v, rx[1], ry[1], rz[1], inv[1], rx[2], ry[2], rz[2], inv[2], ax, ay, az, mine)) msk |= 2u;
  const bool t2 = v.a4v[2] >= 0.f, t3 = v.a4v[3] >= 0.f;
  if (t2 || t3) {
    corner_vector(px, py, pz, cx[3], cy[3], cz[3], rx[3], ry[3], rz[3], inv[3]);
    if (t2 && fil_fp32<2, CHECK>(R4, v, rx[2], ry[2], rz[2], inv[2], rx[3], ry[3], rz[3], inv[3], ax, ay, az, mine))
      msk |= 4u;
    if (t3 && fil_fp32<3, CHECK>(R4, v, rx[3], ry[3], rz[3], inv[3], rx[0], ry[0], rz[0], inv[0], ax, ay, az, mine))
      msk |= 8u;
  }
  return msk;
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
    fil_fp32<0, false>(R4, v, rx[u][0], ry[u][0], rz[u][0], inv[u][0], rx[u][1], ry[u][1], rz[u][1], inv[u][1], ax[u],
                       ay[u], az[u], false);
    fil_fp32<1, false>(R4, v, rx[u][1], ry[u][1], rz[u][1], inv[u][1], rx[u][2], ry[u][2], rz[u][2], inv[u][2], ax[u],
                       ay[u], az[u], false);
  }
  const bool t2 = v.a4v[2] >= 0.f, t3 = v.a4v[3] >= 0.f;
  if (t2 || t3) {
#pragma unroll
    for (int u = 0; u < T; ++u)
      corner_vector(px[u], py[u], pz[u], cx[3], cy[3], cz[3], rx[u][3], ry[u][3], rz[u][3], inv[u][3]);
    if (t2) {
#pragma unroll
      for (int u = 0; u < T; ++u)
        fil_fp32<2, false>(R4, v, rx[u][2], ry[u][2], rz[u][2], inv[u][2], rx[u][3], ry[u][3], rz[u][3], inv[u][3],
                           ax[u], ay[u], az[u], false);
    }
    if (t3) {
#pragma unroll
      for (int u = 0; u < T; ++u)
        fil_fp32<3, false>(R4, v, rx[u][3], ry[u][3], rz[u][3], inv[u][3], rx[u][0], ry[u][0], rz[u][0], inv[u][0],
                           ax[u], ay[u], az[u], false);
    }
  }
}

// One block = 8 consumer warps (256 threads x 2 targets) + 1 producer warp.
// The producer's lane 0 streams the chunk's records through kStages shared
// stages with bulk copies; consumers wait on a stage's FULL barrier, compute,
// and release it through its EMPTY barrier (one arrival per consumer warp).
constexpr int kStages = 4;
constexpr int kTileW = 128;                 // records per stage (24 KB)
constexpr int kConsumerWarps = 8;
constexpr int kBlockW = (kConsumerWarps + 1) * 32;
static_assert(kConsumerWarps * 32 * kTPT == kTargetsPerBlock32, "targets per block");

// LAT: the records are in lattice form (edges 2 and 3 marked when they carry
// no circulation); otherwise every record is evaluated as a whole ring.
template <bool NEAR, bool LAT>
__global__ void __launch_bounds__(kBlockW, 2) k_partial32(const float* __restrict__ rec32,
                                                         const Chunk* __restrict__ chunks,
                                                         const double* __restrict__ P, int M,
                                                         double* __restrict__ part, int* __restrict__ ctl,
                                                         NearPair* __restrict__ near, int near_cap) {
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
  __shared__ NearPair nstage_all[NEAR ? kConsumerWarps * kNearStage : 1];
  NearPair* nstage = nstage_all + (NEAR ? warp * kNearStage : 0);
  int staged = 0;
  int mt[kTPT];
  bool valid[kTPT];
  float px[kTPT], py[kTPT], pz[kTPT];
  double acc64[kTPT][3];
#pragma unroll
  for (int u = 0; u < kTPT; ++u) {
    // runs of 256 targets per u: a warp's targets are two runs of 32
    // consecutive ones (measured 1-2 % faster than one run of 64)
    mt[u] = blockIdx.x * kTargetsPerBlock32 + u * (32 * kConsumerWarps) + tid;
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
    if (ok) {
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
        if (NEAR) {
          // candidate test first (distance to the record's centre against
          // its reach), so that only one target's corner vectors are live in
          // either path below
          const float4 zone = R4[11];  // reach^2, centre of the near zones
          bool candu[kTPT], cand = false;
#pragma unroll
          for (int u = 0; u < kTPT; ++u) {
            const float dx = px[u] - zone.y, dy = py[u] - zone.z, dz = pz[u] - zone.w;
            candu[u] = valid[u] && fmaf(dx, dx, fmaf(dy, dy, dz * dz)) < zone.x;
            cand |= candu[u];
          }
          if (__any_sync(kFull, cand)) {
            // some lane of the warp is within reach of this record
            const int rec = ch.rec_begin + t * kTileW + r;
            if (LAT) {
              RecView v;
              load_view(R4, v);
              unsigned msk[kTPT];
#pragma unroll
              for (int u = 0; u < kTPT; ++u)
                msk[u] = rec_lat<true>(R4, v, cx, cy, cz, px[u], py[u], pz[u], ax[u], ay[u], az[u], candu[u]);
#pragma unroll
              for (int u = 0; u < kTPT; ++u) near_append(msk[u], mt[u], q, rec, lane, ctl, near, near_cap, nstage, staged);
            } else {
#pragma unroll
              for (int u = 0; u < kTPT; ++u) {
                float rx[4], ry[4], rz[4], inv[4];
                corner_vectors(px[u], py[u], pz[u], cx, cy, cz, rx, ry, rz, inv);
                const unsigned msk = ring_fp32<true>(R4, rx, ry, rz, inv, ax[u], ay[u], az[u], candu[u]);
                near_append(msk, mt[u], q, rec, lane, ctl, near, near_cap, nstage, staged);
              }
            }
            continue;
          }
          if (LAT) {
            rec_lat_pair<kTPT>(R4, cx, cy, cz, px, py, pz, ax, ay, az);
            continue;
          }
#pragma unroll
          for (int u = 0; u < kTPT; ++u) {
            float rx[4], ry[4], rz[4], inv[4];
            corner_vectors(px[u], py[u], pz[u], cx, cy, cz, rx, ry, rz, inv);
            ring_fp32<false>(R4, rx, ry, rz, inv, ax[u], ay[u], az[u]);
          }
        } else if (!LAT) {
          // both targets' corner vectors first: more independent work in flight
          float rx[kTPT][4], ry[kTPT][4], rz[kTPT][4], inv[kTPT][4];
#pragma unroll
          for (int u = 0; u < kTPT; ++u) corner_vectors(px[u], py[u], pz[u], cx, cy, cz, rx[u], ry[u], rz[u], inv[u]);
#pragma unroll
          for (int u = 0; u < kTPT; ++u) ring_fp32<false>(R4, rx[u], ry[u], rz[u], inv[u], ax[u], ay[u], az[u]);
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
  if (NEAR) near_flush(nstage, staged, lane, ctl, near, near_cap);
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

// FP64 evaluation of the listed near-field filament-target pairs (filament
// velocity times the circulation), added in fixed point to the accumulators
// of their (chunk, target).
__global__ void k_near64(const NearPair* __restrict__ near, int* __restrict__ ctl, int near_cap,
                         const double* __restrict__ rec64, const double* __restrict__ ew,
                         const double* __restrict__ P, int M, unsigned long long* __restrict__ nacc) {
  const int n = min(ctl[1], near_cap);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const NearPair np = near[i];
    const double* R = rec64 + (size_t)np.rec * kRec64;
    const d3 p = mk3(P[3 * (size_t)np.m], P[3 * (size_t)np.m + 1], P[3 * (size_t)np.m + 2]);
    d3 v;
    if ((int)R[17] & REC_FIL) {
      v = fil_near64(p, mk3(R[0], R[1], R[2]), mk3(R[3], R[4], R[5]), R[12]);
    } else {
      const int k = np.k, j = (k + 1) & 3;
      v = fil_near64(p, mk3(R[3 * k], R[3 * k + 1], R[3 * k + 2]), mk3(R[3 * j], R[3 * j + 1], R[3 * j + 2]),
                     R[12 + k]);
    }
    v = v * (ew ? ew[4 * (size_t)np.rec + np.k] : R[16]);
    unsigned long long* o = nacc + ((size_t)np.q * M + np.m) * 3;
    const double c[3] = {v.x, v.y, v.z};
    for (int a = 0; a < 3; ++a) {
      if (!(fabs(c[a]) < kNearMax)) {
        atomicExch(ctl, 4);
        continue;
      }
      atomicAdd(o + a, (unsigned long long)__double2ll_rn(c[a] * kNearScale));
    }
  }
}

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
  // centre of the near zones: mean of the active filaments' end points
  double mx = 0.0, my = 0.0, mz = 0.0;
  for (int k = 0; k < 4; ++k) {
    mx += cx[k];
    my += cy[k];
    mz += cz[k];
  }
  mx *= 0.25;
  my *= 0.25;
  mz *= 0.25;
  float reach = 0.f;
  bool anyNear = false;
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
    if (on) {
      anyNear = true;
      // farthest point of this filament's near zone from the centre
      const float ax = (float)(cx[k] - mx), ay = (float)(cy[k] - my), az = (float)(cz[k] - mz);
      const float bx = (float)(cx[j] - mx), by = (float)(cy[j] - my), bz = (float)(cz[j] - mz);
      const float da = sqrtf(fmaf(ax, ax, fmaf(ay, ay, az * az)));
      const float db = sqrtf(fmaf(bx, bx, fmaf(by, by, bz * bz)));
      reach = fmaxf(reach, fmaxf(da, db) + nf * rv[k]);
    }
  }
  // margin for the FP32 rounding of corners and of this sum
  const float r = reach * 1.0001f + 1e-6f;
  o[44] = anyNear ? r * r : -1.f;
  o[45] = (float)mx;
  o[46] = (float)my;
  o[47] = (float)mz;
}

}  // namespace

void launch_pack32(const double* rec64, int nrec, double near_factor, float* rec32, cudaStream_t s,
                   const double* ew) {
  if (nrec <= 0) return;
  count_launch();
  k_pack32<<<(nrec + 255) / 256, 256, 0, s>>>(rec64, nrec, near_factor, rec32, ew);
}

void launch_partial32(const float* rec32, const double* rec64, const Chunk* chunks, int nchunks, const double* P,
                      int M, double* part, int* ctl, NearPair* near, int near_cap, long long* nacc, cudaStream_t s,
                      const double* ew) {
  if (M <= 0 || nchunks <= 0) return;
  const int smem = kStages * kTileW * kRec32 * (int)sizeof(float);
  // the dynamic shared-memory opt-in is per device; set it once on each
  static std::atomic<bool> attr[64];
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64 || !attr[dev].load(std::memory_order_acquire)) {
    cudaFuncSetAttribute(k_partial32<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaFuncSetAttribute(k_partial32<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaFuncSetAttribute(k_partial32<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaFuncSetAttribute(k_partial32<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (dev >= 0 && dev < 64) attr[dev].store(true, std::memory_order_release);
  }
  dim3 grid((M + kTargetsPerBlock32 - 1) / kTargetsPerBlock32, nchunks);
  count_launch();
  if (near) {
    if (ew) k_partial32<true, true><<<grid, kBlockW, smem, s>>>(rec32, chunks, P, M, part, ctl, near, near_cap);
    else k_partial32<true, false><<<grid, kBlockW, smem, s>>>(rec32, chunks, P, M, part, ctl, near, near_cap);
    const int sms = device_sm_count();
    count_launch();
    k_near64<<<4 * sms, 128, 0, s>>>(near, ctl, near_cap, rec64, ew, P, M,
                                     reinterpret_cast<unsigned long long*>(nacc));
    const size_t n = (size_t)M * nchunks * 3;
    count_launch();
    k_near_apply<<<(unsigned)std::min<size_t>((n + 255) / 256, (size_t)8 * sms), 256, 0, s>>>(part, nacc, n);
  } else if (ew) {
    k_partial32<false, true><<<grid, kBlockW, smem, s>>>(rec32, chunks, P, M, part, ctl, near, near_cap);
  } else {
    k_partial32<false, false><<<grid, kBlockW, smem, s>>>(rec32, chunks, P, M, part, ctl, near, near_cap);
  }
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

int partial32_slots() {
  static std::atomic<int> cache[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 2 * kPlanSmsWithoutDevice;
  if (!cache[dev]) {
    int per = 0;
    const int smem = kStages * kTileW * kRec32 * (int)sizeof(float);
    cudaFuncSetAttribute(k_partial32<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_partial32<true, false>, kBlockW, smem);
    cache[dev] = device_sm_count() * std::max(1, per);
  }
  return cache[dev];
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
