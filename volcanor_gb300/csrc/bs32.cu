// FP32 Biot-Savart N-body kernel with FP64 accumulation and an FP64
// near-field path, for sm_103a.  Compiled with -ftz=true.
//
// Layout: one block = 256 threads x 2 targets per thread, one chunk of source
// records.  Source records (48 floats, 192 B) stream through a two-stage
// shared-memory pipeline filled by bulk asynchronous copies (cp.async.bulk,
// completion tracked on an mbarrier, every wait bounded); each staged record
// is read with broadcast LDS.128 and evaluated for both targets of a thread.
//
// Per target and ring: 4 corner vectors r_k = P - c_k with rsqrt norms, then
// per filament k -> j = k+1 the Vatistas n=2 kernel (src/classdef.f90:476-503)
//   v = (r_k x r_j) w_k (e.r_k/|r_k| - e.r_j/|r_j|) / sqrt((rvc|e|)^4 + |r_k x r_j|^4)
// with e.r_j = e.r_k - |e|^2 and the source-only terms hoisted into the
// record (w_k = gam/4pi).  A target on the filament line has r_k x r_j = 0
// exactly, so its (finite) factor contributes exactly zero; the reference's
// eps^2 cut-off needs no separate test.  FP32 partial sums are promoted to
// the FP64 accumulator after every tile.
//
// Near field: one compare per ring (distance to corner 0 against the
// record's reach) selects the rare candidates; their filaments inside
// near_factor core radii of the segment are left out of the FP32 sum and
// appended to a list that k_near64 evaluates coherently in FP64.
#include <stdint.h>

#include "vlm_bs.h"
#include "vlm_math.h"

namespace vlm {

namespace {

constexpr int kThreads32 = 256;
constexpr int kTPT = 2;         // targets per thread
constexpr int kTile32 = 128;    // records per stage (128 x 192 B = 24 KB)
constexpr uint32_t kWaitLimit = 1u << 22;
constexpr float kS2Min = 1e-30f;
constexpr float kDenMin = 1.17549435e-38f;

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
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  const uint32_t a = smem_u32(bar);
  for (uint32_t i = 0; i < kWaitLimit; ++i) {
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

template <bool NEAR>
__global__ void __launch_bounds__(kThreads32, 2) k_partial32(const float* __restrict__ rec32,
                                                            const Chunk* __restrict__ chunks,
                                                            const double* __restrict__ P, int M,
                                                            double* __restrict__ part, int* __restrict__ ctl,
                                                            NearPair* __restrict__ near, int near_cap) {
  extern __shared__ __align__(16) float stage[];  // [2][kTile32 * kRec32]
  __shared__ __align__(8) uint64_t bars[2];
  const int q = blockIdx.y;
  const Chunk ch = chunks[q];
  const int tid = threadIdx.x;

  int mt[kTPT];
  float px[kTPT], py[kTPT], pz[kTPT];
  double acc64[kTPT][3];
#pragma unroll
  for (int u = 0; u < kTPT; ++u) {
    mt[u] = (blockIdx.x * kTPT + u) * kThreads32 + tid;
    const int mm = mt[u] < M ? mt[u] : M - 1;
    px[u] = (float)P[3 * (size_t)mm];
    py[u] = (float)P[3 * (size_t)mm + 1];
    pz[u] = (float)P[3 * (size_t)mm + 2];
    acc64[u][0] = acc64[u][1] = acc64[u][2] = 0.0;
  }

  const int ntiles = (ch.rec_count + kTile32 - 1) / kTile32;
  if (tid == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  auto issue = [&](int t) {
    const int n = min(kTile32, ch.rec_count - t * kTile32);
    const uint32_t bytes = (uint32_t)n * kRec32 * 4u;
    uint64_t* bar = &bars[t & 1];
    mbar_expect_tx(bar, bytes);
    bulk_g2s(stage + (t & 1) * kTile32 * kRec32, rec32 + (size_t)(ch.rec_begin + t * kTile32) * kRec32, bytes, bar);
  };
  // pend[b]: tile whose copy into stage b thread 0 has not yet seen complete
  int pend[2] = {-1, -1};
  if (tid == 0 && ntiles > 0) {
    issue(0);
    pend[0] = 0;
  }
  bool ok = true;
  for (int t = 0; t < ntiles; ++t) {
    if (tid == 0 && ok && t + 1 < ntiles) {
      issue(t + 1);
      pend[(t + 1) & 1] = t + 1;
    }
    if (ok && !mbar_wait(&bars[t & 1], (t >> 1) & 1)) {
      ok = false;
      atomicExch(ctl, 1);
    }
    if (ok && tid == 0) pend[t & 1] = -1;
    if (ok) {
      const int n = min(kTile32, ch.rec_count - t * kTile32);
      const float* tile = stage + (t & 1) * kTile32 * kRec32;
      float ax[kTPT], ay[kTPT], az[kTPT];
#pragma unroll
      for (int u = 0; u < kTPT; ++u) ax[u] = ay[u] = az[u] = 0.f;
#pragma unroll 1
      for (int r = 0; r < n; ++r) {
        const float4* R4 = reinterpret_cast<const float4*>(tile + r * kRec32);
        const float4 q0 = R4[0], q1 = R4[1], q2 = R4[2];  // corners
        const float4 q3 = R4[3], q4 = R4[4], q5 = R4[5];  // edges
        const float4 ee = R4[6], a4 = R4[7], w = R4[9];
        const float cx[4] = {q0.x, q0.w, q1.z, q2.y};
        const float cy[4] = {q0.y, q1.x, q1.w, q2.z};
        const float cz[4] = {q0.z, q1.y, q2.x, q2.w};
        const float ex[4] = {q3.x, q3.w, q4.z, q5.y};
        const float ey[4] = {q3.y, q4.x, q4.w, q5.z};
        const float ez[4] = {q3.z, q4.y, q5.x, q5.w};
        const float eev[4] = {ee.x, ee.y, ee.z, ee.w};
        const float a4v[4] = {a4.x, a4.y, a4.z, a4.w};
        const float wv[4] = {w.x, w.y, w.z, w.w};
        float reach2 = -1.f;
        if (NEAR) reach2 = tile[r * kRec32 + 44];
#pragma unroll
        for (int u = 0; u < kTPT; ++u) {
          float rx[4], ry[4], rz[4], inv[4], s0 = 0.f;
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            rx[k] = px[u] - cx[k];
            ry[k] = py[u] - cy[k];
            rz[k] = pz[u] - cz[k];
            const float s = fmaf(rx[k], rx[k], fmaf(ry[k], ry[k], rz[k] * rz[k]));
            if (k == 0) s0 = s;
            inv[k] = rsqrtf(fmaxf(s, kS2Min));
          }
          const bool cand = NEAR && s0 < reach2 && mt[u] < M;
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const int j = (k + 1) & 3;
            const float kx = fmaf(ry[k], rz[j], -rz[k] * ry[j]);
            const float ky = fmaf(rz[k], rx[j], -rx[k] * rz[j]);
            const float kz = fmaf(rx[k], ry[j], -ry[k] * rx[j]);
            const float c2 = fmaf(kx, kx, fmaf(ky, ky, kz * kz));
            const float tt = fmaf(ex[k], rx[k], fmaf(ey[k], ry[k], ez[k] * rz[k]));
            const float d = fmaf(tt, inv[k], -(tt - eev[k]) * inv[j]);
            const float den = fmaxf(fmaf(c2, c2, a4v[k]), kDenMin);
            float f = wv[k] * d * rsqrtf(den);
            if (NEAR && cand) {
              const float nfk = tile[r * kRec32 + 32 + k];
              const float slk = tile[r * kRec32 + 40 + k];
              if (c2 < nfk && c2 > kS2Min && tt > -slk && tt < eev[k] + slk) {
                f = 0.f;
                const int slot = atomicAdd(ctl + 1, 1);
                if (slot < near_cap) {
                  NearPair np;
                  np.m = mt[u];
                  np.q = q;
                  np.rec = ch.rec_begin + t * kTile32 + r;
                  np.k = k;
                  near[slot] = np;
                } else {
                  atomicExch(ctl, 3);
                }
              }
            }
            ax[u] = fmaf(f, kx, ax[u]);
            ay[u] = fmaf(f, ky, ay[u]);
            az[u] = fmaf(f, kz, az[u]);
          }
        }
      }
#pragma unroll
      for (int u = 0; u < kTPT; ++u) {
        acc64[u][0] += (double)ax[u];
        acc64[u][1] += (double)ay[u];
        acc64[u][2] += (double)az[u];
      }
    }
    __syncthreads();
  }
  if (tid == 0) {
    // a copy issued by this thread but never seen complete may still be
    // writing the stage buffers: wait for it (bounded) before the block exits
    for (int b = 0; b < 2; ++b)
      if (pend[b] >= 0 && !mbar_wait(&bars[b], (pend[b] >> 1) & 1)) atomicExch(ctl, 2);
  }
#pragma unroll
  for (int u = 0; u < kTPT; ++u) {
    if (mt[u] < M) {
      double* o = part + ((size_t)q * M + mt[u]) * 3;
      o[0] = acc64[u][0];
      o[1] = acc64[u][1];
      o[2] = acc64[u][2];
    }
  }
}

// FP64 evaluation of the listed near-field pairs (reference arithmetic),
// added to the partial sums of their chunks.
__global__ void k_near64(const NearPair* __restrict__ near, const int* __restrict__ ctl, int near_cap,
                         const double* __restrict__ rec64, const double* __restrict__ P, int M,
                         double* __restrict__ part) {
  const int n = min(ctl[1], near_cap);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const NearPair np = near[i];
    const double* R = rec64 + (size_t)np.rec * kRec64;
    const d3 p = mk3(P[3 * (size_t)np.m], P[3 * (size_t)np.m + 1], P[3 * (size_t)np.m + 2]);
    d3 v;
    if ((int)R[17] & REC_FIL) {
      v = fil_vind64(p, mk3(R[0], R[1], R[2]), mk3(R[3], R[4], R[5]), R[12]);
    } else {
      const int k = np.k, j = (k + 1) & 3;
      v = vf_vind64(make_corner64(p, mk3(R[3 * k], R[3 * k + 1], R[3 * k + 2])),
                    make_corner64(p, mk3(R[3 * j], R[3 * j + 1], R[3 * j + 2])), R[12 + k]);
    }
    v = v * R[16];
    double* o = part + ((size_t)np.q * M + np.m) * 3;
    atomicAdd(o, v.x);
    atomicAdd(o + 1, v.y);
    atomicAdd(o + 2, v.z);
  }
}

__global__ void k_pack32(const double* __restrict__ rec64, int nrec, double near_factor, float* __restrict__ rec32) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nrec) return;
  const double* R = rec64 + (size_t)i * kRec64;
  float* o = rec32 + (size_t)i * kRec32;
  const int flags = (int)R[17];
  const double g = R[16];
  const bool skipped = (flags & REC_SKIP) && !(fabs(g) > kEps);
  d3 c[4];
  double rv[4];
  bool act[4];
  if (flags & REC_FIL) {
    c[0] = mk3(R[0], R[1], R[2]);
    c[1] = mk3(R[3], R[4], R[5]);
    c[2] = c[1];
    c[3] = c[0];
    rv[0] = R[12];
    rv[1] = rv[2] = rv[3] = 0.0;
    act[0] = true;
    act[1] = act[2] = act[3] = false;
  } else {
    for (int k = 0; k < 4; ++k) {
      c[k] = mk3(R[3 * k], R[3 * k + 1], R[3 * k + 2]);
      rv[k] = R[12 + k];
      act[k] = true;
    }
  }
  const double w = g * kInv4Pi;
  double reach = 0.0;
  bool anyNear = false;
  for (int k = 0; k < 4; ++k) {
    const d3 e = c[(k + 1) & 3] - c[k];
    const double ee = dot3(e, e);
    const double s = rv[k] * sqrt(ee);
    o[3 * k] = (float)c[k].x;
    o[3 * k + 1] = (float)c[k].y;
    o[3 * k + 2] = (float)c[k].z;
    o[12 + 3 * k] = (float)e.x;
    o[12 + 3 * k + 1] = (float)e.y;
    o[12 + 3 * k + 2] = (float)e.z;
    o[24 + k] = (float)ee;
    o[28 + k] = (float)pow4(s);
    const bool on = act[k] && !skipped && near_factor > 0.0;
    const double nfs = near_factor * s;
    o[32 + k] = on ? (float)(nfs * nfs) : -1.f;
    o[36 + k] = (act[k] && !skipped) ? (float)w : 0.f;
    o[40 + k] = on ? (float)nfs : 0.f;
    if (on) {
      anyNear = true;
      // farthest point of this filament's near zone from corner 0
      reach = fmax(reach, fmax(norm3(c[k] - c[0]), norm3(c[(k + 1) & 3] - c[0])) + near_factor * rv[k]);
    }
  }
  const double r = reach * 1.0001 + 1e-6;
  o[44] = anyNear ? (float)(r * r) : -1.f;
  o[45] = o[46] = o[47] = 0.f;
}

}  // namespace

void launch_pack32(const double* rec64, int nrec, double near_factor, float* rec32, cudaStream_t s) {
  if (nrec <= 0) return;
  count_launch();
  k_pack32<<<(nrec + 255) / 256, 256, 0, s>>>(rec64, nrec, near_factor, rec32);
}

void launch_partial32(const float* rec32, const double* rec64, const Chunk* chunks, int nchunks, const double* P,
                      int M, double* part, int* ctl, NearPair* near, int near_cap, cudaStream_t s) {
  if (M <= 0 || nchunks <= 0) return;
  const int smem = 2 * kTile32 * kRec32 * (int)sizeof(float);
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_partial32<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    cudaFuncSetAttribute(k_partial32<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    attr = true;
  }
  dim3 grid((M + kTPT * kThreads32 - 1) / (kTPT * kThreads32), nchunks);
  count_launch();
  if (near) {
    k_partial32<true><<<grid, kThreads32, smem, s>>>(rec32, chunks, P, M, part, ctl, near, near_cap);
    count_launch();
    k_near64<<<4 * 152, 128, 0, s>>>(near, ctl, near_cap, rec64, P, M, part);
  } else {
    k_partial32<false><<<grid, kThreads32, smem, s>>>(rec32, chunks, P, M, part, ctl, near, near_cap);
  }
}

}  // namespace vlm
