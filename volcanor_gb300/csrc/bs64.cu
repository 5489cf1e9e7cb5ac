// FP64 Biot-Savart partial sums in the reference's arithmetic, the chunk
// combiner, and the chunk-table builder.
//
// Compiled with -fmad=false: every multiply and add rounds separately, as in
// the oracle (built with -ffp-contract=off), so a chunked FP64 evaluation
// equals the oracle's evaluation with the same chunk size bit for bit.
#include <algorithm>
#include <atomic>

#include "vlm_bs.h"
#include "vlm_math.h"

namespace vlm {

namespace {

constexpr int kThreads64 = 128;  // targets per block
constexpr int kTile64 = 32;      // records staged per shared-memory tile

// One block = kThreads64 targets x one chunk.  Each thread sums its target's
// contributions over the chunk sequentially from zero (blade_vind_bywing /
// blade_vind_bywake accumulation, src/classdef.f90:1342-1513).
__global__ void __launch_bounds__(kThreads64) k_partial64(const double* __restrict__ rec,
                                                         const Chunk* __restrict__ chunks,
                                                         const double* __restrict__ P, int M,
                                                         double* __restrict__ part) {
  __shared__ double tile[kTile64 * kRec64];
  const Chunk ch = chunks[blockIdx.y];
  const int m = blockIdx.x * kThreads64 + threadIdx.x;
  const bool active = m < M;
  d3 p = zero3();
  if (active) p = mk3(P[3 * (size_t)m], P[3 * (size_t)m + 1], P[3 * (size_t)m + 2]);
  d3 acc = zero3();
  for (int t0 = 0; t0 < ch.rec_count; t0 += kTile64) {
    const int nt = min(kTile64, ch.rec_count - t0);
    __syncthreads();
    const double* src = rec + (size_t)(ch.rec_begin + t0) * kRec64;
    for (int k = threadIdx.x; k < nt * kRec64; k += kThreads64) tile[k] = src[k];
    __syncthreads();
    if (!active) continue;
    for (int r = 0; r < nt; ++r) {
      const double* R = tile + r * kRec64;
      const int flags = (int)R[17];
      const double g = R[16];
      if ((flags & REC_SKIP) && !(fabs(g) > kEps)) continue;
      d3 v;
      if (flags & REC_FIL) {
        v = fil_vind64(p, mk3(R[0], R[1], R[2]), mk3(R[3], R[4], R[5]), R[12]);
      } else {
        d3 c[4] = {mk3(R[0], R[1], R[2]), mk3(R[3], R[4], R[5]), mk3(R[6], R[7], R[8]), mk3(R[9], R[10], R[11])};
        v = vr_vind64(p, c, R + 12);
      }
      acc = acc + v * g;
    }
  }
  if (active) {
    double* o = part + ((size_t)blockIdx.y * M + m) * 3;
    o[0] = acc.x;
    o[1] = acc.y;
    o[2] = acc.z;
  }
}

__global__ void k_combine(const double* __restrict__ part, int M, const Group* __restrict__ groups, int ngroups,
                          int mode, double* __restrict__ out) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= M) return;
  d3 wing = zero3(), wake = zero3();
  for (int g = 0; g < ngroups; ++g) {
    const Group G = groups[g];
    d3 gs = zero3();
    int q = G.chunk_begin;
    const int qe = G.chunk_begin + G.chunk_count;
    // loads issued 16 at a time (the adds stay in chunk order): a collocation-
    // point evaluation has few targets and hundreds of chunks
    constexpr int kB = 16;
    for (; q + kB <= qe; q += kB) {
      d3 buf[kB];
#pragma unroll
      for (int i = 0; i < kB; ++i) {
        const double* pp = part + ((size_t)(q + i) * M + m) * 3;
        buf[i] = mk3(pp[0], pp[1], pp[2]);
      }
#pragma unroll
      for (int i = 0; i < kB; ++i) gs = gs + buf[i];
    }
    for (; q < qe; ++q) {
      const double* pp = part + ((size_t)q * M + m) * 3;
      gs = gs + mk3(pp[0], pp[1], pp[2]);
    }
    if (G.kind == 0) wing = wing + gs;
    else wake = wake + gs;
  }
  d3 v;
  if (mode == 0) v = zero3() + (wing + wake);
  else if (mode == 1) v = wake;
  else v = wing + wake;
  out[3 * (size_t)m] = v.x;
  out[3 * (size_t)m + 1] = v.y;
  out[3 * (size_t)m + 2] = v.z;
}

// Unordered combine (FP32 paths, whose summation order is free): G lanes
// per target (G a power of two <= 32); lane l of a target adds chunk
// partials l, l + G, ... of a group in order, then a butterfly over the G
// lanes.  The tree has a fixed shape, so the result is reproducible run to
// run; the serial chain is chunks/G adds long.
__global__ void k_combine_tree(const double* __restrict__ part, int M, const Group* __restrict__ groups, int ngroups,
                               int mode, int G, double* __restrict__ out) {
  const size_t gt = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const int m = (int)(gt / G), l = (int)(gt % G);
  const bool live = m < M;  // dead lanes still take part in the shuffles
  d3 wing = zero3(), wake = zero3();
  for (int g = 0; g < ngroups; ++g) {
    const Group G_ = groups[g];
    d3 gs = zero3();
    if (live)
      for (int q = G_.chunk_begin + l; q < G_.chunk_begin + G_.chunk_count; q += G) {
        const double* pp = part + ((size_t)q * M + m) * 3;
        gs = gs + mk3(pp[0], pp[1], pp[2]);
      }
    for (int o = G >> 1; o > 0; o >>= 1) {
      gs.x = gs.x + __shfl_xor_sync(0xffffffffu, gs.x, o, G);
      gs.y = gs.y + __shfl_xor_sync(0xffffffffu, gs.y, o, G);
      gs.z = gs.z + __shfl_xor_sync(0xffffffffu, gs.z, o, G);
    }
    if (G_.kind == 0) wing = wing + gs;
    else wake = wake + gs;
  }
  if (live && l == 0) {
    d3 v;
    if (mode == 0) v = zero3() + (wing + wake);
    else if (mode == 1) v = wake;
    else v = wing + wake;
    out[3 * (size_t)m] = v.x;
    out[3 * (size_t)m + 1] = v.y;
    out[3 * (size_t)m + 2] = v.z;
  }
}

// Coupled rotors: the groups carry the index of the sum they belong to
// (Group::term, non-decreasing).  mode 0 (wake nodes, src/main.f90:808-827):
// v = 0, then v = v + (wing_t + wake_t) for every term in turn, one term per
// source rotor (libCommon.f90:114-211 adds a rotor's wing and wake);
// out[m] = v.  mode 3 (collocation points, src/main.f90:549-561):
// out[t][m] = 0 + the term's groups in order, one per-rotor wake or wing
// sum each, which the RHS adds to velCP in turn.  With a single term, mode 0
// equals k_combine's mode 0 bit for bit.
__device__ __forceinline__ void term_done(int mode, int t, int M, int m, d3& v, d3& wing, d3& wake, d3& ts,
                                          double* out) {
  if (mode == 0) {
    v = v + (wing + wake);
  } else {
    double* o = out + 3 * ((size_t)t * M + m);
    o[0] = ts.x;
    o[1] = ts.y;
    o[2] = ts.z;
  }
  wing = wake = ts = zero3();
}

__global__ void k_combine_terms(const double* __restrict__ part, int M, const Group* __restrict__ groups,
                                int ngroups, int mode, double* __restrict__ out) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= M || ngroups <= 0) return;
  d3 v = zero3(), wing = zero3(), wake = zero3(), ts = zero3();
  int t = groups[0].term;
  for (int g = 0; g < ngroups; ++g) {
    const Group G = groups[g];
    if (G.term != t) {
      term_done(mode, t, M, m, v, wing, wake, ts, out);
      t = G.term;
    }
    d3 gs = zero3();
    for (int q = G.chunk_begin; q < G.chunk_begin + G.chunk_count; ++q) {
      const double* pp = part + ((size_t)q * M + m) * 3;
      gs = gs + mk3(pp[0], pp[1], pp[2]);
    }
    if (mode == 0) {
      if (G.kind == 0) wing = wing + gs;
      else wake = wake + gs;
    } else {
      ts = ts + gs;
    }
  }
  term_done(mode, t, M, m, v, wing, wake, ts, out);
  if (mode == 0) {
    out[3 * (size_t)m] = v.x;
    out[3 * (size_t)m + 1] = v.y;
    out[3 * (size_t)m + 2] = v.z;
  }
}

// The same with k_combine_tree's fixed-shape tree per group (FP32 paths).
__global__ void k_combine_terms_tree(const double* __restrict__ part, int M, const Group* __restrict__ groups,
                                     int ngroups, int mode, int G, double* __restrict__ out) {
  const size_t gt = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  const int m = (int)(gt / G), l = (int)(gt % G);
  const bool live = m < M;
  if (ngroups <= 0) return;
  d3 v = zero3(), wing = zero3(), wake = zero3(), ts = zero3();
  int t = groups[0].term;
  for (int g = 0; g < ngroups; ++g) {
    const Group G_ = groups[g];
    if (G_.term != t) {
      if (live && l == 0) term_done(mode, t, M, m, v, wing, wake, ts, out);
      t = G_.term;
    }
    d3 gs = zero3();
    if (live)
      for (int q = G_.chunk_begin + l; q < G_.chunk_begin + G_.chunk_count; q += G) {
        const double* pp = part + ((size_t)q * M + m) * 3;
        gs = gs + mk3(pp[0], pp[1], pp[2]);
      }
    for (int o = G >> 1; o > 0; o >>= 1) {
      gs.x = gs.x + __shfl_xor_sync(0xffffffffu, gs.x, o, G);
      gs.y = gs.y + __shfl_xor_sync(0xffffffffu, gs.y, o, G);
      gs.z = gs.z + __shfl_xor_sync(0xffffffffu, gs.z, o, G);
    }
    if (mode == 0) {
      if (G_.kind == 0) wing = wing + gs;
      else wake = wake + gs;
    } else {
      ts = ts + gs;
    }
  }
  if (live && l == 0) {
    term_done(mode, t, M, m, v, wing, wake, ts, out);
    if (mode == 0) {
      out[3 * (size_t)m] = v.x;
      out[3 * (size_t)m + 1] = v.y;
      out[3 * (size_t)m + 2] = v.z;
    }
  }
}

__global__ void k_rings_to_rec64(const double* __restrict__ corners, const double* __restrict__ rvc,
                                 const double* __restrict__ gam, int64_t N, double* __restrict__ rec) {
  const int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (n >= N) return;
  double* R = rec + n * kRec64;
  for (int k = 0; k < 12; ++k) R[k] = corners[n * 12 + k];
  for (int k = 0; k < 4; ++k) R[12 + k] = rvc[n * 4 + k];
  R[16] = gam[n];
  R[17] = 0.0;
}

// Single filaments fc1 -> fc2 (vf_vind, src/classdef.f90:476-503) as
// REC_FIL records; no |gam| skip (gridgen sums every filament,
// src/gridgen.f90:128-136).
__global__ void k_fils_to_rec64(const double* __restrict__ fc, const double* __restrict__ rvc,
                                const double* __restrict__ gam, int64_t N, double* __restrict__ rec) {
  const int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (n >= N) return;
  double* R = rec + n * kRec64;
  for (int k = 0; k < 6; ++k) R[k] = fc[n * 6 + k];
  for (int k = 6; k < 12; ++k) R[k] = 0.0;
  R[12] = rvc[n];
  R[13] = R[14] = R[15] = 0.0;
  R[16] = gam[n];
  R[17] = (double)REC_FIL;
}

}  // namespace

static std::atomic<long> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void count_launches(long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
long launch_count() { return g_launches.load(); }

int build_chunks(Group* groups, int ngroups, int chunk_size, Chunk* chunks, int cap) {
  int nq = 0;
  for (int g = 0; g < ngroups; ++g) {
    Group& G = groups[g];
    G.chunk_begin = nq;
    G.chunk_count = 0;
    if (G.rec_count <= 0) continue;
    const int C = chunk_size > 0 ? chunk_size : G.rec_count;
    for (int r = 0; r < G.rec_count; r += C) {
      if (nq >= cap) return -1;
      chunks[nq].rec_begin = G.rec_begin + r;
      chunks[nq].rec_count = std::min(C, G.rec_count - r);
      ++nq;
      ++G.chunk_count;
    }
  }
  return nq;
}

void launch_partial64(const double* rec, const Chunk* chunks, int nchunks, const double* P, int M, double* part,
                      cudaStream_t s) {
  if (M <= 0 || nchunks <= 0) return;
  dim3 grid((M + kThreads64 - 1) / kThreads64, nchunks);
  count_launch();
  k_partial64<<<grid, kThreads64, 0, s>>>(rec, chunks, P, M, part);
}

void launch_combine(const double* part, int M, const Group* groups, int ngroups, int mode, double* out,
                    cudaStream_t s) {
  if (M <= 0) return;
  count_launch();
  k_combine<<<(M + 127) / 128, 128, 0, s>>>(part, M, groups, ngroups, mode, out);
}

void launch_combine_unordered(const double* part, int M, const Group* groups, int ngroups, int max_chunks, int mode,
                              double* out, cudaStream_t s) {
  if (M <= 0) return;
  // about 8 chunk partials per lane, at most a warp per target
  int G = 1;
  while (G < 32 && G * 8 < max_chunks) G <<= 1;
  const size_t threads = (size_t)M * G;
  count_launch();
  k_combine_tree<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(part, M, groups, ngroups, mode, G, out);
}

void launch_combine_terms(const double* part, int M, const Group* groups, int ngroups, int max_chunks, int mode,
                          bool ordered, double* out, cudaStream_t s) {
  if (M <= 0 || ngroups <= 0) return;
  count_launch();
  if (ordered) {
    k_combine_terms<<<(M + 127) / 128, 128, 0, s>>>(part, M, groups, ngroups, mode, out);
    return;
  }
  int G = 1;
  while (G < 32 && G * 8 < max_chunks) G <<= 1;
  const size_t threads = (size_t)M * G;
  k_combine_terms_tree<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(part, M, groups, ngroups, mode, G, out);
}

void launch_fils_to_rec64(const double* fc, const double* rvc, const double* gam, int64_t N, double* rec,
                          cudaStream_t s) {
  if (N <= 0) return;
  count_launch();
  k_fils_to_rec64<<<(unsigned)((N + 255) / 256), 256, 0, s>>>(fc, rvc, gam, N, rec);
}

void launch_rings_to_rec64(const double* corners, const double* rvc, const double* gam, int64_t N, double* rec,
                           cudaStream_t s) {
  if (N <= 0) return;
  count_launch();
  k_rings_to_rec64<<<(unsigned)((N + 255) / 256), 256, 0, s>>>(corners, rvc, gam, N, rec);
}

}  // namespace vlm
