// Incremental predicted-wake evaluation (FP32 precisions).
//
// The predictor of the reference's predictor-corrector and Adams-Moulton
// schemes (fdSchemeSwitch 1, 3, 4, 5: src/main.f90:844-1406) moves a small
// part of the wake -- its 'P' convection loops `do i = 1, rowNear, nNwake`
// and so visits the first near-wake row only (src/classdef.f90:1549-1575):
// the predicted wake differs from the current one in a few node rows and the
// far-wake filaments.  Every source record and every target point that did not
// move gives the same FP32 pair in both evaluations, so the predicted-wake
// velocity at an unmoved target is the current-wake velocity plus the sum of
// (new - old) over the moved records, and only the moved targets need the full
// sum.  These kernels find the moved records and targets by comparing the two
// gathered record sets and target sets bit by bit, compact them in index order
// (a deterministic order, so that a replayed step gives the same bits) into
// fixed-capacity buffers padded with inert records, and merge the results.
#include <cuda_runtime.h>

#include <algorithm>

#include "vlm_bs.h"

namespace vlm {
namespace {

// small tiles: a record is 18 + 4 doubles, read by one thread, and a few
// hundred blocks keep every SM busy on a 25k-record set
constexpr int kDiffThreads = 128;
constexpr int kDiffItems = 2;  // items per thread per block tile
constexpr int kDiffTile = kDiffThreads * kDiffItems;

__device__ __forceinline__ bool same_bits(const double* a, const double* b, int n) {
  for (int k = 0; k < n; ++k)
    if (__double_as_longlong(a[k]) != __double_as_longlong(b[k])) return false;
  return true;
}
// item i differs between the two sets: its `stride` doubles, or its 4 edge
// weights when the sets carry them
__device__ __forceinline__ bool item_changed(const double* a, const double* b, int stride, const double* ea,
                                             const double* eb, int i) {
  if (!same_bits(a + (size_t)i * stride, b + (size_t)i * stride, stride)) return true;
  return ea && !same_bits(ea + 4 * (size_t)i, eb + 4 * (size_t)i, 4);
}

// exclusive prefix of f over the block's threads in thread order; *total =
// the block's count.  Every thread of the block calls it.
__device__ __forceinline__ int block_prefix(bool f, int* warpTot, int* total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const unsigned b = __ballot_sync(0xffffffffu, f);
  if (lane == 0) warpTot[w] = __popc(b);
  __syncthreads();
  int before = 0, tot = 0;
  for (int k = 0; k < kDiffThreads / 32; ++k) {
    const int c = warpTot[k];
    if (k < w) before += c;
    tot += c;
  }
  __syncthreads();  // warpTot is reused by the next call
  *total = tot;
  return before + __popc(b & ((1u << lane) - 1u));
}

// per block tile of kDiffTile items: the number that changed
__global__ void __launch_bounds__(kDiffThreads) k_diff_count(const double* __restrict__ a, const double* __restrict__ b,
                                                             int stride, const double* __restrict__ ea,
                                                             const double* __restrict__ eb, int n,
                                                             int* __restrict__ blockCount) {
  __shared__ int warpTot[kDiffThreads / 32];
  const int base = blockIdx.x * kDiffTile;
  int cnt = 0;
  for (int u = 0; u < kDiffItems; ++u) {
    const int i = base + u * kDiffThreads + threadIdx.x;
    int tot = 0;
    block_prefix(i < n && item_changed(a, b, stride, ea, eb, i), warpTot, &tot);
    cnt += tot;
  }
  if (threadIdx.x == 0) blockCount[blockIdx.x] = cnt;
}

// exclusive scan of the block counts in place (one block); *total = their sum
__global__ void __launch_bounds__(kDiffThreads) k_diff_scan(int* __restrict__ blockCount, int nb,
                                                            int* __restrict__ total) {
  __shared__ int sh[kDiffThreads];
  int carry = 0;
  for (int base = 0; base < nb; base += kDiffThreads) {
    const int i = base + threadIdx.x;
    const int v = i < nb ? blockCount[i] : 0;
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int off = 1; off < kDiffThreads; off <<= 1) {
      const int t = threadIdx.x >= off ? sh[threadIdx.x - off] : 0;
      __syncthreads();
      sh[threadIdx.x] += t;
      __syncthreads();
    }
    const int incl = sh[threadIdx.x];
    if (i < nb) blockCount[i] = carry + incl - v;
    carry += sh[kDiffThreads - 1];
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
}

// The delta record set: changed record r (o-th in index order) -> slot 2o its
// predicted version (+), slot 2o + 1 its current version with the circulation
// negated (-): the edge weights when the sets carry them, else the record's
// circulation.  Slots from 2 min(total, half) to cap are inert: a copy of
// predicted record 0 with no circulation on any filament (lattice edge weights
// 0; or circulation 0 with the skip flag), which the FP32 packer turns into a
// record of zero weights and no near field.  More changed records than half
// the capacity: ctl = 5 (the step's result is then wrong and reported).
__global__ void __launch_bounds__(kDiffThreads)
    k_delta_records(const double* __restrict__ recP, const double* __restrict__ recC, const double* __restrict__ ewP,
                    const double* __restrict__ ewC, int nrec, const int* __restrict__ blockOff,
                    const int* __restrict__ total, double* __restrict__ dRec, double* __restrict__ dEw, int cap,
                    int* __restrict__ ctl) {
  __shared__ int warpTot[kDiffThreads / 32];
  const int half = cap / 2;
  int off = blockOff[blockIdx.x];
  const int base = blockIdx.x * kDiffTile;
  for (int u = 0; u < kDiffItems; ++u) {
    const int r = base + u * kDiffThreads + threadIdx.x;
    const bool f = r < nrec && item_changed(recP, recC, kRec64, ewP, ewC, r);
    int tot = 0;
    const int p = block_prefix(f, warpTot, &tot);
    const int o = off + p;
    if (f && o < half) {
      const double* P = recP + (size_t)r * kRec64;
      const double* C = recC + (size_t)r * kRec64;
      double* dn = dRec + (size_t)(2 * o) * kRec64;
      double* dd = dn + kRec64;
      for (int k = 0; k < kRec64; ++k) {
        dn[k] = P[k];
        dd[k] = C[k];
      }
      if (ewP) {
        for (int k = 0; k < 4; ++k) {
          dEw[4 * (size_t)(2 * o) + k] = ewP[4 * (size_t)r + k];
          dEw[4 * (size_t)(2 * o + 1) + k] = -ewC[4 * (size_t)r + k];
        }
      } else {
        dd[16] = -C[16];
      }
    }
    off += tot;
  }
  // inert padding, grid-stride over the whole capacity
  const int n = *total;
  const int used = 2 * min(n, half);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < cap; i += gridDim.x * blockDim.x) {
    if (i < used) continue;
    double* dn = dRec + (size_t)i * kRec64;
    for (int k = 0; k < kRec64; ++k) dn[k] = recP[k];
    if (ewP) {
      for (int k = 0; k < 4; ++k) dEw[4 * (size_t)i + k] = 0.0;
    } else {
      dn[16] = 0.0;
      dn[17] = (double)((int)recP[17] | REC_SKIP);
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0 && n > half) atomicCAS(ctl, 0, 5);
}

// The moved targets: o-th moved target (index order) -> idx[o], pos[o];
// slots from min(total, cap) to cap get target 0's position (their results are
// not used).  More than cap: ctl = 5.
__global__ void __launch_bounds__(kDiffThreads)
    k_moved_targets(const double* __restrict__ tP, const double* __restrict__ tC, int M,
                    const int* __restrict__ blockOff, const int* __restrict__ total, int* __restrict__ idx,
                    double* __restrict__ pos, int cap, int* __restrict__ ctl) {
  __shared__ int warpTot[kDiffThreads / 32];
  int off = blockOff[blockIdx.x];
  const int base = blockIdx.x * kDiffTile;
  for (int u = 0; u < kDiffItems; ++u) {
    const int m = base + u * kDiffThreads + threadIdx.x;
    const bool f = m < M && item_changed(tP, tC, 3, nullptr, nullptr, m);
    int tot = 0;
    const int p = block_prefix(f, warpTot, &tot);
    const int o = off + p;
    if (f && o < cap) {
      idx[o] = m;
      for (int k = 0; k < 3; ++k) pos[3 * (size_t)o + k] = tP[3 * (size_t)m + k];
    }
    off += tot;
  }
  const int n = *total;
  const int used = min(n, cap);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < cap; i += gridDim.x * blockDim.x) {
    if (i < used) continue;
    for (int k = 0; k < 3; ++k) pos[3 * (size_t)i + k] = tP[k];
  }
  if (blockIdx.x == 0 && threadIdx.x == 0 && n > cap) atomicCAS(ctl, 0, 5);
}

__global__ void k_incr_add(double* __restrict__ out, const double* __restrict__ delta, int n3) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n3) out[i] = out[i] + delta[i];
}

// also passes the moved targets' evaluation's error code on to the step's
__global__ void k_incr_put(double* __restrict__ out, const int* __restrict__ idx, const double* __restrict__ v,
                           const int* __restrict__ total, int cap, const int* __restrict__ subCtl,
                           int* __restrict__ ctl) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0 && subCtl[0] != 0) atomicCAS(ctl, 0, subCtl[0]);
  if (i >= min(*total, cap)) return;
  const int m = idx[i];
  for (int k = 0; k < 3; ++k) out[3 * (size_t)m + k] = v[3 * (size_t)i + k];
}

inline int diff_blocks(int n) { return (n + kDiffTile - 1) / kDiffTile; }

}  // namespace

int incr_diff_blocks(int n) { return n > 0 ? diff_blocks(n) : 0; }

void launch_diff_count(const double* a, const double* b, int stride, const double* ea, const double* eb, int n,
                       int* blockCount, int* total, cudaStream_t s) {
  const int nb = diff_blocks(n);
  if (nb <= 0) {
    cudaMemsetAsync(total, 0, sizeof(int), s);
    return;
  }
  count_launch();
  k_diff_count<<<nb, kDiffThreads, 0, s>>>(a, b, stride, ea, eb, n, blockCount);
  count_launch();
  k_diff_scan<<<1, kDiffThreads, 0, s>>>(blockCount, nb, total);
}

void launch_delta_records(const double* recP, const double* recC, const double* ewP, const double* ewC, int nrec,
                          const int* blockOff, const int* total, double* dRec, double* dEw, int cap, int* ctl,
                          cudaStream_t s) {
  if (nrec <= 0 || cap <= 0) return;
  count_launch();
  k_delta_records<<<diff_blocks(nrec), kDiffThreads, 0, s>>>(recP, recC, ewP, ewC, nrec, blockOff, total, dRec, dEw,
                                                            cap, ctl);
}

void launch_moved_targets(const double* tP, const double* tC, int M, const int* blockOff, const int* total, int* idx,
                          double* pos, int cap, int* ctl, cudaStream_t s) {
  if (M <= 0 || cap <= 0) return;
  count_launch();
  k_moved_targets<<<diff_blocks(M), kDiffThreads, 0, s>>>(tP, tC, M, blockOff, total, idx, pos, cap, ctl);
}

void launch_incr_merge(double* out, const double* delta, int M, const int* idx, const double* moved,
                       const int* total, int cap, const int* subCtl, int* ctl, cudaStream_t s) {
  if (M <= 0) return;
  count_launch();
  k_incr_add<<<(3 * M + 255) / 256, 256, 0, s>>>(out, delta, 3 * M);
  count_launch();
  k_incr_put<<<(std::max(cap, 1) + 255) / 256, 256, 0, s>>>(out, idx, moved, total, cap, subCtl, ctl);
}

}  // namespace vlm
