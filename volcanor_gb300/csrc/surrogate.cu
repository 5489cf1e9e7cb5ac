// Device side of the learned far-wake surrogate: target sampling, MLP input
// features, merging the MLP's far-wake velocity into an evaluation's result,
// and the audit's error sums.  (The network itself is mlp.cu; the policy --
// collect, train, audit, revert -- is the case's, in case.cpp.)
//
// The surrogate replaces the direct sum over the OLD far wake (the rolled-up
// tip filaments behind the near-wake sheet, past the `young` youngest per
// blade) at the "inner" targets: the collocation points and the near-wake
// nodes, at least the young filaments' length away from the old wake along
// the tip vortex.  Far-wake nodes keep the direct old-far-wake sum, whose
// near field (a filament's neighbours) no smooth model can represent.  (The
// sampling and merge kernels also take a count of young far-wake nodes to
// treat as inner targets; the case passes 0.)
#include <cuda_runtime.h>

#include "vlm_math.h"
#include "vlm_solver.h"

namespace vlm {

namespace {

inline int nblk(long n, int t) { return (int)((n + t - 1) / t); }

__device__ __forceinline__ d3 ld3(const double* p) { return mk3(p[0], p[1], p[2]); }

__device__ __forceinline__ const double* panRec(const Dims& d, const double* fr, int b, int p) {
  return fr + d.fl.pan + ((size_t)b * d.npan + p) * kPan;
}

__device__ __forceinline__ size_t ringI(const Dims& d, int b, int i, int j) {
  return (size_t)b * d.NW * d.ns + (size_t)i + (size_t)d.NW * j;
}

// CPs of the convecting blades, then every stride-th node (from offset) of
// the inner wake: per blade its near-wake nodes (rows rowNear..NW) and its
// `young` youngest far-wake nodes, in the node evaluations' order
__global__ void k_surr_targets(Dims d, DevState s, const double* fr, int rowNear, int rowFar, int young, int stride,
                               int offset, int nNodes, double* P) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int ncp = d.nbC * d.npan;
  if (t >= ncp + nNodes) return;
  d3 p;
  if (t < ncp) {
    p = ld3(panRec(d, fr, t / d.npan, t % d.npan) + 12);
  } else {
    const int rowsN = rowNear <= d.NW ? d.NW - (rowNear - 1) : 0;
    const int nn = rowsN * (d.ns + 1);
    const int per = nn + young;
    const int m = offset + (t - ncp) * stride;
    const int b = m / per, l = m % per;
    if (l < nn) {
      const int j = l % (d.ns + 1), i = rowNear - 1 + l / (d.ns + 1);
      p = j < d.ns ? ld3(s.nC + ringI(d, b, i, j) * 12 + 3) : ld3(s.nC + ringI(d, b, i, d.ns - 1) * 12 + 6);
    } else {
      p = ld3(s.fC + ((size_t)b * d.NF + rowFar - 1 + (l - nn)) * 6);
    }
  }
  P[3 * (size_t)t] = p.x;
  P[3 * (size_t)t + 1] = p.y;
  P[3 * (size_t)t + 2] = p.z;
}

// old far-wake nodes (rows rowFar + young .. NF) of the convecting blades,
// blade-major, oldest last
__global__ void k_surr_far_targets(Dims d, DevState s, int rowFar, int young, int pred, double* P) {
  const int rowsF = d.NF - (rowFar - 1);
  const int nOld = rowsF - young;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (nOld <= 0 || t >= d.nbC * nOld) return;
  const int b = t / nOld, i = rowFar - 1 + young + t % nOld;
  const double* f = (pred ? s.fCP : s.fC) + ((size_t)b * d.NF + i) * 6;
  P[3 * (size_t)t] = f[0];
  P[3 * (size_t)t + 1] = f[1];
  P[3 * (size_t)t + 2] = f[2];
}

// Coarse descriptor of the old far wake (filaments rows rowFar + young ..
// NF of every blade), one block, fixed-order sums: desc[0..2] = its
// |circulation|-weighted centroid about the hub over the rotor radius,
// desc[3] = its mean |circulation| over the wing's largest |circulation|.
__global__ void k_surr_descriptor(Dims d, DevState s, const double* fr, int rowFar, int young, int pred, double invR,
                                  double* desc) {
  __shared__ double red[4][256];
  const double* rot = fr + d.fl.rot;
  const double* fc = pred ? s.fCP : s.fC;
  const int first = rowFar - 1 + young;
  const int nOld = d.NF - first;
  double gx = 0.0, gy = 0.0, gz = 0.0, g = 0.0;
  for (int t = threadIdx.x; t < d.nb * max(nOld, 0); t += blockDim.x) {
    const int b = t / nOld, i = first + t % nOld;
    const size_t f = (size_t)b * d.NF + i;
    const double a = fabs(s.fGam[f]);
    gx += a * 0.5 * (fc[6 * f] + fc[6 * f + 3]);
    gy += a * 0.5 * (fc[6 * f + 1] + fc[6 * f + 4]);
    gz += a * 0.5 * (fc[6 * f + 2] + fc[6 * f + 5]);
    g += a;
  }
  double wmax = 0.0;
  for (int t = threadIdx.x; t < d.nb * d.npan; t += blockDim.x) wmax = fmax(wmax, fabs(s.wGam[t]));
  red[0][threadIdx.x] = gx;
  red[1][threadIdx.x] = gy;
  red[2][threadIdx.x] = gz;
  red[3][threadIdx.x] = g;
  __shared__ double rmax[256];
  rmax[threadIdx.x] = wmax;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      for (int c = 0; c < 4; ++c) red[c][threadIdx.x] += red[c][threadIdx.x + w];
      rmax[threadIdx.x] = fmax(rmax[threadIdx.x], rmax[threadIdx.x + w]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double G = red[3][0];
    const int n = d.nb * max(nOld, 0);
    desc[0] = G > 0.0 ? (red[0][0] / G - rot[3]) * invR : 0.0;
    desc[1] = G > 0.0 ? (red[1][0] / G - rot[4]) * invR : 0.0;
    desc[2] = G > 0.0 ? (red[2][0] / G - rot[5]) * invR : 0.0;
    desc[3] = (n > 0 && rmax[0] > 0.0) ? G / n / rmax[0] : 0.0;
  }
}

// kSurrFeatures features per target: position about the hub over the rotor
// radius, cos/sin of the rotor azimuth (blade 1's azimuth axis in the frame)
// and of nb times it, the old wake's fill fraction, and the old wake's
// descriptor (centroid about the hub / R, relative mean |circulation|)
__global__ void k_surr_features(Dims d, const double* fr, const double* P, int M, double invR, double fill,
                                const double* desc, float* X) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= M) return;
  const double* rot = fr + d.fl.rot;
  const double* ax = fr + d.fl.ax;  // blade 1: xAxisAziFlap first
  const double hx = rot[3], hy = rot[4], hz = rot[5];
  const double n = sqrt(ax[0] * ax[0] + ax[1] * ax[1]);
  const double c = n > 0.0 ? ax[0] / n : 1.0, sn = n > 0.0 ? ax[1] / n : 0.0;
  double cn = 1.0, snb = 0.0;
  for (int k = 0; k < d.nb; ++k) {
    const double a = cn * c - snb * sn, b = cn * sn + snb * c;
    cn = a;
    snb = b;
  }
  float* x = X + (size_t)t * kSurrFeatures;
  x[0] = (float)((P[3 * (size_t)t] - hx) * invR);
  x[1] = (float)((P[3 * (size_t)t + 1] - hy) * invR);
  x[2] = (float)((P[3 * (size_t)t + 2] - hz) * invR);
  x[3] = (float)c;
  x[4] = (float)sn;
  x[5] = (float)cn;
  x[6] = (float)snb;
  x[7] = (float)fill;
  for (int k = 0; k < 4; ++k) x[8 + k] = (float)desc[k];
}

// outv[m] += scale * Y[m] for m < M
__global__ void k_surr_add(int M, const float* Y, const double* scale, double* outv) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= M) return;
  const double sc = scale[0];
  for (int k = 0; k < 3; ++k) outv[3 * (size_t)t + k] += sc * (double)Y[3 * (size_t)t + k];
}

// node evaluation: near-wake nodes and the young far-wake nodes get the
// network's old-far-wake velocity, old far-wake nodes the direct old-far-wake
// sum of the old-far-target evaluation
__global__ void k_surr_merge_nodes(Dims d, int rowNear, int rowFar, int young, int M, const float* Y,
                                   const double* scale, const double* outFar, double* outv) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= M) return;
  const int rowsN = d.NW - (rowNear - 1);
  const int rowsF = max(d.NF - (rowFar - 1), 0);
  const int per = rowsN * (d.ns + 1) + rowsF;
  const int b = m / per, l = m % per;
  const int inner = rowsN * (d.ns + 1) + young;
  if (l < inner) {
    const double sc = scale[0];
    for (int k = 0; k < 3; ++k) outv[3 * (size_t)m + k] += sc * (double)Y[3 * (size_t)m + k];
  } else {
    const size_t f = (size_t)b * (rowsF - young) + (l - inner);
    for (int k = 0; k < 3; ++k) outv[3 * (size_t)m + k] += outFar[3 * f + k];
  }
}

// training samples: X rows as they are, T = direct far-wake velocity (FP32)
__global__ void k_surr_append(int n, const float* Xs, const double* V, float* X, float* T) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  for (int k = 0; k < kSurrFeatures; ++k) X[(size_t)t * kSurrFeatures + k] = Xs[(size_t)t * kSurrFeatures + k];
  for (int k = 0; k < 3; ++k) T[(size_t)t * 3 + k] = (float)V[3 * (size_t)t + k];
}

// audit sums (one block, fixed order): out[0] = sum |scale Y - V|^2,
// out[1] = sum |V|^2
__global__ void k_surr_audit(int n, const float* Y, const double* scale, const double* V, double* out) {
  __shared__ double r0[256], r1[256];
  double a = 0.0, b = 0.0;
  const double sc = scale[0];
  for (int t = threadIdx.x; t < n; t += blockDim.x)
    for (int k = 0; k < 3; ++k) {
      const double v = V[3 * (size_t)t + k];
      const double e = sc * (double)Y[3 * (size_t)t + k] - v;
      a += e * e;
      b += v * v;
    }
  r0[threadIdx.x] = a;
  r1[threadIdx.x] = b;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      r0[threadIdx.x] += r0[threadIdx.x + w];
      r1[threadIdx.x] += r1[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = r0[0];
    out[1] = r1[0];
  }
}

}  // namespace

void launch_surr_targets(const Dims& d, const DevState& s, const double* fr, int rowNear, int rowFar, int young,
                         int stride, int offset, int nNodes, double* P, cudaStream_t st) {
  const int n = d.nbC * d.npan + nNodes;
  if (n <= 0) return;
  count_launch();
  k_surr_targets<<<nblk(n, 256), 256, 0, st>>>(d, s, fr, rowNear, rowFar, young, stride, offset, nNodes, P);
}
void launch_surr_far_targets(const Dims& d, const DevState& s, int rowFar, int young, bool pred, double* P,
                             cudaStream_t st) {
  const int n = d.nbC * (d.NF - (rowFar - 1) - young);
  if (n <= 0) return;
  count_launch();
  k_surr_far_targets<<<nblk(n, 256), 256, 0, st>>>(d, s, rowFar, young, pred ? 1 : 0, P);
}
void launch_surr_features(const Dims& d, const DevState& s, const double* fr, const double* P, int M, double invR,
                          double fill, int rowFar, int young, bool pred, double* desc, float* X, cudaStream_t st) {
  if (M <= 0) return;
  count_launch();
  k_surr_descriptor<<<1, 256, 0, st>>>(d, s, fr, rowFar, young, pred ? 1 : 0, invR, desc);
  count_launch();
  k_surr_features<<<nblk(M, 256), 256, 0, st>>>(d, fr, P, M, invR, fill, desc, X);
}
void launch_surr_add(int M, const float* Y, const double* scale, double* outv, cudaStream_t st) {
  if (M <= 0) return;
  count_launch();
  k_surr_add<<<nblk(M, 256), 256, 0, st>>>(M, Y, scale, outv);
}
void launch_surr_merge_nodes(const Dims& d, int rowNear, int rowFar, int young, int M, const float* Y,
                             const double* scale, const double* outFar, double* outv, cudaStream_t st) {
  if (M <= 0) return;
  count_launch();
  k_surr_merge_nodes<<<nblk(M, 256), 256, 0, st>>>(d, rowNear, rowFar, young, M, Y, scale, outFar, outv);
}
void launch_surr_append(int n, const float* Xs, const double* V, float* X, float* T, cudaStream_t st) {
  if (n <= 0) return;
  count_launch();
  k_surr_append<<<nblk(n, 256), 256, 0, st>>>(n, Xs, V, X, T);
}
void launch_surr_audit(int n, const float* Y, const double* scale, const double* V, double* out, cudaStream_t st) {
  count_launch();
  k_surr_audit<<<1, 256, 0, st>>>(n, Y, scale, V, out);
}

}  // namespace vlm
