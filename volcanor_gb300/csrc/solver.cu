// Time-step kernels of the FP64 free-wake solver: wake shedding, ageing,
// dissipation, predictor/corrector convection with lattice continuity,
// strain, rollup and truncation, AIC assembly and inversion, circulation
// solve and loads.  Compiled with -fmad=false: each kernel performs, per
// element, exactly the IEEE operations of the reference routine it restates.
#include <math.h>

#include "vlm_math.h"
#include "vlm_solver.h"

namespace vlm {

namespace {

__device__ __forceinline__ d3 ld3(const double* p) { return mk3(p[0], p[1], p[2]); }
__device__ __forceinline__ void st3(double* p, d3 v) {
  p[0] = v.x;
  p[1] = v.y;
  p[2] = v.z;
}
__device__ __forceinline__ size_t ringI(const Dims& d, int b, int i, int j) {
  return (size_t)b * d.NW * d.ns + i + (size_t)d.NW * j;
}
__device__ __forceinline__ size_t velI(const Dims& d, int b, int i, int j) {
  return (size_t)b * d.NW * (d.ns + 1) + i + (size_t)d.NW * j;
}
__device__ __forceinline__ const double* panRec(const Dims& d, const double* fr, int b, int p) {
  return fr + d.fl.pan + ((size_t)b * d.npan + p) * kPan;
}
__device__ __forceinline__ m33 frameT(const Dims& d, const double* fr, int b) {
  const double* t = fr + d.fl.rot + 10 + 9 * (b - 1);
  m33 T;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) T.a[r][c] = t[3 * r + c];
  return T;
}

inline int nblk(long n, int t) { return (int)((n + t - 1) / t); }

// ---- shed (classdef.f90:4297-4325) ---------------------------------------
__global__ void k_shed(Dims d, DevState s, const double* fr, int rowNear, int le) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= d.nb * d.ns) return;
  const int b = t / d.ns, j = t % d.ns;
  const int p = (d.nc - 1) + d.nc * j;
  const double* w = panRec(d, fr, b, p);
  if (le) {
    double* c = s.nC + ringI(d, b, rowNear - 1, j) * 12;
    st3(c + 0, ld3(w + 3));
    st3(c + 9, ld3(w + 6));
    s.nGam[ringI(d, b, rowNear - 1, j)] = s.wGam[(size_t)b * d.npan + p];
  } else {
    const int r = max(rowNear - 1, 1) - 1;
    double* c = s.nC + ringI(d, b, r, j) * 12;
    st3(c + 3, ld3(w + 3));
    st3(c + 6, ld3(w + 6));
  }
}

// ---- age (classdef.f90:4331-4354) -----------------------------------------
__global__ void k_age(Dims d, DevState s, int rowNear, int rowFar) {
  const int rows = d.NW - (rowNear - 1);
  const int nNear = d.nb * rows * d.ns;
  const int nFar = d.nb * max(d.NF - (rowFar - 1), 0);
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < nNear) {
    const int b = t / (rows * d.ns), l = t % (rows * d.ns);
    const int j = l / rows, i = rowNear - 1 + l % rows;
    const size_t r = ringI(d, b, i, j);
    s.nAge[r] = s.nAge[r] + d.dt;
  } else if (t < nNear + nFar) {
    const int l = t - nNear;
    const int rf = d.NF - (rowFar - 1);
    const int b = l / rf, i = rowFar - 1 + l % rf;
    const size_t r = (size_t)b * d.NF + i;
    s.fAge[r] = s.fAge[r] + d.dt;
  }
}

// ---- dissipation (classdef.f90:4356-4408) ----------------------------------
__global__ void k_dissip_a(Dims d, DevState s, int rowNear, int rowFar) {
  const int rows = d.NW - (rowNear - 1);
  const int nNear = d.nb * rows * d.ns;
  const int nFar = d.nb * max(d.NF - (rowFar - 1), 0);
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < nNear) {
    const int b = t / (rows * d.ns), l = t % (rows * d.ns);
    const int j = l / rows, i = rowNear - 1 + l % rows;
    const size_t r = ringI(d, b, i, j);
    double* rv = s.nRvc + 4 * r;
    const double a = sqrt(rv[0] * rv[0] + d.dissipAdd);
    rv[0] = a;
    rv[2] = a;
    s.nGam[r] = s.nGam[r] * d.decay;
    rv[1] = sqrt(rv[1] * rv[1] + d.dissipAdd);
  } else if (t < nNear + nFar) {
    const int l = t - nNear;
    const int rf = d.NF - (rowFar - 1);
    const int b = l / rf, i = rowFar - 1 + l % rf;
    const size_t r = (size_t)b * d.NF + i;
    s.fRvc[r] = sqrt(s.fRvc[r] * s.fRvc[r] + d.dissipAdd);
    s.fGam[r] = s.fGam[r] * d.decay;
  }
}
__global__ void k_dissip_b(Dims d, DevState s, int rowNear) {
  const int rows = d.NW - rowNear;  // rows rowNear+1..NW (1-based)
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (rows <= 0 || t >= d.nb * rows * d.ns) return;
  const int b = t / (rows * d.ns), l = t % (rows * d.ns);
  const int j = l / rows, i = rowNear + l % rows;
  s.nRvc[4 * ringI(d, b, i, j) + 3] = s.nRvc[4 * ringI(d, b, i - 1, j) + 1];
}

// ---- predicted copy (main.f90:1012-1019) -----------------------------------
__global__ void k_copy_pred(Dims d, DevState s, int rowNear, int rowFar) {
  const int rows = d.NW - (rowNear - 1);
  const int nNear = d.nbC * rows * d.ns;
  const int nFar = d.nbC * max(d.NF - (rowFar - 1), 0);
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < nNear) {
    const int b = t / (rows * d.ns), l = t % (rows * d.ns);
    const int j = l / rows, i = rowNear - 1 + l % rows;
    const size_t r = ringI(d, b, i, j) * 12;
    for (int k = 0; k < 12; ++k) s.nCP[r + k] = s.nC[r + k];
  } else if (t < nNear + nFar) {
    const int l = t - nNear;
    const int rf = d.NF - (rowFar - 1);
    const int b = l / rf, i = rowFar - 1 + l % rf;
    const size_t r = ((size_t)b * d.NF + i) * 6;
    for (int k = 0; k < 6; ++k) s.fCP[r + k] = s.fC[r + k];
  }
}

// ---- convection shift (classdef.f90:1515-1575) ----------------------------
__global__ void k_shift(Dims d, DevState s, int rowNear, int rowFar, int pred) {
  const int rows = pred ? 1 : d.NW - (rowNear - 1);
  const int i0 = pred ? 0 : rowNear - 1;  // the predicted loop visits row 1 only
  const int nNear = d.nbC * rows * (d.ns + 1);
  const int nFar = d.nbC * max(d.NF - (rowFar - 1), 0);
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  double* nc = pred ? s.nCP : s.nC;
  if (t < nNear) {
    const int b = t / (rows * (d.ns + 1)), l = t % (rows * (d.ns + 1));
    const int j = l / rows, i = i0 + l % rows;
    const d3 dv = ld3(s.vN[0] + 3 * velI(d, b, i, j)) * d.dt;
    double* c = j < d.ns ? nc + ringI(d, b, i, j) * 12 + 3 : nc + ringI(d, b, i, d.ns - 1) * 12 + 6;
    st3(c, ld3(c) + dv);
  } else if (t < nNear + nFar) {
    const int l = t - nNear;
    const int rf = d.NF - (rowFar - 1);
    const int b = l / rf, i = rowFar - 1 + l % rf;
    double* c = (pred ? s.fCP : s.fC) + ((size_t)b * d.NF + i) * 6;
    st3(c, ld3(c) + ld3(s.vF[0] + 3 * ((size_t)b * d.NF + i)) * d.dt);
  }
}

// ---- continuity (classdef.f90:1609-1702) ----------------------------------
__global__ void k_continuity(Dims d, DevState s, int rowNear, int rowFar, int pred) {
  const int rows = d.NW - (rowNear - 1);
  const int nNear = d.nbC * rows * d.ns;
  const int nFar = d.nbC * max(d.NF - rowFar, 0);
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  double* nc = pred ? s.nCP : s.nC;
  if (t < nNear) {
    const int b = t / (rows * d.ns), l = t % (rows * d.ns);
    const int j = l / rows, i = rowNear - 1 + l % rows;
    double* c = nc + ringI(d, b, i, j) * 12;
    if (i > rowNear - 1) {
      if (j < d.ns - 1) {
        st3(c + 0, ld3(nc + ringI(d, b, i - 1, j) * 12 + 3));
        st3(c + 6, ld3(nc + ringI(d, b, i, j + 1) * 12 + 3));
        st3(c + 9, ld3(nc + ringI(d, b, i - 1, j + 1) * 12 + 3));
      } else {
        st3(c + 0, ld3(nc + ringI(d, b, i - 1, j) * 12 + 3));
        st3(c + 9, ld3(nc + ringI(d, b, i - 1, j) * 12 + 6));
      }
    } else if (j < d.ns - 1) {
      st3(c + 6, ld3(nc + ringI(d, b, i, j + 1) * 12 + 3));
    }
  } else if (t < nNear + nFar) {
    const int l = t - nNear;
    const int rf = d.NF - rowFar;
    const int b = l / rf, i = rowFar + l % rf;
    double* fc = pred ? s.fCP : s.fC;
    st3(fc + ((size_t)b * d.NF + i) * 6 + 3, ld3(fc + ((size_t)b * d.NF + i - 1) * 6));
  }
}

// ---- axisymmetric wake copies (classdef.f90:4801-4823) ---------------------
__global__ void k_axisym(Dims d, DevState s, const double* fr, int rowNear, int rowFar, int pred) {
  const int rows = d.NW - (rowNear - 1);
  const int nNear = (d.nb - 1) * rows * d.ns;
  const int rf = max(d.NF - (rowFar - 1), 0);
  const int nFar = (d.nb - 1) * rf;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const d3 hub = ld3(fr + d.fl.rot + 3);
  if (t < nNear) {
    const int b = 1 + t / (rows * d.ns), l = t % (rows * d.ns);
    const int j = l / rows, i = rowNear - 1 + l % rows;
    const m33 T = frameT(d, fr, b);
    const size_t r0 = ringI(d, 0, i, j), r1 = ringI(d, b, i, j);
    double* nc = pred ? s.nCP : s.nC;
    for (int k = 0; k < 4; ++k) st3(nc + r1 * 12 + 3 * k, rot_about(T, ld3(nc + r0 * 12 + 3 * k), hub));
    if (!pred) {
      s.nGam[r1] = s.nGam[r0];
      for (int k = 0; k < 4; ++k) s.nRvc[4 * r1 + k] = s.nRvc[4 * r0 + k];
      s.nAge[r1] = s.nAge[r0];
    }
  } else if (t < nNear + nFar) {
    const int l = t - nNear;
    const int b = 1 + l / rf, i = rowFar - 1 + l % rf;
    const m33 T = frameT(d, fr, b);
    const size_t r0 = i, r1 = (size_t)b * d.NF + i;
    double* fc = pred ? s.fCP : s.fC;
    st3(fc + r1 * 6, rot_about(T, ld3(fc + r0 * 6), hub));
    st3(fc + r1 * 6 + 3, rot_about(T, ld3(fc + r0 * 6 + 3), hub));
    if (!pred) {
      s.fGam[r1] = s.fGam[r0];
      s.fRvc[r1] = s.fRvc[r0];
      s.fRvc0[r1] = s.fRvc0[r0];
      s.fL0[r1] = s.fL0[r0];
      s.fLc[r1] = s.fLc[r0];
      s.fAge[r1] = s.fAge[r0];
    }
  }
}

// ---- strain (classdef.f90:4410-4422, 505-521) ------------------------------
__global__ void k_strain(Dims d, DevState s, int rowFar) {
  const int rf = d.NF - (rowFar - 1);
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (rf <= 0 || t >= d.nb * rf) return;
  const int b = t / rf, i = rowFar - 1 + t % rf;
  const size_t r = (size_t)b * d.NF + i;
  const double lc = norm3(ld3(s.fC + 6 * r) - ld3(s.fC + 6 * r + 3));
  s.fLc[r] = lc;
  s.fRvc[r] = s.fRvc0[r] * sqrt(s.fL0[r] / lc);
}

// ---- prescribed far wake (classdef.f90:998-1066, 5172-5217) ----------------
// One block per convecting blade.  Thread 0 sums the far-wake filaments
// rowStart..NF in the reference's order (radius of node 1 about the z axis,
// descent between consecutive nodes), relaxes the helix pitch and radius,
// and finds the anchor (node 1 of the oldest filament); the threads then
// place the 241 helix nodes about the hub, filament i running from node i+1
// to node i, the first one attached at the anchor.  The helix angles use
// the device's cos/sin/atan2, so the nodes agree with a host evaluation to a
// few ulps, not bit for bit.
__global__ void k_presc_update(Dims d, DevState s, const double* fr, int rowFar, int pred) {
  const int b = blockIdx.x;
  const int rowStart = d.prescGenNt == 0 ? rowFar : d.NF - d.prescGenNt;
  const int i0 = rowStart - 1, i1 = d.NF - 1, n = i1 - i0 + 1;
  const double* fc = (pred ? s.fCP : s.fC) + (size_t)b * d.NF * 6;
  double* H = s.pfHelix + 2 * ((size_t)pred * d.nb + b);
  __shared__ double sh[6];  // pitch, radius, anchor xyz, dTheta
  if (threadIdx.x == 0) {
    double pitch = 0.0, radius = 0.0;
    for (int i = 0; i < n; ++i) {
      const double* c = fc + 6 * (size_t)(i0 + i);
      radius = radius + sqrt(c[1] * c[1] + c[0] * c[0]);
      if (i < n - 1) pitch = pitch + c[2] - fc[6 * (size_t)(i0 + i + 1) + 2];
    }
    const double dpsi = fr[d.fl.rot + 9] * d.dt;
    pitch = fabs(pitch) * (-kTwoPi / dpsi) / (double)(n - 1);
    radius = radius / (double)n;
    H[0] = 0.5 * pitch + (1.0 - 0.5) * H[0];
    H[1] = 0.5 * radius + (1.0 - 0.5) * H[1];
    const double* a = fc + 6 * (size_t)i1;
    sh[0] = H[0];
    sh[1] = H[1];
    sh[2] = a[0], sh[3] = a[1], sh[4] = a[2];
    sh[5] = atan2(a[1], a[0]);
    s.pfGam[(size_t)pred * d.nb + b] = (pred ? s.fGam : s.fGam)[(size_t)b * d.NF + i1];
    s.pfRvc[(size_t)pred * d.nb + b] = s.fRvc[(size_t)b * d.NF + i1];
  }
  __syncthreads();
  __shared__ double node[3 * (kPresc + 1)];
  const d3 hub = ld3(fr + d.fl.rot + 3);
  const double dx = (kTwoPi * 10.0 - 0.0) / (double)kPresc;  // linspace(0, 2 pi nRevs, 241)
  for (int i = threadIdx.x; i <= kPresc; i += blockDim.x) {
    const double th = -1.0 * ((double)i * dx + 0.0);  // a clockwise helix (isClockwiseRotor)
    node[3 * i] = hub.x + sh[1] * cos(th + sh[5]);
    node[3 * i + 1] = hub.y + sh[1] * sin(th + sh[5]);
    node[3 * i + 2] = hub.z + (sh[0] * fabs(th) / kTwoPi + (sh[4] - hub.z));
  }
  __syncthreads();
  double* out = s.pfC + ((size_t)pred * d.nb + b) * kPresc * 6;
  for (int i = threadIdx.x; i < kPresc; i += blockDim.x) {
    for (int k = 0; k < 3; ++k) out[6 * i + k] = node[3 * (i + 1) + k];  // fc1
    for (int k = 0; k < 3; ++k) out[6 * i + 3 + k] = i == 0 ? sh[2 + k] : node[3 * i + k];  // fc2
  }
}
// Axisymmetric copies: blade b's prescribed wake = blade 1's, rotated about
// the hub by b x 2 pi / nb (the wake copies' rotation).
__global__ void k_presc_axisym(Dims d, DevState s, const double* fr, int pred) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (d.nb - 1) * kPresc) return;
  const int b = 1 + t / kPresc, i = t % kPresc;
  const m33 T = frameT(d, fr, b);
  const d3 hub = ld3(fr + d.fl.rot + 3);
  const double* src = s.pfC + ((size_t)pred * d.nb) * kPresc * 6 + 6 * (size_t)i;
  double* dst = s.pfC + ((size_t)pred * d.nb + b) * kPresc * 6 + 6 * (size_t)i;
  st3(dst, rot_about(T, ld3(src), hub));
  st3(dst + 3, rot_about(T, ld3(src + 3), hub));
  if (i == 0) {
    s.pfGam[(size_t)pred * d.nb + b] = s.pfGam[(size_t)pred * d.nb];
    s.pfRvc[(size_t)pred * d.nb + b] = s.pfRvc[(size_t)pred * d.nb];
    s.pfHelix[2 * ((size_t)pred * d.nb + b)] = s.pfHelix[2 * (size_t)pred * d.nb];
    s.pfHelix[2 * ((size_t)pred * d.nb + b) + 1] = s.pfHelix[2 * (size_t)pred * d.nb + 1];
  }
}

// ---- wake burst (classdef.f90:4911-4917, 2306-2339) -------------------------
// Far-wake filament i of every blade against filament i+1: skew =
// |acos(cos(angle between fc2 - fc1 of i and fc1 - fc2 of i+1)) - pi| / pi;
// at or above skewLimit both get the chord as core radius.  Only core radii
// are written, from positions only, so the pairs run in parallel.
__global__ void k_burst(Dims d, DevState s, int rowFar) {
  const int rf = d.NF - (rowFar - 1) - 1;  // pairs (i, i+1)
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (rf <= 0 || t >= d.nb * rf) return;
  const int b = t / rf, i = rowFar - 1 + t % rf;
  const size_t r = (size_t)b * d.NF + i;
  const d3 a = ld3(s.fC + 6 * r + 3) - ld3(s.fC + 6 * r);
  const d3 c = ld3(s.fC + 6 * (r + 1)) - ld3(s.fC + 6 * (r + 1) + 3);
  const double skew = fabs(acos(dot3(a, c) / sqrt(dot3(a, a) * dot3(c, c))) - kPi) / kPi;
  if (skew >= d.skewLimit) {
    s.fRvc[r + 1] = d.chord;
    s.fRvc[r] = d.chord;
  }
}

// ---- far-wake shift for truncation (classdef.f90:4500-4513) ----------------
__global__ void k_far_to_tmp(Dims d, DevState s) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= d.nb * d.NF) return;
  const int b = t / d.NF, i = t % d.NF;
  const size_t src = (size_t)b * d.NF + (i > 0 ? i - 1 : 0);
  double* o = s.fTmp + (size_t)t * 12;
  for (int k = 0; k < 6; ++k) o[k] = s.fC[6 * src + k];
  o[6] = s.fGam[src];
  o[7] = s.fRvc[src];
  o[8] = s.fRvc0[src];
  o[9] = s.fL0[src];
  o[10] = s.fLc[src];
  o[11] = i == 0 ? 0.0 : s.fAge[src];
}
__global__ void k_far_from_tmp(Dims d, DevState s) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= d.nb * d.NF) return;
  const double* o = s.fTmp + (size_t)t * 12;
  for (int k = 0; k < 6; ++k) s.fC[6 * (size_t)t + k] = o[k];
  s.fGam[t] = o[6];
  s.fRvc[t] = o[7];
  s.fRvc0[t] = o[8];
  s.fL0[t] = o[9];
  s.fLc[t] = o[10];
  s.fAge[t] = o[11];
}

// ---- rollup (classdef.f90:4515-4605) ---------------------------------------
__global__ void k_rollup(Dims d, DevState s, int rowFarNext) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= d.nb) return;
  const int NW = d.NW;
  auto ring = [&](int j) { return ringI(d, b, NW - 1, j); };
  double gamRollup = s.nGam[ring(d.ns - 1)];
  d3 cLE = zero3(), cTE = zero3();
  double radius = 0.0, gamSum = 0.0;
  const bool posSense = fsign1(d.omega * d.theta0) > kEps;
  for (int is = d.rollupStart; is <= d.rollupEnd; ++is) {
    const size_t r = ring(is - 1);
    const double g = s.nGam[r];
    cLE = cLE + ld3(s.nC + r * 12 + 9) * g;
    cTE = cTE + ld3(s.nC + r * 12 + 6) * g;
    gamSum = gamSum + g;
    if (posSense) {
      if (g < gamRollup) gamRollup = g;
    } else {
      if (g > gamRollup) gamRollup = g;
    }
    radius = radius + s.nRvc[4 * r + 2] * g;
  }
  const double ageRollup = s.nAge[ring(d.ns - 1)];
  if (fabs(gamSum) > kEps) {
    cLE = cLE / gamSum;
    cTE = cTE / gamSum;
    radius = radius / gamSum;
  } else {
    const size_t r = ring(d.rollupEnd - 1);
    cLE = ld3(s.nC + r * 12 + 3);
    cTE = ld3(s.nC + r * 12 + 6);
    radius = s.nRvc[4 * r + 2];
  }
  if (d.suppressFwake == 1) gamRollup = 0.0;
  if (d.NF > 0) {
    const size_t f = (size_t)b * d.NF + (rowFarNext - 1);
    st3(s.fC + 6 * f + 3, cLE);
    st3(s.fC + 6 * f, cTE);
    s.fGam[f] = gamRollup;
    s.fAge[f] = ageRollup;
    s.fRvc0[f] = radius;
    s.fRvc[f] = radius;
    const double lc = norm3(cTE - cLE);
    s.fLc[f] = lc;
    s.fL0[f] = lc;
    if (rowFarNext < d.NF) st3(s.fC + 6 * (f + 1) + 3, cTE);
  }
}

// ---- near-wake shift after rollup (classdef.f90:4481-4498) -----------------
__global__ void k_near_to_tmp(Dims d, DevState s) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int per = d.NW * d.ns;
  if (t >= d.nb * per) return;
  const int b = t / per, l = t % per;
  const int i = l % d.NW, j = l / d.NW;
  const size_t src = ringI(d, b, i > 0 ? i - 1 : 0, j);
  double* o = s.nTmp + (size_t)t * 18;
  for (int k = 0; k < 12; ++k) o[k] = s.nC[12 * src + k];
  o[12] = s.nGam[src];
  for (int k = 0; k < 4; ++k) o[13 + k] = s.nRvc[4 * src + k];
  o[17] = i == 0 ? 0.0 : s.nAge[src];
}
__global__ void k_near_from_tmp(Dims d, DevState s) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= d.nb * d.NW * d.ns) return;
  const double* o = s.nTmp + (size_t)t * 18;
  for (int k = 0; k < 12; ++k) s.nC[12 * (size_t)t + k] = o[k];
  s.nGam[t] = o[12];
  for (int k = 0; k < 4; ++k) s.nRvc[4 * (size_t)t + k] = o[13 + k];
  s.nAge[t] = o[17];
}

// ---- velocity history algebra (main.f90:844-1406) --------------------------
__global__ void k_velop(DevState s, long nN, long nF, int op) {
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (t >= nN + nF) return;
  const bool nearPart = t < nN;
  const long e = nearPart ? t : t - nN;
  double* a[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) a[k] = nearPart ? s.vN[k] : s.vF[k];
  double v = a[0][e], v1 = a[1][e], v2 = a[2][e], v3 = a[3][e], vp = a[4][e], st = a[5][e];
  switch (op) {
    case VOP_COPY_0_TO_1: a[1][e] = v; break;
    case VOP_COPY_0_TO_2: a[2][e] = v; break;
    case VOP_COPY_0_TO_3: a[3][e] = v; break;
    case VOP_AB2: {
      const double x = 0.5 * (3.0 * v - v1);
      a[5][e] = x;
      a[1][e] = x;
      a[0][e] = x;
    } break;
    case VOP_AM2_PRED:
      a[5][e] = v;
      a[0][e] = 0.5 * (3.0 * v - v1);
      break;
    case VOP_AM2_CORR: a[0][e] = (vp + st) * 0.5; break;
    case VOP_STEP_TO_1: a[1][e] = st; break;
    case VOP_AM3_PRED:
      a[5][e] = v;
      a[0][e] = ((23.0 * v - 16.0 * v2) + 5.0 * v1) / 12.0;
      break;
    case VOP_AM3_CORR: a[0][e] = ((5.0 * vp + 8.0 * st) - 1.0 * v2) / 12.0; break;
    case VOP_AM3_SHIFT:
      a[1][e] = v2;
      a[2][e] = st;
      break;
    case VOP_AM4_PRED:
      a[5][e] = v;
      a[0][e] = (((55.0 * v - 59.0 * v3) + 37.0 * v2) - 9.0 * v1) / 24.0;
      break;
    case VOP_AM4_CORR: a[0][e] = (((9.0 * vp + 19.0 * st) - 5.0 * v3) + 1.0 * v2) / 24.0; break;
    case VOP_AM4_SHIFT:
      a[1][e] = v2;
      a[2][e] = v3;
      a[3][e] = st;
      break;
  }
}

// ---- PC2 averaging (libCommon.f90:213-258) ---------------------------------
__global__ void k_order2(Dims d, DevState s, int rowNear, int rowFar, int phase) {
  const int m = d.NW - (rowNear - 1);
  const int mf = max(d.NF - (rowFar - 1), 0);
  const int nNear = d.nbC * (d.ns + 1) * m * 3;
  const int nFar = d.nbC * mf * 3;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < nNear) {
    const int k = t % 3, q = t / 3;
    const int b = q / ((d.ns + 1) * m), l = q % ((d.ns + 1) * m);
    const int j = l / m, i = l % m;
    const size_t base = velI(d, b, rowNear - 1, j);
    const double* vn = s.vN[0] + 3 * base + k;
    const double* vp = s.vN[4] + 3 * base + k;
    double* tmp = s.vN[6] + 3 * base + k;
    if (phase == 0) {
      double o;
      if (i == 0) o = (vp[0] + vn[0]) * 0.5;
      else if (i < m - 1) o = (((vp[3 * i] + vp[3 * (i - 1)]) + vn[3 * (i + 1)]) + vn[3 * i]) * 0.25;
      else o = (vp[3 * i] + vn[3 * i]) * 0.5;
      if (i == m - 1) o = (vp[3 * i] + vn[3 * i]) * 0.5;
      tmp[3 * i] = o;
    } else {
      s.vN[0][3 * base + k + 3 * i] = tmp[3 * i];
    }
  } else if (t < nNear + nFar) {
    const int l = t - nNear;
    const int k = l % 3, q = l / 3;
    const int b = q / mf, i = q % mf;
    const size_t base = (size_t)b * d.NF + (rowFar - 1);
    const double* vn = s.vF[0] + 3 * base + k;
    const double* vp = s.vF[4] + 3 * base + k;
    double* tmp = s.vF[6] + 3 * base + k;
    if (phase == 0) {
      double o;
      if (i == 0) o = (vp[0] + vn[0]) * 0.5;
      else if (i < mf - 1) o = (((vp[3 * i] + vp[3 * (i - 1)]) + vn[3 * (i + 1)]) + vn[3 * i]) * 0.25;
      else o = (vp[3 * i] + vn[3 * i]) * 0.5;
      if (i == mf - 1) o = (vp[3 * i] + vn[3 * i]) * 0.5;
      tmp[3 * i] = o;
    } else {
      s.vF[0][3 * base + k + 3 * i] = tmp[3 * i];
    }
  }
}

// ---- targets ----------------------------------------------------------------
constexpr int kTileRows = 16, kTileCols = 4;
__device__ __forceinline__ void decode_node(const Dims& d, int rowNear, int rowFar, int m, int& b, int& far, int& i,
                                            int& j) {
  const int rowsN = d.NW - (rowNear - 1);
  const int rowsF = max(d.NF - (rowFar - 1), 0);
  const int per = rowsN * (d.ns + 1) + rowsF;
  b = m / per;
  const int l = m % per;
  if (l < rowsN * (d.ns + 1)) {
    // tiles of kTileRows rows x kTileCols span stations, tile by tile: a run
    // of 32 consecutive targets (one warp's lanes in the FP32 kernel) is a
    // compact patch of the wake sheet, so few source rings come near any of
    // them
    far = 0;
    const int band = l / (kTileRows * (d.ns + 1));
    const int br = min(kTileRows, rowsN - band * kTileRows);
    const int o = l - band * kTileRows * (d.ns + 1);
    const int tc = o / (br * kTileCols);
    const int q = o - tc * br * kTileCols;
    i = rowNear - 1 + band * kTileRows + q % br;
    j = tc * kTileCols + q / br;
  } else {
    far = 1;
    j = 0;
    i = rowFar - 1 + (l - rowsN * (d.ns + 1));
  }
}
__global__ void k_node_targets(Dims d, DevState s, int rowNear, int rowFar, int pred, int M, double* P) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= M) return;
  int b, far, i, j;
  decode_node(d, rowNear, rowFar, m, b, far, i, j);
  const double* nc = pred ? s.nCP : s.nC;
  d3 p;
  if (!far) p = j < d.ns ? ld3(nc + ringI(d, b, i, j) * 12 + 3) : ld3(nc + ringI(d, b, i, d.ns - 1) * 12 + 6);
  else p = ld3((pred ? s.fCP : s.fC) + ((size_t)b * d.NF + i) * 6);
  st3(P + 3 * (size_t)m, p);
}
__global__ void k_cp_targets(Dims d, const double* fr, double* P) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= d.nbC * d.npan) return;
  st3(P + 3 * (size_t)m, ld3(panRec(d, fr, m / d.npan, m % d.npan) + 12));
}
__global__ void k_scatter_nodes(Dims d, DevState s, const double* fr, int rowNear, int rowFar, int pred,
                                double initWakeVel, int addInit, int M) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= M) return;
  int b, far, i, j;
  decode_node(d, rowNear, rowFar, m, b, far, i, j);
  d3 v = ld3(s.outv + 3 * (size_t)m);
  if (addInit) {
    const d3 a = initWakeVel * ld3(fr + d.fl.rot + 6);
    if (pred || far) v = v - a;
    else v = v + a;
  }
  double* dst = far ? s.vF[pred ? 4 : 0] + 3 * ((size_t)b * d.NF + i) : s.vN[pred ? 4 : 0] + 3 * velI(d, b, i, j);
  st3(dst, v);
}

// ---- source gather ----------------------------------------------------------
// Lattice form of near-wake ring (b, i, j) (i the absolute row): the edge
// weights of its record (see vlm_bs.h).  Ring (i, j-1)'s edge 2 runs from
// its c2 to its c3, which are ring (i, j)'s c1 and c0, so with equal cores
// the two filaments are one with the circulation difference; likewise ring
// (i+1, j)'s edge 3 (its c3 -> c0 = ring (i, j)'s c2 -> c1).  Circulations
// at or below eps count as zero (the skip of blade_vind_bywake,
// src/classdef.f90:1452-1466).
__device__ __forceinline__ bool same3(const double* a, const double* b) {
  return a[0] == b[0] && a[1] == b[1] && a[2] == b[2];
}
__device__ void lattice_weights(const Dims& d, const DevState& s, const double* nc, int b, int i, int j, int rowNear,
                                double* W) {
  auto gam = [&](size_t r) {
    const double g = s.nGam[r];
    return fabs(g) > kEps ? g : 0.0;
  };
  // streamwise edge between stations: ring (i, jj-1) edge 2 == ring (i, jj) edge 0
  auto mergeS = [&](int jj) {
    const size_t a = ringI(d, b, i, jj - 1), c = ringI(d, b, i, jj);
    return same3(nc + 12 * a + 9, nc + 12 * c) && same3(nc + 12 * a + 6, nc + 12 * c + 3) &&
           s.nRvc[4 * a + 2] == s.nRvc[4 * c];
  };
  // spanwise edge between rows: ring (ii, j) edge 1 == ring (ii+1, j) edge 3
  auto mergeC = [&](int ii) {
    const size_t a = ringI(d, b, ii, j), c = ringI(d, b, ii + 1, j);
    return same3(nc + 12 * c, nc + 12 * a + 3) && same3(nc + 12 * c + 9, nc + 12 * a + 6) &&
           s.nRvc[4 * c + 3] == s.nRvc[4 * a + 1];
  };
  const double G = gam(ringI(d, b, i, j));
  W[0] = j > 0 && mergeS(j) ? G - gam(ringI(d, b, i, j - 1)) : G;
  W[1] = i + 1 < d.NW && mergeC(i) ? G - gam(ringI(d, b, i + 1, j)) : G;
  W[2] = j + 1 < d.ns && mergeS(j + 1) ? 0.0 : G;
  W[3] = i > rowNear - 1 && mergeC(i - 1) ? 0.0 : G;
}

__global__ void k_gather(Dims d, DevState s, const double* fr, const Group* groups, int ngroups, int nrec,
                         int rowNear, int rowFar, int pred) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nrec) return;
  int g = 0;
  while (g + 1 < ngroups && t >= groups[g + 1].rec_begin) ++g;
  const Group G = groups[g];
  const int l0 = t - G.rec_begin;
  const int b = G.blade;
  double* R = s.rec64 + (size_t)t * kRec64;
  if (G.kind == 0) {
    const int j = l0 / d.nc, i = l0 % d.nc;
    const int p = i + d.nc * j;
    const double* w = panRec(d, fr, b, p);
    for (int k = 0; k < 12; ++k) R[k] = w[k];
    for (int k = 0; k < 4; ++k) R[12 + k] = s.wRvc[4 * ((size_t)b * d.npan + p) + k];
    R[16] = s.wGam[(size_t)b * d.npan + p];
    R[17] = 0.0;
    if (s.edgeW)
      for (int k = 0; k < 4; ++k) s.edgeW[4 * (size_t)t + k] = R[16];  // wing rings: no eps skip
    return;
  }
  const int rowsN = d.NW - (rowNear - 1);
  const int nNear = rowsN * d.ns;
  const int hs = rowFar <= d.NF ? d.ns : 0;
  const double* nc = pred ? s.nCP : s.nC;
  // a far-only group (pad[0] = 1) lists the far filaments alone, from the
  // pad[1]-th active one
  const int l = G.pad[0] ? l0 + nNear + hs + G.pad[1] : l0;
  if (l < nNear) {
    const int j = l / rowsN, i = rowNear - 1 + l % rowsN;
    const size_t r = ringI(d, b, i, j);
    for (int k = 0; k < 12; ++k) R[k] = nc[12 * r + k];
    for (int k = 0; k < 4; ++k) R[12 + k] = s.nRvc[4 * r + k];
    R[16] = s.nGam[r];
    R[17] = (double)REC_SKIP;
    if (s.edgeW) lattice_weights(d, s, nc, b, i, j, rowNear, s.edgeW + 4 * (size_t)t);
  } else if (l < nNear + hs) {
    const size_t r = ringI(d, b, d.NW - 1, l - nNear);
    for (int k = 0; k < 6; ++k) R[k] = nc[12 * r + 3 + k];
    for (int k = 6; k < 12; ++k) R[k] = 0.0;
    R[12] = s.nRvc[4 * r + 1];
    R[13] = R[14] = R[15] = 0.0;
    R[16] = -s.nGam[r];
    R[17] = (double)REC_FIL;
    if (s.edgeW) {
      double* W = s.edgeW + 4 * (size_t)t;
      W[0] = R[16];
      W[1] = W[2] = W[3] = 0.0;
    }
  } else if (l >= nNear + hs + (rowFar <= d.NF ? d.NF - rowFar + 1 : 0)) {
    // prescribed far wake (classdef.f90:1471-1476): single filaments
    const int i = l - nNear - hs - (d.NF - rowFar + 1);
    const size_t pb = (size_t)pred * d.nb + b;
    const double* f = s.pfC + (pb * kPresc + i) * 6;
    for (int k = 0; k < 6; ++k) R[k] = f[k];
    for (int k = 6; k < 12; ++k) R[k] = 0.0;
    R[12] = s.pfRvc[pb];
    R[13] = R[14] = R[15] = 0.0;
    R[16] = s.pfGam[pb];
    R[17] = (double)(REC_FIL | REC_SKIP);
    if (s.edgeW) {
      double* W = s.edgeW + 4 * (size_t)t;
      W[0] = fabs(R[16]) > kEps ? R[16] : 0.0;
      W[1] = W[2] = W[3] = 0.0;
    }
  } else {
    const size_t f = (size_t)b * d.NF + rowFar - 1 + (l - nNear - hs);
    const double* fc = pred ? s.fCP : s.fC;
    for (int k = 0; k < 6; ++k) R[k] = fc[6 * f + k];
    for (int k = 6; k < 12; ++k) R[k] = 0.0;
    R[12] = s.fRvc[f];
    R[13] = R[14] = R[15] = 0.0;
    R[16] = s.fGam[f];
    R[17] = (double)(REC_FIL | REC_SKIP);
    if (s.edgeW) {
      double* W = s.edgeW + 4 * (size_t)t;
      W[0] = fabs(R[16]) > kEps ? R[16] : 0.0;
      W[1] = W[2] = W[3] = 0.0;
    }
  }
}

// ---- AIC and its inverse (classdef.f90:4151-4179, libMath.f90:48-83) ---------
__global__ void k_aic(Dims d, DevState s, const double* fr) {
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const long n = d.n;
  if (t >= n * n) return;
  const int row = (int)(t % n), col = (int)(t / n);
  const double* cp = panRec(d, fr, row / d.npan, row % d.npan);
  const double* w = panRec(d, fr, col / d.npan, col % d.npan);
  d3 c[4] = {ld3(w), ld3(w + 3), ld3(w + 6), ld3(w + 9)};
  const d3 v = vr_vind64(ld3(cp + 12), c, s.wRvc + 4 * (size_t)col);
  s.AIC[row + n * (size_t)col] = dot3(v, ld3(cp + 15));
}

// Right-looking LU with partial pivoting (first index of max |a|) in one block.
__global__ void k_lu(Dims d, DevState s) {
  const int n = d.n;
  double* A = s.LU;
  __shared__ double redv[1024];
  __shared__ int redi[1024];
  __shared__ int pk;
  for (long e = threadIdx.x; e < (long)n * n; e += blockDim.x) A[e] = s.AIC[e];
  __syncthreads();
  for (int k = 0; k < n; ++k) {
    double bv = -1.0;
    int bi = n;
    for (int i = k + threadIdx.x; i < n; i += blockDim.x) {
      const double v = fabs(A[i + (size_t)n * k]);
      if (v > bv || (v == bv && i < bi)) {
        bv = v;
        bi = i;
      }
    }
    redv[threadIdx.x] = bv;
    redi[threadIdx.x] = bi;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
      if (threadIdx.x < w) {
        const double v = redv[threadIdx.x + w];
        const int i = redi[threadIdx.x + w];
        if (v > redv[threadIdx.x] || (v == redv[threadIdx.x] && i < redi[threadIdx.x])) {
          redv[threadIdx.x] = v;
          redi[threadIdx.x] = i;
        }
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      pk = redi[0];
      s.piv[k] = pk;
      if (A[pk + (size_t)n * k] == 0.0) atomicExch(s.err, 10);
    }
    __syncthreads();
    const int p = pk;
    if (p != k)
      for (int j = threadIdx.x; j < n; j += blockDim.x) {
        const double a = A[k + (size_t)n * j];
        A[k + (size_t)n * j] = A[p + (size_t)n * j];
        A[p + (size_t)n * j] = a;
      }
    __syncthreads();
    const double akk = A[k + (size_t)n * k];
    for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x) A[i + (size_t)n * k] = A[i + (size_t)n * k] / akk;
    __syncthreads();
    const long m = n - k - 1;
    for (long e = threadIdx.x; e < m * m; e += blockDim.x) {
      const int i = k + 1 + (int)(e % m), j = k + 1 + (int)(e / m);
      A[i + (size_t)n * j] = A[i + (size_t)n * j] - A[i + (size_t)n * k] * A[k + (size_t)n * j];
    }
    __syncthreads();
  }
}

// X = A^-1 column by column: forward substitution on P e_c, then backward.
__global__ void k_inv_cols(Dims d, DevState s) {
  const int n = d.n;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const double* A = s.LU;
  double* X = s.AICinv + (size_t)n * c;
  int pos = c;  // position of the 1 in P e_c after the row interchanges
  for (int k = 0; k < n; ++k) {
    const int pk = s.piv[k];
    if (pos == k) pos = pk;
    else if (pos == pk) pos = k;
  }
  for (int i = 0; i < n; ++i) {
    double sum = i == pos ? 1.0 : 0.0;
    for (int k = 0; k < i; ++k) sum = sum - A[i + (size_t)n * k] * X[k];
    X[i] = sum;
  }
  for (int i = n - 1; i >= 0; --i) {
    double sum = X[i];
    for (int k = i + 1; k < n; ++k) sum = sum - A[i + (size_t)n * k] * X[k];
    X[i] = sum / A[i + (size_t)n * i];
  }
}

// ---- FP32 LU + FP64 iterative refinement ---------------------------------------
// The AIC (FP64, assembled once like the reference) is factored in FP32 with
// partial pivoting and inverted in FP32 (one unit column per thread); every
// solve then refines in FP64: x <- x + inv32 (b - A x), the residual b - A x
// in FP64.  ||I - inv32 A|| ~ cond(A) x 2^-24 << 1 for vortex-lattice AICs,
// so each pass gains ~7 digits.
__global__ void k_lu32(Dims d, DevState s) {
  const int n = d.n;
  float* A = s.LU32;
  __shared__ float redv[1024];
  __shared__ int redi[1024];
  __shared__ int pk;
  for (long e = threadIdx.x; e < (long)n * n; e += blockDim.x) A[e] = (float)s.AIC[e];
  __syncthreads();
  for (int k = 0; k < n; ++k) {
    float bv = -1.f;
    int bi = n;
    for (int i = k + threadIdx.x; i < n; i += blockDim.x) {
      const float v = fabsf(A[i + (size_t)n * k]);
      if (v > bv || (v == bv && i < bi)) {
        bv = v;
        bi = i;
      }
    }
    redv[threadIdx.x] = bv;
    redi[threadIdx.x] = bi;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
      if (threadIdx.x < w) {
        const float v = redv[threadIdx.x + w];
        const int i = redi[threadIdx.x + w];
        if (v > redv[threadIdx.x] || (v == redv[threadIdx.x] && i < redi[threadIdx.x])) {
          redv[threadIdx.x] = v;
          redi[threadIdx.x] = i;
        }
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      pk = redi[0];
      s.piv32[k] = pk;
      if (A[pk + (size_t)n * k] == 0.f) atomicExch(s.err, 10);
    }
    __syncthreads();
    const int p = pk;
    if (p != k)
      for (int j = threadIdx.x; j < n; j += blockDim.x) {
        const float t = A[k + (size_t)n * j];
        A[k + (size_t)n * j] = A[p + (size_t)n * j];
        A[p + (size_t)n * j] = t;
      }
    __syncthreads();
    const float akk = A[k + (size_t)n * k];
    for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x) A[i + (size_t)n * k] = A[i + (size_t)n * k] / akk;
    __syncthreads();
    const long m = n - k - 1;
    for (long e = threadIdx.x; e < m * m; e += blockDim.x) {
      const int i = k + 1 + (int)(e % m), j = k + 1 + (int)(e / m);
      A[i + (size_t)n * j] = fmaf(-A[i + (size_t)n * k], A[k + (size_t)n * j], A[i + (size_t)n * j]);
    }
    __syncthreads();
  }
}

__global__ void k_inv32_cols(Dims d, DevState s) {
  const int n = d.n;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const float* A = s.LU32;
  float* X = s.AICinv32 + (size_t)n * c;
  int pos = c;
  for (int k = 0; k < n; ++k) {
    const int pk = s.piv32[k];
    if (pos == k) pos = pk;
    else if (pos == pk) pos = k;
  }
  for (int i = 0; i < n; ++i) {
    float sum = i == pos ? 1.f : 0.f;
    for (int k = 0; k < i; ++k) sum = fmaf(-A[i + (size_t)n * k], X[k], sum);
    X[i] = sum;
  }
  for (int i = n - 1; i >= 0; --i) {
    float sum = X[i];
    for (int k = i + 1; k < n; ++k) sum = fmaf(-A[i + (size_t)n * k], X[k], sum);
    X[i] = sum / A[i + (size_t)n * i];
  }
}

// Solve AIC gamVec = -RHS by refinement (one block); records the final
// relative residual max|b - A x| / max|b| in s.luRes[0] and flags err[1]
// when it stays above 1e-9.
constexpr int kRefinePasses = 3;
__global__ void k_solve_refine(Dims d, DevState s) {
  const int n = d.n;
  __shared__ double red[1024];
  double* b = s.RHS;
  double* x = s.refX;
  double* r = s.refR;
  if (d.axisym)
    for (int i = d.npan + threadIdx.x; i < n; i += blockDim.x) b[i] = b[i % d.npan];
  __syncthreads();
  double bmax = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    b[i] = -1.0 * b[i];
    x[i] = 0.0;
    r[i] = b[i];
    bmax = fmax(bmax, fabs(b[i]));
  }
  red[threadIdx.x] = bmax;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + w]);
    __syncthreads();
  }
  bmax = red[0];
  __syncthreads();
  // one warp per row for both products, lanes over the columns, then a
  // butterfly: latency of n/32 multiply-adds instead of n
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
  double rmax = 0.0;
  for (int pass = 0; pass < kRefinePasses; ++pass) {
    // x += inv32 r  (FP32 products of the FP32-rounded residual, FP64 update)
    for (int i = warp; i < n; i += nwarps) {
      float z = 0.f;
      for (int j = lane; j < n; j += 32) z = fmaf(s.AICinv32[i + (size_t)n * j], (float)r[j], z);
      for (int o = 16; o > 0; o >>= 1) z += __shfl_xor_sync(0xffffffffu, z, o);
      if (lane == 0) x[i] += (double)z;
    }
    __syncthreads();
    // r = b - A x in FP64
    rmax = 0.0;
    for (int i = warp; i < n; i += nwarps) {
      double ax = 0.0;
      for (int j = lane; j < n; j += 32) ax = fma(s.AIC[i + (size_t)n * j], x[j], ax);
      for (int o = 16; o > 0; o >>= 1) ax += __shfl_xor_sync(0xffffffffu, ax, o);
      if (lane == 0) {
        r[i] = b[i] - ax;
        rmax = fmax(rmax, fabs(r[i]));
      }
    }
    __syncthreads();
  }
  red[threadIdx.x] = rmax;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + w]);
    __syncthreads();
  }
  const double rel = bmax > 0.0 ? red[0] / bmax : red[0];
  if (threadIdx.x == 0) {
    s.luRes[0] = rel;
    if (!(rel <= 1e-9)) atomicExch(s.err + 1, 12);
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    s.gamVecPrev[i] = s.gamVec[i];
    s.gamVec[i] = x[i];
  }
  __syncthreads();
  for (int t = threadIdx.x; t < d.nbC * d.npan; t += blockDim.x) s.wGam[t] = s.gamVec[t];
  __syncthreads();
  if (d.axisym)
    for (int t = d.npan + threadIdx.x; t < d.nb * d.npan; t += blockDim.x) s.wGam[t] = s.wGam[t % d.npan];
}

// libMath.f90:428-458 (tolerance 1E-04 single precision)
__global__ void k_is_inverse(Dims d, DevState s) {
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const long n = d.n;
  if (t >= n * n) return;
  const int i = (int)(t % n), j = (int)(t / n);
  double sum = 0.0;
  for (int k = 0; k < n; ++k) sum = sum + s.AIC[i + n * (size_t)k] * s.AICinv[k + n * (size_t)j];
  const double tol = (double)1e-4f;
  const bool bad = (i != j) ? (sum > tol) : (sum - 1.0 > tol);
  if (bad) atomicExch(s.err, 11);
}

// ---- circulation solve (main.f90:522-603) ------------------------------------
__global__ void k_rhs(Dims d, DevState s, const double* fr, int withWake) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= d.nbC * d.npan) return;
  const double* w = panRec(d, fr, t / d.npan, t % d.npan);
  d3 v = ld3(w + 24);
  if (withWake) v = v + ld3(s.outv + 3 * (size_t)t);
  st3(s.velCP + 3 * (size_t)t, v);
  s.RHS[t] = dot3(v, ld3(w + 15));
}
__global__ void k_solve(Dims d, DevState s) {
  const int n = d.n;
  if (d.axisym)
    for (int r = d.npan + threadIdx.x; r < n; r += blockDim.x) s.RHS[r] = s.RHS[r % d.npan];
  __syncthreads();
  for (int r = threadIdx.x; r < n; r += blockDim.x) s.RHS[r] = -1.0 * s.RHS[r];
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    double sum = 0.0;
    for (int j = 0; j < n; ++j) sum = sum + s.AICinv[i + (size_t)n * j] * s.RHS[j];
    s.gamVecPrev[i] = s.gamVec[i];
    s.gamVec[i] = sum;
  }
  __syncthreads();
  for (int r = threadIdx.x; r < d.nbC * d.npan; r += blockDim.x) s.wGam[r] = s.gamVec[r];
  __syncthreads();
  if (d.axisym)
    for (int r = d.npan + threadIdx.x; r < d.nb * d.npan; r += blockDim.x) s.wGam[r] = s.wGam[r % d.npan];
}

// ---- loads (main.f90:623-690, classdef.f90:1704-1896, 2196-2232, 4607-4671) ---
// Chunked (sum_chunk) accumulation of one component, as the oracle's ChunkSum
struct ChunkAcc1 {
  int C, cnt;
  double tot, part;
  __device__ ChunkAcc1(int c) : C(c), cnt(0), tot(0.0), part(0.0) {}
  __device__ void add(double x) {
    if (C <= 0) {
      tot = tot + x;
      return;
    }
    part = part + x;
    if (++cnt == C) {
      tot = tot + part;
      part = 0.0;
      cnt = 0;
    }
  }
  __device__ double result() const { return (C > 0 && cnt > 0) ? tot + part : tot; }
};


// Velocity at collocation point t including the wing's own induced velocity
// minus its bound vortices (src/classdef.f90 calc_force's velCPTotal): one
// block per collocation point.  The block's threads evaluate, batch by
// batch, one stream of items over all blades -- per blade the four filament
// velocities of every panel, then the trailing-edge filament of every
// section (times its circulation), padded to a multiple of 4 -- into shared
// memory, and the terms are formed and added in the reference's
// order: the ring term ((f1 + f2) + f3) + f4 is vr_vind's sum, the bound pair
// f2 + f4 and the trailing-edge f2 are the single-filament calls, all of
// which evaluate the same filament function on the same corners.  Threads
// 0..2 do the ordered sums of the x, y, z components.
constexpr int kVcItems = 256;  // items per batch (a multiple of 4)
// fb (coupled rotors, else null): the bound-vortex velocity of every rotor
// at this rotor's collocation points, [rotor][point][xyz]; the entry of this
// rotor (self) is computed here.  velCPTotal = velCP - bound of every rotor in
// rotor order + this rotor's wing (src/main.f90:636-652).
__global__ void __launch_bounds__(256) k_velcp_total(Dims d, DevState s, const double* fr, int sumChunk,
                                                     const double* fb, int nrs, int self) {
  __shared__ double F[kVcItems * 3];
  const int t = blockIdx.x;
  if (t >= d.nbC * d.npan) return;
  const d3 P = ld3(panRec(d, fr, t / d.npan, t % d.npan) + 12);
  const int nf = 4 * d.npan, nte = (d.ns + 3) & ~3, per = nf + nte;
  const int total = d.nb * per;
  // threads 0..2 each sum one component (the d3 sums are component-wise, so
  // the bits equal those of one thread summing d3 values)
  const int c = threadIdx.x;
  double bound = 0.0, wing = 0.0, sb = 0.0;
  ChunkAcc1 acc(sumChunk);
  for (int i0 = 0; i0 < total; i0 += kVcItems) {
    const int n = min(kVcItems, total - i0);
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const int it = i0 + i, b = it / per, o = it % per;
      d3 v = zero3();
      if (o < nf) {
        const int p = o >> 2, k = o & 3;
        const double* w = panRec(d, fr, b, p);
        v = vf_vind64(make_corner64(P, ld3(w + 3 * k)), make_corner64(P, ld3(w + 3 * ((k + 1) & 3))),
                      s.wRvc[4 * ((size_t)b * d.npan + p) + k]);
      } else if (o - nf < d.ns) {
        const int p = (d.nc - 1) + d.nc * (o - nf);
        const double* w = panRec(d, fr, b, p);
        v = vf_vind64(make_corner64(P, ld3(w + 3)), make_corner64(P, ld3(w + 6)),
                      s.wRvc[4 * ((size_t)b * d.npan + p) + 1]) *
            s.wGam[(size_t)b * d.npan + p];
      }
      st3(F + 3 * i, v);
    }
    __syncthreads();
    if (c < 3) {
      for (int i = 0; i < n;) {
        const int it = i0 + i, b = it / per, o = it % per;
        if (o < nf) {
          const int p = o >> 2;
          const double g = s.wGam[(size_t)b * d.npan + p];
          const double f0 = F[3 * i + c], f1 = F[3 * i + 3 + c], f2 = F[3 * i + 6 + c], f3 = F[3 * i + 9 + c];
          sb = sb + (f1 + f3) * g;
          acc.add((((f0 + f1) + f2) + f3) * g);
          i += 4;
        } else {
          if (o - nf < d.ns) sb = sb - F[3 * i + c];
          if (o == per - 1) {
            // the blade's sums are complete
            bound = bound + sb;
            wing = wing + acc.result();
            sb = 0.0;
            acc = ChunkAcc1(sumChunk);
          }
          i += 1;
        }
      }
    }
    __syncthreads();
  }
  if (c < 3) {
    double v = s.velCP[3 * (size_t)t + c];
    if (fb) {
      const size_t M = (size_t)d.nbC * d.npan;
      for (int jr = 0; jr < nrs; ++jr) v = v - (jr == self ? bound : fb[3 * (jr * M + t) + c]);
    } else {
      v = v - bound;
    }
    v = v + wing;
    s.velCPTotal[3 * (size_t)t + c] = v;
  }
}

// Bound vortices of rotor (ds, ss, frs) at the collocation points of rotor
// (dt, frt) (rotor_vind_bywing_boundVortices, src/classdef.f90:1376-1393,
// 4445-4457): per blade, s = 0, s + (filament 2 + filament 4) gam over the
// panels (spanwise stations outer), s - filament 2 gam of the trailing-edge
// panels, blades added to 0 in order.  One thread per point.
__global__ void k_bound_foreign(Dims dt, const double* frt, Dims ds, DevState ss, const double* frs,
                                double* out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= dt.nbC * dt.npan) return;
  const d3 P = ld3(panRec(dt, frt, t / dt.npan, t % dt.npan) + 12);
  d3 bound = zero3();
  for (int b = 0; b < ds.nb; ++b) {
    d3 sb = zero3();
    for (int p = 0; p < ds.npan; ++p) {
      const double* w = panRec(ds, frs, b, p);
      const double* rv = ss.wRvc + 4 * ((size_t)b * ds.npan + p);
      const double g = ss.wGam[(size_t)b * ds.npan + p];
      const d3 f1 = vf_vind64(make_corner64(P, ld3(w + 3)), make_corner64(P, ld3(w + 6)), rv[1]);
      const d3 f3 = vf_vind64(make_corner64(P, ld3(w + 9)), make_corner64(P, ld3(w)), rv[3]);
      sb = sb + (f1 + f3) * g;
    }
    for (int j = 0; j < ds.ns; ++j) {
      const int p = (ds.nc - 1) + ds.nc * j;
      const double* w = panRec(ds, frs, b, p);
      sb = sb - vf_vind64(make_corner64(P, ld3(w + 3)), make_corner64(P, ld3(w + 6)),
                          ss.wRvc[4 * ((size_t)b * ds.npan + p) + 1]) *
                    ss.wGam[(size_t)b * ds.npan + p];
    }
    bound = bound + sb;
  }
  st3(out + 3 * (size_t)t, bound);
}

// ---- image rotors (src/classdef.f90:4990-5131) ------------------------------
// rotor_mirrorVelCP: the source's velCP with the image-plane component negated
__global__ void k_mirror_velcp(Dims d, DevState s, const double* __restrict__ src, int plane) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= d.nb * d.npan) return;
  for (int c = 0; c < 3; ++c) {
    const double v = src[3 * (size_t)t + c];
    s.velCP[3 * (size_t)t + c] = c == plane - 1 ? -1.0 * v : v;
  }
}
// gamVecPrev = gamVec, rotor_mirrorGamma (gamVec = -source gamVec), map_gam
__global__ void k_mirror_gamma(Dims d, DevState s, const double* __restrict__ src) {
  for (int i = threadIdx.x; i < d.n; i += blockDim.x) {
    s.gamVecPrev[i] = s.gamVec[i];
    s.gamVec[i] = -1.0 * src[i];
  }
  __syncthreads();
  for (int r = threadIdx.x; r < d.nbC * d.npan; r += blockDim.x) s.wGam[r] = s.gamVec[r];
  __syncthreads();
  if (d.axisym)
    for (int r = d.npan + threadIdx.x; r < d.nb * d.npan; r += blockDim.x) s.wGam[r] = s.wGam[r % d.npan];
}
// rotor_mirrorWake: mode 0 the active current wake, 1 the active predicted
// wake (node positions; the predicted wake's circulation and cores are the
// current ones, which already mirror the source's), 2 every row of the
// current wake; node coordinates in the image plane and circulation negated
// (vr_mirror, Fwake_mirror: src/classdef.f90:722-735, 982-993)
__global__ void k_mirror_wake(Dims d, DevState dst, DevState src, int mode, int rowNear, int rowFar, int plane) {
  const int r0 = mode == 2 ? 0 : rowNear - 1, f0 = mode == 2 ? 0 : rowFar - 1;
  const long nNear = (long)d.nb * (d.NW - r0) * d.ns;
  const long nFar = d.NF - f0 > 0 ? (long)d.nb * (d.NF - f0) : 0;
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const int k0 = plane - 1;
  if (t < nNear) {
    const int rows = d.NW - r0;
    const int b = (int)(t / ((long)rows * d.ns)), rem = (int)(t % ((long)rows * d.ns));
    const int j = rem / rows, i = r0 + rem % rows;
    const size_t idx = ringI(d, b, i, j);
    const double* sc = (mode == 1 ? src.nCP : src.nC) + 12 * idx;
    double* dc = (mode == 1 ? dst.nCP : dst.nC) + 12 * idx;
    for (int k = 0; k < 12; ++k) dc[k] = k % 3 == k0 ? -1.0 * sc[k] : sc[k];
    if (mode != 1) {
      dst.nGam[idx] = -1.0 * src.nGam[idx];
      for (int q = 0; q < 4; ++q) dst.nRvc[4 * idx + q] = src.nRvc[4 * idx + q];
      dst.nAge[idx] = src.nAge[idx];
    }
  } else if (t < nNear + nFar) {
    const long u = t - nNear;
    const int b = (int)(u / (d.NF - f0)), i = f0 + (int)(u % (d.NF - f0));
    const size_t f = (size_t)b * d.NF + i;
    const double* sc = (mode == 1 ? src.fCP : src.fC) + 6 * f;
    double* dc = (mode == 1 ? dst.fCP : dst.fC) + 6 * f;
    for (int k = 0; k < 6; ++k) dc[k] = k % 3 == k0 ? -1.0 * sc[k] : sc[k];
    if (mode != 1) {
      dst.fGam[f] = -1.0 * src.fGam[f];
      dst.fRvc[f] = src.fRvc[f];
      dst.fRvc0[f] = src.fRvc0[f];
      dst.fL0[f] = src.fL0[f];
      dst.fLc[f] = src.fLc[f];
      dst.fAge[f] = src.fAge[f];
    }
  }
}

// velCP = kinematic velocity + each term in turn (coupled rotors:
// src/main.f90:549-561, the wake of every rotor and the wing of the others,
// one per-rotor sum per term); RHS = velCP . nCap
__global__ void k_rhs_terms(Dims d, DevState s, const double* fr, const double* terms, int nterms, int M) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= d.nbC * d.npan) return;
  const double* w = panRec(d, fr, t / d.npan, t % d.npan);
  d3 v = ld3(w + 24);
  for (int k = 0; k < nterms; ++k) v = v + ld3(terms + 3 * ((size_t)k * M + t));
  st3(s.velCP + 3 * (size_t)t, v);
  s.RHS[t] = dot3(v, ld3(w + 15));
}

// libMath.f90:293-426 (Doolittle inverse of lsq2's 3x3 normal matrix; its
// pivot search never swaps rows for these matrices)
__device__ void inv3_doolittle(const double* A, double* X) {
  double L[9], U[9];
  for (int k = 0; k < 9; ++k) L[k] = U[k] = 0.0;
  auto at = [](int i, int j) { return i + 3 * j; };
  for (int j = 0; j < 3; ++j) U[at(0, j)] = A[at(0, j)];
  for (int i = 0; i < 3; ++i) L[at(i, 0)] = A[at(i, 0)] / A[at(0, 0)];
  for (int i = 1; i < 3; ++i)
    for (int j = 1; j < 3; ++j) {
      double su = 0.0, sl = 0.0;
      for (int k = 0; k < i; ++k) {
        su = su + L[at(i, k)] * U[at(k, j)];
        sl = sl + L[at(j, k)] * U[at(k, i)];
      }
      U[at(i, j)] = A[at(i, j)] - su;
      if (fabs(U[at(i, i)]) > kEps) L[at(j, i)] = (A[at(j, i)] - sl) / U[at(i, i)];
    }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      if (i > j) U[at(i, j)] = 0.0;
      else if (j > i) L[at(i, j)] = 0.0;
    }
  for (int bb = 0; bb < 3; ++bb) {
    double Pb[3], dd[3], x[3];
    for (int i = 0; i < 3; ++i) {
      double sum = 0.0;
      for (int k = 0; k < 3; ++k) sum = sum + (i == k ? 1.0 : 0.0) * (k == bb ? 1.0 : 0.0);
      Pb[i] = sum;
    }
    dd[0] = Pb[0];
    for (int i = 1; i < 3; ++i) {
      double sum = 0.0;
      for (int k = 0; k < i; ++k) sum = sum + L[at(i, k)] * dd[k];
      dd[i] = Pb[i] - sum;
    }
    x[2] = dd[2] / U[at(2, 2)];
    for (int i = 1; i >= 0; --i) {
      double sum = 0.0;
      for (int k = i + 1; k < 3; ++k) sum = sum + U[at(i, k)] * x[k];
      x[i] = (dd[i] - sum) / U[at(i, i)];
    }
    for (int i = 0; i < 3; ++i) X[at(i, bb)] = x[i];
  }
}

// libMath.f90:577-605
__device__ double lsq2_dev(double xq, const double* xd, const double* yd, int n) {
  double s1 = 0, s2 = 0, s3 = 0, s4 = 0, r1 = 0, r2 = 0, r3 = 0;
  for (int i = 0; i < n; ++i) {
    const double x = xd[i];
    s1 = s1 + x;
    s2 = s2 + x * x;
    s3 = s3 + (x * x) * x;
    s4 = s4 + pow4(x);
    r1 = r1 + yd[i];
    r2 = r2 + yd[i] * x;
    r3 = r3 + yd[i] * (x * x);
  }
  const double A[9] = {(double)n, s1, s2, s1, s2, s3, s2, s3, s4};
  double Ai[9];
  inv3_doolittle(A, Ai);
  double c[3];
  for (int i = 0; i < 3; ++i) c[i] = Ai[i] * r1 + Ai[i + 3] * r2 + Ai[i + 6] * r3;
  return c[0] + c[1] * xq + (c[2] * xq) * xq;
}

constexpr int kMaxNc = 64;

__global__ void k_step_begin(Dims d, DevState s) {
  const int it = s.devIter[0] + 1;
  const double* src = s.frames + (size_t)it * d.fl.size;
  for (int i = threadIdx.x; i < d.fl.size; i += blockDim.x) s.curFrame[i] = src[i];
  __syncthreads();
  if (threadIdx.x == 0) s.devIter[0] = it;
}

// ---- airfoil tables (libC81.f90:190-351) ------------------------------------
// interval of x in the ascending axis A[0..n): 1-based (i1, i2) as the
// reference's binary search leaves them, ends snapped within the
// single-precision epsilon
__device__ void c81_interval(const double* A, int n, double x, int& i1, int& i2) {
  i1 = 1;
  i2 = n;
  while (i1 != i2 && i2 != i1 + 1) {
    const int i = (i1 + i2) / 2;
    if (x < A[i - 1]) i2 = i;
    else if (x > A[i - 1]) i1 = i;
    else i1 = i2 = i;
  }
  const double epsf = 1.1920928955078125e-07;  // epsilon(1.) of the default real kind
  if (fabs(A[i1 - 1] - x) <= epsf) i2 = i1;
  else if (fabs(A[i2 - 1] - x) <= epsf) i1 = i2;
}
// coefficient c (0 lift, 1 drag, 2 moment) of table T at (alpha degrees, Mach)
__device__ double c81_get(const double* T, int c, double alpha, double mach) {
  size_t o = 6;
  int nm = 0, na = 0;
  for (int k = 0; k <= c; ++k) {
    nm = (int)T[2 * k];
    na = (int)T[2 * k + 1];
    if (k < c) o += (size_t)nm + na + (size_t)nm * na;
  }
  const double* Ma = T + o;
  const double* A = Ma + nm;
  const double* C = A + na;
  int a1, a2, m1, m2;
  c81_interval(A, na, alpha, a1, a2);
  c81_interval(Ma, nm, mach, m1, m2);
  auto v = [&](int i, int j) { return C[(i - 1) + (size_t)na * (j - 1)]; };
  if (a1 == a2) {
    if (m1 == m2) return v(a1, m1);
    return v(a1, m1) + ((mach - Ma[m1 - 1]) * (v(a1, m2) - v(a1, m1))) / (Ma[m2 - 1] - Ma[m1 - 1]);
  }
  if (m1 == m2) return v(a1, m1) + ((alpha - A[a1 - 1]) * (v(a2, m1) - v(a1, m1))) / (A[a2 - 1] - A[a1 - 1]);
  const double y2m = Ma[m2 - 1] - mach, my1 = mach - Ma[m1 - 1];
  const double lo = v(a1, m1) * y2m + v(a1, m2) * my1;
  const double hi = v(a2, m1) * y2m + v(a2, m2) * my1;
  const double num = (A[a2 - 1] - alpha) * lo + (alpha - A[a1 - 1]) * hi;
  return num / (A[a2 - 1] - A[a1 - 1]) / (Ma[m2 - 1] - Ma[m1 - 1]);
}

__global__ void k_loads(Dims d, DevState s, const double* fr, int iter) {
  if (iter < 0) iter = s.devIter[0];
  const int nsec = d.nbC * d.ns;
  const double iGS = -1.0 * fsign1(d.omega);
  // phase A: sectional resultant velocity and lift/drag directions
  for (int t = threadIdx.x; t < nsec; t += blockDim.x) {
    const int b = t / d.ns, is = t % d.ns;
    const double* sec = fr + d.fl.sec + ((size_t)b * d.ns + is) * kSec;
    const d3 secTauC = ld3(sec), secCP = ld3(sec + 6), pc1 = ld3(sec + 9);
    d3 rv;
    if (d.nc >= 3) {
      double xd[kMaxNc], yd[kMaxNc];
      d3 crv[kMaxNc];
      for (int ic = 0; ic < d.nc; ++ic) {
        const int p = ic + d.nc * is;
        const double* w = panRec(d, fr, b, p);
        crv[ic] = noproj3(ld3(s.velCPTotal + 3 * ((size_t)b * d.npan + p)), ld3(w + 21));
        xd[ic] = dot3(ld3(w + 12) - pc1, secTauC);
      }
      const double xq = dot3(secCP - pc1, secTauC);
      double o[3];
      for (int k = 0; k < 3; ++k) {
        for (int ic = 0; ic < d.nc; ++ic) yd[ic] = k == 0 ? crv[ic].x : (k == 1 ? crv[ic].y : crv[ic].z);
        o[k] = lsq2_dev(xq, xd, yd, d.nc);
      }
      rv = mk3(o[0], o[1], o[2]);
    } else {
      d3 sum = zero3();
      for (int ic = 0; ic < d.nc; ++ic) {
        const int p = ic + d.nc * is;
        const double* w = panRec(d, fr, b, p);
        sum = sum + noproj3(ld3(s.velCPTotal + 3 * ((size_t)b * d.npan + p)), ld3(w + 21));
      }
      rv = sum / (double)d.nc;
    }
    st3(s.secResVel + 3 * (size_t)t, rv);
    const d3 dd = unit3(rv);
    const d3 yAF = ld3(fr + d.fl.ax + 9 * b + 3);
    st3(s.secDragDir + 3 * (size_t)t, dd);
    st3(s.secLiftDir + 3 * (size_t)t, fsign1(d.omega) * unit3(cross3(dd, yAF)));
  }
  __syncthreads();
  // phase B with airfoil tables (forceCalcSwitch 1: blade_calc_force_alpha,
  // src/classdef.f90:2091-2105, 2146-2195, 2234-2250): sectional angle of
  // attack from the resultant velocity, CL and CD from the section's table
  // at that angle and Mach number, lift along the lift direction, the
  // inertial force along y x V with the sign of the section's circulation;
  // the sectional drag stays zero (the reference never assigns it here) and
  // the panel pressures and gamPrev are not computed.
  for (int t = threadIdx.x; d.forceCalc == 1 && t < nsec; t += blockDim.x) {
    const int b = t / d.ns, is = t % d.ns;
    const double* sec = fr + d.fl.sec + ((size_t)b * d.ns + is) * kSec;
    const d3 rv = ld3(s.secResVel + 3 * (size_t)t);
    const double alpha = atan2(dot3(rv, ld3(sec + 3)), dot3(rv, ld3(sec)));
    const double m = norm3(rv);
    const double* T = s.c81 + s.c81Off[s.airfoilNo[t]];
    const double aDeg = alpha * kRad2Deg, mach = m / d.velSound;
    const double cl = c81_get(T, 0, aDeg, mach);
    const double cd = c81_get(T, 1, aDeg, mach);
    const double lead = ((0.5 * d.density) * (m * m)) * s.secArea[t];
    const d3 liftDir = ld3(s.secLiftDir + 3 * (size_t)t);
    const d3 sL = (liftDir * lead) * cl;
    const d3 sLU = (liftDir * lead) * 0.0;
    double gs = 0.0;
    for (int ic = 0; ic < d.nc; ++ic) gs = gs + s.wGam[(size_t)b * d.npan + ic + d.nc * is];
    const d3 yAF = ld3(fr + d.fl.ax + 9 * b + 3);
    d3 fi = fsign1(gs) * unit3(cross3(yAF, rv));
    fi = norm3(sL) * fi;
    fi = fi + 0.0 * unit3(rv);
    st3(s.secForceInertial + 3 * (size_t)t, fi);
    st3(s.secLift + 3 * (size_t)t, sL);
    st3(s.secLiftUnsteady + 3 * (size_t)t, sLU);
    s.secCL[t] = cl;
    s.secCD[t] = cd;
    s.secCLu[t] = 0.0;
  }
  // phase B: panel pressures and sectional forces (blade_calc_force)
  for (int t = threadIdx.x; d.forceCalc != 1 && t < nsec; t += blockDim.x) {
    const int b = t / d.ns, is = t % d.ns;
    const d3 liftDir = ld3(s.secLiftDir + 3 * (size_t)t);
    d3 sFI = zero3(), sL = zero3(), sLU = zero3();
    for (int ic = 0; ic < d.nc; ++ic) {
      const int p = ic + d.nc * is;
      const size_t gp = (size_t)b * d.npan + p;
      const double* w = panRec(d, fr, b, p);
      const d3 velCP = ld3(s.velCP + 3 * gp);
      const double vTC = dot3(velCP, ld3(w + 18));
      const double vTS = dot3(velCP, ld3(w + 21));
      const double g = s.wGam[gp];
      double gEC = ic == 0 ? g : g - s.wGam[gp - 1];
      double gES = is == 0 ? g : g - s.wGam[gp - d.nc];
      gEC = iGS * gEC;
      gES = iGS * gES;
      const double gamTrapz = ic > 0 ? (iGS * 0.5) * (g + s.wGam[gp - 1]) : (iGS * 0.5) * g;
      const double delPU = d.density * (gamTrapz - s.gamPrev[gp]) / d.dt;
      double delP = delPU + d.density * vTC * gEC / s.panMeanChord[gp];
      if (d.spanwiseLift != 0) delP = delP + d.density * vTS * gES / s.panMeanSpan[gp];
      s.gamPrev[gp] = gamTrapz;
      const d3 nCap = ld3(w + 15);
      const d3 nF = (delP * s.panArea[gp]) * nCap;
      const d3 nFU = (delPU * s.panArea[gp]) * nCap;
      sFI = sFI + nF;
      sL = sL + proj3(nF, liftDir);
      sLU = sLU + proj3(nFU, liftDir);
    }
    const d3 xAF = ld3(fr + d.fl.ax + 9 * b), zAF = ld3(fr + d.fl.ax + 9 * b + 6);
    st3(s.secForceInertial + 3 * (size_t)t, sFI);
    st3(s.secLift + 3 * (size_t)t, sL);
    st3(s.secLiftUnsteady + 3 * (size_t)t, sLU);
    st3(s.secLiftInPlane + 3 * (size_t)t, iGS * proj3(sL, xAF));
    st3(s.secLiftOutPlane + 3 * (size_t)t, proj3(sL, zAF));
    const double m = norm3(ld3(s.secResVel + 3 * (size_t)t));
    const double q = (0.5 * d.density) * (m * m);
    const double area = s.secArea[(size_t)b * d.ns + is];
    if (fabs(q) > kEps) {
      const double sg = fsign1(dot3(sL, zAF));
      s.secCL[t] = norm3(sL) * sg / (q * area);
      s.secCD[t] = 0.0 / (q * area);
      s.secCLu[t] = norm3(sLU) * sg / (q * area);
    } else {
      s.secCL[t] = s.secCD[t] = s.secCLu[t] = 0.0;
    }
  }
  __syncthreads();
  // phase C: blade sums (blade_sumSecToNetForces)
  for (int b = threadIdx.x; b < d.nbC; b += blockDim.x) {
    d3 fi = zero3(), li = zero3(), lu = zero3();
    for (int is = 0; is < d.ns; ++is) {
      const size_t t = (size_t)b * d.ns + is;
      fi = fi + ld3(s.secForceInertial + 3 * t);
      li = li + ld3(s.secLift + 3 * t);
      lu = lu + ld3(s.secLiftUnsteady + 3 * t);
    }
    st3(s.bladeForce + 12 * (size_t)b, fi);
    st3(s.bladeForce + 12 * (size_t)b + 3, li);
    st3(s.bladeForce + 12 * (size_t)b + 6, zero3());
    st3(s.bladeForce + 12 * (size_t)b + 9, lu);
  }
  __syncthreads();
  // phase D: rotor sums and the CT row (rotor_sumBladeToNetForces, force2file)
  if (threadIdx.x == 0) {
    d3 FI = zero3(), L = zero3(), LU = zero3();
    if (d.axisym) {
      const double nbd = (double)d.nb;
      FI = nbd * ld3(s.bladeForce);
      L = nbd * ld3(s.bladeForce + 3);
      LU = nbd * ld3(s.bladeForce + 9);
    } else {
      for (int b = 0; b < d.nbC; ++b) {
        FI = FI + ld3(s.bladeForce + 12 * (size_t)b);
        L = L + ld3(s.bladeForce + 12 * (size_t)b + 3);
        LU = LU + ld3(s.bladeForce + 12 * (size_t)b + 9);
      }
    }
    st3(s.rotorLift, L);
    st3(s.rotorLift + 3, FI);
    const double D = d.nonDimDenom;
    const double sl = fsign1(dot3(L, ld3(fr + d.fl.rot)));
    double* row = s.ctHist + 10 * (size_t)iter;
    row[0] = (double)iter;
    row[1] = sl * norm3(L) / D;
    row[2] = 0.0 / D;
    row[3] = norm3(LU) / D;
    row[4] = 0.0 / D;
    row[5] = 0.0 / D;
    row[6] = 0.0 / D;
    row[7] = FI.x / D;
    row[8] = FI.y / D;
    row[9] = FI.z / D;
  }
}

}  // namespace

// ---------------------------------------------------------------------------
void launch_shed(const Dims& d, const DevState& s, const double* frame, int rowNear, bool le, cudaStream_t st) {
  count_launch();
  k_shed<<<nblk(d.nb * d.ns, 128), 128, 0, st>>>(d, s, frame, rowNear, le ? 1 : 0);
}
void launch_age(const Dims& d, const DevState& s, int rowNear, int rowFar, cudaStream_t st) {
  const long n = (long)d.nb * (d.NW - (rowNear - 1)) * d.ns + (long)d.nb * (d.NF - (rowFar - 1) > 0 ? d.NF - (rowFar - 1) : 0);
  if (n > 0) {
    count_launch();
    k_age<<<nblk(n, 256), 256, 0, st>>>(d, s, rowNear, rowFar);
  }
}
void launch_dissipate(const Dims& d, const DevState& s, int rowNear, int rowFar, cudaStream_t st) {
  const long n = (long)d.nb * (d.NW - (rowNear - 1)) * d.ns + (long)d.nb * (d.NF - (rowFar - 1) > 0 ? d.NF - (rowFar - 1) : 0);
  if (n > 0) {
    count_launch();
    k_dissip_a<<<nblk(n, 256), 256, 0, st>>>(d, s, rowNear, rowFar);
  }
  const long n2 = (long)d.nb * (d.NW - rowNear) * d.ns;
  if (n2 > 0) {
    count_launch();
    k_dissip_b<<<nblk(n2, 256), 256, 0, st>>>(d, s, rowNear);
  }
}
void launch_copy_predicted(const Dims& d, const DevState& s, int rowNear, int rowFar, cudaStream_t st) {
  const long n = (long)d.nbC * (d.NW - (rowNear - 1)) * d.ns + (long)d.nbC * (d.NF - (rowFar - 1) > 0 ? d.NF - (rowFar - 1) : 0);
  if (n > 0) {
    count_launch();
    k_copy_pred<<<nblk(n, 256), 256, 0, st>>>(d, s, rowNear, rowFar);
  }
}
void launch_convect(const Dims& d, const DevState& s, const double* frame, int rowNear, int rowFar, bool pred,
                    cudaStream_t st) {
  const int rowsF = d.NF - (rowFar - 1) > 0 ? d.NF - (rowFar - 1) : 0;
  const long n1 = (long)d.nbC * (pred ? 1 : d.NW - (rowNear - 1)) * (d.ns + 1) + (long)d.nbC * rowsF;
  if (n1 > 0) {
    count_launch();
    k_shift<<<nblk(n1, 256), 256, 0, st>>>(d, s, rowNear, rowFar, pred ? 1 : 0);
  }
  const long n2 = (long)d.nbC * (d.NW - (rowNear - 1)) * d.ns + (long)d.nbC * (d.NF - rowFar > 0 ? d.NF - rowFar : 0);
  if (n2 > 0) {
    count_launch();
    k_continuity<<<nblk(n2, 256), 256, 0, st>>>(d, s, rowNear, rowFar, pred ? 1 : 0);
  }
  if (d.axisym && d.nb > 1) {
    const long n3 = (long)(d.nb - 1) * (d.NW - (rowNear - 1)) * d.ns + (long)(d.nb - 1) * rowsF;
    if (n3 > 0) {
      count_launch();
      k_axisym<<<nblk(n3, 256), 256, 0, st>>>(d, s, frame, rowNear, rowFar, pred ? 1 : 0);
    }
  }
}
void launch_presc_update(const Dims& d, const DevState& s, const double* frame, int rowFar, bool pred,
                         cudaStream_t st) {
  if (!s.pfC || d.NF - (rowFar - 1) < 1) return;
  count_launch();
  k_presc_update<<<d.nbC, 256, 0, st>>>(d, s, frame, rowFar, pred ? 1 : 0);
  if (d.axisym && d.nb > 1) {
    count_launch();
    k_presc_axisym<<<nblk((long)(d.nb - 1) * kPresc, 256), 256, 0, st>>>(d, s, frame, pred ? 1 : 0);
  }
}
void launch_burst(const Dims& d, const DevState& s, int rowFar, cudaStream_t st) {
  const long n = (long)d.nb * (d.NF - (rowFar - 1) - 1);
  if (n > 0) {
    count_launch();
    k_burst<<<nblk(n, 256), 256, 0, st>>>(d, s, rowFar);
  }
}
void launch_strain(const Dims& d, const DevState& s, int rowFar, cudaStream_t st) {
  const long n = (long)d.nb * (d.NF - (rowFar - 1));
  if (n > 0) {
    count_launch();
    k_strain<<<nblk(n, 256), 256, 0, st>>>(d, s, rowFar);
  }
}
void launch_rollup(const Dims& d, const DevState& s, int rowFar, cudaStream_t st) {
  int rowFarNext = rowFar - 1;
  if (d.NF > 0 && rowFarNext == 0) {
    const long n = (long)d.nb * d.NF;
    count_launch();
    k_far_to_tmp<<<nblk(n, 256), 256, 0, st>>>(d, s);
    count_launch();
    k_far_from_tmp<<<nblk(n, 256), 256, 0, st>>>(d, s);
    rowFarNext = 1;
  }
  count_launch();
  k_rollup<<<nblk(d.nb, 32), 32, 0, st>>>(d, s, rowFarNext);
  const long n = (long)d.nb * d.NW * d.ns;
  count_launch();
  k_near_to_tmp<<<nblk(n, 256), 256, 0, st>>>(d, s);
  count_launch();
  k_near_from_tmp<<<nblk(n, 256), 256, 0, st>>>(d, s);
}
void launch_velop(const Dims& d, const DevState& s, VelOp op, cudaStream_t st) {
  const long nN = (long)d.nbC * d.NW * (d.ns + 1) * 3, nF = (long)d.nbC * d.NF * 3;
  if (nN + nF > 0) {
    count_launch();
    k_velop<<<nblk(nN + nF, 256), 256, 0, st>>>(s, nN, nF, (int)op);
  }
}
void launch_order2(const Dims& d, const DevState& s, int rowNear, int rowFar, cudaStream_t st) {
  const long n = (long)d.nbC * (d.ns + 1) * (d.NW - (rowNear - 1)) * 3 +
                 (long)d.nbC * (d.NF - (rowFar - 1) > 0 ? d.NF - (rowFar - 1) : 0) * 3;
  if (n <= 0) return;
  count_launch();
  k_order2<<<nblk(n, 256), 256, 0, st>>>(d, s, rowNear, rowFar, 0);
  count_launch();
  k_order2<<<nblk(n, 256), 256, 0, st>>>(d, s, rowNear, rowFar, 1);
}
int node_target_count(const Dims& d, int rowNear, int rowFar) {
  const int rowsN = d.NW - (rowNear - 1);
  const int rowsF = d.NF - (rowFar - 1) > 0 ? d.NF - (rowFar - 1) : 0;
  return d.nbC * (rowsN * (d.ns + 1) + rowsF);
}
void launch_node_targets(const Dims& d, const DevState& s, int rowNear, int rowFar, bool pred, double* P,
                         cudaStream_t st) {
  const int M = node_target_count(d, rowNear, rowFar);
  if (M > 0) {
    count_launch();
    k_node_targets<<<nblk(M, 256), 256, 0, st>>>(d, s, rowNear, rowFar, pred ? 1 : 0, M, P);
  }
}
void launch_cp_targets(const Dims& d, const double* frame, double* P, cudaStream_t st) {
  count_launch();
  k_cp_targets<<<nblk(d.nbC * d.npan, 128), 128, 0, st>>>(d, frame, P);
}
void launch_gather(const Dims& d, const DevState& s, const double* frame, const Group* groups, int ngroups, int nrec,
                   int rowNear, int rowFar, bool pred, cudaStream_t st) {
  if (nrec > 0) {
    count_launch();
    k_gather<<<nblk(nrec, 256), 256, 0, st>>>(d, s, frame, groups, ngroups, nrec, rowNear, rowFar, pred ? 1 : 0);
  }
}
void launch_scatter_nodes(const Dims& d, const DevState& s, const double* frame, int rowNear, int rowFar, bool pred,
                          double initWakeVel, cudaStream_t st) {
  const int M = node_target_count(d, rowNear, rowFar);
  const int addInit = initWakeVel != 0.0 ? 1 : 0;
  if (M > 0)
    count_launch();
    k_scatter_nodes<<<nblk(M, 256), 256, 0, st>>>(d, s, frame, rowNear, rowFar, pred ? 1 : 0, initWakeVel, addInit, M);
}
void launch_aic(const Dims& d, const DevState& s, const double* frame, cudaStream_t st) {
  const long n = (long)d.n * d.n;
  count_launch();
  k_aic<<<nblk(n, 128), 128, 0, st>>>(d, s, frame);
}
void launch_lu_inverse(const Dims& d, const DevState& s, cudaStream_t st) {
  count_launch();
  k_lu<<<1, 1024, 0, st>>>(d, s);
  count_launch();
  k_inv_cols<<<nblk(d.n, 64), 64, 0, st>>>(d, s);
}
void launch_is_inverse(const Dims& d, const DevState& s, cudaStream_t st) {
  const long n = (long)d.n * d.n;
  count_launch();
  k_is_inverse<<<nblk(n, 256), 256, 0, st>>>(d, s);
}
void launch_solve(const Dims& d, const DevState& s, const double* frame, bool withWake, cudaStream_t st) {
  count_launch();
  k_rhs<<<nblk(d.nbC * d.npan, 128), 128, 0, st>>>(d, s, frame, withWake ? 1 : 0);
  count_launch();
  if (s.LU32) k_solve_refine<<<1, 1024, 0, st>>>(d, s);
  else k_solve<<<1, 1024, 0, st>>>(d, s);
}
void launch_lu32(const Dims& d, const DevState& s, cudaStream_t st) {
  count_launch();
  k_lu32<<<1, 1024, 0, st>>>(d, s);
  count_launch();
  k_inv32_cols<<<nblk(d.n, 64), 64, 0, st>>>(d, s);
}
void launch_step_begin(const Dims& d, const DevState& s, cudaStream_t st) {
  count_launch();
  k_step_begin<<<1, 256, 0, st>>>(d, s);
}
void launch_rhs_terms(const Dims& d, const DevState& s, const double* frame, const double* terms, int nterms,
                      cudaStream_t st) {
  count_launch();
  k_rhs_terms<<<nblk(d.nbC * d.npan, 128), 128, 0, st>>>(d, s, frame, terms, nterms, d.nbC * d.npan);
}
void launch_mirror_velcp(const Dims& d, const DevState& s, const double* srcVelCP, int plane, cudaStream_t st) {
  count_launch();
  k_mirror_velcp<<<nblk(d.nb * d.npan, 128), 128, 0, st>>>(d, s, srcVelCP, plane);
}
void launch_mirror_gamma(const Dims& d, const DevState& s, const double* srcGamVec, cudaStream_t st) {
  count_launch();
  k_mirror_gamma<<<1, 1024, 0, st>>>(d, s, srcGamVec);
}
void launch_mirror_wake(const Dims& d, const DevState& dst, const DevState& src, int mode, int rowNear, int rowFar,
                        int plane, cudaStream_t st) {
  const int r0 = mode == 2 ? 0 : rowNear - 1, f0 = mode == 2 ? 0 : rowFar - 1;
  const long n = (long)d.nb * (d.NW - r0) * d.ns + (d.NF - f0 > 0 ? (long)d.nb * (d.NF - f0) : 0);
  if (n <= 0) return;
  count_launch();
  k_mirror_wake<<<nblk(n, 256), 256, 0, st>>>(d, dst, src, mode, rowNear, rowFar, plane);
}
void launch_solve_only(const Dims& d, const DevState& s, cudaStream_t st) {
  count_launch();
  if (s.LU32) k_solve_refine<<<1, 1024, 0, st>>>(d, s);
  else k_solve<<<1, 1024, 0, st>>>(d, s);
}
void launch_bound_foreign(const Dims& dt, const double* frameT, const Dims& ds, const DevState& ss,
                          const double* frameS, double* out, cudaStream_t st) {
  count_launch();
  k_bound_foreign<<<nblk(dt.nbC * dt.npan, 64), 64, 0, st>>>(dt, frameT, ds, ss, frameS, out);
}
void launch_loads(const Dims& d, const DevState& s, const double* frame, int sumChunk, int iter, cudaStream_t st,
                  const double* foreignBound, int nrs, int self) {
  count_launch();
  k_velcp_total<<<d.nbC * d.npan, 256, 0, st>>>(d, s, frame, sumChunk, foreignBound, nrs, self);
  count_launch();
  k_loads<<<1, 256, 0, st>>>(d, s, frame, iter);
}

}  // namespace vlm
