// TEST INFRASTRUCTURE ONLY -- the oracle.
//
// CPU FP64 restatement of VOLCANOR's free-wake unsteady vortex-lattice path
// (reference: cibinjoseph/VOLCANOR, Fortran 2008 + OpenMP).  Only tests/,
// __graft_entry__.smoke() and bench.py's cpu_baseline / reference legs may load
// this library, and only as the checker or the timed CPU baseline.  The product
// (volcanor_gb300/) never links it.
//
// The data model mirrors the reference's derived types one to one:
//   vf_class  (src/classdef.f90:57-79)   -> VF
//   vr_class  (src/classdef.f90:81-104)  -> VR  (4 filaments + gam)
//   wingpanel (src/classdef.f90:106-179) -> WingPanel
//   Fwake     (src/classdef.f90:198-220) -> FW
//   blade     (src/classdef.f90:238-358) -> Blade
//   rotor     (src/classdef.f90:360-467) -> Rotor
// Panel and wake arrays are column major like Fortran: wiP(i,j) -> [i + nc*j],
// waN(i,j) -> [i + nNwake*j] (0-based).
//
// Arithmetic conventions (a fixed, documented choice, because the reference's
// own rounding depends on its compiler's contraction and intrinsic choices):
//   * every Fortran operation is one IEEE double operation; this file is
//     compiled with -ffp-contract=off, so no fused multiply-adds appear;
//   * dot_product / sum / norm2 / matmul accumulate left to right from the
//     first term (norm2 = sqrt of that sum);
//   * x**2._dp = x*x, x**3._dp = (x*x)*x, x**4._dp = (x*x)*(x*x);
//   * the explicit inverse (LAPACK DGETRF+DGETRI in src/libMath.f90:48-83) is
//     a right-looking LU with partial pivoting (first index of max |a|), then
//     one forward/backward substitution per unit column;
//   * DGEMV (src/libMath.f90:105-122) is a sequential dot product per row.
// Summation order of every Biot-Savart sum follows the reference loops exactly.
// Parity with the reference is pinned by the golden vectors of its own unit
// tests (tests/*_test.f90) and full-case CT histories (tests/*.case).

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <limits>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

const double PI = 3.14159265358979323846;          // atan(1._dp)*4._dp
const double EPS = 2.220446049250313080847e-16;    // epsilon(1._dp)
const double TWO_PI = 2.0 * PI;
const double DEG2RAD = PI / 180.0;
const double RAD2DEG = 180.0 / PI;
const double INV4PI = 0.25 / PI;                   // classdef.f90:13

struct V3 {
  double x = 0, y = 0, z = 0;
};
inline V3 mk(double a, double b, double c) { V3 r; r.x = a; r.y = b; r.z = c; return r; }
inline V3 operator+(V3 a, V3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 operator-(V3 a, V3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 operator*(double s, V3 a) { return mk(s * a.x, s * a.y, s * a.z); }
inline V3 operator*(V3 a, double s) { return mk(a.x * s, a.y * s, a.z * s); }
inline V3 operator/(V3 a, double s) { return mk(a.x / s, a.y / s, a.z / s); }
inline V3 neg(V3 a) { return mk(-a.x, -a.y, -a.z); }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline double norm2(V3 a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
inline double sumsq(V3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
// libMath.f90:202-212
inline V3 cross(V3 a, V3 b) {
  return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
// libMath.f90:249-262
inline V3 unitVec(V3 a) {
  double n = norm2(a);
  if (n > EPS) return a / n;
  return V3();
}
// libMath.f90:264-276
inline V3 projVec(V3 a, V3 d) {
  double ns = sumsq(d);
  if (ns > EPS) {
    double k = dot(a, d);
    return mk((k * d.x) / ns, (k * d.y) / ns, (k * d.z) / ns);
  }
  return V3();
}
// libMath.f90:278-291
inline V3 noProjVec(V3 a, V3 d) {
  double ns = sumsq(d);
  if (ns > EPS) {
    double k = dot(a, d);
    return mk(a.x - (k * d.x) / ns, a.y - (k * d.y) / ns, a.z - (k * d.z) / ns);
  }
  return a;
}
inline double fsign(double a, double b) { return std::signbit(b) ? -std::fabs(a) : std::fabs(a); }
inline double p4(double x) { double x2 = x * x; return x2 * x2; }

struct M3 {
  double a[3][3];
};
inline V3 mv(const M3& T, V3 v) {
  return mk(T.a[0][0] * v.x + T.a[0][1] * v.y + T.a[0][2] * v.z,
            T.a[1][0] * v.x + T.a[1][1] * v.y + T.a[1][2] * v.z,
            T.a[2][0] * v.x + T.a[2][1] * v.y + T.a[2][2] * v.z);
}
inline V3 rotAbout(const M3& T, V3 p, V3 o) { return mv(T, p - o) + o; }

// libMath.f90:695-726
M3 getTransformAxis(double theta, V3 axisVec) {
  double n = norm2(axisVec);
  V3 ax = axisVec / n;
  double ct = std::cos(theta), st = std::sin(theta), omct = 1.0 - ct;
  M3 T;
  T.a[0][0] = ct + (ax.x * ax.x) * omct;
  T.a[1][0] = ax.z * st + (ax.y * ax.x) * omct;
  T.a[2][0] = -(ax.y * st) + (ax.z * ax.x) * omct;
  T.a[0][1] = -(ax.z * st) + (ax.x * ax.y) * omct;
  T.a[1][1] = ct + (ax.y * ax.y) * omct;
  T.a[2][1] = ax.x * st + (ax.z * ax.y) * omct;
  T.a[0][2] = ax.y * st + (ax.x * ax.z) * omct;
  T.a[1][2] = -(ax.x * st) + (ax.y * ax.z) * omct;
  T.a[2][2] = ct + (ax.z * ax.z) * omct;
  return T;
}
// libMath.f90:672-693 (cs = cos, sin pairs)
M3 Tgb(double cph, double sph, double cth, double sth, double cps, double sps) {
  M3 T;
  T.a[0][0] = cps * cth;
  T.a[0][1] = (sph * sth) * cps - sps * cph;
  T.a[0][2] = sph * sps + (sth * cph) * cps;
  T.a[1][0] = sps * cth;
  T.a[1][1] = (sph * sps) * sth + cph * cps;
  T.a[1][2] = (sps * sth) * cph - sph * cps;
  T.a[2][0] = -sth;
  T.a[2][1] = sph * cth;
  T.a[2][2] = cph * cth;
  return T;
}
M3 TgbAngles(V3 pts) {
  return Tgb(std::cos(pts.x), std::sin(pts.x), std::cos(pts.y), std::sin(pts.y),
             std::cos(pts.z), std::sin(pts.z));
}

// libMath.f90:138-200
std::vector<double> linspace(double a, double b, int n) {
  std::vector<double> x(n);
  double dx = (b - a) / double(n - 1);
  for (int i = 0; i < n; ++i) x[i] = double(i) * dx + a;
  return x;
}
std::vector<double> cosspace(double a, double b, int n) {
  auto th = linspace(0.0, PI, n);
  std::vector<double> x(n);
  for (int i = 0; i < n; ++i) x[i] = a + ((b - a) * 0.5) * (1.0 - std::cos(th[i]));
  return x;
}
std::vector<double> halfsinspace(double a, double b, int n) {
  auto th = linspace(0.0, PI * 0.5, n);
  std::vector<double> x(n);
  for (int i = 0; i < n; ++i) x[i] = a + (b - a) * std::sin(th[i]);
  return x;
}
std::vector<double> tanspace(double a, double b, int n) {
  const double tl = 1.2;
  auto th = linspace(-tl, tl, n);
  std::vector<double> x(n);
  for (int i = 0; i < n; ++i) x[i] = a + ((b - a) * std::tan(th[i])) / std::tan(tl);
  return x;
}

// libMath.f90:476-517
double pwl_interp1d(const std::vector<double>& x, const std::vector<double>& y, double q) {
  size_t n = x.size();
  if (std::fabs(x[0] - q) < EPS) return y[0];
  if (std::fabs(x[n - 1] - q) < EPS) return y[n - 1];
  std::vector<int> t(n);
  if (x[0] < x[n - 1]) {
    for (size_t i = 0; i < n; ++i) t[i] = x[i] <= q;
  } else if (x[0] > x[n - 1]) {
    for (size_t i = 0; i < n; ++i) t[i] = x[i] >= q;
  } else {
    throw std::runtime_error("pwl_interp1d: neither ascending nor descending");
  }
  bool all = true, none = true;
  for (size_t i = 0; i < n; ++i) { all = all && t[i]; none = none && !t[i]; }
  if (all || none) throw std::runtime_error("pwl_interp1d: out of range");
  size_t idx = 0;
  for (size_t i = 0; i < n; ++i) if (!t[i]) { idx = i - 1; break; }
  return y[idx] + (y[idx + 1] - y[idx]) / (x[idx + 1] - x[idx]) * (q - x[idx]);
}

// libMath.f90:520-575, order 2: Lagrange interpolation through the two or
// three table points around xq (x ascending; xq within the table).
double interp1d2(double xq, const std::vector<double>& x, const std::vector<double>& y) {
  const int n = (int)x.size();
  int ix = -1;
  for (int i = 0; i < n; ++i)
    if (xq <= x[i]) { ix = i; break; }
  if (ix < 0) throw std::runtime_error("interp1d: query beyond the table");
  if (std::fabs(xq - x[ix]) <= EPS) return y[ix];
  if (ix == 0) throw std::runtime_error("interp1d: query before the table");
  if (std::sqrt(y[ix - 1] * y[ix - 1] + y[ix] * y[ix]) <= EPS) return 0.0;
  if (n == 2) return y[ix - 1] + (xq - x[ix - 1]) * (y[ix] - y[ix - 1]) / (x[ix] - x[ix - 1]);
  int a, b, c;
  if (ix == 1) { a = 0; b = 1; c = 2; }
  else { a = ix - 2; b = ix - 1; c = ix; }
  const double L0 = (xq - x[b]) * (xq - x[c]) / ((x[a] - x[b]) * (x[a] - x[c]));
  const double L1 = (xq - x[a]) * (xq - x[c]) / ((x[b] - x[a]) * (x[b] - x[c]));
  const double L2 = (xq - x[a]) * (xq - x[b]) / ((x[c] - x[a]) * (x[c] - x[b]));
  return y[a] * L0 + y[b] * L1 + y[c] * L2;
}

// libMath.f90:293-426 -- native Doolittle inverse used by lsq2.  Its pivot
// search compares the ORIGINAL matrix against the running maximum, so for the
// matrices lsq2 builds it never swaps a row; the literal search is kept.
std::vector<double> invDoolittle(const std::vector<double>& A, int n) {
  auto at = [n](int i, int j) { return i + n * j; };
  std::vector<double> Ad = A, P(n * n, 0.0), L(n * n, 0.0), U(n * n, 0.0), Ainv(n * n, 0.0);
  for (int i = 0; i < n; ++i) P[at(i, i)] = 1.0;
  for (int j = 0; j < n; ++j) {
    double mx = Ad[at(j, j)];
    for (int i = j + 1; i < n; ++i) mx = std::max(mx, Ad[at(i, j)]);
    for (int i = j; i < n; ++i) {
      if (A[at(i, j)] - mx < EPS) {
        for (int k = 0; k < n; ++k) { std::swap(P[at(i, k)], P[at(j, k)]); std::swap(Ad[at(i, k)], Ad[at(j, k)]); }
        break;
      }
    }
  }
  for (int j = 0; j < n; ++j) U[at(0, j)] = Ad[at(0, j)];
  for (int i = 0; i < n; ++i) L[at(i, 0)] = Ad[at(i, 0)] / Ad[at(0, 0)];
  for (int i = 1; i < n; ++i) {
    for (int j = 1; j < n; ++j) {
      double sumu = 0.0, suml = 0.0;
      for (int k = 0; k < i; ++k) {
        sumu = sumu + L[at(i, k)] * U[at(k, j)];
        suml = suml + L[at(j, k)] * U[at(k, i)];
      }
      U[at(i, j)] = Ad[at(i, j)] - sumu;
      if (std::fabs(U[at(i, i)]) > EPS) L[at(j, i)] = (Ad[at(j, i)] - suml) / U[at(i, i)];
    }
  }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      if (i > j) U[at(i, j)] = 0.0;
      else if (j > i) L[at(i, j)] = 0.0;
    }
  for (int i = 0; i < n; ++i)
    if (std::fabs(U[at(i, i)]) < EPS) throw std::runtime_error("inv: matrix is singular or ill-conditioned");
  std::vector<double> Pb(n), d(n), x(n);
  for (int bb = 0; bb < n; ++bb) {
    for (int i = 0; i < n; ++i) {
      double s = 0.0;
      for (int k = 0; k < n; ++k) s = s + P[at(i, k)] * (k == bb ? 1.0 : 0.0);
      Pb[i] = s;
    }
    d[0] = Pb[0];
    for (int i = 1; i < n; ++i) {
      double s = 0.0;
      for (int k = 0; k < i; ++k) s = s + L[at(i, k)] * d[k];
      d[i] = Pb[i] - s;
    }
    x[n - 1] = d[n - 1] / U[at(n - 1, n - 1)];
    for (int i = n - 2; i >= 0; --i) {
      double s = 0.0;
      for (int k = i + 1; k < n; ++k) s = s + U[at(i, k)] * x[k];
      x[i] = (d[i] - s) / U[at(i, i)];
    }
    for (int i = 0; i < n; ++i) Ainv[at(i, bb)] = x[i];
  }
  return Ainv;
}

// libMath.f90:577-605
double lsq2(double xq, const std::vector<double>& xd, const std::vector<double>& yd) {
  size_t n = xd.size();
  double s1 = 0, s2 = 0, s3 = 0, s4 = 0, r1 = 0, r2 = 0, r3 = 0;
  for (size_t i = 0; i < n; ++i) {
    double x = xd[i];
    s1 = s1 + x;
    s2 = s2 + x * x;
    s3 = s3 + (x * x) * x;
    s4 = s4 + p4(x);
    r1 = r1 + yd[i];
    r2 = r2 + yd[i] * x;
    r3 = r3 + yd[i] * (x * x);
  }
  std::vector<double> A = {double(n), s1, s2, s1, s2, s3, s2, s3, s4};  // column major, symmetric
  auto Ai = invDoolittle(A, 3);
  double c[3];
  for (int i = 0; i < 3; ++i) c[i] = Ai[i + 0] * r1 + Ai[i + 3] * r2 + Ai[i + 6] * r3;
  return c[0] + c[1] * xq + (c[2] * xq) * xq;
}

// libMath.f90:224-236
double getAngleTan(V3 a, V3 b) {
  double ma = sumsq(a), mb = sumsq(b), d = dot(a, b);
  return std::atan2(std::sqrt(ma * mb - d * d), d);
}

// ---------------------------------------------------------------------------
// Data model
struct VF {            // classdef.f90:57-79
  V3 fc1, fc2;         // fc(:,1), fc(:,2)
  double l0 = 0, lc = 0, rVc0 = 0, rVc = 0, age = 0, ageAz = 0;
};
struct VR {            // classdef.f90:81-104
  VF vf[4];
  double gam = 0, skew = 0;
  // classdef.f90:556-579
  void assignP(int n, V3 P) {
    switch (n) {
      case 1: vf[3].fc2 = P; vf[0].fc1 = P; break;
      case 2: vf[0].fc2 = P; vf[1].fc1 = P; break;
      case 3: vf[1].fc2 = P; vf[2].fc1 = P; break;
      case 4: vf[2].fc2 = P; vf[3].fc1 = P; break;
    }
  }
  // classdef.f90:581-610
  void shiftdP(int n, V3 d) {
    switch (n) {
      case 1: vf[3].fc2 = vf[3].fc2 + d; vf[0].fc1 = vf[0].fc1 + d; break;
      case 2: vf[0].fc2 = vf[0].fc2 + d; vf[1].fc1 = vf[1].fc1 + d; break;
      case 3: vf[1].fc2 = vf[1].fc2 + d; vf[2].fc1 = vf[2].fc1 + d; break;
      case 4: vf[2].fc2 = vf[2].fc2 + d; vf[3].fc1 = vf[3].fc1 + d; break;
    }
  }
  // classdef.f90:612-628
  void rot(const M3& T, V3 o) {
    for (int i = 0; i < 4; ++i) { vf[i].fc1 = rotAbout(T, vf[i].fc1, o); vf[i].fc2 = rotAbout(T, vf[i].fc2, o); }
  }
  // classdef.f90:505-515 (isOriginal=.true. also records l0)
  void calclength(bool orig) {
    for (int i = 0; i < 4; ++i) {
      double l = norm2(vf[i].fc1 - vf[i].fc2);
      vf[i].lc = l;
      if (orig) vf[i].l0 = l;
    }
  }
};

// classdef.f90:476-503 -- unit-strength filament, Vatistas n=2 core.
inline V3 vf_vind(const VF& f, V3 P) {
  V3 r1 = P - f.fc1, r2 = P - f.fc2, r0 = r1 - r2;
  V3 c = cross(r1, r2);
  double c2 = dot(c, c);
  if (c2 > EPS * EPS) {
    V3 du = unitVec(r1) - unitVec(r2);
    double d = dot(r0, du);
    double a = f.rVc * norm2(r0);
    double den = std::sqrt(p4(a) + c2 * c2);
    return mk(((c.x * INV4PI) * d) / den, ((c.y * INV4PI) * d) / den, ((c.z * INV4PI) * d) / den);
  }
  return V3();
}
// classdef.f90:527-542 -- sum(vindMat, 1) over the 4 filaments in order.
inline V3 vr_vind(const VR& r, V3 P) {
  V3 v = vf_vind(r.vf[0], P);
  v = v + vf_vind(r.vf[1], P);
  v = v + vf_vind(r.vf[2], P);
  v = v + vf_vind(r.vf[3], P);
  return v;
}

// Deterministic chunked summation.  chunk <= 0 reproduces the reference's
// sequential accumulation exactly; chunk = C splits a blade's source sequence
// into consecutive blocks of C records (skipped records still count), sums
// each block from zero and adds the block sums in order.  The GPU FP64 path
// uses the same order, so both produce identical bits for the same C.
struct ChunkSum {
  int C;
  int cnt = 0;
  V3 tot, part;
  explicit ChunkSum(int c) : C(c) {}
  void add(V3 x) {
    if (C <= 0) { tot = tot + x; return; }
    part = part + x;
    tick();
  }
  void tick() {
    if (C > 0 && ++cnt == C) { tot = tot + part; part = V3(); cnt = 0; }
  }
  V3 result() const { return (C > 0 && cnt > 0) ? tot + part : tot; }
};

struct FW {            // classdef.f90:198-220
  VF vf;
  double gam = 0;
};

// classdef.f90:222-236 -- prescribed far wake: a helix of 240 filaments (10
// revolutions) fitted to the free far wake and attached at its oldest node
struct PFwake {
  std::vector<FW> waF = std::vector<FW>(240);
  double nRevs = 10.0, helixPitch = 0.0, helixRadius = 0.0, relaxFactor = 0.5;
  bool isClockwiseRotor = true, isPresent = false;
};

struct WingPanel {     // classdef.f90:106-179
  VR vr;
  double gamPrev = 0, gamTrapz = 0;
  V3 PC[4];
  V3 CP, nCap, tauCapChord, tauCapSpan, velCP, velCPTotal, velCPm, normalForce, normalForceUnsteady, chordwiseResVel;
  double delP = 0, delPUnsteady = 0, meanChord = 0, meanSpan = 0, panelArea = 0, rHinge = 0;
  // classdef.f90:782-797
  void calcCP() { CP = ((PC[0] + PC[3]) * 0.25 + (PC[1] + PC[2]) * 0.75) * 0.5; }
  // classdef.f90:799-815
  void calcN() { nCap = unitVec(cross(PC[2] - PC[0], PC[3] - PC[1])); }
  // classdef.f90:823-841
  void calcTau() {
    tauCapChord = unitVec(((PC[1] + PC[2]) - (PC[0] + PC[3])) * 0.5);
    tauCapSpan = unitVec(((PC[2] + PC[3]) - (PC[1] + PC[0])) * 0.5);
  }
  // classdef.f90:843-859
  void rot(const M3& T, V3 o) {
    for (int i = 0; i < 4; ++i) PC[i] = rotAbout(T, PC[i], o);
    vr.rot(T, o);
    CP = rotAbout(T, CP, o);
    nCap = mv(T, nCap);
    tauCapChord = mv(T, tauCapChord);
    tauCapSpan = mv(T, tauCapSpan);
  }
  // classdef.f90:861-873
  void shiftdP(V3 d) {
    CP = CP + d;
    for (int i = 0; i < 4; ++i) { PC[i] = PC[i] + d; vr.shiftdP(i + 1, d); }
  }
  // classdef.f90:875-880
  void calc_area() { panelArea = 0.5 * norm2(cross(PC[2] - PC[0], PC[3] - PC[1])); }
  // classdef.f90:882-889
  void calc_mean_dimensions() {
    meanSpan = 0.5 * (norm2(PC[3] - PC[0]) + norm2(PC[2] - PC[1]));
    meanChord = 0.5 * (norm2(PC[1] - PC[0]) + norm2(PC[2] - PC[3]));
  }
};

// An airfoil table (libC81.f90:6-30): CL, CD, CM over angle of attack
// (degrees) x Mach; C?(i, j) stored at i + N? * j.
struct C81 {
  int ML = 0, NL = 0, MD = 0, ND = 0, MM = 0, NM = 0;
  std::vector<double> MaL, MaD, MaM, AL, AD, AM, CL, CD, CM;

  // one Fortran Fw.0 input field of `w` characters at `pos` (blank: 0)
  static double fld(const std::string& line, size_t pos, size_t w) {
    if (pos >= line.size()) return 0.0;
    std::string f = line.substr(pos, w);
    size_t a = f.find_first_not_of(' ');
    if (a == std::string::npos) return 0.0;
    return std::strtod(f.c_str() + a, nullptr);
  }
  // libC81.f90:128-188: A30,6I2 header; per coefficient a Mach line
  // (7X,9F7.0) and per angle a line (10F7.0: angle + 9 values), with a
  // (7X,nF7.0) continuation line when there are more than 9 Mach numbers
  void read(const std::string& path) {
    std::ifstream f(path);
    if (!f) throw std::runtime_error("cannot open C81 file " + path);
    std::vector<std::string> L;
    for (std::string line; std::getline(f, line);) {
      if (!line.empty() && line.back() == '\r') line.pop_back();
      L.push_back(line);
    }
    size_t k = 0;
    auto next = [&]() -> const std::string& {
      if (k >= L.size()) throw std::runtime_error("C81 file ends early: " + path);
      return L[k++];
    };
    const std::string& h = next();
    int* dims[6] = {&ML, &NL, &MD, &ND, &MM, &NM};
    for (int i = 0; i < 6; ++i) *dims[i] = (int)fld(h, 30 + 2 * i, 2);
    auto block = [&](int M, int N, std::vector<double>& Ma, std::vector<double>& A, std::vector<double>& C) {
      if (M < 1 || N < 1 || M > 18) throw std::runtime_error("C81 table dimensions out of range: " + path);
      Ma.assign(M, 0.0);
      A.assign(N, 0.0);
      C.assign((size_t)M * N, 0.0);
      const std::string& m1 = next();
      for (int j = 0; j < std::min(9, M); ++j) Ma[j] = fld(m1, 7 + 7 * j, 7);
      if (M > 9) {
        const std::string& m2 = next();
        for (int j = 9; j < M; ++j) Ma[j] = fld(m2, 7 + 7 * (j - 9), 7);
      }
      for (int i = 0; i < N; ++i) {
        const std::string& r1 = next();
        A[i] = fld(r1, 0, 7);
        for (int j = 0; j < std::min(9, M); ++j) C[i + (size_t)N * j] = fld(r1, 7 + 7 * j, 7);
        if (M > 9) {
          const std::string& r2 = next();
          for (int j = 9; j < M; ++j) C[i + (size_t)N * j] = fld(r2, 7 + 7 * (j - 9), 7);
        }
      }
    };
    block(ML, NL, MaL, AL, CL);
    block(MD, ND, MaD, AD, CD);
    block(MM, NM, MaM, AM, CM);
  }
  // libC81.f90:302-332 (1-based indices out); the end tests use the
  // single-precision epsilon(1.)
  static void interval(const std::vector<double>& A, double x, int& i1, int& i2) {
    const int n = (int)A.size();
    i1 = 1;
    i2 = n;
    while (i1 != i2 && i2 != i1 + 1) {
      const int i = (int)std::floor(double(float(i1 + i2) * 0.5f));
      if (x < A[i - 1]) i2 = i;
      else if (x > A[i - 1]) i1 = i;
      else i1 = i2 = i;
    }
    const double epsf = (double)std::numeric_limits<float>::epsilon();
    if (std::fabs(A[i1 - 1] - x) <= epsf) i2 = i1;
    else if (std::fabs(A[i2 - 1] - x) <= epsf) i1 = i2;
  }
  // getCL / getCD / getCM (libC81.f90:190-300) with getBilinearInterp (:334-351)
  static double lookup(const std::vector<double>& A, const std::vector<double>& Ma, const std::vector<double>& C,
                       double alpha, double mach) {
    const int N = (int)A.size();
    int a1, a2, m1, m2;
    interval(A, alpha, a1, a2);
    interval(Ma, mach, m1, m2);
    auto c = [&](int i, int j) { return C[(i - 1) + (size_t)N * (j - 1)]; };
    if (a1 == a2) {
      if (m1 == m2) return c(a1, m1);
      return c(a1, m1) + ((mach - Ma[m1 - 1]) * (c(a1, m2) - c(a1, m1))) / (Ma[m2 - 1] - Ma[m1 - 1]);
    }
    if (m1 == m2) return c(a1, m1) + ((alpha - A[a1 - 1]) * (c(a2, m1) - c(a1, m1))) / (A[a2 - 1] - A[a1 - 1]);
    const double x1 = A[a1 - 1], x2 = A[a2 - 1], y1 = Ma[m1 - 1], y2 = Ma[m2 - 1];
    const double v1 = y2 - mach, v2 = mach - y1;
    const double r1 = c(a1, m1) * v1 + c(a1, m2) * v2;
    const double r2 = c(a2, m1) * v1 + c(a2, m2) * v2;
    double g = (x2 - alpha) * r1 + (alpha - x1) * r2;
    g = g / (x2 - x1) / (y2 - y1);
    return g;
  }
  double getCL(double a, double m) const { return lookup(AL, MaL, CL, a, m); }
  double getCD(double a, double m) const { return lookup(AD, MaD, CD, a, m); }
  double getCM(double a, double m) const { return lookup(AM, MaM, CM, a, m); }
};

struct Blade {         // classdef.f90:238-358
  int nc = 0, ns = 0;
  std::vector<WingPanel> wiP;     // [i + nc*j]
  std::vector<VR> waN, waNP;      // [i + NW*j]
  std::vector<FW> waF, waFP;
  PFwake wapF, wapFP;  // prescribed far wake of the free wake and of the predicted wake
  double theta = 0, psi = 0, pivotLE = 0, preconeAngle = 0;
  double flap = 0, dflap = 0, flapPrev = 0, dflapPrev = 0, MflapLift = 0, MflapLiftPrev = 0;
  V3 flapOrigin, forceInertial, lift, drag, dragInduced, dragProfile, liftUnsteady, dragUnsteady;
  V3 xAxis, yAxis, zAxis, xAxisAzi, yAxisAzi, zAxisAzi, xAxisAziFlap, yAxisAziFlap, zAxisAziFlap;
  // velocity arrays (3, nNwake, ns+1) -> [(i + NW*j)] and (3, nFwake)
  std::vector<V3> velN, velN1, velN2, velN3, velNP, velNStep;
  std::vector<V3> velF, velF1, velF2, velF3, velFP, velFStep;
  std::vector<V3> secTauCapChord, secTauCapSpan, secNormalVec, secForceInertial, secLift, secLiftDir,
      secDragDir, secLiftInPlane, secLiftOutPlane, secLiftInPlaneUnsteady, secLiftOutPlaneUnsteady,
      secLiftUnsteady, secDrag, secDragInduced, secDragProfile, secDragUnsteady, secChordwiseResVel, secCP;
  std::vector<double> secChord, secArea, secAlpha, secPhi, secTheta, secViz, secVix, secCL, secCD, secCLu,
      secMflap, secMflapArm, secCM;
  std::vector<int> airfoilNo;  // 1-based airfoil table of each section
  int spanwiseLiftSwitch = 0;

  WingPanel& w(int i, int j) { return wiP[i + nc * j]; }
  const WingPanel& w(int i, int j) const { return wiP[i + nc * j]; }
};

struct Rotor {
  // readGeom inputs (classdef.f90:2541-2767)
  int surfaceType = 0, imagePlane = 0, imageRotorNum = 0;
  int nb = 1, propConvention = 0, spanSpacing = 1, chordSpacing = 1, nCamberFiles = 0, nc = 1, ns = 1, nNwake = 0;
  std::string geometryFile = "0";
  V3 hubCoords, cgCoords, fromCoords, pts;
  double radius = 0, root_cut = 0, chord = 0, preconeAngle = 0, Omega = 0, omegaSlow = 0;
  V3 shaftAxis, velBody, omegaBody, controlPitch;
  // customTrajectorySwitch = 1: body velocity and rates of every step
  // (velBodyHistory, omegaBodyHistory; classdef.f90:3065-3081)
  std::vector<V3> velBodyHistory, omegaBodyHistory;
  // camber sections (CAMBERSECTIONS namelist, classdef.f90:2614-2687)
  std::vector<double> camberSectionLimit;
  std::vector<std::string> camberFile;
  double thetaTwist = 0;
  int ductSwitch = 0, axisymmetrySwitch = 0, spanwiseLiftSwitch = 0, symmetricTau = 0;
  int customTrajectorySwitch = 0, forceCalcSwitch = 0, nAirfoils = 0;
  std::vector<double> airfoilSectionLimit, alpha0v;
  std::vector<std::string> airfoilFile;
  std::vector<C81> c81;
  double pivotLE = 0, flapHinge = 0;
  double apparentViscCoeff = 0, decayCoeff = 0, spanwiseCore = 0;
  int wakeTruncateNt = 0, prescWakeAfterTruncNt = 0, prescWakeGenNt = 0, prescWakeNt = 0;
  std::vector<double> streamwiseCoreVec;
  double rollupStartRadius = 0, rollupEndRadius = 0, initWakeVel = 0, psiStart = 0, skewLimit = 0;
  int bladeDynamicsSwitch = 0, pitchDynamicsSwitch = 0, bodyDynamicsSwitch = 0, bodyDynamicsIOVars = 0;
  double flapInitial = 0, dflapInitial = 0, Iflap = 0, cflap = 0, kflap = 0, MflapConstant = 0, dpitch = 0;
  int inflowPlotSwitch = 0, gammaPlotSwitch = 0, skewPlotSwitch = 0;
  // derived
  int nFwake = 0, nbConvect = 1, nNwakeEnd = 0, nFwakeEnd = 0, rowNear = 0, rowFar = 0;
  int rollupStart = 0, rollupEnd = 0, suppressFwakeSwitch = 0;
  V3 xAxisBody, yAxisBody, zAxisBody;
  double psi = 0, nonDimforceDenominator = 0;
  V3 forceInertial, lift, liftPrev, drag, dragInduced, dragProfile, liftUnsteady, dragUnsteady;
  std::vector<Blade> blade;
  std::vector<double> AIC, AIC_inv, gamVec, gamVecPrev, RHS;
  int n() const { return nc * ns * nb; }
};

struct Switches {       // classdef.f90:16-55
  int ntSub = 0, ntSubInit = 0, wakeDissipation = 0, wakeStrain = 0, wakeBurst = 0, wakeSuppress = 0;
  int slowStart = 0, slowStartNt = 0, wakeTipPlot = 0, wakePlot = 0, gridPlot = 0, rotorForcePlot = 1;
  int fdScheme = 0, probe = 0, initWakeVelNt = 0, restartFromNt = 0, restartWriteNt = 0;
};

// ---------------------------------------------------------------------------
// Namelist reader (Fortran namelist subset used by config.nml / geomXX.nml)
struct Namelist {
  std::map<std::string, std::vector<std::string>> kv;  // "group.key" lowercase
  static std::string lower(std::string s) {
    for (auto& c : s) c = (char)std::tolower((unsigned char)c);
    return s;
  }
  void parse(const std::string& text) {
    std::string group;
    std::string body;
    // strip comments (outside quotes)
    std::string clean;
    bool inq = false;
    char q = 0;
    for (size_t i = 0; i < text.size(); ++i) {
      char c = text[i];
      if (inq) { clean += c; if (c == q) inq = false; continue; }
      if (c == '\'' || c == '"') { inq = true; q = c; clean += c; continue; }
      if (c == '!') { while (i < text.size() && text[i] != '\n') ++i; clean += '\n'; continue; }
      clean += c;
    }
    // tokenise
    std::vector<std::string> tok;
    std::string cur;
    inq = false;
    auto flush = [&]() { if (!cur.empty()) { tok.push_back(cur); cur.clear(); } };
    for (size_t i = 0; i < clean.size(); ++i) {
      char c = clean[i];
      if (inq) { if (c == q) { inq = false; tok.push_back("\x01" + cur); cur.clear(); } else cur += c; continue; }
      if (c == '\'' || c == '"') { flush(); inq = true; q = c; continue; }
      if (std::isspace((unsigned char)c) || c == ',') { flush(); continue; }
      if (c == '=' || c == '/') { flush(); tok.push_back(std::string(1, c)); continue; }
      if (c == '&') { flush(); cur += c; continue; }
      cur += c;
    }
    flush();
    std::string key;
    for (size_t i = 0; i < tok.size(); ++i) {
      const std::string& t = tok[i];
      if (!t.empty() && t[0] == '&') { group = lower(t.substr(1)); key.clear(); continue; }
      if (t == "/") { group.clear(); key.clear(); continue; }
      if (group.empty()) continue;
      if (i + 1 < tok.size() && tok[i + 1] == "=") { key = lower(t); kv[group + "." + key].clear(); ++i; continue; }
      if (key.empty()) continue;
      std::string v = t;
      if (!v.empty() && v[0] == '\x01') { kv[group + "." + key].push_back(v.substr(1)); continue; }
      size_t star = v.find('*');
      int rep = 1;
      if (star != std::string::npos) { rep = std::atoi(v.substr(0, star).c_str()); v = v.substr(star + 1); }
      for (int r = 0; r < rep; ++r) kv[group + "." + key].push_back(v);
    }
  }
  bool has(const std::string& g, const std::string& k) const { return kv.count(lower(g) + "." + lower(k)) > 0; }
  static double todouble(std::string s) {
    for (auto& c : s) if (c == 'd' || c == 'D') c = 'e';
    return std::strtod(s.c_str(), nullptr);
  }
  double d(const std::string& g, const std::string& k, double def = 0.0, size_t idx = 0) const {
    auto it = kv.find(lower(g) + "." + lower(k));
    if (it == kv.end() || it->second.size() <= idx) return def;
    return todouble(it->second[idx]);
  }
  int i(const std::string& g, const std::string& k, int def = 0) const {
    auto it = kv.find(lower(g) + "." + lower(k));
    if (it == kv.end() || it->second.empty()) return def;
    return (int)std::lround(todouble(it->second[0]));
  }
  std::string s(const std::string& g, const std::string& k, const std::string& def = "0", size_t idx = 0) const {
    auto it = kv.find(lower(g) + "." + lower(k));
    if (it == kv.end() || it->second.size() <= idx) return def;
    return it->second[idx];
  }
  V3 v3(const std::string& g, const std::string& k) const { return mk(d(g, k, 0, 0), d(g, k, 0, 1), d(g, k, 0, 2)); }
  size_t count(const std::string& g, const std::string& k) const {
    auto it = kv.find(lower(g) + "." + lower(k));
    return it == kv.end() ? 0 : it->second.size();
  }
};

std::string readFile(const std::string& path) {
  std::ifstream f(path);
  if (!f) throw std::runtime_error("cannot open " + path);
  std::stringstream ss;
  ss << f.rdbuf();
  return ss.str();
}

// ---------------------------------------------------------------------------
struct Sim {
  // config (libCommon.f90:51-108)
  int nt = 0, nr = 1;
  double dt = 0, density = 1, velSound = 330, kinematicVisc = 0;
  Switches sw;
  Rotor R;
  std::string baseDir;
  int iter = 0;
  double t = 0;
  std::vector<std::vector<double>> ctHist;  // rows of [iter, CL/CT, CD, CLu, CDi, CD0, CDu, CFx, CFy, CFz]
  int nthreads = 0;
  int sumChunk = 0;  // see ChunkSum
  bool started = false;
  // Rotors of a coupled system (nr > 1, main.f90:17-29), in rotor order,
  // this one at index self; empty for a lone rotor.  Every induced-velocity
  // sum over "all rotors" of the reference's loop runs over sys.
  std::vector<Sim*> sys;
  int self = 0;
  bool member = false;  // created as a rotor of a system: nr > 1 allowed
  // an image rotor (surfaceType -1): the rotor it mirrors, initialised first
  // (its parameters, classdef.f90:2797-2910, and its initial normals)
  const Sim* imageOf = nullptr;
  static double& comp(V3& v, int k) { return k == 1 ? v.x : (k == 2 ? v.y : v.z); }

  // ---- blade kinematics -------------------------------------------------
  // classdef.f90:1092-1112
  void blade_move(Blade& b, V3 d) {
    for (int j = 0; j < b.ns; ++j)
      for (int i = 0; i < b.nc; ++i) b.w(i, j).shiftdP(d);
    for (auto& s : b.secCP) s = s + d;
    b.flapOrigin = b.flapOrigin + d;
  }
  // classdef.f90:1114-1158
  void blade_rot_pts(Blade& b, V3 p, V3 o) {
    M3 T = TgbAngles(p);
    for (int j = 0; j < b.ns; ++j) {
      for (int i = 0; i < b.nc; ++i) b.w(i, j).rot(T, o);
      b.secCP[j] = rotAbout(T, b.secCP[j], o);
      b.secTauCapChord[j] = mv(T, b.secTauCapChord[j]);
      b.secNormalVec[j] = mv(T, b.secNormalVec[j]);
    }
    V3* ax[9] = {&b.xAxis, &b.yAxis, &b.zAxis, &b.xAxisAzi, &b.yAxisAzi, &b.zAxisAzi,
                 &b.xAxisAziFlap, &b.yAxisAziFlap, &b.zAxisAziFlap};
    for (auto a : ax) *a = mv(T, *a);
  }
  // classdef.f90:1194-1281
  void blade_rotate(Blade& b, double ang, V3 axis, V3 o, const std::string& type) {
    if (!(std::fabs(ang) > EPS)) return;
    blade_move(b, neg(o));
    M3 T = getTransformAxis(ang, axis);
    V3 zero;
    for (int j = 0; j < b.ns; ++j)
      for (int i = 0; i < b.nc; ++i) b.w(i, j).rot(T, zero);
    blade_move(b, o);
    for (int i = 0; i < b.ns; ++i) {
      b.secCP[i] = rotAbout(T, b.secCP[i], o);
      b.secTauCapChord[i] = mv(T, b.secTauCapChord[i]);
      b.secTauCapSpan[i] = mv(T, b.secTauCapSpan[i]);
      b.secNormalVec[i] = mv(T, b.secNormalVec[i]);
    }
    if (type == "azimuth" || (type != "flap" && type != "pitch")) {
      b.xAxisAziFlap = mv(T, b.xAxisAziFlap); b.yAxisAziFlap = mv(T, b.yAxisAziFlap); b.zAxisAziFlap = mv(T, b.zAxisAziFlap);
      b.xAxisAzi = mv(T, b.xAxisAzi); b.yAxisAzi = mv(T, b.yAxisAzi); b.zAxisAzi = mv(T, b.zAxisAzi);
      b.xAxis = mv(T, b.xAxis); b.yAxis = mv(T, b.yAxis); b.zAxis = mv(T, b.zAxis);
    } else if (type == "flap") {
      b.xAxisAziFlap = mv(T, b.xAxisAziFlap); b.yAxisAziFlap = mv(T, b.yAxisAziFlap); b.zAxisAziFlap = mv(T, b.zAxisAziFlap);
      b.xAxis = mv(T, b.xAxis); b.yAxis = mv(T, b.yAxis); b.zAxis = mv(T, b.zAxis);
    } else {  // pitch
      b.xAxis = mv(T, b.xAxis); b.yAxis = mv(T, b.yAxis); b.zAxis = mv(T, b.zAxis);
    }
  }
  // classdef.f90:1160-1177
  void blade_rot_pitch(Blade& b, double theta) {
    if (std::fabs(theta) > EPS) {
      V3 o = b.w(0, 0).PC[0] * (1.0 - b.pivotLE) + b.w(b.nc - 1, 0).PC[1] * b.pivotLE;
      blade_rotate(b, theta, b.yAxis, o, "pitch");
    }
  }
  // classdef.f90:1179-1188
  void blade_rot_flap(Blade& b, double beta) { blade_rotate(b, beta, b.xAxisAzi, b.flapOrigin, "flap"); }

  // ---- rotor kinematics -------------------------------------------------
  // classdef.f90:4114-4136
  double gettheta(double psiv, int ib /*1-based*/) {
    double off = (TWO_PI / double(R.nb)) * double(ib - 1);
    if (R.pitchDynamicsSwitch == 1) {
      double th = std::min(std::fabs(psiv / R.Omega * R.dpitch), std::fabs(R.controlPitch.x));
      if (R.controlPitch.x < 0) th = -1.0 * th;
      return th;
    }
    return (R.controlPitch.x + R.controlPitch.y * std::cos(psiv + off)) + R.controlPitch.z * std::sin(psiv + off);
  }
  // classdef.f90:4202-4214
  void rotor_move(V3 d) {
    for (auto& b : R.blade) blade_move(b, d);
    R.hubCoords = R.hubCoords + d;
    R.cgCoords = R.cgCoords + d;
  }
  // classdef.f90:4216-4249
  void rotor_rot_pts(V3 p, V3 o) {
    M3 T = TgbAngles(p);
    for (auto& b : R.blade) blade_rot_pts(b, p, o);
    R.shaftAxis = mv(T, R.shaftAxis);
    R.xAxisBody = mv(T, R.xAxisBody);
    R.yAxisBody = mv(T, R.yAxisBody);
    R.zAxisBody = mv(T, R.zAxisBody);
    R.hubCoords = rotAbout(T, R.hubCoords, o);
    R.cgCoords = rotAbout(T, R.cgCoords, o);
  }
  // classdef.f90:4262-4285
  void rotor_rot_advance(double dpsi, bool nopitch) {
    R.psi = R.psi + dpsi;
    for (int ib = 0; ib < R.nb; ++ib) {
      Blade& b = R.blade[ib];
      blade_rotate(b, dpsi, R.shaftAxis, R.hubCoords, "azimuth");
      b.psi = b.psi + dpsi;
      if (!nopitch) {
        double thNext = gettheta(R.psi, ib + 1);
        blade_rot_pitch(b, thNext - b.theta);
        b.theta = thNext;
      }
    }
  }
  // classdef.f90:5133-5148
  void toChordsRevs(int& n) {
    if (n < 0) {
      if (std::fabs(R.Omega) < EPS) n = (int)std::ceil(double(std::abs(n)) * R.chord / (dt * norm2(R.velBody)));
      else n = (int)std::ceil(TWO_PI * double(std::abs(n)) / (std::fabs(R.Omega) * dt));
    }
  }

  // ---- sectional helpers ------------------------------------------------
  // classdef.f90:2267-2304
  void calc_secLocations(Blade& b, double frac, double hingeR) {
    for (int is = 0; is < b.ns; ++is) {
      V3 vecLE = 0.5 * (b.w(0, is).PC[0] + b.w(0, is).PC[3]);
      std::vector<double> xc(b.nc + 1, 0.0), zc(b.nc + 1, 0.0);
      V3 vecPC;
      for (int ic = 0; ic < b.nc; ++ic) {
        vecPC = 0.5 * (b.w(ic, is).PC[1] + b.w(ic, is).PC[2]) - vecLE;
        xc[ic + 1] = norm2(projVec(vecPC, b.secTauCapChord[is]));
        zc[ic + 1] = dot(vecPC, b.secNormalVec[is]);
      }
      double x = norm2(vecPC) * frac;
      double z = pwl_interp1d(xc, zc, x);
      b.secCP[is] = (vecLE + x * b.secTauCapChord[is]) + z * b.secNormalVec[is];
      b.secMflapArm[is] = norm2(projVec(b.secCP[is], b.yAxis)) - hingeR;
    }
  }
  // classdef.f90:2196-2232
  void calc_secChordwiseResVel(Blade& b) {
    if (b.nc >= 3) {
      std::vector<double> xd(b.nc), yd(b.nc);
      for (int is = 0; is < b.ns; ++is) {
        for (int ic = 0; ic < b.nc; ++ic) {
          WingPanel& p = b.w(ic, is);
          p.chordwiseResVel = noProjVec(p.velCPTotal, p.tauCapSpan);
          xd[ic] = dot(p.CP - b.w(0, is).PC[0], b.secTauCapChord[is]);
        }
        double xq = dot(b.secCP[is] - b.w(0, is).PC[0], b.secTauCapChord[is]);
        double out[3];
        for (int k = 0; k < 3; ++k) {
          for (int ic = 0; ic < b.nc; ++ic) {
            V3 c = b.w(ic, is).chordwiseResVel;
            yd[ic] = k == 0 ? c.x : (k == 1 ? c.y : c.z);
          }
          out[k] = lsq2(xq, xd, yd);
        }
        b.secChordwiseResVel[is] = mk(out[0], out[1], out[2]);
      }
    } else {
      for (int is = 0; is < b.ns; ++is) {
        V3 s;
        for (int ic = 0; ic < b.nc; ++ic) {
          WingPanel& p = b.w(ic, is);
          p.chordwiseResVel = noProjVec(p.velCPTotal, p.tauCapSpan);
          s = s + p.chordwiseResVel;
        }
        b.secChordwiseResVel[is] = s / double(b.nc);
      }
    }
  }
  // classdef.f90:2234-2265
  void blade_calc_secAlpha(Blade& b, V3 vert) {
    calc_secChordwiseResVel(b);
    for (int is = 0; is < b.ns; ++is) {
      V3 rv = b.secChordwiseResVel[is];
      b.secAlpha[is] = std::atan2(dot(rv, b.secNormalVec[is]), dot(rv, b.secTauCapChord[is]));
      b.secPhi[is] = getAngleTan(rv, noProjVec(b.w(0, is).velCPm, b.secTauCapSpan[is]));
      V3 vi = rv - b.w(0, is).velCPm;
      b.secViz[is] = vi.z;
      b.secVix[is] = norm2(noProjVec(vi, b.secTauCapSpan[is]) - mk(0, 0, vi.z));
      b.secTheta[is] = PI * 0.5 - getAngleTan(neg(b.secTauCapChord[is]), vert);
    }
  }
  // classdef.f90:4735-4752
  void rotor_calc_secAlpha() {
    for (int ib = 0; ib < R.nbConvect; ++ib) blade_calc_secAlpha(R.blade[ib], R.blade[ib].zAxisAziFlap);
    if (R.axisymmetrySwitch == 1)
      for (int ib = 1; ib < R.nb; ++ib) {
        R.blade[ib].secAlpha = R.blade[0].secAlpha;
        R.blade[ib].secPhi = R.blade[0].secPhi;
        R.blade[ib].secTheta = R.blade[0].secTheta;
      }
  }
  // classdef.f90:2341-2351 and 4938-4952
  void rotor_dirLiftDrag() {
    for (int ib = 0; ib < R.nbConvect; ++ib) {
      Blade& b = R.blade[ib];
      calc_secChordwiseResVel(b);
      for (int is = 0; is < b.ns; ++is) {
        b.secDragDir[is] = unitVec(b.secChordwiseResVel[is]);
        b.secLiftDir[is] = fsign(1.0, R.Omega) * unitVec(cross(b.secDragDir[is], b.yAxisAziFlap));
      }
    }
    if (R.axisymmetrySwitch == 1)
      for (int ib = 1; ib < R.nb; ++ib) {
        R.blade[ib].secDragDir = R.blade[0].secDragDir;
        R.blade[ib].secLiftDir = R.blade[0].secLiftDir;
      }
  }
  // classdef.f90:1704-1896
  void blade_calc_force(Blade& b) {
    int nc = b.nc, ns = b.ns;
    b.forceInertial = V3();
    for (int is = 0; is < ns; ++is) {
      b.secForceInertial[is] = V3(); b.secLift[is] = V3(); b.secDrag[is] = V3();
      b.secLiftInPlane[is] = V3(); b.secLiftOutPlane[is] = V3(); b.secLiftUnsteady[is] = V3();
    }
    double iGS = -1.0 * fsign(1.0, R.Omega);
    std::vector<double> vTC(nc * ns), vTS(nc * ns), gEC(nc * ns), gES(nc * ns);
    auto at = [nc](int ic, int is) { return ic + nc * is; };
    for (int is = 0; is < ns; ++is)
      for (int ic = 0; ic < nc; ++ic) {
        vTC[at(ic, is)] = dot(b.w(ic, is).velCP, b.w(ic, is).tauCapChord);
        vTS[at(ic, is)] = dot(b.w(ic, is).velCP, b.w(ic, is).tauCapSpan);
      }
    for (int is = 0; is < ns; ++is) gEC[at(0, is)] = b.w(0, is).vr.gam;
    for (int ic = 1; ic < nc; ++ic) gEC[at(ic, 0)] = b.w(ic, 0).vr.gam - b.w(ic - 1, 0).vr.gam;
    for (int ic = 0; ic < nc; ++ic) gES[at(ic, 0)] = b.w(ic, 0).vr.gam;
    for (int is = 1; is < ns; ++is) gES[at(0, is)] = b.w(0, is).vr.gam - b.w(0, is - 1).vr.gam;
    for (int is = 1; is < ns; ++is)
      for (int ic = 1; ic < nc; ++ic) {
        gEC[at(ic, is)] = b.w(ic, is).vr.gam - b.w(ic - 1, is).vr.gam;
        gES[at(ic, is)] = b.w(ic, is).vr.gam - b.w(ic, is - 1).vr.gam;
      }
    for (auto& g : gES) g = iGS * g;
    for (auto& g : gEC) g = iGS * g;
    for (int is = 0; is < ns; ++is) {
      for (int ic = 0; ic < nc; ++ic) {
        WingPanel& p = b.w(ic, is);
        if (ic > 0) p.gamTrapz = (iGS * 0.5) * (p.vr.gam + b.w(ic - 1, is).vr.gam);
        else p.gamTrapz = (iGS * 0.5) * p.vr.gam;
        p.delPUnsteady = density * (p.gamTrapz - p.gamPrev) / dt;
        p.delP = p.delPUnsteady + density * vTC[at(ic, is)] * gEC[at(ic, is)] / p.meanChord;
        if (b.spanwiseLiftSwitch != 0) p.delP = p.delP + density * vTS[at(ic, is)] * gES[at(ic, is)] / p.meanSpan;
        p.gamPrev = p.gamTrapz;
        p.normalForce = (p.delP * p.panelArea) * p.nCap;
        p.normalForceUnsteady = (p.delPUnsteady * p.panelArea) * p.nCap;
        b.secForceInertial[is] = b.secForceInertial[is] + p.normalForce;
        b.secLift[is] = b.secLift[is] + projVec(p.normalForce, b.secLiftDir[is]);
        b.secLiftUnsteady[is] = b.secLiftUnsteady[is] + projVec(p.normalForceUnsteady, b.secLiftDir[is]);
      }
      b.secLiftInPlane[is] = iGS * projVec(b.secLift[is], b.xAxisAziFlap);
      b.secLiftOutPlane[is] = projVec(b.secLift[is], b.zAxisAziFlap);
      b.secLiftInPlaneUnsteady[is] = iGS * projVec(b.secLiftUnsteady[is], b.xAxisAziFlap);
      b.secLiftOutPlaneUnsteady[is] = projVec(b.secLiftUnsteady[is], b.zAxisAziFlap);
      b.secDragInduced[is] = V3();
      b.secDragUnsteady[is] = V3();
    }
    for (int is = 0; is < ns; ++is) {
      b.secDragProfile[is] = V3();
      b.secDrag[is] = b.secDragInduced[is] + b.secDragProfile[is];
    }
    for (int is = 0; is < ns; ++is) {
      double m = norm2(b.secChordwiseResVel[is]);
      double q = (0.5 * density) * (m * m);
      if (std::fabs(q) > EPS) {
        double sg = fsign(1.0, dot(b.secLift[is], b.zAxisAziFlap));
        b.secCL[is] = norm2(b.secLift[is]) * sg / (q * b.secArea[is]);
        b.secCD[is] = norm2(b.secDrag[is]) / (q * b.secArea[is]);
        b.secCLu[is] = norm2(b.secLiftUnsteady[is]) * sg / (q * b.secArea[is]);
        b.secMflap[is] = norm2(b.secLift[is]) * sg * b.secMflapArm[is];
      } else {
        b.secCL[is] = b.secCD[is] = b.secCLu[is] = b.secMflap[is] = 0.0;
      }
    }
    // classdef.f90:2368-2380
    auto sumv = [ns](const std::vector<V3>& v) { V3 s; for (int i = 0; i < ns; ++i) s = s + v[i]; return s; };
    b.forceInertial = sumv(b.secForceInertial);
    b.lift = sumv(b.secLift);
    b.drag = sumv(b.secDrag);
    b.liftUnsteady = sumv(b.secLiftUnsteady);
    b.dragProfile = sumv(b.secDragProfile);
    b.dragInduced = sumv(b.secDragInduced);
    b.dragUnsteady = sumv(b.secDragUnsteady);
    double mf = 0.0;
    for (int i = 0; i < ns; ++i) mf = mf + b.secMflap[i];
    b.MflapLift = mf;
  }
  // classdef.f90:4607-4671 and 4954-4988
  void rotor_calc_force() {
    R.forceInertial = V3();
    rotor_dirLiftDrag();
    for (int ib = 0; ib < R.nbConvect; ++ib) blade_calc_force(R.blade[ib]);
    if (R.axisymmetrySwitch == 1) {
      Blade& b0 = R.blade[0];
      for (int ib = 1; ib < R.nb; ++ib) {
        Blade& b = R.blade[ib];
        for (size_t k = 0; k < b.wiP.size(); ++k) {
          b.wiP[k].delP = b0.wiP[k].delP; b.wiP[k].delPUnsteady = b0.wiP[k].delPUnsteady;
          b.wiP[k].gamPrev = b0.wiP[k].gamPrev;
          b.wiP[k].normalForce = b0.wiP[k].normalForce; b.wiP[k].normalForceUnsteady = b0.wiP[k].normalForceUnsteady;
        }
        b.secForceInertial = b0.secForceInertial; b.secLift = b0.secLift; b.secLiftDir = b0.secLiftDir;
        b.secLiftUnsteady = b0.secLiftUnsteady; b.secLiftInPlane = b0.secLiftInPlane;
        b.secLiftOutPlane = b0.secLiftOutPlane; b.secLiftInPlaneUnsteady = b0.secLiftInPlaneUnsteady;
        b.secLiftOutPlaneUnsteady = b0.secLiftOutPlaneUnsteady; b.secDragUnsteady = b0.secDragUnsteady;
        b.secDragProfile = b0.secDragProfile; b.secDrag = b0.secDrag;
        b.secCL = b0.secCL; b.secCD = b0.secCD; b.secCLu = b0.secCLu; b.secMflap = b0.secMflap;
        b.forceInertial = b0.forceInertial; b.lift = b0.lift; b.drag = b0.drag; b.liftUnsteady = b0.liftUnsteady;
        b.dragProfile = b0.dragProfile; b.dragInduced = b0.dragInduced; b.dragUnsteady = b0.dragUnsteady;
        b.MflapLift = b0.MflapLift;
      }
      double nbd = double(R.nb);
      R.forceInertial = nbd * b0.forceInertial;
      R.liftPrev = R.lift;
      R.lift = nbd * b0.lift;
      R.drag = nbd * b0.drag;
      R.liftUnsteady = nbd * b0.liftUnsteady;
      R.dragInduced = nbd * b0.dragInduced;
      R.dragProfile = nbd * b0.dragProfile;
      R.dragUnsteady = nbd * b0.dragUnsteady;
    } else {
      R.forceInertial = V3(); R.liftPrev = R.lift; R.lift = V3(); R.drag = V3(); R.liftUnsteady = V3();
      R.dragInduced = V3(); R.dragProfile = V3(); R.dragUnsteady = V3();
      for (int ib = 0; ib < R.nbConvect; ++ib) {
        Blade& b = R.blade[ib];
        R.forceInertial = R.forceInertial + b.forceInertial;
        R.lift = R.lift + b.lift;
        R.drag = R.drag + b.drag;
        R.liftUnsteady = R.liftUnsteady + b.liftUnsteady;
        R.dragInduced = R.dragInduced + b.dragInduced;
        R.dragProfile = R.dragProfile + b.dragProfile;
        R.dragUnsteady = R.dragUnsteady + b.dragUnsteady;
      }
    }
  }
  // libPostprocess.f90:814-838 (values at full precision)
  void force2file() {
    double D = R.nonDimforceDenominator;
    double sl = fsign(1.0, dot(R.lift, R.zAxisBody));
    std::vector<double> row = {double(iter),
                               sl * norm2(R.lift) / D,
                               norm2(R.drag) / D,
                               norm2(R.liftUnsteady) / D,
                               norm2(R.dragInduced) / D,
                               norm2(R.dragProfile) / D,
                               norm2(R.dragUnsteady) / D,
                               R.forceInertial.x / D,
                               R.forceInertial.y / D,
                               R.forceInertial.z / D};
    ctHist.push_back(row);
  }

  // ---- induced velocities -----------------------------------------------
  // classdef.f90:1342-1357, 4424-4443
  V3 rotor_vind_bywing(V3 P) const {
    V3 acc;
    for (int ib = 0; ib < R.nb; ++ib) {
      const Blade& b = R.blade[ib];
      ChunkSum s(sumChunk);
      for (int j = 0; j < b.ns; ++j)
        for (int i = 0; i < b.nc; ++i) s.add(vr_vind(b.w(i, j).vr, P) * b.w(i, j).vr.gam);
      acc = acc + s.result();
    }
    return acc;
  }
  // classdef.f90:1376-1393, 4445-4457
  V3 rotor_vind_bywing_boundVortices(V3 P) const {
    V3 acc;
    for (int ib = 0; ib < R.nb; ++ib) {
      const Blade& b = R.blade[ib];
      V3 s;
      for (int j = 0; j < b.ns; ++j)
        for (int i = 0; i < b.nc; ++i) {
          const VR& r = b.w(i, j).vr;
          s = s + (vf_vind(r.vf[1], P) + vf_vind(r.vf[3], P)) * r.gam;
        }
      for (int j = 0; j < b.ns; ++j) {
        const VR& r = b.w(b.nc - 1, j).vr;
        s = s - vf_vind(r.vf[1], P) * r.gam;
      }
      acc = acc + s;
    }
    return acc;
  }
  // classdef.f90:1437-1513, 4459-4479
  V3 rotor_vind_bywake(V3 P, bool pred) const {
    V3 acc;
    int NW = R.nNwake, NF = R.nFwake;
    for (int ib = 0; ib < R.nb; ++ib) {
      const Blade& b = R.blade[ib];
      const std::vector<VR>& wn = pred ? b.waNP : b.waN;
      const std::vector<FW>& wf = pred ? b.waFP : b.waF;
      ChunkSum s(sumChunk);
      for (int j = 0; j < b.ns; ++j)
        for (int i = R.rowNear - 1; i < NW; ++i) {
          const VR& r = wn[i + NW * j];
          if (std::fabs(r.gam) > EPS) s.add(vr_vind(r, P) * r.gam);
          else s.tick();
        }
      if (R.rowFar <= NF) {
        // s - v*gam == s + v*(-gam) bit for bit
        for (int j = 0; j < b.ns; ++j) {
          const VR& r = wn[(NW - 1) + NW * j];
          s.add(vf_vind(r.vf[1], P) * (-r.gam));
        }
        for (int i = R.rowFar - 1; i < NF; ++i) {
          const FW& f = wf[i];
          if (std::fabs(f.gam) > EPS) s.add(vf_vind(f.vf, P) * f.gam);
          else s.tick();
        }
        // the prescribed far wake (classdef.f90:1471-1476, 1501-1507): summed
        // only by cases that generate one
        if (R.prescWakeNt > 0) {
          const PFwake& pf = pred ? b.wapFP : b.wapF;
          for (const FW& f : pf.waF) {
            if (std::fabs(f.gam) > EPS) s.add(vf_vind(f.vf, P) * f.gam);
            else s.tick();
          }
        }
      }
      acc = acc + s.result();
    }
    return acc;
  }

  // main.f90:808-827: the zeroed node velocity plus vind_on?wake_byRotor
  // (libCommon.f90:114-211: wing + wake of a rotor) of every rotor in turn
  V3 byAllRotors(V3 P, bool pred) const {
    if (sys.empty()) return V3() + (rotor_vind_bywing(P) + rotor_vind_bywake(P, pred));
    V3 a;
    for (const Sim* o : sys) a = a + (o->rotor_vind_bywing(P) + o->rotor_vind_bywake(P, pred));
    return a;
  }
  // libCommon.f90:114-211 for blade ib; writes vel (rows rowNear..NW) and velF (rowFar..NF)
  void vind_onWake(int ib, bool pred, std::vector<V3>& velN, std::vector<V3>& velF) {
    const Blade& b = R.blade[ib];
    int NW = R.nNwake, NF = R.nFwake, ns = b.ns;
    const std::vector<VR>& wn = pred ? b.waNP : b.waN;
    const std::vector<FW>& wf = pred ? b.waFP : b.waF;
    int rows = NW - (R.rowNear - 1);
    int nT = rows * (ns + 1);
    int nF = NF >= R.rowFar ? NF - R.rowFar + 1 : 0;
#pragma omp parallel for schedule(static)
    for (int t = 0; t < nT + nF; ++t) {
      if (t < nT) {
        int j = t / rows, i = R.rowNear - 1 + t % rows;
        V3 P = j < ns ? wn[i + NW * j].vf[1].fc1 : wn[i + NW * (ns - 1)].vf[2].fc1;
        velN[i + NW * j] = byAllRotors(P, pred);
      } else {
        int i = R.rowFar - 1 + (t - nT);
        V3 P = wf[i].vf.fc1;
        velF[i] = byAllRotors(P, pred);
      }
    }
  }

  // ---- wake operations ---------------------------------------------------
  // classdef.f90:4297-4325
  void assignshed(bool LE) {
    int NW = R.nNwake;
    for (auto& b : R.blade) {
      if (LE) {
        int r = R.rowNear - 1;
        for (int i = 0; i < R.ns; ++i) {
          VR& w = b.waN[r + NW * i];
          w.assignP(1, b.w(R.nc - 1, i).vr.vf[1].fc1);
          w.assignP(4, b.w(R.nc - 1, i).vr.vf[2].fc1);
          w.calclength(true);
        }
        for (int i = 0; i < R.ns; ++i) b.waN[r + NW * i].gam = b.w(R.nc - 1, i).vr.gam;
      } else {
        int r = std::max(R.rowNear - 1, 1) - 1;
        for (int i = 0; i < R.ns; ++i) {
          VR& w = b.waN[r + NW * i];
          w.assignP(2, b.w(R.nc - 1, i).vr.vf[1].fc1);
          w.assignP(3, b.w(R.nc - 1, i).vr.vf[2].fc1);
        }
      }
    }
  }
  // classdef.f90:4331-4354
  void age_wake() {
    int NW = R.nNwake;
    for (auto& b : R.blade) {
      for (int f = 0; f < 4; ++f)
        for (int j = 0; j < R.ns; ++j)
          for (int i = R.rowNear - 1; i < NW; ++i) {
            VF& v = b.waN[i + NW * j].vf[f];
            v.age = v.age + dt;
            v.ageAz = v.ageAz + dt * R.omegaSlow;
          }
      for (int i = R.rowFar - 1; i < R.nFwake; ++i) {
        b.waF[i].vf.age = b.waF[i].vf.age + dt;
        b.waF[i].vf.ageAz = b.waF[i].vf.ageAz + dt * R.omegaSlow;
      }
    }
  }
  // classdef.f90:4356-4408
  void dissipate_wake() {
    const double oseen = 1.2564;
    double add = (((4.0 * oseen) * R.apparentViscCoeff) * kinematicVisc) * dt;
    double decay = std::exp(-(R.decayCoeff * dt));
    int NW = R.nNwake;
    for (auto& b : R.blade) {
      for (int is = 0; is < R.ns; ++is) {
        for (int ic = R.rowNear - 1; ic < NW; ++ic) {
          VR& w = b.waN[ic + NW * is];
          w.vf[0].rVc = std::sqrt(w.vf[0].rVc * w.vf[0].rVc + add);
          w.vf[2].rVc = w.vf[0].rVc;
          w.gam = w.gam * decay;
        }
        for (int ic = R.rowNear - 1; ic < NW; ++ic) {
          VR& w = b.waN[ic + NW * is];
          w.vf[1].rVc = std::sqrt(w.vf[1].rVc * w.vf[1].rVc + add);
        }
        if (R.rowNear != NW)
          for (int ic = R.rowNear; ic < NW; ++ic) b.waN[ic + NW * is].vf[3].rVc = b.waN[ic - 1 + NW * is].vf[1].rVc;
      }
      for (int ic = R.rowFar - 1; ic < R.nFwake; ++ic) {
        FW& f = b.waF[ic];
        f.vf.rVc = std::sqrt(f.vf.rVc * f.vf.rVc + add);
        f.gam = f.gam * decay;
      }
    }
  }
  // classdef.f90:4410-4422
  void strain_wake() {
    for (auto& b : R.blade)
      for (int i = R.rowFar - 1; i < R.nFwake; ++i) {
        VF& v = b.waF[i].vf;
        v.lc = norm2(v.fc1 - v.fc2);
        v.rVc = v.rVc0 * std::sqrt(v.l0 / v.lc);
      }
  }
  // classdef.f90:1515-1575 + 1609-1702
  void blade_convectwake(Blade& b, bool pred) {
    int NW = R.nNwake, NF = R.nFwake, ns = R.ns;
    std::vector<VR>& wn = pred ? b.waNP : b.waN;
    std::vector<FW>& wf = pred ? b.waFP : b.waF;
    if (!pred) {
      for (int j = 0; j < ns; ++j)
        for (int i = R.rowNear - 1; i < NW; ++i) wn[i + NW * j].shiftdP(2, b.velN[i + NW * j] * dt);
      for (int i = R.rowNear - 1; i < NW; ++i) wn[i + NW * (ns - 1)].shiftdP(3, b.velN[i + NW * ns] * dt);
    } else {
      // the reference's loop "do i = 1, rowNear, nNwake" visits row 1 only
      for (int j = 0; j < ns; ++j) wn[0 + NW * j].shiftdP(2, b.velN[0 + NW * j] * dt);
      wn[0 + NW * (ns - 1)].shiftdP(3, b.velN[0 + NW * ns] * dt);
    }
    for (int i = R.rowFar - 1; i < NF; ++i) wf[i].vf.fc1 = wf[i].vf.fc1 + b.velF[i] * dt;
    // continuity
    for (int j = 0; j < ns - 1; ++j)
      for (int i = R.rowNear; i < NW; ++i) {
        wn[i + NW * j].assignP(1, wn[i - 1 + NW * j].vf[1].fc1);
        wn[i + NW * j].assignP(3, wn[i + NW * (j + 1)].vf[1].fc1);
        wn[i + NW * j].assignP(4, wn[i - 1 + NW * (j + 1)].vf[1].fc1);
      }
    for (int j = 0; j < ns - 1; ++j) wn[R.rowNear - 1 + NW * j].assignP(3, wn[R.rowNear - 1 + NW * (j + 1)].vf[1].fc1);
    for (int i = R.rowNear; i < NW; ++i) {
      wn[i + NW * (ns - 1)].assignP(1, wn[i - 1 + NW * (ns - 1)].vf[1].fc1);
      wn[i + NW * (ns - 1)].assignP(4, wn[i - 1 + NW * (ns - 1)].vf[2].fc1);
    }
    for (int i = R.rowFar; i < NF; ++i) wf[i].vf.fc2 = wf[i - 1].vf.fc1;
  }
  // classdef.f90:1283-1340
  void blade_rot_wake_axis(Blade& b, double theta, V3 axis, V3 o, bool pred) {
    if (!(std::fabs(theta) > EPS)) return;
    M3 T = getTransformAxis(theta, axis);
    std::vector<VR>& wn = pred ? b.waNP : b.waN;
    std::vector<FW>& wf = pred ? b.waFP : b.waF;
    int NW = R.nNwake;
    for (int j = 0; j < R.ns; ++j)
      for (int i = R.rowNear - 1; i < NW; ++i) wn[i + NW * j].rot(T, o);
    for (int i = R.rowFar - 1; i < R.nFwake; ++i) {
      wf[i].vf.fc1 = rotAbout(T, wf[i].vf.fc1, o);
      wf[i].vf.fc2 = rotAbout(T, wf[i].vf.fc2, o);
    }
  }
  // classdef.f90:4786-4830
  void rotor_convectwake(bool pred) {
    for (int ib = 0; ib < R.nbConvect; ++ib) blade_convectwake(R.blade[ib], pred);
    if (R.axisymmetrySwitch == 1) {
      int NW = R.nNwake;
      for (int ib = 1; ib < R.nb; ++ib) {
        double off = (TWO_PI / double(R.nb)) * double(ib);
        Blade& b = R.blade[ib];
        const Blade& b0 = R.blade[0];
        std::vector<VR>& dn = pred ? b.waNP : b.waN;
        const std::vector<VR>& sn = pred ? b0.waNP : b0.waN;
        std::vector<FW>& df = pred ? b.waFP : b.waF;
        const std::vector<FW>& sf = pred ? b0.waFP : b0.waF;
        for (int j = 0; j < R.ns; ++j)
          for (int i = R.rowNear - 1; i < NW; ++i) dn[i + NW * j] = sn[i + NW * j];
        for (int i = R.rowFar - 1; i < R.nFwake; ++i) df[i] = sf[i];
        blade_rot_wake_axis(b, off, R.shaftAxis, R.hubCoords, pred);
      }
    }
    if (R.prescWakeNt > 0 && iter > R.prescWakeNt) updatePrescribedWake(pred);
  }
  // classdef.f90:998-1066 (pFwake_update) on the far-wake filaments i0..i1
  void pFwake_update(PFwake& pf, const std::vector<FW>& waF, int i0, int i1, V3 hub, V3 shaft, double dpsi) {
    if (std::fabs(shaft.x) > EPS || std::fabs(shaft.y) > EPS)
      throw std::runtime_error("Prescribed far wake only implemented for shaft along Z-axis");
    pf.isPresent = true;
    const int n = i1 - i0 + 1;
    const V3 anchor = waF[i1].vf.fc1;
    double pitch = 0.0, radius = 0.0;
    for (int i = 0; i < n; ++i) {
      const V3 c = waF[i0 + i].vf.fc1;
      radius = radius + std::sqrt(c.y * c.y + c.x * c.x);
      if (i < n - 1) pitch = pitch + c.z - waF[i0 + i + 1].vf.fc1.z;
    }
    pitch = std::fabs(pitch) * (-TWO_PI / dpsi) / double(n - 1);
    radius = radius / double(n);
    pf.helixPitch = pf.relaxFactor * pitch + (1.0 - pf.relaxFactor) * pf.helixPitch;
    pf.helixRadius = pf.relaxFactor * radius + (1.0 - pf.relaxFactor) * pf.helixRadius;
    const double dTheta = std::atan2(anchor.y, anchor.x);
    const double deltaZ = anchor.z - hub.z;
    const int nc = (int)pf.waF.size() + 1;
    std::vector<double> theta = linspace(0.0, TWO_PI * pf.nRevs, nc);
    if (pf.isClockwiseRotor)
      for (auto& t : theta) t = -1.0 * t;
    std::vector<V3> c(nc);
    for (int i = 0; i < nc; ++i)
      c[i] = mk(pf.helixRadius * std::cos(theta[i] + dTheta), pf.helixRadius * std::sin(theta[i] + dTheta),
                pf.helixPitch * std::fabs(theta[i]) / TWO_PI + deltaZ);
    for (size_t i = 0; i < pf.waF.size(); ++i) {
      pf.waF[i].vf.fc2 = hub + c[i];
      pf.waF[i].vf.fc1 = hub + c[i + 1];
    }
    pf.waF[0].vf.fc2 = anchor;
    for (auto& f : pf.waF) {
      f.gam = waF[i1].gam;
      f.vf.rVc = waF[i1].vf.rVc;
    }
  }
  // classdef.f90:5172-5217
  void updatePrescribedWake(bool pred) {
    const int rowStart = R.prescWakeGenNt == 0 ? R.rowFar : R.nFwake - R.prescWakeGenNt;
    for (int ib = 0; ib < R.nbConvect; ++ib) {
      Blade& b = R.blade[ib];
      pFwake_update(pred ? b.wapFP : b.wapF, pred ? b.waFP : b.waF, rowStart - 1, R.nFwake - 1, R.hubCoords,
                    R.shaftAxis, R.omegaSlow * dt);
    }
    if (R.axisymmetrySwitch == 1)
      for (int ib = 1; ib < R.nb; ++ib) {
        PFwake& d = pred ? R.blade[ib].wapFP : R.blade[ib].wapF;
        d = pred ? R.blade[0].wapFP : R.blade[0].wapF;
        const double off = (TWO_PI / double(R.nb)) * double(ib);
        if (std::fabs(off) > EPS) {  // pFwake_rot_wake_axis, classdef.f90:1068-1086
          const M3 T = getTransformAxis(off, R.shaftAxis);
          for (auto& f : d.waF) {
            f.vf.fc1 = rotAbout(T, f.vf.fc1, R.hubCoords);
            f.vf.fc2 = rotAbout(T, f.vf.fc2, R.hubCoords);
          }
        }
      }
  }
  // classdef.f90:4911-4917, 2306-2339: far-wake filaments whose direction
  // turns by more than skewLimit x pi from the next one's get a core radius
  // of one chord (every blade)
  void burst_wake() {
    for (auto& b : R.blade) {
      if (R.rowFar > R.nFwake) continue;
      for (int i = R.rowFar - 1; i < R.nFwake - 1; ++i) {
        const V3 a = b.waF[i].vf.fc2 - b.waF[i].vf.fc1, c = b.waF[i + 1].vf.fc1 - b.waF[i + 1].vf.fc2;
        const double skew = std::fabs(std::acos(dot(a, c) / std::sqrt(sumsq(a) * sumsq(c))) - PI) / PI;
        if (skew >= R.skewLimit) {
          b.waF[i + 1].vf.rVc = R.chord;
          b.waF[i].vf.rVc = R.chord;
        }
      }
    }
  }
  // classdef.f90:4481-4513
  void shiftwake() {
    int NW = R.nNwake;
    for (auto& b : R.blade) {
      for (int j = 0; j < R.ns; ++j) {
        for (int i = NW - 1; i >= 1; --i) b.waN[i + NW * j] = b.waN[i - 1 + NW * j];
        for (int f = 0; f < 4; ++f) b.waN[0 + NW * j].vf[f].age = 0.0;
      }
    }
  }
  void shiftFwake() {
    for (auto& b : R.blade) {
      for (int i = R.nFwake - 1; i >= 1; --i) b.waF[i] = b.waF[i - 1];
      b.waF[0].vf.age = 0.0;
    }
  }
  // classdef.f90:4515-4605
  void rollup() {
    int NW = R.nNwake, ns = R.ns;
    int rowFarNext = R.rowFar - 1;
    for (int ib = 0; ib < R.nb; ++ib) {
      Blade& b = R.blade[ib];
      auto last = [&](int ispan) -> VR& { return b.waN[(NW - 1) + NW * ispan]; };
      double gamRollup = last(ns - 1).gam;
      V3 cLE, cTE;
      double radius = 0.0, gamSum = 0.0;
      for (int is = R.rollupStart; is <= R.rollupEnd; ++is) {
        VR& w = last(is - 1);
        cLE = cLE + w.vf[3].fc1 * w.gam;
        cTE = cTE + w.vf[2].fc1 * w.gam;
        gamSum = gamSum + w.gam;
        if (fsign(1.0, R.Omega * R.controlPitch.x) > EPS) {
          if (w.gam < gamRollup) gamRollup = w.gam;
        } else {
          if (w.gam > gamRollup) gamRollup = w.gam;
        }
        radius = radius + w.vf[2].rVc * w.gam;
      }
      double ageRollup = last(ns - 1).vf[2].age;
      if (std::fabs(gamSum) > EPS) {
        cLE = cLE / gamSum;
        cTE = cTE / gamSum;
        radius = radius / gamSum;
      } else {
        cLE = last(R.rollupEnd - 1).vf[1].fc1;
        cTE = last(R.rollupEnd - 1).vf[2].fc1;
        radius = last(R.rollupEnd - 1).vf[2].rVc;
      }
      if (R.suppressFwakeSwitch == 1) gamRollup = 0.0;
      if (R.nFwake > 0) {
        if (rowFarNext == 0) {
          // rotor_shiftFwake shifts the far wake of EVERY blade while the
          // first blade is processed; rowFarNext then stays 1 for the others
          shiftFwake();
          rowFarNext = 1;
        }
        FW& f = b.waF[rowFarNext - 1];
        f.vf.fc2 = cLE;
        f.vf.fc1 = cTE;
        f.gam = gamRollup;
        f.vf.age = ageRollup;
        f.vf.rVc0 = radius;
        f.vf.rVc = radius;
        f.vf.lc = norm2(f.vf.fc1 - f.vf.fc2);
        f.vf.l0 = f.vf.lc;
        if (rowFarNext < R.nFwake) b.waF[rowFarNext].vf.fc2 = cTE;
      }
    }
    shiftwake();
  }

  // ---- main program pieces -----------------------------------------------
  // main.f90:119-156 (init) and 521-590 (loop) -- kinematic part of velCP
  V3 kinematicVelCP(const Blade& b, int is, V3 CP) const {
    V3 v = -1.0 * R.velBody;
    v = v - cross(R.omegaBody, CP - R.cgCoords);
    v = v - cross(R.omegaSlow * R.shaftAxis, CP - R.hubCoords);
    double fa = b.secMflapArm[is] * b.dflap;  // scalar broadcast to every component
    v = mk(v.x - fa, v.y - fa, v.z - fa);
    return v;
  }
  void solveCirculation(bool withWake) {
    computeRHS(withWake);
    solveRHS();
  }
  // main.f90:522-591 (and :120-183 without the wake): velCP and the RHS;
  // in a system the wake of every rotor and the wings of the others
  void computeRHS(bool withWake) {
    int nc = R.nc, ns = R.ns;
    std::fill(R.RHS.begin(), R.RHS.end(), 0.0);
    int tot = R.nbConvect * ns * nc;
#pragma omp parallel for schedule(static)
    for (int t = 0; t < tot; ++t) {
      int ic = t % nc, is = (t / nc) % ns, ib = t / (nc * ns);
      Blade& b = R.blade[ib];
      WingPanel& p = b.w(ic, is);
      int row = ic + nc * is + ns * nc * ib;
      p.velCP = kinematicVelCP(b, is, p.CP);
      p.velCPm = p.velCP;
      if (sys.empty()) {
        if (withWake) p.velCP = p.velCP + rotor_vind_bywake(p.CP, false);
      } else {
        for (size_t jr = 0; jr < sys.size(); ++jr) {
          if (withWake) p.velCP = p.velCP + sys[jr]->rotor_vind_bywake(p.CP, false);
          if ((int)jr != self) p.velCP = p.velCP + sys[jr]->rotor_vind_bywing(p.CP);
        }
      }
      R.RHS[row] = dot(p.velCP, p.nCap);
    }
    if (R.axisymmetrySwitch == 1)
      for (int ib = 1; ib < R.nb; ++ib)
        for (int k = 0; k < nc * ns; ++k) R.RHS[nc * ns * ib + k] = R.RHS[k];
    for (auto& r : R.RHS) r = -1.0 * r;
  }
  // main.f90:594-603: gamVec = AIC_inv RHS, map_gam
  void solveRHS() {
    const int n = R.n();
    R.gamVecPrev = R.gamVec;
    matvec(R.AIC_inv, R.RHS, R.gamVec, n);
    map_gam();
  }
  static void matvec(const std::vector<double>& A, const std::vector<double>& x, std::vector<double>& y, int n) {
    for (int i = 0; i < n; ++i) {
      double s = 0.0;
      for (int j = 0; j < n; ++j) s = s + A[i + size_t(n) * j] * x[j];
      y[i] = s;
    }
  }
  // classdef.f90:4181-4196
  void map_gam() {
    int nc = R.nc, ns = R.ns;
    for (int ib = 0; ib < R.nbConvect; ++ib)
      for (int j = 0; j < ns; ++j)
        for (int i = 0; i < nc; ++i) R.blade[ib].w(i, j).vr.gam = R.gamVec[nc * ns * ib + i + nc * j];
    if (R.axisymmetrySwitch == 1)
      for (int ib = 1; ib < R.nb; ++ib)
        for (size_t k = 0; k < R.blade[ib].wiP.size(); ++k) R.blade[ib].wiP[k].vr.gam = R.blade[0].wiP[k].vr.gam;
  }
  // main.f90:240-280 (forceCalcSwitch 0)
  void computeForces() {
    int nc = R.nc, ns = R.ns;
    int tot = R.nbConvect * ns * nc;
#pragma omp parallel for schedule(static)
    for (int t = 0; t < tot; ++t) {
      int ic = t % nc, is = (t / nc) % ns, ib = t / (nc * ns);
      WingPanel& p = R.blade[ib].w(ic, is);
      p.velCPTotal = p.velCP;
      if (sys.empty()) p.velCPTotal = p.velCPTotal - rotor_vind_bywing_boundVortices(p.CP);
      else
        for (const Sim* o : sys) p.velCPTotal = p.velCPTotal - o->rotor_vind_bywing_boundVortices(p.CP);
      p.velCPTotal = p.velCPTotal + rotor_vind_bywing(p.CP);
    }
    if (R.axisymmetrySwitch == 1)
      for (int ib = 1; ib < R.nb; ++ib)
        for (size_t k = 0; k < R.blade[ib].wiP.size(); ++k) R.blade[ib].wiP[k].velCPTotal = R.blade[0].wiP[k].velCPTotal;
    rotor_calc_secAlpha();
    if (R.forceCalcSwitch == 1) rotor_calc_force_alpha();
    else rotor_calc_force();
  }
  // classdef.f90:4734-4747 (rotor_calc_force_alpha) with blade_calc_force_alpha
  // (:2091-2105), blade_lookup_secCoeffs (:2178-2195), blade_secCoeffsToSecForces
  // (:2146-2176), blade_getSecDynamicPressure (:2058-2069), blade_sumSecToNetForces
  // (:2368-2380) and rotor_sumBladeToNetForces (:4954-4988)
  void rotor_calc_force_alpha() {
    R.forceInertial = V3();
    rotor_dirLiftDrag();
    for (int ib = 0; ib < R.nb; ++ib) {
      Blade& b = R.blade[ib];
      const int ns = b.ns;
      b.secCM.assign(ns, 0.0);
      for (int is = 0; is < ns; ++is) {
        const double mach = norm2(b.secChordwiseResVel[is]) / velSound;
        const double aDeg = b.secAlpha[is] * RAD2DEG;
        const C81& t = R.c81[b.airfoilNo[is] - 1];
        b.secCL[is] = t.getCL(aDeg, mach);
        b.secCD[is] = t.getCD(aDeg, mach);
        b.secCM[is] = t.getCM(aDeg, mach);
        b.secCLu[is] = 0.0;
      }
      for (int is = 0; is < ns; ++is) {
        const double m = norm2(b.secChordwiseResVel[is]);
        const double lead = ((0.5 * density) * (m * m)) * b.secArea[is];
        b.secLift[is] = (b.secLiftDir[is] * lead) * b.secCL[is];
        b.secLiftUnsteady[is] = (b.secLiftDir[is] * lead) * b.secCLu[is];
        double gs = 0.0;
        for (int ic = 0; ic < b.nc; ++ic) gs = gs + b.w(ic, is).vr.gam;
        V3 fi = cross(b.yAxis, b.secChordwiseResVel[is]);
        fi = fsign(1.0, gs) * unitVec(fi);
        fi = norm2(b.secLift[is]) * fi;
        fi = fi + norm2(b.secDrag[is]) * unitVec(b.secChordwiseResVel[is]);
        b.secForceInertial[is] = fi;
      }
      for (int is = 0; is < ns; ++is) {
        b.secDragInduced[is] = V3();
        b.secDrag[is] = b.secDragProfile[is] + b.secDragInduced[is];
      }
      V3 fi, li, dr, lu, dp, di, du;
      double mf = 0.0;
      for (int is = 0; is < ns; ++is) {
        fi = fi + b.secForceInertial[is];
        li = li + b.secLift[is];
        dr = dr + b.secDrag[is];
        lu = lu + b.secLiftUnsteady[is];
        dp = dp + b.secDragProfile[is];
        di = di + b.secDragInduced[is];
        du = du + b.secDragUnsteady[is];
        mf = mf + b.secMflap[is];
      }
      b.forceInertial = fi; b.lift = li; b.drag = dr; b.liftUnsteady = lu;
      b.dragProfile = dp; b.dragInduced = di; b.dragUnsteady = du; b.MflapLift = mf;
    }
    R.forceInertial = V3(); R.liftPrev = R.lift; R.lift = V3(); R.drag = V3(); R.liftUnsteady = V3();
    R.dragInduced = V3(); R.dragProfile = V3(); R.dragUnsteady = V3();
    for (int ib = 0; ib < R.nb; ++ib) {
      Blade& b = R.blade[ib];
      R.forceInertial = R.forceInertial + b.forceInertial;
      R.lift = R.lift + b.lift;
      R.drag = R.drag + b.drag;
      R.liftUnsteady = R.liftUnsteady + b.liftUnsteady;
      R.dragInduced = R.dragInduced + b.dragInduced;
      R.dragProfile = R.dragProfile + b.dragProfile;
      R.dragUnsteady = R.dragUnsteady + b.dragUnsteady;
    }
  }
  // classdef.f90:4151-4179 + libMath.f90:48-83
  void calcAIC() {
    int n = R.n(), nc = R.nc, ns = R.ns;
    R.AIC.assign(size_t(n) * n, 0.0);
#pragma omp parallel for schedule(static)
    for (int row = 0; row < n; ++row) {
      int ib = row / (nc * ns), is = (row / nc) % ns, ic = row % nc;
      const WingPanel& cp = R.blade[ib].w(ic, is);
      for (int jb = 0; jb < R.nb; ++jb)
        for (int j = 0; j < ns; ++j)
          for (int i = 0; i < nc; ++i) {
            int col = i + nc * j + ns * nc * jb;
            V3 v = vr_vind(R.blade[jb].w(i, j).vr, cp.CP);
            R.AIC[row + size_t(n) * col] = dot(v, cp.nCap);
          }
    }
    R.AIC_inv = inverseLU(R.AIC, n);
  }
  static std::vector<double> inverseLU(const std::vector<double>& A0, int n) {
    std::vector<double> A = A0;
    std::vector<int> piv(n);
    auto at = [n](int i, int j) { return i + size_t(n) * j; };
    for (int k = 0; k < n; ++k) {
      int p = k;
      double mx = std::fabs(A[at(k, k)]);
      for (int i = k + 1; i < n; ++i)
        if (std::fabs(A[at(i, k)]) > mx) { mx = std::fabs(A[at(i, k)]); p = i; }
      piv[k] = p;
      if (A[at(p, k)] == 0.0) throw std::runtime_error("Matrix is numerically singular!");
      if (p != k)
        for (int j = 0; j < n; ++j) std::swap(A[at(k, j)], A[at(p, j)]);
      double akk = A[at(k, k)];
      for (int i = k + 1; i < n; ++i) A[at(i, k)] = A[at(i, k)] / akk;
#pragma omp parallel for schedule(static) if (n > 256)
      for (int j = k + 1; j < n; ++j) {
        double ukj = A[at(k, j)];
        for (int i = k + 1; i < n; ++i) A[at(i, j)] = A[at(i, j)] - A[at(i, k)] * ukj;
      }
    }
    // X = A^-1: solve L U x = P e_c for every unit column c
    std::vector<double> X(size_t(n) * n, 0.0);
#pragma omp parallel for schedule(static)
    for (int c = 0; c < n; ++c) {
      std::vector<double> y(n, 0.0);
      // apply row interchanges to e_c
      std::vector<double> e(n, 0.0);
      e[c] = 1.0;
      for (int k = 0; k < n; ++k) std::swap(e[k], e[piv[k]]);
      for (int i = 0; i < n; ++i) {
        double s = e[i];
        for (int k = 0; k < i; ++k) s = s - A[at(i, k)] * y[k];
        y[i] = s;
      }
      for (int i = n - 1; i >= 0; --i) {
        double s = y[i];
        for (int k = i + 1; k < n; ++k) s = s - A[at(i, k)] * X[at(k, c)];
        X[at(i, c)] = s / A[at(i, i)];
      }
    }
    return X;
  }
  // libMath.f90:428-458 (tol 1E-04, single precision literal)
  static bool isInverse(const std::vector<double>& A, const std::vector<double>& Ai, int n) {
    const double tol = (double)1e-4f;
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        double s = 0.0;
        for (int k = 0; k < n; ++k) s = s + A[i + size_t(n) * k] * Ai[k + size_t(n) * j];
        if (i != j) { if (s > tol) return false; }
        else if (s - 1.0 > tol) return false;
      }
    return true;
  }

  // ---- setup ---------------------------------------------------------------
  void readConfig(const Namelist& c) {
    std::string ver = c.s("VERSION", "fileFormatVersion", "");
    if (!ver.empty() && std::fabs(Namelist::todouble(ver) - 0.5) > 1e-12) throw std::runtime_error("config.nml template version does not match");
    nt = c.i("PARAMS", "nt");
    dt = c.d("PARAMS", "dt");
    nr = c.i("PARAMS", "nr", 1);
    density = c.d("PARAMS", "density", 1.0);
    velSound = c.d("PARAMS", "velSound", 330.0);
    kinematicVisc = c.d("PARAMS", "kinematicVisc", 0.0);
    sw.restartWriteNt = c.i("OPTIONS", "restartWriteNt");
    sw.restartFromNt = c.i("OPTIONS", "restartFromNt");
    sw.ntSub = c.i("OPTIONS", "ntSub");
    sw.ntSubInit = c.i("OPTIONS", "ntSubInit");
    sw.wakePlot = c.i("OPTIONS", "wakePlot");
    sw.wakeTipPlot = c.i("OPTIONS", "wakeTipPlot");
    sw.rotorForcePlot = c.i("OPTIONS", "rotorForcePlot", 1);
    sw.gridPlot = c.i("OPTIONS", "gridPlot");
    sw.wakeDissipation = c.i("OPTIONS", "wakeDissipation");
    sw.wakeStrain = c.i("OPTIONS", "wakeStrain");
    sw.wakeBurst = c.i("OPTIONS", "wakeBurst");
    sw.wakeSuppress = c.i("OPTIONS", "wakeSuppress");
    sw.slowStart = c.i("OPTIONS", "slowStart");
    sw.slowStartNt = c.i("OPTIONS", "slowStartNt");
    sw.fdScheme = c.i("OPTIONS", "fdScheme");
    sw.initWakeVelNt = c.i("OPTIONS", "initWakeVelNt");
    sw.probe = c.i("OPTIONS", "probe");
    if (nr != 1 && !member) throw std::runtime_error("nr > 1: create the rotors as a system (or_sys_create)");
    if (member && (sw.ntSub != 0 || sw.ntSubInit != 0))
      throw std::runtime_error("coupled rotors: sub-iterations (ntSub, ntSubInit) are not supported");
  }
  void readGeom(const Namelist& g) {
    std::string ver = g.s("VERSION", "fileFormatVersion", "");
    if (!ver.empty() && std::fabs(Namelist::todouble(ver) - 0.15) > 1e-12) throw std::runtime_error("geomXX.nml template version does not match");
    R.surfaceType = g.i("SURFACE", "surfaceType");
    R.imagePlane = g.i("SURFACE", "imagePlane");
    R.imageRotorNum = g.i("SURFACE", "imageRotorNum");
    R.nb = g.i("PANELS", "nb", 1);
    R.propConvention = g.i("PANELS", "propConvention");
    R.spanSpacing = g.i("PANELS", "spanSpacing", 1);
    R.chordSpacing = g.i("PANELS", "chordSpacing", 1);
    R.geometryFile = g.s("PANELS", "geometryFile", "0");
    R.nCamberFiles = g.i("PANELS", "nCamberFiles");
    R.nc = g.i("PANELS", "nc", 1);
    R.ns = g.i("PANELS", "ns", 1);
    R.nNwake = g.i("PANELS", "nNwake");
    R.hubCoords = g.v3("ORIENT", "hubCoords");
    R.cgCoords = g.v3("ORIENT", "cgCoords");
    R.fromCoords = g.v3("ORIENT", "fromCoords");
    R.pts = g.v3("ORIENT", "phiThetaPsi");
    R.radius = g.d("GEOMPARAMS", "span");
    R.root_cut = g.d("GEOMPARAMS", "rootcut");
    R.chord = g.d("GEOMPARAMS", "chord");
    R.preconeAngle = g.d("GEOMPARAMS", "preconeAngle");
    R.Omega = g.d("GEOMPARAMS", "Omega");
    R.shaftAxis = g.v3("GEOMPARAMS", "shaftAxis");
    R.controlPitch = mk(g.d("GEOMPARAMS", "theta0"), g.d("GEOMPARAMS", "thetaC"), g.d("GEOMPARAMS", "thetaS"));
    R.thetaTwist = g.d("GEOMPARAMS", "thetaTwist");
    R.ductSwitch = g.i("GEOMPARAMS", "ductSwitch");
    R.axisymmetrySwitch = g.i("GEOMPARAMS", "axisymmetrySwitch");
    R.pivotLE = g.d("GEOMPARAMS", "pivotLE");
    R.flapHinge = g.d("GEOMPARAMS", "flapHinge");
    R.spanwiseLiftSwitch = g.i("GEOMPARAMS", "spanwiseLiftSwitch");
    R.symmetricTau = g.i("GEOMPARAMS", "symmetricTau");
    R.customTrajectorySwitch = g.i("GEOMPARAMS", "customTrajectorySwitch");
    R.velBody = g.v3("GEOMPARAMS", "velBody");
    R.omegaBody = g.v3("GEOMPARAMS", "omegaBody");
    R.forceCalcSwitch = g.i("GEOMPARAMS", "forceCalcSwitch");
    R.nAirfoils = g.i("GEOMPARAMS", "nAirfoils");
    R.apparentViscCoeff = g.d("WAKEPARAMS", "apparentViscCoeff");
    R.decayCoeff = g.d("WAKEPARAMS", "decayCoeff");
    R.wakeTruncateNt = g.i("WAKEPARAMS", "wakeTruncateNt");
    R.prescWakeAfterTruncNt = g.i("WAKEPARAMS", "prescWakeAfterTruncNt");
    R.prescWakeGenNt = g.i("WAKEPARAMS", "prescWakeGenNt");
    R.spanwiseCore = g.d("WAKEPARAMS", "spanwiseCore");
    // classdef.f90:2720-2724: a single value applies to every station
    std::vector<double> sc(R.ns + 1, 0.0);
    size_t cnt = g.count("WAKEPARAMS", "streamwiseCoreVec");
    for (size_t k = 0; k < std::min(cnt, sc.size()); ++k) sc[k] = g.d("WAKEPARAMS", "streamwiseCoreVec", 0, k);
    double tail = 0.0;
    for (size_t k = 1; k < sc.size(); ++k) tail = tail + sc[k] * sc[k];
    if (std::sqrt(tail) < EPS) std::fill(sc.begin(), sc.end(), sc[0]);
    R.streamwiseCoreVec = sc;
    R.rollupStartRadius = g.d("WAKEPARAMS", "rollupStartRadius");
    R.rollupEndRadius = g.d("WAKEPARAMS", "rollupEndRadius");
    R.initWakeVel = g.d("WAKEPARAMS", "initWakeVel");
    R.psiStart = g.d("WAKEPARAMS", "psiStart");
    R.skewLimit = g.d("WAKEPARAMS", "skewLimit");
    R.bladeDynamicsSwitch = g.i("DYNAMICS", "bladeDynamicsSwitch");
    R.flapInitial = g.d("DYNAMICS", "flapInitial");
    R.dflapInitial = g.d("DYNAMICS", "dflapInitial");
    R.Iflap = g.d("DYNAMICS", "Iflap");
    R.cflap = g.d("DYNAMICS", "cflap");
    R.kflap = g.d("DYNAMICS", "kflap");
    R.MflapConstant = g.d("DYNAMICS", "MflapConstant");
    R.pitchDynamicsSwitch = g.i("DYNAMICS", "pitchDynamicsSwitch");
    R.dpitch = g.d("DYNAMICS", "dpitch");
    R.bodyDynamicsSwitch = g.i("DYNAMICS", "bodyDynamicsSwitch");
    R.bodyDynamicsIOVars = g.i("DYNAMICS", "bodyDynamicsIOVars");
    R.inflowPlotSwitch = g.i("PLOTS", "inflowPlotSwitch");
    R.gammaPlotSwitch = g.i("PLOTS", "gammaPlotSwitch");
    R.skewPlotSwitch = g.i("PLOTS", "skewPlotSwitch");
    if (R.surfaceType < 0 || std::abs(R.surfaceType) == 2) throw std::runtime_error("only lifting surfaces (surfaceType 0/1) are supported");
    if (R.nCamberFiles > 0) {
      for (int k = 0; k < R.nCamberFiles; ++k) {
        R.camberSectionLimit.push_back(g.d("CAMBERSECTIONS", "camberSectionLimit", 1.0, k));
        R.camberFile.push_back(g.s("CAMBERSECTIONS", "camberFile", "0", k));
      }
    }
    if (R.ductSwitch != 0) throw std::runtime_error("ductSwitch is not supported by this oracle");
    if (R.forceCalcSwitch < 0 || R.forceCalcSwitch > 1)
      throw std::runtime_error("only forceCalcSwitch = 0 or 1 is supported");
    // AIRFOILS (classdef.f90:2605, 2754-2765)
    if (R.forceCalcSwitch > 0 && R.nAirfoils == 0) throw std::runtime_error("No. of airfoil tables set to 0 in geomXX.in");
    for (int i = 0; i < R.nAirfoils; ++i) {
      R.airfoilSectionLimit.push_back(g.d("AIRFOILS", "airfoilSectionLimit", 1.0, i));
      R.alpha0v.push_back(g.d("AIRFOILS", "alpha0", 0.0, i));
      R.airfoilFile.push_back(g.s("AIRFOILS", "airfoilFile", "0", i));
    }
    if (R.forceCalcSwitch == 1 && R.axisymmetrySwitch == 1)
      throw std::runtime_error("forceCalcSwitch = 1 with axisymmetry is not supported");
    if (R.bladeDynamicsSwitch != 0 || R.bodyDynamicsSwitch != 0)
      throw std::runtime_error("blade/body dynamics are not supported");
    if (R.customTrajectorySwitch != 0 && R.customTrajectorySwitch != 1)
      throw std::runtime_error("customTrajectorySwitch must be 0 or 1");
  }
  // classdef.f90:3957-4020
  std::vector<V3> readPlot3d(const std::string& path, int& nx, int& ny) {
    std::ifstream f(path);
    if (!f) throw std::runtime_error("cannot open PLOT3D file " + path);
    int nz;
    f >> nx >> ny >> nz;
    if (nz > 1 || nx != R.nc + 1 || ny != R.ns + 1) throw std::runtime_error("Wrong or conflicting data in PLOT3D file");
    std::vector<V3> g(size_t(nx) * ny);
    for (int c = 0; c < 3; ++c)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
          double v;
          f >> v;
          V3& p = g[i + nx * j];
          (c == 0 ? p.x : (c == 1 ? p.y : p.z)) = v;
        }
    return g;
  }
  // classdef.f90:2769-3891
  // rotor_getCamber (classdef.f90:4060-4112): z of the chordwise points x at
  // the spanwise stations y from the camber files (first value the point
  // count, then x z pairs; normalised by the last x), the file of a station
  // the first section whose limit is >= y/span.  Returns [i + nx j].
  std::vector<double> getCamber(const std::vector<double>& x, const std::vector<double>& y) {
    const int nx = (int)x.size(), ny = (int)y.size(), nf = R.nCamberFiles;
    const double chord = x[nx - 1] - x[0];
    const double span = y[ny - 1] - y[0];
    std::vector<std::vector<double>> xc(nf), zc(nf);
    for (int j = 0; j < nf; ++j) {
      if (R.camberFile[j].empty() || R.camberFile[j][0] == '0') {
        xc[j] = {0.0, 1.0};
        zc[j] = {0.0, 0.0};
        continue;
      }
      std::string path = R.camberFile[j];
      if (path[0] != '/' && !baseDir.empty()) path = baseDir + "/" + path;
      std::ifstream f(path);
      if (!f) throw std::runtime_error("cannot open camber file " + path);
      std::stringstream ss;
      ss << f.rdbuf();
      std::string t = ss.str();
      for (char& c : t) if (c == ',') c = ' '; else if (c == 'd' || c == 'D') c = 'e';
      std::istringstream in(t);
      double np = 0;
      if (!(in >> np) || np < 2) throw std::runtime_error(path + ": bad point count");
      for (int i = 0; i < (int)np; ++i) {
        double a, b;
        if (!(in >> a >> b)) throw std::runtime_error(path + ": fewer points than its count");
        xc[j].push_back(a);
        zc[j].push_back(b);
      }
      const double xl = xc[j].back();
      for (auto& v : zc[j]) v = v / xl;
      for (auto& v : xc[j]) v = v / xl;
    }
    std::vector<double> out((size_t)nx * ny, 0.0);
    int fNum = -1;
    for (int j = 0; j < ny; ++j) {
      for (int k = 0; k < nf; ++k)
        if (y[j] / span <= R.camberSectionLimit[k]) { fNum = k; break; }
      if (fNum < 0) throw std::runtime_error("camberSectionLimit does not cover the first station");
      for (int i = 0; i < nx; ++i)
        out[(size_t)i + (size_t)nx * j] = chord * interp1d2((x[i] - x[0]) / chord, xc[fNum], zc[fNum]);
    }
    return out;
  }

  // trajectory01.in (classdef.f90:3065-3081): nt list-directed records of
  // u v w p q r; a record's values may run over lines, extra values on its
  // last line are skipped
  void readTrajectory() {
    std::string path = "trajectory01.in";
    if (!baseDir.empty()) path = baseDir + "/" + path;
    std::ifstream f(path);
    if (!f) throw std::runtime_error("cannot open " + path);
    R.velBodyHistory.assign(nt, V3());
    R.omegaBodyHistory.assign(nt, V3());
    std::string line;
    for (int i = 0; i < nt; ++i) {
      double v[6];
      int got = 0;
      while (got < 6) {
        if (!std::getline(f, line)) throw std::runtime_error(path + ": fewer than nt records");
        for (char& c : line) if (c == ',' || c == 'd' || c == 'D') c = (c == ',') ? ' ' : 'e';
        std::istringstream ls(line);
        double x;
        while (got < 6 && ls >> x) v[got++] = x;
      }
      R.velBodyHistory[i] = mk(v[0], v[1], v[2]);
      R.omegaBodyHistory[i] = mk(v[3], v[4], v[5]);
    }
  }

  void init() {
    Rotor& r = R;
    if (dt < 0 || std::signbit(dt)) {
      if (std::fabs(r.Omega) < EPS) dt = std::fabs(dt) * r.chord / norm2(r.velBody);
      else dt = TWO_PI * std::fabs(dt) / std::fabs(r.Omega);
    }
    if (std::fabs(dt) <= EPS) {
      if (std::fabs(r.Omega) < EPS) dt = (r.chord / double(r.nc)) / norm2(r.velBody);
      else dt = 5.0 * DEG2RAD / std::fabs(r.Omega);
    }
    if (nt <= 0) { if (nt == 0) nt = -10; toChordsRevs(nt); }
    if (sw.slowStart != 0) toChordsRevs(sw.slowStartNt);
    toChordsRevs(sw.wakeTipPlot); toChordsRevs(sw.wakePlot); toChordsRevs(sw.gridPlot);
    toChordsRevs(r.wakeTruncateNt); toChordsRevs(r.prescWakeAfterTruncNt); toChordsRevs(r.prescWakeGenNt);
    toChordsRevs(r.nNwake); toChordsRevs(r.inflowPlotSwitch); toChordsRevs(r.gammaPlotSwitch); toChordsRevs(r.skewPlotSwitch);
    r.prescWakeNt = (r.wakeTruncateNt > 0 && r.prescWakeAfterTruncNt > 0) ? r.wakeTruncateNt + r.prescWakeAfterTruncNt : 0;
    if (r.wakeTruncateNt > 0) r.wakeTruncateNt = std::max(r.wakeTruncateNt, r.nNwake + 1);
    if (r.surfaceType == 0) r.surfaceType = 1;
    if (r.nNwake > 0 && r.nNwake < 2) throw std::runtime_error("Atleast 2 near wake rows mandatory");
    r.xAxisBody = mk(1, 0, 0); r.yAxisBody = mk(0, 1, 0); r.zAxisBody = mk(0, 0, 1);
    r.nNwake = std::min(r.nNwake, nt);
    if (r.customTrajectorySwitch == 1) readTrajectory();
    r.nFwake = r.wakeTruncateNt == 0 ? nt - r.nNwake : r.wakeTruncateNt - r.nNwake;
    if (r.nNwake == 0) r.nFwake = 0;
    r.nbConvect = r.axisymmetrySwitch == 1 ? 1 : r.nb;
    r.nNwakeEnd = r.nNwake;
    r.nFwakeEnd = r.nFwake;
    int nc = r.nc, ns = r.ns, NW = r.nNwake, NF = r.nFwake;
    r.blade.assign(r.nb, Blade());
    int n = r.n();
    r.AIC.assign(size_t(n) * n, 0.0); r.AIC_inv = r.AIC;
    r.gamVec.assign(n, 0.0); r.gamVecPrev.assign(n, 0.0); r.RHS.assign(n, 0.0);
    for (auto& b : r.blade) {
      b.nc = nc; b.ns = ns;
      b.wiP.assign(size_t(nc) * ns, WingPanel());
      if (NW > 0) { b.waN.assign(size_t(NW) * ns, VR()); b.waF.assign(NF, FW()); }
      auto z3 = std::vector<V3>(ns);
      auto z1 = std::vector<double>(ns, 0.0);
      b.secTauCapChord = b.secTauCapSpan = b.secNormalVec = b.secForceInertial = b.secLift = b.secLiftDir = z3;
      b.secDragDir = b.secLiftInPlane = b.secLiftOutPlane = b.secLiftInPlaneUnsteady = b.secLiftOutPlaneUnsteady = z3;
      b.secLiftUnsteady = b.secDrag = b.secDragInduced = b.secDragProfile = b.secDragUnsteady = z3;
      b.secChordwiseResVel = b.secCP = z3;
      b.secChord = b.secArea = b.secAlpha = b.secPhi = b.secTheta = b.secViz = b.secVix = z1;
      b.secCL = b.secCD = b.secCLu = b.secMflap = b.secMflapArm = z1;
    }
    r.controlPitch = r.controlPitch * DEG2RAD;
    r.pts = r.pts * DEG2RAD;
    r.thetaTwist = r.thetaTwist * DEG2RAD;
    r.preconeAngle = r.preconeAngle * DEG2RAD;
    r.psiStart = r.psiStart * DEG2RAD;
    r.spanwiseCore = r.spanwiseCore * r.chord;
    for (auto& s : r.streamwiseCoreVec) s = s * r.chord;
    r.rollupStart = (int)std::ceil(r.rollupStartRadius * double(ns));
    r.rollupEnd = (int)std::floor(r.rollupEndRadius * double(ns));
    r.lift = V3();
    // blade geometry
    if (r.geometryFile.empty() || r.geometryFile[0] == '0') {
      std::vector<double> xVec;
      double cs = r.Omega >= 0 ? -r.chord : r.chord;
      switch (r.chordSpacing) {
        case 1: xVec = linspace(cs, 0.0, nc + 1); break;
        case 2: xVec = cosspace(cs, 0.0, nc + 1); break;
        case 3: xVec = halfsinspace(cs, 0.0, nc + 1); break;
        case 4: xVec = tanspace(cs, 0.0, nc + 1); break;
        default: throw std::runtime_error("bad chordSpacing");
      }
      double s0 = r.root_cut * r.radius, s1 = r.radius;
      std::vector<double> yv;
      switch (r.spanSpacing) {
        case 1: yv = linspace(s0, s1, ns + 1); break;
        case 2: yv = cosspace(s0, s1, ns + 1); break;
        case 3: yv = halfsinspace(s0, s1, ns + 1); break;
        case 4: yv = tanspace(s0, s1, ns + 1); break;
        default: throw std::runtime_error("bad spanSpacing");
      }
      std::vector<double> zv((size_t)(nc + 1) * (ns + 1), 0.0);  // [i + (nc+1) j]
      if (r.nCamberFiles > 0) zv = getCamber(xVec, yv);
      if (imageOf && r.imagePlane == 3)  // classdef.f90:3228-3230
        for (auto& v : zv) v = -1.0 * v;
      auto z = [&](int i, int j) { return zv[(size_t)i + (size_t)(nc + 1) * j]; };
      for (auto& b : r.blade)
        for (int j = 0; j < ns; ++j)
          for (int i = 0; i < nc; ++i) {
            WingPanel& p = b.w(i, j);
            p.PC[0] = mk(xVec[i], yv[j], z(i, j));
            p.PC[1] = mk(xVec[i + 1], yv[j], z(i + 1, j));
            p.PC[2] = mk(xVec[i + 1], yv[j + 1], z(i + 1, j + 1));
            p.PC[3] = mk(xVec[i], yv[j + 1], z(i, j + 1));
          }
    } else {
      int nx, ny;
      std::string path = r.geometryFile;
      if (path[0] != '/' && !baseDir.empty()) path = baseDir + "/" + path;
      auto g = readPlot3d(path, nx, ny);
      if (imageOf && r.imagePlane == 3)  // classdef.f90:3989-3995
        for (auto& q : g) q.z = -1.0 * q.z;
      for (int ib = 0; ib < r.nbConvect; ++ib)
        for (int is = 0; is < ns; ++is)
          for (int ic = 0; ic < nc; ++ic) {
            WingPanel& p = r.blade[ib].w(ic, is);
            p.PC[0] = g[ic + nx * is];
            p.PC[1] = g[ic + 1 + nx * is];
            p.PC[2] = g[ic + 1 + nx * (is + 1)];
            p.PC[3] = g[ic + nx * (is + 1)];
          }
      if (r.axisymmetrySwitch == 1)
        for (int ib = 1; ib < r.nb; ++ib)
          for (size_t k = 0; k < r.blade[ib].wiP.size(); ++k)
            for (int c = 0; c < 4; ++c) r.blade[ib].wiP[k].PC[c] = r.blade[0].wiP[k].PC[c];
    }
    V3 X = mk(1, 0, 0), Y = mk(0, 1, 0), Z = mk(0, 0, 1);
    for (int ib = 0; ib < r.nbConvect; ++ib) {
      Blade& b = r.blade[ib];
      b.xAxis = X; b.yAxis = Y; b.zAxis = Z;
      b.xAxisAzi = X; b.yAxisAzi = Y; b.zAxisAzi = Z;
      b.xAxisAziFlap = X; b.yAxisAziFlap = Y; b.zAxisAziFlap = Z;
      b.flapOrigin = (b.yAxis * r.radius) * r.flapHinge;
      for (int j = 0; j < ns; ++j) {
        b.secTauCapChord[j] = ((b.w(nc - 1, j).PC[2] + b.w(nc - 1, j).PC[1]) - (b.w(0, j).PC[3] + b.w(0, j).PC[0])) * 0.5;
        b.secTauCapSpan[j] = Y;
        b.secNormalVec[j] = cross(b.w(nc - 1, j).PC[1] - b.w(0, j).PC[3], b.w(nc - 1, j).PC[2] - b.w(0, j).PC[0]);
        b.secTauCapChord[j] = unitVec(b.secTauCapChord[j]);
        b.secNormalVec[j] = fsign(1.0, r.Omega) * unitVec(b.secNormalVec[j]);
      }
      for (int j = 0; j < ns; ++j)
        for (int i = 0; i < nc - 1; ++i) {
          WingPanel& p = b.w(i, j);
          const WingPanel& q = b.w(i + 1, j);
          double xs[4];
          xs[0] = (p.PC[1].x - p.PC[0].x) * 0.25;
          xs[1] = (q.PC[1].x - p.PC[1].x) * 0.25;
          xs[2] = (q.PC[2].x - p.PC[2].x) * 0.25;
          xs[3] = (p.PC[2].x - p.PC[3].x) * 0.25;
          for (int c = 0; c < 4; ++c) p.vr.assignP(c + 1, mk(p.PC[c].x + xs[c], p.PC[c].y, p.PC[c].z));
        }
      for (int j = 0; j < ns; ++j) {
        WingPanel& p = b.w(nc - 1, j);
        double xs[4];
        xs[0] = (p.PC[1].x - p.PC[0].x) * 0.25;
        xs[1] = 0.0;
        xs[2] = 0.0;
        xs[3] = (p.PC[2].x - p.PC[3].x) * 0.25;
        for (int c = 0; c < 4; ++c) p.vr.assignP(c + 1, mk(p.PC[c].x + xs[c], p.PC[c].y, p.PC[c].z));
      }
      double dxdymin = 1e300;
      for (int is = 0; is < ns; ++is)
        for (int ic = 0; ic < nc; ++ic) {
          dxdymin = std::min(dxdymin, std::fabs(norm2(b.w(ic, is).PC[1] - b.w(ic, is).PC[0])));
        }
      double dymin = 1e300;
      for (int is = 0; is < ns; ++is)
        for (int ic = 0; ic < nc; ++ic) dymin = std::min(dymin, std::fabs(norm2(b.w(ic, is).PC[2] - b.w(ic, is).PC[1])));
      dxdymin = std::min(dxdymin, dymin);
      // shed last row of vortices (classdef.f90:3388-3400); 0.05 is a
      // single precision literal in the reference
      double velShed;
      if (std::fabs(r.Omega) > EPS) {
        velShed = std::min((double(0.05f) * std::fabs(r.Omega)) * norm2(b.w(nc - 1, ns - 1).vr.vf[1].fc1 - r.hubCoords),
                           0.125 * r.chord / dt);
      } else {
        velShed = 0.3 * norm2(-1.0 * r.velBody);
      }
      V3 sh = mk((fsign(1.0, r.Omega) * velShed) * dt, 0.0, 0.0);
      for (int j = 0; j < ns; ++j) { b.w(nc - 1, j).vr.shiftdP(2, sh); b.w(nc - 1, j).vr.shiftdP(3, sh); }
      for (int j = 0; j < ns; ++j)
        for (int i = 0; i < nc; ++i) {
          WingPanel& p = b.w(i, j);
          p.calcCP();
          p.calcN();
          if (fsign(1.0, r.Omega) < 0.0) p.nCap = -1.0 * p.nCap;
          p.calcTau();
          p.rHinge = norm2((b.w(0, j).PC[0] + b.w(0, j).PC[3]) * 0.5 - p.CP);
          p.calc_area();
          p.calc_mean_dimensions();
        }
      if (imageOf)  // classdef.f90:3434-3443: the source's normals, mirrored
        for (int j = 0; j < ns; ++j)
          for (int i = 0; i < nc; ++i) {
            V3 n = imageOf->R.blade[ib].w(i, j).nCap;
            comp(n, r.imagePlane) = -1.0 * comp(n, r.imagePlane);
            b.w(i, j).nCap = n;
          }
      for (int is = 0; is < ns; ++is) {
        double s = 0.0;
        for (int ic = 0; ic < nc; ++ic) s = s + b.w(ic, is).panelArea;
        b.secArea[is] = s;
        b.secChord[is] = norm2(0.5 * ((b.w(0, is).PC[0] + b.w(0, is).PC[3]) - (b.w(nc - 1, is).PC[1] + b.w(nc - 1, is).PC[2])));
      }
      b.spanwiseLiftSwitch = r.spanwiseLiftSwitch;
      for (int j = 0; j < ns; ++j) {
        b.secTauCapSpan[j] = b.yAxis;
        for (int i = 0; i < nc; ++i) b.w(i, j).tauCapSpan = b.yAxis;
      }
      if (r.symmetricTau == 1)
        for (int j = 0; j < ns / 2; ++j) {
          b.secTauCapSpan[j] = -1.0 * b.secTauCapSpan[j];
          for (int i = 0; i < nc; ++i) b.w(i, j).tauCapSpan = -1.0 * b.w(i, j).tauCapSpan;
        }
      calc_secLocations(b, 0.5, r.flapHinge * r.radius);
      for (auto& p : b.wiP) { p.vr.gam = 0.0; p.vr.skew = 0.0; }
      b.pivotLE = r.pivotLE;
      double rw = std::min(r.spanwiseCore, dxdymin * 0.1);
      for (auto& p : b.wiP)
        for (int f = 0; f < 4; ++f) p.vr.vf[f].rVc0 = rw;
      for (int j = 0; j < ns; ++j) b.w(nc - 1, j).vr.vf[1].rVc0 = r.spanwiseCore;
      for (auto& p : b.wiP)
        for (int f = 0; f < 4; ++f) p.vr.vf[f].rVc = p.vr.vf[f].rVc0;
    }
    if (r.axisymmetrySwitch == 1) {
      Blade& b0 = r.blade[0];
      for (int ib = 1; ib < r.nb; ++ib) {
        Blade& b = r.blade[ib];
        b.xAxis = b0.xAxis; b.yAxis = b0.yAxis; b.zAxis = b0.zAxis;
        b.xAxisAzi = b0.xAxisAzi; b.yAxisAzi = b0.yAxisAzi; b.zAxisAzi = b0.zAxisAzi;
        b.xAxisAziFlap = b0.xAxisAziFlap; b.yAxisAziFlap = b0.yAxisAziFlap; b.zAxisAziFlap = b0.zAxisAziFlap;
        b.flapOrigin = b0.flapOrigin;
        b.secTauCapChord = b0.secTauCapChord; b.secTauCapSpan = b0.secTauCapSpan; b.secNormalVec = b0.secNormalVec;
        for (size_t k = 0; k < b.wiP.size(); ++k) {
          WingPanel& p = b.wiP[k];
          const WingPanel& q = b0.wiP[k];
          p.vr = q.vr; p.CP = q.CP; p.nCap = q.nCap; p.tauCapChord = q.tauCapChord; p.rHinge = q.rHinge;
          p.panelArea = q.panelArea; p.meanChord = q.meanChord; p.meanSpan = q.meanSpan; p.tauCapSpan = q.tauCapSpan;
        }
        b.secArea = b0.secArea; b.secChord = b0.secChord; b.spanwiseLiftSwitch = b0.spanwiseLiftSwitch;
        b.secCP = b0.secCP; b.secMflapArm = b0.secMflapArm; b.pivotLE = b0.pivotLE;
      }
    }
    for (auto& b : r.blade) blade_move(b, r.hubCoords - r.fromCoords);
    for (auto& b : r.blade) {
      b.preconeAngle = r.preconeAngle;
      b.dflap = r.dflapInitial; b.flap = r.flapInitial;
      b.dflapPrev = b.dflap; b.flapPrev = b.flap;
      blade_rot_flap(b, r.preconeAngle);
      blade_rot_flap(b, r.flapInitial);
    }
    for (int ib = 1; ib < r.nb; ++ib) {
      double off = ((fsign(1.0, r.Omega) * TWO_PI) / double(r.nb)) * double(ib);
      blade_rotate(r.blade[ib], off, r.shaftAxis, r.hubCoords, "azimuth");
    }
    rotor_rot_pts(r.pts, r.cgCoords);
    rotor_rot_advance(fsign(1.0, r.Omega) * r.psiStart, true);
    if (std::fabs(r.Omega) > EPS) {
      if (r.propConvention == 0) {
        double ro = r.radius * r.Omega;
        r.nonDimforceDenominator = (density * (PI * (r.radius * r.radius))) * (ro * ro);
      } else {
        double f = r.Omega / TWO_PI;
        r.nonDimforceDenominator = (density * (f * f)) * p4(2.0 * r.radius);
      }
    } else {
      r.nonDimforceDenominator = ((0.5 * density) * ((r.radius * (1.0 - r.root_cut)) * r.chord)) * dot(r.velBody, r.velBody);
    }
    // section airfoils (classdef.f90:3693-3725)
    if (r.nAirfoils > 0) {
      r.c81.assign(r.nAirfoils, C81());
      for (int i = 0; i < r.nAirfoils; ++i)
        if (!r.airfoilFile[i].empty() && r.airfoilFile[i][0] != '0') {
          const std::string& f = r.airfoilFile[i];
          r.c81[i].read(f[0] == '/' || baseDir.empty() ? f : baseDir + "/" + f);
        }
      const double secCPLoc = 0.5;
      for (auto& b : r.blade) {
        b.airfoilNo.assign(ns, 1);
        if (r.nAirfoils == 1) continue;
        const V3 leftTip = b.w(0, 0).PC[3] * (1.0 - secCPLoc) + b.w(nc - 1, 0).PC[2] * secCPLoc;
        for (int is = 0; is < ns; ++is) {
          const double rbyR = std::fabs(dot(b.secCP[is] - leftTip, b.xAxis)) + r.root_cut;
          if (rbyR > 1.0) throw std::runtime_error("r/R value is greater than 1 in airfoil selection");
          for (int i = 0; i < r.nAirfoils; ++i)
            if (r.airfoilSectionLimit[i] >= rbyR) {
              b.airfoilNo[is] = i + 1;
              break;
            }
        }
      }
    }
    for (auto& b : r.blade) {
      if (NW > 0) {
        size_t nn = size_t(NW) * (ns + 1);
        b.velN.assign(nn, V3()); b.velN1 = b.velN2 = b.velN3 = b.velNP = b.velNStep = b.velN;
        b.velF.assign(NF, V3()); b.velF1 = b.velF2 = b.velF3 = b.velFP = b.velFStep = b.velF;
        b.waNP.assign(size_t(NW) * ns, VR());
        b.waFP.assign(NF, FW());
        for (int j = 0; j < ns; ++j)
          for (int i = 0; i < NW; ++i) {
            VR& w = b.waN[i + NW * j];
            w.vf[1].rVc0 = w.vf[1].rVc = r.spanwiseCore;
            w.vf[3].rVc0 = w.vf[3].rVc = r.spanwiseCore;
            w.gam = 0.0;
            w.vf[0].rVc0 = w.vf[0].rVc = r.streamwiseCoreVec[j];
            w.vf[2].rVc0 = w.vf[2].rVc = r.streamwiseCoreVec[j + 1];
          }
        for (auto& f : b.waF) { f.gam = 0.0; f.vf.rVc0 = f.vf.rVc = r.streamwiseCoreVec[ns]; }
      }
    }
  }

  // main.f90:43-58, 62-81, 95-377
  void start() {
    startGeometry();
    for (int i = 0; i <= sw.ntSubInit; ++i) {
      solveCirculation(false);
      if (sw.ntSubInit != 0) {
        double s = 0.0;
        for (int k = 0; k < R.n(); ++k) s = s + (R.gamVec[k] - R.gamVecPrev[k]) * (R.gamVec[k] - R.gamVecPrev[k]);
        if (std::sqrt(s) <= EPS) break;
      }
    }
    startWake();
    startLoads();
  }
  // main.f90:43-58, 62-81, 95-116: initial pitch, AIC and its inverse, rotor speed
  void startGeometry() {
    for (int ib = 0; ib < R.nb; ++ib) {
      Blade& b = R.blade[ib];
      if (imageOf) {
        // an image takes its source's pitch, negated in the z plane
        b.theta = imageOf->R.blade[ib].theta;
        if (R.imagePlane == 3) b.theta = -1.0 * b.theta;
      } else {
        b.theta = gettheta(R.psiStart, ib + 1);
      }
      blade_rot_pitch(b, fsign(1.0, R.Omega) * b.theta);
    }
    if (!imageOf) {
      calcAIC();
      if (!isInverse(R.AIC, R.AIC_inv, R.n())) throw std::runtime_error("Computed AIC_inv does not seem to be correct");
    }
    R.omegaSlow = sw.slowStart > 0 ? 0.0 : R.Omega;
    t = 0.0;
    iter = 0;
    if (R.customTrajectorySwitch == 1) {  // main.f90:111-116
      R.velBody = R.velBodyHistory[0];
      R.omegaBody = R.omegaBodyHistory[0];
    }
  }
  // main.f90:226-233: wake rows and the first trailing-edge shed row
  void startWake() {
    R.rowFar = R.nFwake + 1;
    R.rowNear = R.nNwake + 1;
    if (R.nNwake > 0) assignshed(false);
  }
  // main.f90:235-377: the loads of the initial solution
  void startLoads() {
    if (sw.rotorForcePlot != 0) {
      computeForces();
      for (auto& b : R.blade) b.MflapLiftPrev = b.MflapLift;
      force2file();
    }
    started = true;
  }

  // main.f90:400-1452 (one iteration)
  void step() {
    stepOpen();
    stepClose();
  }
  // main.f90:400-764: the iteration up to its loads (the point where the
  // reference writes filaments2file and probes2file, :788,795)
  void stepOpen() {
    if (!started) start();
    if (iter >= nt) throw std::runtime_error("all timesteps done");
    advanceKinematics();
    preWake();
    for (int i = 0; i <= sw.ntSub; ++i) {
      solveCirculation(true);
      if (sw.ntSub != 0) {
        double s = 0.0;
        for (int k = 0; k < R.n(); ++k) s = s + (R.gamVec[k] - R.gamVecPrev[k]) * (R.gamVec[k] - R.gamVecPrev[k]);
        if (std::sqrt(s) <= EPS) break;
      }
    }
    if (sw.rotorForcePlot != 0 && iter % sw.rotorForcePlot == 0) {
      computeForces();
      force2file();
    }
  }
  // main.f90:464-490: leading-edge shed row, ageing, dissipation, burst
  void preWake() {
    if (sw.wakeSuppress == 0 && R.nNwake > 0) {
      assignshed(true);
      age_wake();
      if (sw.wakeDissipation == 1) dissipate_wake();
      if (sw.wakeBurst != 0 && iter % sw.wakeBurst == 0) burst_wake();
    }
  }
  // main.f90:799-1452: the rest of the iteration (wake update)
  void stepClose() {
    if (sw.wakeSuppress == 0 && R.nNwake > 0) wakeUpdate();
  }

  // Iterations iter+1..k with their kinematics only (counters, slow start,
  // body motion, azimuth and pitch): the prescribed motion does not depend on
  // the flow, so this reaches iteration k's wing geometry exactly; the flow
  // state of iteration k is then set from outside (or_set).
  void skipTo(int k) {
    if (!started) start();
    if (k < iter || k > nt) throw std::runtime_error("skip target out of range");
    while (iter < k) advanceKinematics();
  }

  // main.f90:410-463: the iteration counter, rowNear/rowFar, custom
  // trajectory, slow start and the rotor's motion for one iteration
  void advanceKinematics() {
    ++iter;
    t = t + dt;
    R.rowNear = std::max(R.rowNear - 1, 1);
    if (iter > R.nNwake) R.rowFar = std::max(R.rowFar - 1, 1);
    if (R.customTrajectorySwitch == 1) {  // main.f90:419-424
      R.velBody = R.velBodyHistory[iter - 1];
      R.omegaBody = R.omegaBodyHistory[iter - 1];
    }
    switch (sw.slowStart) {
      case 0: R.omegaSlow = R.Omega; break;
      case 1: R.omegaSlow = double(std::min(float(sw.slowStartNt), float(iter + 1))) * R.Omega / double(sw.slowStartNt); break;
      case 2: R.omegaSlow = std::tanh(5.0 * double(iter) / double(sw.slowStartNt)) * R.Omega; break;
      case 3:
        R.omegaSlow = ((std::tanh(6.0 * double(float(iter)) / double(float(sw.slowStartNt)) - 3.0) + 1.0) * 0.5) * R.Omega;
        break;
      default: break;
    }
    rotor_move(R.velBody * dt);
    rotor_rot_pts(R.omegaBody * dt, R.cgCoords);
    rotor_rot_advance(R.omegaSlow * dt, false);
  }

  void addInitWakeVel(Blade& b, bool pred) {
    if (!(iter < sw.initWakeVelNt)) return;
    int NW = R.nNwake, ns = R.ns;
    std::vector<V3>& vn = pred ? b.velNP : b.velN;
    std::vector<V3>& vf = pred ? b.velFP : b.velF;
    V3 a = R.initWakeVel * R.shaftAxis;
    for (int j = 0; j <= ns; ++j)
      for (int i = R.rowNear - 1; i < NW; ++i) vn[i + NW * j] = pred ? vn[i + NW * j] - a : vn[i + NW * j] + a;
    for (int i = R.rowFar - 1; i < R.nFwake; ++i) vf[i] = vf[i] - a;
  }
  void evalWakeVel(bool pred) {
    int NW = R.nNwake, ns = R.ns;
    for (int ib = 0; ib < R.nbConvect; ++ib) {
      Blade& b = R.blade[ib];
      std::vector<V3>& vn = pred ? b.velNP : b.velN;
      std::vector<V3>& vf = pred ? b.velFP : b.velF;
      for (int j = 0; j <= ns; ++j)
        for (int i = R.rowNear - 1; i < NW; ++i) vn[i + NW * j] = V3();
      for (int i = R.rowFar - 1; i < R.nFwake; ++i) vf[i] = V3();
      vind_onWake(ib, pred, vn, vf);
      addInitWakeVel(b, pred);
    }
  }
  void copyPredicted() {
    int NW = R.nNwake;
    for (int ib = 0; ib < R.nbConvect; ++ib) {
      Blade& b = R.blade[ib];
      for (int j = 0; j < R.ns; ++j)
        for (int i = R.rowNear - 1; i < NW; ++i) b.waNP[i + NW * j] = b.waN[i + NW * j];
      for (int i = R.rowFar - 1; i < R.nFwake; ++i) b.waFP[i] = b.waF[i];
    }
  }
  template <class F>
  void forAllVel(F f) {
    for (int ib = 0; ib < R.nbConvect; ++ib) {
      Blade& b = R.blade[ib];
      for (size_t k = 0; k < b.velN.size(); ++k) f(b.velN[k], b.velN1[k], b.velN2[k], b.velN3[k], b.velNP[k], b.velNStep[k]);
      for (size_t k = 0; k < b.velF.size(); ++k) f(b.velF[k], b.velF1[k], b.velF2[k], b.velF3[k], b.velFP[k], b.velFStep[k]);
    }
  }
  // ---- image rotors (classdef.f90:4990-5131) ----------------------------------
  // rotor_mirrorVelCP: velCP and velCPm of the source, the image-plane
  // component negated
  void mirrorVelCP() {
    const int pl = R.imagePlane;
    for (int ib = 0; ib < R.nb; ++ib)
      for (size_t k = 0; k < R.blade[ib].wiP.size(); ++k) {
        WingPanel& p = R.blade[ib].wiP[k];
        const WingPanel& q = imageOf->R.blade[ib].wiP[k];
        p.velCP = q.velCP;
        p.velCPm = q.velCPm;
        comp(p.velCP, pl) = -1.0 * comp(p.velCP, pl);
        comp(p.velCPm, pl) = -1.0 * comp(p.velCPm, pl);
      }
  }
  // rotor_mirrorGamma (after gamVecPrev = gamVec, main.f90:594-600) + map_gam
  void mirrorGamma() {
    R.gamVecPrev = R.gamVec;
    for (size_t i = 0; i < R.gamVec.size(); ++i) R.gamVec[i] = -1.0 * imageOf->R.gamVec[i];
    map_gam();
  }
  // rotor_mirrorWake: mode 'C' the active current wake, 'P' the active
  // predicted wake, 'A' every row of the current wake; whole ring / filament
  // objects copied, then their node coordinates in the image plane and their
  // circulation negated (vr_mirror, Fwake_mirror: classdef.f90:722-735, 982-993)
  void mirrorWake(char mode) {
    const int pl = R.imagePlane, NW = R.nNwake, NF = R.nFwake;
    const int r0 = mode == 'A' ? 0 : R.rowNear - 1, f0 = mode == 'A' ? 0 : R.rowFar - 1;
    for (int ib = 0; ib < R.nb; ++ib) {
      Blade& b = R.blade[ib];
      const Blade& q = imageOf->R.blade[ib];
      std::vector<VR>& wn = mode == 'P' ? b.waNP : b.waN;
      const std::vector<VR>& qn = mode == 'P' ? q.waNP : q.waN;
      std::vector<FW>& wf = mode == 'P' ? b.waFP : b.waF;
      const std::vector<FW>& qf = mode == 'P' ? q.waFP : q.waF;
      for (int j = 0; j < b.ns; ++j)
        for (int i = r0; i < NW; ++i) {
          VR& v = wn[i + NW * j];
          v = qn[i + NW * j];
          for (auto& f : v.vf) {
            comp(f.fc1, pl) = -1.0 * comp(f.fc1, pl);
            comp(f.fc2, pl) = -1.0 * comp(f.fc2, pl);
          }
          v.gam = -1.0 * v.gam;
        }
      for (int i = f0; i < NF; ++i) {
        FW& f = wf[i];
        f = qf[i];
        comp(f.vf.fc1, pl) = -1.0 * comp(f.vf.fc1, pl);
        comp(f.vf.fc2, pl) = -1.0 * comp(f.vf.fc2, pl);
        f.gam = -1.0 * f.gam;
      }
    }
  }
  // the wake update of an image (main.f90:844-1439): no velocities; the
  // source's wake mirrored where the source convects
  void imageWakeStage(int st) {
    if (st == 1) mirrorWake(predicts() ? 'P' : 'C');
    else if (st == 3) {
      if (predicts()) mirrorWake('C');
      mirrorWake('A');
    }
  }

  // main.f90:799-1439, run as four stages so that a system of rotors runs
  // each stage for every rotor before the next (the reference's do-ir loops):
  // 0 the node velocities, 1 the scheme up to the predicted wake, 2 the
  // predicted-wake velocities, 3 the corrector, strain and roll-up.
  void wakeUpdate() {
    for (int st = 0; st < 4; ++st) wakeStage(st);
  }
  // whether this iteration's scheme evaluates the predicted wake
  bool predicts() const {
    switch (sw.fdScheme) {
      case 1: return true;
      case 3: return iter != 1;
      case 4: return iter != 2;  // the reference tests iter == 0 (never true), main.f90:1118
      case 5: return iter > 3;
      default: return false;
    }
  }
  void wakeStage(int st) {
    int fd = sw.fdScheme;
    if (st == 0) {
      evalWakeVel(false);
      return;
    }
    if (st == 2) {
      if (predicts()) evalWakeVel(true);
      return;
    }
    if (st == 3) {
      wakeCorrector();
      if (sw.wakeStrain == 1) strain_wake();
      if (R.rowNear == 1) { rollup(); assignshed(false); }
      else assignshed(false);
      return;
    }
    // st == 1: the scheme up to its predicted wake (all of it when it has none)
    if (fd == 0) {
      rotor_convectwake(false);
    } else if (fd == 1) {
      copyPredicted();
      rotor_convectwake(true);
    } else if (fd == 2) {
      if (iter == 1) {
        rotor_convectwake(false);
        forAllVel([](V3& v, V3& v1, V3&, V3&, V3&, V3&) { v1 = v; });
      } else {
        forAllVel([](V3& v, V3& v1, V3&, V3&, V3&, V3& st) {
          st = 0.5 * (3.0 * v - v1);
          v1 = st;
          v = st;
        });
        rotor_convectwake(false);
      }
    } else if (fd == 3) {
      if (iter == 1) {
        rotor_convectwake(false);
        forAllVel([](V3& v, V3& v1, V3&, V3&, V3&, V3&) { v1 = v; });
      } else {
        copyPredicted();
        forAllVel([](V3& v, V3& v1, V3&, V3&, V3&, V3& st) {
          st = v;
          v = 0.5 * (3.0 * v - v1);
        });
        rotor_convectwake(true);
      }
    } else if (fd == 4) {
      if (iter == 2) {
        rotor_convectwake(false);
        forAllVel([](V3& v, V3&, V3& v2, V3&, V3&, V3&) { v2 = v; });
      } else {
        copyPredicted();
        forAllVel([](V3& v, V3& v1, V3& v2, V3&, V3&, V3& st) {
          st = v;
          v = ((23.0 * v - 16.0 * v2) + 5.0 * v1) / 12.0;
        });
        rotor_convectwake(true);
      }
    } else if (fd == 5) {
      if (iter <= 3) {
        rotor_convectwake(false);
        int it = iter;
        forAllVel([it](V3& v, V3& v1, V3& v2, V3& v3, V3&, V3&) {
          if (it == 1) v1 = v; else if (it == 2) v2 = v; else v3 = v;
        });
      } else {
        copyPredicted();
        forAllVel([](V3& v, V3& v1, V3& v2, V3& v3, V3&, V3& st) {
          st = v;
          v = (((55.0 * v - 59.0 * v3) + 37.0 * v2) - 9.0 * v1) / 24.0;
        });
        rotor_convectwake(true);
      }
    } else {
      throw std::runtime_error("bad fdScheme");
    }
  }
  // the schemes' corrector (after the predicted-wake velocities)
  void wakeCorrector() {
    if (!predicts()) return;
    int fd = sw.fdScheme;
    if (fd == 1) {
      // libCommon.f90:213-258: stencil indices are relative to rowNear/rowFar
      int NW = R.nNwake, ns = R.ns;
      for (int ib = 0; ib < R.nbConvect; ++ib) {
        Blade& b = R.blade[ib];
        int r0 = R.rowNear - 1, m = NW - r0;
        std::vector<V3> out(size_t(m) * (ns + 1));
        for (int j = 0; j <= ns; ++j) {
          auto vn = [&](int i) { return b.velN[r0 + i + NW * j]; };
          auto vp = [&](int i) { return b.velNP[r0 + i + NW * j]; };
          out[0 + m * j] = (vp(0) + vn(0)) * 0.5;
          for (int i = 1; i < m - 1; ++i) out[i + m * j] = (((vp(i) + vp(i - 1)) + vn(i + 1)) + vn(i)) * 0.25;
          out[(m - 1) + m * j] = (vp(m - 1) + vn(m - 1)) * 0.5;
        }
        for (int j = 0; j <= ns; ++j)
          for (int i = 0; i < m; ++i) b.velN[r0 + i + NW * j] = out[i + m * j];
        int f0 = R.rowFar - 1, mf = R.nFwake - f0;
        if (mf > 0) {
          std::vector<V3> of(mf);
          auto fn = [&](int i) { return b.velF[f0 + i]; };
          auto fp = [&](int i) { return b.velFP[f0 + i]; };
          of[0] = (fp(0) + fn(0)) * 0.5;
          for (int i = 1; i < mf - 1; ++i) of[i] = (((fp(i) + fp(i - 1)) + fn(i + 1)) + fn(i)) * 0.25;
          of[mf - 1] = (fp(mf - 1) + fn(mf - 1)) * 0.5;
          for (int i = 0; i < mf; ++i) b.velF[f0 + i] = of[i];
        }
      }
      rotor_convectwake(false);
    } else if (fd == 3) {
      forAllVel([](V3& v, V3&, V3&, V3&, V3& vp, V3& st) { v = (vp + st) * 0.5; });
      rotor_convectwake(false);
      forAllVel([](V3&, V3& v1, V3&, V3&, V3&, V3& st) { v1 = st; });
    } else if (fd == 4) {
      forAllVel([](V3& v, V3&, V3& v2, V3&, V3& vp, V3& st) { v = ((5.0 * vp + 8.0 * st) - 1.0 * v2) / 12.0; });
      rotor_convectwake(false);
      forAllVel([](V3&, V3& v1, V3& v2, V3&, V3&, V3& st) { v1 = v2; v2 = st; });
    } else if (fd == 5) {
      forAllVel([](V3& v, V3&, V3& v2, V3& v3, V3& vp, V3& st) {
        v = (((9.0 * vp + 19.0 * st) - 5.0 * v3) + 1.0 * v2) / 24.0;
      });
      rotor_convectwake(false);
      forAllVel([](V3&, V3& v1, V3& v2, V3& v3, V3&, V3& st) { v1 = v2; v2 = v3; v3 = st; });
    }
  }
};

// Coupled rotors (nr > 1): rotor(1..nr) of main.f90, each a Sim whose
// induced-velocity sums run over all of them (Sim::sys), advanced with
// every do-ir loop of the reference's iteration run over the rotors in
// order: kinematics, shedding/ageing/dissipation, all RHS (every wake, the
// other wings, main.f90:522-591), all solves, all loads (every rotor's bound
// vortices, :623-690), and the wake update stage by stage (node velocities
// from every rotor's wing and wake, :799-1439).  Lifting surfaces only
// (no image rotors, surfaceType >= 0) and no sub-iterations.
struct System {
  std::vector<std::unique_ptr<Sim>> r;
  // main.f90:17-39: config.nml once, geomXX.nml per rotor; each rotor's init
  // sees dt, nt and the switches as the previous one left them
  // (classdef.f90:2778-3011, intent(inout))
  void create(int nr, const std::string& config, const std::vector<std::string>& geoms, const std::string& base) {
    Namelist c;
    c.parse(config);
    if (nr < 1 || (int)geoms.size() != nr) throw std::runtime_error("system: one geometry per rotor");
    for (int ir = 0; ir < nr; ++ir) {
      auto s = std::make_unique<Sim>();
      s->member = true;
      s->baseDir = base;
      s->readConfig(c);
      if (s->nr != nr) throw std::runtime_error("system: config.nml nr does not match the number of geometries");
      if (ir > 0) {
        s->dt = r[ir - 1]->dt;
        s->nt = r[ir - 1]->nt;
        s->sw = r[ir - 1]->sw;
      }
      Namelist g;
      g.parse(geoms[ir]);
      const int st = g.i("SURFACE", "surfaceType");
      if (std::abs(st) == 2) throw std::runtime_error("system: non-lifting surfaces are not supported");
      if (st < 0) {
        // an image: its source's parameters (classdef.f90:2797-2910) with its
        // own surface entries and geometry file, hub and cg mirrored
        const int src = g.i("SURFACE", "imageRotorNum");
        if (src < 1 || src > ir || r[src - 1]->imageOf)
          throw std::runtime_error("system: an image rotor must mirror an earlier lifting rotor");
        Namelist gs;
        gs.parse(geoms[src - 1]);
        s->readGeom(gs);
        s->R.surfaceType = st;
        s->R.imagePlane = g.i("SURFACE", "imagePlane");
        s->R.imageRotorNum = src;
        s->R.geometryFile = g.s("PANELS", "geometryFile", "0");
        if (s->R.imagePlane < 1 || s->R.imagePlane > 3) throw std::runtime_error("imagePlane must be 1, 2 or 3");
        const Rotor& q = r[src - 1]->R;
        if (q.customTrajectorySwitch != 0 || q.prescWakeAfterTruncNt > 0)
          throw std::runtime_error("system: images of rotors with custom trajectories or prescribed wakes");
        s->imageOf = r[src - 1].get();
        s->R.hubCoords = q.hubCoords;
        s->R.cgCoords = q.cgCoords;
        s->R.fromCoords = q.fromCoords;
        comp(s->R.hubCoords, s->R.imagePlane) = -1.0 * comp(s->R.hubCoords, s->R.imagePlane);
        comp(s->R.cgCoords, s->R.imagePlane) = -1.0 * comp(s->R.cgCoords, s->R.imagePlane);
      } else {
        s->readGeom(g);
      }
      s->init();
      r.push_back(std::move(s));
    }
    std::vector<Sim*> all;
    for (auto& s : r) all.push_back(s.get());
    for (int ir = 0; ir < nr; ++ir) {
      r[ir]->sys = all;
      r[ir]->self = ir;
    }
  }
  const Switches& sw() const { return r[0]->sw; }
  static double& comp(V3& v, int k) { return Sim::comp(v, k); }
  void start() {
    for (auto& s : r) s->startGeometry();
    for (auto& s : r) {
      if (s->imageOf) s->mirrorVelCP();
      else s->computeRHS(false);
    }
    for (auto& s : r) {
      if (s->imageOf) s->mirrorGamma();
      else s->solveRHS();
    }
    for (auto& s : r) s->startWake();
    for (auto& s : r) s->startLoads();
    for (auto& s : r) s->started = true;
  }
  void step() {
    if (!r[0]->started) throw std::runtime_error("system: start first");
    if (r[0]->iter >= r[0]->nt) throw std::runtime_error("all timesteps done");
    for (auto& s : r) s->advanceKinematics();
    for (auto& s : r) s->preWake();
    for (auto& s : r) {
      if (s->imageOf) s->mirrorVelCP();
      else s->computeRHS(true);
    }
    for (auto& s : r) {
      if (s->imageOf) s->mirrorGamma();
      else s->solveRHS();
    }
    if (sw().rotorForcePlot != 0 && r[0]->iter % sw().rotorForcePlot == 0)
      for (auto& s : r) {
        s->computeForces();
        s->force2file();
      }
    if (sw().wakeSuppress == 0)
      for (int st = 0; st < 4; ++st)
        for (auto& s : r)
          if (s->R.nNwake > 0) {
            if (s->imageOf) s->imageWakeStage(st);
            else s->wakeStage(st);
          }
  }
};

thread_local std::string g_err;

template <class F>
int guarded(F f) {
  try {
    f();
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return -1;
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// C API (ctypes)
extern "C" {

const char* or_last_error() { return g_err.c_str(); }

void* or_sim_create(const char* config_text, const char* geom_text, const char* base_dir) {
  Sim* s = nullptr;
  int rc = guarded([&]() {
    s = new Sim();
    Namelist c, g;
    c.parse(config_text);
    g.parse(geom_text);
    s->baseDir = base_dir ? base_dir : "";
    s->readConfig(c);
    s->readGeom(g);
    s->init();
  });
  if (rc != 0) { delete s; return nullptr; }
  return s;
}

void or_sim_free(void* h) { delete static_cast<Sim*>(h); }

// A system of nr coupled rotors from config.nml and geom01..geomNN.nml texts.
void* or_sys_create(int nr, const char* config_text, const char* const* geom_texts, const char* base_dir) {
  System* y = nullptr;
  int rc = guarded([&]() {
    y = new System();
    std::vector<std::string> g;
    for (int i = 0; i < nr; ++i) g.push_back(geom_texts[i]);
    y->create(nr, config_text, g, base_dir ? base_dir : "");
  });
  if (rc != 0) { delete y; return nullptr; }
  return y;
}
void or_sys_free(void* h) { delete static_cast<System*>(h); }
int or_sys_set_sum_chunk(void* h, int c) {
  return guarded([&]() { for (auto& s : static_cast<System*>(h)->r) s->sumChunk = c; });
}
int or_sys_start(void* h) { return guarded([&]() { static_cast<System*>(h)->start(); }); }
int or_sys_step(void* h, int n) {
  return guarded([&]() { for (int k = 0; k < n; ++k) static_cast<System*>(h)->step(); });
}
// Coefficient c (0 CL, 1 CD, 2 CM) of the C81 file at path, at
// (alpha degrees, Mach) (libC81.f90 getCL/getCD/getCM); NaN on error.
double or_c81_lookup(const char* path, int c, double alpha, double mach) {
  double v = std::nan("");
  guarded([&]() {
    C81 t;
    t.read(path);
    v = c == 0 ? t.getCL(alpha, mach) : (c == 1 ? t.getCD(alpha, mach) : t.getCM(alpha, mach));
  });
  return v;
}

// Rotor ir (0-based) as a Sim handle for or_get / or_geti (owned by the system).
void* or_sys_rotor(void* h, int ir) {
  System* y = static_cast<System*>(h);
  return ir >= 0 && ir < (int)y->r.size() ? y->r[ir].get() : nullptr;
}

void or_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

void or_set_sum_chunk(void* h, int c) { static_cast<Sim*>(h)->sumChunk = c; }

int or_sim_start(void* h) { return guarded([&]() { static_cast<Sim*>(h)->start(); }); }
int or_sim_step(void* h, int nsteps) {
  return guarded([&]() {
    for (int k = 0; k < nsteps; ++k) static_cast<Sim*>(h)->step();
  });
}

// unit-test primitives (mirror the calls made by tests/*_test.f90)
int or_rot_pitch(void* h, int ib, double theta) {
  return guarded([&]() { Sim* s = static_cast<Sim*>(h); s->blade_rot_pitch(s->R.blade[ib - 1], theta); });
}
double or_gettheta(void* h, double psi, int ib) { return static_cast<Sim*>(h)->gettheta(psi, ib); }
int or_set_blade_theta(void* h, int ib, double theta) { static_cast<Sim*>(h)->R.blade[ib - 1].theta = theta; return 0; }
int or_calc_aic(void* h) { return guarded([&]() { static_cast<Sim*>(h)->calcAIC(); }); }
// velCP = -velBody [- Omega*shaft x (CP-hub)], velCPm = velCPTotal = velCP,
// RHS = -velCP.nCap, gamVec = AIC_inv*RHS, gamVecPrev = 0, map_gam
int or_test_freestream(void* h, int withOmega) {
  return guarded([&]() {
    Sim* s = static_cast<Sim*>(h);
    Rotor& r = s->R;
    for (int ib = 0; ib < r.nbConvect; ++ib)
      for (int is = 0; is < r.ns; ++is)
        for (int ic = 0; ic < r.nc; ++ic) {
          WingPanel& p = r.blade[ib].w(ic, is);
          V3 v = -1.0 * r.velBody;
          if (withOmega) v = v - cross(r.Omega * r.shaftAxis, p.CP - r.hubCoords);
          p.velCP = v; p.velCPm = v; p.velCPTotal = v;
          r.RHS[ic + r.nc * is + r.nc * r.ns * ib] = dot(v, p.nCap);
        }
    for (auto& x : r.RHS) x = -1.0 * x;
    Sim::matvec(r.AIC_inv, r.RHS, r.gamVec, r.n());
    std::fill(r.gamVecPrev.begin(), r.gamVecPrev.end(), 0.0);
    s->map_gam();
  });
}
int or_dir_lift_drag(void* h) { return guarded([&]() { static_cast<Sim*>(h)->rotor_dirLiftDrag(); }); }
int or_calc_sec_alpha(void* h) { return guarded([&]() { static_cast<Sim*>(h)->rotor_calc_secAlpha(); }); }
int or_calc_force(void* h) { return guarded([&]() { static_cast<Sim*>(h)->rotor_calc_force(); }); }

// One iteration in two halves: up to its loads, then the wake update.
int or_sim_step_open(void* h) { return guarded([&]() { static_cast<Sim*>(h)->stepOpen(); }); }
int or_sim_step_close(void* h) { return guarded([&]() { static_cast<Sim*>(h)->stepClose(); }); }

// Kinematics-only advance to iteration k (see Sim::skipTo).
int or_sim_skip_to(void* h, int k) { return guarded([&]() { static_cast<Sim*>(h)->skipTo(k); }); }

// Sets a named flow-state array (the layouts of or_get; n values).  With
// or_sim_skip_to this restores a state taken from elsewhere at iteration k:
//   gam, gamPrev (blade)              [ic + nc*is]  wing circulation, previous trapezoidal circulation
//   gamVec                            n
//   waN (blade)                       [i + NW*j][filament][fc1, fc2]
//   waN_gam, waN_age (blade)          [i + NW*j] (the age goes to all four filaments)
//   waN_rvc (blade)                   [i + NW*j][filament]
//   waF (blade)                       [i][fc1, fc2]
//   waF_gam, waF_rvc, waF_rvc0, waF_l0, waF_lc, waF_age (blade)   [i]
//   velN, velN1, velN2, velN3 (blade) [i + NW*j][xyz] (j to ns)
//   velF, velF1, velF2, velF3 (blade) [i][xyz]
int or_set(void* h, const char* name, int ib, const double* in, long n) {
  return guarded([&]() {
    Sim* s = static_cast<Sim*>(h);
    Rotor& r = s->R;
    const std::string k = name;
    auto need = [&](size_t m) {
      if ((size_t)n != m) throw std::runtime_error("or_set " + k + ": expected " + std::to_string(m) + " values");
    };
    auto v3 = [&](size_t i) { return mk(in[3 * i], in[3 * i + 1], in[3 * i + 2]); };
    if (k == "gamVec") {
      need(r.gamVec.size());
      for (size_t i = 0; i < r.gamVec.size(); ++i) r.gamVec[i] = in[i];
      return;
    }
    if (ib < 1 || ib > (int)r.blade.size()) throw std::runtime_error("or_set: blade out of range");
    Blade& b = r.blade[ib - 1];
    auto vel = [&](std::vector<V3>& a) { need(3 * a.size()); for (size_t i = 0; i < a.size(); ++i) a[i] = v3(i); };
    if (k == "gam") { need(b.wiP.size()); for (size_t i = 0; i < b.wiP.size(); ++i) b.wiP[i].vr.gam = in[i]; }
    else if (k == "gamPrev") { need(b.wiP.size()); for (size_t i = 0; i < b.wiP.size(); ++i) b.wiP[i].gamPrev = in[i]; }
    else if (k == "waN") {
      need(b.waN.size() * 24);
      for (size_t i = 0; i < b.waN.size(); ++i)
        for (int f = 0; f < 4; ++f) {
          b.waN[i].vf[f].fc1 = v3(8 * i + 2 * f);
          b.waN[i].vf[f].fc2 = v3(8 * i + 2 * f + 1);
        }
    } else if (k == "waN_gam") { need(b.waN.size()); for (size_t i = 0; i < b.waN.size(); ++i) b.waN[i].gam = in[i]; }
    else if (k == "waN_age") {
      need(b.waN.size());
      for (size_t i = 0; i < b.waN.size(); ++i) for (int f = 0; f < 4; ++f) b.waN[i].vf[f].age = in[i];
    } else if (k == "waN_rvc") {
      need(b.waN.size() * 4);
      for (size_t i = 0; i < b.waN.size(); ++i) for (int f = 0; f < 4; ++f) b.waN[i].vf[f].rVc = in[4 * i + f];
    } else if (k == "waF") {
      need(b.waF.size() * 6);
      for (size_t i = 0; i < b.waF.size(); ++i) { b.waF[i].vf.fc1 = v3(2 * i); b.waF[i].vf.fc2 = v3(2 * i + 1); }
    } else if (k == "waF_gam") { need(b.waF.size()); for (size_t i = 0; i < b.waF.size(); ++i) b.waF[i].gam = in[i]; }
    else if (k == "waF_rvc") { need(b.waF.size()); for (size_t i = 0; i < b.waF.size(); ++i) b.waF[i].vf.rVc = in[i]; }
    else if (k == "waF_rvc0") { need(b.waF.size()); for (size_t i = 0; i < b.waF.size(); ++i) b.waF[i].vf.rVc0 = in[i]; }
    else if (k == "waF_l0") { need(b.waF.size()); for (size_t i = 0; i < b.waF.size(); ++i) b.waF[i].vf.l0 = in[i]; }
    else if (k == "waF_lc") { need(b.waF.size()); for (size_t i = 0; i < b.waF.size(); ++i) b.waF[i].vf.lc = in[i]; }
    else if (k == "waF_age") { need(b.waF.size()); for (size_t i = 0; i < b.waF.size(); ++i) b.waF[i].vf.age = in[i]; }
    else if (k == "velN") vel(b.velN);
    else if (k == "velN1") vel(b.velN1);
    else if (k == "velN2") vel(b.velN2);
    else if (k == "velN3") vel(b.velN3);
    else if (k == "velF") vel(b.velF);
    else if (k == "velF1") vel(b.velF1);
    else if (k == "velF2") vel(b.velF2);
    else if (k == "velF3") vel(b.velF3);
    else throw std::runtime_error("or_set: unknown array " + k);
  });
}

// Integer state: name in {nt, nb, nc, ns, n, nNwake, nFwake, rowNear, rowFar, iter, nbConvect, ctRows,
// wakeTruncateNt, rollupStart, rollupEnd, wakeSuppress}
long or_geti(void* h, const char* name) {
  Sim* s = static_cast<Sim*>(h);
  std::string k = name;
  const Rotor& r = s->R;
  if (k == "nt") return s->nt;
  if (k == "nb") return r.nb;
  if (k == "nc") return r.nc;
  if (k == "ns") return r.ns;
  if (k == "n") return r.n();
  if (k == "nNwake") return r.nNwake;
  if (k == "nFwake") return r.nFwake;
  if (k == "rowNear") return r.rowNear;
  if (k == "rowFar") return r.rowFar;
  if (k == "iter") return s->iter;
  if (k == "nbConvect") return r.nbConvect;
  if (k == "ctRows") return (long)s->ctHist.size();
  if (k == "wakeTruncateNt") return r.wakeTruncateNt;
  if (k == "rollupStart") return r.rollupStart;
  if (k == "rollupEnd") return r.rollupEnd;
  if (k == "wakeSuppress") return s->sw.wakeSuppress;
  return -1;
}

// Copy a named array into out (capacity cap doubles); returns the element
// count (or -1 for an unknown name).  ib is the 1-based blade for per-blade
// arrays.  Layouts:
//   dt, nonDimDenom, psi            scalar
//   AIC, AIC_inv                    n x n column major
//   gamVec, RHS                     n
//   ct_hist                         rows x 10 (iter, CL/CT, CD, CLu, CDi, CD0, CDu, CFx, CFy, CFz)
//   PC                              [ic + nc*is][corner 0..3][xyz]
//   vr                              [ic + nc*is][filament 0..3][fc1 xyz, fc2 xyz]
//   CP, nCap, velCP, velCPTotal, normalForce     [ic + nc*is][xyz]
//   delP, gam                       [ic + nc*is]
//   secLiftDir, secDragDir, secLift, secForceInertial, secLiftInPlane,
//   secLiftOutPlane, secChordwiseResVel, secCP   [is][xyz]
//   secCL, secTheta, secAlpha, secArea, secChord, forceDist   [is] (forceDist: [is][16])
//   forceInertial, lift, yAxis      xyz (blade); hub: xyz (rotor)
//   rotorLift, rotorForceInertial   xyz (rotor)
//   waN                             [i + NW*j][filament][fc1, fc2] (all rows)
//   waN_gam, waN_rvc                [i + NW*j], [i + NW*j][filament]
//   waF                             [i][fc1, fc2]; waF_gam, waF_rvc  [i]
//   waNP, waFP                      the predicted wake of the last predictor, as waN, waF
//   velN                            [i + NW*j][xyz] (j to ns), velF [i][xyz]
long or_get(void* h, const char* name, int ib, double* out, long cap) {
  Sim* s = static_cast<Sim*>(h);
  Rotor& r = s->R;
  std::vector<double> v;
  std::string k = name;
  auto push3 = [&v](V3 a) { v.push_back(a.x); v.push_back(a.y); v.push_back(a.z); };
  Blade* b = (ib >= 1 && ib <= (int)r.blade.size()) ? &r.blade[ib - 1] : nullptr;
  if (k == "dt") v = {s->dt};
  else if (k == "nonDimDenom") v = {r.nonDimforceDenominator};
  else if (k == "psi") v = {r.psi};
  else if (k == "AIC") v = r.AIC;
  else if (k == "AIC_inv") v = r.AIC_inv;
  else if (k == "gamVec") v = r.gamVec;
  else if (k == "RHS") v = r.RHS;
  else if (k == "ct_hist") { for (auto& row : s->ctHist) v.insert(v.end(), row.begin(), row.end()); }
  else if (k == "rotorLift") push3(r.lift);
  else if (k == "rotorForceInertial") push3(r.forceInertial);
  else if (k == "hub") push3(r.hubCoords);
  else if (b) {
    if (k == "PC") { for (auto& p : b->wiP) for (int c = 0; c < 4; ++c) push3(p.PC[c]); }
    else if (k == "vr") { for (auto& p : b->wiP) for (int f = 0; f < 4; ++f) { push3(p.vr.vf[f].fc1); push3(p.vr.vf[f].fc2); } }
    else if (k == "vr_rvc") { for (auto& p : b->wiP) for (int f = 0; f < 4; ++f) v.push_back(p.vr.vf[f].rVc); }
    else if (k == "CP") { for (auto& p : b->wiP) push3(p.CP); }
    else if (k == "nCap") { for (auto& p : b->wiP) push3(p.nCap); }
    else if (k == "velCP") { for (auto& p : b->wiP) push3(p.velCP); }
    else if (k == "velCPTotal") { for (auto& p : b->wiP) push3(p.velCPTotal); }
    else if (k == "normalForce") { for (auto& p : b->wiP) push3(p.normalForce); }
    else if (k == "delP") { for (auto& p : b->wiP) v.push_back(p.delP); }
    else if (k == "gam") { for (auto& p : b->wiP) v.push_back(p.vr.gam); }
    else if (k == "secLiftDir") { for (auto& a : b->secLiftDir) push3(a); }
    else if (k == "secDragDir") { for (auto& a : b->secDragDir) push3(a); }
    else if (k == "secLift") { for (auto& a : b->secLift) push3(a); }
    else if (k == "secForceInertial") { for (auto& a : b->secForceInertial) push3(a); }
    else if (k == "secLiftInPlane") { for (auto& a : b->secLiftInPlane) push3(a); }
    else if (k == "secLiftOutPlane") { for (auto& a : b->secLiftOutPlane) push3(a); }
    else if (k == "secChordwiseResVel") { for (auto& a : b->secChordwiseResVel) push3(a); }
    else if (k == "secCP") { for (auto& a : b->secCP) push3(a); }
    else if (k == "yAxis") push3(b->yAxis);
    else if (k == "secCL") v = b->secCL;
    else if (k == "secTheta") v = b->secTheta;
    else if (k == "secAlpha") v = b->secAlpha;
    else if (k == "secArea") v = b->secArea;
    else if (k == "secChord") v = b->secChord;
    else if (k == "forceInertial") push3(b->forceInertial);
    else if (k == "lift") push3(b->lift);
    else if (k == "forceDist") {
      for (int is = 0; is < r.ns; ++is) {
        v.push_back(dot(b->secCP[is] - r.hubCoords, b->yAxis));
        v.push_back(b->secCL[is]); v.push_back(b->secCD[is]); v.push_back(b->secCLu[is]);
        v.push_back(norm2(b->secLift[is])); v.push_back(norm2(b->secDrag[is]));
        v.push_back(norm2(b->secLiftInPlane[is])); v.push_back(norm2(b->secLiftOutPlane[is]));
        v.push_back(b->secArea[is]); v.push_back(norm2(b->secChordwiseResVel[is])); v.push_back(b->secChord[is]);
        v.push_back(b->secTheta[is] * RAD2DEG); v.push_back(b->secAlpha[is] * RAD2DEG); v.push_back(b->secPhi[is] * RAD2DEG);
        v.push_back(b->secViz[is]); v.push_back(b->secVix[is]);
      }
    }
    else if (k == "waN") { for (auto& w : b->waN) for (int f = 0; f < 4; ++f) { push3(w.vf[f].fc1); push3(w.vf[f].fc2); } }
    else if (k == "waN_gam") { for (auto& w : b->waN) v.push_back(w.gam); }
    else if (k == "waN_rvc") { for (auto& w : b->waN) for (int f = 0; f < 4; ++f) v.push_back(w.vf[f].rVc); }
    else if (k == "waF") { for (auto& f : b->waF) { push3(f.vf.fc1); push3(f.vf.fc2); } }
    // the predicted wake of the last predictor (the layouts of waN, waF)
    else if (k == "waNP") { for (auto& w : b->waNP) for (int f = 0; f < 4; ++f) { push3(w.vf[f].fc1); push3(w.vf[f].fc2); } }
    else if (k == "waFP") { for (auto& f : b->waFP) { push3(f.vf.fc1); push3(f.vf.fc2); } }
    else if (k == "waF_gam") { for (auto& f : b->waF) v.push_back(f.gam); }
    else if (k == "waF_rvc") { for (auto& f : b->waF) v.push_back(f.vf.rVc); }
    else if (k == "velN") { for (auto& a : b->velN) push3(a); }
    else if (k == "velF") { for (auto& a : b->velF) push3(a); }
    else if (k == "velN1") { for (auto& a : b->velN1) push3(a); }
    else if (k == "velN2") { for (auto& a : b->velN2) push3(a); }
    else if (k == "velN3") { for (auto& a : b->velN3) push3(a); }
    else if (k == "velF1") { for (auto& a : b->velF1) push3(a); }
    else if (k == "velF2") { for (auto& a : b->velF2) push3(a); }
    else if (k == "velF3") { for (auto& a : b->velF3) push3(a); }
    else if (k == "gamPrev") { for (auto& p : b->wiP) v.push_back(p.gamPrev); }
    else if (k == "waP") { for (auto& f : b->wapF.waF) { push3(f.vf.fc1); push3(f.vf.fc2); } }
    else if (k == "waP_gam") v = {b->wapF.waF[0].gam};
    else if (k == "waP_rvc") v = {b->wapF.waF[0].vf.rVc};
    else if (k == "waN_age") { for (auto& w : b->waN) v.push_back(w.vf[0].age); }
    else if (k == "waF_rvc0") { for (auto& f : b->waF) v.push_back(f.vf.rVc0); }
    else if (k == "waF_l0") { for (auto& f : b->waF) v.push_back(f.vf.l0); }
    else if (k == "waF_lc") { for (auto& f : b->waF) v.push_back(f.vf.lc); }
    else if (k == "waF_age") { for (auto& f : b->waF) v.push_back(f.vf.age); }
    else return -1;
  } else return -1;
  long nOut = (long)v.size();
  if (out) std::memcpy(out, v.data(), sizeof(double) * std::min<long>(nOut, cap));
  return nOut;
}

// Induced velocity of every target P (3 x M, xyz contiguous) by the current
// wing + wake of the rotor (vind_bywing + vind_bywake), i.e. the quantity
// libCommon.f90:114-211 evaluates per wake node.
int or_sim_vind_points(void* h, const double* P, long M, double* V, int pred) {
  return guarded([&]() {
    Sim* s = static_cast<Sim*>(h);
#pragma omp parallel for schedule(static)
    for (long m = 0; m < M; ++m) {
      V3 p = mk(P[3 * m], P[3 * m + 1], P[3 * m + 2]);
      V3 v = s->rotor_vind_bywing(p) + s->rotor_vind_bywake(p, pred != 0);
      V[3 * m] = v.x; V[3 * m + 1] = v.y; V[3 * m + 2] = v.z;
    }
  });
}

// Isolated ring kernel: V[m] = sum_n vr_vind(ring n, P[m]) * gam[n], rings in
// order n = 0..N-1 (blade_vind_bywing's accumulation), in chunked order when
// chunk > 0 (see ChunkSum).  corners: N x 4 x 3,
// rvc: N x 4 (core radius of filament k = corner k -> corner k+1), P and V: M x 3.
int or_vind_rings(const double* corners, const double* rvc, const double* gam, long N,
                  const double* P, long M, double* V, int chunk) {
  return guarded([&]() {
    std::vector<VR> rings(N);
    for (long n = 0; n < N; ++n) {
      V3 c[4];
      for (int k = 0; k < 4; ++k) c[k] = mk(corners[12 * n + 3 * k], corners[12 * n + 3 * k + 1], corners[12 * n + 3 * k + 2]);
      for (int k = 0; k < 4; ++k) {
        rings[n].vf[k].fc1 = c[k];
        rings[n].vf[k].fc2 = c[(k + 1) % 4];
        rings[n].vf[k].rVc = rvc[4 * n + k];
      }
      rings[n].gam = gam[n];
    }
#pragma omp parallel for schedule(static)
    for (long m = 0; m < M; ++m) {
      V3 p = mk(P[3 * m], P[3 * m + 1], P[3 * m + 2]);
      ChunkSum s(chunk);
      for (long n = 0; n < N; ++n) s.add(vr_vind(rings[n], p) * rings[n].gam);
      V3 r = V3() + s.result();
      V[3 * m] = r.x; V[3 * m + 1] = r.y; V[3 * m + 2] = r.z;
    }
  });
}

// Isolated filaments: V[m] = sum_n vf_vind(filament n, P[m]) * gam[n] in
// order (chunked when chunk > 0), no |gam| skip (src/gridgen.f90:128-136).
// fc: N x 2 x 3, rvc and gam: N.
int or_vind_filaments(const double* fc, const double* rvc, const double* gam, long N, const double* P, long M,
                      double* V, int chunk) {
  return guarded([&]() {
    std::vector<VF> f(N);
    for (long n = 0; n < N; ++n) {
      f[n].fc1 = mk(fc[6 * n], fc[6 * n + 1], fc[6 * n + 2]);
      f[n].fc2 = mk(fc[6 * n + 3], fc[6 * n + 4], fc[6 * n + 5]);
      f[n].rVc = rvc[n];
    }
#pragma omp parallel for schedule(static)
    for (long m = 0; m < M; ++m) {
      V3 p = mk(P[3 * m], P[3 * m + 1], P[3 * m + 2]);
      ChunkSum s(chunk);
      for (long n = 0; n < N; ++n) s.add(vf_vind(f[n], p) * gam[n]);
      V3 r = V3() + s.result();
      V[3 * m] = r.x; V[3 * m + 1] = r.y; V[3 * m + 2] = r.z;
    }
  });
}

// Single filament (vf_vind) for kernel unit checks.
void or_vf_vind(const double* fc1, const double* fc2, double rvc, const double* P, double* V) {
  VF f;
  f.fc1 = mk(fc1[0], fc1[1], fc1[2]);
  f.fc2 = mk(fc2[0], fc2[1], fc2[2]);
  f.rVc = rvc;
  V3 v = vf_vind(f, mk(P[0], P[1], P[2]));
  V[0] = v.x; V[1] = v.y; V[2] = v.z;
}

// Explicit inverse (libMath.f90:48-83 restated) and DGEMV (libMath.f90:105-122)
int or_inv2(const double* A, int n, double* Ainv) {
  return guarded([&]() {
    std::vector<double> a(A, A + size_t(n) * n);
    auto x = Sim::inverseLU(a, n);
    std::memcpy(Ainv, x.data(), sizeof(double) * x.size());
  });
}
void or_matvec(const double* A, const double* x, int n, double* y) {
  std::vector<double> a(A, A + size_t(n) * n), xv(x, x + n), yv(n);
  Sim::matvec(a, xv, yv, n);
  std::memcpy(y, yv.data(), sizeof(double) * n);
}
double or_lsq2(double xq, const double* xd, const double* yd, int n) {
  std::vector<double> x(xd, xd + n), y(yd, yd + n);
  return lsq2(xq, x, y);
}

}  // extern "C"
