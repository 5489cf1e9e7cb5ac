// FP64 vector helpers shared by the host case builder and the device kernels.
//
// Every helper is one IEEE double operation per Fortran operation of the
// reference (cibinjoseph/VOLCANOR src/libMath.f90); host code is compiled with
// -ffp-contract=off and the FP64 kernels with -fmad=false, so the host
// kinematics and the device FP64 path perform exactly the same roundings.
// Sums accumulate left to right from the first term; norm2 = sqrt of that sum;
// x**4._dp is (x*x)*(x*x).
#pragma once

#include <math.h>
#include <stdint.h>

#if defined(__CUDACC__)
#define VLM_HD __host__ __device__ __forceinline__
#else
#define VLM_HD inline
#endif

namespace vlm {

constexpr double kPi = 3.14159265358979323846;        // atan(1._dp)*4._dp
constexpr double kEps = 2.220446049250313080847e-16;  // epsilon(1._dp)
constexpr double kTwoPi = 2.0 * kPi;
constexpr double kDeg2Rad = kPi / 180.0;
constexpr double kRad2Deg = 180.0 / kPi;
constexpr double kInv4Pi = 0.25 / kPi;                // src/classdef.f90:13

struct d3 {
  double x, y, z;
};

VLM_HD d3 mk3(double a, double b, double c) {
  d3 r;
  r.x = a;
  r.y = b;
  r.z = c;
  return r;
}
VLM_HD d3 zero3() { return mk3(0.0, 0.0, 0.0); }
VLM_HD d3 operator+(d3 a, d3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
VLM_HD d3 operator-(d3 a, d3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
VLM_HD d3 operator*(double s, d3 a) { return mk3(s * a.x, s * a.y, s * a.z); }
VLM_HD d3 operator*(d3 a, double s) { return mk3(a.x * s, a.y * s, a.z * s); }
VLM_HD d3 operator/(d3 a, double s) { return mk3(a.x / s, a.y / s, a.z / s); }
VLM_HD d3 neg3(d3 a) { return mk3(-a.x, -a.y, -a.z); }
VLM_HD double dot3(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
VLM_HD double sumsq3(d3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
VLM_HD double norm3(d3 a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
// libMath.f90:202-212
VLM_HD d3 cross3(d3 a, d3 b) { return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
// libMath.f90:249-262
VLM_HD d3 unit3(d3 a) {
  double n = norm3(a);
  if (n > kEps) return a / n;
  return zero3();
}
// libMath.f90:264-276
VLM_HD d3 proj3(d3 a, d3 d) {
  double ns = sumsq3(d);
  if (ns > kEps) {
    double k = dot3(a, d);
    return mk3((k * d.x) / ns, (k * d.y) / ns, (k * d.z) / ns);
  }
  return zero3();
}
// libMath.f90:278-291
VLM_HD d3 noproj3(d3 a, d3 d) {
  double ns = sumsq3(d);
  if (ns > kEps) {
    double k = dot3(a, d);
    return mk3(a.x - (k * d.x) / ns, a.y - (k * d.y) / ns, a.z - (k * d.z) / ns);
  }
  return a;
}
VLM_HD double fsign1(double b) { return signbit(b) ? -1.0 : 1.0; }  // sign(1._dp, b)
VLM_HD double pow4(double x) {
  double x2 = x * x;
  return x2 * x2;
}

// 3x3 matrix, row-major a[row][col]
struct m33 {
  double a[3][3];
};
VLM_HD d3 mul33(const m33& T, d3 v) {
  return mk3(T.a[0][0] * v.x + T.a[0][1] * v.y + T.a[0][2] * v.z, T.a[1][0] * v.x + T.a[1][1] * v.y + T.a[1][2] * v.z,
             T.a[2][0] * v.x + T.a[2][1] * v.y + T.a[2][2] * v.z);
}
VLM_HD d3 rot_about(const m33& T, d3 p, d3 o) { return mul33(T, p - o) + o; }

// ---------------------------------------------------------------------------
// Biot-Savart, FP64, reference arithmetic (src/classdef.f90:476-542).
//
// A ring is 4 corners c[0..3]; filament k runs c[k] -> c[(k+1)%4] with core
// radius rvc[k].  Corner quantities (P - c[k] and its unit vector) are the same
// values the reference recomputes for the two filaments sharing the corner, so
// computing them once per corner leaves every rounding unchanged.
struct corner64 {
  d3 r, u;
};
VLM_HD corner64 make_corner64(d3 P, d3 c) {
  corner64 k;
  k.r = P - c;
  k.u = unit3(k.r);
  return k;
}
// vf_vind with r1 = P - fc1 and r2 = P - fc2 (classdef.f90:476-503)
VLM_HD d3 vf_vind64(const corner64& a, const corner64& b, double rvc) {
  d3 r0 = a.r - b.r;
  d3 c = cross3(a.r, b.r);
  double c2 = dot3(c, c);
  if (c2 > kEps * kEps) {
    d3 du = a.u - b.u;
    double d = dot3(r0, du);
    double s = rvc * norm3(r0);
    double den = sqrt(pow4(s) + c2 * c2);
    return mk3(((c.x * kInv4Pi) * d) / den, ((c.y * kInv4Pi) * d) / den, ((c.z * kInv4Pi) * d) / den);
  }
  return zero3();
}
// vr_vind: sum(vindMat, 1) over filaments 1..4 in order (classdef.f90:527-542)
VLM_HD d3 vr_vind64(d3 P, const d3* c, const double* rvc) {
  corner64 k0 = make_corner64(P, c[0]);
  corner64 k1 = make_corner64(P, c[1]);
  corner64 k2 = make_corner64(P, c[2]);
  corner64 k3 = make_corner64(P, c[3]);
  d3 v = vf_vind64(k0, k1, rvc[0]);
  v = v + vf_vind64(k1, k2, rvc[1]);
  v = v + vf_vind64(k2, k3, rvc[2]);
  v = v + vf_vind64(k3, k0, rvc[3]);
  return v;
}
VLM_HD d3 fil_vind64(d3 P, d3 a, d3 b, double rvc) {
  corner64 ka = make_corner64(P, a);
  corner64 kb = make_corner64(P, b);
  return vf_vind64(ka, kb, rvc);
}

// libMath.f90:695-726
inline m33 transform_axis(double theta, d3 axisVec) {
  d3 ax = axisVec / norm3(axisVec);
  double ct = cos(theta), st = sin(theta), omct = 1.0 - ct;
  m33 T;
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
// libMath.f90:672-693 from angles (phi, theta, psi)
inline m33 tgb_angles(d3 p) {
  double cph = cos(p.x), sph = sin(p.x), cth = cos(p.y), sth = sin(p.y), cps = cos(p.z), sps = sin(p.z);
  m33 T;
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

}  // namespace vlm
