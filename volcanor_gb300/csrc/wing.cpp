// Case input parsing, lifting-surface geometry and prescribed kinematics.
// Built with -ffp-contract=off: one IEEE operation per reference operation.
#include "wing.h"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <stdexcept>

#include "vlm_solver.h"

namespace vlm {

// ---------------------------------------------------------------------------
// Namelist
static std::string lower(std::string s) {
  for (auto& c : s) c = (char)std::tolower((unsigned char)c);
  return s;
}
static double to_double(std::string s) {
  for (auto& c : s)
    if (c == 'd' || c == 'D') c = 'e';
  return std::strtod(s.c_str(), nullptr);
}

void Namelist::parse(const std::string& text) {
  // drop comments outside quotes, then split into tokens
  std::vector<std::string> tok;
  std::string cur;
  bool inq = false;
  char q = 0;
  auto flush = [&]() {
    if (!cur.empty()) {
      tok.push_back(cur);
      cur.clear();
    }
  };
  for (size_t i = 0; i < text.size(); ++i) {
    const char c = text[i];
    if (inq) {
      if (c == q) {
        inq = false;
        tok.push_back(std::string("\x01") + cur);
        cur.clear();
      } else {
        cur += c;
      }
      continue;
    }
    if (c == '!') {
      flush();
      while (i < text.size() && text[i] != '\n') ++i;
      continue;
    }
    if (c == '\'' || c == '"') {
      flush();
      inq = true;
      q = c;
      continue;
    }
    if (std::isspace((unsigned char)c) || c == ',') {
      flush();
      continue;
    }
    if (c == '=' || c == '/') {
      flush();
      tok.push_back(std::string(1, c));
      continue;
    }
    cur += c;
  }
  flush();
  std::string group, key;
  for (size_t i = 0; i < tok.size(); ++i) {
    const std::string& t = tok[i];
    if (!t.empty() && t[0] == '&') {
      group = lower(t.substr(1));
      key.clear();
      continue;
    }
    if (t == "/") {
      group.clear();
      key.clear();
      continue;
    }
    if (group.empty()) continue;
    if (i + 1 < tok.size() && tok[i + 1] == "=") {
      key = lower(t);
      kv_[group + "." + key].clear();
      ++i;
      continue;
    }
    if (key.empty()) continue;
    std::vector<std::string>& vals = kv_[group + "." + key];
    if (t[0] == '\x01') {
      vals.push_back(t.substr(1));
      continue;
    }
    std::string v = t;
    int rep = 1;
    const size_t star = v.find('*');
    if (star != std::string::npos) {
      rep = std::atoi(v.substr(0, star).c_str());
      v = v.substr(star + 1);
    }
    for (int r = 0; r < rep; ++r) vals.push_back(v);
  }
}
bool Namelist::has(const std::string& g, const std::string& k) const { return kv_.count(lower(g) + "." + lower(k)) > 0; }
double Namelist::d(const std::string& g, const std::string& k, double def, size_t idx) const {
  auto it = kv_.find(lower(g) + "." + lower(k));
  if (it == kv_.end() || it->second.size() <= idx) return def;
  return to_double(it->second[idx]);
}
int Namelist::i(const std::string& g, const std::string& k, int def) const {
  auto it = kv_.find(lower(g) + "." + lower(k));
  if (it == kv_.end() || it->second.empty()) return def;
  return (int)std::lround(to_double(it->second[0]));
}
std::string Namelist::s(const std::string& g, const std::string& k, const std::string& def, size_t idx) const {
  auto it = kv_.find(lower(g) + "." + lower(k));
  if (it == kv_.end() || it->second.size() <= idx) return def;
  return it->second[idx];
}
d3 Namelist::v3(const std::string& g, const std::string& k) const { return mk3(d(g, k, 0, 0), d(g, k, 0, 1), d(g, k, 0, 2)); }
size_t Namelist::count(const std::string& g, const std::string& k) const {
  auto it = kv_.find(lower(g) + "." + lower(k));
  return it == kv_.end() ? 0 : it->second.size();
}

// ---------------------------------------------------------------------------
// spacing helpers (src/libMath.f90:138-200)
static std::vector<double> linspace(double a, double b, int n) {
  std::vector<double> x(n);
  const double dx = (b - a) / double(n - 1);
  for (int i = 0; i < n; ++i) x[i] = double(i) * dx + a;
  return x;
}
static std::vector<double> spacing(int kind, double a, double b, int n) {
  std::vector<double> x(n);
  if (kind == 1) return linspace(a, b, n);
  if (kind == 2) {
    auto th = linspace(0.0, kPi, n);
    for (int i = 0; i < n; ++i) x[i] = a + ((b - a) * 0.5) * (1.0 - std::cos(th[i]));
    return x;
  }
  if (kind == 3) {
    auto th = linspace(0.0, kPi * 0.5, n);
    for (int i = 0; i < n; ++i) x[i] = a + (b - a) * std::sin(th[i]);
    return x;
  }
  if (kind == 4) {
    const double tl = 1.2;
    auto th = linspace(-tl, tl, n);
    for (int i = 0; i < n; ++i) x[i] = a + ((b - a) * std::tan(th[i])) / std::tan(tl);
    return x;
  }
  throw std::runtime_error("spacing switch must be 1..4");
}

// src/libMath.f90:476-517
static double pwl_interp1d(const std::vector<double>& x, const std::vector<double>& y, double q) {
  const size_t n = x.size();
  if (std::fabs(x[0] - q) < kEps) return y[0];
  if (std::fabs(x[n - 1] - q) < kEps) return y[n - 1];
  std::vector<int> t(n);
  if (x[0] < x[n - 1]) {
    for (size_t i = 0; i < n; ++i) t[i] = x[i] <= q;
  } else if (x[0] > x[n - 1]) {
    for (size_t i = 0; i < n; ++i) t[i] = x[i] >= q;
  } else {
    throw std::runtime_error("pwl_interp1d: neither ascending nor descending");
  }
  size_t idx = n;
  for (size_t i = 0; i < n; ++i)
    if (!t[i]) {
      idx = i;
      break;
    }
  if (idx == 0 || idx == n) throw std::runtime_error("pwl_interp1d: out of range");
  idx -= 1;
  return y[idx] + (y[idx + 1] - y[idx]) / (x[idx + 1] - x[idx]) * (q - x[idx]);
}

// ---------------------------------------------------------------------------
void Panel::shift(d3 d) {
  CP = CP + d;
  for (int k = 0; k < 4; ++k) {
    PC[k] = PC[k] + d;
    C[k] = C[k] + d;
  }
}
void Panel::rot(const m33& T, d3 o) {
  for (int k = 0; k < 4; ++k) PC[k] = rot_about(T, PC[k], o);
  for (int k = 0; k < 4; ++k) C[k] = rot_about(T, C[k], o);
  CP = rot_about(T, CP, o);
  nCap = mul33(T, nCap);
  tauC = mul33(T, tauC);
  tauS = mul33(T, tauS);
}

void Wing::load(const std::string& configText, const std::string& geomText, const std::string& base) {
  baseDir = base;
  Namelist c, g;
  c.parse(configText);
  g.parse(geomText);
  readConfig(c);
  readGeom(g);
  init();
}

void Wing::loadMember(const std::string& configText, const std::string& geomText, const std::string& base,
                      const Wing* prev) {
  baseDir = base;
  member = true;
  Namelist c, g;
  c.parse(configText);
  g.parse(geomText);
  readConfig(c);
  if (prev) {
    dt = prev->dt;
    nt = prev->nt;
    sw = prev->sw;
  }
  readGeom(g);
  init();
}

void Wing::loadImage(const std::string& configText, const std::string& imageGeomText,
                     const std::string& sourceGeomText, const std::string& base, const Wing* prev, const Wing* src) {
  baseDir = base;
  member = true;
  imageOf = src;
  Namelist c, gi, gs;
  c.parse(configText);
  gi.parse(imageGeomText);
  gs.parse(sourceGeomText);
  readConfig(c);
  if (prev) {
    dt = prev->dt;
    nt = prev->nt;
    sw = prev->sw;
  }
  readGeom(gs);
  RotorParams& r = P;
  r.surfaceType = gi.i("SURFACE", "surfaceType");
  r.imagePlane = gi.i("SURFACE", "imagePlane");
  r.imageRotorNum = gi.i("SURFACE", "imageRotorNum");
  r.geometryFile = gi.s("PANELS", "geometryFile", "0");
  if (r.surfaceType != -1) throw std::runtime_error("unsupported: image of a non-lifting surface");
  if (r.imagePlane < 1 || r.imagePlane > 3) throw std::runtime_error("imagePlane must be 1, 2 or 3");
  if (src->P.customTrajectorySwitch != 0 || src->P.prescWakeNt > 0 || src->P.forceCalcSwitch != 0)
    throw std::runtime_error("unsupported: an image of a rotor with a custom trajectory, a prescribed wake or airfoil "
                             "tables");
  auto mir = [&](d3 v) {
    (r.imagePlane == 1 ? v.x : (r.imagePlane == 2 ? v.y : v.z)) *= -1.0;
    return v;
  };
  r.hubCoords = mir(src->initHub);
  r.cgCoords = mir(src->initCg);
  r.fromCoords = src->P.fromCoords;
  init();
}

// src/libCommon.f90:51-108
void Wing::readConfig(const Namelist& c) {
  const std::string ver = c.s("VERSION", "fileFormatVersion", "");
  if (!ver.empty() && std::fabs(to_double(ver) - 0.5) > 1e-12) throw std::runtime_error("config.nml template version does not match");
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
  if (nr != 1 && !member) throw std::runtime_error("nr > 1: coupled rotors are created with vlm_system_create");
  if (member && (sw.ntSub != 0 || sw.ntSubInit != 0))
    throw std::runtime_error("unsupported: sub-iterations (ntSub, ntSubInit) of coupled rotors");
  if (sw.restartFromNt != 0) throw std::runtime_error("unsupported: restartFromNt (use the case checkpoint API)");
  if (sw.fdScheme < 0 || sw.fdScheme > 5) throw std::runtime_error("fdScheme must be 0..5");
}

// src/classdef.f90:2541-2767
void Wing::readGeom(const Namelist& g) {
  const std::string ver = g.s("VERSION", "fileFormatVersion", "");
  if (!ver.empty() && std::fabs(to_double(ver) - 0.15) > 1e-12) throw std::runtime_error("geomXX.nml template version does not match");
  RotorParams& r = P;
  r.surfaceType = g.i("SURFACE", "surfaceType");
  r.imagePlane = g.i("SURFACE", "imagePlane");
  r.imageRotorNum = g.i("SURFACE", "imageRotorNum");
  r.thetaTwist = g.d("GEOMPARAMS", "thetaTwist");
  r.nAirfoils = g.i("GEOMPARAMS", "nAirfoils");
  r.alpha0 = r.nAirfoils > 0 ? g.d("AIRFOILS", "alpha0") : 0.0;
  r.Iflap = g.d("DYNAMICS", "Iflap");
  r.cflap = g.d("DYNAMICS", "cflap");
  r.kflap = g.d("DYNAMICS", "kflap");
  r.MflapConstant = g.d("DYNAMICS", "MflapConstant");
  r.nb = g.i("PANELS", "nb", 1);
  r.propConvention = g.i("PANELS", "propConvention");
  r.spanSpacing = g.i("PANELS", "spanSpacing", 1);
  r.chordSpacing = g.i("PANELS", "chordSpacing", 1);
  r.geometryFile = g.s("PANELS", "geometryFile", "0");
  r.nCamberFiles = g.i("PANELS", "nCamberFiles");
  r.nc = g.i("PANELS", "nc", 1);
  r.ns = g.i("PANELS", "ns", 1);
  r.nNwake = g.i("PANELS", "nNwake");
  r.hubCoords = g.v3("ORIENT", "hubCoords");
  r.cgCoords = g.v3("ORIENT", "cgCoords");
  r.fromCoords = g.v3("ORIENT", "fromCoords");
  r.pts = g.v3("ORIENT", "phiThetaPsi");
  r.radius = g.d("GEOMPARAMS", "span");
  r.root_cut = g.d("GEOMPARAMS", "rootcut");
  r.chord = g.d("GEOMPARAMS", "chord");
  r.preconeAngle = g.d("GEOMPARAMS", "preconeAngle");
  r.Omega = g.d("GEOMPARAMS", "Omega");
  r.shaftAxis = g.v3("GEOMPARAMS", "shaftAxis");
  r.controlPitch = mk3(g.d("GEOMPARAMS", "theta0"), g.d("GEOMPARAMS", "thetaC"), g.d("GEOMPARAMS", "thetaS"));
  r.ductSwitch = g.i("GEOMPARAMS", "ductSwitch");
  r.axisymmetrySwitch = g.i("GEOMPARAMS", "axisymmetrySwitch");
  r.pivotLE = g.d("GEOMPARAMS", "pivotLE");
  r.flapHinge = g.d("GEOMPARAMS", "flapHinge");
  r.spanwiseLiftSwitch = g.i("GEOMPARAMS", "spanwiseLiftSwitch");
  r.symmetricTau = g.i("GEOMPARAMS", "symmetricTau");
  r.customTrajectorySwitch = g.i("GEOMPARAMS", "customTrajectorySwitch");
  r.velBody = g.v3("GEOMPARAMS", "velBody");
  r.velBodyInput = r.velBody;
  r.omegaBody = g.v3("GEOMPARAMS", "omegaBody");
  r.forceCalcSwitch = g.i("GEOMPARAMS", "forceCalcSwitch");
  r.apparentViscCoeff = g.d("WAKEPARAMS", "apparentViscCoeff");
  r.decayCoeff = g.d("WAKEPARAMS", "decayCoeff");
  r.wakeTruncateNt = g.i("WAKEPARAMS", "wakeTruncateNt");
  r.prescWakeAfterTruncNt = g.i("WAKEPARAMS", "prescWakeAfterTruncNt");
  r.prescWakeGenNt = g.i("WAKEPARAMS", "prescWakeGenNt");
  r.spanwiseCore = g.d("WAKEPARAMS", "spanwiseCore");
  std::vector<double> sc(r.ns + 1, 0.0);
  const size_t cnt = g.count("WAKEPARAMS", "streamwiseCoreVec");
  for (size_t k = 0; k < std::min(cnt, sc.size()); ++k) sc[k] = g.d("WAKEPARAMS", "streamwiseCoreVec", 0, k);
  double tail = 0.0;
  for (size_t k = 1; k < sc.size(); ++k) tail = tail + sc[k] * sc[k];
  if (std::sqrt(tail) < kEps) std::fill(sc.begin(), sc.end(), sc[0]);  // classdef.f90:2720-2724
  r.streamwiseCoreVec = sc;
  r.rollupStartRadius = g.d("WAKEPARAMS", "rollupStartRadius");
  r.rollupEndRadius = g.d("WAKEPARAMS", "rollupEndRadius");
  r.initWakeVel = g.d("WAKEPARAMS", "initWakeVel");
  r.psiStart = g.d("WAKEPARAMS", "psiStart");
  r.skewLimit = g.d("WAKEPARAMS", "skewLimit");
  r.bladeDynamicsSwitch = g.i("DYNAMICS", "bladeDynamicsSwitch");
  r.flapInitial = g.d("DYNAMICS", "flapInitial");
  r.dflapInitial = g.d("DYNAMICS", "dflapInitial");
  r.pitchDynamicsSwitch = g.i("DYNAMICS", "pitchDynamicsSwitch");
  r.dpitch = g.d("DYNAMICS", "dpitch");
  r.bodyDynamicsSwitch = g.i("DYNAMICS", "bodyDynamicsSwitch");
  r.inflowPlotSwitch = g.i("PLOTS", "inflowPlotSwitch");
  r.gammaPlotSwitch = g.i("PLOTS", "gammaPlotSwitch");
  r.skewPlotSwitch = g.i("PLOTS", "skewPlotSwitch");
  if (r.surfaceType < 0 || std::abs(r.surfaceType) == 2) throw std::runtime_error("unsupported: image or non-lifting surfaces");
  for (int k = 0; k < r.nCamberFiles; ++k) {
    r.camberSectionLimit.push_back(g.d("CAMBERSECTIONS", "camberSectionLimit", 1.0, k));
    r.camberFile.push_back(g.s("CAMBERSECTIONS", "camberFile", "0", k));
  }
  if (r.ductSwitch != 0) throw std::runtime_error("unsupported: ductSwitch");
  if (r.forceCalcSwitch < 0 || r.forceCalcSwitch > 1)
    throw std::runtime_error("unsupported: forceCalcSwitch 2 (alpha from the sectional circulation)");
  if (r.forceCalcSwitch > 0 && r.nAirfoils == 0) throw std::runtime_error("No. of airfoil tables set to 0 in geomXX.in");
  for (int a = 0; a < r.nAirfoils; ++a) {
    r.airfoilSectionLimit.push_back(g.d("AIRFOILS", "airfoilSectionLimit", 1.0, a));
    r.airfoilFile.push_back(g.s("AIRFOILS", "airfoilFile", "0", a));
  }
  if (r.forceCalcSwitch == 1 && r.axisymmetrySwitch == 1)
    throw std::runtime_error("unsupported: forceCalcSwitch 1 with axisymmetrySwitch 1");
  if (r.bladeDynamicsSwitch != 0 || r.bodyDynamicsSwitch != 0)
    throw std::runtime_error("unsupported: blade/body dynamics");
  if (r.customTrajectorySwitch != 0 && r.customTrajectorySwitch != 1)
    throw std::runtime_error("customTrajectorySwitch must be 0 or 1");
  if (r.nc < 1 || r.ns < 1 || r.nb < 1) throw std::runtime_error("nb, nc and ns must be positive");
}

// libMath interp1d with order 2 (src/libMath.f90:520-575): Lagrange
// interpolation through the two or three table points around xq (x
// ascending, xq within the table).
static double interp1d2(double xq, const std::vector<double>& x, const std::vector<double>& y) {
  const int n = (int)x.size();
  int ix = -1;
  for (int i = 0; i < n; ++i)
    if (xq <= x[i]) {
      ix = i;
      break;
    }
  if (ix < 0) throw std::runtime_error("camber interpolation beyond the table");
  if (std::fabs(xq - x[ix]) <= kEps) return y[ix];
  if (ix == 0) throw std::runtime_error("camber interpolation before the table");
  if (std::sqrt(y[ix - 1] * y[ix - 1] + y[ix] * y[ix]) <= kEps) return 0.0;
  if (n == 2) return y[ix - 1] + (xq - x[ix - 1]) * (y[ix] - y[ix - 1]) / (x[ix] - x[ix - 1]);
  const int a = ix == 1 ? 0 : ix - 2, b = a + 1, c = a + 2;
  const double L0 = (xq - x[b]) * (xq - x[c]) / ((x[a] - x[b]) * (x[a] - x[c]));
  const double L1 = (xq - x[a]) * (xq - x[c]) / ((x[b] - x[a]) * (x[b] - x[c]));
  const double L2 = (xq - x[a]) * (xq - x[b]) / ((x[c] - x[a]) * (x[c] - x[b]));
  return y[a] * L0 + y[b] * L1 + y[c] * L2;
}

// rotor_getCamber (src/classdef.f90:4060-4112): z of the chordwise points x
// at the spanwise stations y from the camber files (a point count, then x z
// pairs, normalised by the last x; '0' = no camber), each station using the
// first section whose limit is >= y/span.  Returns [i + nx j].
std::vector<double> Wing::getCamber(const std::vector<double>& x, const std::vector<double>& y) const {
  const int nx = (int)x.size(), ny = (int)y.size(), nf = P.nCamberFiles;
  const double chord = x[nx - 1] - x[0];
  const double span = y[ny - 1] - y[0];
  std::vector<std::vector<double>> xc(nf), zc(nf);
  for (int j = 0; j < nf; ++j) {
    if (P.camberFile[j].empty() || P.camberFile[j][0] == '0') {
      xc[j] = {0.0, 1.0};
      zc[j] = {0.0, 0.0};
      continue;
    }
    std::string path = P.camberFile[j];
    if (path[0] != '/' && !baseDir.empty()) path = baseDir + "/" + path;
    std::ifstream f(path);
    if (!f) throw std::runtime_error("cannot open camber file " + path);
    std::stringstream ss;
    ss << f.rdbuf();
    std::string t = ss.str();
    for (char& c : t) {
      if (c == ',') c = ' ';
      else if (c == 'd' || c == 'D') c = 'e';
    }
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
      if (y[j] / span <= P.camberSectionLimit[k]) {
        fNum = k;
        break;
      }
    if (fNum < 0) throw std::runtime_error("camberSectionLimit does not cover the first station");
    for (int i = 0; i < nx; ++i) out[(size_t)i + (size_t)nx * j] = chord * interp1d2((x[i] - x[0]) / chord, xc[fNum], zc[fNum]);
  }
  return out;
}

// trajectory01.in (src/classdef.f90:3065-3081): nt list-directed records of
// u v w p q r (body velocity and rates); a record's values may run over
// lines, extra values on its last line are skipped.
void Wing::readTrajectory() {
  std::string path = "trajectory01.in";
  if (!baseDir.empty()) path = baseDir + "/" + path;
  std::ifstream f(path);
  if (!f) throw std::runtime_error("cannot open " + path);
  P.velBodyHistory.assign(nt, zero3());
  P.omegaBodyHistory.assign(nt, zero3());
  std::string line;
  for (int i = 0; i < nt; ++i) {
    double v[6];
    int got = 0;
    while (got < 6) {
      if (!std::getline(f, line)) throw std::runtime_error(path + ": fewer than nt records");
      for (char& c : line) {
        if (c == ',') c = ' ';
        else if (c == 'd' || c == 'D') c = 'e';
      }
      std::istringstream ls(line);
      double x;
      while (got < 6 && ls >> x) v[got++] = x;
    }
    P.velBodyHistory[i] = mk3(v[0], v[1], v[2]);
    P.omegaBodyHistory[i] = mk3(v[3], v[4], v[5]);
  }
}

// src/classdef.f90:5133-5148
void Wing::toChordsRevs(int& n) const {
  if (n < 0) {
    if (std::fabs(P.Omega) < kEps) n = (int)std::ceil(double(std::abs(n)) * P.chord / (dt * norm3(P.velBody)));
    else n = (int)std::ceil(kTwoPi * double(std::abs(n)) / (std::fabs(P.Omega) * dt));
  }
}

void Wing::blade_move(Blade& b, d3 d) {
  for (auto& p : b.p) p.shift(d);
  for (auto& s : b.secCP) s = s + d;
  b.flapOrigin = b.flapOrigin + d;
}
void Wing::blade_rot_pts(Blade& b, d3 pts, d3 o) {
  const m33 T = tgb_angles(pts);
  for (int j = 0; j < b.ns; ++j) {
    for (int i = 0; i < b.nc; ++i) b.w(i, j).rot(T, o);
    b.secCP[j] = rot_about(T, b.secCP[j], o);
    b.secTauC[j] = mul33(T, b.secTauC[j]);
    b.secNormal[j] = mul33(T, b.secNormal[j]);
  }
  d3* ax[9] = {&b.xA, &b.yA, &b.zA, &b.xAzi, &b.yAzi, &b.zAzi, &b.xAF, &b.yAF, &b.zAF};
  for (auto a : ax) *a = mul33(T, *a);
}
// type: 0 azimuth, 1 flap, 2 pitch
void Wing::blade_rotate(Blade& b, double ang, d3 axis, d3 o, int type) {
  if (!(std::fabs(ang) > kEps)) return;
  blade_move(b, neg3(o));
  const m33 T = transform_axis(ang, axis);
  for (auto& p : b.p) p.rot(T, zero3());
  blade_move(b, o);
  for (int i = 0; i < b.ns; ++i) {
    b.secCP[i] = rot_about(T, b.secCP[i], o);
    b.secTauC[i] = mul33(T, b.secTauC[i]);
    b.secTauS[i] = mul33(T, b.secTauS[i]);
    b.secNormal[i] = mul33(T, b.secNormal[i]);
  }
  if (type == 0) {
    b.xAF = mul33(T, b.xAF); b.yAF = mul33(T, b.yAF); b.zAF = mul33(T, b.zAF);
    b.xAzi = mul33(T, b.xAzi); b.yAzi = mul33(T, b.yAzi); b.zAzi = mul33(T, b.zAzi);
  } else if (type == 1) {
    b.xAF = mul33(T, b.xAF); b.yAF = mul33(T, b.yAF); b.zAF = mul33(T, b.zAF);
  }
  b.xA = mul33(T, b.xA);
  b.yA = mul33(T, b.yA);
  b.zA = mul33(T, b.zA);
}
void Wing::blade_rot_pitch(Blade& b, double theta) {
  if (std::fabs(theta) > kEps) {
    const d3 o = b.w(0, 0).PC[0] * (1.0 - b.pivotLE) + b.w(b.nc - 1, 0).PC[1] * b.pivotLE;
    blade_rotate(b, theta, b.yA, o, 2);
  }
}
double Wing::gettheta(double psiv, int ib) const {
  const double off = (kTwoPi / double(P.nb)) * double(ib - 1);
  if (P.pitchDynamicsSwitch == 1) {
    double th = std::min(std::fabs(psiv / P.Omega * P.dpitch), std::fabs(P.controlPitch.x));
    if (P.controlPitch.x < 0) th = -1.0 * th;
    return th;
  }
  return (P.controlPitch.x + P.controlPitch.y * std::cos(psiv + off)) + P.controlPitch.z * std::sin(psiv + off);
}
void Wing::rot_pts(d3 pts, d3 o) {
  const m33 T = tgb_angles(pts);
  for (auto& b : bl) blade_rot_pts(b, pts, o);
  shaftAxis = mul33(T, shaftAxis);
  xBody = mul33(T, xBody);
  yBody = mul33(T, yBody);
  zBody = mul33(T, zBody);
  hub = rot_about(T, hub, o);
  cg = rot_about(T, cg, o);
}
void Wing::rot_advance(double dpsi, bool nopitch) {
  psi = psi + dpsi;
  for (int ib = 0; ib < P.nb; ++ib) {
    Blade& b = bl[ib];
    blade_rotate(b, dpsi, shaftAxis, hub, 0);
    b.psi = b.psi + dpsi;
    if (!nopitch) {
      const double th = gettheta(psi, ib + 1);
      blade_rot_pitch(b, th - b.theta);
      b.theta = th;
    }
  }
}
// src/classdef.f90:2267-2304
void Wing::calc_secLocations(Blade& b, double frac, double hingeR) {
  for (int is = 0; is < b.ns; ++is) {
    const d3 vecLE = 0.5 * (b.w(0, is).PC[0] + b.w(0, is).PC[3]);
    std::vector<double> xc(b.nc + 1, 0.0), zc(b.nc + 1, 0.0);
    d3 vecPC = zero3();
    for (int ic = 0; ic < b.nc; ++ic) {
      vecPC = 0.5 * (b.w(ic, is).PC[1] + b.w(ic, is).PC[2]) - vecLE;
      xc[ic + 1] = norm3(proj3(vecPC, b.secTauC[is]));
      zc[ic + 1] = dot3(vecPC, b.secNormal[is]);
    }
    const double x = norm3(vecPC) * frac;
    const double z = pwl_interp1d(xc, zc, x);
    b.secCP[is] = (vecLE + x * b.secTauC[is]) + z * b.secNormal[is];
    b.secMflapArm[is] = norm3(proj3(b.secCP[is], b.yA)) - hingeR;
  }
}

// src/classdef.f90:2769-3891 for lifting surfaces
void Wing::init() {
  RotorParams& r = P;
  if (dt < 0 || std::signbit(dt)) {
    if (std::fabs(r.Omega) < kEps) dt = std::fabs(dt) * r.chord / norm3(r.velBody);
    else dt = kTwoPi * std::fabs(dt) / std::fabs(r.Omega);
  }
  if (std::fabs(dt) <= kEps) {
    if (std::fabs(r.Omega) < kEps) dt = (r.chord / double(r.nc)) / norm3(r.velBody);
    else dt = 5.0 * kDeg2Rad / std::fabs(r.Omega);
  }
  if (nt <= 0) {
    if (nt == 0) nt = -10;
    toChordsRevs(nt);
  }
  if (sw.slowStart != 0) toChordsRevs(sw.slowStartNt);
  toChordsRevs(sw.wakeTipPlot);
  toChordsRevs(sw.wakePlot);
  toChordsRevs(sw.gridPlot);
  toChordsRevs(r.wakeTruncateNt);
  toChordsRevs(r.prescWakeAfterTruncNt);
  toChordsRevs(r.prescWakeGenNt);
  toChordsRevs(r.nNwake);
  toChordsRevs(r.inflowPlotSwitch);
  toChordsRevs(r.gammaPlotSwitch);
  toChordsRevs(r.skewPlotSwitch);
  r.prescWakeNt = (r.wakeTruncateNt > 0 && r.prescWakeAfterTruncNt > 0) ? r.wakeTruncateNt + r.prescWakeAfterTruncNt : 0;
  if (r.wakeTruncateNt > 0) r.wakeTruncateNt = std::max(r.wakeTruncateNt, r.nNwake + 1);
  if (r.surfaceType == 0) r.surfaceType = 1;
  if (r.nNwake > 0 && r.nNwake < 2) throw std::runtime_error("at least 2 near wake rows are required");
  xBody = mk3(1, 0, 0);
  yBody = mk3(0, 1, 0);
  zBody = mk3(0, 0, 1);
  r.nNwake = std::min(r.nNwake, nt);
  if (r.customTrajectorySwitch == 1) readTrajectory();
  nFwake = r.wakeTruncateNt == 0 ? nt - r.nNwake : r.wakeTruncateNt - r.nNwake;
  if (r.nNwake == 0) nFwake = 0;
  nbConvect = r.axisymmetrySwitch == 1 ? 1 : r.nb;
  const int nc = r.nc, ns = r.ns;
  bl.assign(r.nb, Blade());
  for (auto& b : bl) {
    b.nc = nc;
    b.ns = ns;
    b.p.assign((size_t)nc * ns, Panel());
    b.secTauC.assign(ns, zero3());
    b.secTauS = b.secNormal = b.secCP = b.secTauC;
    b.secArea.assign(ns, 0.0);
    b.secChord = b.secMflapArm = b.secArea;
  }
  r.controlPitch = r.controlPitch * kDeg2Rad;
  r.pts = r.pts * kDeg2Rad;
  r.preconeAngle = r.preconeAngle * kDeg2Rad;
  r.psiStart = r.psiStart * kDeg2Rad;
  r.thetaTwist = r.thetaTwist * kDeg2Rad;  // read, converted and printed, never applied to the geometry
  r.spanwiseCore = r.spanwiseCore * r.chord;
  for (auto& s : r.streamwiseCoreVec) s = s * r.chord;
  rollupStart = (int)std::ceil(r.rollupStartRadius * double(ns));
  rollupEnd = (int)std::floor(r.rollupEndRadius * double(ns));
  hub = r.hubCoords;
  cg = r.cgCoords;
  shaftAxis = r.shaftAxis;
  // panel corners
  if (r.geometryFile.empty() || r.geometryFile[0] == '0') {
    const double cs = r.Omega >= 0 ? -r.chord : r.chord;
    const auto xv = spacing(r.chordSpacing, cs, 0.0, nc + 1);
    const auto yv = spacing(r.spanSpacing, r.root_cut * r.radius, r.radius, ns + 1);
    std::vector<double> zv((size_t)(nc + 1) * (ns + 1), 0.0);  // [i + (nc+1) j]
    if (r.nCamberFiles > 0) zv = getCamber(xv, yv);
    if (imageOf && r.imagePlane == 3)
      for (auto& v : zv) v = -1.0 * v;
    auto z = [&](int i, int j) { return zv[(size_t)i + (size_t)(nc + 1) * j]; };
    for (auto& b : bl)
      for (int j = 0; j < ns; ++j)
        for (int i = 0; i < nc; ++i) {
          Panel& p = b.w(i, j);
          p.PC[0] = mk3(xv[i], yv[j], z(i, j));
          p.PC[1] = mk3(xv[i + 1], yv[j], z(i + 1, j));
          p.PC[2] = mk3(xv[i + 1], yv[j + 1], z(i + 1, j + 1));
          p.PC[3] = mk3(xv[i], yv[j + 1], z(i, j + 1));
        }
  } else {
    // src/classdef.f90:3957-4020 (PLOT3D, nx = nc+1, ny = ns+1, nz = 1)
    std::string path = r.geometryFile;
    if (path[0] != '/' && !baseDir.empty()) path = baseDir + "/" + path;
    std::ifstream f(path);
    if (!f) throw std::runtime_error("cannot open PLOT3D file " + path);
    int nx, ny, nz;
    f >> nx >> ny >> nz;
    if (nz > 1 || nx != nc + 1 || ny != ns + 1) throw std::runtime_error("wrong or conflicting data in PLOT3D file");
    std::vector<d3> grid((size_t)nx * ny);
    for (int c = 0; c < 3; ++c)
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
          double v;
          if (!(f >> v)) throw std::runtime_error("PLOT3D file too short");
          d3& q = grid[i + (size_t)nx * j];
          (c == 0 ? q.x : (c == 1 ? q.y : q.z)) = v;
        }
    if (imageOf && r.imagePlane == 3)
      for (auto& q : grid) q.z = -1.0 * q.z;
    for (int ib = 0; ib < nbConvect; ++ib)
      for (int is = 0; is < ns; ++is)
        for (int ic = 0; ic < nc; ++ic) {
          Panel& p = bl[ib].w(ic, is);
          p.PC[0] = grid[ic + (size_t)nx * is];
          p.PC[1] = grid[ic + 1 + (size_t)nx * is];
          p.PC[2] = grid[ic + 1 + (size_t)nx * (is + 1)];
          p.PC[3] = grid[ic + (size_t)nx * (is + 1)];
        }
    if (r.axisymmetrySwitch == 1)
      for (int ib = 1; ib < r.nb; ++ib)
        for (size_t k = 0; k < bl[ib].p.size(); ++k)
          for (int c = 0; c < 4; ++c) bl[ib].p[k].PC[c] = bl[0].p[k].PC[c];
  }
  const d3 X = mk3(1, 0, 0), Y = mk3(0, 1, 0), Z = mk3(0, 0, 1);
  for (int ib = 0; ib < nbConvect; ++ib) {
    Blade& b = bl[ib];
    b.xA = X; b.yA = Y; b.zA = Z;
    b.xAzi = X; b.yAzi = Y; b.zAzi = Z;
    b.xAF = X; b.yAF = Y; b.zAF = Z;
    b.flapOrigin = (b.yA * r.radius) * r.flapHinge;
    for (int j = 0; j < ns; ++j) {
      b.secTauC[j] = ((b.w(nc - 1, j).PC[2] + b.w(nc - 1, j).PC[1]) - (b.w(0, j).PC[3] + b.w(0, j).PC[0])) * 0.5;
      b.secTauS[j] = Y;
      b.secNormal[j] = cross3(b.w(nc - 1, j).PC[1] - b.w(0, j).PC[3], b.w(nc - 1, j).PC[2] - b.w(0, j).PC[0]);
      b.secTauC[j] = unit3(b.secTauC[j]);
      b.secNormal[j] = fsign1(r.Omega) * unit3(b.secNormal[j]);
    }
    // vortex-ring corners: quarter-chord shift, last row separately (classdef.f90:3311-3367)
    for (int j = 0; j < ns; ++j)
      for (int i = 0; i < nc; ++i) {
        Panel& p = b.w(i, j);
        double xs[4];
        if (i < nc - 1) {
          const Panel& q = b.w(i + 1, j);
          xs[0] = (p.PC[1].x - p.PC[0].x) * 0.25;
          xs[1] = (q.PC[1].x - p.PC[1].x) * 0.25;
          xs[2] = (q.PC[2].x - p.PC[2].x) * 0.25;
          xs[3] = (p.PC[2].x - p.PC[3].x) * 0.25;
        } else {
          xs[0] = (p.PC[1].x - p.PC[0].x) * 0.25;
          xs[1] = 0.0;
          xs[2] = 0.0;
          xs[3] = (p.PC[2].x - p.PC[3].x) * 0.25;
        }
        for (int c = 0; c < 4; ++c) p.C[c] = mk3(p.PC[c].x + xs[c], p.PC[c].y, p.PC[c].z);
      }
    double dxmin = 1e300, dymin = 1e300;
    for (const auto& p : b.p) {
      dxmin = std::min(dxmin, std::fabs(norm3(p.PC[1] - p.PC[0])));
      dymin = std::min(dymin, std::fabs(norm3(p.PC[2] - p.PC[1])));
    }
    const double dxdymin = std::min(dxmin, dymin);
    // shed offset of the trailing-edge row; 0.05 is a single precision literal
    double velShed;
    if (std::fabs(r.Omega) > kEps)
      velShed = std::min((double(0.05f) * std::fabs(r.Omega)) * norm3(b.w(nc - 1, ns - 1).C[1] - hub), 0.125 * r.chord / dt);
    else
      velShed = 0.3 * norm3(-1.0 * r.velBody);
    const d3 sh = mk3((fsign1(r.Omega) * velShed) * dt, 0.0, 0.0);
    for (int j = 0; j < ns; ++j) {
      b.w(nc - 1, j).C[1] = b.w(nc - 1, j).C[1] + sh;
      b.w(nc - 1, j).C[2] = b.w(nc - 1, j).C[2] + sh;
    }
    for (int j = 0; j < ns; ++j)
      for (int i = 0; i < nc; ++i) {
        Panel& p = b.w(i, j);
        p.CP = ((p.PC[0] + p.PC[3]) * 0.25 + (p.PC[1] + p.PC[2]) * 0.75) * 0.5;
        p.nCap = unit3(cross3(p.PC[2] - p.PC[0], p.PC[3] - p.PC[1]));
        if (fsign1(r.Omega) < 0.0) p.nCap = -1.0 * p.nCap;
        p.tauC = unit3(((p.PC[1] + p.PC[2]) - (p.PC[0] + p.PC[3])) * 0.5);
        p.tauS = unit3(((p.PC[2] + p.PC[3]) - (p.PC[1] + p.PC[0])) * 0.5);
        p.area = 0.5 * norm3(cross3(p.PC[2] - p.PC[0], p.PC[3] - p.PC[1]));
        p.meanSpan = 0.5 * (norm3(p.PC[3] - p.PC[0]) + norm3(p.PC[2] - p.PC[1]));
        p.meanChord = 0.5 * (norm3(p.PC[1] - p.PC[0]) + norm3(p.PC[2] - p.PC[3]));
      }
    if (imageOf)
      for (size_t k = 0; k < b.p.size(); ++k) {
        d3 n = imageOf->initNCap[ib][k];
        (r.imagePlane == 1 ? n.x : (r.imagePlane == 2 ? n.y : n.z)) *= -1.0;
        b.p[k].nCap = n;
      }
    for (int is = 0; is < ns; ++is) {
      double s = 0.0;
      for (int ic = 0; ic < nc; ++ic) s = s + b.w(ic, is).area;
      b.secArea[is] = s;
      b.secChord[is] = norm3(0.5 * ((b.w(0, is).PC[0] + b.w(0, is).PC[3]) - (b.w(nc - 1, is).PC[1] + b.w(nc - 1, is).PC[2])));
    }
    for (int j = 0; j < ns; ++j) {
      b.secTauS[j] = b.yA;
      for (int i = 0; i < nc; ++i) b.w(i, j).tauS = b.yA;
    }
    if (r.symmetricTau == 1)
      for (int j = 0; j < ns / 2; ++j) {
        b.secTauS[j] = -1.0 * b.secTauS[j];
        for (int i = 0; i < nc; ++i) b.w(i, j).tauS = -1.0 * b.w(i, j).tauS;
      }
    calc_secLocations(b, 0.5, r.flapHinge * r.radius);
    b.pivotLE = r.pivotLE;
    const double rw = std::min(r.spanwiseCore, dxdymin * 0.1);
    for (auto& p : b.p)
      for (int k = 0; k < 4; ++k) p.rvc[k] = rw;
    for (int j = 0; j < ns; ++j) b.w(nc - 1, j).rvc[1] = r.spanwiseCore;
  }
  if (r.axisymmetrySwitch == 1) {
    const Blade& b0 = bl[0];
    for (int ib = 1; ib < r.nb; ++ib) {
      Blade& b = bl[ib];
      b.xA = b0.xA; b.yA = b0.yA; b.zA = b0.zA;
      b.xAzi = b0.xAzi; b.yAzi = b0.yAzi; b.zAzi = b0.zAzi;
      b.xAF = b0.xAF; b.yAF = b0.yAF; b.zAF = b0.zAF;
      b.flapOrigin = b0.flapOrigin;
      b.secTauC = b0.secTauC; b.secTauS = b0.secTauS; b.secNormal = b0.secNormal;
      for (size_t k = 0; k < b.p.size(); ++k) {
        Panel& p = b.p[k];
        const Panel& q = b0.p[k];
        for (int c = 0; c < 4; ++c) p.C[c] = q.C[c];
        for (int c = 0; c < 4; ++c) p.rvc[c] = q.rvc[c];
        p.CP = q.CP; p.nCap = q.nCap; p.tauC = q.tauC; p.tauS = q.tauS;
        p.area = q.area; p.meanChord = q.meanChord; p.meanSpan = q.meanSpan;
      }
      b.secArea = b0.secArea; b.secChord = b0.secChord;
      b.secCP = b0.secCP; b.secMflapArm = b0.secMflapArm; b.pivotLE = b0.pivotLE;
    }
  }
  for (auto& b : bl) blade_move(b, hub - r.fromCoords);
  for (auto& b : bl) {
    b.dflap = r.dflapInitial;
    b.flap = r.flapInitial;
    blade_rotate(b, r.preconeAngle, b.xAzi, b.flapOrigin, 1);
    blade_rotate(b, r.flapInitial, b.xAzi, b.flapOrigin, 1);
  }
  for (int ib = 1; ib < r.nb; ++ib) {
    const double off = ((fsign1(r.Omega) * kTwoPi) / double(r.nb)) * double(ib);
    blade_rotate(bl[ib], off, shaftAxis, hub, 0);
  }
  rot_pts(r.pts, cg);
  rot_advance(fsign1(r.Omega) * r.psiStart, true);
  if (std::fabs(r.Omega) > kEps) {
    if (r.propConvention == 0) {
      const double ro = r.radius * r.Omega;
      nonDimDenom = (density * (kPi * (r.radius * r.radius))) * (ro * ro);
    } else {
      const double f = r.Omega / kTwoPi;
      nonDimDenom = (density * (f * f)) * pow4(2.0 * r.radius);
    }
  } else {
    nonDimDenom = ((0.5 * density) * ((r.radius * (1.0 - r.root_cut)) * r.chord)) * dot3(r.velBody, r.velBody);
  }
  omegaSlow = sw.slowStart > 0 ? 0.0 : r.Omega;
  initHub = hub;
  initCg = cg;
  initNCap.assign(r.nb, {});
  for (int ib = 0; ib < r.nb; ++ib)
    for (const Panel& q : bl[ib].p) initNCap[ib].push_back(q.nCap);
  // airfoil tables and the table of every section (classdef.f90:3693-3725):
  // the first table whose r/R limit reaches the section's CP, r/R measured
  // along the blade's x axis from the root section's point at half chord
  if (r.forceCalcSwitch == 1) {
    for (const std::string& f : r.airfoilFile) {
      if (f.empty() || f[0] == '0') throw std::runtime_error("forceCalcSwitch 1 needs every airfoilFile");
      airfoils.add_c81(f[0] == '/' || baseDir.empty() ? f : baseDir + "/" + f);
    }
    airfoilOfSection.assign((size_t)r.nb * r.ns, 0);
    for (int ib = 0; ib < r.nb; ++ib) {
      const Blade& b = bl[ib];
      if (r.nAirfoils == 1) continue;
      const d3 root = b.w(0, 0).PC[3] * 0.5 + b.w(r.nc - 1, 0).PC[2] * 0.5;
      for (int is = 0; is < r.ns; ++is) {
        const double rr = std::fabs(dot3(b.secCP[is] - root, b.xA)) + r.root_cut;
        if (rr > 1.0) throw std::runtime_error("r/R value is greater than 1 in airfoil selection");
        int a = 0;
        while (a < r.nAirfoils && !(r.airfoilSectionLimit[a] >= rr)) ++a;
        airfoilOfSection[(size_t)ib * r.ns + is] = a < r.nAirfoils ? a : 0;
      }
    }
  }
}

// A C81 file into the flat table (the layout of AirfoilTables).
void AirfoilTables::add_c81(const std::string& path) {
  std::ifstream in(path);
  if (!in) throw std::runtime_error("cannot open " + path);
  std::vector<std::string> lines;
  for (std::string t; std::getline(in, t);) {
    if (!t.empty() && t.back() == '\r') t.pop_back();
    lines.push_back(t);
  }
  auto column = [](const std::string& t, size_t at, size_t width) {
    const std::string f = at < t.size() ? t.substr(at, width) : std::string();
    const size_t b = f.find_first_not_of(' ');
    return b == std::string::npos ? 0.0 : std::strtod(f.c_str() + b, nullptr);
  };
  size_t ln = 0;
  auto line = [&]() -> const std::string& {
    if (ln >= lines.size()) throw std::runtime_error("C81 file too short: " + path);
    return lines[ln++];
  };
  const std::string head = line();
  int cnt[6];
  for (int k = 0; k < 6; ++k) cnt[k] = (int)column(head, 30 + 2 * (size_t)k, 2);
  offset.push_back((int)data.size());
  for (int k = 0; k < 6; ++k) data.push_back(cnt[k]);
  for (int c = 0; c < 3; ++c) {
    const int nm = cnt[2 * c], na = cnt[2 * c + 1];
    if (nm < 1 || nm > 18 || na < 1) throw std::runtime_error("C81 table sizes out of range: " + path);
    std::vector<double> mach(nm), alpha(na), val((size_t)na * nm);
    // a row of values: up to 9 after `skip` columns, the rest on a second line
    auto values = [&](const std::string& first, double* out, size_t stride) {
      for (int j = 0; j < nm; ++j) {
        if (j == 9) {
          const std::string& more = line();
          for (int jj = 9; jj < nm; ++jj) out[(size_t)jj * stride] = column(more, 7 + 7 * (size_t)(jj - 9), 7);
          break;
        }
        out[(size_t)j * stride] = column(first, 7 + 7 * (size_t)j, 7);
      }
    };
    values(line(), mach.data(), 1);
    for (int i = 0; i < na; ++i) {
      const std::string& row = line();
      alpha[i] = column(row, 0, 7);
      values(row, val.data() + i, (size_t)na);
    }
    data.insert(data.end(), mach.begin(), mach.end());
    data.insert(data.end(), alpha.begin(), alpha.end());
    data.insert(data.end(), val.begin(), val.end());
  }
}

void Wing::start_pitch() {
  for (int ib = 0; ib < P.nb; ++ib) {
    Blade& b = bl[ib];
    if (imageOf) {
      // src/main.f90:45-50: the source's initial pitch, negated in the z plane
      b.theta = imageOf->gettheta(imageOf->P.psiStart, ib + 1);
      if (P.imagePlane == 3) b.theta = -1.0 * b.theta;
    } else {
      b.theta = gettheta(P.psiStart, ib + 1);
    }
    blade_rot_pitch(b, fsign1(P.Omega) * b.theta);
  }
  if (P.customTrajectorySwitch == 1) {  // src/main.f90:111-116, before the initial solve
    P.velBody = P.velBodyHistory[0];
    P.omegaBody = P.omegaBodyHistory[0];
  }
}

// src/main.f90:412-463
void Wing::advance(int iter) {
  if (P.customTrajectorySwitch == 1) {  // src/main.f90:419-424
    P.velBody = P.velBodyHistory[iter - 1];
    P.omegaBody = P.omegaBodyHistory[iter - 1];
  }
  switch (sw.slowStart) {
    case 0: omegaSlow = P.Omega; break;
    case 1: omegaSlow = double(std::min(float(sw.slowStartNt), float(iter + 1))) * P.Omega / double(sw.slowStartNt); break;
    case 2: omegaSlow = std::tanh(5.0 * double(iter) / double(sw.slowStartNt)) * P.Omega; break;
    case 3:
      omegaSlow = ((std::tanh(6.0 * double(float(iter)) / double(float(sw.slowStartNt)) - 3.0) + 1.0) * 0.5) * P.Omega;
      break;
    default: break;
  }
  const d3 d = P.velBody * dt;
  for (auto& b : bl) blade_move(b, d);
  hub = hub + d;
  cg = cg + d;
  rot_pts(P.omegaBody * dt, cg);
  rot_advance(omegaSlow * dt, false);
}

void Wing::write_frame(double* out) const {
  const int nb = P.nb, nc = P.nc, ns = P.ns, npan = nc * ns;
  const FrameLayout fl = frame_layout(nb, nc, ns);
  auto put = [](double* o, d3 v) {
    o[0] = v.x;
    o[1] = v.y;
    o[2] = v.z;
  };
  for (int b = 0; b < nb; ++b) {
    const Blade& B = bl[b];
    for (int is = 0; is < ns; ++is)
      for (int ic = 0; ic < nc; ++ic) {
        const int p = ic + nc * is;
        const Panel& q = B.p[p];
        double* o = out + fl.pan + ((size_t)b * npan + p) * kPan;
        for (int k = 0; k < 4; ++k) put(o + 3 * k, q.C[k]);
        put(o + 12, q.CP);
        put(o + 15, q.nCap);
        put(o + 18, q.tauC);
        put(o + 21, q.tauS);
        // src/main.f90:530-538
        d3 v = -1.0 * P.velBody;
        v = v - cross3(P.omegaBody, q.CP - cg);
        v = v - cross3(omegaSlow * shaftAxis, q.CP - hub);
        const double fa = B.secMflapArm[is] * B.dflap;
        v = mk3(v.x - fa, v.y - fa, v.z - fa);
        put(o + 24, v);
      }
    for (int is = 0; is < ns; ++is) {
      double* o = out + fl.sec + ((size_t)b * ns + is) * kSec;
      put(o, B.secTauC[is]);
      put(o + 3, B.secNormal[is]);
      put(o + 6, B.secCP[is]);
      put(o + 9, B.w(0, is).PC[0]);
    }
    put(out + fl.ax + 9 * b, B.xAF);
    put(out + fl.ax + 9 * b + 3, B.yAF);
    put(out + fl.ax + 9 * b + 6, B.zAF);
  }
  double* r = out + fl.rot;
  put(r, zBody);
  put(r + 3, hub);
  put(r + 6, shaftAxis);
  r[9] = omegaSlow;
  for (int b = 1; b < nb; ++b) {
    const m33 T = transform_axis((kTwoPi / double(nb)) * double(b), shaftAxis);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) r[10 + 9 * (b - 1) + 3 * i + j] = T.a[i][j];
  }
}

namespace {

// List-directed output as the reference's golden rXXParams.json files show
// it: integers right-justified in 12 columns; reals in 24 columns, as
// F-form with 15 significant digits followed by 5 blanks when
// 0.1 <= |x| < 1e15, else (and for zero) as d.ddddddddddddddd with a signed
// three-digit exponent.  A blank separates a number from a following
// character item.
std::string ld_int(long v) {
  char b[32];
  std::snprintf(b, sizeof b, "%12ld", v);
  return b;
}

std::string ld_real(double x) {
  char b[64];
  if (x != 0.0 && std::isfinite(x)) {
    std::snprintf(b, sizeof b, "%.14e", std::fabs(x));  // rounded to 15 significant digits
    const int e10 = std::atoi(std::strchr(b, 'e') + 1);
    if (e10 >= -1 && e10 <= 14) {
      char f[48];
      std::snprintf(f, sizeof f, "%.*f", 14 - e10, x);
      std::snprintf(b, sizeof b, "%19s     ", f);
      return b;
    }
  }
  if (!std::isfinite(x)) {
    std::snprintf(b, sizeof b, "%24s", std::isnan(x) ? "NaN" : (x > 0 ? "Infinity" : "-Infinity"));
    return b;
  }
  char m[48];
  int e10 = 0;
  if (x != 0.0) {
    std::snprintf(m, sizeof m, "%.15e", x);
    char* e = std::strchr(m, 'e');
    e10 = std::atoi(e + 1);
    *e = 0;
  } else {
    std::snprintf(m, sizeof m, "%.15f", 0.0);
  }
  char t[64];
  std::snprintf(t, sizeof t, "%sE%c%03d", m, e10 < 0 ? '-' : '+', std::abs(e10));
  std::snprintf(b, sizeof b, "%24s", t);
  return b;
}

}  // namespace

// params2file (src/libPostprocess.f90:52-141): the case's parameters after
// rotor_init, in the reference's key order; step counts given in chords or
// revolutions are the converted ones, angles are printed in degrees except
// phiThetaPsi (radians, as the reference prints rotor%pts).
std::string Wing::params_json() const {
  const RotorParams& r = P;
  std::string o = " {\n";
  auto ki = [&](const char* k, long v, bool last = false) {
    o += std::string(" \"") + k + "\": " + ld_int(v) + (last ? "" : " ,") + "\n";
  };
  auto kr = [&](const char* k, double v, bool last = false) {
    o += std::string(" \"") + k + "\": " + ld_real(v) + (last ? "" : " ,") + "\n";
  };
  ki("nt", nt);
  kr("dt", dt);
  ki("nr", nr);
  ki("restartWriteNt", sw.restartWriteNt);
  ki("restartFromNt", sw.restartFromNt);
  ki("ntSub", sw.ntSub);
  ki("ntSubInit", sw.ntSubInit);
  kr("density", density);
  kr("velSound", velSound);
  ki("wakePlot", sw.wakePlot);
  ki("wakeTipPlot", sw.wakeTipPlot);
  ki("rotorForcePlot", sw.rotorForcePlot);
  ki("gridPlot", sw.gridPlot);
  ki("wakeDissipation", sw.wakeDissipation);
  ki("wakeStrain", sw.wakeStrain);
  ki("wakeBurst", sw.wakeBurst);
  ki("slowStart", sw.slowStart);
  ki("slowStartNt", sw.slowStartNt);
  ki("fdScheme", sw.fdScheme);
  ki("initWakeVelNt", sw.initWakeVelNt);
  ki("probe", sw.probe);
  ki("nb", r.nb);
  ki("propConvention", r.propConvention);
  std::string gf = r.geometryFile.substr(0, 30);  // character(len=30)
  gf.resize(30, ' ');
  o += " \"geometryFile\": \"" + gf + "\",\n";
  ki("spanSpacing", r.spanSpacing);
  ki("chordSpacing", r.chordSpacing);
  ki("nCamberFiles", r.nCamberFiles);
  ki("surfaceType", r.surfaceType);
  ki("imagePlane", r.imagePlane);
  ki("imageRotorNum", r.imageRotorNum);
  ki("nc", r.nc);
  ki("ns", r.ns);
  ki("nNwake", r.nNwake);
  kr("radius", r.radius);
  kr("root_cut", r.root_cut);
  kr("chord", r.chord);
  kr("preconeAngle", r.preconeAngle * kRad2Deg);
  kr("Omega", r.Omega);
  kr("phi", r.pts.x);
  kr("theta", r.pts.y);
  kr("psi", r.pts.z);
  kr("theta0", r.controlPitch.x * kRad2Deg);
  kr("thetaC", r.controlPitch.y * kRad2Deg);
  kr("thetaS", r.controlPitch.z * kRad2Deg);
  kr("thetaTwist", r.thetaTwist * kRad2Deg);
  kr("u", r.velBodyInput.x);  // params2file runs before any trajectory step
  kr("v", r.velBodyInput.y);
  kr("w", r.velBodyInput.z);
  kr("nonDimForceDenom", nonDimDenom);
  kr("alpha0", r.nAirfoils > 0 ? r.alpha0 : 0.0);
  ki("wakeTruncateNt", r.wakeTruncateNt);
  ki("prescWakeNt", r.prescWakeNt);
  kr("initWakeVel", r.initWakeVel);
  kr("psiStart", r.psiStart * kRad2Deg);
  kr("forceCalcSwitch", double(r.forceCalcSwitch) * kRad2Deg);
  kr("apparentViscCoeff", r.apparentViscCoeff);
  kr("decayCoeff", r.decayCoeff);
  ki("axisymmetrySwitch", r.axisymmetrySwitch);
  ki("bladeDynamicsSwitch", r.bladeDynamicsSwitch);
  kr("flapInitial", r.flapInitial);
  kr("dFlapInitial", r.dflapInitial);
  kr("Iflap", r.Iflap);
  kr("cflap", r.cflap);
  kr("kflap", r.kflap);
  kr("MflapConstant", r.MflapConstant);
  ki("pitchDynamicsSwitch", r.pitchDynamicsSwitch);
  kr("dpitch", r.dpitch, true);
  o += " }\n";
  return o;
}

}  // namespace vlm
