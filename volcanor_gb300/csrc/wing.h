// Host-side case description and lifting-surface kinematics.
//
// The wing geometry and its prescribed motion are computed on the host in
// FP64 (compiled with -ffp-contract=off and the host libm), in the same
// operation order as the reference (src/classdef.f90 rotor_init, blade_move,
// blade_rot_pts, blade_rotate, rotor_rot_advance), and uploaded to the GPU as
// one frame per timestep.  Nothing here depends on the flow solution, so all
// frames of a run are produced before the first step.
#pragma once

#include <map>
#include <string>
#include <vector>

#include "vlm_math.h"

namespace vlm {

// Fortran namelist subset used by config.nml / geomXX.nml.
class Namelist {
 public:
  void parse(const std::string& text);
  bool has(const std::string& group, const std::string& key) const;
  double d(const std::string& group, const std::string& key, double def = 0.0, size_t idx = 0) const;
  int i(const std::string& group, const std::string& key, int def = 0) const;
  std::string s(const std::string& group, const std::string& key, const std::string& def = "0", size_t idx = 0) const;
  d3 v3(const std::string& group, const std::string& key) const;
  size_t count(const std::string& group, const std::string& key) const;

 private:
  std::map<std::string, std::vector<std::string>> kv_;
};

struct Switches {  // src/classdef.f90:16-55
  int ntSub = 0, ntSubInit = 0, wakeDissipation = 0, wakeStrain = 0, wakeBurst = 0, wakeSuppress = 0;
  int slowStart = 0, slowStartNt = 0, wakeTipPlot = 0, wakePlot = 0, gridPlot = 0, rotorForcePlot = 1;
  int fdScheme = 0, probe = 0, initWakeVelNt = 0, restartFromNt = 0, restartWriteNt = 0;
};

struct RotorParams {  // rotor_readGeom inputs (src/classdef.f90:2541-2767)
  int surfaceType = 0, nb = 1, propConvention = 0, spanSpacing = 1, chordSpacing = 1, nCamberFiles = 0;
  int nc = 1, ns = 1, nNwake = 0;
  std::string geometryFile = "0";
  d3 hubCoords{0, 0, 0}, cgCoords{0, 0, 0}, fromCoords{0, 0, 0}, pts{0, 0, 0};
  double radius = 0, root_cut = 0, chord = 0, preconeAngle = 0, Omega = 0;
  d3 shaftAxis{0, 0, 0}, velBody{0, 0, 0}, omegaBody{0, 0, 0}, controlPitch{0, 0, 0};
  int ductSwitch = 0, axisymmetrySwitch = 0, spanwiseLiftSwitch = 0, symmetricTau = 0;
  int customTrajectorySwitch = 0, forceCalcSwitch = 0;
  double pivotLE = 0, flapHinge = 0, apparentViscCoeff = 0, decayCoeff = 0, spanwiseCore = 0;
  int wakeTruncateNt = 0, prescWakeAfterTruncNt = 0, prescWakeGenNt = 0, prescWakeNt = 0;
  double skewLimit = 0.0;  // wake burst: the turn (in units of pi) between far filaments that bursts them
  std::vector<double> streamwiseCoreVec;
  double rollupStartRadius = 0, rollupEndRadius = 0, initWakeVel = 0, psiStart = 0;
  int bladeDynamicsSwitch = 0, pitchDynamicsSwitch = 0, bodyDynamicsSwitch = 0;
  double flapInitial = 0, dflapInitial = 0, dpitch = 0;
  int inflowPlotSwitch = 0, gammaPlotSwitch = 0, skewPlotSwitch = 0;
  // customTrajectorySwitch = 1: body velocity and rates of every step from
  // trajectory01.in (velBodyHistory / omegaBodyHistory,
  // src/classdef.f90:3065-3081); velBodyInput is the namelist value
  std::vector<d3> velBodyHistory, omegaBodyHistory;
  d3 velBodyInput{0, 0, 0};
  // camber sections (CAMBERSECTIONS namelist, src/classdef.f90:2614-2687)
  std::vector<double> camberSectionLimit;
  std::vector<std::string> camberFile;
  // forceCalcSwitch 1: one airfoil table per entry of the AIRFOILS namelist
  // (classdef.f90:2605, 2754-2765), sections up to airfoilSectionLimit (r/R)
  std::vector<double> airfoilSectionLimit;
  std::vector<std::string> airfoilFile;
  // read only to be echoed into rXXParams.json
  int imagePlane = 0, imageRotorNum = 0, nAirfoils = 0;
  double thetaTwist = 0, Iflap = 0, cflap = 0, kflap = 0, MflapConstant = 0, alpha0 = 0;
};

struct Panel {
  d3 PC[4];  // panel corners
  d3 C[4];   // vortex-ring corners
  d3 CP, nCap, tauC, tauS;
  double area = 0, meanChord = 0, meanSpan = 0, rvc[4] = {0, 0, 0, 0};
  void shift(d3 d);
  void rot(const m33& T, d3 o);
};

struct Blade {
  int nc = 0, ns = 0;
  std::vector<Panel> p;  // [i + nc*j]
  std::vector<d3> secTauC, secTauS, secNormal, secCP;
  std::vector<double> secArea, secChord, secMflapArm;
  d3 xA, yA, zA, xAzi, yAzi, zAzi, xAF, yAF, zAF, flapOrigin;
  double theta = 0, psi = 0, pivotLE = 0, flap = 0, dflap = 0;
  Panel& w(int i, int j) { return p[i + nc * j]; }
  const Panel& w(int i, int j) const { return p[i + nc * j]; }
};

// The airfoil tables of a rotor in one flat array of doubles, as the loads
// kernel reads them: per airfoil, at offset[a], the counts ML NL MD ND MM NM
// then for lift, drag and moment in turn the Mach numbers, the angles of
// attack (degrees) and the coefficients (angle fastest).  Read from C81
// files (fixed columns: a 30-character name and six 2-digit counts, then
// per coefficient a line of Mach numbers in 7-column fields after 7 blank
// columns, and per angle a line of the angle and the values in 7-column
// fields; more than 9 Mach numbers continue on a second line).
struct AirfoilTables {
  std::vector<double> data;
  std::vector<int> offset;
  void add_c81(const std::string& path);
};

// One case: parsed inputs, derived sizes and the moving lifting surface.
class Wing {
 public:
  // config / geometry (throws std::runtime_error on invalid or unsupported input)
  void load(const std::string& configText, const std::string& geomText, const std::string& baseDir);
  // Rotor ir of coupled rotors (nr > 1): the reference initialises its rotors
  // in turn with dt, nt and the switches intent(inout) (src/main.f90:32-39,
  // src/classdef.f90:2778-3011), so rotor ir > 0 starts from the values
  // rotor ir - 1 left (prev; null for the first rotor).
  void loadMember(const std::string& configText, const std::string& geomText, const std::string& baseDir,
                  const Wing* prev);
  // An image rotor (surfaceType -1) of rotor `src` (initialised before it):
  // the reference copies every parameter from the source except the image's
  // surfaceType, imagePlane, imageRotorNum and geometryFile, mirrors hub and
  // cg in the image plane, z-mirrors the geometry for imagePlane 3 and takes
  // the source's initial normals mirrored (src/classdef.f90:2797-2910,
  // 3228-3230, 3434-3443, 3989-3995); the source's geomXX.nml text supplies
  // the shared parameters.
  void loadImage(const std::string& configText, const std::string& imageGeomText, const std::string& sourceGeomText,
                 const std::string& baseDir, const Wing* prev, const Wing* src);
  void start_pitch();                  // src/main.f90:43-58
  void advance(int iter);              // src/main.f90:412-463 kinematics of one step
  void write_frame(double* out) const;  // see vlm_solver.h for the layout
  double gettheta(double psi, int ib) const;
  // rXXParams.json text (params2file, src/libPostprocess.f90:52-141)
  std::string params_json() const;

  int nt = 0, nr = 1;
  double dt = 0, density = 1, velSound = 330, kinematicVisc = 0;
  Switches sw;
  RotorParams P;
  int nFwake = 0, nbConvect = 1, rollupStart = 0, rollupEnd = 0;
  double nonDimDenom = 0, omegaSlow = 0, psi = 0;
  d3 hub, cg, shaftAxis, xBody, yBody, zBody;
  std::vector<Blade> bl;
  std::string baseDir;
  // forceCalcSwitch 1: the tables and each blade section's 0-based table
  // (blade-major), assigned at initialisation (classdef.f90:3693-3725)
  AirfoilTables airfoils;
  std::vector<int> airfoilOfSection;
  bool member = false;  // a rotor of coupled rotors: nr > 1 allowed
  const Wing* imageOf = nullptr;  // an image rotor: its source
  // the state at the end of initialisation that an image of this rotor copies
  d3 initHub, initCg;
  std::vector<std::vector<d3>> initNCap;  // [blade][panel]

 private:
  void readConfig(const Namelist& c);
  void readGeom(const Namelist& g);
  void init();
  void toChordsRevs(int& n) const;
  void readTrajectory();
  std::vector<double> getCamber(const std::vector<double>& x, const std::vector<double>& y) const;
  void blade_move(Blade& b, d3 d);
  void blade_rot_pts(Blade& b, d3 pts, d3 o);
  void blade_rotate(Blade& b, double ang, d3 axis, d3 o, int type);
  void blade_rot_pitch(Blade& b, double theta);
  void rot_pts(d3 pts, d3 o);
  void rot_advance(double dpsi, bool nopitch);
  void calc_secLocations(Blade& b, double frac, double hingeR);
};

}  // namespace vlm
