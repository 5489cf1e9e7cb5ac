// Device state of one rotor case and the launchers of the time-step kernels.
//
// Storage (all FP64, all blades, device memory owned by the case):
//   wing panel p of blade b        -> index b*npan + (i + nc*j)      (src/classdef.f90 wiP(i,j))
//   near-wake ring (i,j) of blade b -> index b*NW*ns + (i + NW*j)     (waN(i,j))
//   far-wake filament i of blade b  -> index b*NF + i                (waF(i))
//   node velocity (i,j), j <= ns    -> index b*NW*(ns+1) + (i + NW*j) (velNwake(:,i,j))
// A near-wake ring stores its 4 corners (12 doubles): corner k is both
// vf(k)%fc(:,1) and vf(k-1)%fc(:,2) of the reference ring, which the
// reference always assigns, shifts and rotates together.
//
// Per-step wing kinematics are computed on the host (the prescribed motion
// does not depend on the solution) and uploaded as one FRAME per timestep:
//   PAN: per blade, per panel: corners[12] CP[3] nCap[3] tauC[3] tauS[3] velKin[3]  (27)
//   SEC: per blade, per section: secTauC[3] secNormal[3] secCP[3] PC1(1,is)[3]      (12)
//   AX:  per blade: xAxisAziFlap[3] yAxisAziFlap[3] zAxisAziFlap[3]                 (9)
//   ROT: zAxisBody[3] hub[3] shaftAxis[3] omegaSlow, then for blades 2..nb the
//        3x3 wake-copy rotation (row major)                                        (10 + 9(nb-1))
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "vlm_bs.h"

namespace vlm {

constexpr int kPan = 27;
constexpr int kSec = 12;

struct FrameLayout {
  int pan, sec, ax, rot, size;
};

inline FrameLayout frame_layout(int nb, int nc, int ns) {
  FrameLayout f;
  f.pan = 0;
  f.sec = f.pan + nb * nc * ns * kPan;
  f.ax = f.sec + nb * ns * kSec;
  f.rot = f.ax + nb * 9;
  f.size = f.rot + 10 + 9 * (nb > 1 ? nb - 1 : 0);
  return f;
}

struct Dims {
  int nb, nc, ns, npan, n, NW, NF, nbC;
  int axisym;
  int spanwiseLift;
  int rollupStart, rollupEnd;  // 1-based, as the reference
  int suppressFwake;
  double omega, theta0, density, dt, nonDimDenom, dissipAdd, decay;
  // prescribed far wake (src/classdef.f90:998-1066, 5172-5217): active on
  // iterations > prescNt when prescNt > 0; fitted to far-wake filaments
  // rowStart..NF (rowStart = rowFar, or NF - prescGenNt when that is > 0)
  int prescNt, prescGenNt;
  // wake burst (src/classdef.f90:2306-2339): skew limit, large core radius
  double skewLimit, chord;
  // loads from airfoil tables (forceCalcSwitch 1) and the speed of sound
  // their Mach number uses
  int forceCalc;
  double velSound;
  FrameLayout fl;
};

// Prescribed far wake: filaments per blade (10 revolutions of 15 degrees)
constexpr int kPresc = 240;

struct DevState {
  // wing (static)
  double *wRvc, *panArea, *panMeanChord, *panMeanSpan, *secArea;
  // forceCalcSwitch 1: airfoil tables (AirfoilTables layout), their offsets,
  // the table of every blade section
  double* c81;
  int *c81Off, *airfoilNo;
  // frames [(nt+1) * fl.size]
  double* frames;
  // wing dynamic
  double *wGam, *gamPrev, *gamVec, *gamVecPrev, *RHS, *velCP, *velCPTotal;
  double *AIC, *AICinv, *LU;
  int* piv;
  // FP32 LU + FP64 refinement (null when the solve uses the FP64 inverse)
  float *LU32, *AICinv32;
  int* piv32;
  double *refX, *refR, *luRes;
  // near wake
  double *nC, *nCP, *nGam, *nRvc, *nAge, *nTmp;
  // far wake
  double *fC, *fCP, *fGam, *fRvc, *fRvc0, *fL0, *fLc, *fAge, *fTmp;
  // prescribed far wake [2: free wake, predicted wake][nb]: filaments
  // [kPresc][fc1 xyz, fc2 xyz], one circulation and core radius per blade,
  // helix pitch and radius (their relaxation state); null when the case has none
  double *pfC, *pfGam, *pfRvc, *pfHelix;
  // node velocities: 0 vel, 1 vel1, 2 vel2, 3 vel3, 4 velPredicted, 5 velStep, 6 scratch
  double* vN[7];
  double* vF[7];
  // loads outputs (per blade, per section, xyz)
  double *secResVel, *secLiftDir, *secDragDir, *secLift, *secForceInertial, *secLiftUnsteady, *secLiftInPlane,
      *secLiftOutPlane, *secCL, *secCD, *secCLu;
  double *bladeForce;  // [nb][4][3]: forceInertial, lift, drag(0), liftUnsteady
  double* rotorLift;   // [6] lift (liftPrev of the next step), forceInertial
  double* ctHist;      // [(nt+1) * 10]
  // N-body scratch
  double *rec64, *targets, *part, *outv;
  float* rec32;
  // lattice-form edge weights of the gathered records ([rec][4]; null: the
  // records are evaluated ring by ring), written by the gather
  double* edgeW;
  void* nearScratch;  // near-field grid scratch (null unless FP32 + FP64 near field)
  size_t nearBytes;
  long long* nacc;  // fixed-point near-field accumulators, zero between evaluations
  // step replay by a CUDA graph: the step counter on the device and the
  // frame of the step being computed (filled by launch_step_begin)
  int* devIter;
  double* curFrame;
  int* err;  // [0] LU/inverse check, [1] refinement residual, [2] FP32 pipeline or near-list error, [3] near-pair count
};

// ---- wake bookkeeping (src/classdef.f90:4297-4605, 1515-1702, 4786-4830) ----
void launch_shed(const Dims& d, const DevState& s, const double* frame, int rowNear, bool leadingEdge, cudaStream_t st);
void launch_age(const Dims& d, const DevState& s, int rowNear, int rowFar, cudaStream_t st);
void launch_dissipate(const Dims& d, const DevState& s, int rowNear, int rowFar, cudaStream_t st);
void launch_copy_predicted(const Dims& d, const DevState& s, int rowNear, int rowFar, cudaStream_t st);
// shift (pred: predicted wake with the reference's row-1 loop) + continuity + axisymmetric copies
void launch_convect(const Dims& d, const DevState& s, const double* frame, int rowNear, int rowFar, bool pred,
                    cudaStream_t st);
void launch_strain(const Dims& d, const DevState& s, int rowFar, cudaStream_t st);
// the prescribed far wake of the free (pred = false) or predicted wake
// fitted to its far wake, then copied and rotated to the other blades under
// axisymmetry (classdef.f90:5172-5217)
void launch_presc_update(const Dims& d, const DevState& s, const double* frame, int rowFar, bool pred, cudaStream_t st);
// wake burst of every blade's far wake (classdef.f90:4911-4917, 2306-2339)
void launch_burst(const Dims& d, const DevState& s, int rowFar, cudaStream_t st);
void launch_rollup(const Dims& d, const DevState& s, int rowFar, cudaStream_t st);
// velocity-history algebra over full arrays (blades < nbC)
enum VelOp {
  VOP_COPY_0_TO_1,     // v1 = v
  VOP_COPY_0_TO_2,     // v2 = v
  VOP_COPY_0_TO_3,     // v3 = v
  VOP_AB2,             // st = 0.5(3v - v1); v1 = st; v = st
  VOP_AM2_PRED,        // st = v; v = 0.5(3v - v1)
  VOP_AM2_CORR,        // v = (vp + st) 0.5
  VOP_STEP_TO_1,       // v1 = st
  VOP_AM3_PRED,        // st = v; v = (23v - 16v2 + 5v1)/12
  VOP_AM3_CORR,        // v = (5vp + 8st - v2)/12
  VOP_AM3_SHIFT,       // v1 = v2; v2 = st
  VOP_AM4_PRED,        // st = v; v = (55v - 59v3 + 37v2 - 9v1)/24
  VOP_AM4_CORR,        // v = (9vp + 19st - 5v3 + v2)/24
  VOP_AM4_SHIFT,       // v1 = v2; v2 = v3; v3 = st
};
void launch_velop(const Dims& d, const DevState& s, VelOp op, cudaStream_t st);
// PC2 averaging (src/libCommon.f90:213-258)
void launch_order2(const Dims& d, const DevState& s, int rowNear, int rowFar, cudaStream_t st);

// ---- Biot-Savart evaluations ---------------------------------------------
// targets: wake nodes of blades < nbC (count returned by node_target_count)
int node_target_count(const Dims& d, int rowNear, int rowFar);
void launch_node_targets(const Dims& d, const DevState& s, int rowNear, int rowFar, bool pred, double* P,
                         cudaStream_t st);
void launch_cp_targets(const Dims& d, const double* frame, double* P, cudaStream_t st);
// record gather for the given groups (kind 0 wing, kind 1 wake)
void launch_gather(const Dims& d, const DevState& s, const double* frame, const Group* groups, int ngroups,
                   int nrec, int rowNear, int rowFar, bool pred, cudaStream_t st);
// node velocities from outv (0 + v), plus the initial wake velocity terms
void launch_scatter_nodes(const Dims& d, const DevState& s, const double* frame, int rowNear, int rowFar, bool pred,
                          double initWakeVel, cudaStream_t st);

// ---- circulation and loads -----------------------------------------------
void launch_aic(const Dims& d, const DevState& s, const double* frame, cudaStream_t st);
void launch_lu_inverse(const Dims& d, const DevState& s, cudaStream_t st);
void launch_is_inverse(const Dims& d, const DevState& s, cudaStream_t st);
// FP32 LU with partial pivoting of the AIC and its FP32 inverse (solves then
// refine in FP64: launch_solve uses them when s.LU32 is set)
void launch_lu32(const Dims& d, const DevState& s, cudaStream_t st);
// velCP = velKin (+ wake velocity in outv if withWake); RHS; gamVec = AICinv RHS; map to wing gam
void launch_solve(const Dims& d, const DevState& s, const double* frame, bool withWake, cudaStream_t st);
// start of a replayed step: devIter += 1, curFrame = frame[devIter]
void launch_step_begin(const Dims& d, const DevState& s, cudaStream_t st);
// velCPTotal, sectional resultant velocity, lift direction, forces, CT row
// (iter < 0: the row of the device step counter)
void launch_loads(const Dims& d, const DevState& s, const double* frame, int sumChunk, int iter, cudaStream_t st,
                  const double* foreignBound = nullptr, int nrs = 1, int self = 0);
// Coupled rotors (src/main.f90:522-603, 623-690): the RHS from the kinematic
// velocity plus nterms per-rotor sums ([term][point][xyz]); the solve alone;
// the bound vortices of rotor (ds, ss) at the collocation points of rotor dt.
void launch_rhs_terms(const Dims& d, const DevState& s, const double* frame, const double* terms, int nterms,
                      cudaStream_t st);
void launch_solve_only(const Dims& d, const DevState& s, cudaStream_t st);
// Image rotors (src/classdef.f90:4990-5131): velCP and the circulation of the
// source mirrored; its wake mirrored (mode 0 the active current wake, 1 the
// active predicted wake, 2 every row of the current wake; d, rows of the image)
void launch_mirror_velcp(const Dims& d, const DevState& s, const double* srcVelCP, int plane, cudaStream_t st);
void launch_mirror_gamma(const Dims& d, const DevState& s, const double* srcGamVec, cudaStream_t st);
void launch_mirror_wake(const Dims& d, const DevState& dst, const DevState& src, int mode, int rowNear, int rowFar,
                        int plane, cudaStream_t st);
void launch_bound_foreign(const Dims& dt, const double* frameT, const Dims& ds, const DevState& ss,
                          const double* frameS, double* out, cudaStream_t st);

// ---- learned far-wake surrogate (surrogate.cu) ------------------------------
// targets: the convecting blades' CPs, then nNodes inner-wake nodes (every
// stride-th from offset; per blade the near-wake nodes of rows rowNear..NW
// and the `young` youngest far-wake nodes)
void launch_surr_targets(const Dims& d, const DevState& s, const double* fr, int rowNear, int rowFar, int young,
                         int stride, int offset, int nNodes, double* P, cudaStream_t st);
// old far-wake nodes (all but the `young` youngest) of the convecting blades
void launch_surr_far_targets(const Dims& d, const DevState& s, int rowFar, int young, bool pred, double* P,
                             cudaStream_t st);
// FP32 features per target (position about the hub / R, rotor azimuth
// harmonics, old-wake fill) and the old far wake's coarse descriptor
// (|circulation|-weighted centroid about the hub / R, relative mean
// |circulation|), computed into desc[4] first
constexpr int kSurrFeatures = 12;
void launch_surr_features(const Dims& d, const DevState& s, const double* fr, const double* P, int M, double invR,
                          double fill, int rowFar, int young, bool pred, double* desc, float* X, cudaStream_t st);
void launch_surr_add(int M, const float* Y, const double* scale, double* outv, cudaStream_t st);
void launch_surr_merge_nodes(const Dims& d, int rowNear, int rowFar, int young, int M, const float* Y,
                             const double* scale, const double* outFar, double* outv, cudaStream_t st);
void launch_surr_append(int n, const float* Xs, const double* V, float* X, float* T, cudaStream_t st);
void launch_surr_audit(int n, const float* Y, const double* scale, const double* V, double* out, cudaStream_t st);

}  // namespace vlm
