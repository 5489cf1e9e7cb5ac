// vlm_case: device state, per-step plans and the time loop of one rotor case,
// plus the extern "C" API declared in include/vlm.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <memory>
#include <mutex>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/vlm.h"
#include "vlm_bs.h"
#include "vlm_solver.h"
#include "wing.h"

namespace vlm {

thread_local std::string g_err;

struct CudaError : std::runtime_error {
  using std::runtime_error::runtime_error;
};
struct StatusError : std::runtime_error {
  int code;
  StatusError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define VLM_CUDA(x)                                                                                \
  do {                                                                                             \
    cudaError_t e_ = (x);                                                                          \
    if (e_ != cudaSuccess) throw CudaError(std::string(#x) + ": " + cudaGetErrorString(e_));       \
  } while (0)

template <class T>
static T* dalloc(size_t n, std::vector<void*>& owned) {
  void* p = nullptr;
  if (n == 0) n = 1;
  VLM_CUDA(cudaMalloc(&p, n * sizeof(T)));
  VLM_CUDA(cudaMemset(p, 0, n * sizeof(T)));
  owned.push_back(p);
  return static_cast<T*>(p);
}

// Source/target layout of one Biot-Savart evaluation at one step.
struct EvalPlan {
  int goff = 0, ngroups = 0;  // into the step plan's group table
  int coff = 0, nchunks = 0;  // into the chunk table
  int nrec = 0;
  int maxq = 0;  // most chunks of one group
};
struct StepPlan {
  int rowNear = 0, rowFar = 0;
  EvalPlan rhs, node;
};

struct Case {
  Wing W;
  vlm_options opt{};
  Dims d{};
  DevState s{};
  std::vector<void*> owned;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::vector<StepPlan> plans;  // index = iteration (0..nt)
  double* hFrames = nullptr;    // pinned host copy of every frame; uploaded per vlm_case_step call
  std::vector<Group> hGroups;
  std::vector<Chunk> hChunks;
  Group* dGroups = nullptr;
  Chunk* dChunks = nullptr;
  int iter = 0;
  bool started = false;
  int chunk64 = 0;
  int slots32 = 0;  // resident FP32-kernel blocks on the device (chunk planner input)
  double lastMs = 0;
  int maxTargets = 0, maxRecords = 0, maxChunks = 0;
  int64_t maxPart = 1;  // largest (chunks x targets) of any evaluation

  ~Case() {
    if (stream) cudaStreamSynchronize(stream);
    for (void* p : owned) cudaFree(p);
    if (hFrames) cudaFreeHost(hFrames);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (stream) cudaStreamDestroy(stream);
  }

  // chunk table of one evaluation: the FP64 summation order, or the FP32
  // kernel's planned chunks for M targets
  int chunkTable(Group* g, int ng, int M, Chunk* out, int cap) const {
    if (opt.precision == VLM_PREC_FP64) return build_chunks(g, ng, chunk64, out, cap);
    return plan_chunks32(g, ng, M, slots32, out, cap);
  }

  // groups of one evaluation: wing sums (kind 0) for every blade when
  // withWing, then wake sums (kind 1) for every blade
  void addEval(EvalPlan& e, bool withWing, int rowNear, int rowFar, int M) {
    const int NW = d.NW, NF = d.NF, ns = d.ns;
    e.goff = (int)hGroups.size();
    int rec = 0;
    if (withWing)
      for (int b = 0; b < d.nb; ++b) {
        Group g{};
        g.rec_begin = rec;
        g.rec_count = d.npan;
        g.kind = 0;
        g.blade = b;
        rec += g.rec_count;
        hGroups.push_back(g);
      }
    for (int b = 0; b < d.nb; ++b) {
      Group g{};
      const int nNear = (NW - (rowNear - 1)) * ns;
      const int hs = rowFar <= NF ? ns : 0;
      const int nFar = rowFar <= NF ? NF - rowFar + 1 : 0;
      g.rec_begin = rec;
      g.rec_count = nNear + hs + nFar;
      g.kind = 1;
      g.blade = b;
      rec += g.rec_count;
      hGroups.push_back(g);
    }
    e.ngroups = (int)hGroups.size() - e.goff;
    e.nrec = rec;
    e.coff = (int)hChunks.size();
    std::vector<Chunk> tmp(rec + e.ngroups + 1);
    const int nq = chunkTable(hGroups.data() + e.goff, e.ngroups, M, tmp.data(), (int)tmp.size());
    if (nq < 0) throw std::runtime_error("chunk table overflow");
    hChunks.insert(hChunks.end(), tmp.begin(), tmp.begin() + nq);
    e.nchunks = nq;
    for (int g = e.goff; g < e.goff + e.ngroups; ++g) e.maxq = std::max(e.maxq, hGroups[g].chunk_count);
    maxRecords = std::max(maxRecords, rec);
    maxChunks = std::max(maxChunks, nq);
    maxPart = std::max(maxPart, (int64_t)nq * M);
  }

  void create(const std::string& cfg, const std::string& geo, const std::string& base, const vlm_options* o) {
    vlm_default_options(&opt);
    if (o) opt = *o;
    if (opt.precision < 0 || opt.precision > 2) throw StatusError(VLM_ERR_INVALID, "precision must be 0, 1 or 2");
    chunk64 = opt.sum_chunk;
    W.load(cfg, geo, base);
    const RotorParams& P = W.P;
    d.nb = P.nb;
    d.nc = P.nc;
    d.ns = P.ns;
    d.npan = P.nc * P.ns;
    d.n = d.npan * P.nb;
    d.NW = P.nNwake;
    d.NF = W.nFwake;
    d.nbC = W.nbConvect;
    d.axisym = P.axisymmetrySwitch == 1 ? 1 : 0;
    d.spanwiseLift = P.spanwiseLiftSwitch;
    d.rollupStart = W.rollupStart;
    d.rollupEnd = W.rollupEnd;
    d.suppressFwake = 0;
    d.omega = P.Omega;
    d.theta0 = P.controlPitch.x;
    d.density = W.density;
    d.dt = W.dt;
    d.nonDimDenom = W.nonDimDenom;
    d.dissipAdd = (((4.0 * 1.2564) * P.apparentViscCoeff) * W.kinematicVisc) * W.dt;
    d.decay = std::exp(-(P.decayCoeff * W.dt));
    d.fl = frame_layout(d.nb, d.nc, d.ns);
    if (d.nc > 64) throw StatusError(VLM_ERR_UNSUPPORTED, "nc > 64 chordwise panels");
    if (d.n > 8192) throw StatusError(VLM_ERR_UNSUPPORTED, "more than 8192 panels per rotor");
    const int nt = W.nt;

    VLM_CUDA(cudaSetDevice(opt.device));
    slots32 = partial32_slots();
    VLM_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    VLM_CUDA(cudaEventCreate(&ev0));
    VLM_CUDA(cudaEventCreate(&ev1));

    // frames: 0 = after the initial pitch, k = after the kinematics of step k
    std::vector<double> frames((size_t)(nt + 1) * d.fl.size);
    W.start_pitch();
    W.write_frame(frames.data());
    for (int k = 1; k <= nt; ++k) {
      W.advance(k);
      W.write_frame(frames.data() + (size_t)k * d.fl.size);
    }
    // plans
    plans.assign(nt + 1, StepPlan());
    int rowNear = d.NW + 1, rowFar = d.NF + 1;
    plans[0].rowNear = rowNear;
    plans[0].rowFar = rowFar;
    maxTargets = d.nbC * d.npan;
    for (int k = 1; k <= nt; ++k) {
      rowNear = std::max(rowNear - 1, 1);
      if (k > d.NW) rowFar = std::max(rowFar - 1, 1);
      StepPlan& pl = plans[k];
      pl.rowNear = rowNear;
      pl.rowFar = rowFar;
      if (d.NW > 0) {
        addEval(pl.rhs, false, rowNear, rowFar, d.nbC * d.npan);
        addEval(pl.node, true, rowNear, rowFar, node_target_count(d, rowNear, rowFar));
        maxTargets = std::max(maxTargets, node_target_count(d, rowNear, rowFar));
      }
    }

    // device memory
    const int nb = d.nb, npan = d.npan, NW = d.NW, NF = d.NF, ns = d.ns;
    s.frames = dalloc<double>(frames.size(), owned);
    VLM_CUDA(cudaMallocHost(&hFrames, frames.size() * sizeof(double)));
    std::memcpy(hFrames, frames.data(), frames.size() * sizeof(double));
    VLM_CUDA(cudaMemcpy(s.frames, hFrames, (size_t)d.fl.size * sizeof(double), cudaMemcpyHostToDevice));
    std::vector<double> rvc((size_t)nb * npan * 4), area((size_t)nb * npan), mc((size_t)nb * npan),
        msp((size_t)nb * npan), sa((size_t)nb * ns);
    for (int b = 0; b < nb; ++b) {
      for (int p = 0; p < npan; ++p) {
        const Panel& q = W.bl[b].p[p];
        for (int k = 0; k < 4; ++k) rvc[4 * ((size_t)b * npan + p) + k] = q.rvc[k];
        area[(size_t)b * npan + p] = q.area;
        mc[(size_t)b * npan + p] = q.meanChord;
        msp[(size_t)b * npan + p] = q.meanSpan;
      }
      for (int is = 0; is < ns; ++is) sa[(size_t)b * ns + is] = W.bl[b].secArea[is];
    }
    auto up = [&](const std::vector<double>& h) {
      double* p = dalloc<double>(h.size(), owned);
      VLM_CUDA(cudaMemcpy(p, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice));
      return p;
    };
    s.wRvc = up(rvc);
    s.panArea = up(area);
    s.panMeanChord = up(mc);
    s.panMeanSpan = up(msp);
    s.secArea = up(sa);
    s.wGam = dalloc<double>((size_t)nb * npan, owned);
    s.gamPrev = dalloc<double>((size_t)nb * npan, owned);
    s.gamVec = dalloc<double>(d.n, owned);
    s.gamVecPrev = dalloc<double>(d.n, owned);
    s.RHS = dalloc<double>(d.n, owned);
    s.velCP = dalloc<double>((size_t)3 * nb * npan, owned);
    s.velCPTotal = dalloc<double>((size_t)3 * nb * npan, owned);
    s.AIC = dalloc<double>((size_t)d.n * d.n, owned);
    s.AICinv = dalloc<double>((size_t)d.n * d.n, owned);
    s.LU = dalloc<double>((size_t)d.n * d.n, owned);
    s.piv = dalloc<int>(d.n, owned);
    const size_t nring = (size_t)nb * std::max(NW, 1) * ns;
    s.nC = dalloc<double>(nring * 12, owned);
    s.nCP = dalloc<double>(nring * 12, owned);
    s.nGam = dalloc<double>(nring, owned);
    s.nRvc = dalloc<double>(nring * 4, owned);
    s.nAge = dalloc<double>(nring, owned);
    s.nTmp = dalloc<double>(nring * 18, owned);
    const size_t nfar = (size_t)nb * std::max(NF, 1);
    s.fC = dalloc<double>(nfar * 6, owned);
    s.fCP = dalloc<double>(nfar * 6, owned);
    s.fGam = dalloc<double>(nfar, owned);
    s.fRvc = dalloc<double>(nfar, owned);
    s.fRvc0 = dalloc<double>(nfar, owned);
    s.fL0 = dalloc<double>(nfar, owned);
    s.fLc = dalloc<double>(nfar, owned);
    s.fAge = dalloc<double>(nfar, owned);
    s.fTmp = dalloc<double>(nfar * 12, owned);
    for (int k = 0; k < 7; ++k) {
      s.vN[k] = dalloc<double>((size_t)nb * std::max(NW, 1) * (ns + 1) * 3, owned);
      s.vF[k] = dalloc<double>(nfar * 3, owned);
    }
    const size_t nsec = (size_t)nb * ns;
    s.secResVel = dalloc<double>(3 * nsec, owned);
    s.secLiftDir = dalloc<double>(3 * nsec, owned);
    s.secDragDir = dalloc<double>(3 * nsec, owned);
    s.secLift = dalloc<double>(3 * nsec, owned);
    s.secForceInertial = dalloc<double>(3 * nsec, owned);
    s.secLiftUnsteady = dalloc<double>(3 * nsec, owned);
    s.secLiftInPlane = dalloc<double>(3 * nsec, owned);
    s.secLiftOutPlane = dalloc<double>(3 * nsec, owned);
    s.secCL = dalloc<double>(nsec, owned);
    s.secCD = dalloc<double>(nsec, owned);
    s.secCLu = dalloc<double>(nsec, owned);
    s.bladeForce = dalloc<double>((size_t)nb * 12, owned);
    s.rotorLift = dalloc<double>(3, owned);
    s.ctHist = dalloc<double>((size_t)(nt + 1) * 10, owned);
    s.err = dalloc<int>(4, owned);
    // initial wake cores (classdef.f90:3864-3891)
    if (NW > 0) {
      std::vector<double> nr(nring * 4), fr(nfar, P.streamwiseCoreVec[ns]);
      for (int b = 0; b < nb; ++b)
        for (int j = 0; j < ns; ++j)
          for (int i = 0; i < NW; ++i) {
            double* r = nr.data() + 4 * ((size_t)b * NW * ns + i + (size_t)NW * j);
            r[0] = P.streamwiseCoreVec[j];
            r[1] = P.spanwiseCore;
            r[2] = P.streamwiseCoreVec[j + 1];
            r[3] = P.spanwiseCore;
          }
      VLM_CUDA(cudaMemcpy(s.nRvc, nr.data(), nr.size() * sizeof(double), cudaMemcpyHostToDevice));
      VLM_CUDA(cudaMemcpy(s.fRvc, fr.data(), fr.size() * sizeof(double), cudaMemcpyHostToDevice));
      VLM_CUDA(cudaMemcpy(s.fRvc0, fr.data(), fr.size() * sizeof(double), cudaMemcpyHostToDevice));
    }
    // N-body scratch
    maxRecords = std::max(maxRecords, d.n);
    s.rec64 = dalloc<double>((size_t)maxRecords * kRec64, owned);
    s.rec32 = dalloc<float>((size_t)maxRecords * kRec32, owned);
    s.targets = dalloc<double>((size_t)maxTargets * 3, owned);
    s.outv = dalloc<double>((size_t)maxTargets * 3, owned);
    s.part = dalloc<double>((size_t)maxPart * 3, owned);
    s.nearCap = opt.precision == VLM_PREC_FP32_NEAR64 ? 256 * maxTargets : 1;
    s.near = dalloc<NearPair>((size_t)s.nearCap, owned);
    // zero here; every near-field evaluation leaves them zero
    s.nacc = dalloc<long long>(opt.precision == VLM_PREC_FP32_NEAR64 ? (size_t)maxPart * 3 : 1, owned);
    dGroups = dalloc<Group>(std::max<size_t>(hGroups.size(), 1), owned);
    dChunks = dalloc<Chunk>(std::max<size_t>(hChunks.size(), 1), owned);
    if (!hGroups.empty())
      VLM_CUDA(cudaMemcpy(dGroups, hGroups.data(), hGroups.size() * sizeof(Group), cudaMemcpyHostToDevice));
    if (!hChunks.empty())
      VLM_CUDA(cudaMemcpy(dChunks, hChunks.data(), hChunks.size() * sizeof(Chunk), cudaMemcpyHostToDevice));
  }

  const double* frame(int k) const { return s.frames + (size_t)k * d.fl.size; }

  // one Biot-Savart evaluation of plan e into s.outv (targets already in s.targets)
  void evaluate(const EvalPlan& e, int M, int mode) {
    const Chunk* ch = dChunks + e.coff;
    if (opt.precision == VLM_PREC_FP64) {
      launch_partial64(s.rec64, ch, e.nchunks, s.targets, M, s.part, stream);
    } else {
      const bool nearOn = opt.precision == VLM_PREC_FP32_NEAR64;
      launch_pack32(s.rec64, e.nrec, nearOn ? opt.near_factor : 0.0, s.rec32, stream);
      VLM_CUDA(cudaMemsetAsync(s.err + 3, 0, sizeof(int), stream));
      launch_partial32(s.rec32, s.rec64, ch, e.nchunks, s.targets, M, s.part, s.err + 2, nearOn ? s.near : nullptr,
                       s.nearCap, s.nacc, stream);
    }
    if (opt.precision == VLM_PREC_FP64) launch_combine(s.part, M, dGroups + e.goff, e.ngroups, mode, s.outv, stream);
    else launch_combine_unordered(s.part, M, dGroups + e.goff, e.ngroups, e.maxq, mode, s.outv, stream);
  }

  void evalNodes(int k, bool pred) {
    const StepPlan& pl = plans[k];
    const int M = node_target_count(d, pl.rowNear, pl.rowFar);
    launch_node_targets(d, s, pl.rowNear, pl.rowFar, pred, s.targets, stream);
    launch_gather(d, s, frame(k), dGroups + pl.node.goff, pl.node.ngroups, pl.node.nrec, pl.rowNear, pl.rowFar, pred,
                  stream);
    evaluate(pl.node, M, 0);
    const double iwv = k < W.sw.initWakeVelNt ? W.P.initWakeVel : 0.0;
    launch_scatter_nodes(d, s, frame(k), pl.rowNear, pl.rowFar, pred, iwv, stream);
  }

  void start() {
    if (started) throw StatusError(VLM_ERR_STATE, "case already started");
    launch_aic(d, s, frame(0), stream);
    launch_lu_inverse(d, s, stream);
    launch_is_inverse(d, s, stream);
    int err = 0;
    VLM_CUDA(cudaMemcpyAsync(&err, s.err, sizeof(int), cudaMemcpyDeviceToHost, stream));
    VLM_CUDA(cudaStreamSynchronize(stream));
    if (err == 10) throw StatusError(VLM_ERR_SINGULAR, "Matrix is numerically singular!");
    if (err == 11) throw StatusError(VLM_ERR_SINGULAR, "Computed AIC_inv does not seem to be correct within given tolerance");
    launch_solve(d, s, frame(0), false, stream);
    if (d.NW > 0) launch_shed(d, s, frame(0), d.NW + 1, false, stream);
    if (W.sw.rotorForcePlot != 0) launch_loads(d, s, frame(0), chunk64, 0, stream);
    VLM_CUDA(cudaGetLastError());
    VLM_CUDA(cudaStreamSynchronize(stream));
    iter = 0;
    started = true;
  }

  void enqueueStep(int k) {
    const StepPlan& pl = plans[k];
    const int rN = pl.rowNear, rF = pl.rowFar;
    const double* fr = frame(k);
    const bool wake = d.NW > 0 && W.sw.wakeSuppress == 0;
    if (wake) {
      launch_shed(d, s, fr, rN, true, stream);
      launch_age(d, s, rN, rF, stream);
      if (W.sw.wakeDissipation == 1) launch_dissipate(d, s, rN, rF, stream);
    }
    if (d.NW > 0) {
      launch_cp_targets(d, fr, s.targets, stream);
      launch_gather(d, s, fr, dGroups + pl.rhs.goff, pl.rhs.ngroups, pl.rhs.nrec, rN, rF, false, stream);
      evaluate(pl.rhs, d.nbC * d.npan, 1);
      launch_solve(d, s, fr, true, stream);
    } else {
      launch_solve(d, s, fr, false, stream);
    }
    if (W.sw.rotorForcePlot != 0 && k % W.sw.rotorForcePlot == 0) launch_loads(d, s, fr, chunk64, k, stream);
    if (!wake) return;
    evalNodes(k, false);
    switch (W.sw.fdScheme) {
      case 0:
        launch_convect(d, s, fr, rN, rF, false, stream);
        break;
      case 1:
        launch_copy_predicted(d, s, rN, rF, stream);
        launch_convect(d, s, fr, rN, rF, true, stream);
        evalNodes(k, true);
        launch_order2(d, s, rN, rF, stream);
        launch_convect(d, s, fr, rN, rF, false, stream);
        break;
      case 2:
        if (k == 1) {
          launch_convect(d, s, fr, rN, rF, false, stream);
          launch_velop(d, s, VOP_COPY_0_TO_1, stream);
        } else {
          launch_velop(d, s, VOP_AB2, stream);
          launch_convect(d, s, fr, rN, rF, false, stream);
        }
        break;
      case 3:
        if (k == 1) {
          launch_convect(d, s, fr, rN, rF, false, stream);
          launch_velop(d, s, VOP_COPY_0_TO_1, stream);
        } else {
          launch_copy_predicted(d, s, rN, rF, stream);
          launch_velop(d, s, VOP_AM2_PRED, stream);
          launch_convect(d, s, fr, rN, rF, true, stream);
          evalNodes(k, true);
          launch_velop(d, s, VOP_AM2_CORR, stream);
          launch_convect(d, s, fr, rN, rF, false, stream);
          launch_velop(d, s, VOP_STEP_TO_1, stream);
        }
        break;
      case 4:
        // the reference tests iter == 0 for the start-up branch (never true)
        if (k == 2) {
          launch_convect(d, s, fr, rN, rF, false, stream);
          launch_velop(d, s, VOP_COPY_0_TO_2, stream);
        } else {
          launch_copy_predicted(d, s, rN, rF, stream);
          launch_velop(d, s, VOP_AM3_PRED, stream);
          launch_convect(d, s, fr, rN, rF, true, stream);
          evalNodes(k, true);
          launch_velop(d, s, VOP_AM3_CORR, stream);
          launch_convect(d, s, fr, rN, rF, false, stream);
          launch_velop(d, s, VOP_AM3_SHIFT, stream);
        }
        break;
      case 5:
        if (k <= 3) {
          launch_convect(d, s, fr, rN, rF, false, stream);
          launch_velop(d, s, k == 1 ? VOP_COPY_0_TO_1 : (k == 2 ? VOP_COPY_0_TO_2 : VOP_COPY_0_TO_3), stream);
        } else {
          launch_copy_predicted(d, s, rN, rF, stream);
          launch_velop(d, s, VOP_AM4_PRED, stream);
          launch_convect(d, s, fr, rN, rF, true, stream);
          evalNodes(k, true);
          launch_velop(d, s, VOP_AM4_CORR, stream);
          launch_convect(d, s, fr, rN, rF, false, stream);
          launch_velop(d, s, VOP_AM4_SHIFT, stream);
        }
        break;
    }
    if (W.sw.wakeStrain == 1) launch_strain(d, s, rF, stream);
    if (rN == 1) launch_rollup(d, s, rF, stream);
    launch_shed(d, s, fr, rN, false, stream);
  }

  void step(int nsteps, double* ctRows) {
    if (!started) throw StatusError(VLM_ERR_STATE, "vlm_case_start must be called before vlm_case_step");
    if (nsteps < 0 || iter + nsteps > W.nt)
      throw StatusError(VLM_ERR_INVALID, "nsteps runs past the case's nt timesteps");
    // this call's inputs: the wing frames of its steps (host -> device)
    if (nsteps > 0)
      VLM_CUDA(cudaMemcpyAsync(s.frames + (size_t)(iter + 1) * d.fl.size, hFrames + (size_t)(iter + 1) * d.fl.size,
                               sizeof(double) * d.fl.size * nsteps, cudaMemcpyHostToDevice, stream));
    VLM_CUDA(cudaEventRecord(ev0, stream));
    for (int k = iter + 1; k <= iter + nsteps; ++k) enqueueStep(k);
    VLM_CUDA(cudaEventRecord(ev1, stream));
    VLM_CUDA(cudaGetLastError());
    if (ctRows && nsteps > 0)
      VLM_CUDA(cudaMemcpyAsync(ctRows, s.ctHist + (size_t)(iter + 1) * 10, sizeof(double) * 10 * nsteps,
                               cudaMemcpyDeviceToHost, stream));
    int errs[4] = {0, 0, 0, 0};
    VLM_CUDA(cudaMemcpyAsync(errs, s.err, sizeof(errs), cudaMemcpyDeviceToHost, stream));
    VLM_CUDA(cudaStreamSynchronize(stream));
    const int err = errs[2];
    float ms = 0.f;
    VLM_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
    lastMs = ms;
    iter += nsteps;
    if (err == 3) throw StatusError(VLM_ERR_CUDA, "near-field pair list overflowed");
    if (err == 4) throw StatusError(VLM_ERR_NONFINITE, "near-field velocity outside the fixed-point range");
    if (err) throw StatusError(VLM_ERR_CUDA, "device wait limit expired in a Biot-Savart tile pipeline");
    if (ctRows)
      for (int k = 0; k < 10 * nsteps; ++k)
        if (!std::isfinite(ctRows[k])) throw StatusError(VLM_ERR_NONFINITE, "non-finite load in the CT history");
  }

  // Times the partial-sum kernel of the next step's wake-node evaluation on
  // the current state (reps launches between CUDA events); reports the mean
  // launch time and the ring / single-filament pair counts of one launch.
  void profileEval(int reps, double* msPerLaunch, double* ringPairs, double* filPairs) {
    if (!started || d.NW == 0 || iter >= W.nt) throw StatusError(VLM_ERR_STATE, "needs a started case with steps left");
    const int k = iter + 1;
    const StepPlan& pl = plans[k];
    VLM_CUDA(cudaMemcpyAsync(s.frames + (size_t)k * d.fl.size, hFrames + (size_t)k * d.fl.size,
                             sizeof(double) * d.fl.size, cudaMemcpyHostToDevice, stream));
    const int M = node_target_count(d, pl.rowNear, pl.rowFar);
    launch_node_targets(d, s, pl.rowNear, pl.rowFar, false, s.targets, stream);
    launch_gather(d, s, frame(k), dGroups + pl.node.goff, pl.node.ngroups, pl.node.nrec, pl.rowNear, pl.rowFar, false,
                  stream);
    const Chunk* ch = dChunks + pl.node.coff;
    const double nf = opt.precision == VLM_PREC_FP32_NEAR64 ? opt.near_factor : 0.0;
    if (opt.precision != VLM_PREC_FP64) launch_pack32(s.rec64, pl.node.nrec, nf, s.rec32, stream);
    auto launch = [&]() {
      if (opt.precision == VLM_PREC_FP64) launch_partial64(s.rec64, ch, pl.node.nchunks, s.targets, M, s.part, stream);
      else {
        VLM_CUDA(cudaMemsetAsync(s.err + 3, 0, sizeof(int), stream));
        launch_partial32(s.rec32, s.rec64, ch, pl.node.nchunks, s.targets, M, s.part, s.err + 2,
                         opt.precision == VLM_PREC_FP32_NEAR64 ? s.near : nullptr, s.nearCap, s.nacc, stream);
      }
    };
    launch();  // warm
    VLM_CUDA(cudaEventRecord(ev0, stream));
    for (int r = 0; r < reps; ++r) launch();
    VLM_CUDA(cudaEventRecord(ev1, stream));
    VLM_CUDA(cudaStreamSynchronize(stream));
    float ms = 0.f;
    VLM_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
    *msPerLaunch = ms / reps;
    // records: wing rings, near rings, horseshoe + far single filaments
    long rings = (long)d.nb * d.npan, fils = 0;
    const int rowsN = d.NW - (pl.rowNear - 1);
    rings += (long)d.nb * rowsN * d.ns;
    if (pl.rowFar <= d.NF) fils += (long)d.nb * (d.ns + d.NF - pl.rowFar + 1);
    *ringPairs = (double)rings * M;
    *filPairs = (double)fils * M;
  }

  std::vector<double> dget(const double* p, size_t n) {
    std::vector<double> h(n);
    VLM_CUDA(cudaStreamSynchronize(stream));
    if (n) VLM_CUDA(cudaMemcpy(h.data(), p, n * sizeof(double), cudaMemcpyDeviceToHost));
    return h;
  }

  int64_t get(const std::string& k, int blade, double* out, int64_t cap) {
    std::vector<double> v;
    const int b = blade - 1;
    const bool bok = b >= 0 && b < d.nb;
    const size_t npan = d.npan, NW = d.NW, NF = d.NF, ns = d.ns;
    if (k == "dt") v = {W.dt};
    else if (k == "nonDimDenom") v = {W.nonDimDenom};
    else if (k == "ct_hist") v = dget(s.ctHist, (size_t)(iter + 1) * 10);
    else if (k == "gamVec") v = dget(s.gamVec, d.n);
    else if (k == "AIC") v = dget(s.AIC, (size_t)d.n * d.n);
    else if (k == "AIC_inv") v = dget(s.AICinv, (size_t)d.n * d.n);
    else if (bok && k == "gam") {
      auto a = dget(s.wGam + b * npan, npan);
      v = a;
    } else if (bok && k == "velCP") v = dget(s.velCP + 3 * b * npan, 3 * npan);
    else if (bok && k == "velCPTotal") v = dget(s.velCPTotal + 3 * b * npan, 3 * npan);
    else if (bok && k == "waN") v = dget(s.nC + 12 * b * NW * ns, 12 * NW * ns);
    else if (bok && k == "waN_gam") v = dget(s.nGam + b * NW * ns, NW * ns);
    else if (bok && k == "waN_rvc") v = dget(s.nRvc + 4 * b * NW * ns, 4 * NW * ns);
    else if (bok && k == "waF") v = dget(s.fC + 6 * b * NF, 6 * NF);
    else if (bok && k == "waF_gam") v = dget(s.fGam + b * NF, NF);
    else if (bok && k == "waF_rvc") v = dget(s.fRvc + b * NF, NF);
    else if (bok && k == "velN") v = dget(s.vN[0] + 3 * b * NW * (ns + 1), 3 * NW * (ns + 1));
    else if (bok && k == "velF") v = dget(s.vF[0] + 3 * b * NF, 3 * NF);
    else if (bok && k == "secCL") v = dget(s.secCL + b * ns, ns);
    else if (bok && k == "secLiftDir") v = dget(s.secLiftDir + 3 * b * ns, 3 * ns);
    else if (bok && k == "secChordwiseResVel") v = dget(s.secResVel + 3 * b * ns, 3 * ns);
    else if (bok && k == "secLift") v = dget(s.secLift + 3 * b * ns, 3 * ns);
    else if (bok && (k == "CP" || k == "nCap" || k == "vr")) {
      auto f = dget(frame(iter), d.fl.size);
      for (size_t p = 0; p < npan; ++p) {
        const double* r = f.data() + d.fl.pan + (b * npan + p) * kPan;
        if (k == "CP") v.insert(v.end(), r + 12, r + 15);
        else if (k == "nCap") v.insert(v.end(), r + 15, r + 18);
        else v.insert(v.end(), r, r + 12);
      }
    } else return -1;
    const int64_t n = (int64_t)v.size();
    if (out) std::memcpy(out, v.data(), sizeof(double) * std::min<int64_t>(n, cap));
    return n;
  }

  void vindPoints(const double* P, int64_t M, double* V) {
    if (!started) throw StatusError(VLM_ERR_STATE, "vlm_case_start must be called first");
    if (M <= 0) return;
    // groups of the current state: wing + wake at the current rows
    const StepPlan& pl = plans[std::max(iter, 1)];
    const int rN = iter == 0 ? d.NW + 1 : pl.rowNear, rF = iter == 0 ? d.NF + 1 : pl.rowFar;
    std::vector<Group> g;
    int rec = 0;
    for (int b = 0; b < d.nb; ++b) {
      Group q{};
      q.rec_begin = rec;
      q.rec_count = d.npan;
      q.kind = 0;
      q.blade = b;
      rec += d.npan;
      g.push_back(q);
    }
    if (d.NW > 0 && rN <= d.NW)
      for (int b = 0; b < d.nb; ++b) {
        Group q{};
        const int nNear = (d.NW - (rN - 1)) * d.ns;
        const int hs = rF <= d.NF ? d.ns : 0;
        const int nFar = rF <= d.NF ? d.NF - rF + 1 : 0;
        q.rec_begin = rec;
        q.rec_count = nNear + hs + nFar;
        q.kind = 1;
        q.blade = b;
        rec += q.rec_count;
        g.push_back(q);
      }
    std::vector<Chunk> ch(rec + g.size() + 1);
    const int nq = chunkTable(g.data(), (int)g.size(), (int)M, ch.data(), (int)ch.size());
    if (nq < 0) throw std::runtime_error("chunk table overflow");
    std::vector<void*> tmpOwned;
    Group* dg = dalloc<Group>(g.size(), tmpOwned);
    Chunk* dc = dalloc<Chunk>(nq, tmpOwned);
    double* rec64 = dalloc<double>((size_t)rec * kRec64, tmpOwned);
    float* rec32 = dalloc<float>((size_t)rec * kRec32, tmpOwned);
    double* dP = dalloc<double>((size_t)M * 3, tmpOwned);
    double* dV = dalloc<double>((size_t)M * 3, tmpOwned);
    double* part = dalloc<double>((size_t)M * nq * 3, tmpOwned);
    auto cleanup = [&]() {
      for (void* p : tmpOwned) cudaFree(p);
    };
    try {
      VLM_CUDA(cudaMemcpy(dg, g.data(), g.size() * sizeof(Group), cudaMemcpyHostToDevice));
      VLM_CUDA(cudaMemcpy(dc, ch.data(), nq * sizeof(Chunk), cudaMemcpyHostToDevice));
      VLM_CUDA(cudaMemcpy(dP, P, (size_t)M * 3 * sizeof(double), cudaMemcpyHostToDevice));
      DevState t = s;
      t.rec64 = rec64;
      launch_gather(d, t, frame(iter), dg, (int)g.size(), rec, rN, rF, false, stream);
      if (opt.precision == VLM_PREC_FP64) {
        launch_partial64(rec64, dc, nq, dP, (int)M, part, stream);
      } else {
        const bool nearOn = opt.precision == VLM_PREC_FP32_NEAR64;
        launch_pack32(rec64, rec, nearOn ? opt.near_factor : 0.0, rec32, stream);
        const int cap = nearOn ? (int)std::min<int64_t>(64 * M + (1 << 16), 1 << 26) : 1;
        NearPair* np = dalloc<NearPair>(cap, tmpOwned);
        long long* nacc = dalloc<long long>(nearOn ? (size_t)M * nq * 3 : 1, tmpOwned);
        VLM_CUDA(cudaMemsetAsync(s.err + 3, 0, sizeof(int), stream));
        launch_partial32(rec32, rec64, dc, nq, dP, (int)M, part, s.err + 2, nearOn ? np : nullptr, cap, nacc, stream);
      }
      if (opt.precision == VLM_PREC_FP64) launch_combine(part, (int)M, dg, (int)g.size(), 2, dV, stream);
      else {
        int maxq = 0;
        for (const Group& q : g) maxq = std::max(maxq, q.chunk_count);
        launch_combine_unordered(part, (int)M, dg, (int)g.size(), maxq, 2, dV, stream);
      }
      VLM_CUDA(cudaMemcpyAsync(V, dV, (size_t)M * 3 * sizeof(double), cudaMemcpyDeviceToHost, stream));
      VLM_CUDA(cudaStreamSynchronize(stream));
    } catch (...) {
      cleanup();
      throw;
    }
    cleanup();
  }
};

// ---------------------------------------------------------------------------
// Isolated ring kernel scratch, one grow-only buffer set per device.
struct RingScratch {
  std::mutex mu;
  double* rec64 = nullptr;
  float* rec32 = nullptr;
  double* part = nullptr;
  Chunk* chunks = nullptr;
  Group* group = nullptr;
  int* err = nullptr;
  NearPair* near = nullptr;
  long long* nacc = nullptr;  // zero between calls
  size_t cap64 = 0, cap32 = 0, capPart = 0, capChunks = 0, capNear = 0, capNacc = 0;
};
static RingScratch g_ring[64];

static void grow(void** p, size_t& cap, size_t need) {
  if (need <= cap) return;
  if (*p) cudaFree(*p);
  *p = nullptr;
  VLM_CUDA(cudaMalloc(p, need));
  cap = need;
}

static int ring_chunk(int64_t N, int64_t M, int precision) {
  // enough (target block x chunk) work items to fill the GPU several times
  const int64_t blocks = precision == VLM_PREC_FP64 ? (M + 127) / 128 : (M + 255) / 256;
  const int64_t want = 4 * 152;
  int64_t q = std::max<int64_t>(1, (want + blocks - 1) / blocks);
  q = std::min<int64_t>(q, std::max<int64_t>(1, N / 64));
  return (int)((N + q - 1) / q);
}

// Chunk table of an isolated ring evaluation (one group of N rings): the
// FP64 summation blocks, or the FP32 kernel's planned chunks.
static int ring_plan(int64_t N, int64_t M, int precision, Group& g, std::vector<Chunk>& ch) {
  g = Group{};
  g.rec_begin = 0;
  g.rec_count = (int)N;
  g.kind = 0;
  if (N <= 0) {
    ch.assign(1, Chunk{});
    return 0;
  }
  if (precision == VLM_PREC_FP64) {
    const int C = ring_chunk(N, M, precision);
    ch.assign((size_t)((N + C - 1) / C), Chunk{});
    return build_chunks(&g, 1, C, ch.data(), (int)ch.size());
  }
  ch.assign((size_t)std::min<int64_t>(N, 1 << 16) + 1, Chunk{});
  const int nq = plan_chunks32(&g, 1, (int)M, partial32_slots(), ch.data(), (int)ch.size());
  if (nq < 0) throw std::runtime_error("chunk table overflow");
  return nq;
}

static int64_t ring_near_cap(int64_t M) { return std::min<int64_t>(16 * M + (1 << 20), 1 << 27); }

int64_t ring_scratch_bytes(int64_t N, int64_t M, int precision) {
  Group g;
  std::vector<Chunk> ch;
  const int64_t Q = std::max(1, ring_plan(N, M, precision, g, ch));
  int64_t b = N * kRec64 * 8 + M * Q * 3 * 8 + Q * (int64_t)sizeof(Chunk) + 64;
  if (precision != VLM_PREC_FP64) b += N * kRec32 * 4;
  if (precision == VLM_PREC_FP32_NEAR64) b += ring_near_cap(M) * (int64_t)sizeof(NearPair) + M * Q * 3 * 8;
  return b;
}

int64_t ring_sum_chunk(int64_t N, int64_t M, int precision) {
  if (N <= 0) return 0;
  Group g;
  std::vector<Chunk> ch;
  const int nq = ring_plan(N, M, precision, g, ch);
  int64_t c = 0;
  for (int i = 0; i < nq; ++i) c = std::max<int64_t>(c, ch[i].rec_count);
  return c;
}

void rings_device(const double* corners, const double* rvc, const double* gam, int64_t N, const double* P, int64_t M,
                  double* V, int precision, cudaStream_t st) {
  if (precision < 0 || precision > 2) throw StatusError(VLM_ERR_INVALID, "precision must be 0, 1 or 2");
  if (N < 0 || M < 0 || N > (1LL << 30) || M > (1LL << 30)) throw StatusError(VLM_ERR_INVALID, "N and M must be in [0, 2^30]");
  if (M == 0) return;
  int dev = 0;
  VLM_CUDA(cudaGetDevice(&dev));
  RingScratch& R = g_ring[dev & 63];
  std::lock_guard<std::mutex> lock(R.mu);
  Group g;
  std::vector<Chunk> ch;
  const int nq = ring_plan(N, M, precision, g, ch);
  const int Q = std::max(nq, 1);
  grow((void**)&R.rec64, R.cap64, (size_t)std::max<int64_t>(N, 1) * kRec64 * 8);
  if (precision != VLM_PREC_FP64) grow((void**)&R.rec32, R.cap32, (size_t)std::max<int64_t>(N, 1) * kRec32 * 4);
  grow((void**)&R.part, R.capPart, (size_t)M * Q * 3 * 8);
  grow((void**)&R.chunks, R.capChunks, (size_t)Q * sizeof(Chunk) + sizeof(Group) + 64);
  R.group = reinterpret_cast<Group*>(R.chunks + Q);
  if (!R.err) VLM_CUDA(cudaMalloc(&R.err, 4 * sizeof(int)));
  const int nearCap = precision == VLM_PREC_FP32_NEAR64 ? (int)ring_near_cap(M) : 1;
  grow((void**)&R.near, R.capNear, (size_t)nearCap * sizeof(NearPair));
  if (precision == VLM_PREC_FP32_NEAR64 && (size_t)M * Q * 3 * 8 > R.capNacc) {
    grow((void**)&R.nacc, R.capNacc, (size_t)M * Q * 3 * 8);
    VLM_CUDA(cudaMemset(R.nacc, 0, R.capNacc));
  }
  // the tables are tiny; copy them synchronously with the stream so that the
  // caller's later reuse of the scratch is ordered after this launch
  VLM_CUDA(cudaMemcpyAsync(R.chunks, ch.data(), sizeof(Chunk) * std::max(nq, 1), cudaMemcpyHostToDevice, st));
  VLM_CUDA(cudaMemcpyAsync(R.group, &g, sizeof(Group), cudaMemcpyHostToDevice, st));
  VLM_CUDA(cudaMemsetAsync(R.err, 0, 4 * sizeof(int), st));
  if (N > 0) {
    launch_rings_to_rec64(corners, rvc, gam, N, R.rec64, st);
    if (precision == VLM_PREC_FP64) {
      launch_partial64(R.rec64, R.chunks, nq, P, (int)M, R.part, st);
    } else {
      const bool nearOn = precision == VLM_PREC_FP32_NEAR64;
      launch_pack32(R.rec64, (int)N, nearOn ? 4.0 : 0.0, R.rec32, st);
      launch_partial32(R.rec32, R.rec64, R.chunks, nq, P, (int)M, R.part, R.err, nearOn ? R.near : nullptr, nearCap,
                       R.nacc, st);
    }
    if (precision == VLM_PREC_FP64) launch_combine(R.part, (int)M, R.group, 1, 2, V, st);
    else launch_combine_unordered(R.part, (int)M, R.group, 1, nq, 2, V, st);
  } else {
    VLM_CUDA(cudaMemsetAsync(V, 0, (size_t)M * 3 * 8, st));
  }
  VLM_CUDA(cudaGetLastError());
  // the host-side tables above live on this stack frame and the scratch is
  // shared by every call on this device: finish before returning
  int ctl[2] = {0, 0};
  VLM_CUDA(cudaMemcpyAsync(ctl, R.err, sizeof(ctl), cudaMemcpyDeviceToHost, st));
  VLM_CUDA(cudaStreamSynchronize(st));
  if (ctl[0] == 3) throw StatusError(VLM_ERR_CUDA, "near-field pair list overflowed");
  if (ctl[0] == 4) throw StatusError(VLM_ERR_NONFINITE, "near-field velocity outside the fixed-point range");
  if (ctl[0]) throw StatusError(VLM_ERR_CUDA, "device wait limit expired in a Biot-Savart tile pipeline");
}

}  // namespace vlm

// ---------------------------------------------------------------------------
// C API
using namespace vlm;

struct vlm_case {
  Case c;
};

template <class F>
static int guard(F f) {
  try {
    f();
    return VLM_OK;
  } catch (const StatusError& e) {
    g_err = e.what();
    return e.code;
  } catch (const CudaError& e) {
    g_err = e.what();
    return VLM_ERR_CUDA;
  } catch (const std::bad_alloc&) {
    g_err = "host out of memory";
    return VLM_ERR_CUDA;
  } catch (const std::exception& e) {
    g_err = e.what();
    const std::string m = e.what();
    if (m.rfind("unsupported", 0) == 0) return VLM_ERR_UNSUPPORTED;
    if (m.find("cannot open") != std::string::npos) return VLM_ERR_IO;
    return VLM_ERR_INVALID;
  }
}

extern "C" {

const char* vlm_version(void) { return "vlm_gb300 0.1 (sm_103a)"; }

int vlm_last_error(char* buf, size_t len) {
  if (!buf || len == 0) return VLM_ERR_INVALID;
  std::snprintf(buf, len, "%s", g_err.c_str());
  return VLM_OK;
}

void vlm_default_options(vlm_options* o) {
  if (!o) return;
  o->precision = VLM_PREC_FP64;
  o->sum_chunk = 256;
  o->near_factor = 4.0;
  o->device = 0;
  o->use_graph = 1;
}

int vlm_device_info(int device, int* sm_count, int* cc_major, int* cc_minor) {
  return guard([&]() {
    cudaDeviceProp p;
    VLM_CUDA(cudaGetDeviceProperties(&p, device));
    if (sm_count) *sm_count = p.multiProcessorCount;
    if (cc_major) *cc_major = p.major;
    if (cc_minor) *cc_minor = p.minor;
  });
}

int vlm_biot_savart_rings_device(const double* corners, const double* rvc, const double* gam, int64_t N,
                                 const double* P, int64_t M, double* V, int precision, void* stream) {
  return guard([&]() { rings_device(corners, rvc, gam, N, P, M, V, precision, (cudaStream_t)stream); });
}

int64_t vlm_biot_savart_rings_scratch_bytes(int64_t N, int64_t M, int precision) {
  return ring_scratch_bytes(N, M, precision);
}

int64_t vlm_biot_savart_rings_sum_chunk(int64_t N, int64_t M, int precision) {
  return ring_sum_chunk(N, M, precision);
}

int vlm_biot_savart_rings(const double* corners, const double* rvc, const double* gam, int64_t N, const double* P,
                          int64_t M, double* V, int precision) {
  return guard([&]() {
    std::vector<void*> own;
    auto cleanup = [&]() {
      for (void* p : own) cudaFree(p);
    };
    try {
      double* dc = dalloc<double>((size_t)std::max<int64_t>(N, 1) * 12, own);
      double* dr = dalloc<double>((size_t)std::max<int64_t>(N, 1) * 4, own);
      double* dg = dalloc<double>((size_t)std::max<int64_t>(N, 1), own);
      double* dp = dalloc<double>((size_t)std::max<int64_t>(M, 1) * 3, own);
      double* dv = dalloc<double>((size_t)std::max<int64_t>(M, 1) * 3, own);
      if (N > 0) {
        VLM_CUDA(cudaMemcpy(dc, corners, (size_t)N * 12 * 8, cudaMemcpyHostToDevice));
        VLM_CUDA(cudaMemcpy(dr, rvc, (size_t)N * 4 * 8, cudaMemcpyHostToDevice));
        VLM_CUDA(cudaMemcpy(dg, gam, (size_t)N * 8, cudaMemcpyHostToDevice));
      }
      if (M > 0) VLM_CUDA(cudaMemcpy(dp, P, (size_t)M * 3 * 8, cudaMemcpyHostToDevice));
      rings_device(dc, dr, dg, N, dp, M, dv, precision, nullptr);
      if (M > 0) VLM_CUDA(cudaMemcpy(V, dv, (size_t)M * 3 * 8, cudaMemcpyDeviceToHost));
    } catch (...) {
      cleanup();
      throw;
    }
    cleanup();
  });
}

int vlm_case_create(const char* config_text, const char* geom_text, const char* base_dir, const vlm_options* opt,
                    vlm_case** out) {
  if (!out || !config_text || !geom_text) {
    g_err = "null argument";
    return VLM_ERR_INVALID;
  }
  *out = nullptr;
  auto c = std::make_unique<vlm_case>();
  const int rc = guard([&]() { c->c.create(config_text, geom_text, base_dir ? base_dir : "", opt); });
  if (rc == VLM_OK) *out = c.release();
  return rc;
}

int vlm_case_create_from_dir(const char* case_dir, const vlm_options* opt, vlm_case** out) {
  if (!case_dir) {
    g_err = "null case_dir";
    return VLM_ERR_INVALID;
  }
  std::string cfg, geo;
  const int rc = guard([&]() {
    auto rd = [](const std::string& p) {
      std::ifstream f(p);
      if (!f) throw std::runtime_error("cannot open " + p);
      std::stringstream ss;
      ss << f.rdbuf();
      return ss.str();
    };
    cfg = rd(std::string(case_dir) + "/config.nml");
    geo = rd(std::string(case_dir) + "/geom01.nml");
  });
  if (rc != VLM_OK) return rc;
  return vlm_case_create(cfg.c_str(), geo.c_str(), case_dir, opt, out);
}

int vlm_case_destroy(vlm_case* c) {
  delete c;
  return VLM_OK;
}

int vlm_case_start(vlm_case* c) {
  if (!c) return VLM_ERR_INVALID;
  return guard([&]() { c->c.start(); });
}

int vlm_case_step(vlm_case* c, int nsteps, double* ct_rows) {
  if (!c) return VLM_ERR_INVALID;
  return guard([&]() { c->c.step(nsteps, ct_rows); });
}

int vlm_case_get_int(vlm_case* c, const char* name, int64_t* value) {
  if (!c || !name || !value) return VLM_ERR_INVALID;
  const std::string k = name;
  const Case& C = c->c;
  const StepPlan& pl = C.plans[C.iter];
  if (k == "nt") *value = C.W.nt;
  else if (k == "nb") *value = C.d.nb;
  else if (k == "nc") *value = C.d.nc;
  else if (k == "ns") *value = C.d.ns;
  else if (k == "n") *value = C.d.n;
  else if (k == "nNwake") *value = C.d.NW;
  else if (k == "nFwake") *value = C.d.NF;
  else if (k == "rowNear") *value = pl.rowNear;
  else if (k == "rowFar") *value = pl.rowFar;
  else if (k == "iter") *value = C.iter;
  else if (k == "nbConvect") *value = C.d.nbC;
  else if (k == "wakeTruncateNt") *value = C.W.P.wakeTruncateNt;
  else if (k == "nearPairs" || k == "nodeChunks") {
    // near-field filament-target pairs of the last FP32 evaluation; chunks
    // of the next step's wake-node evaluation
    if (k == "nodeChunks") {
      *value = C.iter < C.W.nt ? C.plans[C.iter + 1].node.nchunks : 0;
    } else {
      int v = 0;
      if (cudaStreamSynchronize(C.stream) != cudaSuccess ||
          cudaMemcpy(&v, C.s.err + 3, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) {
        g_err = "cannot read the near-pair count";
        return VLM_ERR_CUDA;
      }
      *value = v;
    }
  } else {
    g_err = std::string("unknown integer ") + name;
    return VLM_ERR_INVALID;
  }
  return VLM_OK;
}

int64_t vlm_case_get(vlm_case* c, const char* name, int blade, double* out, int64_t cap) {
  if (!c || !name) return -1;
  int64_t n = -1;
  const int rc = guard([&]() { n = c->c.get(name, blade, out, cap); });
  return rc == VLM_OK ? n : -1;
}

int vlm_case_vind_points(vlm_case* c, const double* P, int64_t M, double* V) {
  if (!c || (M > 0 && (!P || !V))) return VLM_ERR_INVALID;
  return guard([&]() { c->c.vindPoints(P, M, V); });
}

int vlm_case_profile_eval(vlm_case* c, int reps, double* ms_per_launch, double* ring_pairs, double* fil_pairs) {
  if (!c || reps <= 0 || !ms_per_launch || !ring_pairs || !fil_pairs) return VLM_ERR_INVALID;
  return guard([&]() { c->c.profileEval(reps, ms_per_launch, ring_pairs, fil_pairs); });
}

int64_t vlm_kernel_launch_count(void) { return vlm::launch_count(); }

int vlm_case_last_step_ms(vlm_case* c, double* ms) {
  if (!c || !ms) return VLM_ERR_INVALID;
  *ms = c->c.lastMs;
  return VLM_OK;
}

}  // extern "C"
