// vlm_case: device state, per-step plans and the time loop of one rotor case,
// plus the extern "C" API declared in include/vlm.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/vlm.h"
#include "mlp.h"
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
  int maxq = 0;   // most chunks of one group
  int shape = 0;  // FP32 kernel tile shape (launch_partial32)
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
  bool ownStream = true;  // false for the rotors of a system after the first (one stream for all)
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // the loads (CT row) of a step only read the solution and feed no later
  // part of the step: they run on a side stream, joined at the step's end
  cudaStream_t side = nullptr;
  cudaEvent_t evFork = nullptr, evJoin = nullptr;
  // the near-field chain of an FP32 evaluation runs on its own stream
  // alongside the pair kernel (launch_partial32)
  NearOverlap nearOv{nullptr, nullptr, nullptr};
  bool loadsForked = false;
  std::vector<StepPlan> plans;  // index = iteration (0..nt)
  double* hFrames = nullptr;    // pinned host copy of every frame; uploaded per vlm_case_step call
  // per frame, per blade: the blade's yAxis[3] and secTauCapSpan[ns][3], which
  // only the sectional output (force2file) reads
  std::vector<double> secAxes;
  std::vector<Group> hGroups;
  std::vector<Chunk> hChunks;
  Group* dGroups = nullptr;
  Chunk* dChunks = nullptr;
  int iter = 0;
  bool started = false;
  int chunk64 = 0;
  int surrYoung = 0;  // youngest far-wake filaments per blade the surrogate leaves to the direct sum
  bool refine = false;  // FP32 LU + FP64 iterative refinement instead of the FP64 inverse
  int slots32 = 0;  // resident FP32-kernel blocks on the device (chunk planner input)
  double lastMs = 0;
  int maxTargets = 0, maxRecords = 0, maxChunks = 0;
  int64_t maxPart = 1;  // largest (chunks x targets) of any evaluation

  ~Case() {
    if (stream) cudaStreamSynchronize(stream);
    for (void* p : owned) cudaFree(p);
    for (void* p : scratchOwned) cudaFree(p);
    for (void* p : surrOwned) cudaFree(p);
    if (incrStream) cudaStreamSynchronize(incrStream);
    if (incrOv.stream) cudaStreamSynchronize(incrOv.stream);
    for (void* p : incrOwned) cudaFree(p);
    if (incrFork) cudaEventDestroy(incrFork);
    if (incrJoin) cudaEventDestroy(incrJoin);
    if (incrOv.fork) cudaEventDestroy(incrOv.fork);
    if (incrOv.join) cudaEventDestroy(incrOv.join);
    if (incrOv.stream) cudaStreamDestroy(incrOv.stream);
    if (incrStream) cudaStreamDestroy(incrStream);
    surr.net.destroy();
    if (gexec) cudaGraphExecDestroy(gexec);
    if (hIter) cudaFreeHost(hIter);
    if (hFrames) cudaFreeHost(hFrames);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (side) cudaStreamSynchronize(side);
    if (evFork) cudaEventDestroy(evFork);
    if (evJoin) cudaEventDestroy(evJoin);
    if (side) cudaStreamDestroy(side);
    if (nearOv.stream) cudaStreamSynchronize(nearOv.stream);
    if (nearOv.fork) cudaEventDestroy(nearOv.fork);
    if (nearOv.join) cudaEventDestroy(nearOv.join);
    if (nearOv.stream) cudaStreamDestroy(nearOv.stream);
    if (stream && ownStream) cudaStreamDestroy(stream);
  }

  // chunk table of one evaluation: the FP64 summation order, or the FP32
  // kernel's planned chunks for M targets
  int chunkTable(Group* g, int ng, int M, Chunk* out, int cap) const {
    if (opt.precision == VLM_PREC_FP64) return build_chunks(g, ng, chunk64, out, cap);
    return plan_chunks32(g, ng, M, slots32, out, cap);
  }

  // groups of one evaluation: wing sums (kind 0) for every blade when
  // withWing, then wake sums (kind 1) for every blade.  farMode 0: the whole
  // wake; 1: without the old far-wake filaments (all far-wake filaments but
  // the surrYoung youngest of each blade); 2: the old far-wake filaments alone.
  // force64: FP64 summation blocks whatever the case's precision.
  void addEval(EvalPlan& e, bool withWing, int rowNear, int rowFar, int M, int farMode = 0, bool force64 = false) {
    const int NW = d.NW, NF = d.NF, ns = d.ns;
    e = EvalPlan();
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
      const int nYoung = std::min(nFar, surrYoung);
      g.rec_begin = rec;
      g.rec_count = farMode == 0 ? nNear + hs + nFar + prescRecords(rowFar) : (farMode == 1 ? nNear + hs + nYoung : nFar - nYoung);
      g.kind = 1;
      g.blade = b;
      g.pad[0] = farMode == 2 ? 1 : 0;
      g.pad[1] = farMode == 2 ? nYoung : 0;
      rec += g.rec_count;
      hGroups.push_back(g);
    }
    e.ngroups = (int)hGroups.size() - e.goff;
    e.nrec = rec;
    e.coff = (int)hChunks.size();
    std::vector<Chunk> tmp(rec + e.ngroups + 1);
    const int nq = force64 ? build_chunks(hGroups.data() + e.goff, e.ngroups, chunk64, tmp.data(), (int)tmp.size())
                           : chunkTable(hGroups.data() + e.goff, e.ngroups, M, tmp.data(), (int)tmp.size());
    if (nq < 0) throw std::runtime_error("chunk table overflow");
    hChunks.insert(hChunks.end(), tmp.begin(), tmp.begin() + nq);
    e.nchunks = nq;
    for (int g = e.goff; g < e.goff + e.ngroups; ++g) e.maxq = std::max(e.maxq, hGroups[g].chunk_count);
    maxRecords = std::max(maxRecords, rec);
    maxChunks = std::max(maxChunks, nq);
    maxPart = std::max(maxPart, (int64_t)std::max(nq, 1) * M);
    maxTargets = std::max(maxTargets, M);
  }

  // prescribed far-wake filaments a blade's wake sum holds (summed, when the
  // case generates a prescribed wake, whenever the far wake exists)
  int prescRecords(int rowFar) const { return d.prescNt > 0 && rowFar <= d.NF ? kPresc : 0; }

  void create(const std::string& cfg, const std::string& geo, const std::string& base, const vlm_options* o,
              const Case* prevRotor = nullptr, bool asMember = false, cudaStream_t sharedStream = nullptr,
              const Case* imageSource = nullptr) {
    vlm_default_options(&opt);
    geomText = geo;
    imgSrc = imageSource;
    if (o) opt = *o;
    if (opt.precision < 0 || opt.precision > 2) throw StatusError(VLM_ERR_INVALID, "precision must be 0, 1 or 2");
    if (opt.solve_mode < -1 || opt.solve_mode > 1) throw StatusError(VLM_ERR_INVALID, "solve_mode must be -1, 0 or 1");
    refine = opt.solve_mode == 1 || (opt.solve_mode == -1 && opt.precision != VLM_PREC_FP64);
    chunk64 = opt.sum_chunk;
    member = asMember;
    if (imgSrc) W.loadImage(cfg, geo, imgSrc->geomText, base, prevRotor ? &prevRotor->W : nullptr, &imgSrc->W);
    else if (member) W.loadMember(cfg, geo, base, prevRotor ? &prevRotor->W : nullptr);
    else W.load(cfg, geo, base);
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
    d.prescNt = P.prescWakeNt;
    d.prescGenNt = P.prescWakeGenNt;
    d.skewLimit = P.skewLimit;
    d.chord = P.chord;
    d.forceCalc = P.forceCalcSwitch;
    d.velSound = W.velSound;
    d.fl = frame_layout(d.nb, d.nc, d.ns);
    if (d.nc > 64) throw StatusError(VLM_ERR_UNSUPPORTED, "nc > 64 chordwise panels");
    if (d.n > 8192) throw StatusError(VLM_ERR_UNSUPPORTED, "more than 8192 panels per rotor");
    const int nt = W.nt;

    VLM_CUDA(cudaSetDevice(opt.device));
    slots32 = opt.nbody_slots > 0 ? opt.nbody_slots : partial32_slots();
    if (sharedStream) {
      stream = sharedStream;
      ownStream = false;
    } else {
      VLM_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    }
    VLM_CUDA(cudaEventCreate(&ev0));
    VLM_CUDA(cudaEventCreate(&ev1));
    VLM_CUDA(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking));
    VLM_CUDA(cudaEventCreateWithFlags(&evFork, cudaEventDisableTiming));
    VLM_CUDA(cudaEventCreateWithFlags(&evJoin, cudaEventDisableTiming));
    VLM_CUDA(cudaStreamCreateWithFlags(&nearOv.stream, cudaStreamNonBlocking));
    VLM_CUDA(cudaEventCreateWithFlags(&nearOv.fork, cudaEventDisableTiming));
    VLM_CUDA(cudaEventCreateWithFlags(&nearOv.join, cudaEventDisableTiming));

    // frames: 0 = after the initial pitch, k = after the kinematics of step k
    std::vector<double> frames((size_t)(nt + 1) * d.fl.size);
    const size_t axStride = (size_t)d.nb * (3 + 3 * d.ns);
    secAxes.assign((size_t)(nt + 1) * axStride, 0.0);
    auto putAxes = [&](int k) {
      double* o = secAxes.data() + (size_t)k * axStride;
      for (int b = 0; b < d.nb; ++b) {
        const Blade& B = W.bl[b];
        *o++ = B.yA.x, *o++ = B.yA.y, *o++ = B.yA.z;
        for (int is = 0; is < d.ns; ++is) *o++ = B.secTauS[is].x, *o++ = B.secTauS[is].y, *o++ = B.secTauS[is].z;
      }
    };
    W.start_pitch();
    W.write_frame(frames.data());
    putAxes(0);
    for (int k = 1; k <= nt; ++k) {
      W.advance(k);
      W.write_frame(frames.data() + (size_t)k * d.fl.size);
      putAxes(k);
    }
    if (d.prescNt > 0) {
      if (d.NF < 2) throw StatusError(VLM_ERR_UNSUPPORTED, "a prescribed far wake needs at least 2 far-wake filaments");
      // classdef.f90:1009-1011, checked for every step that updates it
      for (int k = d.prescNt + 1; k <= nt; ++k) {
        const double* sh = frames.data() + (size_t)k * d.fl.size + d.fl.rot + 6;
        if (std::fabs(sh[0]) > kEps || std::fabs(sh[1]) > kEps)
          throw StatusError(VLM_ERR_UNSUPPORTED, "Prescribed far wake only implemented for shaft along Z-axis");
      }
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
    if (d.forceCalc == 1) {
      s.c81 = up(W.airfoils.data);
      s.c81Off = dalloc<int>(W.airfoils.offset.size(), owned);
      VLM_CUDA(cudaMemcpy(s.c81Off, W.airfoils.offset.data(), sizeof(int) * W.airfoils.offset.size(),
                          cudaMemcpyHostToDevice));
      s.airfoilNo = dalloc<int>(W.airfoilOfSection.size(), owned);
      VLM_CUDA(cudaMemcpy(s.airfoilNo, W.airfoilOfSection.data(), sizeof(int) * W.airfoilOfSection.size(),
                          cudaMemcpyHostToDevice));
    }
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
    if (d.prescNt > 0) {
      s.pfC = dalloc<double>((size_t)2 * nb * kPresc * 6, owned);
      s.pfGam = dalloc<double>((size_t)2 * nb, owned);
      s.pfRvc = dalloc<double>((size_t)2 * nb, owned);
      s.pfHelix = dalloc<double>((size_t)2 * nb * 2, owned);
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
    s.rotorLift = dalloc<double>(6, owned);
    s.ctHist = dalloc<double>((size_t)(nt + 1) * 10, owned);
    s.err = dalloc<int>(4, owned);
    s.devIter = dalloc<int>(1, owned);
    s.curFrame = dalloc<double>(d.fl.size, owned);
    VLM_CUDA(cudaMallocHost(&hIter, sizeof(int)));
    if (refine) {
      s.LU32 = dalloc<float>((size_t)d.n * d.n, owned);
      s.AICinv32 = dalloc<float>((size_t)d.n * d.n, owned);
      s.piv32 = dalloc<int>(d.n, owned);
      s.refX = dalloc<double>(d.n, owned);
      s.refR = dalloc<double>(d.n, owned);
      s.luRes = dalloc<double>(1, owned);
    }
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
    maxRecords = std::max(maxRecords, d.n);
    allocScratch();
  }

  // N-body scratch and plan tables (again after the surrogate adds plans)
  std::vector<void*> scratchOwned;
  void allocScratch() {
    for (void* p : scratchOwned) cudaFree(p);
    scratchOwned.clear();
    s.rec64 = dalloc<double>((size_t)maxRecords * kRec64, scratchOwned);
    s.rec32 = dalloc<float>((size_t)maxRecords * kRec32, scratchOwned);
    s.edgeW = lattice() ? dalloc<double>((size_t)maxRecords * 4, scratchOwned) : nullptr;
    s.targets = dalloc<double>((size_t)maxTargets * 3, scratchOwned);
    s.outv = dalloc<double>((size_t)maxTargets * 3, scratchOwned);
    s.part = dalloc<double>((size_t)maxPart * 3, scratchOwned);
    s.nearBytes = opt.precision == VLM_PREC_FP32_NEAR64 ? near_scratch_bytes(maxTargets, (size_t)256 * maxTargets) : 0;
    s.nearScratch = s.nearBytes ? dalloc<unsigned char>(s.nearBytes, scratchOwned) : nullptr;
    // zero here; every near-field evaluation leaves them zero
    s.nacc = dalloc<long long>(opt.precision == VLM_PREC_FP32_NEAR64 ? (size_t)maxPart * 3 : 1, scratchOwned);
    dGroups = dalloc<Group>(std::max<size_t>(hGroups.size(), 1), scratchOwned);
    dChunks = dalloc<Chunk>(std::max<size_t>(hChunks.size(), 1), scratchOwned);
    if (!hGroups.empty())
      VLM_CUDA(cudaMemcpy(dGroups, hGroups.data(), hGroups.size() * sizeof(Group), cudaMemcpyHostToDevice));
    if (!hChunks.empty())
      VLM_CUDA(cudaMemcpy(dChunks, hChunks.data(), hChunks.size() * sizeof(Chunk), cudaMemcpyHostToDevice));
  }

  const double* frame(int k) const { return s.frames + (size_t)k * d.fl.size; }
  // every entry point works on the case's own device, whatever is current
  void useDevice() const { VLM_CUDA(cudaSetDevice(opt.device)); }
  // the frame a step's kernels read: while a step is captured for replay, the
  // device-side current frame that launch_step_begin fills
  const double* stepFrame(int k) const { return replaying ? s.curFrame : frame(k); }

  // ---- CUDA-graph replay of steady-state steps ------------------------------
  // A step whose plan (near/far rows, chunk tables) and host-side branches
  // equal its predecessor's is captured once and replayed: the graph starts
  // with launch_step_begin (device step counter + 1, current frame copied in)
  // and its loads write the CT row of the device counter.
  bool replaying = false;
  cudaGraphExec_t gexec = nullptr;
  int graphRN = -1, graphRF = -1;
  long graphKernels = 0;
  int* hIter = nullptr;  // pinned source of the device step counter
  bool iterSynced = false;

  bool steadyStep(int k) const {
    if (!opt.use_graph || surr.on || k <= 3 || k <= W.sw.initWakeVelNt || W.sw.rotorForcePlot > 1) return false;
    // a burst every wakeBurst steps, a prescribed far wake from step prescNt + 1
    if (W.sw.wakeBurst != 0 || (d.prescNt > 0 && k <= d.prescNt + 1)) return false;
    return plans[k].rowNear == plans[k - 1].rowNear && plans[k].rowFar == plans[k - 1].rowFar;
  }

  void captureStep(int k) {
    if (gexec) cudaGraphExecDestroy(gexec);
    gexec = nullptr;
    cudaGraph_t g = nullptr;
    const long l0 = launch_count();
    VLM_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    replaying = true;
    try {
      launch_step_begin(d, s, stream);
      enqueueStep(k);
    } catch (...) {
      replaying = false;
      cudaStreamEndCapture(stream, &g);
      if (g) cudaGraphDestroy(g);
      throw;
    }
    replaying = false;
    VLM_CUDA(cudaStreamEndCapture(stream, &g));
    const cudaError_t e = cudaGraphInstantiate(&gexec, g, 0);
    cudaGraphDestroy(g);
    VLM_CUDA(e);
    graphKernels = launch_count() - l0;
    count_launches(-graphKernels);  // counted when replayed
    graphRN = plans[k].rowNear;
    graphRF = plans[k].rowFar;
  }

  void replayStep(int k) {
    if (!gexec || graphRN != plans[k].rowNear || graphRF != plans[k].rowFar) captureStep(k);
    if (!iterSynced) {
      *hIter = k - 1;
      VLM_CUDA(cudaMemcpyAsync(s.devIter, hIter, sizeof(int), cudaMemcpyHostToDevice, stream));
      iterSynced = true;
    }
    VLM_CUDA(cudaGraphLaunch(gexec, stream));
    count_launches(graphKernels);
  }

  // one Biot-Savart evaluation of plan e (its records already gathered) at the
  // M targets P into out; prec -1 = the case's precision
  void evaluate(const EvalPlan& e, int M, int mode, const double* P = nullptr, double* out = nullptr, int prec = -1,
                int nterms = 0) {
    if (!P) P = s.targets;
    if (!out) out = s.outv;
    if (prec < 0) prec = opt.precision;
    const Chunk* ch = dChunks + e.coff;
    if (prec == VLM_PREC_FP64) {
      launch_partial64(s.rec64, ch, e.nchunks, P, M, s.part, stream);
    } else {
      const bool nearOn = prec == VLM_PREC_FP32_NEAR64;
      launch_pack32(s.rec64, e.nrec, nearOn ? opt.near_factor : 0.0, s.rec32, stream, s.edgeW);
      VLM_CUDA(cudaMemsetAsync(s.err + 3, 0, sizeof(int), stream));
      launch_partial32(s.rec32, s.rec64, ch, e.nchunks, e.nrec, P, M, s.part, s.err + 2,
                       nearOn ? s.nearScratch : nullptr, s.nearBytes, s.nacc, stream, s.edgeW, e.shape,
                       opt.nbody_slots > 0 ? nullptr : &nearOv);  // a batch's cases already run side by side
    }
    if (e.nchunks == 0) {
      VLM_CUDA(cudaMemsetAsync(out, 0, sizeof(double) * 3 * (size_t)M * std::max(nterms, 1), stream));
      return;
    }
    if (nterms > 0)
      launch_combine_terms(s.part, M, dGroups + e.goff, e.ngroups, e.maxq, mode, prec == VLM_PREC_FP64, out, stream);
    else if (prec == VLM_PREC_FP64) launch_combine(s.part, M, dGroups + e.goff, e.ngroups, mode, out, stream);
    else launch_combine_unordered(s.part, M, dGroups + e.goff, e.ngroups, e.maxq, mode, out, stream);
  }

  // ---- autotuner of the FP32 N-body tile shape and chunking ----------------
  // The chunk planner's wave model (plan.cpp) picks a chunk count per
  // evaluation shape for tile shape 0.  At the first step whose (rowNear,
  // rowFar) signature repeats the previous step's -- the steady state that
  // every later step of a truncated wake repeats, and the one captured as a
  // graph -- the case times, on its live state, the wake-node and the
  // collocation-point evaluations for both tile shapes at the model's chunk
  // count and at 1/2, 3/4, 3/2 and 2 times it, then the best shape at +-1, 2
  // and 3 chunks of its best count (5 launches each after a warm one, CUDA
  // events), and keeps the fastest for every later step of that
  // signature if it beats the model's plan by more than 3 % (near ties keep
  // the model's plan, so that a choice does not flip with timing noise).
  // Only the FP32 pair kernel is timed (the near-field correction does not
  // depend on the chunking).  Decisions are kept for the process, keyed by
  // the device, precision, form and evaluation shape: every later case of
  // the same shape -- another run of the same case file, the step driven
  // phase by phase, a resumed checkpoint -- reuses them without timing, so
  // runs in one process give the same bits.  Results: vlm_case_get
  // "autotune"; vlm_case_set_tile fixes a plan instead.
  struct TuneResult {
    int rN = -1, rF = -1, candidates = 0;
    int shape[2] = {0, 0}, chunks[2] = {0, 0};  // [0] wake nodes, [1] collocation points
    double ms[2] = {0, 0}, modelMs[2] = {0, 0};
  };
  std::vector<TuneResult> tuned;
  bool tileForced = false;  // vlm_case_set_tile fixed the shape: no autotuning
  struct TileChoice {
    int shape = 0, n = 0;
    double ms = 0, modelMs = 0;
  };
  static std::mutex& tuneMutex() {
    static std::mutex m;
    return m;
  }
  static std::map<std::vector<int64_t>, TileChoice>& tuneCache() {
    static std::map<std::vector<int64_t>, TileChoice> c;
    return c;
  }
  // the (shape, n) table of evaluation `which` for every step from k on with
  // pl's signature
  void applyTile(int k, const StepPlan& pl, int which, const EvalPlan& e, int M, int shape, int n) {
    std::vector<Group> g(hGroups.begin() + e.goff, hGroups.begin() + e.goff + e.ngroups);
    const int cap = e.nrec + e.ngroups + 1;
    std::vector<Chunk> ch((size_t)cap);
    const int nq = build_chunks32(g.data(), e.ngroups, n, ch.data(), cap);
    if (nq < 0) throw std::runtime_error("chunk table overflow");
    const int off = (int)hChunks.size();
    hChunks.insert(hChunks.end(), ch.begin(), ch.begin() + nq);
    int maxq = 0;
    for (const Group& x : g) maxq = std::max(maxq, x.chunk_count);
    for (int kk = k; kk <= W.nt; ++kk) {
      StepPlan& p2 = plans[kk];
      if (p2.rowNear != pl.rowNear || p2.rowFar != pl.rowFar) continue;
      EvalPlan& e2 = which == 0 ? p2.node : p2.rhs;
      e2.shape = shape;
      e2.coff = off;
      e2.nchunks = nq;
      e2.maxq = maxq;
      for (int gi = 0; gi < e2.ngroups; ++gi) {
        hGroups[e2.goff + gi].chunk_begin = g[gi].chunk_begin;
        hGroups[e2.goff + gi].chunk_count = g[gi].chunk_count;
      }
    }
    maxChunks = std::max(maxChunks, nq);
    maxPart = std::max(maxPart, (int64_t)nq * M);
  }
  bool tuneOn() const {
    return opt.precision != VLM_PREC_FP64 && opt.nbody_slots <= 0 && !member && !surr.on && d.NW > 0 &&
           !tileForced;
  }
  // vlm_case_set_tile: every evaluation of the steps after the current one
  // re-planned with tile shape `shape` and `n` chunks for the largest group
  // (0: the wave model's count for that shape); shape -1 gives the choice back
  // to the autotuner (the wave model's plans for shape 0 until it runs)
  void setTile(int shape, int n) {
    useDevice();
    if (opt.precision == VLM_PREC_FP64) throw StatusError(VLM_ERR_INVALID, "tile shapes apply to the FP32 precisions");
    if (shape < -1 || shape >= kPartial32Shapes || n < 0)
      throw StatusError(VLM_ERR_INVALID, "shape must be -1 or 0.." + std::to_string(kPartial32Shapes - 1) +
                                             ", chunks >= 0");
    if (member || surr.on || opt.nbody_slots > 0)
      throw StatusError(VLM_ERR_UNSUPPORTED, "tile shapes are set on a lone case without the surrogate");
    VLM_CUDA(cudaStreamSynchronize(stream));
    const int sh = shape < 0 ? 0 : shape;
    for (int k = iter + 1; k <= W.nt; ++k)
      for (int which = 0; which < 2; ++which) {
        StepPlan& pl = plans[k];
        EvalPlan& e = which == 0 ? pl.node : pl.rhs;
        if (e.ngroups == 0) continue;
        const int M = which == 0 ? node_target_count(d, pl.rowNear, pl.rowFar) : d.nbC * d.npan;
        Group* g = hGroups.data() + e.goff;
        const int cap = e.nrec + e.ngroups + 1;
        const int nn = n > 0 ? n : plan_count32(g, e.ngroups, M, partial32_slots(sh), cap,
                                                partial32_targets_per_block(sh));
        std::vector<Chunk> ch((size_t)cap);
        const int nq = build_chunks32(g, e.ngroups, nn, ch.data(), cap);
        if (nq < 0) throw std::runtime_error("chunk table overflow");
        e.coff = (int)hChunks.size();
        hChunks.insert(hChunks.end(), ch.begin(), ch.begin() + nq);
        e.nchunks = nq;
        e.shape = sh;
        e.maxq = 0;
        for (int gi = 0; gi < e.ngroups; ++gi) e.maxq = std::max(e.maxq, g[gi].chunk_count);
        maxChunks = std::max(maxChunks, nq);
        maxPart = std::max(maxPart, (int64_t)std::max(nq, 1) * M);
      }
    tileForced = shape >= 0;
    tuned.clear();
    // a captured step graph holds the old tables
    if (gexec) {
      cudaGraphExecDestroy(gexec);
      gexec = nullptr;
    }
    allocScratch();
  }
  bool sigRepeats(int k) const {
    return k > 3 && plans[k].rowNear == plans[k - 1].rowNear && plans[k].rowFar == plans[k - 1].rowFar;
  }
  bool tunedFor(const StepPlan& pl) const {
    for (const TuneResult& t : tuned)
      if (t.rN == pl.rowNear && t.rF == pl.rowFar) return true;
    return false;
  }
  void autotune(int k) {
    useDevice();
    VLM_CUDA(cudaStreamSynchronize(stream));
    const StepPlan pl = plans[k];
    TuneResult tr;
    tr.rN = pl.rowNear;
    tr.rF = pl.rowFar;
    constexpr int kReps = 5;
    constexpr int64_t kMaxTunePart = (int64_t)1 << 22;  // (chunks x targets) of a candidate
    constexpr double kMargin = 0.97;                    // a plan must beat the model's by 3 %
    std::vector<void*> tmp;
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    VLM_CUDA(cudaEventCreate(&t0));
    VLM_CUDA(cudaEventCreate(&t1));
    bool changed = false;
    for (int which = 0; which < 2; ++which) {
      const EvalPlan e = which == 0 ? pl.node : pl.rhs;
      const int M = which == 0 ? node_target_count(d, pl.rowNear, pl.rowFar) : d.nbC * d.npan;
      if (M <= 0 || e.nrec <= 0) continue;
      std::vector<int64_t> key = {opt.device, opt.precision, lattice() ? 1 : 0, which, M, e.ngroups};
      for (int gi = 0; gi < e.ngroups; ++gi) key.push_back(hGroups[e.goff + gi].rec_count);
      int bestShape = 0, bestN = 0;
      double bestMs = 0.0, curMs = 0.0;
      {
        std::lock_guard<std::mutex> lk(tuneMutex());
        auto it = tuneCache().find(key);
        if (it != tuneCache().end()) {
          bestShape = it->second.shape;
          bestN = it->second.n;
          bestMs = it->second.ms;
          curMs = it->second.modelMs;
        }
      }
      if (bestN > 0) {
        applyTile(k, pl, which, e, M, bestShape, bestN);
        tr.shape[which] = bestShape;
        tr.chunks[which] = bestN;
        tr.ms[which] = bestMs;
        tr.modelMs[which] = curMs;
        changed = true;
        continue;
      }
      if (which == 0) launch_node_targets(d, s, pl.rowNear, pl.rowFar, false, s.targets, stream);
      else launch_cp_targets(d, frame(k), s.targets, stream);
      launch_gather(d, s, frame(k), dGroups + e.goff, e.ngroups, e.nrec, pl.rowNear, pl.rowFar, false, stream);
      launch_pack32(s.rec64, e.nrec, 0.0, s.rec32, stream, s.edgeW);
      std::vector<Group> g0(hGroups.begin() + e.goff, hGroups.begin() + e.goff + e.ngroups);
      const int cap = e.nrec + e.ngroups + 1;
      Chunk* dch = dalloc<Chunk>((size_t)cap, tmp);
      double* dpart = dalloc<double>((size_t)kMaxTunePart * 3, tmp);
      bestMs = 1e30;
      curMs = 1e30;
      int modelN = 0;  // the wave model's count for shape 0
      int maxRec = 0;
      for (const Group& g : g0) maxRec = std::max(maxRec, g.rec_count);
      std::vector<std::pair<int, int>> seen;
      // one candidate (tile shape, chunk count of the largest group) timed;
      // skipped when already timed or too large for the timing buffer
      auto timeOne = [&](int shape, int n) {
        n = std::min(n, std::max(1, maxRec));
        if (n < 1 || std::find(seen.begin(), seen.end(), std::make_pair(shape, n)) != seen.end()) return;
        seen.emplace_back(shape, n);
        std::vector<Group> g = g0;
        std::vector<Chunk> ch((size_t)cap);
        const int nq = build_chunks32(g.data(), e.ngroups, n, ch.data(), cap);
        if (nq <= 0 || (int64_t)nq * M > kMaxTunePart) return;
        VLM_CUDA(cudaMemcpyAsync(dch, ch.data(), sizeof(Chunk) * nq, cudaMemcpyHostToDevice, stream));
        auto launch = [&]() {
          launch_partial32(s.rec32, s.rec64, dch, nq, e.nrec, s.targets, M, dpart, s.err + 2, nullptr, 0, nullptr,
                           stream, s.edgeW, shape);
        };
        launch();
        VLM_CUDA(cudaEventRecord(t0, stream));
        for (int r = 0; r < kReps; ++r) launch();
        VLM_CUDA(cudaEventRecord(t1, stream));
        VLM_CUDA(cudaEventSynchronize(t1));
        float ms = 0.f;
        VLM_CUDA(cudaEventElapsedTime(&ms, t0, t1));
        const double per = ms / kReps;
        ++tr.candidates;
        if (shape == 0 && n == modelN) curMs = per;
        if (per < bestMs) {
          bestMs = per;
          bestShape = shape;
          bestN = n;
        }
      };
      modelN = plan_count32(g0.data(), e.ngroups, M, partial32_slots(0), cap, partial32_targets_per_block(0));
      // coarse: each shape at its wave model's count and 1/2, 3/4, 3/2, 2 x it
      for (int shape = 0; shape < kPartial32Shapes; ++shape) {
        const int n0 = plan_count32(g0.data(), e.ngroups, M, partial32_slots(shape), cap,
                                    partial32_targets_per_block(shape));
        for (int n : {n0, std::max(1, n0 / 2), std::max(1, 3 * n0 / 4), (3 * n0 + 1) / 2, 2 * n0}) timeOne(shape, n);
      }
      // fine: the best shape at +-1, 2, 3 chunks of its best count (the last
      // wave of blocks is what a chunk count moves)
      if (bestN > 0) {
        const int cs = bestShape, cn = bestN;
        for (int dn : {-3, -2, -1, 1, 2, 3}) timeOne(cs, cn + dn);
      }
      if (bestN <= 0) continue;
      // near ties keep the wave model's plan
      if (modelN > 0 && !(bestMs < kMargin * curMs)) {
        bestShape = 0;
        bestN = modelN;
        bestMs = curMs;
      }
      {
        std::lock_guard<std::mutex> lk(tuneMutex());
        tuneCache()[key] = TileChoice{bestShape, bestN, bestMs, curMs};
      }
      tr.shape[which] = bestShape;
      tr.chunks[which] = bestN;
      tr.ms[which] = bestMs;
      tr.modelMs[which] = curMs;
      applyTile(k, pl, which, e, M, bestShape, bestN);
      changed = true;
    }
    VLM_CUDA(cudaStreamSynchronize(stream));
    for (void* q : tmp) cudaFree(q);
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    // the timing launches wrote no state; the device error word of the
    // stream-ordered checks stays as it was (no near-field list was used)
    if (changed) allocScratch();
    tuned.push_back(tr);
  }

  // ---- incremental predicted-wake evaluation (incr.cu) ---------------------
  // The predictor of the Adams-Moulton / predictor-corrector schemes moves the
  // first near-wake node row (the reference's 'P' loop `do i = 1, rowNear,
  // nNwake`, src/classdef.f90:1549-1575) and the far wake; every other
  // record and target of the predicted-wake evaluation equals the
  // current-wake evaluation's of the same step.  On the FP32 precisions the
  // predicted-wake velocity is then the current-wake velocity (still in
  // s.outv) plus the changed records' new minus old contributions at every
  // target, and the full sum at the moved targets alone.  The changed records
  // and moved targets are found on the device by a bit-by-bit comparison
  // every step; their numbers, fixed by the wake's structure for a (rowNear,
  // rowFar) signature, are measured once -- at the case's first
  // predicted-wake evaluation of a signature that lasts at least kIncrMinRun
  // steps, never inside a captured graph (a host synchronisation) -- and size
  // the fixed-capacity buffers a captured step graph needs.  A signature whose
  // incremental work is not below half the full evaluation's keeps the full
  // evaluation.  The choice depends only on the case and the signature, so
  // runs resumed anywhere give the same bits.
  struct IncrPlan {
    int rN = 0, rF = 0;
    bool on = false;
    int nrec = 0, M = 0, changed = 0, moved = 0;
    int dcap = 0, mcap = 0;           // delta records (2 per changed record + inert), moved targets
    int dq = 0, dmaxq = 0, mq = 0, mmaxq = 0, mng = 0;
    Group *dG = nullptr, *mG = nullptr;
    Chunk *dC = nullptr, *mC = nullptr;
    double *dRec = nullptr, *dEw = nullptr, *outD = nullptr, *tPos = nullptr, *tOut = nullptr;
    double *dPart = nullptr, *mPart = nullptr;
    long long *dNacc = nullptr, *mNacc = nullptr;
    int* tIdx = nullptr;
    // the moved targets' evaluation runs beside the delta set's: its own
    // FP32 records, near-field scratch and streams
    float* mRec32 = nullptr;
    void* mNear = nullptr;
    size_t mNearBytes = 0;
  };
  static constexpr int kMaxIncrPlans = 8;
  std::vector<IncrPlan> incr;
  std::vector<void*> incrOwned;
  double *recP = nullptr, *ewP = nullptr, *tgtP = nullptr;  // the predicted records, edge weights, targets
  int* incrCnt = nullptr;                                   // [0] changed records, [1] moved targets
  int* incrBlk = nullptr;                                   // per-tile offsets: records, then targets
  cudaStream_t incrStream = nullptr;                        // the moved targets' evaluation
  NearOverlap incrOv{nullptr, nullptr, nullptr};            // its near-field chain
  cudaEvent_t incrFork = nullptr, incrJoin = nullptr;
  int* incrCtl = nullptr;  // the moved targets' evaluation's error code and near-pair cursor

  bool incrAllowed() const {
    return opt.incremental != 0 && opt.precision != VLM_PREC_FP64 && !member && !surr.on && d.NW > 0;
  }
  bool sameSig(int a, int b) const {
    return a >= 1 && b >= 1 && a <= W.nt && b <= W.nt && plans[a].rowNear == plans[b].rowNear &&
           plans[a].rowFar == plans[b].rowFar;
  }
  int incrIndex(int k) const {
    for (size_t i = 0; i < incr.size(); ++i)
      if (incr[i].rN == plans[k].rowNear && incr[i].rF == plans[k].rowFar) return (int)i;
    return -1;
  }
  // steps in the run of consecutive steps with step k's signature
  mutable std::vector<int> sigRunLen;
  int sigRun(int k) const {
    if (sigRunLen.empty()) {
      sigRunLen.assign((size_t)W.nt + 1, 0);
      for (int a = 1; a <= W.nt;) {
        int b = a;
        while (b + 1 <= W.nt && sameSig(a, b + 1)) ++b;
        for (int i = a; i <= b; ++i) sigRunLen[i] = b - a + 1;
        a = b + 1;
      }
    }
    return k >= 1 && k <= W.nt ? sigRunLen[k] : 0;
  }
  static constexpr int kIncrMinRun = 16;  // a signature worth a measurement lasts this many steps
  // step k's predicted-wake evaluation measures its signature first
  bool incrMeasureDue(int k) const {
    return incrAllowed() && predicts(k) && incrIndex(k) < 0 && (int)incr.size() < kMaxIncrPlans &&
           sigRun(k) >= kIncrMinRun;
  }
  void allocIncrBase() {
    if (recP) return;
    recP = dalloc<double>((size_t)maxRecords * kRec64, incrOwned);
    ewP = lattice() ? dalloc<double>((size_t)maxRecords * 4, incrOwned) : nullptr;
    tgtP = dalloc<double>((size_t)maxTargets * 3, incrOwned);
    incrCnt = dalloc<int>(2, incrOwned);
    incrCtl = dalloc<int>(2, incrOwned);
    incrBlk = dalloc<int>((size_t)incr_diff_blocks(maxRecords) + incr_diff_blocks(maxTargets) + 2, incrOwned);
    VLM_CUDA(cudaStreamCreateWithFlags(&incrStream, cudaStreamNonBlocking));
    VLM_CUDA(cudaStreamCreateWithFlags(&incrOv.stream, cudaStreamNonBlocking));
    VLM_CUDA(cudaEventCreateWithFlags(&incrOv.fork, cudaEventDisableTiming));
    VLM_CUDA(cudaEventCreateWithFlags(&incrOv.join, cudaEventDisableTiming));
    VLM_CUDA(cudaEventCreateWithFlags(&incrFork, cudaEventDisableTiming));
    VLM_CUDA(cudaEventCreateWithFlags(&incrJoin, cudaEventDisableTiming));
  }
  // the predicted targets and records beside the current ones, and the
  // comparison (counts and per-tile offsets)
  void incrDiff(int k, int M) {
    const StepPlan& pl = plans[k];
    const EvalPlan& e = pl.node;
    launch_node_targets(d, s, pl.rowNear, pl.rowFar, true, tgtP, stream);
    DevState sp = s;
    sp.rec64 = recP;
    sp.edgeW = s.edgeW ? ewP : nullptr;
    launch_gather(d, sp, stepFrame(k), dGroups + e.goff, e.ngroups, e.nrec, pl.rowNear, pl.rowFar, true, stream);
    launch_diff_count(recP, s.rec64, kRec64, sp.edgeW, s.edgeW, e.nrec, incrBlk, incrCnt, stream);
    launch_diff_count(tgtP, s.targets, 3, nullptr, nullptr, M, incrBlk + incr_diff_blocks(e.nrec), incrCnt + 1,
                      stream);
  }
  static int roundUp(int x, int m) { return (x + m - 1) / m * m; }
  void measureIncr(int k, int M) {
    const EvalPlan& e = plans[k].node;
    IncrPlan ip;
    ip.rN = plans[k].rowNear;
    ip.rF = plans[k].rowFar;
    ip.nrec = e.nrec;
    ip.M = M;
    if (M > 0 && e.nrec > 0) {
      allocIncrBase();
      incrDiff(k, M);
      int cnt[2] = {0, 0};
      VLM_CUDA(cudaMemcpyAsync(cnt, incrCnt, sizeof(cnt), cudaMemcpyDeviceToHost, stream));
      VLM_CUDA(cudaStreamSynchronize(stream));
      ip.changed = cnt[0];
      ip.moved = cnt[1];
      // slack for records or targets that happened not to move this step
      ip.dcap = 2 * roundUp(cnt[0] + cnt[0] / 32 + 16, 32);
      ip.mcap = roundUp(cnt[1] + cnt[1] / 32 + 16, 32);
      const double full = (double)e.nrec * M;
      const double inc = (double)ip.dcap * M + (double)e.nrec * ip.mcap + (double)(1 << 23);
      ip.on = ip.dcap <= e.nrec && ip.mcap < M && inc < 0.5 * full;
    }
    if (ip.on) buildIncr(ip, e);
    incr.push_back(ip);
  }
  void buildIncr(IncrPlan& ip, const EvalPlan& e) {
    const int slots = partial32_slots(0), tpb = partial32_targets_per_block(0);
    // the delta set: one wake group of dcap records at the M targets
    Group g{};
    g.rec_begin = 0;
    g.rec_count = ip.dcap;
    g.kind = 1;
    std::vector<Chunk> dch((size_t)ip.dcap + 2);
    const int dn = plan_count32(&g, 1, ip.M, slots, ip.dcap + 2, tpb);
    ip.dq = build_chunks32(&g, 1, std::max(dn, 1), dch.data(), ip.dcap + 2);
    ip.dmaxq = g.chunk_count;
    // the moved targets: the node evaluation's groups re-chunked for mcap targets
    std::vector<Group> mg(hGroups.begin() + e.goff, hGroups.begin() + e.goff + e.ngroups);
    const int mcapCh = e.nrec + e.ngroups + 1;
    std::vector<Chunk> mch((size_t)mcapCh);
    const int mn = plan_count32(mg.data(), e.ngroups, ip.mcap, slots, mcapCh, tpb);
    ip.mq = build_chunks32(mg.data(), e.ngroups, std::max(mn, 1), mch.data(), mcapCh);
    if (ip.dq <= 0 || ip.mq <= 0) throw std::runtime_error("chunk table overflow");
    ip.mng = e.ngroups;
    ip.mmaxq = 0;
    for (const Group& x : mg) ip.mmaxq = std::max(ip.mmaxq, x.chunk_count);
    ip.dG = dalloc<Group>(1, incrOwned);
    ip.dC = dalloc<Chunk>((size_t)ip.dq, incrOwned);
    ip.mG = dalloc<Group>((size_t)e.ngroups, incrOwned);
    ip.mC = dalloc<Chunk>((size_t)ip.mq, incrOwned);
    VLM_CUDA(cudaMemcpy(ip.dG, &g, sizeof(Group), cudaMemcpyHostToDevice));
    VLM_CUDA(cudaMemcpy(ip.dC, dch.data(), sizeof(Chunk) * ip.dq, cudaMemcpyHostToDevice));
    VLM_CUDA(cudaMemcpy(ip.mG, mg.data(), sizeof(Group) * e.ngroups, cudaMemcpyHostToDevice));
    VLM_CUDA(cudaMemcpy(ip.mC, mch.data(), sizeof(Chunk) * ip.mq, cudaMemcpyHostToDevice));
    ip.dRec = dalloc<double>((size_t)ip.dcap * kRec64, incrOwned);
    ip.dEw = lattice() ? dalloc<double>((size_t)ip.dcap * 4, incrOwned) : nullptr;
    ip.outD = dalloc<double>((size_t)ip.M * 3, incrOwned);
    ip.tIdx = dalloc<int>((size_t)ip.mcap, incrOwned);
    ip.tPos = dalloc<double>((size_t)ip.mcap * 3, incrOwned);
    ip.tOut = dalloc<double>((size_t)ip.mcap * 3, incrOwned);
    const bool nearOn = opt.precision == VLM_PREC_FP32_NEAR64;
    const size_t nd = (size_t)ip.dq * ip.M * 3, nm = (size_t)ip.mq * ip.mcap * 3;
    ip.dPart = dalloc<double>(nd, incrOwned);
    ip.mPart = dalloc<double>(nm, incrOwned);
    // zero (dalloc), and every near-field evaluation leaves them zero
    ip.dNacc = dalloc<long long>(nearOn ? nd : 1, incrOwned);
    ip.mNacc = dalloc<long long>(nearOn ? nm : 1, incrOwned);
    ip.mRec32 = dalloc<float>((size_t)ip.nrec * kRec32, incrOwned);
    ip.mNearBytes = nearOn ? near_scratch_bytes(ip.mcap, (size_t)256 * ip.mcap) : 0;
    ip.mNear = nearOn ? (void*)dalloc<unsigned char>(ip.mNearBytes, incrOwned) : nullptr;
  }
  // the predicted-wake velocities into s.outv, which holds the current-wake ones
  void evalPredIncr(int k, int M, const IncrPlan& ip) {
    const EvalPlan& e = plans[k].node;
    const bool nearOn = opt.precision == VLM_PREC_FP32_NEAR64;
    const double nf = nearOn ? opt.near_factor : 0.0;
    incrDiff(k, M);
    const double* ew = s.edgeW ? ewP : nullptr;
    launch_moved_targets(tgtP, s.targets, M, incrBlk + incr_diff_blocks(e.nrec), incrCnt + 1, ip.tIdx, ip.tPos,
                         ip.mcap, s.err + 2, stream);
    // every predicted record at the moved targets, on its own streams (a
    // batch's case on its own stream: the batch's cases already run side by side)
    const bool side = opt.nbody_slots <= 0;
    cudaStream_t ms = side ? incrStream : stream;
    if (side) {
      VLM_CUDA(cudaEventRecord(incrFork, stream));
      VLM_CUDA(cudaStreamWaitEvent(incrStream, incrFork, 0));
    }
    launch_pack32(recP, e.nrec, nf, ip.mRec32, ms, ew);
    VLM_CUDA(cudaMemsetAsync(incrCtl + 1, 0, sizeof(int), ms));
    launch_partial32(ip.mRec32, recP, ip.mC, ip.mq, e.nrec, ip.tPos, ip.mcap, ip.mPart, incrCtl, ip.mNear,
                     ip.mNearBytes, ip.mNacc, ms, ew, 0, side ? &incrOv : nullptr);
    launch_combine_unordered(ip.mPart, ip.mcap, ip.mG, ip.mng, ip.mmaxq, 0, ip.tOut, ms);
    if (side) VLM_CUDA(cudaEventRecord(incrJoin, incrStream));
    // the changed records (new +, old -) at every target: the current-wake
    // targets, whose near-field grid the current-wake evaluation left in the
    // scratch (the moved targets' results are replaced below)
    launch_delta_records(recP, s.rec64, ew, s.edgeW, e.nrec, incrBlk, incrCnt, ip.dRec, ip.dEw, ip.dcap, s.err + 2,
                         stream);
    launch_pack32(ip.dRec, ip.dcap, nf, s.rec32, stream, ip.dEw);
    VLM_CUDA(cudaMemsetAsync(s.err + 3, 0, sizeof(int), stream));
    launch_partial32(s.rec32, ip.dRec, ip.dC, ip.dq, ip.dcap, s.targets, M, ip.dPart, s.err + 2,
                     nearOn ? s.nearScratch : nullptr, s.nearBytes, ip.dNacc, stream, ip.dEw, 0,
                     side ? &nearOv : nullptr, true);
    launch_combine_unordered(ip.dPart, M, ip.dG, 1, ip.dmaxq, 0, ip.outD, stream);
    if (side) VLM_CUDA(cudaStreamWaitEvent(stream, incrJoin, 0));
    launch_incr_merge(s.outv, ip.outD, M, ip.tIdx, ip.tOut, incrCnt + 1, ip.mcap, incrCtl, s.err + 2, stream);
  }

  // ---- coupled rotors (nr > 1, vlm_system) ----------------------------------
  // Every rotor of a system is a Case on the system's one stream.  Its RHS
  // and wake-node evaluations sum the records of every rotor: each source
  // rotor's records are gathered from that rotor's state into a segment of
  // this rotor's record array, and the group table carries the per-rotor
  // sums (Group::term) in the reference's order (src/main.f90:549-561,
  // 817-826; libCommon.f90:114-211).
  bool member = false;
  int self = 0;
  std::vector<Case*> sys;
  std::string geomText;          // this rotor's geomXX.nml (an image of it reads its parameters)
  const Case* imgSrc = nullptr;  // an image rotor (surfaceType -1): the rotor it mirrors
  struct SysSeg {
    int jr = 0, lgoff = 0, lng = 0, nrec = 0, recOff = 0;  // source rotor, its local groups, records, offset
  };
  struct SysEval {
    EvalPlan e;
    int soff = 0, nseg = 0, nterms = 0;
  };
  std::vector<SysSeg> hSegs;
  std::vector<SysEval> sysRhs, sysNode;  // per iteration
  SysEval sysStart;                      // the initial solution: the other rotors' wings
  double* sysOut = nullptr;              // [term][collocation point][xyz]
  double* sysBound = nullptr;            // [rotor][collocation point][xyz] bound-vortex velocities
  int maxTerms = 1;

  // records of one blade's wake sum (the whole wake)
  int wakeRecords(int rowNear, int rowFar) const {
    const int nNear = (d.NW - (rowNear - 1)) * d.ns;
    const int hs = rowFar <= d.NF ? d.ns : 0;
    const int nFar = rowFar <= d.NF ? d.NF - rowFar + 1 : 0;
    return nNear + hs + nFar + prescRecords(rowFar);
  }

  // kind 0: the initial solution (main.f90:147-153: the other rotors' wings);
  // 1: the RHS of step k (every rotor's wake, then its wing unless it is this
  // rotor, one term each); 2: the wake nodes of step k (wing + wake of every
  // rotor, one term per rotor)
  void addSysEval(SysEval& se, int kind, int k, int M) {
    se = SysEval();
    se.soff = (int)hSegs.size();
    std::vector<Group> comb;
    int rec = 0, term = 0;
    for (int jr = 0; jr < (int)sys.size(); ++jr) {
      const Case& o = *sys[jr];
      const int rN = o.plans[k].rowNear, rF = o.plans[k].rowFar;
      std::vector<Group> loc;
      int lrec = 0;
      auto add = [&](int kindG, int t) {
        for (int b = 0; b < o.d.nb; ++b) {
          Group g{};
          g.rec_begin = lrec;
          g.rec_count = kindG == 0 ? o.d.npan : o.wakeRecords(rN, rF);
          g.kind = kindG;
          g.blade = b;
          g.term = t;
          lrec += g.rec_count;
          loc.push_back(g);
        }
      };
      if (kind == 0) {
        if (jr == self) continue;
        add(0, term++);
      } else if (kind == 1) {
        add(1, term++);
        if (jr != self) add(0, term++);
      } else {
        add(0, term);
        add(1, term);
        ++term;
      }
      SysSeg sg;
      sg.jr = jr;
      sg.lgoff = (int)hGroups.size();
      sg.lng = (int)loc.size();
      sg.nrec = lrec;
      sg.recOff = rec;
      hGroups.insert(hGroups.end(), loc.begin(), loc.end());
      hSegs.push_back(sg);
      for (Group g : loc) {
        g.rec_begin += rec;
        comb.push_back(g);
      }
      rec += lrec;
    }
    se.nseg = (int)hSegs.size() - se.soff;
    se.nterms = term;
    EvalPlan& e = se.e;
    e.goff = (int)hGroups.size();
    hGroups.insert(hGroups.end(), comb.begin(), comb.end());
    e.ngroups = (int)comb.size();
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
    maxPart = std::max(maxPart, (int64_t)std::max(nq, 1) * M);
    maxTargets = std::max(maxTargets, M);
    maxTerms = std::max(maxTerms, term);
  }

  // after every rotor of the system exists
  void buildSystemPlans() {
    const int nt = W.nt, Mcp = d.nbC * d.npan;
    sysRhs.assign(nt + 1, SysEval());
    sysNode.assign(nt + 1, SysEval());
    addSysEval(sysStart, 0, 0, Mcp);
    for (int k = 1; k <= nt; ++k) {
      addSysEval(sysRhs[k], 1, k, Mcp);
      addSysEval(sysNode[k], 2, k, node_target_count(d, plans[k].rowNear, plans[k].rowFar));
    }
    allocScratch();
    sysOut = dalloc<double>((size_t)maxTerms * Mcp * 3, owned);
    sysBound = dalloc<double>(sys.size() * (size_t)Mcp * 3, owned);
  }

  // the records of every source rotor at step k (frame fk), each from its own state
  void sysGather(const SysEval& se, int k, bool pred, int fk) {
    for (int i = 0; i < se.nseg; ++i) {
      const SysSeg& g = hSegs[se.soff + i];
      const Case& o = *sys[g.jr];
      DevState sj = o.s;
      sj.rec64 = s.rec64 + (size_t)g.recOff * kRec64;
      sj.edgeW = s.edgeW ? s.edgeW + 4 * (size_t)g.recOff : nullptr;
      launch_gather(o.d, sj, o.frame(fk), dGroups + g.lgoff, g.lng, g.nrec, o.plans[k].rowNear, o.plans[k].rowFar,
                    pred, stream);
    }
  }
  // velCP and the RHS at step k (frame k; k = 0: the initial solution)
  void sysRhsPhase(int k) {
    const SysEval& se = k == 0 ? sysStart : sysRhs[k];
    const int Mcp = d.nbC * d.npan;
    launch_cp_targets(d, frame(k), s.targets, stream);
    sysGather(se, k, false, k);
    evaluate(se.e, Mcp, 3, nullptr, sysOut, -1, se.nterms);
    launch_rhs_terms(d, s, frame(k), sysOut, se.nterms, stream);
  }
  // an image rotor's place in the RHS and solve loops (src/main.f90:584-598)
  void imageMirrorVelCP() { launch_mirror_velcp(d, s, imgSrc->s.velCP, W.P.imagePlane, stream); }
  void imageMirrorGamma() { launch_mirror_gamma(d, s, imgSrc->s.gamVec, stream); }
  // an image rotor's wake update (src/main.f90:844-1439): no velocities; the
  // source's wake mirrored where the source convects (its predicted wake at
  // the predictor, its current wake at the corrector), then every row at the
  // end of the step
  void imageWakeStage(int k, int st) {
    const StepPlan& pl = plans[k];
    const int plane = W.P.imagePlane;
    if (st == 1) {
      launch_mirror_wake(d, s, imgSrc->s, predicts(k) ? 1 : 0, pl.rowNear, pl.rowFar, plane, stream);
    } else if (st == 3) {
      if (predicts(k)) launch_mirror_wake(d, s, imgSrc->s, 0, pl.rowNear, pl.rowFar, plane, stream);
      launch_mirror_wake(d, s, imgSrc->s, 2, pl.rowNear, pl.rowFar, plane, stream);
    }
  }
  // the loads with every rotor's bound vortices (src/main.f90:632-652)
  void sysLoads(int k) {
    const int Mcp = d.nbC * d.npan;
    for (int jr = 0; jr < (int)sys.size(); ++jr)
      if (jr != self)
        launch_bound_foreign(d, frame(k), sys[jr]->d, sys[jr]->s, sys[jr]->frame(k), sysBound + 3 * (size_t)jr * Mcp,
                             stream);
    launch_loads(d, s, frame(k), chunk64, k, stream, sysBound, (int)sys.size(), self);
  }

  // ---- learned far-wake surrogate ----------------------------------------
  struct SurrPlans {
    EvalPlan rhsNoFar, nodeNoFar, farFar, farCollect, farAudit;
    int collectNodes = 0, collectStride = 1, auditNodes = 0, auditStride = 1;
  };
  struct Surrogate {
    vlm_surrogate_options o{};
    bool on = false;
    int phase = 0;  // VLM_SURR_WAIT / COLLECT / ACTIVE
    int collected = 0, startStep = 0;
    int64_t nsamp = 0, cap = 0;
    Mlp net;
    float *X = nullptr, *T = nullptr, *fX = nullptr, *fY = nullptr;
    double *sP = nullptr, *sV = nullptr, *outFar = nullptr, *farP = nullptr, *scale = nullptr, *audit = nullptr;
    double* desc = nullptr;  // coarse old-far-wake descriptor of the current evaluation
    double invR = 1.0;
    bool useNow = false;
    vlm_surrogate_stats st{};
  };
  Surrogate surr;
  std::vector<SurrPlans> splans;
  std::vector<void*> surrOwned;

  // lattice form of the near-wake rings for the FP32 precisions
  bool lattice() const { return opt.precision != VLM_PREC_FP64 && opt.lattice != 0; }

  int nearNodeCount(int rowNear) const { return d.nbC * (d.NW - (rowNear - 1)) * (d.ns + 1); }
  int farRows(int rowFar) const { return std::max(d.NF - (rowFar - 1), 0); }

  void setSurrogate(const vlm_surrogate_options& o) {
    useDevice();
    if (started) throw StatusError(VLM_ERR_STATE, "set the surrogate before vlm_case_start");
    if (!o.enable) {
      surr.on = false;
      return;
    }
    if (opt.precision == VLM_PREC_FP64) throw StatusError(VLM_ERR_INVALID, "the surrogate runs with the FP32 precisions only");
    if (d.NW == 0 || d.NF == 0) throw StatusError(VLM_ERR_UNSUPPORTED, "the surrogate needs a far wake");
    if (d.prescNt > 0) throw StatusError(VLM_ERR_UNSUPPORTED, "the surrogate with a prescribed far wake");
    if (o.collect_steps <= 0 || o.sample_stride <= 0 || o.train_iters < 0 || o.batch <= 0 || o.audit_samples <= 0 ||
        o.hidden <= 0 || o.hidden > 1024 || o.layers < 2 || o.layers > kMlpMaxLayers || !(o.audit_tol > 0.0) ||
        !(o.lr > 0.f))
      throw StatusError(VLM_ERR_INVALID, "invalid surrogate options");
    if (surr.on) throw StatusError(VLM_ERR_STATE, "the surrogate is already set");
    if (o.young_far < 0 || o.min_far <= 0) throw StatusError(VLM_ERR_INVALID, "invalid surrogate options");
    surr.o = o;
    surr.on = true;
    surrYoung = o.young_far;
    // per-step plans: the same evaluations without the far wake, the far
    // wake alone on the far-wake nodes, on the collection sample (FP32) and
    // on the audit sample (FP64, which decides the audit)
    splans.assign(W.nt + 1, SurrPlans());
    for (int k = 1; k <= W.nt; ++k) {
      const StepPlan& pl = plans[k];
      SurrPlans& sp = splans[k];
      const int rN = pl.rowNear, rF = pl.rowFar;
      const int rNprev = std::max(plans[k - 1].rowNear, 1);
      addEval(sp.rhsNoFar, false, rN, rF, d.nbC * d.npan, 1);
      addEval(sp.nodeNoFar, true, rN, rF, node_target_count(d, rN, rF), 1);
      addEval(sp.farFar, false, rN, rF, d.nbC * farRows(rF), 2);
      const int nodes = plans[k - 1].rowNear <= d.NW ? nearNodeCount(rNprev) : 0;
      sp.collectStride = o.sample_stride;
      sp.collectNodes = nodes / o.sample_stride;
      sp.auditStride = std::max(1, nodes / o.audit_samples);
      sp.auditNodes = nodes > 0 ? std::min(o.audit_samples, nodes) : 0;
      addEval(sp.farCollect, false, rN, rF, d.nbC * d.npan + sp.collectNodes, 2);
      addEval(sp.farAudit, false, rN, rF, d.nbC * d.npan + sp.auditNodes, 2, true);
    }
    allocScratch();
    // surrogate buffers
    int maxSample = 0, maxFar = 0;
    for (int k = 1; k <= W.nt; ++k) {
      maxSample = std::max(maxSample, d.nbC * d.npan + std::max(splans[k].collectNodes, splans[k].auditNodes));
      maxFar = std::max(maxFar, d.nbC * farRows(plans[k].rowFar));
    }
    int64_t perStep = d.nbC * d.npan;
    for (int k = 1; k <= W.nt; ++k) perStep = std::max<int64_t>(perStep, d.nbC * d.npan + splans[k].collectNodes);
    surr.cap = perStep * o.collect_steps;
    surr.X = dalloc<float>((size_t)surr.cap * kSurrFeatures, surrOwned);
    surr.T = dalloc<float>((size_t)surr.cap * 3, surrOwned);
    surr.fX = dalloc<float>((size_t)std::max(maxTargets, maxSample) * kSurrFeatures, surrOwned);
    surr.desc = dalloc<double>(4, surrOwned);
    surr.fY = dalloc<float>((size_t)std::max(maxTargets, maxSample) * 3, surrOwned);
    surr.sP = dalloc<double>((size_t)maxSample * 3, surrOwned);
    surr.sV = dalloc<double>((size_t)maxSample * 3, surrOwned);
    surr.outFar = dalloc<double>((size_t)std::max(maxFar, 1) * 3, surrOwned);
    surr.farP = dalloc<double>((size_t)std::max(maxFar, 1) * 3, surrOwned);
    surr.scale = dalloc<double>(1, surrOwned);
    surr.audit = dalloc<double>(2, surrOwned);
    std::vector<int> sizes(o.layers + 1, o.hidden);
    sizes.front() = kSurrFeatures;
    sizes.back() = 3;
    surr.net.create(sizes, o.seed, stream);
    surr.net.reserve(std::max(o.batch, 1 << 14));
    // length scale of the features: the farthest collocation point from the hub
    const double* f0 = hFrames;
    double r2 = 0.0;
    for (int b = 0; b < d.nb; ++b)
      for (int p = 0; p < d.npan; ++p) {
        const double* c = f0 + d.fl.pan + ((size_t)b * d.npan + p) * kPan + 12;
        const double* h = f0 + d.fl.rot + 3;
        const double dx = c[0] - h[0], dy = c[1] - h[1], dz = c[2] - h[2];
        r2 = std::max(r2, dx * dx + dy * dy + dz * dz);
      }
    surr.invR = r2 > 0.0 ? 1.0 / std::sqrt(r2) : 1.0;
    surr.phase = VLM_SURR_WAIT;
    surr.st = vlm_surrogate_stats{};
  }

  // old far-wake filaments per blade over their most
  double farFill(int rowFar) const {
    const int most = d.NF - surrYoung;
    return most > 0 ? (double)std::max(farRows(rowFar) - surrYoung, 0) / most : 0.0;
  }
  int youngAt(int k) const { return std::min(surrYoung, farRows(plans[k].rowFar)); }

  // direct far-wake velocity at the sample targets of step k's start state
  // (CPs at frame k-1 and every stride-th near-wake node from offset)
  int surrSample(int k, const EvalPlan& e, int nodes, int stride, int offset, int prec) {
    const int M = d.nbC * d.npan + nodes;
    const int rNprev = plans[k - 1].rowNear;
    launch_surr_targets(d, s, frame(k - 1), rNprev, plans[k].rowFar, 0, stride, offset, nodes, surr.sP, stream);
    launch_gather(d, s, frame(k - 1), dGroups + e.goff, e.ngroups, e.nrec, plans[k].rowNear, plans[k].rowFar, false,
                  stream);
    evaluate(e, M, 2, surr.sP, surr.sV, prec);
    launch_surr_features(d, s, frame(k - 1), surr.sP, M, surr.invR, farFill(plans[k].rowFar), plans[k].rowFar,
                         youngAt(k), false, surr.desc, surr.fX, stream);
    return M;
  }

  void surrTrain() {
    Surrogate& S = surr;
    const int64_t n = S.nsamp;
    constexpr int F = kSurrFeatures;
    std::vector<float> hX((size_t)n * F), hT((size_t)n * 3);
    VLM_CUDA(cudaMemcpyAsync(hX.data(), S.X, sizeof(float) * hX.size(), cudaMemcpyDeviceToHost, stream));
    VLM_CUDA(cudaMemcpyAsync(hT.data(), S.T, sizeof(float) * hT.size(), cudaMemcpyDeviceToHost, stream));
    VLM_CUDA(cudaStreamSynchronize(stream));
    double ss = 0.0;
    for (float t : hT) ss += (double)t * t;
    const double scale = std::sqrt(ss / std::max<size_t>(hT.size(), 1)) + 1e-30;
    // a seeded shuffle, then targets in units of the rms velocity
    std::vector<int64_t> idx((size_t)n);
    for (int64_t i = 0; i < n; ++i) idx[(size_t)i] = i;
    uint64_t r = S.o.seed * 0x9E3779B97F4A7C15ull + (uint64_t)S.st.trainings + 1;
    for (int64_t i = n - 1; i > 0; --i) {
      r ^= r << 13;
      r ^= r >> 7;
      r ^= r << 17;
      std::swap(idx[(size_t)i], idx[(size_t)(r % (uint64_t)(i + 1))]);
    }
    std::vector<float> sX((size_t)n * F), sT((size_t)n * 3);
    for (int64_t i = 0; i < n; ++i) {
      std::memcpy(&sX[(size_t)i * F], &hX[(size_t)idx[(size_t)i] * F], F * sizeof(float));
      for (int c = 0; c < 3; ++c) sT[(size_t)i * 3 + c] = (float)(hT[(size_t)idx[(size_t)i] * 3 + c] / scale);
    }
    VLM_CUDA(cudaMemcpyAsync(S.X, sX.data(), sizeof(float) * sX.size(), cudaMemcpyHostToDevice, stream));
    VLM_CUDA(cudaMemcpyAsync(S.T, sT.data(), sizeof(float) * sT.size(), cudaMemcpyHostToDevice, stream));
    VLM_CUDA(cudaMemcpyAsync(S.scale, &scale, sizeof(double), cudaMemcpyHostToDevice, stream));
    const int b = (int)std::min<int64_t>(S.o.batch, n);
    const int64_t nb = std::max<int64_t>(n / b, 1);
    for (int it = 0; it < S.o.train_iters; ++it) {
      const int64_t q = it % nb;
      S.net.grad(S.X + (size_t)q * b * kSurrFeatures, S.T + (size_t)q * b * 3, b);
      // the last third of the iterations at a fifth of the rate
      S.net.adam(it < (2 * S.o.train_iters) / 3 ? S.o.lr : 0.2f * S.o.lr);
    }
    VLM_CUDA(cudaGetLastError());
    float loss = 0.f;
    VLM_CUDA(cudaMemcpyAsync(&loss, S.net.loss, sizeof(float), cudaMemcpyDeviceToHost, stream));
    VLM_CUDA(cudaStreamSynchronize(stream));
    S.st.last_loss = loss;
    S.st.trainings += 1;
  }

  // the surrogate's work before step k: collect samples, train, or audit
  void surrPreStep(int k) {
    Surrogate& S = surr;
    S.useNow = false;
    const SurrPlans& sp = splans[k];
    const int rowsF = farRows(plans[k].rowFar);
    const int rowsOld = rowsF - youngAt(k);
    if (S.phase == VLM_SURR_WAIT && rowsOld >= S.o.min_far && sp.collectNodes > 0) {
      S.phase = VLM_SURR_COLLECT;
      S.collected = 0;
      S.nsamp = 0;
    }
    if (S.phase == VLM_SURR_COLLECT) {
      const int off = (int)((uint64_t)k * 2654435761ull % (uint64_t)sp.collectStride);
      const int M = surrSample(k, sp.farCollect, sp.collectNodes, sp.collectStride, off, opt.precision);
      const int n = (int)std::min<int64_t>(M, S.cap - S.nsamp);
      launch_surr_append(n, S.fX, S.sV, S.X + (size_t)S.nsamp * kSurrFeatures, S.T + (size_t)S.nsamp * 3, stream);
      S.nsamp += n;
      if (++S.collected >= S.o.collect_steps) {
        surrTrain();
        S.phase = VLM_SURR_ACTIVE;
      }
      S.st.samples = S.nsamp;
      return;
    }
    if (S.phase != VLM_SURR_ACTIVE || rowsOld <= 0) return;
    // audit: the network against the direct FP64 far-wake sum on a random sample
    const int off = (int)((uint64_t)k * 2246822519ull % (uint64_t)sp.auditStride);
    const int M = surrSample(k, sp.farAudit, sp.auditNodes, sp.auditStride, off, VLM_PREC_FP64);
    S.net.forward(S.fX, M, S.fY);
    launch_surr_audit(M, S.fY, S.scale, S.sV, S.audit, stream);
    double a[2] = {0.0, 0.0};
    VLM_CUDA(cudaMemcpyAsync(a, S.audit, sizeof(a), cudaMemcpyDeviceToHost, stream));
    VLM_CUDA(cudaStreamSynchronize(stream));
    const double e = std::sqrt(a[0] / std::max(a[1], 1e-300));
    S.st.audits += 1;
    S.st.last_audit_err = e;
    S.st.max_audit_err = std::max(S.st.max_audit_err, e);
    if (e <= S.o.audit_tol) {
      S.useNow = true;
      S.st.active_steps += 1;
    } else {
      // revert: this step sums the far wake directly; collect fresh data
      S.st.reverts += 1;
      S.phase = VLM_SURR_COLLECT;
      S.collected = 0;
      S.nsamp = 0;
    }
  }

  void evalNodes(int k, bool pred) {
    const StepPlan& pl = plans[k];
    const int M = node_target_count(d, pl.rowNear, pl.rowFar);
    if (pred && !replaying && incrMeasureDue(k)) measureIncr(k, M);
    const int ii = pred && incrAllowed() ? incrIndex(k) : -1;
    if (ii >= 0 && incr[ii].on) {
      evalPredIncr(k, M, incr[ii]);
    } else {
      evalNodesFull(k, pred, M);
    }
    const double iwv = k < W.sw.initWakeVelNt ? W.P.initWakeVel : 0.0;
    launch_scatter_nodes(d, s, stepFrame(k), pl.rowNear, pl.rowFar, pred, iwv, stream);
  }
  void evalNodesFull(int k, bool pred, int M) {
    const StepPlan& pl = plans[k];
    launch_node_targets(d, s, pl.rowNear, pl.rowFar, pred, s.targets, stream);
    if (member) {
      const SysEval& se = sysNode[k];
      sysGather(se, k, pred, k);
      evaluate(se.e, M, 0, nullptr, nullptr, -1, se.nterms);
    } else if (surr.on && surr.useNow) {
      // near-wake nodes: direct without the far wake + the network's far-wake
      // velocity; far-wake nodes: + the direct far-wake sum
      const SurrPlans& sp = splans[k];
      launch_gather(d, s, stepFrame(k), dGroups + sp.nodeNoFar.goff, sp.nodeNoFar.ngroups, sp.nodeNoFar.nrec, pl.rowNear,
                    pl.rowFar, pred, stream);
      evaluate(sp.nodeNoFar, M, 0);
      // every far-wake node, young or old, sums the old far wake directly
      const int Mf = d.nbC * farRows(pl.rowFar);
      launch_surr_far_targets(d, s, pl.rowFar, 0, pred, surr.farP, stream);
      launch_gather(d, s, stepFrame(k), dGroups + sp.farFar.goff, sp.farFar.ngroups, sp.farFar.nrec, pl.rowNear, pl.rowFar,
                    pred, stream);
      evaluate(sp.farFar, Mf, 2, surr.farP, surr.outFar);
      launch_surr_features(d, s, frame(pred ? k : k - 1), s.targets, M, surr.invR, farFill(pl.rowFar), pl.rowFar,
                           youngAt(k), pred, surr.desc, surr.fX, stream);
      surr.net.forward(surr.fX, M, surr.fY);
      launch_surr_merge_nodes(d, pl.rowNear, pl.rowFar, 0, M, surr.fY, surr.scale, surr.outFar, s.outv, stream);
    } else {
      launch_gather(d, s, stepFrame(k), dGroups + pl.node.goff, pl.node.ngroups, pl.node.nrec, pl.rowNear, pl.rowFar,
                    pred, stream);
      evaluate(pl.node, M, 0);
    }
  }

  // The AIC of the initial geometry, its FP64 LU and explicit inverse, the
  // inverse check, and (refined solves) its FP32 LU (src/main.f90:62-81:
  // rotor%calcAIC, inv2, isInverse).  Once per case.
  bool factored = false;
  void aicFactor() {
    useDevice();
    if (started) throw StatusError(VLM_ERR_STATE, "case already started");
    if (factored) return;
    launch_aic(d, s, frame(0), stream);
    launch_lu_inverse(d, s, stream);
    launch_is_inverse(d, s, stream);
    int err = 0;
    VLM_CUDA(cudaMemcpyAsync(&err, s.err, sizeof(int), cudaMemcpyDeviceToHost, stream));
    VLM_CUDA(cudaStreamSynchronize(stream));
    if (err == 10) throw StatusError(VLM_ERR_SINGULAR, "Matrix is numerically singular!");
    if (err == 11) throw StatusError(VLM_ERR_SINGULAR, "Computed AIC_inv does not seem to be correct within given tolerance");
    if (refine) launch_lu32(d, s, stream);
    VLM_CUDA(cudaGetLastError());
    factored = true;
  }

  void start() {
    useDevice();
    if (started) throw StatusError(VLM_ERR_STATE, "case already started");
    aicFactor();
    launch_solve(d, s, frame(0), false, stream);
    if (d.NW > 0) launch_shed(d, s, frame(0), d.NW + 1, false, stream);
    if (W.sw.rotorForcePlot != 0) launch_loads(d, s, frame(0), chunk64, 0, stream);
    VLM_CUDA(cudaGetLastError());
    VLM_CUDA(cudaStreamSynchronize(stream));
    iter = 0;
    started = true;
  }

  void enqueueStep(int k) {
    loadsForked = false;
    enqueueStepBody(k);
    if (loadsForked) VLM_CUDA(cudaStreamWaitEvent(stream, evJoin, 0));
  }

  void enqueueStepBody(int k) {
    enqueueSolvePhase(k);
    if (W.sw.rotorForcePlot != 0 && k % W.sw.rotorForcePlot == 0) {
      VLM_CUDA(cudaEventRecord(evFork, stream));
      VLM_CUDA(cudaStreamWaitEvent(side, evFork, 0));
      launch_loads(d, s, stepFrame(k), chunk64, replaying ? -1 : k, side);
      VLM_CUDA(cudaEventRecord(evJoin, side));
      loadsForked = true;
    }
    enqueueWakePhase(k);
  }

  // Phase 1 of step k (src/main.f90:466-603): shedding of the leading-edge
  // row, wake ageing and dissipation, the wake-induced velocity at the
  // collocation points, the RHS, the circulation solve.
  void enqueueSolvePhase(int k) {
    prePhase(k);
    const StepPlan& pl = plans[k];
    const int rN = pl.rowNear, rF = pl.rowFar;
    const double* fr = stepFrame(k);
    if (d.NW > 0) {
      const int Mcp = d.nbC * d.npan;
      launch_cp_targets(d, fr, s.targets, stream);
      if (surr.on && surr.useNow) {
        const EvalPlan& e = splans[k].rhsNoFar;
        launch_gather(d, s, fr, dGroups + e.goff, e.ngroups, e.nrec, rN, rF, false, stream);
        evaluate(e, Mcp, 1);
        launch_surr_features(d, s, frame(k - 1), s.targets, Mcp, surr.invR, farFill(rF), rF, youngAt(k), false,
                             surr.desc, surr.fX, stream);
        surr.net.forward(surr.fX, Mcp, surr.fY);
        launch_surr_add(Mcp, surr.fY, surr.scale, s.outv, stream);
      } else {
        launch_gather(d, s, fr, dGroups + pl.rhs.goff, pl.rhs.ngroups, pl.rhs.nrec, rN, rF, false, stream);
        evaluate(pl.rhs, Mcp, 1);
      }
      launch_solve(d, s, fr, true, stream);
    } else {
      launch_solve(d, s, fr, false, stream);
    }
  }

  // src/main.f90:464-490: leading-edge shed row, ageing, dissipation, burst
  void prePhase(int k) {
    const StepPlan& pl = plans[k];
    const int rN = pl.rowNear, rF = pl.rowFar;
    const double* fr = stepFrame(k);
    const bool wake = d.NW > 0 && W.sw.wakeSuppress == 0;
    if (wake) {
      launch_shed(d, s, fr, rN, true, stream);
      launch_age(d, s, rN, rF, stream);
      if (W.sw.wakeDissipation == 1) launch_dissipate(d, s, rN, rF, stream);
      if (W.sw.wakeBurst != 0 && k % W.sw.wakeBurst == 0) launch_burst(d, s, rF, stream);
    }
  }

  // rotor_convectwake (src/classdef.f90:4786-4830): shift + continuity +
  // axisymmetric copies, then the prescribed far wake once it is active
  void convect(int k, const double* fr, int rN, int rF, bool pred) {
    launch_convect(d, s, fr, rN, rF, pred, stream);
    if (d.prescNt > 0 && k > d.prescNt) launch_presc_update(d, s, fr, rF, pred, stream);
  }

  // Phase 3 of step k (src/main.f90:799-1439): wake-node velocities, the
  // finite-difference scheme (predictor, predicted-wake velocities,
  // corrector), strain, roll-up / far-wake shift, trailing-edge shedding.
  // (Phase 2, the loads, only reads the solution.)
  void enqueueWakePhase(int k) {
    const bool wake = d.NW > 0 && W.sw.wakeSuppress == 0;
    if (!wake) return;
    for (int st = 0; st < 4; ++st) wakeStage(k, st);
  }

  // whether step k's scheme evaluates the predicted wake
  bool predicts(int k) const {
    switch (W.sw.fdScheme) {
      case 1: return true;
      case 3: return k != 1;
      case 4: return k != 2;  // the reference tests iter == 0 for the start-up branch (never true)
      case 5: return k > 3;
      default: return false;
    }
  }

  // The wake update in four stages, so that coupled rotors run each stage for
  // every rotor before the next (the reference's do-ir loops): 0 the node
  // velocities, 1 the scheme up to the predicted wake (all of it when it has
  // none), 2 the predicted-wake velocities, 3 the corrector, strain, roll-up
  // / far-wake shift and the trailing-edge shed row.
  void wakeStage(int k, int st) {
    const StepPlan& pl = plans[k];
    const int rN = pl.rowNear, rF = pl.rowFar;
    const double* fr = stepFrame(k);
    if (st == 0) {
      evalNodes(k, false);
      return;
    }
    if (st == 2) {
      if (predicts(k)) evalNodes(k, true);
      return;
    }
    if (st == 1) {
      switch (W.sw.fdScheme) {
        case 0:
          convect(k, fr, rN, rF, false);
          break;
        case 1:
          launch_copy_predicted(d, s, rN, rF, stream);
          convect(k, fr, rN, rF, true);
          break;
        case 2:
          if (k == 1) {
            convect(k, fr, rN, rF, false);
            launch_velop(d, s, VOP_COPY_0_TO_1, stream);
          } else {
            launch_velop(d, s, VOP_AB2, stream);
            convect(k, fr, rN, rF, false);
          }
          break;
        case 3:
          if (k == 1) {
            convect(k, fr, rN, rF, false);
            launch_velop(d, s, VOP_COPY_0_TO_1, stream);
          } else {
            launch_copy_predicted(d, s, rN, rF, stream);
            launch_velop(d, s, VOP_AM2_PRED, stream);
            convect(k, fr, rN, rF, true);
          }
          break;
        case 4:
          if (k == 2) {
            convect(k, fr, rN, rF, false);
            launch_velop(d, s, VOP_COPY_0_TO_2, stream);
          } else {
            launch_copy_predicted(d, s, rN, rF, stream);
            launch_velop(d, s, VOP_AM3_PRED, stream);
            convect(k, fr, rN, rF, true);
          }
          break;
        case 5:
          if (k <= 3) {
            convect(k, fr, rN, rF, false);
            launch_velop(d, s, k == 1 ? VOP_COPY_0_TO_1 : (k == 2 ? VOP_COPY_0_TO_2 : VOP_COPY_0_TO_3), stream);
          } else {
            launch_copy_predicted(d, s, rN, rF, stream);
            launch_velop(d, s, VOP_AM4_PRED, stream);
            convect(k, fr, rN, rF, true);
          }
          break;
      }
      return;
    }
    if (predicts(k)) {
      switch (W.sw.fdScheme) {
        case 1:
          launch_order2(d, s, rN, rF, stream);
          convect(k, fr, rN, rF, false);
          break;
        case 3:
          launch_velop(d, s, VOP_AM2_CORR, stream);
          convect(k, fr, rN, rF, false);
          launch_velop(d, s, VOP_STEP_TO_1, stream);
          break;
        case 4:
          launch_velop(d, s, VOP_AM3_CORR, stream);
          convect(k, fr, rN, rF, false);
          launch_velop(d, s, VOP_AM3_SHIFT, stream);
          break;
        case 5:
          launch_velop(d, s, VOP_AM4_CORR, stream);
          convect(k, fr, rN, rF, false);
          launch_velop(d, s, VOP_AM4_SHIFT, stream);
          break;
      }
    }
    if (W.sw.wakeStrain == 1) launch_strain(d, s, rF, stream);
    if (rN == 1) launch_rollup(d, s, rF, stream);
    launch_shed(d, s, fr, rN, false, stream);
  }

  // ---- the time loop: inputs in, steps enqueued, results out ---------------
  void checkSteps(int nsteps) const {
    if (!started) throw StatusError(VLM_ERR_STATE, "vlm_case_start must be called before vlm_case_step");
    if (phase != 0) throw StatusError(VLM_ERR_STATE, "a step opened by vlm_case_solve_circulation is not finished");
    if (nsteps < 0 || iter + nsteps > W.nt)
      throw StatusError(VLM_ERR_INVALID, "nsteps runs past the case's nt timesteps");
  }
  // this call's inputs: the wing frames of its steps (host -> device)
  void uploadFrames(int nsteps) {
    if (nsteps > 0)
      VLM_CUDA(cudaMemcpyAsync(s.frames + (size_t)(iter + 1) * d.fl.size, hFrames + (size_t)(iter + 1) * d.fl.size,
                               sizeof(double) * d.fl.size * nsteps, cudaMemcpyHostToDevice, stream));
  }
  void enqueueOne(int k) {
    if (tuneOn() && sigRepeats(k) && !tunedFor(plans[k])) autotune(k);
    if (steadyStep(k) && !incrMeasureDue(k)) {
      replayStep(k);
      return;
    }
    iterSynced = false;
    if (surr.on) surrPreStep(k);
    enqueueStep(k);
  }
  // after the stream has run the steps: CT rows out, device error flags
  void finishSteps(int nsteps, double* ctRows) {
    if (ctRows && nsteps > 0)
      VLM_CUDA(cudaMemcpyAsync(ctRows, s.ctHist + (size_t)(iter + 1) * 10, sizeof(double) * 10 * nsteps,
                               cudaMemcpyDeviceToHost, stream));
    int errs[4] = {0, 0, 0, 0};
    VLM_CUDA(cudaMemcpyAsync(errs, s.err, sizeof(errs), cudaMemcpyDeviceToHost, stream));
    VLM_CUDA(cudaStreamSynchronize(stream));
    iter += nsteps;
    const int err = errs[2];
    if (err == 3) throw StatusError(VLM_ERR_CUDA, "near-field pair list overflowed");
    if (err == 4) throw StatusError(VLM_ERR_NONFINITE, "near-field velocity outside the fixed-point range");
    if (err == 5)
      throw StatusError(VLM_ERR_CUDA, "predicted wake: more changed records or moved targets than its plan holds");
    if (err) throw StatusError(VLM_ERR_CUDA, "device wait limit expired in a Biot-Savart tile pipeline");
    if (errs[1]) throw StatusError(VLM_ERR_SINGULAR, "FP32 LU iterative refinement left a relative residual above 1e-9");
    if (ctRows)
      for (int k = 0; k < 10 * nsteps; ++k)
        if (!std::isfinite(ctRows[k])) throw StatusError(VLM_ERR_NONFINITE, "non-finite load in the CT history");
  }

  void step(int nsteps, double* ctRows) {
    useDevice();
    checkSteps(nsteps);
    uploadFrames(nsteps);
    VLM_CUDA(cudaEventRecord(ev0, stream));
    for (int k = iter + 1; k <= iter + nsteps; ++k) enqueueOne(k);
    VLM_CUDA(cudaEventRecord(ev1, stream));
    VLM_CUDA(cudaGetLastError());
    VLM_CUDA(cudaEventSynchronize(ev1));
    float ms = 0.f;
    VLM_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
    lastMs = ms;
    finishSteps(nsteps, ctRows);
  }

  // ---- the step as three calls (a host that drives its own time loop) -------
  // phase: 0 between steps; 1 after the circulation solve of step iter + 1;
  // 2 after its loads.  The three phases enqueue exactly the kernels of
  // vlm_case_step in the same order on the case stream (the loads on the
  // stream itself instead of the side stream: they only read the solution),
  // so the results are the same bits.
  int phase = 0;
  void phaseSolve(const double* kinVel, double* gamOut) {
    useDevice();
    if (phase != 0) throw StatusError(VLM_ERR_STATE, "step already open: finish it with vlm_case_wake_step");
    checkSteps(1);
    const int k = iter + 1;
    double* hf = hFrames + (size_t)k * d.fl.size;
    if (kinVel) {
      // the caller's kinematic velocity at the collocation points replaces the
      // frame's (same panel order as the reference's RHS rows)
      for (int p = 0; p < d.nb * d.npan; ++p)
        for (int a = 0; a < 3; ++a) hf[d.fl.pan + (size_t)p * kPan + 24 + a] = kinVel[3 * (size_t)p + a];
    }
    uploadFrames(1);
    iterSynced = false;
    if (tuneOn() && sigRepeats(k) && !tunedFor(plans[k])) autotune(k);
    if (surr.on) surrPreStep(k);
    enqueueSolvePhase(k);
    VLM_CUDA(cudaGetLastError());
    if (gamOut) VLM_CUDA(cudaMemcpyAsync(gamOut, s.gamVec, sizeof(double) * d.n, cudaMemcpyDeviceToHost, stream));
    VLM_CUDA(cudaStreamSynchronize(stream));
    int errs[4] = {0, 0, 0, 0};
    VLM_CUDA(cudaMemcpy(errs, s.err, sizeof(errs), cudaMemcpyDeviceToHost));
    if (errs[1]) throw StatusError(VLM_ERR_SINGULAR, "FP32 LU iterative refinement left a relative residual above 1e-9");
    if (gamOut)
      for (int i = 0; i < d.n; ++i)
        if (!std::isfinite(gamOut[i])) throw StatusError(VLM_ERR_NONFINITE, "non-finite circulation");
    phase = 1;
  }
  void phaseLoads(double* row) {
    useDevice();
    if (phase != 1) throw StatusError(VLM_ERR_STATE, "vlm_case_loads needs a solved step (vlm_case_solve_circulation)");
    const int k = iter + 1;
    launch_loads(d, s, frame(k), chunk64, k, stream);
    VLM_CUDA(cudaGetLastError());
    double r[10];
    VLM_CUDA(cudaMemcpyAsync(r, s.ctHist + (size_t)k * 10, sizeof(r), cudaMemcpyDeviceToHost, stream));
    VLM_CUDA(cudaStreamSynchronize(stream));
    for (double x : r)
      if (!std::isfinite(x)) throw StatusError(VLM_ERR_NONFINITE, "non-finite load in the CT row");
    if (row) std::memcpy(row, r, sizeof(r));
    phase = 2;
  }
  void phaseWake() {
    useDevice();
    if (phase == 0) throw StatusError(VLM_ERR_STATE, "vlm_case_wake_step needs a solved step (vlm_case_solve_circulation)");
    const int k = iter + 1;
    enqueueWakePhase(k);
    VLM_CUDA(cudaGetLastError());
    phase = 0;
    finishSteps(1, nullptr);
  }

  // ---- checkpoint / resume (the reference's Restart/restartNNNNN.dat:
  // src/main.f90:389-397 reads t and the rotor object, :1443-1450 writes
  // them every restartWriteNt steps) -------------------------------------------
  // the solver state (all FP64) and, last, the FP32 factors of the refined
  // solve (present when `refined`)
  std::vector<std::pair<void*, size_t>> stateArrays(bool refined) {
    const size_t nb = d.nb, npan = d.npan, n = d.n, ns = d.ns;
    const size_t nring = nb * std::max(d.NW, 1) * ns, nfar = nb * std::max(d.NF, 1), nsec = nb * ns;
    const size_t D = sizeof(double);
    std::vector<std::pair<void*, size_t>> v = {
        {s.wGam, nb * npan * D},   {s.gamPrev, nb * npan * D},     {s.gamVec, n * D},
        {s.gamVecPrev, n * D},     {s.RHS, n * D},                 {s.velCP, 3 * nb * npan * D},
        {s.velCPTotal, 3 * nb * npan * D}, {s.AIC, n * n * D},     {s.AICinv, n * n * D},
        {s.LU, n * n * D},         {s.piv, n * sizeof(int)},       {s.nC, nring * 12 * D},
        {s.nCP, nring * 12 * D},   {s.nGam, nring * D},            {s.nRvc, nring * 4 * D},
        {s.nAge, nring * D},       {s.fC, nfar * 6 * D},           {s.fCP, nfar * 6 * D},
        {s.fGam, nfar * D},        {s.fRvc, nfar * D},             {s.fRvc0, nfar * D},
        {s.fL0, nfar * D},         {s.fLc, nfar * D},              {s.fAge, nfar * D},
        {s.secResVel, 3 * nsec * D}, {s.secLiftDir, 3 * nsec * D}, {s.secDragDir, 3 * nsec * D},
        {s.secLift, 3 * nsec * D}, {s.secForceInertial, 3 * nsec * D}, {s.secLiftUnsteady, 3 * nsec * D},
        {s.secLiftInPlane, 3 * nsec * D}, {s.secLiftOutPlane, 3 * nsec * D}, {s.secCL, nsec * D},
        {s.secCD, nsec * D},       {s.secCLu, nsec * D},           {s.bladeForce, nb * 12 * D},
        {s.rotorLift, 6 * D},      {s.ctHist, (size_t)(W.nt + 1) * 10 * D}};
    for (int k = 0; k < 7; ++k) {
      v.push_back({s.vN[k], nb * std::max(d.NW, 1) * (ns + 1) * 3 * D});
      v.push_back({s.vF[k], nfar * 3 * D});
    }
    if (s.pfC) {
      v.push_back({s.pfC, 2 * nb * kPresc * 6 * D});
      v.push_back({s.pfGam, 2 * nb * D});
      v.push_back({s.pfRvc, 2 * nb * D});
      v.push_back({s.pfHelix, 2 * nb * 2 * D});
    }
    if (refined) {
      v.push_back({s.LU32, n * n * sizeof(float)});
      v.push_back({s.AICinv32, n * n * sizeof(float)});
      v.push_back({s.piv32, n * sizeof(int)});
      v.push_back({s.luRes, D});
    }
    return v;
  }
  static constexpr uint64_t kCkptMagic = 0x3254504b434d4c56ull;  // "VLMCKPT2"
  std::vector<int64_t> ckptHeader() const {
    return {(int64_t)kCkptMagic, iter, d.nb, d.nc, d.ns, d.NW, d.NF, W.nt, opt.precision, opt.sum_chunk,
            refine ? 1 : 0};
  }

  void checkpointSave(const std::string& path) {
    useDevice();
    if (!started) throw StatusError(VLM_ERR_STATE, "checkpoint before vlm_case_start");
    // a case with the surrogate saves its flow state; the network and the
    // surrogate's phase are not part of a checkpoint
    VLM_CUDA(cudaStreamSynchronize(stream));
    std::ofstream f(path, std::ios::binary);
    if (!f) throw StatusError(VLM_ERR_IO, "cannot open " + path);
    const auto h = ckptHeader();
    const int64_t nh = (int64_t)h.size();
    f.write(reinterpret_cast<const char*>(&nh), sizeof(nh));
    f.write(reinterpret_cast<const char*>(h.data()), sizeof(int64_t) * h.size());
    std::vector<char> buf;
    for (auto& a : stateArrays(refine)) {
      buf.resize(a.second);
      VLM_CUDA(cudaMemcpy(buf.data(), a.first, a.second, cudaMemcpyDeviceToHost));
      const int64_t nb = (int64_t)a.second;
      f.write(reinterpret_cast<const char*>(&nb), sizeof(nb));
      f.write(buf.data(), (std::streamsize)buf.size());
    }
    if (!f) throw StatusError(VLM_ERR_IO, "write failed: " + path);
  }

  void checkpointLoad(const std::string& path) {
    useDevice();
    if (surr.on) throw StatusError(VLM_ERR_UNSUPPORTED, "checkpoints of a case with the surrogate");
    std::ifstream f(path, std::ios::binary);
    if (!f) throw StatusError(VLM_ERR_IO, "cannot open " + path);
    int64_t nh = 0;
    f.read(reinterpret_cast<char*>(&nh), sizeof(nh));
    auto mine = ckptHeader();
    if (!f || nh != (int64_t)mine.size()) throw StatusError(VLM_ERR_INVALID, "not a checkpoint of this format: " + path);
    std::vector<int64_t> h((size_t)nh);
    f.read(reinterpret_cast<char*>(h.data()), sizeof(int64_t) * nh);
    if (!f || h[0] != (int64_t)kCkptMagic) throw StatusError(VLM_ERR_INVALID, "not a checkpoint: " + path);
    // the case's dimensions must agree; the arithmetic options (precision,
    // summation blocks, solve mode) may differ: the state is FP64 in every
    // precision, so a state saved by one precision continues in another
    for (size_t i = 2; i <= 7; ++i)
      if (h[i] != mine[i]) throw StatusError(VLM_ERR_INVALID, "checkpoint of a different case: " + path);
    if (h[1] < 0 || h[1] > W.nt) throw StatusError(VLM_ERR_INVALID, "checkpoint step out of range");
    const bool fileRefined = h[10] != 0;
    VLM_CUDA(cudaStreamSynchronize(stream));
    std::vector<char> buf;
    // (the FP32 factors of a case that does not refine are not allocated:
    // only their sizes are used, to read past them)
    const auto arrays = stateArrays(true);
    const size_t common = stateArrays(false).size();
    const size_t nread = fileRefined ? arrays.size() : common;
    for (size_t i = 0; i < nread; ++i) {
      const auto& a = arrays[i];
      int64_t nb = 0;
      f.read(reinterpret_cast<char*>(&nb), sizeof(nb));
      if (!f || nb != (int64_t)a.second) throw StatusError(VLM_ERR_INVALID, "checkpoint arrays do not match: " + path);
      buf.resize(a.second);
      f.read(buf.data(), (std::streamsize)buf.size());
      if (!f) throw StatusError(VLM_ERR_IO, "truncated checkpoint: " + path);
      // the FP32 factors only matter to a case that refines
      if (i < common || refine) VLM_CUDA(cudaMemcpy(a.first, buf.data(), a.second, cudaMemcpyHostToDevice));
    }
    // a refining case restored from a state without FP32 factors factors the
    // restored AIC itself (the same FP32 LU its start would have made)
    if (refine && !fileRefined) {
      launch_lu32(d, s, stream);
      VLM_CUDA(cudaGetLastError());
      VLM_CUDA(cudaStreamSynchronize(stream));
    }
    // the frame of the restored step (later steps upload their own)
    iter = (int)h[1];
    factored = true;
    phase = 0;
    VLM_CUDA(cudaMemcpy(s.frames + (size_t)iter * d.fl.size, hFrames + (size_t)iter * d.fl.size,
                        sizeof(double) * d.fl.size, cudaMemcpyHostToDevice));
    started = true;
    iterSynced = false;
  }

  // Times the partial-sum kernel of the next step's wake-node evaluation on
  // the current state (reps launches between CUDA events); reports the mean
  // launch time and the ring / single-filament pair counts of one launch.
  double profileWork[2] = {0.0, 0.0};  // executed flops, filament-target evaluations of the last profileEval
  void profileEval(int reps, double* msPerLaunch, double* ringPairs, double* filPairs) {
    useDevice();
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
    if (opt.precision != VLM_PREC_FP64) launch_pack32(s.rec64, pl.node.nrec, nf, s.rec32, stream, s.edgeW);
    // the work the FP32 kernel executes per target (9 flop per corner vector,
    // 35 per filament): a whole ring 4 + 4; a lattice-form record 3 corners
    // and edges 0, 1, plus corner c3 and edges 2 / 3 where they carry
    // circulation
    profileWork[0] = profileWork[1] = 0.0;
    if (opt.precision != VLM_PREC_FP64) {
      double corners = 4.0 * pl.node.nrec, fils = 4.0 * pl.node.nrec;
      if (s.edgeW) {
        const auto ew = dget(s.edgeW, (size_t)pl.node.nrec * 4);
        corners = fils = 0.0;
        for (int r = 0; r < pl.node.nrec; ++r) {
          const bool t2 = ew[4 * r + 2] != 0.0, t3 = ew[4 * r + 3] != 0.0;
          corners += (t2 || t3) ? 4.0 : 3.0;
          fils += 2.0 + (t2 ? 1.0 : 0.0) + (t3 ? 1.0 : 0.0);
        }
      }
      profileWork[0] = (9.0 * corners + 35.0 * fils) * M;
      profileWork[1] = fils * M;
    }
    auto launch = [&]() {
      if (opt.precision == VLM_PREC_FP64) launch_partial64(s.rec64, ch, pl.node.nchunks, s.targets, M, s.part, stream);
      else {
        VLM_CUDA(cudaMemsetAsync(s.err + 3, 0, sizeof(int), stream));
        launch_partial32(s.rec32, s.rec64, ch, pl.node.nchunks, pl.node.nrec, s.targets, M, s.part, s.err + 2,
                         opt.precision == VLM_PREC_FP32_NEAR64 ? s.nearScratch : nullptr, s.nearBytes, s.nacc,
                         stream, s.edgeW, pl.node.shape, &nearOv);
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
    if (pl.rowFar <= d.NF) fils += (long)d.nb * (d.ns + d.NF - pl.rowFar + 1 + prescRecords(pl.rowFar));
    *ringPairs = (double)rings * M;
    *filPairs = (double)fils * M;
  }

  std::vector<double> dget(const double* p, size_t n) {
    std::vector<double> h(n);
    VLM_CUDA(cudaStreamSynchronize(stream));
    if (n) VLM_CUDA(cudaMemcpy(h.data(), p, n * sizeof(double), cudaMemcpyDeviceToHost));
    return h;
  }

  // getAngleTan (src/libMath.f90:224-236)
  static double angleTan(d3 a, d3 b) {
    const double ma = sumsq3(a), mb = sumsq3(b), dd = dot3(a, b);
    return std::atan2(std::sqrt(ma * mb - dd * dd), dd);
  }

  // The sixteen per-section columns force2file writes to
  // rXXbYYForceDistNNNNN.csv (src/libPostprocess.f90:850-878) for the current
  // iteration, with the angles of blade_calc_secAlpha
  // (src/classdef.f90:2234-2265) evaluated here from the device's sectional
  // resultant velocity and the host's copy of the step's kinematics.  Row
  // major: ns rows of secSpan secCL secCD secCLu secLift secDrag secLiftInPl
  // secLiftOutPl secArea secVel secChord secTheta secAlpha secPhi secViz secVix.
  std::vector<double> forceDist(int b) {
    const size_t ns = d.ns, off = (size_t)b * ns;
    const auto rv = dget(s.secResVel + 3 * off, 3 * ns), lift = dget(s.secLift + 3 * off, 3 * ns);
    const auto inP = dget(s.secLiftInPlane + 3 * off, 3 * ns), outP = dget(s.secLiftOutPlane + 3 * off, 3 * ns);
    const auto cl = dget(s.secCL + off, ns), cd = dget(s.secCD + off, ns), clu = dget(s.secCLu + off, ns);
    const double* fr = hFrames + (size_t)iter * d.fl.size;
    const double* ax = secAxes.data() + (size_t)iter * d.nb * (3 + 3 * ns) + (size_t)b * (3 + 3 * ns);
    auto at = [](const double* p) { return mk3(p[0], p[1], p[2]); };
    const d3 hub = at(fr + d.fl.rot + 3), zAF = at(fr + d.fl.ax + 9 * b + 6), yAxis = at(ax);
    const Blade& B = W.bl[b];
    std::vector<double> v;
    v.reserve(16 * ns);
    for (size_t is = 0; is < ns; ++is) {
      const double* sec = fr + d.fl.sec + (off + is) * kSec;
      const d3 tauC = at(sec), normal = at(sec + 3), secCP = at(sec + 6), tauS = at(ax + 3 + 3 * is);
      const d3 velCPm = at(fr + d.fl.pan + ((size_t)b * d.npan + is * d.nc) * kPan + 24);  // panel (1, is)
      const d3 r = at(rv.data() + 3 * is);
      const double alpha = std::atan2(dot3(r, normal), dot3(r, tauC));
      const double phi = angleTan(r, noproj3(velCPm, tauS));
      const d3 vi = r - velCPm;
      const double vix = norm3(noproj3(vi, tauS) - mk3(0.0, 0.0, vi.z));
      const double theta = kPi * 0.5 - angleTan(neg3(tauC), zAF);
      const double row[16] = {dot3(secCP - hub, yAxis), cl[is], cd[is], clu[is], norm3(at(lift.data() + 3 * is)),
                              norm3(zero3()), norm3(at(inP.data() + 3 * is)), norm3(at(outP.data() + 3 * is)),
                              B.secArea[is], norm3(r), B.secChord[is], theta * kRad2Deg, alpha * kRad2Deg,
                              phi * kRad2Deg, vi.z, vix};
      v.insert(v.end(), row, row + 16);
    }
    return v;
  }

  // The eleven values force2file writes to rXXForceDim.csv after the
  // iteration (src/libPostprocess.f90:840-846): |lift|, |drag|, lift, drag,
  // forceInertial.  Drag is zero for the circulation-based loads
  // (blade_calc_force_gamma, src/classdef.f90:1704-1896).
  std::vector<double> forceDim() {
    const auto lf = dget(s.rotorLift, 6);
    const d3 L = mk3(lf[0], lf[1], lf[2]);
    return {norm3(L), norm3(zero3()), L.x, L.y, L.z, 0.0, 0.0, 0.0, lf[3], lf[4], lf[5]};
  }

  int64_t get(const std::string& k, int blade, double* out, int64_t cap) {
    useDevice();
    std::vector<double> v;
    const int b = blade - 1;
    const bool bok = b >= 0 && b < d.nb;
    const size_t npan = d.npan, NW = d.NW, NF = d.NF, ns = d.ns;
    if (k == "dt") v = {W.dt};
    else if (k == "Omega") v = {d.omega};
    else if (k == "theta0") v = {d.theta0};
    else if (k == "lu_residual") v = refine ? dget(s.luRes, 1) : std::vector<double>{0.0};
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
    else if (bok && k == "waF_rvc0") v = dget(s.fRvc0 + b * NF, NF);
    else if (bok && k == "waF_l0") v = dget(s.fL0 + b * NF, NF);
    else if (bok && k == "waF_lc") v = dget(s.fLc + b * NF, NF);
    else if (bok && k == "waF_age") v = dget(s.fAge + b * NF, NF);
    else if (bok && k == "waN_age") v = dget(s.nAge + b * NW * ns, NW * ns);
    else if (bok && k == "vr_rvc") v = dget(s.wRvc + 4 * b * npan, 4 * npan);
    else if (bok && k == "velN") v = dget(s.vN[0] + 3 * b * NW * (ns + 1), 3 * NW * (ns + 1));
    else if (bok && k == "velF") v = dget(s.vF[0] + 3 * b * NF, 3 * NF);
    else if (bok && (k == "velN1" || k == "velN2" || k == "velN3"))
      v = dget(s.vN[k[4] - '0'] + 3 * b * NW * (ns + 1), 3 * NW * (ns + 1));
    else if (bok && (k == "velF1" || k == "velF2" || k == "velF3")) v = dget(s.vF[k[4] - '0'] + 3 * b * NF, 3 * NF);
    else if (bok && k == "gamPrev") v = dget(s.gamPrev + b * npan, npan);
    else if (k == "hub" || (bok && (k == "yAxis" || k == "secCP"))) {
      // kinematics of the current iteration (of the open step between its phases)
      const int fi = phase != 0 ? iter + 1 : iter;
      const double* f = hFrames + (size_t)fi * d.fl.size;
      if (k == "hub") v.assign(f + d.fl.rot + 3, f + d.fl.rot + 6);
      else if (k == "yAxis") {
        const double* ax = secAxes.data() + (size_t)fi * d.nb * (3 + 3 * ns) + (size_t)b * (3 + 3 * ns);
        v.assign(ax, ax + 3);
      } else {
        for (size_t is = 0; is < ns; ++is) {
          const double* sec = f + d.fl.sec + ((size_t)b * ns + is) * kSec + 6;
          v.insert(v.end(), sec, sec + 3);
        }
      }
    }
    else if (bok && s.pfC && k == "waP") v = dget(s.pfC + (size_t)b * kPresc * 6, (size_t)kPresc * 6);
    else if (bok && s.pfC && k == "waP_gam") v = dget(s.pfGam + b, 1);
    else if (bok && s.pfC && k == "waP_rvc") v = dget(s.pfRvc + b, 1);
    else if (bok && k == "velKin") {
      // the prescribed kinematic velocity at the collocation points of the
      // current iteration (of the open step between its phases)
      const double* f = hFrames + (size_t)(phase != 0 ? iter + 1 : iter) * d.fl.size;
      for (size_t q = 0; q < npan; ++q) {
        const double* r = f + d.fl.pan + (b * npan + q) * kPan + 24;
        v.insert(v.end(), r, r + 3);
      }
    }
    else if (bok && k == "secCL") v = dget(s.secCL + b * ns, ns);
    else if (bok && k == "secLiftDir") v = dget(s.secLiftDir + 3 * b * ns, 3 * ns);
    else if (bok && k == "secChordwiseResVel") v = dget(s.secResVel + 3 * b * ns, 3 * ns);
    else if (bok && k == "secLift") v = dget(s.secLift + 3 * b * ns, 3 * ns);
    else if (bok && b < d.nbC && k == "forceDist") v = forceDist(b);
    else if (k == "forceDim") v = forceDim();
    else if (k == "profileWork") v = {profileWork[0], profileWork[1]};
    else if (k == "incremental") {
      // per measured signature: rowNear, rowFar, used (0/1), changed records,
      // moved targets, record capacity, target capacity, records, targets
      for (const IncrPlan& ip : incr)
        v.insert(v.end(), {(double)ip.rN, (double)ip.rF, ip.on ? 1.0 : 0.0, (double)ip.changed, (double)ip.moved,
                           (double)ip.dcap, (double)ip.mcap, (double)ip.nrec, (double)ip.M});
    }
    else if (k == "autotune") {
      // per tuned signature: rowNear, rowFar, candidates timed, then for the
      // wake nodes and the collocation points: shape, chunk count of the
      // largest group, ms per launch of the choice, ms of the planner's plan
      for (const TuneResult& t : tuned) {
        v.insert(v.end(), {(double)t.rN, (double)t.rF, (double)t.candidates});
        for (int w = 0; w < 2; ++w) v.insert(v.end(), {(double)t.shape[w], (double)t.chunks[w], t.ms[w], t.modelMs[w]});
      }
    }
    else if (bok && (k == "CP" || k == "nCap" || k == "vr")) {
      // the wing of the current iteration (of the open step between its phases)
      auto f = dget(frame(phase != 0 ? iter + 1 : iter), d.fl.size);
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
    useDevice();
    if (!started) throw StatusError(VLM_ERR_STATE, "vlm_case_start must be called first");
    if (M <= 0) return;
    // groups of the current state: wing + wake at the current rows (of the
    // open step between its phases)
    const int fi = phase != 0 ? iter + 1 : iter;
    const StepPlan& pl = plans[std::max(fi, 1)];
    const int rN = fi == 0 ? d.NW + 1 : pl.rowNear, rF = fi == 0 ? d.NF + 1 : pl.rowFar;
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
        q.rec_count = nNear + hs + nFar + prescRecords(rF);
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
      t.edgeW = nullptr;  // ring by ring: the probe's record count is not the plans'
      launch_gather(d, t, frame(fi), dg, (int)g.size(), rec, rN, rF, false, stream);
      if (opt.precision == VLM_PREC_FP64) {
        launch_partial64(rec64, dc, nq, dP, (int)M, part, stream);
      } else {
        const bool nearOn = opt.precision == VLM_PREC_FP32_NEAR64;
        launch_pack32(rec64, rec, nearOn ? opt.near_factor : 0.0, rec32, stream);
        const size_t nb = nearOn ? near_scratch_bytes((int)M, (size_t)std::min<int64_t>(64 * M + (1 << 16), 1 << 26)) : 1;
        unsigned char* ns = dalloc<unsigned char>(nb, tmpOwned);
        long long* nacc = dalloc<long long>(nearOn ? (size_t)M * nq * 3 : 1, tmpOwned);
        VLM_CUDA(cudaMemsetAsync(s.err + 3, 0, sizeof(int), stream));
        launch_partial32(rec32, rec64, dc, nq, rec, dP, (int)M, part, s.err + 2, nearOn ? ns : nullptr, nb, nacc,
                         stream);
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
  unsigned char* near = nullptr;
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
  const int64_t want = 4 * (int64_t)device_sm_count();
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


// near-pair list capacity of an isolated evaluation at M targets
static size_t ring_near_cap(int64_t M) { return (size_t)std::min<int64_t>(16 * M + (1 << 20), 1 << 27); }

int64_t ring_scratch_bytes(int64_t N, int64_t M, int precision) {
  Group g;
  std::vector<Chunk> ch;
  const int64_t Q = std::max(1, ring_plan(N, M, precision, g, ch));
  int64_t b = N * kRec64 * 8 + M * Q * 3 * 8 + Q * (int64_t)sizeof(Chunk) + 64;
  if (precision != VLM_PREC_FP64) b += N * kRec32 * 4;
  if (precision == VLM_PREC_FP32_NEAR64) b += (int64_t)near_scratch_bytes((int)M, ring_near_cap(M)) + M * Q * 3 * 8;
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

// fil: the sources are single filaments (corners = N x [fc1, fc2], rvc and
// gam one per filament) instead of rings.
void rings_device(const double* corners, const double* rvc, const double* gam, int64_t N, const double* P, int64_t M,
                  double* V, int precision, cudaStream_t st, bool fil = false) {
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
  const size_t nearBytes = precision == VLM_PREC_FP32_NEAR64 ? near_scratch_bytes((int)M, ring_near_cap(M)) : 1;
  grow((void**)&R.near, R.capNear, nearBytes);
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
    if (fil) launch_fils_to_rec64(corners, rvc, gam, N, R.rec64, st);
    else launch_rings_to_rec64(corners, rvc, gam, N, R.rec64, st);
    if (precision == VLM_PREC_FP64) {
      launch_partial64(R.rec64, R.chunks, nq, P, (int)M, R.part, st);
    } else {
      const bool nearOn = precision == VLM_PREC_FP32_NEAR64;
      launch_pack32(R.rec64, (int)N, nearOn ? 4.0 : 0.0, R.rec32, st);
      launch_partial32(R.rec32, R.rec64, R.chunks, nq, (int)N, P, (int)M, R.part, R.err, nearOn ? R.near : nullptr,
                       nearBytes,
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

// Coupled rotors (nr > 1): rotor(1..nr) of src/main.f90, each a Case on one
// stream, advanced with every do-ir loop of the reference's iteration run
// over the rotors in turn (src/main.f90:400-1452).
struct vlm_system {
  std::vector<std::unique_ptr<vlm_case>> r;
  int iter = 0;
  bool started = false;
  double lastMs = 0;

  Case& rotor(int i) { return r[i]->c; }
  cudaStream_t stream() { return r[0]->c.stream; }
  // rotor 0 owns the stream the others use: release them first
  ~vlm_system() {
    while (!r.empty()) r.pop_back();
  }

  void create(const std::string& cfg, const std::vector<std::string>& geoms, const std::string& base,
              const vlm_options* o) {
    const int nr = (int)geoms.size();
    if (nr < 1) throw StatusError(VLM_ERR_INVALID, "a system needs at least one rotor");
    for (int ir = 0; ir < nr; ++ir) {
      Namelist g;
      g.parse(geoms[ir]);
      const int st = g.i("SURFACE", "surfaceType");
      const Case* src = nullptr;
      if (st < 0) {
        const int sr = g.i("SURFACE", "imageRotorNum");
        if (sr < 1 || sr > ir || rotor(sr - 1).imgSrc)
          throw StatusError(VLM_ERR_UNSUPPORTED, "unsupported: an image rotor must mirror an earlier lifting rotor");
        src = &rotor(sr - 1);
      }
      auto c = std::make_unique<vlm_case>();
      c->c.create(cfg, geoms[ir], base, o, ir ? &rotor(ir - 1) : nullptr, true, ir ? stream() : nullptr, src);
      if (c->c.W.nr != nr)
        throw StatusError(VLM_ERR_INVALID, "config.nml nr = " + std::to_string(c->c.W.nr) + " but " +
                                               std::to_string(nr) + " rotor geometries");
      if (c->c.d.NW <= 0) throw StatusError(VLM_ERR_UNSUPPORTED, "unsupported: a rotor of a system without a wake");
      r.push_back(std::move(c));
    }
    std::vector<Case*> all;
    for (auto& c : r) all.push_back(&c->c);
    for (int ir = 0; ir < nr; ++ir) {
      rotor(ir).sys = all;
      rotor(ir).self = ir;
    }
    for (int ir = 0; ir < nr; ++ir) rotor(ir).buildSystemPlans();
  }

  // src/main.f90:43-377: pitch, AIC, the initial solution with the other
  // rotors' wings, the first shed row and the loads of iteration 0
  void start() {
    if (started) throw StatusError(VLM_ERR_STATE, "system already started");
    for (auto& c : r)
      if (!c->c.imgSrc) c->c.aicFactor();
    cudaStream_t st = stream();
    for (auto& c : r) {
      if (c->c.imgSrc) c->c.imageMirrorVelCP();
      else c->c.sysRhsPhase(0);
    }
    for (auto& c : r) {
      if (c->c.imgSrc) c->c.imageMirrorGamma();
      else launch_solve_only(c->c.d, c->c.s, st);
    }
    for (auto& c : r) launch_shed(c->c.d, c->c.s, c->c.frame(0), c->c.d.NW + 1, false, st);
    if (rotor(0).W.sw.rotorForcePlot != 0)
      for (auto& c : r) c->c.sysLoads(0);
    VLM_CUDA(cudaGetLastError());
    for (auto& c : r) c->c.finishSteps(0, nullptr);
    for (auto& c : r) {
      c->c.iter = 0;
      c->c.started = true;
    }
    iter = 0;
    started = true;
  }

  // nsteps iterations; ct_rows (if not null): [step][rotor][10]
  void step(int nsteps, double* ctRows) {
    if (!started) throw StatusError(VLM_ERR_STATE, "vlm_system_start must be called before vlm_system_step");
    Case& c0 = rotor(0);
    c0.useDevice();
    for (auto& c : r) c->c.checkSteps(nsteps);
    for (auto& c : r) c->c.uploadFrames(nsteps);
    cudaStream_t st = stream();
    const Switches& sw = c0.W.sw;
    VLM_CUDA(cudaEventRecord(c0.ev0, st));
    for (int k = iter + 1; k <= iter + nsteps; ++k) {
      for (auto& c : r) c->c.prePhase(k);
      for (auto& c : r) {
        if (c->c.imgSrc) c->c.imageMirrorVelCP();
        else c->c.sysRhsPhase(k);
      }
      for (auto& c : r) {
        if (c->c.imgSrc) c->c.imageMirrorGamma();
        else launch_solve_only(c->c.d, c->c.s, st);
      }
      if (sw.rotorForcePlot != 0 && k % sw.rotorForcePlot == 0)
        for (auto& c : r) c->c.sysLoads(k);
      if (sw.wakeSuppress == 0)
        for (int stg = 0; stg < 4; ++stg)
          for (auto& c : r) {
            if (c->c.imgSrc) c->c.imageWakeStage(k, stg);
            else c->c.wakeStage(k, stg);
          }
    }
    VLM_CUDA(cudaEventRecord(c0.ev1, st));
    VLM_CUDA(cudaGetLastError());
    VLM_CUDA(cudaEventSynchronize(c0.ev1));
    float ms = 0.f;
    VLM_CUDA(cudaEventElapsedTime(&ms, c0.ev0, c0.ev1));
    lastMs = ms;
    const int nr = (int)r.size();
    std::vector<double> rows((size_t)nsteps * 10);
    for (int ir = 0; ir < nr; ++ir) {
      rotor(ir).finishSteps(nsteps, ctRows ? rows.data() : nullptr);
      if (ctRows)
        for (int k = 0; k < nsteps; ++k)
          std::memcpy(ctRows + ((size_t)k * nr + ir) * 10, rows.data() + (size_t)k * 10, 10 * sizeof(double));
    }
    iter += nsteps;
  }
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
  o->solve_mode = -1;
  o->nbody_slots = 0;
  o->lattice = -1;
  o->incremental = 1;
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

// Host-buffer form of rings_device: nc / nr doubles per source of corners /
// core radii (rings 12 / 4, filaments 6 / 1).
static int sources_host(const double* corners, const double* rvc, const double* gam, int64_t N, const double* P,
                        int64_t M, double* V, int precision, bool fil) {
  const size_t nc = fil ? 6 : 12, nr = fil ? 1 : 4;
  return guard([&]() {
    if (N < 0 || M < 0) throw StatusError(VLM_ERR_INVALID, "N and M must be non-negative");
    if ((N > 0 && (!corners || !rvc || !gam)) || (M > 0 && (!P || !V))) throw StatusError(VLM_ERR_INVALID, "null array");
    std::vector<void*> own;
    auto cleanup = [&]() {
      for (void* p : own) cudaFree(p);
    };
    try {
      double* dc = dalloc<double>((size_t)std::max<int64_t>(N, 1) * nc, own);
      double* dr = dalloc<double>((size_t)std::max<int64_t>(N, 1) * nr, own);
      double* dg = dalloc<double>((size_t)std::max<int64_t>(N, 1), own);
      double* dp = dalloc<double>((size_t)std::max<int64_t>(M, 1) * 3, own);
      double* dv = dalloc<double>((size_t)std::max<int64_t>(M, 1) * 3, own);
      if (N > 0) {
        VLM_CUDA(cudaMemcpy(dc, corners, (size_t)N * nc * 8, cudaMemcpyHostToDevice));
        VLM_CUDA(cudaMemcpy(dr, rvc, (size_t)N * nr * 8, cudaMemcpyHostToDevice));
        VLM_CUDA(cudaMemcpy(dg, gam, (size_t)N * 8, cudaMemcpyHostToDevice));
      }
      if (M > 0) VLM_CUDA(cudaMemcpy(dp, P, (size_t)M * 3 * 8, cudaMemcpyHostToDevice));
      rings_device(dc, dr, dg, N, dp, M, dv, precision, nullptr, fil);
      if (M > 0) VLM_CUDA(cudaMemcpy(V, dv, (size_t)M * 3 * 8, cudaMemcpyDeviceToHost));
    } catch (...) {
      cleanup();
      throw;
    }
    cleanup();
  });
}

int vlm_biot_savart_rings(const double* corners, const double* rvc, const double* gam, int64_t N, const double* P,
                          int64_t M, double* V, int precision) {
  return sources_host(corners, rvc, gam, N, P, M, V, precision, false);
}

int vlm_biot_savart_filaments(const double* fc, const double* rvc, const double* gam, int64_t N, const double* P,
                              int64_t M, double* V, int precision) {
  return sources_host(fc, rvc, gam, N, P, M, V, precision, true);
}

int vlm_biot_savart_filaments_device(const double* fc, const double* rvc, const double* gam, int64_t N,
                                     const double* P, int64_t M, double* V, int precision, void* stream) {
  return guard([&]() { rings_device(fc, rvc, gam, N, P, M, V, precision, (cudaStream_t)stream, true); });
}

// ---------------------------------------------------------------------------
// Batch: many independent cases advanced together.  Each case keeps its own
// stream; a step of the batch enqueues every case's step on its stream, so
// the cases' kernels run concurrently.  Once every case is in its steady
// state, one step of the whole batch is captured as ONE CUDA graph (a fork
// from the batch stream into every case stream and a join back) and
// replayed with a single graph launch per step.  Each case's FP32 chunk plan
// is made for its share of the device's block slots.
struct vlm_batch {
  std::vector<vlm_case*> cases;
  cudaStream_t origin = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, fork = nullptr;
  std::vector<cudaEvent_t> joins;
  cudaGraphExec_t gexec = nullptr;
  std::vector<std::pair<int, int>> gsig;  // (rowNear, rowFar) per case of the captured step
  long graphKernels = 0;
  double lastMs = 0.0;

  ~vlm_batch() {
    if (origin) cudaStreamSynchronize(origin);
    if (gexec) cudaGraphExecDestroy(gexec);
    for (cudaEvent_t e : joins) cudaEventDestroy(e);
    for (cudaEvent_t e : {ev0, ev1, fork})
      if (e) cudaEventDestroy(e);
    if (origin) cudaStreamDestroy(origin);
    for (vlm_case* c : cases) delete c;
  }

  // all case streams wait for the batch stream's work so far
  void forkAll() {
    VLM_CUDA(cudaEventRecord(fork, origin));
    for (vlm_case* c : cases) VLM_CUDA(cudaStreamWaitEvent(c->c.stream, fork, 0));
  }
  // the batch stream waits for every case stream's work so far
  void joinAll() {
    for (size_t i = 0; i < cases.size(); ++i) {
      VLM_CUDA(cudaEventRecord(joins[i], cases[i]->c.stream));
      VLM_CUDA(cudaStreamWaitEvent(origin, joins[i], 0));
    }
  }

  bool allSteady(int k) const {
    for (vlm_case* c : cases)
      if (!c->c.steadyStep(k)) return false;
    return true;
  }
  // a case's first step of a signature measures its incremental predicted-wake plan (not in a graph)
  bool anyMeasureDue(int k) const {
    for (vlm_case* c : cases)
      if (c->c.incrMeasureDue(k)) return true;
    return false;
  }

  void capture(int k) {
    if (gexec) cudaGraphExecDestroy(gexec);
    gexec = nullptr;
    cudaGraph_t g = nullptr;
    const long l0 = launch_count();
    VLM_CUDA(cudaStreamBeginCapture(origin, cudaStreamCaptureModeThreadLocal));
    try {
      forkAll();
      for (vlm_case* c : cases) {
        Case& C = c->c;
        C.replaying = true;
        launch_step_begin(C.d, C.s, C.stream);
        C.enqueueStep(k);
        C.replaying = false;
      }
      joinAll();
    } catch (...) {
      for (vlm_case* c : cases) c->c.replaying = false;
      cudaStreamEndCapture(origin, &g);
      if (g) cudaGraphDestroy(g);
      throw;
    }
    VLM_CUDA(cudaStreamEndCapture(origin, &g));
    const cudaError_t e = cudaGraphInstantiate(&gexec, g, 0);
    cudaGraphDestroy(g);
    VLM_CUDA(e);
    graphKernels = launch_count() - l0;
    count_launches(-graphKernels);
    gsig.clear();
    for (vlm_case* c : cases) gsig.emplace_back(c->c.plans[k].rowNear, c->c.plans[k].rowFar);
  }

  bool sigMatches(int k) const {
    if (!gexec || gsig.size() != cases.size()) return false;
    for (size_t i = 0; i < cases.size(); ++i)
      if (gsig[i] != std::make_pair(cases[i]->c.plans[k].rowNear, cases[i]->c.plans[k].rowFar)) return false;
    return true;
  }

  void step(int nsteps, double* ctRows) {
    if (cases.empty()) return;
    cases[0]->c.useDevice();
    const int it0 = cases[0]->c.iter;
    for (vlm_case* c : cases) {
      if (c->c.iter != it0) throw StatusError(VLM_ERR_STATE, "the batch's cases are at different steps");
      c->c.checkSteps(nsteps);
    }
    for (vlm_case* c : cases) c->c.uploadFrames(nsteps);
    VLM_CUDA(cudaEventRecord(ev0, origin));
    joinAll();  // the frames are in
    for (int k = it0 + 1; k <= it0 + nsteps; ++k) {
      if (allSteady(k) && !anyMeasureDue(k)) {
        if (!sigMatches(k)) capture(k);
        // device step counters for replay (the graph advances them)
        for (vlm_case* c : cases) {
          Case& C = c->c;
          if (!C.iterSynced) {
            *C.hIter = k - 1;
            VLM_CUDA(cudaMemcpyAsync(C.s.devIter, C.hIter, sizeof(int), cudaMemcpyHostToDevice, origin));
            C.iterSynced = true;
          }
        }
        VLM_CUDA(cudaGraphLaunch(gexec, origin));
        count_launches(graphKernels);
      } else {
        forkAll();
        for (vlm_case* c : cases) c->c.enqueueOne(k);
        joinAll();
      }
    }
    forkAll();  // later work on the case streams follows the batch's steps
    VLM_CUDA(cudaEventRecord(ev1, origin));
    VLM_CUDA(cudaGetLastError());
    VLM_CUDA(cudaEventSynchronize(ev1));
    float ms = 0.f;
    VLM_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
    lastMs = ms;
    for (size_t i = 0; i < cases.size(); ++i)
      cases[i]->c.finishSteps(nsteps, ctRows ? ctRows + (size_t)i * nsteps * 10 : nullptr);
  }
};

int vlm_batch_create(int ncases, const char* const* configs, const char* const* geoms, const char* const* base_dirs,
                     const vlm_options* opt, vlm_batch** out) {
  if (!out || ncases <= 0 || !configs || !geoms) {
    g_err = "invalid batch arguments";
    return VLM_ERR_INVALID;
  }
  *out = nullptr;
  auto b = std::make_unique<vlm_batch>();
  const int rc = guard([&]() {
    vlm_options o;
    vlm_default_options(&o);
    if (opt) o = *opt;
    VLM_CUDA(cudaSetDevice(o.device));
    if (o.nbody_slots <= 0) o.nbody_slots = std::max(1, partial32_slots() / ncases);
    for (int i = 0; i < ncases; ++i) {
      if (!configs[i] || !geoms[i]) throw StatusError(VLM_ERR_INVALID, "null case text");
      auto c = std::make_unique<vlm_case>();
      c->c.create(configs[i], geoms[i], base_dirs && base_dirs[i] ? base_dirs[i] : "", &o);
      b->cases.push_back(c.release());
    }
    VLM_CUDA(cudaStreamCreateWithFlags(&b->origin, cudaStreamNonBlocking));
    VLM_CUDA(cudaEventCreate(&b->ev0));
    VLM_CUDA(cudaEventCreate(&b->ev1));
    VLM_CUDA(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
    b->joins.resize(ncases);
    for (int i = 0; i < ncases; ++i) VLM_CUDA(cudaEventCreateWithFlags(&b->joins[i], cudaEventDisableTiming));
  });
  if (rc == VLM_OK) *out = b.release();
  return rc;
}

int vlm_batch_destroy(vlm_batch* b) {
  delete b;
  return VLM_OK;
}

int vlm_batch_case(vlm_batch* b, int i, vlm_case** out) {
  if (!b || !out || i < 0 || i >= (int)b->cases.size()) return VLM_ERR_INVALID;
  *out = b->cases[i];
  return VLM_OK;
}

int vlm_batch_start(vlm_batch* b) {
  if (!b) return VLM_ERR_INVALID;
  return guard([&]() {
    for (vlm_case* c : b->cases) c->c.start();
  });
}

int vlm_batch_step(vlm_batch* b, int nsteps, double* ct_rows) {
  if (!b) return VLM_ERR_INVALID;
  return guard([&]() { b->step(nsteps, ct_rows); });
}

int vlm_batch_last_step_ms(vlm_batch* b, double* ms) {
  if (!b || !ms) return VLM_ERR_INVALID;
  *ms = b->lastMs;
  return VLM_OK;
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

// A rotor of a system advances only with its system (vlm_system_step).
static int member_refused() {
  g_err = "this case is a rotor of a system: it advances with vlm_system_start / vlm_system_step";
  return VLM_ERR_STATE;
}

int vlm_system_create(const char* config_text, int nr, const char* const* geom_texts, const char* base_dir,
                      const vlm_options* opt, vlm_system** out) {
  if (!out || !config_text || !geom_texts || nr < 1) {
    g_err = "null argument or nr < 1";
    return VLM_ERR_INVALID;
  }
  *out = nullptr;
  for (int i = 0; i < nr; ++i)
    if (!geom_texts[i]) {
      g_err = "null geometry text";
      return VLM_ERR_INVALID;
    }
  auto y = std::make_unique<vlm_system>();
  const int rc = guard([&]() {
    std::vector<std::string> g(geom_texts, geom_texts + nr);
    y->create(config_text, g, base_dir ? base_dir : "", opt);
  });
  if (rc == VLM_OK) *out = y.release();
  return rc;
}

int vlm_system_create_from_dir(const char* case_dir, const vlm_options* opt, vlm_system** out) {
  if (!case_dir || !out) {
    g_err = "null argument";
    return VLM_ERR_INVALID;
  }
  std::string cfg;
  std::vector<std::string> geoms;
  const int rc = guard([&]() {
    auto rd = [](const std::string& p) {
      std::ifstream f(p);
      if (!f) throw std::runtime_error("cannot open " + p);
      std::stringstream ss;
      ss << f.rdbuf();
      return ss.str();
    };
    cfg = rd(std::string(case_dir) + "/config.nml");
    Namelist c;
    c.parse(cfg);
    const int nr = c.i("PARAMS", "nr", 1);
    if (nr < 1 || nr > 99) throw StatusError(VLM_ERR_INVALID, "config.nml: nr out of range");
    for (int i = 1; i <= nr; ++i) {
      char name[16];
      std::snprintf(name, sizeof(name), "/geom%02d.nml", i);
      geoms.push_back(rd(std::string(case_dir) + name));
    }
  });
  if (rc != VLM_OK) return rc;
  std::vector<const char*> g;
  for (const auto& t : geoms) g.push_back(t.c_str());
  return vlm_system_create(cfg.c_str(), (int)g.size(), g.data(), case_dir, opt, out);
}

int vlm_system_destroy(vlm_system* y) {
  if (y && !y->r.empty()) cudaStreamSynchronize(y->stream());
  delete y;
  return VLM_OK;
}

int vlm_system_rotor_count(const vlm_system* y) { return y ? (int)y->r.size() : -1; }

int vlm_system_rotor(vlm_system* y, int ir, vlm_case** out) {
  if (!y || !out || ir < 0 || ir >= (int)y->r.size()) return VLM_ERR_INVALID;
  *out = y->r[ir].get();
  return VLM_OK;
}

int vlm_system_start(vlm_system* y) {
  if (!y) return VLM_ERR_INVALID;
  return guard([&]() { y->start(); });
}

int vlm_system_step(vlm_system* y, int nsteps, double* ct_rows) {
  if (!y) return VLM_ERR_INVALID;
  return guard([&]() { y->step(nsteps, ct_rows); });
}

int vlm_system_last_step_ms(vlm_system* y, double* ms) {
  if (!y || !ms) return VLM_ERR_INVALID;
  *ms = y->lastMs;
  return VLM_OK;
}

int vlm_case_start(vlm_case* c) {
  if (!c) return VLM_ERR_INVALID;
  if (c->c.member) return member_refused();
  return guard([&]() { c->c.start(); });
}

int vlm_case_step(vlm_case* c, int nsteps, double* ct_rows) {
  if (!c) return VLM_ERR_INVALID;
  if (c->c.member) return member_refused();
  return guard([&]() { c->c.step(nsteps, ct_rows); });
}

int vlm_case_aic_factor(vlm_case* c) {
  if (!c) return VLM_ERR_INVALID;
  if (c->c.member) return member_refused();
  return guard([&]() { c->c.aicFactor(); });
}

int vlm_case_solve_circulation(vlm_case* c, const double* kinematic_vel, double* gam_out) {
  if (!c) return VLM_ERR_INVALID;
  if (c->c.member) return member_refused();
  return guard([&]() { c->c.phaseSolve(kinematic_vel, gam_out); });
}

int vlm_case_loads(vlm_case* c, double* ct_row) {
  if (!c) return VLM_ERR_INVALID;
  if (c->c.member) return member_refused();
  return guard([&]() { c->c.phaseLoads(ct_row); });
}

int vlm_case_wake_step(vlm_case* c) {
  if (!c) return VLM_ERR_INVALID;
  if (c->c.member) return member_refused();
  return guard([&]() { c->c.phaseWake(); });
}

int vlm_case_get_wake(vlm_case* c, int blade, double* waN, double* waN_gam, double* waF, double* waF_gam) {
  if (!c) return VLM_ERR_INVALID;
  return guard([&]() {
    Case& C = c->c;
    if (blade < 1 || blade > C.d.nb) throw StatusError(VLM_ERR_INVALID, "blade out of range");
    const size_t NW = C.d.NW, NF = C.d.NF, ns = C.d.ns;
    const std::pair<const char*, std::pair<double*, size_t>> parts[] = {
        {"waN", {waN, 12 * NW * ns}}, {"waN_gam", {waN_gam, NW * ns}}, {"waF", {waF, 6 * NF}}, {"waF_gam", {waF_gam, NF}}};
    for (const auto& q : parts)
      if (q.second.first) C.get(q.first, blade, q.second.first, (int64_t)q.second.second);
  });
}

int vlm_case_get_int(vlm_case* c, const char* name, int64_t* value) {
  if (!c || !name || !value) return VLM_ERR_INVALID;
  const std::string k = name;
  const Case& C = c->c;
  // rowNear/rowFar of the current iteration (of the open step between its phases)
  const StepPlan& pl = C.plans[C.phase != 0 ? C.iter + 1 : C.iter];
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
  else if (k == "rotorForcePlot") *value = C.W.sw.rotorForcePlot;
  else if (k == "wakePlot") *value = C.W.sw.wakePlot;
  else if (k == "wakeTipPlot") *value = C.W.sw.wakeTipPlot;
  else if (k == "gridPlot") *value = C.W.sw.gridPlot;
  else if (k == "probe") *value = C.W.sw.probe;
  else if (k == "wakeSuppress") *value = C.W.sw.wakeSuppress;
  else if (k == "skewPlotSwitch") *value = C.W.P.skewPlotSwitch;
  else if (k == "inflowPlotSwitch") *value = C.W.P.inflowPlotSwitch;
  else if (k == "gammaPlotSwitch") *value = C.W.P.gammaPlotSwitch;
  else if (k == "rollupStart") *value = C.d.rollupStart;
  else if (k == "rollupEnd") *value = C.d.rollupEnd;
  else if (k == "nodeShape") *value = C.plans[std::min(C.iter + 1, C.W.nt)].node.shape;
  else if (k == "nearPairs" || k == "nodeChunks") {
    // near-field filament-target pairs of the last FP32 evaluation; chunks
    // of the next step's wake-node evaluation
    if (k == "nodeChunks") {
      *value = C.plans[std::min(C.iter + 1, C.W.nt)].node.nchunks;
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

static int64_t copy_text(const std::string& t, char* buf, int64_t cap) {
  if (cap > 0) {
    const size_t n = std::min<size_t>(t.size(), (size_t)cap - 1);
    std::memcpy(buf, t.data(), n);
    buf[n] = 0;
  }
  return (int64_t)t.size();
}

int64_t vlm_case_params_json(vlm_case* c, char* buf, int64_t cap) {
  if (!c || cap < 0 || (cap > 0 && !buf)) return -1;
  std::string t;
  if (guard([&]() { t = c->c.W.params_json(); }) != VLM_OK) return -1;
  return copy_text(t, buf, cap);
}

int64_t vlm_params_json(const char* config_text, const char* geom_text, const char* base_dir, char* buf,
                        int64_t cap) {
  if (!config_text || !geom_text || cap < 0 || (cap > 0 && !buf)) return -1;
  std::string t;
  const int rc = guard([&]() {
    vlm::Wing w;
    w.load(config_text, geom_text, base_dir ? base_dir : "");
    t = w.params_json();
  });
  if (rc != VLM_OK) return -1;
  return copy_text(t, buf, cap);
}

int64_t vlm_wing_kinematics(const char* config_text, const char* geom_text, const char* base_dir, int iter,
                            const char* name, int blade, double* out, int64_t cap) {
  if (!config_text || !geom_text || !name || iter < 0 || cap < 0 || (cap > 0 && !out)) return -1;
  std::vector<double> v;
  const int rc = guard([&]() {
    vlm::Wing w;
    w.load(config_text, geom_text, base_dir ? base_dir : "");
    if (blade < 1 || blade > (int)w.bl.size()) throw StatusError(VLM_ERR_INVALID, "blade out of range");
    if (iter > w.nt) throw StatusError(VLM_ERR_INVALID, "iteration beyond nt");
    w.start_pitch();
    for (int k = 1; k <= iter; ++k) w.advance(k);
    const vlm::Blade& B = w.bl[blade - 1];
    const std::string k = name;
    auto put = [&](vlm::d3 a) { v.push_back(a.x), v.push_back(a.y), v.push_back(a.z); };
    if (k == "PC") { for (const auto& p : B.p) for (int c = 0; c < 4; ++c) put(p.PC[c]); }
    else if (k == "vr") { for (const auto& p : B.p) for (int c = 0; c < 4; ++c) put(p.C[c]); }
    else if (k == "CP") { for (const auto& p : B.p) put(p.CP); }
    else if (k == "nCap") { for (const auto& p : B.p) put(p.nCap); }
    else if (k == "secCP") { for (const auto& c : B.secCP) put(c); }
    else if (k == "vr_rvc") { for (const auto& p : B.p) v.insert(v.end(), p.rvc, p.rvc + 4); }
    else if (k == "secArea") v = B.secArea;
    else if (k == "secChord") v = B.secChord;
    else throw StatusError(VLM_ERR_INVALID, "unknown kinematics array " + k);
  });
  if (rc != VLM_OK) return -1;
  if (out && cap > 0) std::memcpy(out, v.data(), sizeof(double) * std::min<int64_t>((int64_t)v.size(), cap));
  return (int64_t)v.size();
}

int vlm_case_vind_points(vlm_case* c, const double* P, int64_t M, double* V) {
  if (!c || (M > 0 && (!P || !V))) return VLM_ERR_INVALID;
  if (c->c.member) return member_refused();
  return guard([&]() { c->c.vindPoints(P, M, V); });
}

int vlm_selftest_bounded_wait(int limit, int* expired) {
  if (!expired || limit <= 0) return VLM_ERR_INVALID;
  const int r = selftest_bounded_wait((uint32_t)limit);
  if (r < 0) {
    g_err = "CUDA error in the bounded-wait self-test";
    return VLM_ERR_CUDA;
  }
  *expired = r;
  return VLM_OK;
}

void vlm_default_surrogate_options(vlm_surrogate_options* o) {
  if (!o) return;
  o->enable = 1;
  o->young_far = 216;
  o->min_far = 72;
  o->collect_steps = 72;
  o->sample_stride = 4;
  o->train_iters = 3000;
  o->batch = 1024;
  o->lr = 1e-3f;
  o->audit_samples = 256;
  o->audit_tol = 0.1;
  o->hidden = 128;
  o->layers = 4;
  o->seed = 1;
}

int vlm_case_set_tile(vlm_case* c, int shape, int chunks) {
  if (!c) return VLM_ERR_INVALID;
  return guard([&]() { c->c.setTile(shape, chunks); });
}

int vlm_case_set_surrogate(vlm_case* c, const vlm_surrogate_options* o) {
  if (!c || !o) return VLM_ERR_INVALID;
  if (c->c.member) return member_refused();
  return guard([&]() { c->c.setSurrogate(*o); });
}

int vlm_case_surrogate_stats(vlm_case* c, vlm_surrogate_stats* out) {
  if (!c || !out) return VLM_ERR_INVALID;
  *out = c->c.surr.st;
  out->phase = c->c.surr.on ? c->c.surr.phase : VLM_SURR_OFF;
  return VLM_OK;
}

int vlm_case_checkpoint_save(vlm_case* c, const char* path) {
  if (!c || !path) return VLM_ERR_INVALID;
  return guard([&]() { c->c.checkpointSave(path); });
}

int vlm_case_checkpoint_load(vlm_case* c, const char* path) {
  if (!c || !path) return VLM_ERR_INVALID;
  if (c->c.member) return member_refused();
  return guard([&]() { c->c.checkpointLoad(path); });
}

int vlm_case_profile_eval(vlm_case* c, int reps, double* ms_per_launch, double* ring_pairs, double* fil_pairs) {
  if (!c || reps <= 0 || !ms_per_launch || !ring_pairs || !fil_pairs) return VLM_ERR_INVALID;
  if (c->c.member) return member_refused();
  return guard([&]() { c->c.profileEval(reps, ms_per_launch, ring_pairs, fil_pairs); });
}

int64_t vlm_kernel_launch_count(void) { return vlm::launch_count(); }

int vlm_case_last_step_ms(vlm_case* c, double* ms) {
  if (!c || !ms) return VLM_ERR_INVALID;
  *ms = c->c.lastMs;
  return VLM_OK;
}

}  // extern "C"
