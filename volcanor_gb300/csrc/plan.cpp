// Chunk planner of the FP32 Biot-Savart kernel.
//
// The FP32 kernel's grid is (target blocks) x (chunks): one block sums one
// chunk of consecutive source records for 512 targets.  The FP64 path's
// chunking fixes its summation order and so its bits; the FP32 path's does
// not, so it is chosen for speed.  A solver step evaluates shapes from a few
// dozen collocation points (one target block) to tens of thousands of wake
// nodes against groups of very different sizes (a blade's wing: tens of
// records; its wake: thousands), so a fixed chunk size either leaves most
// block slots of the GPU idle or pays for many tiny chunks.
//
// Model: a block costs kOverhead + (its chunk's record count) time units
// (one unit = one record for a full block of targets).  For each candidate
// count n of chunks of the largest group, every group is split into
// ceil(size / C) chunks of balanced size, C = ceil(largest / n); the grid's
// time is estimated as the number of waves, ceil(total cost / (slots x
// largest block cost)), times the largest block cost.  The cheapest estimate
// wins, the smaller chunk count on ties; chunks x targets stays below 2^24
// (the partial sums' memory) unless one chunk per group already exceeds it.  The plan is a pure function of the
// shapes and the slot count, so it is reproducible run to run.
#include <algorithm>
#include <cmath>
#include <cstdint>

#include "vlm_bs.h"

namespace vlm {

namespace {
constexpr double kOverhead = 8.0;  // block start-up, target load and partial write, in record units
constexpr int kMinChunk = 16;
constexpr int64_t kMaxPartials = 1 << 24;  // (chunks x targets) bound: 384 MB of FP64 partial sums
}  // namespace

int plan_count32(const Group* groups, int ngroups, int M, int slots, int cap, int targets_per_block) {
  int64_t total = 0;
  int maxRec = 0;
  for (int g = 0; g < ngroups; ++g) {
    total += std::max(0, groups[g].rec_count);
    maxRec = std::max(maxRec, groups[g].rec_count);
  }
  if (total == 0 || M <= 0) return 0;
  slots = std::max(1, slots);
  const int64_t bx = (M + targets_per_block - 1) / targets_per_block;
  const int nmax = std::max(1, std::min(maxRec / kMinChunk, 4 * slots));
  int bestN = 1;
  double bestT = 0.0;
  int64_t bestQ = 0;
  for (int n = 1; n <= nmax; ++n) {
    const int C = (maxRec + n - 1) / n;
    int64_t Q = 0;
    int cmax = 0;
    for (int g = 0; g < ngroups; ++g) {
      const int rc = groups[g].rec_count;
      if (rc <= 0) continue;
      const int ng = (rc + C - 1) / C;
      Q += ng;
      cmax = std::max(cmax, (rc + ng - 1) / ng);
    }
    if (Q > cap || (n > 1 && Q * (int64_t)M > kMaxPartials)) break;
    const double blockMax = kOverhead + cmax;
    const double work = (double)bx * ((double)Q * kOverhead + (double)total);
    const double waves = std::max(1.0, std::ceil(work / (slots * blockMax)));
    const double T = waves * blockMax;
    if (n == 1 || T < bestT * (1.0 - 1e-9) || (T <= bestT * (1.0 + 1e-9) && Q < bestQ)) {
      bestT = T;
      bestN = n;
      bestQ = Q;
    }
  }
  return bestN;
}

int build_chunks32(Group* groups, int ngroups, int n, Chunk* chunks, int cap) {
  int maxRec = 0;
  for (int g = 0; g < ngroups; ++g) maxRec = std::max(maxRec, groups[g].rec_count);
  if (n <= 0 || maxRec <= 0) {
    for (int g = 0; g < ngroups; ++g) groups[g].chunk_begin = groups[g].chunk_count = 0;
    return 0;
  }
  const int C = (maxRec + n - 1) / n;
  int nq = 0;
  for (int g = 0; g < ngroups; ++g) {
    Group& G = groups[g];
    G.chunk_begin = nq;
    G.chunk_count = 0;
    const int rc = G.rec_count;
    if (rc <= 0) continue;
    const int ng = (rc + C - 1) / C;
    for (int i = 0; i < ng; ++i) {
      // chunk i of ng: records [rc*i/ng, rc*(i+1)/ng)
      const int b = (int)((int64_t)rc * i / ng), e = (int)((int64_t)rc * (i + 1) / ng);
      if (nq >= cap) return -1;
      chunks[nq].rec_begin = G.rec_begin + b;
      chunks[nq].rec_count = e - b;
      ++nq;
      ++G.chunk_count;
    }
  }
  return nq;
}

int plan_chunks32(Group* groups, int ngroups, int M, int slots, Chunk* chunks, int cap, int targets_per_block) {
  const int n = plan_count32(groups, ngroups, M, slots, cap, targets_per_block);
  return build_chunks32(groups, ngroups, n, chunks, cap);
}

}  // namespace vlm
