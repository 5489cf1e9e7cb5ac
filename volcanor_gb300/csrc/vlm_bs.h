// Source records, chunk tables and launchers of the Biot-Savart N-body kernels.
//
// A Biot-Savart evaluation sums, for every target point, the unit-strength
// Vatistas velocity of a sequence of vortex sources times their circulation.
// The sequence is split into GROUPS -- the reference's per-blade sums
// (rotor_vind_bywing / rotor_vind_bywake, src/classdef.f90:4424-4479) -- and
// every group into CHUNKS of consecutive records.  One kernel computes a
// partial sum per (target, chunk); a second adds the chunk partials of each
// group in order and the group sums in order, reproducing the reference's
// accumulation exactly when a chunk spans a whole group.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace vlm {

// Number of kernels this library has launched (all threads, all cases).
void count_launch();
void count_launches(long n);  // kernels of a replayed graph (negative: undo a capture's count)
long launch_count();

// FP64 source record, 18 doubles:
//   [0..11] ring corners c0..c3 (xyz); a single filament uses [0..5] = fc1, fc2
//   [12..15] core radius of filament k (c_k -> c_{k+1}); a filament uses [12]
//   [16] circulation (a horseshoe closing filament stores -gam)
//   [17] flags: REC_FIL (single filament) | REC_SKIP (skip if |gam| <= eps)
constexpr int kRec64 = 18;
constexpr int REC_FIL = 1;
constexpr int REC_SKIP = 2;

// FP32 source record, 48 floats (192 B, 16-byte aligned for bulk copies):
//   [0..11]  corners c0..c3
//   [12..23] weighted edge vectors w_k e_k, e_k = c_{k+1} - c_k, w_k = gam_k/(4 pi)
//            (gam_k = gam, or the edge's own circulation in lattice form)
//   [24..27] w_k |e_k|^2
//   [28..31] (rvc_k |e_k|)^4, floored at 1e-36 so the kernel needs no clamp;
//            [30], [31] are -1 when edge 2 / edge 3 carries no circulation
//            (the kernel then skips it and, if both, corner c3's vector)
//   [32..35] near-field threshold on |r1 x r2|^2: (near_factor rvc_k |e_k|)^2, -1 if off
//   [36..39] lower near-field bound on (w_k e_k).r1
//   [40..43] upper near-field bound on (w_k e_k).r1
//   [44..47] unused (zero; pads the record to 192 B)
// A pair is near when the target lies within near_factor core radii of the
// filament SEGMENT: |r1 x r2|^2 < [32+k] and -s < e.r1 < |e|^2 + s with
// s = near_factor rvc_k |e_k|; the second test is stored multiplied by w_k,
// so [36+k] < (w_k e_k).r1 < [40+k] (bounds swapped when w_k < 0).
constexpr int kRec32 = 48;

// Lattice form (FP32 paths): a near-wake lattice has every interior
// filament twice, once in each of the two rings that share it, in opposite
// directions.  With an edge-weight array ew (4 doubles per record), ring
// (i, j) carries edge 0 (c0 -> c1, shared with ring (i, j-1)) and edge 1
// (c1 -> c2, shared with ring (i+1, j)) with the circulation difference of
// the two rings, and edges 2 and 3 only where no neighbour absorbs them
// (the lattice's border, or a neighbour whose shared corners or core radius
// differ).  The sum over the lattice is unchanged; an interior ring costs two
// filament evaluations and three corner vectors instead of four and four.
// Records outside lattices get ew = gam on their active filaments.

#ifdef __CUDACC__
#define VLM_BS_HD __host__ __device__
#else
#define VLM_BS_HD
#endif

// One near-field filament-target pair: target m, chunk q (partial sum to
// correct), global record index, filament k.
struct NearPair {
  int32_t m, q, rec, k;
};

// Near-field scratch of an evaluation at M targets: the targets binned in a
// uniform grid whose occupied cells sit in an open-addressing hash table
// (T slots, T = the smallest power of two >= max(1024, M): at least two
// targets per occupied cell on the wakes this serves), carved from
// one caller buffer: header, [T] cell keys, [T] per-slot target counts (the
// fill cursors after the scan), [T + 1] slot starts, [M] float4 entries in
// slot order (the target's FP32 position and, in w, its index's bits).
struct GridHdr {
  double zsum;         // sum of the near-zone radii (the cell size is a multiple of their mean)
  unsigned int zcount;
  int T;               // table slots
  int lo[3], hi[3];    // bounding box of the binned FP32 target positions (order-preserving int codes)
};
VLM_BS_HD constexpr int grid_buckets(int M) {
  int T = 1024;
  while (T < M && T < (1 << 28)) T <<= 1;
  return T;
}
VLM_BS_HD constexpr size_t grid_align(size_t b) { return (b + 255) & ~size_t(255); }
struct GridLayout {
  size_t key, count, start, entry, total;
};
VLM_BS_HD constexpr GridLayout grid_layout(int M) {
  const size_t T = (size_t)grid_buckets(M);
  const size_t key = grid_align(sizeof(GridHdr));
  const size_t count = key + grid_align(T * sizeof(unsigned long long));
  const size_t start = count + grid_align(T * sizeof(int));
  const size_t entry = start + grid_align((T + 1) * sizeof(int));
  return GridLayout{key, count, start, entry, entry + grid_align((size_t)M * 4 * sizeof(float))};
}
// Bytes of the grid part of the near-field scratch of an evaluation at M
// targets; the near-pair list (NearPair entries) follows it.
VLM_BS_HD constexpr size_t near_grid_bytes(int M) { return grid_layout(M).total; }
constexpr int kNearAlign = 256;
// Near-field scratch for M targets and a list of cap near pairs.
VLM_BS_HD constexpr size_t near_scratch_bytes(int M, size_t cap) {
  return near_grid_bytes(M) + grid_align(cap * sizeof(NearPair));
}

// Fixed-point scale of the near-field accumulators: FP64 near-field
// velocities are added as integers (v * 2^44, |v| < 2^18) so that their sum
// does not depend on the order in which the pairs are processed.
constexpr double kNearScale = 17592186044416.0;  // 2^44
constexpr double kNearMax = 262144.0;            // 2^18

struct Group {
  int32_t rec_begin;    // first record (index into the record array)
  int32_t rec_count;    // number of records
  int32_t chunk_begin;  // first chunk of this group in the chunk table
  int32_t chunk_count;
  int32_t kind;         // 0 = wing sum, 1 = wake sum
  int32_t blade;        // blade whose wing or wake the group sums
  int32_t pad[2];       // pad[0] = 1: a wake group of the far-wake filaments alone, from the pad[1]-th
  // coupled rotors: the sum (one rotor's wing, wake, or wing + wake) this
  // group belongs to; non-decreasing along a group table (launch_combine_terms)
  int32_t term = 0;
  int32_t pad2 = 0;
};

struct Chunk {
  int32_t rec_begin;
  int32_t rec_count;
};

// Builds the chunk table for `groups` (in place: fills chunk_begin/count).
// Returns the number of chunks.
int build_chunks(Group* groups, int ngroups, int chunk_size, Chunk* chunks, int cap);

// Targets one FP32 kernel block covers (tile shape 0, the default).
constexpr int kTargetsPerBlock32 = 512;
// Compiled tile shapes of the FP32 kernel (launch_partial32's `shape`).
constexpr int kPartial32Shapes = 2;
int partial32_targets_per_block(int shape);

// Chunk plan for the FP32 kernel (whose summation order is free): picks the
// number of chunks per group that minimises the modelled run time of a grid
// of ceil(M / targets_per_block) x chunks blocks on `slots` resident block
// slots, with chunks of balanced size inside each group.  Fills the groups'
// chunk_begin/count like build_chunks; returns the number of chunks, or -1
// if cap is too small.
int plan_chunks32(Group* groups, int ngroups, int M, int slots, Chunk* chunks, int cap,
                  int targets_per_block = kTargetsPerBlock32);
// The two halves of plan_chunks32: the modelled best chunk count of the
// largest group, and the table for a given count (the autotuner times
// counts around the model's).
int plan_count32(const Group* groups, int ngroups, int M, int slots, int cap, int targets_per_block);
int build_chunks32(Group* groups, int ngroups, int n, Chunk* chunks, int cap);
// Resident block slots of the FP32 kernel on the current device
// (SMs x resident blocks per SM).
int partial32_slots(int shape = 0);
// Streaming multiprocessors of the current device (cached per device).
int device_sm_count();


// FP64 reference-arithmetic partial sums: part[(q * M + m) * 3 + k].
void launch_partial64(const double* rec, const Chunk* chunks, int nchunks, const double* P, int M, double* part,
                      cudaStream_t s);
// FP32 pairs with FP64 accumulation over the nrec records the chunks cover.
// When near_scratch is non-null (near_bytes = near_scratch_bytes(M, cap) for a list of cap
// near pairs), the
// pairs inside the records' near-field thresholds are then corrected to FP64
// through the fixed-point accumulators nacc (M x nchunks x 3, zero on entry
// and left zero on return).  ctl[0] receives a nonzero code if a bounded wait
// on the tile pipeline expired (1, 2), the near-field scratch was too small
// or the near-pair list was too small (3) or a near-field correction left the
// fixed-point range (4); ctl[1] counts the near pairs.  ctl must be zeroed before the call.
// ew: the records' edge weights in lattice form (FP64 near field multiplies
// by ew[4 rec + k] instead of the record's circulation), or null.
// A second stream and two events on which launch_partial32 runs the
// near-field detection and correction alongside the pair kernel.
// reuse_grid: near_scratch already holds the target grid of these M targets P
// (built by the previous near-field evaluation at the same targets, whose
// records set its cell size), so only the pair search over these records runs.
struct NearOverlap {
  cudaStream_t stream;
  cudaEvent_t fork, join;
};
void launch_partial32(const float* rec32, const double* rec64, const Chunk* chunks, int nchunks, int nrec,
                      const double* P, int M, double* part, int* ctl, void* near_scratch, size_t near_bytes,
                      long long* nacc, cudaStream_t s, const double* ew = nullptr, int shape = 0,
                      const NearOverlap* ov = nullptr, bool reuse_grid = false);
// Converts FP64 records to FP32 records (near_factor <= 0 disables near-field);
// ew as above (null: every active filament of a record carries its gam).
void launch_pack32(const double* rec64, int nrec, double near_factor, float* rec32, cudaStream_t s,
                   const double* ew = nullptr);

// Combines partials: total = sum over wing groups + sum over wake groups,
// each group the in-order sum of its chunk partials, each from zero.
//   mode 0: out[m] = 0 + (wing + wake)      (wake-node velocity, libCommon.f90:114-211)
//   mode 1: out[m] = wake                   (rotor_vind_bywake at a collocation point)
//   mode 2: out[m] = wing + wake            (point query)
void launch_combine(const double* part, int M, const Group* groups, int ngroups, int mode, double* out,
                    cudaStream_t s);

// As launch_combine, but each group's chunk partials are added as a fixed
// tree (up to a warp per target, sized by max_chunks, the largest chunk count
// of a group) instead of in chunk order: for the FP32 paths, whose chunking
// is itself free.
void launch_combine_unordered(const double* part, int M, const Group* groups, int ngroups, int max_chunks, int mode,
                              double* out, cudaStream_t s);

// Coupled rotors: chunk partials -> per-term sums (Group::term).  mode 0:
// out[m] = sum over terms of (wing + wake), in term order; mode 3:
// out[t * M + m] = the term's own sum.  ordered: the FP64 chunk order;
// else the FP32 paths' fixed tree.
void launch_combine_terms(const double* part, int M, const Group* groups, int ngroups, int max_chunks, int mode,
                          bool ordered, double* out, cudaStream_t s);

// Incremental predicted-wake evaluation (incr.cu).  Items of two sets that
// differ bit by bit (records: kRec64 doubles and, with ea/eb, 4 edge weights;
// targets: 3 doubles): launch_diff_count leaves per-tile exclusive offsets in
// blockCount (incr_diff_blocks(n) entries) and the number in *total.
int incr_diff_blocks(int n);
void launch_diff_count(const double* a, const double* b, int stride, const double* ea, const double* eb, int n,
                       int* blockCount, int* total, cudaStream_t s);
// The delta set of the changed records (predicted +, current with negated
// circulation -), padded to cap (even) with inert records; ctl = 5 when more
// than cap / 2 records changed.
void launch_delta_records(const double* recP, const double* recC, const double* ewP, const double* ewC, int nrec,
                          const int* blockOff, const int* total, double* dRec, double* dEw, int cap, int* ctl,
                          cudaStream_t s);
// The moved targets' indices and positions, padded to cap; ctl = 5 when more than cap moved.
void launch_moved_targets(const double* tP, const double* tC, int M, const int* blockOff, const int* total, int* idx,
                          double* pos, int cap, int* ctl, cudaStream_t s);
// out[m] += delta[m] at every target, then out[idx[i]] = moved[i] for the
// moved ones; a nonzero subCtl[0] (the moved targets' evaluation's launch_partial32
// code) is passed on to ctl.
void launch_incr_merge(double* out, const double* delta, int M, const int* idx, const double* moved,
                       const int* total, int cap, const int* subCtl, int* ctl, cudaStream_t s);

// Launches a wait that nothing releases, bounded by `limit` polls: 1 if it
// gave up and reported (the expected outcome), 0 if it did not, -1 on a CUDA
// error.
int selftest_bounded_wait(uint32_t limit);

// Isolated rings (vlm_biot_savart_rings): AoS corners (N x 4 x 3), rvc (N x 4), gam (N) -> FP64 records.
void launch_rings_to_rec64(const double* corners, const double* rvc, const double* gam, int64_t N, double* rec,
                           cudaStream_t s);
// Single filaments (fc: N x [fc1 xyz, fc2 xyz], one core radius and one
// circulation each) to FP64 records.
void launch_fils_to_rec64(const double* fc, const double* rvc, const double* gam, int64_t N, double* rec,
                          cudaStream_t s);

}  // namespace vlm
