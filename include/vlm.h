/*
 * vlm.h -- C ABI of libvlm_gb300.so, the GB300 (sm_103a) free-wake unsteady
 * vortex-lattice engine that replaces the hot path of cibinjoseph/VOLCANOR.
 *
 * Boundary: the reference has no plugin layer; its hot path is the set of
 * type-bound procedures src/main.f90 calls between OpenMP regions.  Each entry
 * below names the reference call site it replaces.  A Fortran caller binds
 * these through ISO_C_BINDING; Python binds them through
 * ctypes (volcanor_gb300/lib.py).
 *
 * Conventions
 *   - every function returns an int status, VLM_OK (0) on success; the
 *     library never aborts; vlm_last_error() describes the last failure of
 *     the calling thread;
 *   - all arrays are caller-owned host memory unless the name ends in
 *     _device; vectors are xyz-contiguous, i.e. a Fortran real(dp) (3, m)
 *     array passes as c_loc(array) without repacking;
 *   - a vlm_case owns its device memory and one CUDA stream; call it from one
 *     host thread at a time.
 */
#ifndef VLM_GB300_H
#define VLM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define VLM_OK 0
#define VLM_ERR_INVALID 1     /* bad argument or unsupported option value */
#define VLM_ERR_CUDA 2        /* CUDA runtime error or no usable GPU */
#define VLM_ERR_IO 3          /* case file missing or unreadable */
#define VLM_ERR_UNSUPPORTED 4 /* case feature outside the accelerated path */
#define VLM_ERR_SINGULAR 5    /* AIC singular or its inverse failed the check */
#define VLM_ERR_NONFINITE 6   /* NaN/Inf detected in a step's result */
#define VLM_ERR_STATE 7       /* call out of order (e.g. step before start) */

/* arithmetic of the Biot-Savart pair evaluations */
#define VLM_PREC_FP64 0           /* reference arithmetic in FP64 */
#define VLM_PREC_FP32 1           /* FP32 pairs, FP64 accumulation of per-tile sums */
#define VLM_PREC_FP32_NEAR64 2    /* as FP32, near-field pairs recomputed in FP64 */

typedef struct vlm_case vlm_case;

typedef struct vlm_options {
  int precision;       /* VLM_PREC_* (default VLM_PREC_FP64) */
  int sum_chunk;       /* FP64 summation block size; 0 = the reference's sequential order */
  double near_factor;  /* near-field radius in core radii for VLM_PREC_FP32_NEAR64 (default 4) */
  int device;          /* CUDA device ordinal (default 0) */
  int use_graph;       /* capture multi-step runs in a CUDA graph (default 1) */
} vlm_options;

/* ---- library ------------------------------------------------------------ */
const char* vlm_version(void);
/* Copies the calling thread's last error message into buf (always NUL terminated). */
int vlm_last_error(char* buf, size_t len);
void vlm_default_options(vlm_options* opt);
/* Kernels launched by this library so far (all threads and cases). */
int64_t vlm_kernel_launch_count(void);
/* SM count and compute capability of `device`. */
int vlm_device_info(int device, int* sm_count, int* cc_major, int* cc_minor);

/* ---- isolated Biot-Savart kernel ------------------------------------------
 * V[m] = sum_n vr_vind(ring n, P[m]) * gam[n]: the unit-strength Vatistas
 * vortex-ring velocity summed over N rings at M points.
 * Replaces vr_vind/vf_vind summation (src/classdef.f90:476-542,
 * blade_vind_bywing src/classdef.f90:1342-1357).
 *   corners: N x 4 x 3 (ring corner k, filament k runs corner k -> k+1)
 *   rvc:     N x 4     (core radius of filament k)
 *   gam:     N; P, V: M x 3
 * Host-buffer form: copies in, evaluates, copies out. */
int vlm_biot_savart_rings(const double* corners, const double* rvc, const double* gam, int64_t N,
                          const double* P, int64_t M, double* V, int precision);
/* Device-buffer form on a caller stream (cudaStream_t passed as void*, NULL =
 * legacy default stream).  Its scratch is shared by all calls on a device, so
 * it returns after the stream has finished the evaluation. */
int vlm_biot_savart_rings_device(const double* corners, const double* rvc, const double* gam, int64_t N,
                                 const double* P, int64_t M, double* V, int precision, void* stream);
/* Scratch bytes the device form needs for (N, M, precision); it allocates
 * them itself on first use and keeps them per device. */
int64_t vlm_biot_savart_rings_scratch_bytes(int64_t N, int64_t M, int precision);
/* Summation block size the ring kernel uses for (N, M, precision): the rings
 * are summed in consecutive blocks of this many, each block from zero, the
 * block sums then added in order (N = one block = the reference's order). */
int64_t vlm_biot_savart_rings_sum_chunk(int64_t N, int64_t M, int precision);

/* Allocation-free form of the device-buffer ring kernel.  It has no
 * counterpart in the reference.  It is for callers that cannot allocate
 * device memory when they call it (a host solver that reserves its device
 * memory once at start-up, a process under a hard device-memory cap, or a
 * caller that must not trigger the device-wide synchronisation an allocation
 * may cause): its scratch is one fixed 8 MiB array compiled into the library,
 * held on every device that loads the library until the process exits.
 * Limits: N <= 16384 rings, M <= 65536 points, at most 65536 near-field
 * pairs (VLM_PREC_FP32_NEAR64); larger sizes return VLM_ERR_INVALID with a
 * message.  The rings are summed in one block, i.e. in the reference's order.
 * The first call on a device looks up the scratch array's device address,
 * so make that first call before any CUDA stream capture.  All calls on a
 * device share the scratch and the call returns after its stream has
 * finished; calls that overlap on the GPU (other host threads or streams at
 * the same time) race on the scratch and must be serialised by the caller. */
int vlm_biot_savart_rings_noalloc(const double* corners, const double* rvc, const double* gam, int64_t N,
                                  const double* P, int64_t M, double* V, int precision, void* stream);

/* ---- one rotor case ----------------------------------------------------------
 * Replaces readConfig + rotor%readGeom + rotor%init (src/main.f90:12-40,
 * src/libCommon.f90:51-108, src/classdef.f90:2541-3891).  config_text and
 * geom_text hold config.nml and geom01.nml; base_dir resolves geometryFile. */
int vlm_case_create(const char* config_text, const char* geom_text, const char* base_dir, const vlm_options* opt,
                    vlm_case** out);
/* Reads case_dir/config.nml and case_dir/geom01.nml. */
int vlm_case_create_from_dir(const char* case_dir, const vlm_options* opt, vlm_case** out);
int vlm_case_destroy(vlm_case* c);
/* Initial pitch, AIC assembly + inverse + check, wake-free initial solution,
 * iteration-0 loads (src/main.f90:43-377; rotor_calcAIC
 * src/classdef.f90:4151-4179, inv2 src/libMath.f90:48-83). */
int vlm_case_start(vlm_case* c);
/* Advance nsteps timesteps (src/main.f90:400-1452): kinematics, shed, wake
 * ageing/dissipation, circulation solve, loads, wake velocities, predictor-
 * corrector convection, strain, rollup/truncation.  If ct_rows is not NULL it
 * receives nsteps x 10 rows (iter, CL/CT, CD/CQ, CLu, CDi, CD0, CDu, CFx, CFy,
 * CFz) -- the rXXForceNonDim.csv columns (src/libPostprocess.f90:814-838). */
int vlm_case_step(vlm_case* c, int nsteps, double* ct_rows);
/* Integer state: nt, nb, nc, ns, n, nNwake, nFwake, rowNear, rowFar, iter,
 * nbConvect, wakeTruncateNt; nearPairs (near-field filament-target pairs of the
 * last FP32 evaluation) and nodeChunks (chunks of the next step's wake-node
 * evaluation) describe this library's kernels. */
int vlm_case_get_int(vlm_case* c, const char* name, int64_t* value);
/* Copy a named array (see the design doc for the list and layouts) into out.
 * Returns the element count, or -1 for an unknown name. */
int64_t vlm_case_get(vlm_case* c, const char* name, int blade, double* out, int64_t cap);
/* Induced velocity of the current wing + wake at M points (probes / gridgen:
 * src/libPostprocess.f90:333-361, src/gridgen.f90:115-140). */
int vlm_case_vind_points(vlm_case* c, const double* P, int64_t M, double* V);
/* Device time of the kernels of the last vlm_case_step call, milliseconds
 * (CUDA events after the call's input upload). */
int vlm_case_last_step_ms(vlm_case* c, double* ms);
/* Launches the Biot-Savart partial-sum kernel of the next step's wake-node
 * evaluation `reps` times on the current state (no state change) and reports
 * its mean launch time and the ring-target and filament-target pair counts of
 * one launch (roofline accounting). */
int vlm_case_profile_eval(vlm_case* c, int reps, double* ms_per_launch, double* ring_pairs, double* fil_pairs);

#ifdef __cplusplus
}
#endif

#endif /* VLM_GB300_H */
