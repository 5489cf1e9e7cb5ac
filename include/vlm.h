/*
 * vlm.h -- C ABI of libvlm_gb300.so, the GB300 (sm_103a) free-wake unsteady
 * vortex-lattice engine that replaces the hot path of cibinjoseph/VOLCANOR.
 *
 * Boundary: the reference has no plugin layer; its hot path is the set of
 * type-bound procedures src/main.f90 calls between OpenMP regions.  Each entry
 * below names the reference call site it replaces.  A Fortran caller binds
 * these through ISO_C_BINDING interface blocks; Python binds them through
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
  int solve_mode;      /* circulation solve: 0 = FP64 explicit inverse (the reference's inv2 +
                          matmulAX), 1 = FP32 LU with partial pivoting + FP64 iterative
                          refinement (3 passes; lu_residual reports max|b-Ax|/max|b|),
                          -1 = 1 for the FP32 precisions, 0 for FP64 (default) */
  int nbody_slots;     /* resident block slots the FP32 chunk planner plans for (0 = the whole
                          device; a batch gives each of its cases a share) */
  int lattice;         /* FP32 precisions: evaluate each near-wake lattice edge by edge, a
                          filament shared by two rings once with their circulation
                          difference (0 = ring by ring as the reference; -1 / nonzero =
                          lattice form, the default).  No effect on VLM_PREC_FP64. */
  int incremental;     /* FP32 precisions, schemes with a predictor (fdSchemeSwitch 1, 3, 4, 5):
                          the predicted-wake velocities as the current-wake ones plus the
                          changed sources' difference, and the full sum at the moved wake nodes
                          only, on steps whose (rowNear, rowFar) signature lasts at least 16
                          steps and where that is less than half the full sum's work (1 = on,
                          the default; 0 = the full sum).  Not for coupled rotors or with the
                          surrogate; no effect on FP64. */
} vlm_options;

/* ---- library ------------------------------------------------------------ */
const char* vlm_version(void);
/* Copies the calling thread's last error message into buf (always NUL terminated). */
int vlm_last_error(char* buf, size_t len);
void vlm_default_options(vlm_options* opt);
/* Kernels launched by this library so far (all threads and cases). */
int64_t vlm_kernel_launch_count(void);
/* Failure-path self-test (no counterpart in the reference): launches a wait
 * on a device barrier that nothing releases, bounded by `limit` polls, the
 * same bounded wait the N-body pipeline uses.  *expired = 1 when the wait gave
 * up and reported, as it must; the context stays usable. */
int vlm_selftest_bounded_wait(int limit, int* expired);
/* SM count and compute capability of `device`. */
int vlm_device_info(int device, int* sm_count, int* cc_major, int* cc_minor);
/* FP32 CUDA-core throughput of `device` as measured (no counterpart in the
 * reference): a kernel of independent FMA chains on every SM, `reps` timed
 * launches after one warm-up, CUDA events.  *tflops = 2 flop per FMA / time;
 * the denominator of the N-body kernel's measured roofline fraction. */
int vlm_measure_fp32_peak(int device, int reps, double* tflops, double* ms_per_launch);

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
/* V[m] = sum_n vf_vind(filament n, P[m]) * gam[n] over N single filaments
 * (src/classdef.f90:476-503; the trailing-edge and far-wake filaments of
 * gridgen, src/gridgen.f90:128-136).  fc: N x 2 x 3 (fc(:,1), fc(:,2));
 * rvc, gam: N.  No |gam| skip.  Same summation blocks, scratch and
 * precisions as the ring kernel. */
int vlm_biot_savart_filaments(const double* fc, const double* rvc, const double* gam, int64_t N,
                              const double* P, int64_t M, double* V, int precision);
int vlm_biot_savart_filaments_device(const double* fc, const double* rvc, const double* gam, int64_t N,
                                     const double* P, int64_t M, double* V, int precision, void* stream);

/* Allocation-free form of the device-buffer ring kernel.  It has no
 * counterpart in the reference.  It is for callers that cannot allocate
 * device memory when they call it (a host solver that reserves its device
 * memory once at start-up, a process under a hard device-memory cap, or a
 * caller that must not trigger the device-wide synchronisation an allocation
 * may cause): its scratch is one fixed 11.5 MiB array compiled into the
 * library, held on every device that loads the library until the process
 * exits.  Limits: N <= 16384 rings, M <= 65536 points; larger sizes return
 * VLM_ERR_INVALID with a message, as does a VLM_PREC_FP32_NEAR64 call with
 * more than 65536 near-field pairs.  FP64 sums the rings in one block,
 * i.e. in the reference's order; the FP32 precisions split them into as
 * many blocks as fill the device (at most 256 and 65536 / M).
 * The call waits for its stream before it returns, so it cannot be
 * captured into a CUDA graph: on a capturing stream it returns
 * VLM_ERR_INVALID without launching anything.  The first call on a device
 * looks up the scratch array's device address and keeps it for the life of
 * the process: do not reset the device (cudaDeviceReset) once it has been
 * made.  All calls on a
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
/* ---- the time step as separate calls ---------------------------------------
 * For a host that keeps its own time loop and replaces the reference's
 * procedures one by one.  vlm_case_aic_factor replaces rotor%calcAIC + inv2
 * + isInverse at start-up (src/main.f90:62-81; vlm_case_start calls it when
 * the host has not).  One iteration k = iter + 1 is then
 *   vlm_case_solve_circulation  -- the RHS loop + matmulAX + map_gam
 *       (src/main.f90:466-603: leading-edge shedding, wake ageing and
 *       dissipation, wake-induced velocity at the collocation points, RHS,
 *       gamVec); kinematic_vel (3 x n, the RHS rows' order ic + nc(is-1) +
 *       nc ns(ib-1); NULL = the library's own prescribed kinematics) is the
 *       kinematic part of velCP the reference computes at main.f90:522-560;
 *       gam_out (n, or NULL) receives gamVec;
 *   vlm_case_loads (optional)   -- calc_force + the CT row of force2file
 *       (src/main.f90:623-764); ct_row (10, or NULL) receives the
 *       rXXForceNonDim.csv row.  The reference computes loads only on
 *       iterations that are multiples of rotorForcePlot, and so does
 *       vlm_case_step; the loads carry the unsteady term's previous
 *       circulation from one call to the next;
 *   vlm_case_wake_step          -- wake-node velocities, the FD scheme,
 *       strain, roll-up / truncation, trailing-edge shedding
 *       (src/main.f90:799-1439); the case is then at iteration k.
 * Between vlm_case_loads and vlm_case_wake_step the case holds the state the
 * reference writes its per-step files from (filaments2file, probes2file,
 * src/main.f90:788,795): vlm_case_get / vlm_case_get_wake /
 * vlm_case_vind_points read it there (the wing arrays and rowNear / rowFar
 * are those of the open step; iter stays at the last finished one).  The three calls in sequence produce
 * the same bits as vlm_case_step(c, 1, row) (loads called on the iterations
 * vlm_case_step computes them). */
int vlm_case_aic_factor(vlm_case* c);
int vlm_case_solve_circulation(vlm_case* c, const double* kinematic_vel, double* gam_out);
int vlm_case_loads(vlm_case* c, double* ct_row);
int vlm_case_wake_step(vlm_case* c);
/* The wake of blade (1-based) as the reference stores it (waN, waF of
 * blade_class): near-wake ring corners (3, 4, nNwake, ns), their
 * circulations (nNwake, ns), far-wake filament nodes (3, 2, nFwake), their
 * circulations (nFwake).  Any pointer may be NULL. */
int vlm_case_get_wake(vlm_case* c, int blade, double* waN, double* waN_gam, double* waF, double* waF_gam);

/* Integer state: nt, nb, nc, ns, n, nNwake, nFwake, rowNear, rowFar, iter,
 * nbConvect, wakeTruncateNt, rotorForcePlot, the output switches (wakePlot, wakeTipPlot, gridPlot,
 * probe, wakeSuppress, skewPlotSwitch, inflowPlotSwitch, gammaPlotSwitch, after the reference's
 * conversion of chords/revolutions), rollupStart, rollupEnd; nearPairs (near-field filament-target pairs of the
 * last FP32 evaluation), nodeChunks and nodeShape (chunks and FP32 tile
 * shape of the next step's wake-node evaluation; after the last step, of the
 * last one) describe this library's kernels. */
int vlm_case_get_int(vlm_case* c, const char* name, int64_t* value);
/* FP32 N-body tile shape (no counterpart in the reference).  By default a
 * case autotunes: at the first steady-state step of each (rowNear, rowFar)
 * signature (every later step of a truncated wake repeats it) it times its
 * live wake-node and collocation-point evaluations with each compiled tile
 * shape (0: 512 targets per block, 4 stages, 2 blocks per SM; 1: 256 targets
 * per block, 3 stages, 3 blocks per SM) at the wave model's chunk count and at
 * 1/2, 3/4, 3/2 and 2 times it, then the best shape at +-1, 2, 3 chunks of
 * its best count, and keeps the fastest (vlm_case_get
 * "autotune").  This call re-plans every step after the current one with
 * `shape` and `chunks` chunks for the largest group of each evaluation (0 =
 * the wave model's count) and turns the tuner off; shape -1 turns it back
 * on.  FP32 precisions of a lone case without the surrogate; results change
 * only in the FP32 summation order. */
int vlm_case_set_tile(vlm_case* c, int shape, int chunks);
/* Copy a named array into out (at most cap doubles); blade is 1-based where
 * the array is per blade.  Returns the element count, or -1 for an unknown
 * name.  Names and layouts (Fortran column-major, xyz fastest):
 *   dt, nonDimDenom, lu_residual    scalars (lu_residual: last refined solve, 0 without refinement)
 *   Omega, theta0                   scalars: rotor speed (rad/s), collective pitch (rad)
 *   ct_hist                         (10, iter+1) CT rows so far
 *   AIC, AIC_inv                    (n, n); gamVec (n)
 *   gam (blade)                     (nc, ns) wing circulation
 *   CP, nCap, velCP, velCPTotal     (3, nc, ns) per blade
 *   vr (blade)                      (3, 4, nc, ns) wing ring corners
 *   waN (blade)                     (3, 4, nNwake, ns) near-wake ring corners
 *   waN_gam, waN_rvc (blade)        (nNwake, ns), (4, nNwake, ns)
 *   waF (blade)                     (3, 2, nFwake) far-wake filament nodes
 *   waF_gam, waF_rvc (blade)        (nFwake)
 *   waF_rvc0, waF_l0, waF_lc, waF_age (blade)  (nFwake) initial core, original and current
 *                                   length, age of the far-wake filaments
 *   waN_age (blade)                 (nNwake, ns) near-wake ring ages
 *   vr_rvc (blade)                  (4, nc, ns) wing ring filament core radii
 *   velN, velF (blade)              (3, nNwake, ns+1), (3, nFwake) node velocities
 *   velN1..velN3, velF1..velF3 (blade)  the same shapes: the velocity history of the
 *                                   multi-step schemes (velNwake1..3, velFwake1..3)
 *   velKin (blade)                  (3, nc, ns) the kinematic velocity at the collocation points
 *                                   of the current iteration (during an open step, of that step)
 *   autotune                        per steady-state signature the FP32 tile autotuner
 *                                   timed (first steady step of each): rowNear, rowFar,
 *                                   candidates timed, then for the wake nodes and for
 *                                   the collocation points: chosen tile shape, chunk
 *                                   count of the largest group, ms per launch of the
 *                                   choice, ms of the wave model's plan (11 per signature)
 *   incremental                     per measured signature of the incremental predicted-wake
 *                                   evaluation: rowNear, rowFar, used (0/1), changed records,
 *                                   moved nodes, record capacity, node capacity, records,
 *                                   nodes (9 per signature)
 *   hub                             (3) hub coordinates; yAxis (blade) (3) the blade's y axis;
 *   secCP (blade)                   (3, ns) section points -- all of the current iteration
 *                                   (of the open step between its phases)
 *   waP (blade)                     (3, 2, 240) the prescribed far wake's filaments (fc(:,1), fc(:,2)),
 *                                   cases with prescWakeAfterTruncNt > 0 only (src/classdef.f90:222-236)
 *   waP_gam, waP_rvc (blade)        scalars: its circulation and core radius
 *   gamPrev (blade)                 (nc, ns) the previous step's trapezoidal circulation
 *                                   (the unsteady term of the loads)
 *   secCL, secLift, secLiftDir, secChordwiseResVel (blade)  per section
 *   forceDist (blade <= nbConvect)  (16, ns): the columns of rXXbYYForceDistNNNNN.csv
 *                                   (src/libPostprocess.f90:850-878) for the current iteration
 *   forceDim                        (11): the rXXForceDim.csv values (src/libPostprocess.f90:840-846)
 *   profileWork                     (2): flops and filament-target evaluations the FP32 kernel
 *                                   executed per launch in the last vlm_case_profile_eval */
int64_t vlm_case_get(vlm_case* c, const char* name, int blade, double* out, int64_t cap);
/* The rXXParams.json text the reference writes at start-up (params2file,
 * src/libPostprocess.f90:52-141): the case's parameters after rotor_init in
 * the reference's key order and number layout.  Copies at most cap-1 bytes
 * and a terminating NUL into buf (buf may be NULL when cap is 0); returns the
 * full text length, or -1 on error. */
int64_t vlm_case_params_json(vlm_case* c, char* buf, int64_t cap);
/* The same text from the case files alone (host only, no device use). */
int64_t vlm_params_json(const char* config_text, const char* geom_text, const char* base_dir, char* buf,
                        int64_t cap);
/* Prescribed wing kinematics from the case files alone (host only, no
 * device use): the initial pitch and the motion of iterations 1..iter
 * (src/main.f90:43-58,412-463; blade_rotate / blade_move,
 * src/classdef.f90:1160-1281) applied to the geometry of rotor_init, then
 * one array of blade `blade` (1-based) copied into out (at most cap doubles):
 *   PC    (3, 4, nc, ns) panel corners      vr    (3, 4, nc, ns) vortex-ring corners
 *   CP    (3, nc, ns) collocation points    nCap  (3, nc, ns) panel normals
 *   secCP (3, ns) section reference points
 *   vr_rvc (4, nc, ns) ring filament core radii; secArea, secChord (ns)
 * Returns the element count, or -1 on error (vlm_last_error says why). */
int64_t vlm_wing_kinematics(const char* config_text, const char* geom_text, const char* base_dir, int iter,
                            const char* name, int blade, double* out, int64_t cap);
/* Induced velocity of the current wing + wake at M points (probes / gridgen:
 * src/libPostprocess.f90:333-361, src/gridgen.f90:115-140).  Between the
 * phases of an open step it is the state inside that iteration (the wing
 * and wake rows of the open step), which is where the reference evaluates
 * its probe and inflow files (src/main.f90:764-797). */
int vlm_case_vind_points(vlm_case* c, const double* P, int64_t M, double* V);
/* Checkpoint / resume: replaces the reference's restart files
 * (Restart/restartNNNNN.dat written every restartWriteNt steps and read for
 * restartFromNt, src/main.f90:389-397,1443-1450).  save writes the case's
 * whole solver state (step counter, circulations, wake, loads history, AIC
 * factors) to a binary file; load restores it into a case created from the
 * same case files (started or not).  With the same options the case then
 * continues bit-identically; the state is FP64 in every precision, so a case
 * of another precision, summation block or solve mode may also load it and
 * continue in its own arithmetic (a refining case factors the restored AIC
 * in FP32 when the file has no FP32 factors).  A case of other dimensions or
 * another format -> VLM_ERR_INVALID.  A case with the surrogate saves its
 * flow state (not the network or the surrogate's phase, so another case --
 * e.g. the plain FP64 form -- can continue from it); it cannot load one
 * (VLM_ERR_UNSUPPORTED). */
int vlm_case_checkpoint_save(vlm_case* c, const char* path);
int vlm_case_checkpoint_load(vlm_case* c, const char* path);
/* Device time of the kernels of the last vlm_case_step call, milliseconds
 * (CUDA events after the call's input upload). */
int vlm_case_last_step_ms(vlm_case* c, double* ms);
/* Launches the Biot-Savart partial-sum kernel of the next step's wake-node
 * evaluation `reps` times on the current state (no state change) and reports
 * its mean launch time and the ring-target and filament-target pair counts of
 * one launch (roofline accounting). */
int vlm_case_profile_eval(vlm_case* c, int reps, double* ms_per_launch, double* ring_pairs, double* fil_pairs);

/* ---- many independent cases in one launch per step -------------------------
 * The reference has no batch mode (nr > 1 couples rotors aerodynamically);
 * this runs ncases independent cases (each its own case files, precision
 * and options from opt) on one GPU.  A batch step enqueues every case's step
 * on the case's own stream, so their kernels run concurrently; once every
 * case is in its steady state (same near/far rows step after step), one
 * batch step is captured as one CUDA graph and replayed with one launch per
 * step.  Each case's FP32 chunk plan is made for its share of the device
 * (opt->nbody_slots, default all slots / ncases). */
typedef struct vlm_batch vlm_batch;
int vlm_batch_create(int ncases, const char* const* configs, const char* const* geoms, const char* const* base_dirs,
                     const vlm_options* opt, vlm_batch** out);
int vlm_batch_destroy(vlm_batch* b);
/* Borrowed handle of case i (getters; do not destroy or step it alone). */
int vlm_batch_case(vlm_batch* b, int i, vlm_case** out);
int vlm_batch_start(vlm_batch* b);
/* Every case advances nsteps; ct_rows (if not NULL) receives ncases x nsteps x 10. */
int vlm_batch_step(vlm_batch* b, int nsteps, double* ct_rows);
/* Device time of the last vlm_batch_step call (all cases), milliseconds. */
int vlm_batch_last_step_ms(vlm_batch* b, double* ms);

/* ---- coupled rotors (nr > 1) -------------------------------------------------
 * Replaces the multi-rotor form of src/main.f90: rotor(nr) allocated and
 * read from geom01.nml .. geomNN.nml (:17-39), and every induced-velocity sum
 * of the iteration run over all rotors -- the initial solution with the other
 * rotors' wings (:147-153), the RHS with every rotor's wake and the other
 * rotors' wings (:549-561), the loads without every rotor's bound vortices
 * (:632-652), and the wake-node velocities from every rotor's wing and wake
 * (:808-827, 1052-1076) -- with each do-ir loop of the iteration run over the
 * rotors in turn.  Every rotor is a lifting surface with a wake (nNwake > 0)
 * or an image of an earlier one (surfaceType -1, imagePlane 1..3,
 * imageRotorNum; ground effect): its parameters are the source's, its
 * geometry mirrored at initialisation, and each step its circulation, velCP
 * and wake are the source's mirrored (rotor_mirrorGamma/VelCP/Wake,
 * src/classdef.f90:4990-5131, in the reference's places of the loop).
 * Non-lifting surfaces and sub-iterations (ntSub, ntSubInit) give
 * VLM_ERR_UNSUPPORTED.  Rotor ir > 0
 * is initialised with dt, nt and the switches as rotor ir - 1 left them
 * (rotor_init's intent(inout) arguments, src/classdef.f90:2778-3011).  opt
 * applies to every rotor; all rotors run on one stream; no graph replay.
 * A rotor's vlm_case handle (vlm_system_rotor) serves the getters, files and
 * checkpoint saves; stepping, phase, surrogate, point-query and checkpoint
 * load calls on it return VLM_ERR_STATE. */
typedef struct vlm_system vlm_system;
int vlm_system_create(const char* config_text, int nr, const char* const* geom_texts, const char* base_dir,
                      const vlm_options* opt, vlm_system** out);
/* config.nml and geom01.nml .. geomNN.nml (NN = nr of config.nml) of a case directory */
int vlm_system_create_from_dir(const char* case_dir, const vlm_options* opt, vlm_system** out);
int vlm_system_destroy(vlm_system* y);
int vlm_system_rotor_count(const vlm_system* y);
/* Borrowed handle of rotor ir (0-based). */
int vlm_system_rotor(vlm_system* y, int ir, vlm_case** out);
int vlm_system_start(vlm_system* y);
/* nsteps iterations of every rotor; ct_rows (if not NULL): nsteps x nr x 10
 * (each rotor's rXXForceNonDim.csv row of each step). */
int vlm_system_step(vlm_system* y, int nsteps, double* ct_rows);
/* Device time of the last vlm_system_step call, milliseconds. */
int vlm_system_last_step_ms(vlm_system* y, double* ms);

/* ---- learned far-wake surrogate of a case -----------------------------------
 * No counterpart in the reference (it sums the far wake directly).  With the
 * FP32 precisions, the OLD far wake -- the rolled-up tip filaments behind the
 * near-wake sheet past the young_far youngest of each blade -- is the
 * surrogate's domain.  Once it holds min_far filaments per blade, the case
 * collects training pairs for collect_steps steps -- features of the
 * collocation points and every sample_stride-th near-wake node (position
 * about the hub over the rotor radius, rotor-azimuth harmonics, old-wake fill)
 * and a coarse descriptor of the old wake (its |circulation|-weighted
 * centroid about the hub / R, its mean |circulation| relative to the wing's
 * largest) -> their direct old-far-wake velocity -- and trains an MLP (layers linear
 * layers of width hidden, tanh) for train_iters Adam steps on the GPU.  From
 * then on the network replaces the old-far-wake sum at the collocation
 * points and near-wake nodes (far-wake nodes, next to the old wake along the
 * tip vortex, keep the direct sum).  Before every step an audit compares it
 * with the direct FP64 old-far-wake sum at the collocation points and
 * audit_samples near-wake nodes; when the relative rms error exceeds
 * audit_tol that step sums the old far wake directly and data collection and
 * training start again. */
#define VLM_SURR_OFF -1
#define VLM_SURR_WAIT 0
#define VLM_SURR_COLLECT 1
#define VLM_SURR_ACTIVE 2
typedef struct vlm_surrogate_options {
  int enable;          /* default 1 */
  int young_far;       /* youngest far-wake filaments per blade kept in the direct sum (216) */
  int min_far;         /* old far-wake filaments per blade before collecting (72) */
  int collect_steps;   /* steps of training data (72) */
  int sample_stride;   /* every k-th near-wake node is a training sample (4) */
  int train_iters;     /* Adam steps per training (3000) */
  int batch;           /* samples per Adam step (1024) */
  float lr;            /* learning rate (1e-3; the last third at a fifth) */
  int audit_samples;   /* near-wake nodes audited per step (256) */
  double audit_tol;    /* relative rms error of the old-far-wake velocity that reverts (0.1) */
  int hidden;          /* width (128) */
  int layers;          /* linear layers (4) */
  uint64_t seed;       /* weights and shuffles (1) */
} vlm_surrogate_options;
typedef struct vlm_surrogate_stats {
  int phase;           /* VLM_SURR_* */
  int trainings;
  int audits;
  int reverts;
  int active_steps;    /* steps that used the network */
  int64_t samples;     /* training pairs of the current data set */
  double last_audit_err, max_audit_err;
  float last_loss;     /* training loss (targets in units of their rms) */
} vlm_surrogate_stats;
void vlm_default_surrogate_options(vlm_surrogate_options* o);
/* Before vlm_case_start. */
int vlm_case_set_surrogate(vlm_case* c, const vlm_surrogate_options* o);
int vlm_case_surrogate_stats(vlm_case* c, vlm_surrogate_stats* out);

/* ---- multilayer perceptron of the learned far-wake surrogate ---------------
 * No counterpart in the reference (its far wake is always summed directly).
 * An FP32 MLP with tanh hidden layers and a linear output layer; sizes[0]
 * inputs, sizes[nsizes-1] outputs, row-major W_l (out x in) then b_l per
 * layer in the parameter vector; MSE loss over all outputs of a batch; Adam.
 * Forward, backward and update run as this library's CUDA kernels; every
 * reduction has a fixed order, so results are reproducible.  Buffers are
 * host memory, row major (n x in, n x out). */
typedef struct vlm_mlp vlm_mlp;
int vlm_mlp_create(const int* sizes, int nsizes, uint64_t seed, vlm_mlp** out);
int vlm_mlp_destroy(vlm_mlp* m);
int64_t vlm_mlp_param_count(const vlm_mlp* m);
int vlm_mlp_get_params(vlm_mlp* m, float* out);
int vlm_mlp_set_params(vlm_mlp* m, const float* in);
int vlm_mlp_forward(vlm_mlp* m, const float* X, int64_t n, float* Y);
/* Forward-pass arithmetic: 1 = tensor cores (tcgen05 MMAs, BF16 weights and
 * activations, FP32 accumulation, all layers fused in one kernel; the
 * default when every layer is at most 256 wide), 0 = FP32 CUDA cores (the
 * arithmetic of training).  VLM_ERR_UNSUPPORTED if the network does not fit
 * the tensor-core kernel.  get returns the current mode. */
int vlm_mlp_set_inference(vlm_mlp* m, int mode);
int vlm_mlp_get_inference(const vlm_mlp* m);
/* Gradient of the batch MSE with respect to every parameter, and the loss. */
int vlm_mlp_gradient(vlm_mlp* m, const float* X, const float* T, int64_t n, float* grad, float* loss);
/* iters Adam steps (learning rate lr) over consecutive batches of the
 * n samples (shuffle them beforehand); final_loss = loss of the last batch. */
int vlm_mlp_train(vlm_mlp* m, const float* X, const float* T, int64_t n, int batch, int iters, float lr,
                  float* final_loss);

#ifdef __cplusplus
}
#endif

#endif /* VLM_GB300_H */
