/* gravidy_gb300.h -- C ABI of the GB300 (sm_103a) Hermite4 block-step path.
 *
 * Drop-in boundary for the GPU backend of GraviDy: the class Hermite4GPU
 * (src/include/gpu/Hermite4GPU.cuh:100-144) and the Hermite4 base methods it
 * inherits (src/include/Hermite4.hpp:60-63).  The reference keeps the
 * particle state in host arrays of NbodySystem (src/include/NbodySystem.hpp:
 * 98-134) and copies them to and from the device around every kernel; here
 * the state lives in device memory for the lifetime of a handle and is copied
 * to the host only on request (h4_download) -- for logs and snapshots.
 *
 * Conventions
 *  - Every call returns an h4_status (0 = success).  Nothing exits or aborts
 *    the process (the reference's CSC macro calls exit(EXIT_FAILURE),
 *    Hermite4GPU.cuh:43-50).  h4_last_error() gives a message for the last
 *    failure on the calling thread.
 *  - A handle is not thread safe; calls on one handle must be serialised.
 *  - Host arrays use the reference layouts: h4_double4 is CUDA's double4
 *    (x, y, z, w; w = mass for positions), h4_forces is the reference's Forces
 *    (a[3], a1[3]; common.hpp:227-231), h4_double3 is double3.
 *  - All work is issued on the handle's stream (h4_set_stream); calls that
 *    return host values synchronise that stream.
 */
#ifndef GRAVIDY_GB300_H
#define GRAVIDY_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define H4_ABI_VERSION 2

typedef struct { double x, y, z, w; } h4_double4;
typedef struct { double x, y, z; } h4_double3;
typedef struct { double a[3]; double a1[3]; } h4_forces;

typedef enum {
    H4_OK = 0,
    H4_ERR_ARG = 1,        /* invalid argument (null pointer, size, range) */
    H4_ERR_CUDA = 2,       /* CUDA runtime error; see h4_last_error() */
    H4_ERR_ALLOC = 3,      /* device or host allocation failed */
    H4_ERR_STATE = 4,      /* call out of order (e.g. step before init) */
    H4_ERR_NONFINITE = 5,  /* non-finite value found in the state */
    H4_ERR_UNSUPPORTED = 6 /* feature not available for this handle */
} h4_status;

/* Arithmetic of the O(N_act N) force sum. */
typedef enum {
    H4_FORCE_FP64 = 0,   /* FP64 pair arithmetic, j-split + fixed-order sums */
    H4_FORCE_EXACT = 1,  /* FP64 in the reference's exact operation order:
                            bit-identical forces to the reference CPU path
                            (slow; a validation mode) */
    H4_FORCE_MIXED = 2   /* FP32 pair arithmetic, double-single position
                            deltas, compensated FP32 partial sums, FP64
                            per-particle reduction */
} h4_force_mode;

typedef struct h4_system_s *h4_handle;

/* Message of the last failure on this thread ("" if none). */
const char *h4_last_error(void);
const char *h4_status_string(int status);
int h4_abi_version(void);
/* Build variant of the loaded library (no reference counterpart): bit
 * H4_BUILD_BOUNDS_CHECK is set in the bounds-checked build, whose kernels
 * check every index range before touching it and report a violation as
 * H4_ERR_STATE ("bounds check failed at site N") instead of accessing memory
 * out of bounds. */
#define H4_BUILD_BOUNDS_CHECK 1
int h4_build_flags(void);

/* Creation.  Replaces Hermite4GPU::Hermite4GPU + alloc_arrays_device
 * (Hermite4GPU.cu:40-165) and Hermite4::init_data (Hermite4.cpp:194-240).
 *   n      number of particles (n >= 1)
 *   e2     softening squared, as NbodySystem::e2 (NbodySystem.cpp:50)
 *   eta    timestep accuracy parameter, NbodySystem::eta (-e flag)
 *   r, v   host arrays of n double4 (r.w = mass, rounded to float as the
 *          reference does; v.w ignored)
 *   mode   an h4_force_mode
 * The state starts as init_data leaves it: predictors = (r, v, m), forces,
 * timesteps and times zero. */
int h4_create(h4_handle *out, unsigned int n, double e2, float eta,
              const h4_double4 *r, const h4_double4 *v, int mode);
int h4_destroy(h4_handle h);

/* Run the handle's work on a caller-provided stream (cudaStream_t passed as
 * void*; NULL selects the handle's own non-blocking stream, so the legacy
 * default stream cannot be selected). */
int h4_set_stream(h4_handle h, void *stream);
/* Timestep bounds, D_TIME_MIN / D_TIME_MAX of common.hpp:122,129 (defaults
 * 2^-23 and 2^-3).  Both must be powers of two with dt_min <= dt_max. */
int h4_set_dt_limits(h4_handle h, double dt_min, double dt_max);
int h4_set_force_mode(h4_handle h, int mode);
/* H4_FORCE_MIXED: active-set size from which the shared-memory tiled kernel
 * (lanes over active particles) is used instead of warp items (lanes over j).
 * Default 192 for N >= 131072, 320 for N >= 65536, else 768 (measured
 * crossover on GB300). */
int h4_set_mixed_threshold(h4_handle h, unsigned int nact_threshold);

/* Hermite4GPU::init_acc_jrk (Hermite4GPU.cu:333-375): acc and jerk of all
 * particles from the current predictors (O(N^2)). */
int h4_init_acc_jrk(h4_handle h);

/* Hermite4::init_dt (Hermite4.cpp:108-140): Aarseth initial block timesteps
 * with accuracy parameter eta (the reference passes ETA_S), t = itime for all
 * particles; *atime = min(*atime, min dt) as the reference's CTIME. */
int h4_init_dt(h4_handle h, double *atime, float eta, double itime);

/* Hermite4::find_particles_to_move (Hermite4.cpp:63-84): the active set
 * {i : |itime - (t_i + dt_i)| < 2 DBL_EPSILON} in ascending i, kept on the
 * device; *nact receives its size. */
int h4_find_particles_to_move(h4_handle h, double itime, unsigned int *nact);

/* Hermite4::save_old_acc_jrk (Hermite4.cpp:145-153). */
int h4_save_old_acc_jrk(h4_handle h, unsigned int nact);

/* Hermite4GPU::predicted_pos_vel (Hermite4GPU.cu:201-268): third-order
 * Taylor prediction of all particles to itime. */
int h4_predicted_pos_vel(h4_handle h, double itime);

/* Hermite4GPU::update_acc_jrk (Hermite4GPU.cu:385-535): new acc and jerk of
 * the nact active particles against all N. */
int h4_update_acc_jrk(h4_handle h, unsigned int nact);

/* Hermite4GPU::correction_pos_vel (Hermite4GPU.cu:274-328, restating
 * Hermite4CPU.cpp:370-411): Hermite corrector, t = itime, and the new block
 * timestep (NbodyUtils::get_timestep_normal + normalize_dt,
 * NbodyUtils.cpp:337-424) of the active particles. */
int h4_correction_pos_vel(h4_handle h, double itime, unsigned int nact);

/* Hermite4::next_integration_time (Hermite4.cpp:90-102). */
int h4_next_integration_time(h4_handle h, double *atime);

/* Hermite4GPU::get_energy_gpu (Hermite4GPU.cu:540-592): kinetic and
 * unsoftened potential energy of the corrected state; returns the total in
 * *etot (any output pointer may be NULL). */
int h4_get_energy(h4_handle h, double *ekin, double *epot, double *etot);

/* One whole block step on the device (the loop body of
 * Hermite4GPU_integration.cpp:81-99): itime = *atime, find active set, save
 * old forces, predict, force, correct, next time.  Outputs may be NULL;
 * a non-NULL nact/itime/atime synchronises the stream. */
int h4_step(h4_handle h, double *atime, double *itime, unsigned int *nact);

/* Advance with device-resident block steps until the block time reaches
 * t_stop (the reference's "while (ITIME < integration_time)" loop) or a step
 * reaches t_log (the energy log condition ITIME >= interval * k).  The step
 * sequence is replayed from a CUDA graph; the host waits once at the end.
 * *atime is the next block time in and out; the counters accumulate.
 *   stats[0] = block steps done   stats[1] = particle steps (sum of nact)
 *   stats[2] = interactions (sum of nact * N)   stats[3] = last itime
 *   stats[4] = nact of the last step */
int h4_advance(h4_handle h, double t_stop, double t_log, double *atime,
               double *itime, double stats[5]);

/* Copy the state to host arrays (any pointer may be NULL; n elements each;
 * move receives the current active list, entries past nact undefined). */
int h4_download(h4_handle h, h4_double4 *r, h4_double4 *v, h4_forces *f,
                h4_forces *old, h4_double3 *a2, h4_double3 *a3, double *t,
                double *dt, unsigned int *move);
/* Replace parts of the state (any pointer may be NULL). */
int h4_upload(h4_handle h, const h4_double4 *r, const h4_double4 *v,
              const h4_forces *f, const h4_forces *old, const double *t,
              const double *dt);
/* Resume from a saved state: replaces r, v, f, t, dt (n elements each) and
 * marks the forces valid, so h4_step/h4_advance continue from *atime
 * without h4_init_acc_jrk/h4_init_dt.  With the state written by
 * h4_download the continuation is bit-identical to an uninterrupted run.
 * (The reference resumes from 4-digit snapshots and recomputes forces and
 * timesteps, OptionsParser.cpp:122-323, NbodySystem.cpp:106-147.) */
int h4_restore(h4_handle h, const h4_double4 *r, const h4_double4 *v,
               const h4_forces *f, const double *t, const double *dt,
               double atime);
/* Predicted positions/velocities (Predictor array of the reference,
 * common.hpp:213-218, as two double4 arrays; pr.w = mass). */
int h4_download_predicted(h4_handle h, h4_double4 *pr, h4_double4 *pv);

/* Stateless force sum for tests and tools: acc/jerk of the particles
 * listed in move[0..nact) against all n, from predictors (pr.w = mass). */
int h4_forces_for(h4_handle h, const h4_double4 *pr, const h4_double4 *pv,
                  unsigned int nact, const unsigned int *move, h4_forces *out);

/* ---- Batched ensemble ------------------------------------------------------
 * Many independent systems (e.g. star clusters of uneven N), each with its own
 * block time and active set, advanced together: one persistent fused kernel
 * per iteration does one block step of every unfinished system (active set +
 * predictor, force sum from one work queue over all systems, corrector +
 * timesteps + next time), replayed from a CUDA graph with a device-side while
 * loop.  No counterpart in the reference, which integrates one system per
 * process (src/gravidy.cpp:54-115); per system the arithmetic is that of the
 * calls above.  Systems are stored back to back: system c owns particles
 * [sum n[0..c), sum n[0..c]) of every concatenated array. */
typedef struct h4_ensemble_s *h4_ens_handle;
/* Tuning table: for (N bucket b, active-count bucket a) at index b*NB_A + a,
 * the shape of the force work of a system's block step.  N buckets: <=512,
 * <=1k, <=2k, <=4k, <=8k, larger; active buckets: 1, 2-3, 4-15, 16-63,
 * 64-255, 256-1023, 1024-4095, >=4096.
 *   ig     FP64 and exact forms: particles per warp item (1, 2 or 4).
 *          Mixed form: 1, 2 or 4 = warp items (lanes over j; 2 = one
 *          packed pair, 4 = two), or a power of two in [16, 512] =
 *          block-tiled items of ig particles (lanes over i, j tiles in
 *          shared memory).
 *   chunk  j per item (rounded up to whole tiles for block items).
 *   jtile  j per shared-memory tile of a block item, 128 or 256 (NULL: 256). */
#define H4_ENS_TUNE_NB_N 6
#define H4_ENS_TUNE_NB_A 8
const char *h4_ens_last_error(void);
int h4_ens_create(h4_ens_handle *out, unsigned int nsys, const unsigned int *n,
                  const double *e2, const float *eta, const h4_double4 *r,
                  const h4_double4 *v, int mode);
int h4_ens_destroy(h4_ens_handle e);
int h4_ens_set_stream(h4_ens_handle e, void *stream);
int h4_ens_set_tuning(h4_ens_handle e, const unsigned int *ig,
                      const unsigned int *chunk, const unsigned int *jtile);
int h4_ens_set_dt_limits(h4_ens_handle e, double dt_min, double dt_max);
/* init_acc_jrk + init_dt (ETA_S) of every system. */
int h4_ens_init(h4_ens_handle e);
/* Block steps until every system's block time reaches its t_end[c] (the
 * reference's while (ITIME < integration_time) per system).
 * stats: [0] block steps (all systems) in this call, [1] particle steps and
 * [2] interactions since creation, [3] kernel iterations (launches). */
int h4_ens_advance(h4_ens_handle e, const double *t_end, double stats[4]);
/* Kinetic and unsoftened potential energy of every system. */
int h4_ens_energy(h4_ens_handle e, double *ekin, double *epot);
int h4_ens_download(h4_ens_handle e, h4_double4 *r, h4_double4 *v,
                    h4_forces *f, double *t, double *dt);
int h4_ens_system_stats(h4_ens_handle e, double *itime, double *atime,
                        unsigned long long *steps, unsigned long long *psteps,
                        unsigned long long *inter);
/* Autotuner probe: the force phase alone with every system's first nact
 * particles active (positions as stored), using (ig, chunk) everywhere;
 * *ms = device time.  Leaves the integration state unchanged. */
int h4_ens_tune_force(h4_ens_handle e, unsigned int nact, unsigned int ig,
                      unsigned int chunk, unsigned int jtile, float *ms);
/* Block steps and interactions (N_act * N) per tuning bucket, summed over the
 * systems' steps since creation (index b*NB_A + a as the tuning table): the
 * mixture of (N, N_act) a tuning should be weighted by.  Either may be NULL. */
int h4_ens_bucket_stats(h4_ens_handle e, unsigned long long *steps,
                        unsigned long long *inter);
int h4_ens_timings(h4_ens_handle e, float *advance_ms,
                   unsigned long long *kernel_launches);
/* Device time per phase of the persistent ensemble kernel since creation
 * (ms): 0 next block time + active sets + work layout (per system), 1
 * predictor, 2 force sums, 3 reduction + corrector; read on the device clock
 * at the grid barriers between phases. */
int h4_ens_phase_times(h4_ens_handle e, double ms[4]);

/* Force sum that allocates nothing.  No counterpart in the reference.
 *
 * For callers that cannot call cudaMalloc -- an application that hands all
 * of the GPU's memory to its own pool at start-up, or a time-critical loop
 * that cannot take the synchronisation an allocation may imply.  The FP64
 * force kernel; it agrees with h4_forces_for of an FP64-mode handle to within
 * rounding (for large nact the j-split, and so the summation order, may
 * differ, since the scratch is smaller than a handle's), but every buffer is
 * the caller's device memory and no handle is needed:
 *   n           particles, 1 .. 2^28 (the limit of h4_create)
 *   d_pr, d_pv  n predicted positions (w = mass) and velocities, 32-byte
 *               aligned device arrays of h4_double4
 *   d_move      nact particle indices (device), d_out nact h4_forces (device)
 *   stream      cudaStream_t as void* (NULL = the legacy default stream)
 * The partial sums use a fixed file-scope device array of
 * H4_NOALLOC_SCRATCH_DOUBLES doubles (16 MiB), held on every GPU that loads
 * this library until the process exits; nact above H4_NOALLOC_MAX_NACT is
 * rejected with H4_ERR_ARG.  The first call on a device is its set-up: it
 * looks up the array's device address (cudaGetSymbolAddress) with that
 * device current, which may load the library's device code there; make that
 * first call before any stream capture.  Later calls repeat the cheap
 * look-up.  Calls share the array, and each call clears the part of it that
 * must start at zero: calls that overlap on the GPU race and must be
 * serialised by the caller.
 * The call is asynchronous on `stream`; the message of a failure is
 * returned by h4_forces_noalloc_error(). */
#define H4_NOALLOC_SCRATCH_DOUBLES (2u * 1024u * 1024u)
#define H4_NOALLOC_MAX_NACT (H4_NOALLOC_SCRATCH_DOUBLES / 6u)
int h4_forces_noalloc(unsigned int n, double e2, const h4_double4 *d_pr,
                      const h4_double4 *d_pv, unsigned int nact,
                      const unsigned int *d_move, h4_forces *d_out,
                      void *stream);
const char *h4_forces_noalloc_error(void);

/* ---- Cluster diagnostics (NbodyUtils, src/include/utils/NbodyUtils.cpp) ----
 * On the corrected state; nothing here feeds back into the dynamics.
 * Center of density (get_center_of_density, :163-220): density of every
 * particle from its 6th-neighbour distance, density-weighted mean position;
 * needs n >= 8. */
int h4_center_of_density(h4_handle h, double cod[3]);
/* Mass radii about `center` (get_core_radius :108-143 with CORE_MASS = 0.1,
 * get_halfmass_radius :223-260, get_radii + get_layers :285-328 with
 * LAGRANGE_RADII = {0.01, 0.05, 0.1, 0.2, 0.5, 0.75}); total_mass is
 * NbodySystem::total_mass (float).  Any output pointer may be NULL. */
int h4_mass_radii(h4_handle h, const double center[3], float total_mass,
                  double *core, double *halfmass, double lagrange[6]);
const char *h4_diag_last_error(void);

/* Device time (ms) of the last force kernel launch and of the last
 * h4_advance call, measured with CUDA events on the handle's stream. */
int h4_last_timings(h4_handle h, float *force_ms, float *advance_ms);
/* Block steps run by h4_advance since creation, by active-set size:
 * counts[k] = steps with 2^k <= nact < 2^(k+1). */
int h4_nact_histogram(h4_handle h, unsigned long long counts[32]);
/* Device time per phase since creation, CUDA events on the handle's stream,
 * with the phase names of the reference's Gtime (common.hpp:287-310):
 * 0 prediction, 1 update (force sum + reduction), 2 grav (force kernel
 * alone), 3 correction, 4 active_set, 5 next_time, 6 energy, 7 advance
 * (device-resident loop; its inner phases are not split).  counts = calls. */
#define H4_PHASES 8
int h4_phase_times(h4_handle h, double ms[H4_PHASES], unsigned long long counts[H4_PHASES]);
const char *h4_phase_name(int phase);
/* Kernels launched by this handle since creation. */
int h4_kernel_launches(h4_handle h, unsigned long long *count);

/* Self-test of the bounded device wait every inter-block wait of this library
 * uses (ensemble grid barriers): one thread waits on a flag that nothing sets,
 * for `seconds` (<= 5); *timed_out = 1 when the wait gave up as designed.
 * The context stays usable. */
int h4_selftest_bounded_wait(double seconds, int *timed_out);

/* Throughput of the FP64 and FP32 pipes on this GPU (flop/s, FMA = 2),
 * measured with a short dependent-FMA kernel; used as roofline peaks. */
int h4_probe_peaks(double *fp64_flops, double *fp32_flops);

#ifdef __cplusplus
}
#endif
#endif /* GRAVIDY_GB300_H */
