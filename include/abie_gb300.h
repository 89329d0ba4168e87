/*
 * abie_gb300 -- GB300 (sm_103a) implementation of ABIE's gravity hot path.
 *
 * C ABI of libabie_gb300.so.  The first block keeps the exact names and
 * argument meanings of the reference library that abie/clibabie.py loads
 * through ctypes, so that library can be swapped for this one.  Positions,
 * velocities and accelerations are caller-owned float64 arrays laid out
 * x0,y0,z0,x1,... (3N entries); masses and radii hold N entries.  The
 * library keeps one simulation state, resident in GPU memory.
 *
 * Size arguments declared size_t receive ctypes c_int from the reference's
 * Python caller (abie/clibabie.py:43-46, :61); the library reads only their
 * low 32 bits.
 *
 * Return codes: 0 normal; 1 and 2 keep the reference's meaning (too many
 * close encounters / collisions, src/common.h:6-8); negative values are
 * errors of this library (ABIE_ERR_*) with a message available from
 * abie_last_error().  The library never exits the process.
 */
#ifndef ABIE_GB300_H
#define ABIE_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ABIE_OK 0
#define ABIE_EXIT_MAX_N_CE 1          /* src/common.h:6 */
#define ABIE_EXIT_MAX_N_COLLISIONS 2  /* src/common.h:7 */
#define ABIE_ERR_NO_DEVICE (-1)       /* no usable sm_103 GPU */
#define ABIE_ERR_NOT_INITIALIZED (-2)
#define ABIE_ERR_CUDA (-3)
#define ABIE_ERR_UNSUPPORTED (-4)     /* valid call, feature not on the GPU path */
#define ABIE_ERR_ARGUMENT (-5)
#define ABIE_ERR_CAPACITY (-6)        /* N above the capacity given to initialize_code */
#define ABIE_ERR_TIMEOUT (-7)         /* a device-side wait gave up */
#define ABIE_ERR_NUMERICS (-8)        /* NaN/Inf in the state */

/* Force forms (abie_set_force_mode). */
#define ABIE_FORCE_EXACT 0  /* reference operation order per sink: bit-identical to src/common.c:39-77 */
#define ABIE_FORCE_FP64 1   /* fast FP64: reassociated sums, refined reciprocal square root */
#define ABIE_FORCE_MIXED 2  /* FP32 pair terms on anchored coordinates, compensated sums; heavy sources in FP64 */
#define ABIE_FORCE_NAIVE 3  /* one thread per sink over global memory: src/gpuforce.cu:61-84 semantics */

/* ---- reference-compatible entry points (src/common.h:74-122) ---------- */

/* src/common.c:226-275.  Binds GPU deviceID, sizes device buffers for
 * N_MAX bodies and the event ring buffers.  Once per process, like the
 * reference (a second call returns 0 and does nothing).  A negative
 * deviceID (the reference's default, which selects its CPU code) binds
 * GPU 0, with a notice on stderr: this library has no CPU path. */
int initialize_code(double G, double C, size_t N_MAX, size_t MAX_N_CE,
                    size_t MAX_N_COLLISIONS, int deviceID);
/* src/common.c:382-398.  Frees device and host buffers. */
int finalize_code(void);
/* src/common.c:309-325.  Copies the caller's arrays into device memory. */
void set_state(double *pos, double *vel, double *m, double *r, size_t N,
               double G, double C);
/* src/common.c:327-338.  Copies the device state out; returns N. */
int get_state(double *pos, double *vel, double *m, double *r);
/* src/common.c:200-202 */
double get_model_time(void);
/* src/common.c:277-283 */
void set_close_encounter_distance(double d);
double get_close_encounter_distance(void);
/* src/common.c:285-307 (4*MAX doubles each: t, i, j, distance) */
void get_close_encounter_buffer(double *buf_ce);
void get_collision_buffer(double *buf_collision);
void reset_close_encounter_buffer(void);
void reset_collision_buffer(void);
/* src/common.c:364-380.  A constant 3N acceleration added to every force
 * call of calculate_accelerations and Radau15 (stateful and on caller
 * arrays), as the reference's calculate_accelerations adds it
 * (src/common.c:107-112).  ext_acc == NULL switches it off again (an
 * addition: the reference cannot). */
size_t set_additional_forces(size_t N, double *ext_acc);
/* src/common.c:400-403 -> src/integrator_gauss_radau15.c:221-380.
 * Gauss-Radau 15 from t to the first accepted time past t_end, on the
 * device-resident state; dt is ignored as in the reference.  With a stored
 * C > 0 the accelerations include the post-Newtonian terms
 * (src/additional_forces.c) of the massive bodies. */
int integrator_gr(double t, double t_end, double dt);
/* src/common.c:410-413 -> src/integrator_wisdom_holman.c:498-522.
 * Fixed-step Wisdom-Holman on a heliocentric state. */
int integrator_wh(double t, double t_end, double dt);
/* src/common.c:405-408 -> src/integrator_runge_kutta.c:6-50.  Classical
 * RK4 on the device-resident state in the current force form (the exact
 * form reproduces the reference's doubles for non-negative masses); like
 * the reference, it leaves the model time unchanged. */
int integrator_rk(double t, double t_end, double dt);
/* src/common.c:340-357.  Total energy of the stored state (FP64): the
 * reference's kinetic and pair terms, summed in double-double in a fixed
 * order and rounded once. */
double calculate_energy(void);
/* src/common.c:39-77 (and the GPU offload src/gpuforce.cu:129-170):
 * accelerations of N bodies from host arrays, computed on the GPU in the
 * current force form.  Does not touch the stored simulation state. */
size_t ode_n_body_second_order(const double *pos, size_t N, double G,
                               const double *masses, const double *radii,
                               double *acc);
/* src/common.c:82-114: ode_n_body_second_order, the post-Newtonian terms
 * when the stored C is positive (src/additional_forces.c:14-121: in the
 * exact form the reference's operations, bit for bit; in the fast form the
 * same terms regrouped without square root or division, within 1e-13 per
 * body), then the external accelerations set by set_additional_forces. */
size_t calculate_accelerations(const double *pos, const double *vel, size_t N,
                               double G, const double *masses,
                               const double *radii, double *acc);
/* src/integrator_gauss_radau15.c:221: Radau15 on caller arrays (the
 * state is uploaded, integrated on the device and copied back). */
size_t integrator_gauss_radau15(double *pos, double *vel, double *m_vec,
                                double *r_vec, size_t N, double G, double t,
                                double t_end, double dt);
/* src/integrator_runge_kutta.c:52-60 on caller arrays. */
void integrator_runge_kutta(double *pos, double *vel, double *m_vec,
                            double *r_vec, size_t N, double G, double t,
                            double t_end, double dt);
/* src/integrator_wisdom_holman.c:498 on caller arrays. */
void integrator_wisdom_holman(double *pos, double *vel, double *m_vec,
                              double *r_vec, size_t N, double G, double t,
                              double t_end, double dt);

/* ---- additions of this library (no counterpart in the reference) ------ */

typedef struct {
    long long force_calls;       /* all-pairs evaluations */
    long long iterations;        /* Radau15 corrector iterations */
    long long attempts;          /* Radau15 step attempts */
    long long accepts;
    long long rejects;
    long long kepler_failures;   /* WH Kepler solves that hit the iteration cap */
    long long wh_steps;
    double last_h;
    long long learned_fallbacks; /* ensemble attempts redone from the plain guess after the
                                    learned guess gave a non-finite state */
} abie_counters;

/* Last error message ("" when none). Returns its length. */
int abie_last_error(char *buf, size_t len);
/* Force form used by every later call (ABIE_FORCE_*). Returns the previous one. */
int abie_set_force_mode(int mode);
int abie_get_force_mode(void);
/* Counters since initialize_code or the last reset. */
int abie_get_counters(abie_counters *out);
void abie_reset_counters(void);
/* Device-pointer all-pairs force: d_pos[3N], d_m[N] -> d_acc[3N], all in
 * GPU memory of the initialized device, on the given CUDA stream (NULL for
 * the library's stream).  Returns when the work is queued.  Allocates
 * scratch on first use and when N grows. */
int abie_force_device(const double *d_pos, const double *d_m, size_t N,
                      double G, double *d_acc, int mode, void *stream);
/* Host-pointer force in an explicit form (copies in, computes, copies out). */
int abie_force_host(const double *pos, const double *m, size_t N, double G,
                    double *acc, int mode);
/* Energy of caller arrays, computed on the GPU (FP64). */
double abie_energy_host(const double *pos, const double *vel, const double *m,
                        size_t N, double G);

/* Batched ensemble: n_systems independent systems packed ragged; system s
 * owns bodies offsets[s] .. offsets[s+1]-1 (at most 21 bodies each).  Each
 * system is integrated with Radau15 from t0 to the first accepted time past
 * t_end, exactly as integrator_gr would integrate it alone.  pos/vel are
 * updated in place, t_out[s] receives each system's final time, status[s]
 * its return code (0, or a negative error), steps[s] its accepted steps.
 * flags: bit 0 learned predictor, bit 1 collect training samples, bit 2
 * consistent-g plain predictor (below). */
int abie_gr_ensemble(double *pos, double *vel, const double *m,
                     const long long *offsets, int n_systems, double G,
                     double t0, double t_end, double *t_out, int *status,
                     long long *steps, int flags);
/* Seconds of GPU time spent in the last abie_gr_ensemble call (the run
 * itself; the autotuner's trials are reported by abie_ensemble_last_tuning). */
double abie_last_ensemble_seconds(void);
/* The launch shape the last abie_gr_ensemble call used: *heavy_div = the
 * slowest 1 in heavy_div systems ran on four-warp groups; *source = 0 when
 * the autotuner measured it in that call (or the default applied), 1 when
 * it came from the tuner's cache file, 2 from abie_debug_ensemble_heavy;
 * *tune_seconds = GPU seconds of that call's tuning trials.  Returns the
 * number of candidate shapes timed (0 without tuning).  The tuner times
 * candidate shares on slices of the batch itself and caches the choice per
 * device, library build, force form and workload (ABIE_ENSEMBLE_TUNE=0
 * switches it off; ABIE_TUNE_CACHE names the cache file). */
int abie_ensemble_last_tuning(int *heavy_div, int *source, double *tune_seconds);

/* Device snapshots, replacing abie/integrator.py:158-204 with store_state
 * (:233-252) and Particles.calculate_aei (abie/particles.py:352-376): the
 * stored state is integrated from t to t_end in chunks of store_dt, with
 * integrate()'s schedule (next_t = t + dt - ((t + dt) % dt), dt =
 * min(store_dt, t_end - t)), by integrator_gr (integrator 0) or
 * integrator_wh with step h (integrator 1).  After each chunk the GPU keeps
 * the model time, positions, velocities, a/e/i of every body about the
 * primary (ABIE_PRIMARY_* or a body index; NaN for the primary itself) and
 * the energy; they reach the caller's arrays (max_snaps rows of 1, 3N, 3N,
 * 3N and 1 doubles, any may be NULL) once, at the end.  *n_snaps = rows
 * written.  Returns 0; an event flag 1 / 2 after storing the snapshot at the
 * event (the run stops there so that the caller can handle it); a negative
 * error, ABIE_ERR_CAPACITY when more than max_snaps chunks are needed. */
#define ABIE_PRIMARY_COM (-1)    /* "#COM#": centre of mass, total mass */
#define ABIE_PRIMARY_M_MAX (-2)  /* "#M_MAX#": the most massive body */
#define ABIE_PRIMARY_M_MIN (-3)  /* "#M_MIN#": the least massive body */
int abie_integrate_snapshots(int integrator, double t, double t_end, double store_dt, double h,
                             int primary, int max_snaps, double *snap_t, double *snap_pos,
                             double *snap_vel, double *snap_aei, double *snap_energy,
                             int *n_snaps);

/* Learned Radau15 predictor (BF16 MLP 30 -> 128 -> 128 -> 21; see
 * abie_gb300/csrc/mlp.cuh for features and targets).  abie_gr_ensemble
 * flags: bit 0 starts every step from the network's guess, with the g
 * coefficients made consistent with it (requires abie_mlp_enable(1));
 * bit 2 the same consistent g with the plain guess and no network; bit 1
 * appends training samples (64 floats each: 32 features, 32 targets) to the
 * device sample store.  tau: 7 output scales, one per coefficient order
 * (NULL: all 1). */
int abie_mlp_init(int seed, const double *tau);       /* fresh weights, zero output layer */
int abie_mlp_set_params(const float *params, int n, const double *tau);
int abie_mlp_get_params(float *params, int n);
int abie_mlp_n_params(void);
void abie_mlp_enable(int on);
void abie_mlp_set_capacity(long long samples);      /* sample store size for collection */
int abie_mlp_load_samples(const float *samples, long long rows);
long long abie_mlp_sample_count(void);
int abie_mlp_get_samples(float *out, long long rows);
void abie_mlp_clear_samples(void);
/* Network outputs (rows x 32) on the first rows stored samples. */
int abie_mlp_forward(long long rows, float *Y);
/* Loss and summed gradient over the first rows stored samples. */
int abie_mlp_loss_grad(long long rows, float *grad, double *loss);
/* Adam on random minibatches of the stored samples. */
int abie_mlp_train(int steps, int batch, double lr, int seed, double *last_loss);

/* Measured FMA throughput of the bound device in TFLOP/s (one FMA = 2
 * flops), the denominators of the compute-bound rooflines.  iters <= 0
 * picks a default length. */
int abie_measure_fp64_peak(int iters, double *tflops);
int abie_measure_fp32_peak(int iters, double *tflops);
/* The FP64 probe with only the first active_lanes (1..32) lanes of each warp
 * working, its rate counted over all 32 lanes: shows what a partly idle warp
 * costs the FP64 pipe. */
int abie_measure_fp64_issue(int active_lanes, double *tflops);
/* No counterpart in the reference.  The fast FP64 all-pairs force on device
 * pointers for callers that cannot call cudaMalloc: a real-time or
 * host-callback loop that must not block on the allocator, or a process
 * whose memory budget gives the library only the caller's own buffers.
 * Scratch is a fixed area compiled into the library, held by every GPU that
 * loads it until exit: N above ABIE_NOALLOC_MAX_BODIES (checked on the full
 * size_t) returns ABIE_ERR_CAPACITY.  It always runs the one-chunk,
 * one-sided force kernel: below 8,192 bodies that is the kernel
 * abie_force_device(ABIE_FORCE_FP64) runs; from 8,192 bodies that entry
 * point takes the symmetric or two-chunk forms, and the results agree to
 * rounding (1e-13 per body), not bit for bit.  Sinks with m < 0 keep their
 * acc entries, as in abie_force_device.  Calls share the scratch area, so
 * calls that overlap on the GPU race; order them on one stream.  The first
 * call on each device (with it current) looks up the area's device address;
 * make it before any stream capture.  Runs on the given stream (NULL: the
 * default stream) and returns once queued. */
#define ABIE_NOALLOC_MAX_BODIES 65536
int abie_force_device_noalloc(const double *d_pos, const double *d_m, size_t N,
                              double G, double *d_acc, void *stream);
/* Fixes the fast FP64 force kernel's launch shape: lanes_per_sink in
 * {1, 8, 32} and the number of source chunks; (0, 0) restores the
 * automatic choice.  For tests and the autotuner. */
void abie_debug_force_shape(int lanes_per_sink, int chunks);
/* abie_gr_ensemble: the slowest 1 in div systems (longest first) run on
 * four-warp groups; 0 restores the default (1 in 4 in the fast forms, 1 in
 * 256 in the exact form).  For tests and tuning. */
void abie_debug_ensemble_heavy(int div);
/* Fixes the Radau15 engine's launch shape: lanes per body in {1, 4, 8, 16,
 * 32} (the exact form takes 1 or 4) and threads per block (a multiple of 32
 * up to 256); 0 keeps the automatic choice.  For tests and tuning. */
void abie_debug_engine_shape(int lanes_per_body, int block);
/* Chooses the Radau15 path for systems beyond the split engine: 1 the
 * persistent engine, 2 the stepped engine (one kernel per phase, the
 * standalone force kernel for every substep; fast form without
 * post-Newtonian terms only), 0 automatic (stepped from 2^20 interactions
 * per force evaluation).  For tests and tuning. */
void abie_debug_radau_path(int path);
/* Sets the persistent Radau15 engines' grid-barrier wait limit in
 * nanoseconds (a negative value restores the automatic limit, two seconds
 * plus a term for the phase's work).  A wait past the limit stops the run
 * with ABIE_ERR_TIMEOUT and every block leaves at its next barrier.  For the
 * failure-detection tests. */
void abie_debug_engine_timeout(long long ns);

#ifdef __cplusplus
}
#endif
#endif
