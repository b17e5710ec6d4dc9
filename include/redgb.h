/*
 * redgb.h -- C ABI of the GB300 (sm_103a) implementation of red.cuda's hot path:
 * direct-summation gravity, Runge-Kutta stage combination with the embedded error
 * norm (RK4, RKF5, RKF7(8)) and close-encounter / collision-merge / ejection /
 * hit-star event detection.
 *
 * The reference has no FFI layer: the path sits behind two C++ classes,
 * `pp_disk` (red.cuda/src/red.cuda/pp_disk.h:14-195) and `integrator`
 * (red.cuda/src/red.cuda/integrator.h:17-88), built by `options::create_pp_disk` /
 * `options::create_integrator` (red.cuda/src/red.cuda/options.cpp:197-274) and driven by
 * the time loop in red.cuda/src/red.cuda/main.cu:176-263.  Every entry point below
 * names the reference member function it replaces.
 *
 * Conventions
 *  - plain pointers and sizes, no C++ or torch types; every call returns an int status
 *    (RG_OK == 0, negative on error) instead of throwing, and rg_last_error() gives the
 *    message of the calling thread's last failure;
 *  - records use the reference's own layouts (red.cuda/red.type/red_type.h, as compiled
 *    on Linux: natural alignment, no forced 16-byte alignment); sizes are asserted in
 *    redgb_types.h;
 *  - caller-facing units are the reference's file units: AU, solar masses, days and
 *    AU/day; internally time runs in units of 1/k days (k = Gauss' constant) exactly as
 *    in the reference (pp_disk.cu:1512-1551, integrator.cu:29) so that G = 1;
 *  - one context drives one GPU (the device current at rg_create) on its own stream.
 */
#ifndef REDGB_H
#define REDGB_H

#include <stddef.h>
#include <stdint.h>

#include "redgb_types.h"

#if defined(__GNUC__)
#define RG_API __attribute__((visibility("default")))
#else
#define RG_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status codes */
enum {
    RG_OK                  = 0,
    RG_ERR_ARG             = -1,  /* bad argument (null pointer, size, enum value)       */
    RG_ERR_CUDA            = -2,  /* a CUDA runtime call or kernel launch failed          */
    RG_ERR_EVENT_OVERFLOW  = -3,  /* more events in one step than the event buffer holds  */
    RG_ERR_DT_NONFINITE    = -4,  /* the step-size controller produced inf/nan or 0       */
    RG_ERR_STATE           = -5,  /* call out of order (e.g. rg_step before an integrator) */
    RG_ERR_NOT_IMPLEMENTED = -6,  /* reference refuses it too (super-planetesimal merge)  */
    RG_ERR_NOMEM           = -7,  /* device or host allocation failed                     */
    RG_ERR_NO_DEVICE       = -8   /* no CUDA device / the library was built without one   */
};

/* gravity kernels */
enum {
    RG_GRAVITY_FP64  = 0, /* FP64, reference operation order, bit-identical to the CPU path */
    RG_GRAVITY_MIXED = 1  /* FP64 displacements, FP32 rsqrt + FP64 Newton, compensated FP32 */
};

/* semantics switches (both default to the reference's CPU path, the oracle) */
enum {
    RG_EVENT_TIME_CPU   = 0, /* NSI/NI sinks stamp events with the step-start time
                                (pp_disk.cu:576,581)                                        */
    RG_EVENT_TIME_STAGE = 1  /* every sink stamps its stage time (GPU path, pp_disk.cu:279)  */
};

/* ------------------------------------------------------------------ library */

/* Message of the calling thread's most recent failed call ("" if none). */
RG_API const char* rg_last_error(void);

/* Library version string and the device architecture it was compiled for. */
RG_API const char* rg_version(void);

/* Number of CUDA devices visible to the library (0 if none).  Never fails. */
RG_API int rg_device_count(void);

/* ------------------------------------------------------------------ one disk */

typedef struct rg_ctx rg_ctx;

/*
 * Replaces pp_disk::pp_disk + pp_disk::load (pp_disk.cu:1204-1235,1614-1683) and the
 * set-up in options::create_pp_disk (options.cpp:197-235): bodies are given in the
 * reference's storage order (stars, giants, rocky, proto, super-planetesimals,
 * planetesimals, test particles -- the counts in `n`), in AU and AU/day.  As in the
 * reference the system is moved to its barycentre if body 0 sits at rest in the origin,
 * velocities and epochs are rescaled to internal time units, and `thr` (the five
 * threshold_t values, red_type.h:46-54) is copied as by pp_disk::copy_threshold
 * (pp_disk.cu:1441-1452).  `epoch` may be NULL.  `event_capacity` bounds the number
 * of raw event records one step may produce (0 -> max(n_total, 1024)); the reference
 * sizes this buffer to n_total and never checks it (pp_disk.cu:1262,1267).
 */
RG_API int rg_create(const rg_counts_t* n, const rg_vec_t* r, const rg_vec_t* v,
              const rg_param_t* p, const rg_body_metadata_t* md, const double* epoch,
              const double thr[RG_THRESHOLD_N], int event_capacity, rg_ctx** out);

/*
 * rg_create in a chosen frame: frame_center is RG_FRAME_BARY (rg_create) or RG_FRAME_ASTRO,
 * the reference's parameter-file key `frame_center` (parameter.cpp:257-266) as
 * options::create_pp_disk applies it (options.cpp:206-220): a system whose body 0 sits at
 * rest in the origin is moved to its barycentre in the barycentric frame; any other system
 * is moved to body 0, the star, in the astrocentric frame (tools.cpp:180-236).  The
 * astrocentric frame follows the reference's CPU path: the self-interacting block's sinks
 * and sources start at body 1 (number_of_bodies.cpp:205-222), each sink starts from the
 * star's pull and every source adds its direct term and subtracts its indirect term
 * (pp_disk.cu:413-454), the star's own acceleration stays zero, and close-encounter
 * elements use the coordinates as they are (pp_disk.cu:554-560).  RG_ERR_NOT_IMPLEMENTED
 * for the astrocentric frame with super-planetesimals, planetesimals or test particles:
 * their blocks take the star, at the origin, as a source whose indirect term is
 * m / (0 sqrt(0)) 0, so the reference's own run turns NaN at its first step; and for
 * mixed-precision gravity (rg_set_gravity_mode) in that frame.
 */
RG_API int rg_create_in_frame(const rg_counts_t* n, const rg_vec_t* r, const rg_vec_t* v, const rg_param_t* p,
                              const rg_body_metadata_t* md, const double* epoch, const double thr[RG_THRESHOLD_N],
                              int event_capacity, int frame_center, rg_ctx** out);

/* Frees every host and device buffer of the context (pp_disk::~pp_disk, pp_disk.cu:1237). */
RG_API int rg_destroy(rg_ctx* ctx);

/*
 * Replaces options::create_integrator (options.cpp:237-274) and the integrator
 * constructors (integrator.cu:27-52, int_rungekutta4.cu:102, int_rungekutta8.cu:463).
 * `type` is an integrator_type_t: RG_INT_EULER, RG_INT_RK4, RG_INT_RK5 (Cash-Karp,
 * restated from int_rungekutta5.cu, which does not build in the reference) or
 * RG_INT_RKF78.  `dt_day` is the first trial step in days (main.cu:141 uses 0.001).
 */
RG_API int rg_set_integrator(rg_ctx* ctx, int type, double dt_day, int adaptive, double tolerance,
                      int error_check_for_tp);

/*
 * The reference's event switches: `close_encounter` and `inner_steps`
 * (parameter.cpp:36-37,160-190; pp_disk.h:126-127).  `hill_factor` > 0 additionally
 * logs a CLOSE_ENCOUNTER for every interacting pair closer than hill_factor mutual
 * Hill radii (not in the reference; 3 for the planetesimal-disk workloads).
 * `event_time_mode` is RG_EVENT_TIME_CPU (default) or RG_EVENT_TIME_STAGE.
 */
RG_API int rg_set_event_options(rg_ctx* ctx, int close_encounter, int inner_steps,
                         double hill_factor, int event_time_mode);

/* Selects the gravity kernel (RG_GRAVITY_FP64 default, RG_GRAVITY_MIXED). */
RG_API int rg_set_gravity_mode(rg_ctx* ctx, int mode);

/* Sets the simulation clock in days (pp_disk::t = parameter::start_time). */
RG_API int rg_set_time(rg_ctx* ctx, double t_day);

/*
 * One integration step with the reference's step-size control: replaces
 * rungekutta4::step (int_rungekutta4.cu:189-273), rungekutta5::step
 * (int_rungekutta5.cu:202-282), rungekutta8::step (int_rungekutta8.cu:704-797) and
 * euler::step.  Collision / close-encounter records found in the stages are kept for
 * rg_check_for_collision exactly as the reference keeps them in d_events.
 */
RG_API int rg_step(rg_ctx* ctx, double* dt_did_day);

/* pp_disk::check_for_ejection_hit_centrum (pp_disk.cu:683-715) with its handler
 * (pp_disk.cu:1091-1109): `n_handled` receives the number of events. */
RG_API int rg_check_for_ejection_hit_centrum(rg_ctx* ctx, int* n_handled);

/* pp_disk::check_for_collision (pp_disk.cu:717-738): dedup per pair keeping the
 * earliest record (pp_disk.cu:1111-1149) and merge (pp_disk.cu:1151-1202). */
RG_API int rg_check_for_collision(rg_ctx* ctx, int* n_handled);

/* pp_disk::check_for_close_encounter(true) (pp_disk.cu:742-770): moves the recorded
 * close encounters into the event log. */
RG_API int rg_check_for_close_encounter(rg_ctx* ctx, int* n_handled);

/* pp_disk::check_for_rebuild_vectors (pp_disk.cu:893-907): compacts the storage once
 * at least `n` events have been handled since the last compaction. */
RG_API int rg_check_for_rebuild_vectors(rg_ctx* ctx, int n, int* rebuilt);

/*
 * The time loop of main.cu:176-263 without file output: ejection / hit-star check,
 * step, collision or close-encounter handling and compaction, repeated while
 * t <= t_stop_day (main.cu:176) and fewer than `max_steps` steps were taken
 * (max_steps <= 0: no limit).  `n_steps` (may be NULL) receives the steps taken.
 */
RG_API int rg_advance(rg_ctx* ctx, double t_stop_day, int64_t max_steps, int64_t* n_steps);

/*
 * Drains the event log: the records pp_disk::print_event_data writes
 * (pp_disk.cu:1772-1848), in the order it writes them, with the reference's internal
 * units (t in 1/k days, velocities in AU per 1/k days).  Copies at most `cap`
 * records, returns the number copied in *n and removes them from the log.
 */
RG_API int rg_events(rg_ctx* ctx, rg_event_t* out, int cap, int* n);
RG_API int rg_event_count(rg_ctx* ctx, int* n);

/* Current body count (active + inactive until the next compaction). */
RG_API int rg_get_n_total(rg_ctx* ctx, rg_counts_t* n, int* n_total);

/*
 * Copies the state out in the reference's record layouts and file units (AU, AU/day,
 * days), like pp_disk::copy_to_host + print_result_ascii (pp_disk.cu:1426,1685).
 * Any output pointer may be NULL.  Arrays must hold n_total records.
 */
RG_API int rg_get_state(rg_ctx* ctx, rg_vec_t* r, rg_vec_t* v, rg_param_t* p,
                 rg_body_metadata_t* md, double* t_day);

/* Same, in internal units (velocities in AU per 1/k days), bit-exact device contents. */
RG_API int rg_get_state_internal(rg_ctx* ctx, rg_vec_t* r, rg_vec_t* v, rg_param_t* p,
                          rg_body_metadata_t* md, double* t_internal);

/* Replaces the positions and velocities (file units) of all n_total bodies. */
RG_API int rg_set_state(rg_ctx* ctx, const rg_vec_t* r, const rg_vec_t* v);

/* One force evaluation at the current state (pp_disk::calc_dydx(1, ...),
 * pp_disk.cu:998-1041) in internal units; events it finds are discarded. */
RG_API int rg_calc_accel(rg_ctx* ctx, rg_vec_t* a);

/*
 * Autotuner (not in the reference): times every candidate launch shape of the force
 * evaluation in the current gravity mode on the current state (`reps` evaluations each,
 * CUDA events on the context's stream) and keeps the fastest.  FP64 mode: sinks per
 * pair-parallel CTA x the row-kernel source limit -- every candidate sums in the same
 * order, so results stay bit-exact; mixed mode: first the row-kernel limit, then the mixed
 * kernel's sources per grid.y chunk (whole tiles of 256 sources: for each chunk count up to
 * 24 the smallest chunk that gives it and one tile less, so that the grid's last wave of
 * CTAs can be filled; reported in `mixed_chunks`, 0 = from the SM count).  Counters are left
 * as they were.  `out` (may be NULL) receives the choice.
 */
RG_API int rg_autotune(rg_ctx* ctx, int reps, rg_tune_t* out);

/*
 * Sets the launch shape directly (not in the reference): `shape->pairpar_sinks` (8, 12, 16,
 * 18, 24, 32 or 36; 8, 16 or 32 in the astrocentric frame), `rowseq_max_src` (>= 1) and
 * `mixed_chunks` (0 = from the SM count, else a positive multiple of 256 sources); the other
 * fields are ignored.  For a run that reuses the shape an earlier rg_autotune chose on the
 * same kind of disk without timing the candidates again.  FP64 results do not depend on the
 * shape.  RG_ERR_ARG for a value outside those sets.
 */
RG_API int rg_set_launch_shape(rg_ctx* ctx, const rg_tune_t* shape);

/* Synthetic disks generated on the GPU (the seeded initial-condition generator of this
 * project; the reference's own generator is the separate red.cuda.initial program): disk s
 * gets the records [off_s, off_s + n_total_s) of r, v (AU, AU/day, heliocentric), p and md,
 * off_s the sum of the previous disks' totals, and its body counts in counts[s].  One thread
 * per body; each body's random numbers come from Philox4x32-10 with the disk's seed as the
 * key and (body slot, draw block) as the counter, so the result does not depend on the
 * launch shape; orbital elements go to Cartesian by the reference's calculate_phase
 * (tools.cpp:292-359).  Invalid specifications return RG_ERR_ARG. */
RG_API int rg_generate_disks(int n_sys, const rg_disk_spec_t* specs, rg_counts_t* counts, rg_vec_t* r,
                             rg_vec_t* v, rg_param_t* p, rg_body_metadata_t* md);

/*
 * Disks from per-body-type distributions, on the GPU: the reference's initial-condition
 * program (red.cuda.initial populate_disk, main.cu:29-86, and its driver, main.cu:470-538)
 * for many disks at once.  Per body: the physical properties (mass, radius, density, drag
 * coefficient) from their distributions, the one of mass, radius and density that is not
 * given derived from the other two (tools.cpp:238-261; superplanetesimals keep what they
 * drew); the orbital elements (the star: all 0).  Per disk, when pp_total_mass > 0: the
 * protoplanets' masses scaled to that sum (summed from the last body down, as
 * tools::get_total_mass does) and their radius or density derived again.  Then positions
 * and velocities by calculate_phase with mu = k^2 (m_0 + m_i), m_0 the disk's first body,
 * which sits at rest in the origin; with to_bc the disk is moved to its barycentre
 * (tools::transform_to_bc).  Draws: Philox4x32-10 keyed by the disk's seed, counter (body
 * slot, item, attempt), so a disk does not depend on its batch.  The power law repeats the
 * reference's rejection steps (at most 10 000 attempts); the lognormal, whose rejection in
 * the reference samples the true truncated density, is drawn by its inverse distribution
 * function.  The reference's element ranges are not part of the spec, since its redraw
 * condition (util_init.cpp:61-69) can never hold.  Disk s gets the records
 * [off_s, off_s + n_s) of r, v (AU, AU/day), p and md (ids 1..n_s) and counts[s].
 * RG_ERR_ARG: an invalid distribution, a body type with other than exactly one of mass,
 * radius and density missing ("Missing physical parameters!" in the reference), a phase the
 * Kepler solver does not converge for, a mass scaling that misses its target by more than
 * 1e-15 (the reference's own checks), or a power-law draw that reached its attempt limit.
 */
RG_API int rg_populate_disks(int n_sys, const rg_body_disk_t* disks, rg_counts_t* counts, rg_vec_t* r,
                             rg_vec_t* v, rg_param_t* p, rg_body_metadata_t* md);

/* Masses of a minimum-mass solar nebula's gas and solids (Hayashi 1981; red.cuda.initial
 * nebula.cpp:23-95): the integral of 2 pi r Sigma(r), Sigma = f_neb Sigma_1 r^p times the gas
 * ratio (gas) or, beyond the snow line, the ice factor (solids), over [r_1, r_2]. */
RG_API int rg_mmsn_gas_mass(const rg_mmsn_component_t* c, double* m);
RG_API int rg_mmsn_solid_mass(const rg_mmsn_component_t* c, double* m);

/* Test hook for the failure path (no counterpart in the reference): with `on`, the mixed
 * kernel issues none of its tile copies, so each CTA's bounded wait (one second of the GPU's
 * global timer) runs out; the evaluation then reports RG_ERR_CUDA ("a gravity tile copy did
 * not arrive within the wait limit") and the context stays usable.  Nothing faults: the
 * kernel waits on its own barriers, stops waiting and returns. */
RG_API int rg_test_hold_tile_copies(rg_ctx* ctx, int on);

/* Integrator and event counters (integrator.cu:258-278, pp_disk.h:129-133). */
RG_API int rg_get_counters(rg_ctx* ctx, rg_counters_t* c);

/* Total energy and angular momentum over the force model's pair set (internal units,
 * G = 1), FP64 with compensated sums.  Not in the reference. */
RG_API int rg_energy(rg_ctx* ctx, double* energy, double angmom[3]);

/*
 * No counterpart in the reference.  rg_energy for a caller that cannot allocate device
 * memory -- one that owns a fixed memory budget it has already handed out (an arena or
 * pool sized at start-up, as a host code that keeps the reference's pp_disk device arrays
 * does), or that must not let a library call cudaMalloc / cudaFree, which synchronise the
 * device, in the middle of its loop.  The bodies are the caller's device arrays in the
 * reference's layouts and internal units (velocities in AU per 1/k days, as pp_disk keeps
 * them): n_total = the sum of *counts records each of r, v, p and md, in the reference's
 * body order.  Same results as rg_energy on the same state.
 *
 * The call allocates nothing: its scratch is a fixed device array of
 * RG_ENERGY_NOALLOC_MAX_BODIES bodies (2.5 MiB per device, part of the library image), and
 * a larger n_total is rejected with RG_ERR_ARG before any device work.  The first call on
 * each device looks the scratch's address up with that device current and keeps it for
 * later calls.  That address belongs to the CUDA runtime's primary context of the device:
 * callers that make their own driver-API context current are not supported, and a
 * cudaDeviceReset invalidates the kept address.  Nothing in the scratch needs to start at
 * zero.  There is one scratch per device, so calls on the same device must not overlap
 * (from two threads, or on two streams with both in flight): they would race on it.
 * The work runs on `stream` (NULL: the legacy default stream), and the call copies the
 * four results to the host and synchronises that stream before it returns.  It therefore
 * cannot be made on a stream that is being captured into a CUDA graph, nor on the legacy
 * NULL stream while any global-mode capture is in progress.
 */
#define RG_ENERGY_NOALLOC_MAX_BODIES 65536
RG_API int rg_energy_noalloc(const rg_counts_t* counts, const rg_vec_t* r, const rg_vec_t* v, const rg_param_t* p,
                             const rg_body_metadata_t* md, void* stream, double* energy, double angmom[3]);

/* Last step-size values in days: the step that was taken and the next trial step. */
RG_API int rg_get_dt(rg_ctx* ctx, double* dt_did_day, double* dt_try_day);

/* ------------------------------------------------------------------ ensembles */

/*
 * Many independent disks integrated together on one GPU (not in the reference, which
 * runs one disk per process).  Every disk follows the reference's RKF7(8) adaptive step
 * (int_rungekutta8.cu:704-797) with its own step size and clock; the step-size controller
 * runs on the device.  Collisions, ejections and hit-star events follow the reference's
 * rules (pp_disk.cu:683-1202) and are applied on the device right after the attempt that
 * found them (merges, retirements, the event records), as are the Hill-sphere records, so
 * rg_ens_advance is one CUDA-graph launch whose conditional while-node repeats the attempt
 * until every disk is done (in chunks of at most 4096 attempts per launch; the host only
 * reads whether to launch the next).  Differences from rg_advance: the controller's pow and
 * the merged radius's pow (tools.cpp:238-243) are the device's, which may differ from
 * glibc's in the last bit, and inactive bodies stay in storage (no compaction; indices do
 * not change).  Each disk has its own thresholds, collision factor included.
 */
typedef struct rg_ens rg_ens;

/* Bodies of disk s are records [off_s, off_s + n_total_s) of the arrays, off_s the sum of
 * the previous disks' totals; `thr` holds RG_THRESHOLD_N values per disk. */
RG_API int rg_ens_create(int n_sys, const rg_counts_t* counts, const rg_vec_t* r, const rg_vec_t* v,
                         const rg_param_t* p, const rg_body_metadata_t* md, const double* thr,
                         int event_capacity, rg_ens** out);
RG_API int rg_ens_destroy(rg_ens* ens);

/* RKF7(8) with tolerance `tol` (the only integrator of the ensemble), first trial step
 * dt_day for every disk. */
RG_API int rg_ens_set_integrator(rg_ens* ens, double dt_day, double tol, int error_check_for_tp);

/* gravity mode (RG_GRAVITY_*), Hill-sphere close-encounter factor (0: off), CUDA graphs
 * on/off (on by default). */
RG_API int rg_ens_set_options(rg_ens* ens, int gravity_mode, double hill_factor, int use_graph);

/* Integrates every disk until its clock exceeds t_stop_day (the reference's
 * `while (t <= stop)` loop) or max_attempts attempts (<= 0: no limit) were run.  Event
 * records of the interval are appended to the log rg_ens_events drains (at most
 * 16 x the body count, between 4096 and 2^18 records per call: RG_ERR_EVENT_OVERFLOW beyond). */
RG_API int rg_ens_advance(rg_ens* ens, double t_stop_day, int64_t max_attempts, int64_t* n_attempts);

/* State of disk `sys` in file units (arrays of its n_total records; any may be NULL). */
RG_API int rg_ens_get_state(rg_ens* ens, int sys, rg_vec_t* r, rg_vec_t* v, rg_param_t* p,
                            rg_body_metadata_t* md, double* t_day);
RG_API int rg_ens_get_stats(rg_ens* ens, int sys, rg_ens_stats_t* stats);

/* Drains the event log of all disks (records as rg_events; sys_of_event[k] = disk). */
RG_API int rg_ens_events(rg_ens* ens, rg_event_t* out, int* sys_of_event, int cap, int* n);
RG_API int rg_ens_event_count(rg_ens* ens, int* n);

/* Drains the log of attempts (one record per disk and attempt, in launch order per disk)
 * recorded since the last call; at most `cap` records.  Logging is on when
 * rg_ens_set_step_log(ens, capacity) gave a capacity > 0. */
RG_API int rg_ens_set_step_log(rg_ens* ens, int capacity);
RG_API int rg_ens_step_log(rg_ens* ens, rg_step_rec_t* out, int cap, int* n);

/* Energy and angular momentum of disk `sys` (as rg_energy). */
RG_API int rg_ens_energy(rg_ens* ens, int sys, double* energy, double angmom[3]);

/* Kernel timing of the ensemble (no counterpart in the reference): with `on`, every attempt
 * is launched directly, not as a graph replay, with CUDA events on the ensemble's stream
 * around its force evaluations (gravity), its stage combinations and error norm (stage),
 * and its other kernels (state copy, ejection screen, controller, features: other);
 * rg_ens_get_profile sums their device times since the last call. */
RG_API int rg_ens_set_profiling(rg_ens* ens, int on);
RG_API int rg_ens_get_profile(rg_ens* ens, rg_profile_t* prof);

/* The stream the ensemble launches on, and its kernel-launch count. */
RG_API int rg_ens_get_stream(rg_ens* ens, void** stream);
RG_API int rg_ens_kernel_count(rg_ens* ens, int64_t* n_kernels, int64_t* n_graph_launches);

/* Tile-shape autotuner of the ensemble (no counterpart in the reference, which has one
 * launch shape per kernel): times one gravity evaluation of every disk for each candidate
 * shape of the current gravity mode (`reps` evaluations each, CUDA events on the ensemble's
 * stream) and keeps the fastest.  FP64 mode: sinks per pair-parallel CTA x the row-kernel
 * source limit -- every candidate sums in the reference's order, so results stay bit-exact;
 * mixed mode: sources per few-sink CTA -- for disks of a few heavy bodies and many light
 * ones, the light bodies per CTA of the symmetric heavy-light kernel, about, in whole waves
 * (0 = automatic, about 2048; 512, 1024, 2048; reported in `mixed_chunks`) -- x the row-kernel
 * limit.  The ensemble's state is not changed.  `out` (may be NULL) receives the choice. */
RG_API int rg_ens_autotune(rg_ens* ens, int reps, rg_tune_t* out);

/* ------------------------------------------------------------------ learned step proposer */

/*
 * A small perceptron (8 inputs -> 64 -> 64 -> 1, SiLU, BF16 weights, FP32 accumulation)
 * that proposes each disk's next trial step from features the integrator logs (not in the
 * reference).  Trained on the GPU by the library's own forward / backward / AdamW kernels.
 * Parameter vector layout (RG_MLP_NPARAM FP32 values): W1[64][8] b1[64] W2[64][64] b2[64]
 * w3[64] b3.  Inputs are standardised with (x - mean) / std before the first layer.
 */
#define RG_MLP_IN 8
#define RG_MLP_NPARAM 4801
typedef struct rg_mlp rg_mlp;

RG_API int rg_mlp_create(uint64_t seed, rg_mlp** out);
RG_API int rg_mlp_destroy(rg_mlp* mlp);
RG_API int rg_mlp_set_normalisation(rg_mlp* mlp, const float mean[RG_MLP_IN], const float stdev[RG_MLP_IN]);
RG_API int rg_mlp_get_normalisation(rg_mlp* mlp, float mean[RG_MLP_IN], float stdev[RG_MLP_IN]);
RG_API int rg_mlp_get_params(rg_mlp* mlp, float* params, int n);
RG_API int rg_mlp_set_params(rg_mlp* mlp, const float* params, int n);
/* predictions for n samples (x: n x RG_MLP_IN, raw features) */
RG_API int rg_mlp_forward(rg_mlp* mlp, const float* x, int n, float* y);
/* gradient of the mean squared error over the n samples (no update) */
RG_API int rg_mlp_gradient(rg_mlp* mlp, const float* x, const float* y, int n, float* grads, float* loss);
/* AdamW over `epochs` shuffled passes in minibatches of `batch` */
RG_API int rg_mlp_train(rg_mlp* mlp, const float* x, const float* y, int n, int epochs, int batch, float lr,
                        float weight_decay, uint64_t seed, float* final_loss);

/*
 * Attaches a trained network to an ensemble (NULL detaches).  The network predicts
 * log(ideal step / last ideal step), where a step's ideal size is the one the controller's
 * error model says meets the tolerance exactly, dt * (tol / err)^(1/8).  At the start of
 * every step a disk's trial step becomes safety * last ideal step * exp(network(features)),
 * bounded to [1/2, 2] times the plain controller's own estimate; the embedded RKF error
 * estimate accepts or rejects it, a rejected attempt retries with the plain controller's
 * step, and after two steps in a row whose proposals were rejected the disk uses the plain
 * controller alone for `cooldown` steps.  Features (rg_step_rec_t.feat): log10 min(d /
 * mutual Hill radius) over pairs with a massive non-star body, log10 max |a|, log10 last
 * accepted dt [day], log10 last error / tolerance, last attempt accepted (0/1), log of the
 * last three ratios of consecutive ideal steps.
 */
RG_API int rg_ens_set_proposer(rg_ens* ens, rg_mlp* mlp, double safety, int cooldown);
/*
 * Training-data collection: every step whose trial size comes from the plain controller
 * starts from that size times exp(sigma * u), u uniform in [-1, 1) from (seed, disk, step),
 * so that the attempt log covers error ratios away from the plain controller's fixed point.
 * The error estimate still accepts or rejects every attempt.  sigma in [0, 1]; 0 is off.
 */
RG_API int rg_ens_set_dither(rg_ens* ens, double sigma, uint64_t seed);

/* ------------------------------------------------------------------ measurement */

/* The CUDA stream (cudaStream_t) the context launches on, for callers that time or
 * order their own work against it. */
RG_API int rg_get_stream(rg_ctx* ctx, void** stream);

/* Records CUDA events around every force evaluation and stage kernel of the context
 * (on its stream) when `on` is non-zero; rg_get_profile sums their device times. */
RG_API int rg_set_profiling(rg_ctx* ctx, int on);
RG_API int rg_get_profile(rg_ctx* ctx, rg_profile_t* prof);

/* Measured throughput of one arithmetic pipe of the current device, in TFLOP/s
 * (an FMA counts 2): kind 0 = FP32 FMA, 1 = FP64 FMA.  A chain of independent FMAs
 * per thread on every SM, timed with CUDA events. */
RG_API int rg_measure_pipe_peak(int kind, double* tflops);

#ifdef __cplusplus
}
#endif

#endif /* REDGB_H */
