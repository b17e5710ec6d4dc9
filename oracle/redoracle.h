/*
 * redoracle.h -- ORACLE: a plain-C restatement of the reference's FP64 CPU path, used
 * only as the checker by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg.  Nothing in the product links or calls it.
 *
 * Pinned against: the reference's golden TwoBody run
 * (TestRun/InputTest/Debug/TwoBody/D_cpu_ns_fs_E_result.txt), the known-answer values of
 * red.cuda.utility/red_test.cpp:592-840, the COLLISION record of
 * TestRun/InputTest/Release/N1_massive_N3_test, and fixtures made by running the
 * reference's own CPU path (built by oracle/ref.mk) -- see tests/golden/.
 *
 * The API mirrors include/redgb.h (same names with an `ro_` prefix, same units and
 * status codes) so tests can drive both the same way.
 */
#ifndef REDORACLE_H
#define REDORACLE_H

#include <stdint.h>
#include "../include/redgb_types.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ro_sys ro_sys;

int  ro_create(const rg_counts_t* n, const rg_vec_t* r, const rg_vec_t* v,
               const rg_param_t* p, const rg_body_metadata_t* md, const double* epoch,
               const double thr[RG_THRESHOLD_N], ro_sys** out);
int  ro_create_in_frame(const rg_counts_t* n, const rg_vec_t* r, const rg_vec_t* v,
                        const rg_param_t* p, const rg_body_metadata_t* md, const double* epoch,
                        const double thr[RG_THRESHOLD_N], int frame_center, ro_sys** out);
void ro_destroy(ro_sys* s);
int  ro_set_integrator(ro_sys* s, int type, double dt_day, int adaptive, double tolerance,
                       int error_check_for_tp);
int  ro_set_event_options(ro_sys* s, int close_encounter, int inner_steps,
                          double hill_factor, int event_time_mode);
int  ro_set_time(ro_sys* s, double t_day);
int  ro_step(ro_sys* s, double* dt_did_day);
int  ro_check_for_ejection_hit_centrum(ro_sys* s, int* n_handled);
int  ro_check_for_collision(ro_sys* s, int* n_handled);
int  ro_check_for_close_encounter(ro_sys* s, int* n_handled);
int  ro_check_for_rebuild_vectors(ro_sys* s, int n, int* rebuilt);
int  ro_advance(ro_sys* s, double t_stop_day, int64_t max_steps, int64_t* n_steps);
int  ro_events(ro_sys* s, rg_event_t* out, int cap, int* n);
int  ro_event_count(ro_sys* s, int* n);
int  ro_get_n_total(ro_sys* s, rg_counts_t* n, int* n_total);
int  ro_get_state(ro_sys* s, rg_vec_t* r, rg_vec_t* v, rg_param_t* p,
                  rg_body_metadata_t* md, double* t_day);
int  ro_get_state_internal(ro_sys* s, rg_vec_t* r, rg_vec_t* v, rg_param_t* p,
                           rg_body_metadata_t* md, double* t_internal);
int  ro_set_state(ro_sys* s, const rg_vec_t* r, const rg_vec_t* v);
int  ro_calc_accel(ro_sys* s, rg_vec_t* a);
int  ro_get_counters(ro_sys* s, rg_counters_t* c);
int  ro_energy(ro_sys* s, double* energy, double angmom[3]);
int  ro_get_dt(ro_sys* s, double* dt_did_day, double* dt_try_day);

/* Replay: the next `n` attempts use these trial steps (internal units) instead of the
 * controller's, so a run can be re-traced from a log of another implementation. */
int  ro_set_dt_replay(ro_sys* s, const double* dt_internal, int n);

/* Gravity of sinks [i_begin, i_end) over the reference's source ranges, without events,
 * on caller arrays (internal units).  Used to sample large systems. */
int  ro_grav_accel_rows(const rg_counts_t* n, const rg_vec_t* r, const rg_param_t* p,
                        const rg_body_metadata_t* md, int i_begin, int i_end, rg_vec_t* a);

/* tools.cpp restatements used by the known-answer tests */
double ro_calculate_radius(double m, double density);
double ro_calculate_density(double m, double radius);
double ro_calculate_mass(double radius, double density);
void   ro_calc_position_after_collision(double m1, double m2, const rg_vec_t* r1,
                                        const rg_vec_t* r2, rg_vec_t* r);
void   ro_calc_velocity_after_collision(double m1, double m2, const rg_vec_t* v1,
                                        const rg_vec_t* v2, rg_vec_t* v);
void   ro_calc_physical_properties(const rg_param_t* p1, const rg_param_t* p2, rg_param_t* p);
int    ro_kepler_equation_solver(double ecc, double mean, double eps, double* E);
int    ro_calculate_phase(double mu, const rg_orbelem_t* oe, rg_vec_t* r, rg_vec_t* v);
int    ro_calculate_orbital_element(double mu, rg_orbelem_t* oe, const rg_vec_t* r,
                                    const rg_vec_t* v);
void   ro_transform_to_bc(int n, const rg_param_t* p, rg_vec_t* r, rg_vec_t* v);

#ifdef __cplusplus
}
#endif
#endif
