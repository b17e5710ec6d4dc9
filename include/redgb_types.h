/*
 * redgb_types.h -- record layouts and enumerations shared by the C ABI (redgb.h), the
 * CUDA library and the CPU oracle.  They are the reference's own types
 * (red.cuda/red.type/red_type.h) as laid out by gcc on Linux, where __BUILTIN_ALIGN__
 * is empty (red_type.h:117-121): natural alignment, so a body file written by the
 * reference, or a record array handed over by reference-side code, can be passed in
 * unchanged.
 */
#ifndef REDGB_TYPES_H
#define REDGB_TYPES_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* red_type.h:136-143 vec_t (w is always 0; it only pads the record to 32 bytes) */
typedef struct rg_vec { double x, y, z, w; } rg_vec_t;

/* red_type.h:146-152 param_t */
typedef struct rg_param { double mass, radius, density, cd; } rg_param_t;

/* red_type.h:155-161 body_metadata_t (24 bytes: 3 int32 + 4 pad + double) */
typedef struct rg_body_metadata {
    int32_t id;
    int32_t body_type;
    int32_t mig_type;
    double  mig_stop_at;
} rg_body_metadata_t;

/* red_type.h:101-115 orbelem_t */
typedef struct rg_orbelem { double sma, ecc, inc, peri, node, mean; } rg_orbelem_t;

/* red_type.h:230-277 event_data_t, 472 bytes */
typedef struct rg_event {
    int32_t      event_name;   /* event_name_t                                */
    double       t;            /* time of the event (internal units)          */
    double       d;            /* distance of the bodies                      */
    int32_t      id1, idx1;    /* survivor                                    */
    rg_param_t   p1;
    rg_vec_t     r1, v1;
    rg_orbelem_t oe1;
    int32_t      id2, idx2;    /* merger                                      */
    rg_param_t   p2;
    rg_vec_t     r2, v2;
    rg_orbelem_t oe2;
    rg_param_t   ps;           /* survivor after the event                    */
    rg_vec_t     rs, vs;
    rg_orbelem_t oes;
} rg_event_t;

/* number_of_bodies constructor arguments (number_of_bodies.h:7) */
typedef struct rg_counts {
    int32_t n_s, n_gp, n_rp, n_pp, n_spl, n_pl, n_tp;
} rg_counts_t;

/* integrator counters (integrator.h:65-67) and event counters (pp_disk.h:129-133) */
typedef struct rg_counters {
    int64_t n_failed_step, n_passed_step, n_tried_step;
    int64_t n_hit_centrum[3], n_ejection[3], n_collision[3], n_close_encounter[3], n_event[3];
    int64_t n_gravity_evals;   /* force evaluations (not in the reference) */
    int64_t n_pairs;           /* interacting pairs evaluated              */
    int64_t n_kernels;         /* CUDA kernels launched by the library     */
} rg_counters_t;

/* kernel timing of a context (rg_set_profiling): CUDA events around every launch */
typedef struct rg_profile {
    int64_t gravity_launches;  /* force evaluations timed                                */
    double  gravity_ms;        /* their summed device time                               */
    int64_t stage_launches;    /* stage-combine / error kernels timed                    */
    double  stage_ms;
    int64_t other_launches;    /* the rest of a step: state copy, ejection / hit-star
                                  screen, step-size controller, features (ensembles)     */
    double  other_ms;
} rg_profile_t;

/* one synthetic disk for rg_generate_disks: a 1 Msun star at rest in the origin, giants on
 * the given orbits (random mean anomaly and argument of pericentre, i = 0), n_pl bodies of
 * type pl_type (RG_BODY_PROTOPLANET: self-gravitating, or RG_BODY_PLANETESIMAL) and n_tp test
 * particles */
typedef struct rg_disk_spec {
    uint64_t seed;           /* key of the disk's Philox4x32-10 streams                       */
    int32_t  n_pl, pl_type, n_tp, n_giants;  /* n_giants <= 4                                  */
    double   giant_m[4], giant_a[4], giant_e[4];  /* [Msun], [AU]; radii from 1.33 g/cm^3      */
    double   m_lo, m_hi;     /* planetesimal masses, log-uniform [Msun]                      */
    double   a_lo, a_hi;     /* semi-major axes [AU]                                          */
    int32_t  a_mode;         /* 0: Sigma ~ r^-1.5 (dN/da ~ a^-0.5); 1: uniform (also the TPs' rule) */
    int32_t  pad;
    double   sigma_e, sigma_i;  /* Rayleigh scales of e (capped at 0.9) and i [rad]           */
    double   rho_pl;         /* planetesimal density [g/cm^3]                                 */
} rg_disk_spec_t;

/* The distributions of the reference's initial-condition program (red.cuda.initial
 * distribution.h:34-119), one per orbital element and physical property of a body type.
 * Parameters by kind (u uniform on (0, 1]):                                                */
enum {
    RG_DIST_NONE = 0,        /* not given: the element is 0; of mass, radius and density the
                                one not given is derived from the other two               */
    RG_DIST_UNIFORM = 1,     /* p[0] x_min, p[1] x_max: x_min + (x_max - x_min) u           */
    RG_DIST_EXPONENTIAL = 2, /* p[0] lambda: -log(u) / lambda                               */
    RG_DIST_RAYLEIGH = 3,    /* p[0] sigma: sigma sqrt(-2 log u)                            */
    RG_DIST_NORMAL = 4,      /* p[0] mean, p[1] scale (the reference calls it variance):
                                mean + scale sqrt(-2 log u) cos(2 pi u')                   */
    RG_DIST_POWER_LAW = 5,   /* p[0] x_min > 0, p[1] x_max, p[2] power: the reference's
                                rejection steps, density ~ x^power - min(x_min^power,
                                x_max^power)                                               */
    RG_DIST_LOGNORMAL = 6,   /* p[0] x_min, p[1] x_max, p[2] mu, p[3] sigma: lognormal
                                density truncated to [x_min, x_max]                        */
    RG_DIST_LOG_UNIFORM = 7  /* p[0] x_min > 0, p[1] x_max (not in the reference)          */
};
typedef struct rg_dist {
    int32_t kind;
    int32_t pad;
    double  p[4];
} rg_dist_t;

enum { RG_OE_SMA = 0, RG_OE_ECC = 1, RG_OE_INC = 2, RG_OE_PERI = 3, RG_OE_NODE = 4, RG_OE_MEAN = 5, RG_OE_N = 6 };
enum { RG_PP_MASS = 0, RG_PP_RADIUS = 1, RG_PP_DENSITY = 2, RG_PP_DRAG_COEFF = 3, RG_PP_N = 4 };

/* one disk for rg_populate_disks (red.cuda.initial's body_disk_t, main.cu:29-86 and the
 * driver steps of main.cu:470-538) */
typedef struct rg_body_disk {
    uint64_t  seed;                 /* key of the disk's Philox4x32-10 streams                */
    int32_t   n_body[7];            /* per body type, the reference's order (star first)      */
    int32_t   to_bc;                /* 1: move the disk to its barycentre (transform_to_bc)   */
    double    pp_total_mass;        /* > 0: scale the protoplanets' masses to this sum [Msun]
                                       and re-derive their radius or density                 */
    rg_dist_t oe[7][RG_OE_N];       /* sma [AU], ecc, inc, peri, node, mean [rad]; star: none */
    rg_dist_t pp[7][RG_PP_N];       /* mass [Msun], radius [AU], density [Msun/AU^3], cd      */
} rg_body_disk_t;

/* one component of a minimum-mass solar nebula (red.cuda.initial nebula.h:5-48) */
typedef struct rg_mmsn_component {
    double r_1, r_2;   /* inner and outer radius [AU]                                          */
    double r_SL;       /* the snow line [AU]                                                   */
    double f_neb;      /* nebular mass factor (1: the MMSN)                                    */
    double Sigma_1;    /* surface density of solids at 1 AU [mass / AU^2]                     */
    double f;          /* gas: the gas-to-dust ratio; solids: the ice condensation factor      */
    double p;          /* profile index of the surface density                                 */
} rg_mmsn_component_t;

/* launch shape of a context's force evaluation (rg_autotune) */
typedef struct rg_tune {
    int32_t pairpar_sinks;   /* FP64 mode: sinks per pair-parallel CTA (8, 12, 16, 18, 24, 32, 36) */
    int32_t rowseq_max_src;  /* blocks with at most this many sources use the row kernel         */
    int32_t mixed_chunks;    /* mixed mode: sources per grid.y chunk -- of the mixed kernel
                                (rg_autotune) or the few-sink kernel and the light bodies per
                                CTA of the symmetric heavy-light kernel (rg_ens_autotune); 0:
                                chosen from the SM count                                        */
    int32_t candidates;      /* configurations timed                                             */
    double  ms_per_eval;     /* the chosen configuration: CUDA-event time of one evaluation       */
    double  ms_before;       /* the configuration in place before tuning                         */
} rg_tune_t;

/* per-system statistics of an ensemble (rg_ens_get_stats) */
typedef struct rg_ens_stats {
    double  t_day;          /* simulation clock of the system            */
    double  dt_try_day;     /* next trial step                           */
    double  dt_did_day;     /* last accepted step                        */
    int64_t n_tried_step, n_passed_step, n_failed_step;
    int32_t status;         /* RG_SYS_*                                  */
    int32_t n_total;        /* bodies (active and inactive)              */
    int64_t n_proposed, n_proposal_accepted, n_fallback;  /* learned step proposer */
} rg_ens_stats_t;

enum { RG_SYS_RUNNING = 0, RG_SYS_HELD = 1, RG_SYS_DONE = 2, RG_SYS_ERROR = 3 };

/* one attempt of one disk of an ensemble (rg_ens_step_log): the integrator's own record,
 * also the training data of the learned step proposer */
typedef struct rg_step_rec {
    int32_t sys;
    int32_t accepted;      /* the RKF error estimate accepted the attempt          */
    int32_t proposed;      /* the trial step came from the learned proposer          */
    int32_t step;          /* accepted steps of the disk before this attempt        */
    double  dt;            /* trial step, internal units (1/k days)                 */
    double  err;           /* |dt * 41/840 * max(err)|, the controller's error      */
    float   feat[8];       /* proposer inputs at the attempt (see rg_ens_set_proposer) */
} rg_step_rec_t;

/* red_type.h:46-54 threshold_t */
enum {
    RG_THRESHOLD_HIT_CENTRUM_DISTANCE = 0,
    RG_THRESHOLD_EJECTION_DISTANCE = 1,
    RG_THRESHOLD_RADII_ENHANCE_FACTOR = 2,
    RG_THRESHOLD_HIT_CENTRUM_DISTANCE_SQUARED = 3,
    RG_THRESHOLD_EJECTION_DISTANCE_SQUARED = 4,
    RG_THRESHOLD_N = 5
};

/* red_type.h:56-64 integrator_type_t */
enum {
    RG_INT_EULER = 0,
    RG_INT_RK2 = 1,
    RG_INT_RK4 = 2,
    RG_INT_RK5 = 3,
    RG_INT_RKF78 = 4
};

/* red_type.h:66-74 event_name_t */
enum {
    RG_EVENT_NONE = 0,
    RG_EVENT_HIT_CENTRUM = 1,
    RG_EVENT_EJECTION = 2,
    RG_EVENT_CLOSE_ENCOUNTER = 3,
    RG_EVENT_COLLISION = 4
};

/* red_type.h:90-99 body_type_t */
enum {
    RG_BODY_STAR = 0,
    RG_BODY_GIANTPLANET = 1,
    RG_BODY_ROCKYPLANET = 2,
    RG_BODY_PROTOPLANET = 3,
    RG_BODY_SUPERPLANETESIMAL = 4,
    RG_BODY_PLANETESIMAL = 5,
    RG_BODY_TESTPARTICLE = 6,
    RG_BODY_PADDINGPARTICLE = 7
};

/* red_type.h:38-43 frame_center_t: the origin of the coordinates (parameter.cpp:257-266) */
enum { RG_FRAME_ASTRO = 0, RG_FRAME_BARY = 1 };

/* red_type.h:76-82 event_counter_name_t */
enum { RG_COUNTER_TOTAL = 0, RG_COUNTER_LAST_CLEAR = 1, RG_COUNTER_LAST_STEP = 2 };

#ifdef __cplusplus
}
#endif

#if defined(__cplusplus)
static_assert(sizeof(rg_vec_t) == 32, "vec_t is 32 bytes");
static_assert(sizeof(rg_param_t) == 32, "param_t is 32 bytes");
static_assert(sizeof(rg_body_metadata_t) == 24, "body_metadata_t is 24 bytes");
static_assert(sizeof(rg_orbelem_t) == 48, "orbelem_t is 48 bytes");
static_assert(sizeof(rg_event_t) == 472, "event_data_t is 472 bytes");
#elif defined(__STDC_VERSION__) && __STDC_VERSION__ >= 201112L
_Static_assert(sizeof(rg_vec_t) == 32, "vec_t is 32 bytes");
_Static_assert(sizeof(rg_param_t) == 32, "param_t is 32 bytes");
_Static_assert(sizeof(rg_body_metadata_t) == 24, "body_metadata_t is 24 bytes");
_Static_assert(sizeof(rg_orbelem_t) == 48, "orbelem_t is 48 bytes");
_Static_assert(sizeof(rg_event_t) == 472, "event_data_t is 472 bytes");
#endif

#endif /* REDGB_TYPES_H */
