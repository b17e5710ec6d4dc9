/*
 * redoracle.c -- ORACLE (test infrastructure only): a plain-C restatement of the
 * reference's FP64 CPU path (`red -cpu`).  Used by tests/, __graft_entry__.smoke() and
 * the CPU-baseline leg of bench.py as the checker; the product never calls it.
 *
 * Every function names the reference lines it restates (paths relative to the
 * reference project root, red.cuda/...).  Floating-point expressions keep the
 * reference's operation order and are compiled with -ffp-contract=off (the reference
 * builds with -fmad=false, red.cuda/Makefile:17), so results are bit-identical to the
 * reference's CPU path on the same machine.
 *
 * Deliberate differences, all documented in the repository's design notes:
 *  - event slots are zeroed before a record is written (the reference reuses stale slot
 *    contents for the fields a record type does not set);
 *  - RKF5 is restated from the tables of int_rungekutta5.cu, which does not compile in
 *    the reference: all six stages are evaluated before y_{n+1} (the reference code
 *    would read stage 6 before computing it);
 *  - new, not in the reference: the mutual-Hill-radius close-encounter log, the energy
 *    and angular-momentum diagnostics and the dt replay hook.
 */
#include "redoracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define RO_OK 0
#define RO_ERR_ARG (-1)
#define RO_ERR_EVENT_OVERFLOW (-3)
#define RO_ERR_STATE (-5)
#define RO_ERR_NOT_IMPLEMENTED (-6)
#define RO_ERR_NOMEM (-7)

/* red.cuda/red.type/red_constants.h:21-22 */
static const double GAUSS = 1.720209895e-2;
static const double GAUSS2 = 2.959122082855911025e-4;
#define RO_PI 3.1415926535897932384626 /* red_macro.h:13 */

#define SQR(x) ((x) * (x))
#define CUBE(x) ((x) * (x) * (x))

typedef struct ro_sys {
    /* number_of_bodies (number_of_bodies.h:48-62) */
    int n_s, n_gp, n_rp, n_pp, n_spl, n_pl, n_tp;
    int n_i[7];
    int n_cap;
    /* sim_data_t host arrays (red_type.h:168-228) */
    rg_vec_t *y[2], *yout[2];
    rg_param_t* p;
    rg_body_metadata_t* md;
    double* epoch;
    double t;
    double thr[RG_THRESHOLD_N];
    int close_encounter, inner_steps;
    double hill_factor;
    int event_time_mode;
    int frame; /* RG_FRAME_BARY or RG_FRAME_ASTRO (pp_disk.h frame_center) */
    /* pp_disk::events / event_counter (pp_disk.h:187-192) */
    rg_event_t* events;
    int event_counter, event_cap;
    int overflow;
    /* Hill close-encounter candidates of the last step-start evaluation (new) */
    rg_event_t* hill;
    int n_hill, hill_cap;
    int64_t* hill_pairs; /* (id1 << 32 | id2) of pairs currently inside the Hill sphere */
    int n_hill_pairs, hill_pairs_cap;
    /* event log == everything print_event_data writes */
    rg_event_t* log;
    int n_log, log_cap;
    int64_t n_hit_centrum[3], n_ejection[3], n_collision[3], n_close_encounter[3], n_event[3];
    int64_t n_gravity_evals, n_pairs;
    /* integrator (integrator.h:60-84) */
    int int_type, adaptive, error_check_for_tp, r_max, order, has_int;
    double dt_try, dt_did, tol;
    int64_t n_failed, n_passed, n_tried;
    rg_vec_t* dydx[2][13];
    rg_vec_t* ytemp[2];
    double* err[2];
    /* replay */
    double* replay;
    int n_replay, i_replay;
} ro_sys;

/* ------------------------------------------------------------ number_of_bodies */
static int n_SI(const ro_sys* s) { return s->n_s + s->n_gp + s->n_rp + s->n_pp; }
static int n_NSI(const ro_sys* s) { return s->n_spl + s->n_pl; }
static int n_NI(const ro_sys* s) { return s->n_tp; }
static int n_massive(const ro_sys* s) { return n_SI(s) + n_NSI(s); }
static int n_total(const ro_sys* s) { return n_massive(s) + n_NI(s); }

/* ------------------------------------------------------------ tools.cpp restatements */

/* tools.cpp:238-243 */
double ro_calculate_radius(double m, double density)
{
    static const double four_pi_over_three = 4.1887902047863909846168578443727;
    return pow(1.0 / four_pi_over_three * m / density, 1.0 / 3.0);
}

/* tools.cpp:245-254 */
double ro_calculate_density(double m, double R)
{
    static const double four_pi_over_three = 4.1887902047863909846168578443727;
    if (R == 0.0) return 0.0;
    return m / (four_pi_over_three * CUBE(R));
}

/* tools.cpp:256-261 */
double ro_calculate_mass(double R, double density)
{
    static const double four_pi_over_three = 4.1887902047863909846168578443727;
    return four_pi_over_three * CUBE(R) * density;
}

/* tools.cpp:263-270 */
void ro_calc_position_after_collision(double m1, double m2, const rg_vec_t* r1,
                                      const rg_vec_t* r2, rg_vec_t* r)
{
    const double M = m1 + m2;
    r->x = (m1 * r1->x + m2 * r2->x) / M;
    r->y = (m1 * r1->y + m2 * r2->y) / M;
    r->z = (m1 * r1->z + m2 * r2->z) / M;
}

/* tools.cpp:272-279 */
void ro_calc_velocity_after_collision(double m1, double m2, const rg_vec_t* v1,
                                      const rg_vec_t* v2, rg_vec_t* v)
{
    const double M = m1 + m2;
    v->x = (m1 * v1->x + m2 * v2->x) / M;
    v->y = (m1 * v1->y + m2 * v2->y) / M;
    v->z = (m1 * v1->z + m2 * v2->z) / M;
}

/* tools.cpp:281-290 */
void ro_calc_physical_properties(const rg_param_t* p1, const rg_param_t* p2, rg_param_t* p)
{
    double volume = 4.188790204786391 * (CUBE(p1->radius) + CUBE(p2->radius));
    p->mass = p1->mass + p2->mass;
    p->density = p->mass / volume;
    p->radius = ro_calculate_radius(p->mass, p->density);
    p->cd = p1->cd;
}

/* tools.cpp:292-315 */
int ro_kepler_equation_solver(double ecc, double mean, double eps, double* E)
{
    if (ecc == 0.0 || mean == 0.0 || mean == RO_PI) {
        *E = mean;
        return 0;
    }
    *E = mean + ecc * (sin(mean)) / (1.0 - sin(mean + ecc) + sin(mean));
    double E1 = 0.0;
    double error;
    int step = 0;
    do {
        E1 = *E - (*E - ecc * sin(*E) - mean) / (1.0 - ecc * cos(*E));
        error = fabs(E1 - *E);
        *E = E1;
    } while (error > eps && step++ <= 15);
    if (step > 15) return 1;
    return 0;
}

/* tools.cpp:317-359 */
int ro_calculate_phase(double mu, const rg_orbelem_t* oe, rg_vec_t* rVec, rg_vec_t* vVec)
{
    double ecc = oe->ecc;
    double E = 0.0;
    if (ro_kepler_equation_solver(ecc, oe->mean, 1.0e-14, &E) == 1) return 1;
    double v = 2.0 * atan(sqrt((1.0 + ecc) / (1.0 - ecc)) * tan(E / 2.0));

    double p = oe->sma * (1.0 - SQR(ecc));
    double r = p / (1.0 + ecc * cos(v));
    double kszi = r * cos(v);
    double eta = r * sin(v);
    double vKszi = -sqrt(mu / p) * sin(v);
    double vEta = sqrt(mu / p) * (ecc + cos(v));

    double cw = cos(oe->peri), sw = sin(oe->peri);
    double cO = cos(oe->node), sO = sin(oe->node);
    double ci = cos(oe->inc), si = sin(oe->inc);

    rg_vec_t P, Q;
    P.x = cw * cO - sw * sO * ci;
    P.y = cw * sO + sw * cO * ci;
    P.z = sw * si;
    Q.x = -sw * cO - cw * sO * ci;
    Q.y = -sw * sO + cw * cO * ci;
    Q.z = cw * si;

    rVec->x = kszi * P.x + eta * Q.x;
    rVec->y = kszi * P.y + eta * Q.y;
    rVec->z = kszi * P.z + eta * Q.z;
    vVec->x = vKszi * P.x + vEta * Q.x;
    vVec->y = vKszi * P.y + vEta * Q.y;
    vVec->z = vKszi * P.z + vEta * Q.z;
    return 0;
}

/* tools.cpp:473-484 */
static void shift_into_range(double lower, double upper, double* value)
{
    double range = upper - lower;
    while (*value >= upper) *value -= range;
    while (*value < lower) *value += range;
}

/* tools.cpp:361-471 */
int ro_calculate_orbital_element(double mu, rg_orbelem_t* oe, const rg_vec_t* rVec,
                                 const rg_vec_t* vVec)
{
    const double sq2 = 1.0e-14;
    const double sq3 = 1.0e-14;

    double v2 = SQR(vVec->x) + SQR(vVec->y) + SQR(vVec->z);
    double r2 = SQR(rVec->x) + SQR(rVec->y) + SQR(rVec->z);
    double r = sqrt(r2);
    double h = v2 / 2.0 - (mu / sqrt(r2));

    rg_vec_t cVec = {rVec->y * vVec->z - rVec->z * vVec->y, rVec->z * vVec->x - rVec->x * vVec->z,
                     rVec->x * vVec->y - rVec->y * vVec->x, 0.0};
    rg_vec_t lVec = {(-mu / r) * rVec->x + vVec->y * cVec.z - vVec->z * cVec.y,
                     (-mu / r) * rVec->y + vVec->z * cVec.x - vVec->x * cVec.z,
                     (-mu / r) * rVec->z + vVec->x * cVec.y - vVec->y * cVec.x, 0.0};

    double rv = rVec->x * vVec->x + rVec->y * vVec->y + rVec->z * vVec->z;
    double c = sqrt(SQR(cVec.x) + SQR(cVec.y) + SQR(cVec.z));
    double l = sqrt(SQR(lVec.x) + SQR(lVec.y) + SQR(lVec.z));

    double e2 = 1.0 + 2.0 * SQR(c) * h / (mu * mu);
    if (fabs(e2) < sq3) e2 = 0.0;
    double e = sqrt(e2);
    double a = -mu / (2.0 * h);

    double cosi = cVec.z / c;
    double sini = sqrt(SQR(cVec.x) + SQR(cVec.y)) / c;
    double incl = acos(cosi);
    if (incl < sq2)
        incl = 0.0;
    else if (incl > (RO_PI - sq2))
        incl = RO_PI;

    double node = 0.0;
    if (incl != 0.0 && incl != RO_PI) {
        double tmpx = -cVec.y / (c * sini);
        double tmpy = cVec.x / (c * sini);
        node = atan2(tmpy, tmpx);
        shift_into_range(0.0, 2.0 * RO_PI, &node);
    }

    double E = 0.0, H = 0.0, shH = 0.0, peri = 0.0;
    if (e2 != 0.0) {
        double tmpx = (lVec.x * cos(node) + lVec.y * sin(node)) / l;
        double tmpy = (-lVec.x * sin(node) + lVec.y * cos(node)) / (l * cosi);
        peri = atan2(tmpy, tmpx);
        shift_into_range(0.0, 2.0 * RO_PI, &peri);
        if (h >= 0.0) {
            shH = rv / (SQR(a * mu) / CUBE(c) * e * pow(e2 - 1, 1.5));
            H = asinh(shH);
        } else {
            tmpx = 1.0 / e * (1.0 - r / a);
            tmpy = rv / (sqrt(mu * a) * e);
            E = atan2(tmpy, tmpx);
            shift_into_range(0.0, 2.0 * RO_PI, &E);
        }
    } else {
        peri = 0.0;
        E = atan2(rVec->y, rVec->x);
        shift_into_range(0, 2.0 * RO_PI, &E);
    }

    double M = 0.0;
    if (h >= 0.0) {
        M = e * shH - H;
    } else {
        M = E - e * sin(E);
        shift_into_range(0, 2.0 * RO_PI, &M);
    }
    oe->sma = a;
    oe->ecc = e;
    oe->inc = incl;
    oe->peri = peri;
    oe->node = node;
    oe->mean = M;
    return 0;
}

/* tools.cpp:109-178 compute_bc + transform_to_bc (both loops run j = n-1 .. 0) */
void ro_transform_to_bc(int n, const rg_param_t* p, rg_vec_t* r, rg_vec_t* v)
{
    rg_vec_t R0 = {0.0, 0.0, 0.0, 0.0};
    rg_vec_t V0 = {0.0, 0.0, 0.0, 0.0};
    for (int j = n - 1; j >= 0; j--) {
        double m = p[j].mass;
        R0.x += m * r[j].x;
        R0.y += m * r[j].y;
        R0.z += m * r[j].z;
        V0.x += m * v[j].x;
        V0.y += m * v[j].y;
        V0.z += m * v[j].z;
    }
    double M0 = 0.0;
    for (int j = n - 1; j >= 0; j--) M0 += p[j].mass;
    R0.x /= M0; R0.y /= M0; R0.z /= M0;
    V0.x /= M0; V0.y /= M0; V0.z /= M0;
    for (int j = n - 1; j >= 0; j--) {
        r[j].x -= R0.x; r[j].y -= R0.y; r[j].z -= R0.z;
        v[j].x -= V0.x; v[j].y -= V0.y; v[j].z -= V0.z;
    }
}

/* ------------------------------------------------------------ storage */

static int alloc_integrator_storage(ro_sys* s)
{
    int n = s->n_cap;
    for (int i = 0; i < 2; i++) {
        s->ytemp[i] = (rg_vec_t*)calloc((size_t)n, sizeof(rg_vec_t));
        if (!s->ytemp[i]) return RO_ERR_NOMEM;
        for (int r = 0; r < 13; r++) {
            s->dydx[i][r] = (rg_vec_t*)calloc((size_t)n, sizeof(rg_vec_t));
            if (!s->dydx[i][r]) return RO_ERR_NOMEM;
        }
        s->err[i] = (double*)calloc((size_t)4 * n, sizeof(double));
        if (!s->err[i]) return RO_ERR_NOMEM;
    }
    return RO_OK;
}

static void free_integrator_storage(ro_sys* s)
{
    for (int i = 0; i < 2; i++) {
        free(s->ytemp[i]);
        s->ytemp[i] = NULL;
        for (int r = 0; r < 13; r++) {
            free(s->dydx[i][r]);
            s->dydx[i][r] = NULL;
        }
        free(s->err[i]);
        s->err[i] = NULL;
    }
}

/* pp_disk::get_mass_of_star (pp_disk.cu:1483-1496) */
static double mass_of_star(const ro_sys* s)
{
    int n = n_massive(s);
    for (int j = 0; j < n; j++)
        if (s->md[j].body_type == RG_BODY_STAR) return s->p[j].mass;
    return 0.0;
}

/* tools.cpp:180-236 get_star_bc_phase + transform_to_ac: every body minus body 0's phase
 * (the reference tests body 0's type for every j, so body 0 must be the star), the loop
 * running j = n-1 .. 0 so that body 0 ends exactly at rest in the origin. */
static int transform_to_ac(int n, const rg_body_metadata_t* md, rg_vec_t* r, rg_vec_t* v)
{
    if (md[0].body_type != RG_BODY_STAR) return RO_ERR_ARG; /* "No star is included!" */
    const rg_vec_t R0 = r[0], V0 = v[0];
    for (int j = n - 1; j >= 0; j--) {
        r[j].x -= R0.x; r[j].y -= R0.y; r[j].z -= R0.z;
        v[j].x -= V0.x; v[j].y -= V0.y; v[j].z -= V0.z;
    }
    return RO_OK;
}

/* pp_disk::pp_disk + load + options::create_pp_disk (pp_disk.cu:1204-1235,1614-1683;
 * options.cpp:197-235) in the barycentric frame. */
int ro_create(const rg_counts_t* n, const rg_vec_t* r, const rg_vec_t* v, const rg_param_t* p,
              const rg_body_metadata_t* md, const double* epoch, const double thr[RG_THRESHOLD_N],
              ro_sys** out)
{
    return ro_create_in_frame(n, r, v, p, md, epoch, thr, RG_FRAME_BARY, out);
}

/* The same in either frame (options.cpp:206-220): a system whose body 0 sits at rest in the
 * origin is moved to its barycentre in the barycentric frame; any other system is moved to
 * body 0 (the star) in the astrocentric frame.  The astrocentric frame is refused for
 * systems with non-self-interacting bodies (super-planetesimals, planetesimals, test
 * particles): their blocks take the star, at the origin, as source 0, whose indirect term
 * m_0 / (0 * sqrt(0)) * 0 (pp_disk.cu:447-454) makes the reference's accelerations NaN. */
int ro_create_in_frame(const rg_counts_t* n, const rg_vec_t* r, const rg_vec_t* v, const rg_param_t* p,
                       const rg_body_metadata_t* md, const double* epoch, const double thr[RG_THRESHOLD_N],
                       int frame_center, ro_sys** out)
{
    if (!n || !r || !v || !p || !md || !thr || !out) return RO_ERR_ARG;
    if (n->n_s < 0 || n->n_gp < 0 || n->n_rp < 0 || n->n_pp < 0 || n->n_spl < 0 || n->n_pl < 0 ||
        n->n_tp < 0)
        return RO_ERR_ARG;
    if (frame_center != RG_FRAME_BARY && frame_center != RG_FRAME_ASTRO) return RO_ERR_ARG;
    if (frame_center == RG_FRAME_ASTRO && (n->n_spl > 0 || n->n_pl > 0 || n->n_tp > 0))
        return RO_ERR_NOT_IMPLEMENTED;
    ro_sys* s = (ro_sys*)calloc(1, sizeof(ro_sys));
    if (!s) return RO_ERR_NOMEM;
    s->n_s = n->n_s; s->n_gp = n->n_gp; s->n_rp = n->n_rp; s->n_pp = n->n_pp;
    s->n_spl = n->n_spl; s->n_pl = n->n_pl; s->n_tp = n->n_tp;
    int nt = n_total(s);
    if (nt <= 0) { free(s); return RO_ERR_ARG; }
    s->n_cap = nt;
    for (int i = 0; i < 2; i++) {
        s->y[i] = (rg_vec_t*)calloc((size_t)nt, sizeof(rg_vec_t));
        s->yout[i] = (rg_vec_t*)calloc((size_t)nt, sizeof(rg_vec_t));
    }
    s->p = (rg_param_t*)calloc((size_t)nt, sizeof(rg_param_t));
    s->md = (rg_body_metadata_t*)calloc((size_t)nt, sizeof(rg_body_metadata_t));
    s->epoch = (double*)calloc((size_t)nt, sizeof(double));
    s->event_cap = nt > 1024 ? nt : 1024;
    s->events = (rg_event_t*)calloc((size_t)s->event_cap, sizeof(rg_event_t));
    s->hill_cap = s->event_cap;
    s->hill = (rg_event_t*)calloc((size_t)s->hill_cap, sizeof(rg_event_t));
    if (!s->y[0] || !s->y[1] || !s->yout[0] || !s->yout[1] || !s->p || !s->md || !s->epoch ||
        !s->events || !s->hill) {
        ro_destroy(s);
        return RO_ERR_NOMEM;
    }
    for (int i = 0; i < nt; i++) {
        s->y[0][i] = r[i];
        s->y[1][i] = v[i];
        s->y[0][i].w = s->y[1][i].w = 0.0; /* pp_disk.cu:1611 */
        s->p[i] = p[i];
        s->md[i] = md[i];
        s->epoch[i] = epoch ? epoch[i] : 0.0;
    }
    s->close_encounter = 0;
    s->inner_steps = 1;
    s->frame = frame_center;
    for (int i = 0; i < RG_THRESHOLD_N; i++) s->thr[i] = thr[i];

    /* options.cpp:206-220: barycentric transform if the first body sits at rest in 0,
     * astrocentric transform otherwise */
    if (0 == fabs(s->y[0][0].x) && 0 == fabs(s->y[0][0].y) && 0 == fabs(s->y[0][0].z) &&
        0 == fabs(s->y[1][0].x) && 0 == fabs(s->y[1][0].y) && 0 == fabs(s->y[1][0].z)) {
        if (frame_center == RG_FRAME_BARY) ro_transform_to_bc(nt, s->p, s->y[0], s->y[1]);
    } else if (frame_center == RG_FRAME_ASTRO) {
        if (transform_to_ac(nt, s->md, s->y[0], s->y[1]) != RO_OK) {
            ro_destroy(s);
            return RO_ERR_ARG;
        }
    }
    /* pp_disk::transform_time / transform_velocity (pp_disk.cu:1512-1551) */
    for (int j = 0; j < nt; j++) s->epoch[j] *= GAUSS;
    for (int j = 0; j < nt; j++) {
        s->y[1][j].x /= GAUSS;
        s->y[1][j].y /= GAUSS;
        s->y[1][j].z /= GAUSS;
    }
    s->t = 0.0;
    *out = s;
    return RO_OK;
}

void ro_destroy(ro_sys* s)
{
    if (!s) return;
    for (int i = 0; i < 2; i++) {
        free(s->y[i]);
        free(s->yout[i]);
    }
    free(s->p);
    free(s->md);
    free(s->epoch);
    free(s->events);
    free(s->hill);
    free(s->hill_pairs);
    free(s->log);
    free(s->replay);
    free_integrator_storage(s);
    free(s);
}

int ro_set_event_options(ro_sys* s, int close_encounter, int inner_steps, double hill_factor,
                         int event_time_mode)
{
    if (!s || hill_factor < 0.0 || (event_time_mode != 0 && event_time_mode != 1))
        return RO_ERR_ARG;
    s->close_encounter = close_encounter ? 1 : 0;
    s->inner_steps = inner_steps ? 1 : 0;
    s->hill_factor = hill_factor;
    s->event_time_mode = event_time_mode;
    return RO_OK;
}

int ro_set_time(ro_sys* s, double t_day)
{
    if (!s) return RO_ERR_ARG;
    s->t = t_day * GAUSS; /* parameter.cpp:287-292 */
    return RO_OK;
}

/* ------------------------------------------------------------ events */

static rg_event_t* new_event(ro_sys* s)
{
    if (s->event_counter >= s->event_cap) {
        s->overflow = 1;
        return NULL;
    }
    rg_event_t* e = &s->events[s->event_counter];
    memset(e, 0, sizeof(*e));
    return e;
}

static int log_push(ro_sys* s, const rg_event_t* e)
{
    if (s->n_log == s->log_cap) {
        int cap = s->log_cap ? 2 * s->log_cap : 256;
        rg_event_t* nl = (rg_event_t*)realloc(s->log, (size_t)cap * sizeof(rg_event_t));
        if (!nl) return RO_ERR_NOMEM;
        s->log = nl;
        s->log_cap = cap;
    }
    s->log[s->n_log++] = *e;
    return RO_OK;
}

/* pp_disk::increment_event_counter (pp_disk.cu:1059-1067) */
static void increment_event_counter(ro_sys* s, int64_t* counter)
{
    for (int i = 0; i < 3; i++) {
        counter[i]++;
        s->n_event[i]++;
    }
}

/* Astrocentric orbital elements of one body of the given state arrays, as the CPU
 * close-encounter branch computes them (pp_disk.cu:526-553): transform_to_ac of a copy
 * (tools.cpp:180-236, star = body 0) and velocities rescaled by k. */
static void event_elements(const ro_sys* s, const rg_vec_t* r, const rg_vec_t* v, int idx,
                           double mu, rg_orbelem_t* oe)
{
    rg_vec_t ra = {r[idx].x - r[0].x, r[idx].y - r[0].y, r[idx].z - r[0].z, 0.0};
    rg_vec_t va = {v[idx].x - v[0].x, v[idx].y - v[0].y, v[idx].z - v[0].z, 0.0};
    if (idx == 0) {
        ra.x = ra.y = ra.z = 0.0;
        va.x = va.y = va.z = 0.0;
    }
    if (s->frame == RG_FRAME_ASTRO) { /* pp_disk.cu:554-560: the coordinates as they are */
        ra = r[idx];
        ra.w = 0.0;
        va = v[idx];
    }
    rg_vec_t vt = {va.x * GAUSS, va.y * GAUSS, va.z * GAUSS, 0.0};
    ro_calculate_orbital_element(mu, oe, &ra, &vt);
}

/* ------------------------------------------------------------ gravity */

/* pp_disk::cpu_calc_grav_accel_SI (pp_disk.cu:404-572), barycentric frame, for the sinks
 * of one interaction block.  `t_event` is the time stamped on the records (the caller
 * passes curr_t for SI and, like pp_disk.cu:576,581, the step-start time for NSI/NI
 * unless the stage-time mode is selected).  `record` enables event records. */
static void grav_block(ro_sys* s, double t_event, int sink_x, int sink_y, int src_x, int src_y,
                       const rg_vec_t* r, const rg_vec_t* v, rg_vec_t* a, int record, int hill)
{
    const rg_param_t* p = s->p;
    const rg_body_metadata_t* md = s->md;
    const double f_rad = s->thr[RG_THRESHOLD_RADII_ENHANCE_FACTOR];
    const double M_star = p[0].mass;
    const double f3 = s->hill_factor * s->hill_factor * s->hill_factor;
    const int astro = s->frame == RG_FRAME_ASTRO;
    for (int i = sink_x; i < sink_y; i++) {
        if (!astro) {
            a[i].x = a[i].y = a[i].z = a[i].w = 0.0;
        } else {
            /* pp_disk.cu:413-420: the star's pull as the starting value */
            const double mu = mass_of_star(s) + p[i].mass;
            const double r2 = SQR(r[i].x) + SQR(r[i].y) + SQR(r[i].z);
            a[i].x = -mu / (r2 * sqrt(r2)) * r[i].x;
            a[i].y = -mu / (r2 * sqrt(r2)) * r[i].y;
            a[i].z = -mu / (r2 * sqrt(r2)) * r[i].z;
        }
        if (0 < md[i].id) {
            rg_vec_t dVec = {0.0, 0.0, 0.0, 0.0};
            for (int j = src_x; j < src_y; j++) {
                if (i == j || 0 > md[j].id) continue;
                dVec.x = r[j].x - r[i].x;
                dVec.y = r[j].y - r[i].y;
                dVec.z = r[j].z - r[i].z;
                dVec.w = SQR(dVec.x) + SQR(dVec.y) + SQR(dVec.z);
                double d = sqrt(dVec.w);
                dVec.w = p[j].mass / (d * dVec.w);
                a[i].x += dVec.w * dVec.x;
                a[i].y += dVec.w * dVec.y;
                a[i].z += dVec.w * dVec.z;
                if (astro) {
                    /* pp_disk.cu:447-454: the indirect term of source j */
                    const double r2 = SQR(r[j].x) + SQR(r[j].y) + SQR(r[j].z);
                    a[i].x -= p[j].mass / (r2 * sqrt(r2)) * r[j].x;
                    a[i].y -= p[j].mass / (r2 * sqrt(r2)) * r[j].y;
                    a[i].z -= p[j].mass / (r2 * sqrt(r2)) * r[j].z;
                }
                s->n_pairs++;

                if (record && i > 0 && i > j && d < f_rad * (p[i].radius + p[j].radius)) {
                    rg_event_t* e = new_event(s);
                    if (e) {
                        int surv = i, merg = j;
                        if (!s->close_encounter) {
                            /* pp_disk.cu:470-492 */
                            if (p[merg].mass > p[surv].mass) {
                                int tmp = surv;
                                surv = merg;
                                merg = tmp;
                            }
                            e->event_name = RG_EVENT_COLLISION;
                            e->d = d;
                            e->t = t_event;
                            e->id1 = md[surv].id;
                            e->id2 = md[merg].id;
                            e->idx1 = surv;
                            e->idx2 = merg;
                            e->r1 = r[surv];
                            e->v1 = v[surv];
                            e->r2 = r[merg];
                            e->v2 = v[merg];
                        } else {
                            /* pp_disk.cu:494-563 */
                            e->event_name = RG_EVENT_CLOSE_ENCOUNTER;
                            e->d = d;
                            e->t = t_event;
                            e->id1 = md[surv].id;
                            e->id2 = md[merg].id;
                            e->idx1 = surv;
                            e->idx2 = merg;
                            e->p1 = p[surv];
                            e->p2 = p[merg];
                            e->r1 = r[surv];
                            e->v1 = v[surv];
                            e->r2 = r[merg];
                            e->v2 = v[merg];
                            const double ms = mass_of_star(s);
                            const double mu1 = GAUSS2 * (ms + p[surv].mass);
                            const double mu2 = GAUSS2 * (ms + p[merg].mass);
                            event_elements(s, r, v, surv, mu1, &e->oe1);
                            event_elements(s, r, v, merg, mu2, &e->oe2);
                        }
                        s->event_counter++;
                    }
                }
                /* new: mutual Hill sphere test, d < f (m_i+m_j)^(1/3) (3 M*)^(-1/3) (r_i+r_j)/2
                 * evaluated as cubes so that no cube root enters the comparison */
                if (hill && i > 0 && i > j && j > 0) {
                    double ri = sqrt(SQR(r[i].x - r[0].x) + SQR(r[i].y - r[0].y) + SQR(r[i].z - r[0].z));
                    double rj = sqrt(SQR(r[j].x - r[0].x) + SQR(r[j].y - r[0].y) + SQR(r[j].z - r[0].z));
                    double h = 0.5 * (ri + rj);
                    double lhs = d * d * d;
                    double rhs = ((f3 * (p[i].mass + p[j].mass)) / (3.0 * M_star)) * (h * h * h);
                    if (lhs < rhs && s->n_hill < s->hill_cap) {
                        rg_event_t* e = &s->hill[s->n_hill++];
                        memset(e, 0, sizeof(*e));
                        e->event_name = RG_EVENT_CLOSE_ENCOUNTER;
                        e->d = d;
                        e->t = s->t;
                        e->id1 = md[i].id;
                        e->id2 = md[j].id;
                        e->idx1 = i;
                        e->idx2 = j;
                        e->p1 = p[i];
                        e->p2 = p[j];
                        e->r1 = r[i];
                        e->v1 = v[i];
                        e->r2 = r[j];
                        e->v2 = v[j];
                    }
                }
            }
        }
    }
}

/* pp_disk::cpu_calc_grav_accel (pp_disk.cu:585-607) with the bounds of
 * number_of_bodies::get_bound_SI/NSI/NI (number_of_bodies.cpp:196-258): the astrocentric
 * frame starts the SI block's sinks and sources at 1, so the star's row is never written
 * (its derivative buffers stay at their initial zero, pp_disk's calloc-like allocation). */
static void cpu_calc_grav_accel(ro_sys* s, double curr_t, const rg_vec_t* r, const rg_vec_t* v,
                                rg_vec_t* a, int record, int hill)
{
    const int nsi = n_SI(s), nnsi = n_NSI(s), nni = n_NI(s), nm = n_massive(s);
    const double t_nsi = s->event_time_mode ? curr_t : s->t;
    const int b = s->frame == RG_FRAME_ASTRO ? 1 : 0;
    record = record && s->inner_steps;
    s->n_gravity_evals++;
    if (b < nsi) grav_block(s, curr_t, b, nsi, b, nm, r, v, a, record, hill);
    if (0 < nnsi) grav_block(s, t_nsi, nsi, nsi + nnsi, 0, nsi, r, v, a, record, hill);
    if (0 < nni) grav_block(s, t_nsi, nm, nm + nni, 0, nm, r, v, a, record, 0);
}

int ro_grav_accel_rows(const rg_counts_t* n, const rg_vec_t* r, const rg_param_t* p,
                       const rg_body_metadata_t* md, int i_begin, int i_end, rg_vec_t* a)
{
    if (!n || !r || !p || !md || !a) return RO_ERR_ARG;
    const int nsi = n->n_s + n->n_gp + n->n_rp + n->n_pp;
    const int nm = nsi + n->n_spl + n->n_pl;
    const int nt = nm + n->n_tp;
    if (i_begin < 0 || i_end > nt || i_begin > i_end) return RO_ERR_ARG;
    for (int i = i_begin; i < i_end; i++) {
        const int src_y = (i >= nsi && i < nm) ? nsi : nm;
        rg_vec_t acc = {0.0, 0.0, 0.0, 0.0};
        if (0 < md[i].id) {
            for (int j = 0; j < src_y; j++) {
                if (i == j || 0 > md[j].id) continue;
                double dx = r[j].x - r[i].x;
                double dy = r[j].y - r[i].y;
                double dz = r[j].z - r[i].z;
                double r2 = SQR(dx) + SQR(dy) + SQR(dz);
                double d = sqrt(r2);
                double s = p[j].mass / (d * r2);
                acc.x += s * dx;
                acc.y += s * dy;
                acc.z += s * dz;
            }
        }
        a[i - i_begin] = acc;
    }
    return RO_OK;
}

/* pp_disk::calc_dydx (pp_disk.cu:998-1041): i = 0 copies v, i = 1 evaluates gravity */
static void calc_dydx(ro_sys* s, int i, int rr, double curr_t, const rg_vec_t* r,
                      const rg_vec_t* v, rg_vec_t* dy)
{
    if (i == 0) {
        memcpy(dy, v, (size_t)n_total(s) * sizeof(rg_vec_t));
    } else {
        int hill = (rr == 0) && (s->hill_factor > 0.0);
        if (hill) s->n_hill = 0;
        cpu_calc_grav_accel(s, curr_t, r, v, dy, 1, hill);
    }
}

/* ------------------------------------------------------------ integrators */

/* integrator::get_max_error, CPU branch (integrator.cu:211-256): signed maximum that
 * starts from 0 (the device branch reaches the same value because the w components of
 * the error vector are 0). */
static double max_err_raw(ro_sys* s, int n_var)
{
    double max_err_r = 0.0, max_err_v = 0.0;
    for (int i = 0; i < n_var; i++) {
        if (max_err_r < s->err[0][i]) max_err_r = s->err[0][i];
        if (max_err_v < s->err[1][i]) max_err_v = s->err[1][i];
    }
    /* std::max(a, b) == (a < b) ? b : a */
    return (max_err_r < max_err_v) ? max_err_v : max_err_r;
}

static double next_trial(ro_sys* s)
{
    if (s->i_replay < s->n_replay) return s->replay[s->i_replay++];
    return s->dt_try;
}

int ro_set_dt_replay(ro_sys* s, const double* dt, int n)
{
    if (!s || n < 0 || (n > 0 && !dt)) return RO_ERR_ARG;
    free(s->replay);
    s->replay = NULL;
    s->n_replay = s->i_replay = 0;
    if (n > 0) {
        s->replay = (double*)malloc((size_t)n * sizeof(double));
        if (!s->replay) return RO_ERR_NOMEM;
        memcpy(s->replay, dt, (size_t)n * sizeof(double));
        s->n_replay = n;
    }
    return RO_OK;
}

static void swap_y(ro_sys* s)
{
    for (int i = 0; i < 2; i++) {
        rg_vec_t* tmp = s->y[i];
        s->y[i] = s->yout[i];
        s->yout[i] = tmp;
    }
}

/* integrator::update_counters (integrator.cu:258-263) */
static void update_counters(ro_sys* s, int iter)
{
    s->n_tried += iter;
    s->n_failed += (iter - 1);
    s->n_passed++;
}

static int n_var_err(ro_sys* s)
{
    return 4 * (s->error_check_for_tp ? n_total(s) : n_massive(s));
}

/* ---- Euler (int_euler.cu:22-33,76-141) ---- */
static int step_euler(ro_sys* s)
{
    const int n = 4 * n_total(s);
    const double* y0;
    calc_dydx(s, 0, 0, s->t, s->y[0], s->y[1], s->dydx[0][0]);
    calc_dydx(s, 1, 0, s->t, s->y[0], s->y[1], s->dydx[1][0]);
    for (int i = 0; i < 2; i++) {
        y0 = (const double*)s->y[i];
        const double* f0 = (const double*)s->dydx[i][0];
        double* y1 = (double*)s->yout[i];
        for (int k = 0; k < n; k++) y1[k] = y0[k] + s->dt_try * f0[k];
    }
    s->dt_did = s->dt_try;
    update_counters(s, 1);
    s->t += s->dt_did;
    swap_y(s);
    return RO_OK;
}

/* ---- RK4 (int_rungekutta4.cu:29-32 tables, 77-99 CPU kernels, 189-273 step) ---- */
static const double rk4_c[] = {0.0, 1.0 / 2.0, 1.0 / 2.0, 1.0, 1.0};
static const double rk4_a[] = {0.0, 1.0 / 2.0, 1.0 / 2.0, 1.0, 1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0};
static const double rk4_b[] = {1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0 - 1.0 / 10.0, 1.0 / 10.0};

static int step_rk4(ro_sys* s)
{
    const int nvt = 4 * n_total(s);
    double ttemp = s->t + rk4_c[0] * s->dt_try;
    for (int i = 0; i < 2; i++) calc_dydx(s, i, 0, ttemp, s->y[0], s->y[1], s->dydx[i][0]);

    double max_err = 0.0;
    int iter = 0;
    do {
        s->dt_try = next_trial(s);
        s->dt_did = s->dt_try;
        for (int r = 1; r < 4; r++) {
            ttemp = s->t + rk4_c[r] * s->dt_try;
            for (int i = 0; i < 2; i++) {
                const double* yn = (const double*)s->y[i];
                const double* fr = (const double*)s->dydx[i][r - 1];
                double* yt = (double*)s->ytemp[i];
                const double bf = rk4_a[r] * s->dt_try;
                for (int k = 0; k < nvt; k++) yt[k] = yn[k] + bf * fr[k];
            }
            for (int i = 0; i < 2; i++) calc_dydx(s, i, r, ttemp, s->ytemp[0], s->ytemp[1], s->dydx[i][r]);
        }
        for (int i = 0; i < 2; i++) {
            const double* yn = (const double*)s->y[i];
            double* y1 = (double*)s->yout[i];
            const double *f1 = (const double*)s->dydx[i][0], *f2 = (const double*)s->dydx[i][1];
            const double *f3 = (const double*)s->dydx[i][2], *f4 = (const double*)s->dydx[i][3];
            const double b0 = rk4_b[0] * s->dt_try, b1 = rk4_b[1] * s->dt_try;
            for (int k = 0; k < nvt; k++) y1[k] = yn[k] + b0 * (f1[k] + f4[k]) + b1 * (f2[k] + f3[k]);
        }
        if (s->adaptive) {
            ttemp = s->t + rk4_c[4] * s->dt_try;
            for (int i = 0; i < 2; i++) calc_dydx(s, i, 4, ttemp, s->yout[0], s->yout[1], s->dydx[i][4]);
            const int n_var = n_var_err(s);
            for (int i = 0; i < 2; i++) {
                const double *f4 = (const double*)s->dydx[i][3], *f5 = (const double*)s->dydx[i][4];
                for (int k = 0; k < n_var; k++) s->err[i][k] = f4[k] - f5[k];
            }
            max_err = fabs(s->dt_try * (1.0 / 10.0) * max_err_raw(s, n_var));
            s->dt_try *= 0.9 * pow(s->tol / max_err, 1.0 / 4.0);
            if (s->event_counter > 0) {
                if (s->dt_try < s->dt_did) s->dt_try = s->dt_did;
                break;
            }
        }
        iter++;
    } while (s->adaptive && max_err > s->tol);
    update_counters(s, iter);
    s->t += s->dt_did;
    swap_y(s);
    return RO_OK;
}

/* ---- RKF5, Cash-Karp tables of int_rungekutta5.cu:24-32, kernels 41-93, step 202-282 */
static const double rk5_c[] = {0.0, 1.0 / 5.0, 3.0 / 10.0, 3.0 / 5.0, 1.0, 7.0 / 8.0};
static const double rk5_a[] = {0.0,
                               1.0 / 5.0,
                               3.0 / 40.0, 9.0 / 40.0,
                               3.0 / 10.0, -9.0 / 10.0, 6.0 / 5.0,
                               -11.0 / 54.0, 5.0 / 2.0, -70.0 / 27.0, 35.0 / 27.0,
                               1631.0 / 55296.0, 175.0 / 512.0, 575.0 / 13824.0, 44275.0 / 110592.0, 253.0 / 4096.0};
static const double rk5_bh[] = {37.0 / 378.0, 0.0, 250.0 / 621.0, 125.0 / 594.0, 0.0, 512.0 / 1771.0};
static const double rk5_b[] = {2825.0 / 27648.0, 0.0, 18575.0 / 48384.0, 13525.0 / 55296.0, 277.0 / 14336.0, 1.0 / 4.0};
static const int rk5_idx[] = {0, 1, 2, 4, 7, 11};

static void rk5_ytemp(ro_sys* s, int nvt, int r)
{
    for (int i = 0; i < 2; i++) {
        const double* yn = (const double*)s->y[i];
        double* yt = (double*)s->ytemp[i];
        for (int k = 0; k < nvt; k++) {
            double acc = yn[k];
            for (int q = 0; q < r; q++) {
                const double aq = rk5_a[rk5_idx[r] + q];
                if (0.0 == aq) continue;
                acc += s->dt_try * aq * ((const double*)s->dydx[i][q])[k];
            }
            yt[k] = acc;
        }
    }
}

static int step_rk5(ro_sys* s)
{
    const int nvt = 4 * n_total(s);
    double ttemp = s->t + rk5_c[0] * s->dt_try;
    for (int i = 0; i < 2; i++) calc_dydx(s, i, 0, ttemp, s->y[0], s->y[1], s->dydx[i][0]);

    double max_err = 0.0;
    int iter = 0;
    do {
        s->dt_try = next_trial(s);
        s->dt_did = s->dt_try;
        for (int r = 1; r < 6; r++) {
            ttemp = s->t + rk5_c[r] * s->dt_try;
            rk5_ytemp(s, nvt, r);
            for (int i = 0; i < 2; i++) calc_dydx(s, i, r, ttemp, s->ytemp[0], s->ytemp[1], s->dydx[i][r]);
        }
        for (int i = 0; i < 2; i++) {
            const double* yn = (const double*)s->y[i];
            double* y1 = (double*)s->yout[i];
            for (int k = 0; k < nvt; k++) {
                double acc = yn[k];
                for (int q = 0; q < 6; q++) {
                    if (0.0 == rk5_b[q]) continue;
                    acc += s->dt_try * rk5_b[q] * ((const double*)s->dydx[i][q])[k];
                }
                y1[k] = acc;
            }
        }
        if (s->adaptive) {
            const int n_var = n_var_err(s);
            for (int i = 0; i < 2; i++) {
                for (int k = 0; k < n_var; k++) {
                    double e = (rk5_bh[0] - rk5_b[0]) * ((const double*)s->dydx[i][0])[k];
                    for (int q = 1; q < 6; q++) e += (rk5_bh[q] - rk5_b[q]) * ((const double*)s->dydx[i][q])[k];
                    s->err[i][k] = e;
                }
            }
            max_err = fabs(s->dt_try * max_err_raw(s, n_var));
            s->dt_try *= 0.9 * pow(s->tol / max_err, 1.0 / 5);
            if (s->event_counter > 0) {
                if (s->dt_try < s->dt_did) s->dt_try = s->dt_did;
                break;
            }
        }
        iter++;
    } while (s->adaptive && max_err > s->tol);
    update_counters(s, iter);
    s->t += s->dt_did;
    swap_y(s);
    return RO_OK;
}

/* ---- RKF7(8) (int_rungekutta8.cu:29-47 tables, 336-460 CPU kernels, 476-797 step) ---- */
static const double rk8_c[] = {0.0, 2.0 / 27.0, 1.0 / 9.0, 1.0 / 6.0, 5.0 / 12.0, 1.0 / 2.0, 5.0 / 6.0,
                               1.0 / 6.0, 2.0 / 3.0, 1.0 / 3.0, 1.0, 0.0, 1.0};
static const double rk8_a[] = {
    0.0,
    2.0 / 27.0,
    1.0 / 36.0, 1.0 / 12.0,
    1.0 / 24.0, 0.0, 1.0 / 8.0,
    5.0 / 12.0, 0.0, -25.0 / 16.0, 25.0 / 16.0,
    1.0 / 20.0, 0.0, 0.0, 1.0 / 4.0, 1.0 / 5.0,
    -25.0 / 108.0, 0.0, 0.0, 125.0 / 108.0, -65.0 / 27.0, 125.0 / 54.0,
    31.0 / 300.0, 0.0, 0.0, 0.0, 61.0 / 225.0, -2.0 / 9.0, 13.0 / 900.0,
    2.0, 0.0, 0.0, -53.0 / 6.0, 704.0 / 45.0, -107.0 / 9.0, 67.0 / 90.0, 3.0,
    -91.0 / 108.0, 0.0, 0.0, 23.0 / 108.0, -976.0 / 135.0, 311.0 / 54.0, -19.0 / 60.0, 17.0 / 6.0, -1.0 / 12.0,
    2383.0 / 4100.0, 0.0, 0.0, -341.0 / 164.0, 4496.0 / 1025.0, -301.0 / 82.0, 2133.0 / 4100.0, 45.0 / 82.0, 45.0 / 164.0, 18.0 / 41.0,
    3.0 / 205.0, 0.0, 0.0, 0.0, 0.0, -6.0 / 41.0, -3.0 / 205.0, -3.0 / 41.0, 3.0 / 41.0, 6.0 / 41.0, 0.0,
    -1777.0 / 4100.0, 0.0, 0.0, -341.0 / 164.0, 4496.0 / 1025.0, -289.0 / 82.0, 2193.0 / 4100.0, 51.0 / 82.0, 33.0 / 164.0, 12.0 / 41.0, 0.0, 1.0};
static const double rk8_b[] = {41.0 / 840.0, 0.0, 0.0, 0.0, 0.0, 34.0 / 105.0, 9.0 / 35.0, 9.0 / 35.0, 9.0 / 280.0, 9.0 / 280.0, 41.0 / 840.0};

/* Stage rows as the reference's calc_ytemp_for_f1..f12 spell them out
 * (int_rungekutta8.cu:336-442, index offsets from 476-633): the stages that enter
 * stage r, and the a[] index of each coefficient. */
static const int rk8_nterm[13] = {0, 1, 2, 2, 3, 3, 4, 4, 6, 7, 8, 6, 9};
static const int rk8_stage[13][9] = {
    {0}, {0}, {0, 1}, {0, 2}, {0, 2, 3}, {0, 3, 4}, {0, 3, 4, 5}, {0, 4, 5, 6},
    {0, 3, 4, 5, 6, 7}, {0, 3, 4, 5, 6, 7, 8}, {0, 3, 4, 5, 6, 7, 8, 9},
    {0, 5, 6, 7, 8, 9}, {0, 3, 4, 5, 6, 7, 8, 9, 11}};
static const int rk8_aidx[13][9] = {
    {0}, {1}, {2, 3}, {4, 6}, {7, 9, 10}, {11, 14, 15}, {16, 19, 20, 21}, {22, 26, 27, 28},
    {29, 32, 33, 34, 35, 36}, {37, 40, 41, 42, 43, 44, 45}, {46, 49, 50, 51, 52, 53, 54, 55},
    {56, 61, 62, 63, 64, 65}, {67, 70, 71, 72, 73, 74, 75, 76, 78}};

static void rk8_ytemp(ro_sys* s, int nvt, int r)
{
    for (int i = 0; i < 2; i++) {
        const double* yn = (const double*)s->y[i];
        double* yt = (double*)s->ytemp[i];
        const double* f[9];
        for (int q = 0; q < rk8_nterm[r]; q++) f[q] = (const double*)s->dydx[i][rk8_stage[r][q]];
        for (int k = 0; k < nvt; k++) {
            double sum = rk8_a[rk8_aidx[r][0]] * f[0][k];
            for (int q = 1; q < rk8_nterm[r]; q++) sum = sum + rk8_a[rk8_aidx[r][q]] * f[q][k];
            yt[k] = yn[k] + s->dt_try * sum;
        }
    }
}

static int step_rkf78(ro_sys* s)
{
    const int nvt = 4 * n_total(s);
    double ttemp = s->t + rk8_c[0] * s->dt_try;
    for (int i = 0; i < 2; i++) calc_dydx(s, i, 0, ttemp, s->y[0], s->y[1], s->dydx[i][0]);

    double max_err = 0.0;
    int iter = 0;
    do {
        if (0 < s->event_counter) s->event_counter = 0; /* int_rungekutta8.cu:730-733 */
        s->dt_try = next_trial(s);
        s->dt_did = s->dt_try;
        for (int r = 1; r <= 10; r++) {
            ttemp = s->t + rk8_c[r] * s->dt_try;
            rk8_ytemp(s, nvt, r);
            for (int i = 0; i < 2; i++) calc_dydx(s, i, r, ttemp, s->ytemp[0], s->ytemp[1], s->dydx[i][r]);
        }
        for (int i = 0; i < 2; i++) {
            const double* yn = (const double*)s->y[i];
            double* y1 = (double*)s->yout[i];
            const double *f0 = (const double*)s->dydx[i][0], *f5 = (const double*)s->dydx[i][5];
            const double *f6 = (const double*)s->dydx[i][6], *f7 = (const double*)s->dydx[i][7];
            const double *f8 = (const double*)s->dydx[i][8], *f9 = (const double*)s->dydx[i][9];
            const double* f10 = (const double*)s->dydx[i][10];
            for (int k = 0; k < nvt; k++)
                y1[k] = yn[k] + s->dt_try * (rk8_b[0] * f0[k] + rk8_b[5] * f5[k] + rk8_b[6] * (f6[k] + f7[k]) +
                                             rk8_b[8] * (f8[k] + f9[k]) + rk8_b[10] * f10[k]);
        }
        if (s->adaptive) {
            for (int r = 11; r < s->r_max; r++) {
                ttemp = s->t + rk8_c[r] * s->dt_try;
                rk8_ytemp(s, nvt, r);
                for (int i = 0; i < 2; i++) calc_dydx(s, i, r, ttemp, s->ytemp[0], s->ytemp[1], s->dydx[i][r]);
            }
            const int n_var = n_var_err(s);
            for (int i = 0; i < 2; i++) {
                const double *f0 = (const double*)s->dydx[i][0], *f10 = (const double*)s->dydx[i][10];
                const double *f11 = (const double*)s->dydx[i][11], *f12 = (const double*)s->dydx[i][12];
                for (int k = 0; k < n_var; k++) s->err[i][k] = (f0[k] + f10[k] - f11[k] - f12[k]);
            }
            max_err = fabs(s->dt_try * (41.0 / 840.0) * max_err_raw(s, n_var));
            s->dt_try *= 0.9 * pow(s->tol / max_err, 1.0 / (s->order + 1));
        }
        iter++;
    } while (s->adaptive && max_err > s->tol);
    update_counters(s, iter);
    s->t += s->dt_did;
    swap_y(s);
    return RO_OK;
}

/* options::create_integrator (options.cpp:237-274) + integrator constructors */
int ro_set_integrator(ro_sys* s, int type, double dt_day, int adaptive, double tolerance,
                      int error_check_for_tp)
{
    if (!s || !(dt_day == dt_day)) return RO_ERR_ARG;
    switch (type) {
    case RG_INT_EULER: s->r_max = 1; s->order = 1; adaptive = 0; break;
    case RG_INT_RK4: s->r_max = adaptive ? 5 : 4; s->order = 4; break;
    case RG_INT_RK5: s->r_max = 6; s->order = 5; break;
    case RG_INT_RKF78: s->r_max = adaptive ? 13 : 11; s->order = 7; break;
    default: return RO_ERR_ARG;
    }
    if (!s->ytemp[0]) {
        int rc = alloc_integrator_storage(s);
        if (rc) return rc;
    }
    s->int_type = type;
    s->adaptive = adaptive ? 1 : 0;
    s->tol = tolerance;
    s->error_check_for_tp = error_check_for_tp ? 1 : 0;
    s->dt_try = dt_day * GAUSS; /* integrator.cu:29 */
    s->dt_did = 0.0;
    s->n_failed = s->n_passed = s->n_tried = 0;
    s->has_int = 1;
    return RO_OK;
}

int ro_step(ro_sys* s, double* dt_did_day)
{
    if (!s) return RO_ERR_ARG;
    if (!s->has_int) return RO_ERR_STATE;
    int rc;
    switch (s->int_type) {
    case RG_INT_EULER: rc = step_euler(s); break;
    case RG_INT_RK4: rc = step_rk4(s); break;
    case RG_INT_RK5: rc = step_rk5(s); break;
    default: rc = step_rkf78(s); break;
    }
    if (rc) return rc;
    if (dt_did_day) *dt_did_day = s->dt_did / GAUSS;
    if (s->overflow) {
        s->overflow = 0;
        return RO_ERR_EVENT_OVERFLOW;
    }
    return RO_OK;
}

/* ------------------------------------------------------------ event handling */

/* pp_disk::store_event_data, host version (pp_disk.cu:909-932) */
static void store_event_data(ro_sys* s, int name, double t, double d, int idx1, int idx2,
                             rg_event_t* e)
{
    memset(e, 0, sizeof(*e));
    e->event_name = name;
    e->d = d;
    e->t = t;
    e->id1 = s->md[idx1].id;
    e->id2 = s->md[idx2].id;
    e->idx1 = idx1;
    e->idx2 = idx2;
    e->r1 = s->y[0][idx1];
    e->v1 = s->y[1][idx1];
    e->r2 = s->y[0][idx2];
    e->v2 = s->y[1][idx2];
    if (RG_EVENT_EJECTION == name) {
        e->p1 = s->p[idx1];
        e->p2 = s->p[idx2];
        e->rs = e->r1;
        e->vs = e->v1;
        e->ps = e->p1;
    }
}

/* pp_disk::handle_collision_pair (pp_disk.cu:1151-1202) */
static int handle_collision_pair(ro_sys* s, rg_event_t* c)
{
    int surv = c->idx1, merg = c->idx2;
    if (RG_BODY_SUPERPLANETESIMAL == s->md[merg].body_type) return RO_ERR_NOT_IMPLEMENTED;
    c->p1 = s->p[surv];
    c->p2 = s->p[merg];
    ro_calc_position_after_collision(c->p1.mass, c->p2.mass, &c->r1, &c->r2, &c->rs);
    ro_calc_velocity_after_collision(c->p1.mass, c->p2.mass, &c->v1, &c->v2, &c->vs);
    s->y[0][surv] = c->rs;
    s->y[1][surv] = c->vs;
    ro_calc_physical_properties(&c->p1, &c->p2, &c->ps);
    s->p[surv] = c->ps;
    s->md[merg].id *= -1;
    s->p[merg].mass = 0.0;
    s->p[merg].density = 0.0;
    s->p[merg].radius = 0.0;
    s->y[0][merg].x = 1.0e20;
    s->y[0][merg].y = 0.0;
    s->y[0][merg].z = 0.0;
    s->y[1][merg].x = 0.0;
    s->y[1][merg].y = 0.0;
    s->y[1][merg].z = 0.0;
    return RO_OK;
}

/* pp_disk::cpu_check_for_ejection_hit_centrum (pp_disk.cu:934-976) +
 * check_for_ejection_hit_centrum (683-715) + handle_ejection_hit_centrum (1091-1109);
 * the caller's clear_event_counter (main.cu:201-205) is included. */
int ro_check_for_ejection_hit_centrum(ro_sys* s, int* n_handled)
{
    if (!s) return RO_ERR_ARG;
    const int nt = n_total(s);
    const rg_vec_t* r = s->y[0];
    for (int i = 0; i < nt; i++) {
        if (0 < s->md[i].id && RG_BODY_STAR != s->md[i].body_type) {
            double r2 = SQR(r[i].x) + SQR(r[i].y) + SQR(r[i].z);
            if (0.0 < s->thr[RG_THRESHOLD_EJECTION_DISTANCE] &&
                s->thr[RG_THRESHOLD_EJECTION_DISTANCE_SQUARED] < r2) {
                if (s->event_counter >= s->event_cap) return RO_ERR_EVENT_OVERFLOW;
                store_event_data(s, RG_EVENT_EJECTION, s->t, sqrt(r2), 0, i, &s->events[s->event_counter]);
                s->md[i].id *= -1;
                s->event_counter++;
            } else if (0.0 < s->thr[RG_THRESHOLD_HIT_CENTRUM_DISTANCE] &&
                       s->thr[RG_THRESHOLD_HIT_CENTRUM_DISTANCE_SQUARED] > r2) {
                if (s->event_counter >= s->event_cap) return RO_ERR_EVENT_OVERFLOW;
                store_event_data(s, RG_EVENT_HIT_CENTRUM, s->t, sqrt(r2), 0, i, &s->events[s->event_counter]);
                s->md[i].id *= -1;
                s->event_counter++;
            }
        }
    }
    int n_event = s->event_counter;
    if (n_handled) *n_handled = n_event;
    if (0 < n_event) {
        for (int i = 0; i < n_event; i++) {
            rg_event_t e = s->events[i];
            if (e.event_name == RG_EVENT_EJECTION) {
                increment_event_counter(s, s->n_ejection);
            } else {
                int rc = handle_collision_pair(s, &e);
                if (rc) return rc;
                increment_event_counter(s, s->n_hit_centrum);
            }
            int rc = log_push(s, &e);
            if (rc) return rc;
        }
        s->n_ejection[RG_COUNTER_LAST_STEP] = 0;
        s->n_hit_centrum[RG_COUNTER_LAST_STEP] = 0;
        s->event_counter = 0;
    }
    return RO_OK;
}

/* pp_disk::check_for_collision (pp_disk.cu:717-738) -> handle_collision (1078-1089) ->
 * create_sp_events (1111-1149) -> handle_collision_pair; the caller's
 * clear_event_counter (main.cu:245-249) is included. */
int ro_check_for_collision(ro_sys* s, int* n_handled)
{
    if (!s) return RO_ERR_ARG;
    const int ec = s->event_counter;
    if (n_handled) *n_handled = 0;
    if (ec <= 0) return RO_OK;
    rg_event_t* sp = (rg_event_t*)malloc((size_t)ec * sizeof(rg_event_t));
    char* processed = (char*)calloc((size_t)ec, 1);
    if (!sp || !processed) {
        free(sp);
        free(processed);
        return RO_ERR_NOMEM;
    }
    int n = 0;
    for (int k = 0; k < ec; k++) {
        if (processed[k]) continue;
        processed[k] = 1;
        sp[n] = s->events[k];
        for (int i = k + 1; i < ec; i++) {
            if (sp[n].id1 == s->events[i].id1 && sp[n].id2 == s->events[i].id2) {
                processed[i] = 1;
                if (sp[n].t > s->events[i].t) sp[n] = s->events[i];
            }
        }
        n++;
    }
    int rc = RO_OK;
    for (int i = 0; i < n && !rc; i++) {
        rc = handle_collision_pair(s, &sp[i]);
        if (rc) break;
        increment_event_counter(s, s->n_collision);
        rc = log_push(s, &sp[i]);
    }
    free(sp);
    free(processed);
    if (rc) return rc;
    s->n_collision[RG_COUNTER_LAST_STEP] = 0;
    s->event_counter = 0;
    if (n_handled) *n_handled = n;
    return RO_OK;
}

/* pp_disk::check_for_close_encounter(true) (pp_disk.cu:742-770) + clear (main.cu:228-231) */
int ro_check_for_close_encounter(ro_sys* s, int* n_handled)
{
    if (!s) return RO_ERR_ARG;
    const int ec = s->event_counter;
    if (n_handled) *n_handled = ec;
    if (ec <= 0) return RO_OK;
    for (int i = 0; i < ec; i++) {
        int rc = log_push(s, &s->events[i]);
        if (rc) return rc;
        increment_event_counter(s, s->n_close_encounter);
    }
    s->n_close_encounter[RG_COUNTER_LAST_STEP] = 0;
    s->event_counter = 0;
    return RO_OK;
}

/* New: log the pairs that entered their mutual Hill sphere at the start of the last
 * step (candidates recorded by the stage-0 force evaluation). */
static int handle_hill(ro_sys* s)
{
    if (s->hill_factor <= 0.0) return RO_OK;
    int64_t* cur = (int64_t*)malloc((size_t)(s->n_hill > 0 ? s->n_hill : 1) * sizeof(int64_t));
    if (!cur) return RO_ERR_NOMEM;
    int n_cur = 0;
    for (int k = 0; k < s->n_hill; k++) {
        const rg_event_t* e = &s->hill[k];
        int64_t key = ((int64_t)(uint32_t)e->id1 << 32) | (int64_t)(uint32_t)e->id2;
        int seen = 0;
        for (int q = 0; q < s->n_hill_pairs; q++)
            if (s->hill_pairs[q] == key) { seen = 1; break; }
        if (!seen) {
            int rc = log_push(s, e);
            if (rc) { free(cur); return rc; }
            increment_event_counter(s, s->n_close_encounter);
        }
        cur[n_cur++] = key;
    }
    free(s->hill_pairs);
    s->hill_pairs = cur;
    s->n_hill_pairs = n_cur;
    s->n_hill = 0;
    return RO_OK;
}

/* number_of_bodies::update_numbers (number_of_bodies.cpp:27-104) +
 * pp_disk::remove_inactive_bodies (pp_disk.cu:1324-1409) */
static int remove_inactive_bodies(ro_sys* s)
{
    const int old_n = n_total(s);
    int inactive[7] = {0};
    for (int i = 0; i < old_n; i++) {
        if (!(0 < s->md[i].id && RG_BODY_PADDINGPARTICLE > s->md[i].body_type)) {
            int ty = s->md[i].body_type;
            if (ty < 0 || ty > 6) return RO_ERR_ARG;
            inactive[ty]++;
        }
    }
    for (int k = 0; k < 7; k++) s->n_i[k] += inactive[k];
    s->n_s -= inactive[0]; s->n_gp -= inactive[1]; s->n_rp -= inactive[2]; s->n_pp -= inactive[3];
    s->n_spl -= inactive[4]; s->n_pl -= inactive[5]; s->n_tp -= inactive[6];
    int k = 0;
    for (int i = 0; i < old_n; i++) {
        if (0 < s->md[i].id && RG_BODY_PADDINGPARTICLE > s->md[i].body_type) {
            s->y[0][k] = s->y[0][i];
            s->y[1][k] = s->y[1][i];
            s->p[k] = s->p[i];
            s->md[k] = s->md[i];
            k++;
        }
    }
    if (k != n_total(s)) return RO_ERR_STATE;
    return RO_OK;
}

/* pp_disk::check_for_rebuild_vectors (pp_disk.cu:893-907) */
int ro_check_for_rebuild_vectors(ro_sys* s, int n, int* rebuilt)
{
    if (!s) return RO_ERR_ARG;
    if (rebuilt) *rebuilt = 0;
    if (s->n_event[RG_COUNTER_LAST_CLEAR] >= n) {
        int rc = remove_inactive_bodies(s);
        if (rc) return rc;
        s->n_hit_centrum[RG_COUNTER_LAST_CLEAR] = 0;
        s->n_ejection[RG_COUNTER_LAST_CLEAR] = 0;
        s->n_collision[RG_COUNTER_LAST_CLEAR] = 0;
        s->n_close_encounter[RG_COUNTER_LAST_CLEAR] = 0;
        s->n_event[RG_COUNTER_LAST_CLEAR] = 0;
        if (rebuilt) *rebuilt = 1;
    }
    return RO_OK;
}

/* main.cu:176-263, without file output */
int ro_advance(ro_sys* s, double t_stop_day, int64_t max_steps, int64_t* n_steps)
{
    if (!s) return RO_ERR_ARG;
    if (!s->has_int) return RO_ERR_STATE;
    const double stop = t_stop_day * GAUSS;
    int64_t k = 0;
    int rc = RO_OK;
    while (s->t <= stop && (max_steps <= 0 || k < max_steps)) {
        rc = ro_check_for_ejection_hit_centrum(s, NULL);
        if (rc) break;
        rc = ro_step(s, NULL);
        if (rc) break;
        k++;
        rc = handle_hill(s);
        if (rc) break;
        if (s->close_encounter && s->inner_steps) {
            if (0.0 < s->thr[RG_THRESHOLD_RADII_ENHANCE_FACTOR]) rc = ro_check_for_close_encounter(s, NULL);
        } else if (!s->close_encounter && s->inner_steps) {
            if (0.0 < s->thr[RG_THRESHOLD_RADII_ENHANCE_FACTOR]) rc = ro_check_for_collision(s, NULL);
            if (!rc) rc = ro_check_for_rebuild_vectors(s, 8, NULL);
        }
        if (rc) break;
        if (!isfinite(s->dt_try) || s->dt_try == 0.0) { rc = -4; break; }
    }
    if (n_steps) *n_steps = k;
    return rc;
}

/* ------------------------------------------------------------ accessors */

int ro_events(ro_sys* s, rg_event_t* out, int cap, int* n)
{
    if (!s || !n || cap < 0 || (cap > 0 && !out)) return RO_ERR_ARG;
    int m = s->n_log < cap ? s->n_log : cap;
    if (m > 0) memcpy(out, s->log, (size_t)m * sizeof(rg_event_t));
    memmove(s->log, s->log + m, (size_t)(s->n_log - m) * sizeof(rg_event_t));
    s->n_log -= m;
    *n = m;
    return RO_OK;
}

int ro_event_count(ro_sys* s, int* n)
{
    if (!s || !n) return RO_ERR_ARG;
    *n = s->n_log;
    return RO_OK;
}

int ro_get_n_total(ro_sys* s, rg_counts_t* n, int* nt)
{
    if (!s) return RO_ERR_ARG;
    if (n) {
        n->n_s = s->n_s; n->n_gp = s->n_gp; n->n_rp = s->n_rp; n->n_pp = s->n_pp;
        n->n_spl = s->n_spl; n->n_pl = s->n_pl; n->n_tp = s->n_tp;
    }
    if (nt) *nt = n_total(s);
    return RO_OK;
}

int ro_get_state_internal(ro_sys* s, rg_vec_t* r, rg_vec_t* v, rg_param_t* p,
                          rg_body_metadata_t* md, double* t)
{
    if (!s) return RO_ERR_ARG;
    const int nt = n_total(s);
    if (r) memcpy(r, s->y[0], (size_t)nt * sizeof(rg_vec_t));
    if (v) memcpy(v, s->y[1], (size_t)nt * sizeof(rg_vec_t));
    if (p) memcpy(p, s->p, (size_t)nt * sizeof(rg_param_t));
    if (md) memcpy(md, s->md, (size_t)nt * sizeof(rg_body_metadata_t));
    if (t) *t = s->t;
    return RO_OK;
}

/* file units as print_result_ascii writes them (pp_disk.cu:1710,1720-1722) */
int ro_get_state(ro_sys* s, rg_vec_t* r, rg_vec_t* v, rg_param_t* p, rg_body_metadata_t* md,
                 double* t_day)
{
    int rc = ro_get_state_internal(s, r, v, p, md, NULL);
    if (rc) return rc;
    const int nt = n_total(s);
    if (v)
        for (int i = 0; i < nt; i++) {
            v[i].x = v[i].x * GAUSS;
            v[i].y = v[i].y * GAUSS;
            v[i].z = v[i].z * GAUSS;
        }
    if (t_day) *t_day = s->t / GAUSS;
    return RO_OK;
}

int ro_set_state(ro_sys* s, const rg_vec_t* r, const rg_vec_t* v)
{
    if (!s || !r || !v) return RO_ERR_ARG;
    const int nt = n_total(s);
    for (int i = 0; i < nt; i++) {
        s->y[0][i] = r[i];
        s->y[0][i].w = 0.0;
        s->y[1][i] = v[i];
        s->y[1][i].x /= GAUSS;
        s->y[1][i].y /= GAUSS;
        s->y[1][i].z /= GAUSS;
        s->y[1][i].w = 0.0;
    }
    return RO_OK;
}

int ro_calc_accel(ro_sys* s, rg_vec_t* a)
{
    if (!s || !a) return RO_ERR_ARG;
    int saved = s->event_counter;
    cpu_calc_grav_accel(s, s->t, s->y[0], s->y[1], a, 0, 0);
    s->event_counter = saved;
    return RO_OK;
}

int ro_get_counters(ro_sys* s, rg_counters_t* c)
{
    if (!s || !c) return RO_ERR_ARG;
    memset(c, 0, sizeof(*c));
    c->n_failed_step = s->n_failed;
    c->n_passed_step = s->n_passed;
    c->n_tried_step = s->n_tried;
    for (int i = 0; i < 3; i++) {
        c->n_hit_centrum[i] = s->n_hit_centrum[i];
        c->n_ejection[i] = s->n_ejection[i];
        c->n_collision[i] = s->n_collision[i];
        c->n_close_encounter[i] = s->n_close_encounter[i];
        c->n_event[i] = s->n_event[i];
    }
    c->n_gravity_evals = s->n_gravity_evals;
    c->n_pairs = s->n_pairs;
    return RO_OK;
}

int ro_get_dt(ro_sys* s, double* dt_did_day, double* dt_try_day)
{
    if (!s) return RO_ERR_ARG;
    if (dt_did_day) *dt_did_day = s->dt_did / GAUSS;
    if (dt_try_day) *dt_try_day = s->dt_try / GAUSS;
    return RO_OK;
}

/* New (not in the reference): E = sum m v^2 / 2 - sum_{pairs} m_i m_j / r_ij over the
 * pairs the force model couples (every pair with at least one self-interacting body,
 * both massive and active), G = 1 in internal units; L = sum m r x v.  Neumaier
 * compensated sums, pairs visited as i ascending, j < i ascending. */
typedef struct { double s, c; } ksum;
static void kadd(ksum* k, double x)
{
    double t = k->s + x;
    if (fabs(k->s) >= fabs(x))
        k->c += (k->s - t) + x;
    else
        k->c += (x - t) + k->s;
    k->s = t;
}

int ro_energy(ro_sys* s, double* energy, double angmom[3])
{
    if (!s) return RO_ERR_ARG;
    const int nsi = n_SI(s), nm = n_massive(s), nt = n_total(s);
    const rg_vec_t* r = s->y[0];
    const rg_vec_t* v = s->y[1];
    ksum T = {0, 0}, U = {0, 0}, Lx = {0, 0}, Ly = {0, 0}, Lz = {0, 0};
    for (int i = 0; i < nt; i++) {
        if (s->md[i].id <= 0) continue;
        const double m = s->p[i].mass;
        kadd(&T, 0.5 * m * (v[i].x * v[i].x + v[i].y * v[i].y + v[i].z * v[i].z));
        kadd(&Lx, m * (r[i].y * v[i].z - r[i].z * v[i].y));
        kadd(&Ly, m * (r[i].z * v[i].x - r[i].x * v[i].z));
        kadd(&Lz, m * (r[i].x * v[i].y - r[i].y * v[i].x));
    }
    for (int i = 1; i < nm; i++) {
        if (s->md[i].id <= 0) continue;
        const int jmax = (i < nsi) ? i : nsi; /* NSI bodies couple to SI bodies only */
        for (int j = 0; j < jmax; j++) {
            if (s->md[j].id <= 0) continue;
            double dx = r[j].x - r[i].x, dy = r[j].y - r[i].y, dz = r[j].z - r[i].z;
            double d = sqrt(dx * dx + dy * dy + dz * dz);
            kadd(&U, -(s->p[i].mass * s->p[j].mass) / d);
        }
    }
    if (energy) *energy = (T.s + T.c) + (U.s + U.c);
    if (angmom) {
        angmom[0] = Lx.s + Lx.c;
        angmom[1] = Ly.s + Ly.c;
        angmom[2] = Lz.s + Lz.c;
    }
    return RO_OK;
}
