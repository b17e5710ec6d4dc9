// host_tools.h -- host-side physics helpers of the event handlers: collision merge
// formulas and orbital elements, restated from red.cuda/src/red.cuda.utility/tools.cpp.
// Built with -ffp-contract=off so every expression rounds as the reference's does.
#pragma once

#include <cmath>

#include "../../include/redgb_types.h"

namespace redgb {
namespace host {

constexpr double PI = 3.1415926535897932384626;  // red_macro.h:13
constexpr double FOUR_PI_OVER_THREE = 4.1887902047863909846168578443727;

#define RG_SQR(x) ((x) * (x))
#define RG_CUBE(x) ((x) * (x) * (x))

// tools.cpp:238-243
inline double calculate_radius(double m, double density)
{
    return std::pow(1.0 / FOUR_PI_OVER_THREE * m / density, 1.0 / 3.0);
}

// tools.cpp:263-270
inline void calc_position_after_collision(double m1, double m2, const rg_vec_t* r1, const rg_vec_t* r2, rg_vec_t* r)
{
    const double M = m1 + m2;
    r->x = (m1 * r1->x + m2 * r2->x) / M;
    r->y = (m1 * r1->y + m2 * r2->y) / M;
    r->z = (m1 * r1->z + m2 * r2->z) / M;
}

// tools.cpp:272-279
inline void calc_velocity_after_collision(double m1, double m2, const rg_vec_t* v1, const rg_vec_t* v2, rg_vec_t* v)
{
    const double M = m1 + m2;
    v->x = (m1 * v1->x + m2 * v2->x) / M;
    v->y = (m1 * v1->y + m2 * v2->y) / M;
    v->z = (m1 * v1->z + m2 * v2->z) / M;
}

// tools.cpp:281-290: volume-additive merge, survivor keeps its drag coefficient
inline void calc_physical_properties(const rg_param_t& p1, const rg_param_t& p2, rg_param_t* p)
{
    const double volume = 4.188790204786391 * (RG_CUBE(p1.radius) + RG_CUBE(p2.radius));
    p->mass = p1.mass + p2.mass;
    p->density = p->mass / volume;
    p->radius = calculate_radius(p->mass, p->density);
    p->cd = p1.cd;
}

// tools.cpp:473-484
inline void shift_into_range(double lower, double upper, double& value)
{
    const double range = upper - lower;
    while (value >= upper) value -= range;
    while (value < lower) value += range;
}

// tools.cpp:361-471: phase -> orbital elements
inline int calculate_orbital_element(double mu, rg_orbelem_t* oe, const rg_vec_t* rVec, const rg_vec_t* vVec)
{
    const double sq2 = 1.0e-14;
    const double sq3 = 1.0e-14;
    const double v2 = RG_SQR(vVec->x) + RG_SQR(vVec->y) + RG_SQR(vVec->z);
    const double r2 = RG_SQR(rVec->x) + RG_SQR(rVec->y) + RG_SQR(rVec->z);
    const double r = std::sqrt(r2);
    const double h = v2 / 2.0 - (mu / std::sqrt(r2));
    const rg_vec_t cVec = {rVec->y * vVec->z - rVec->z * vVec->y, rVec->z * vVec->x - rVec->x * vVec->z,
                           rVec->x * vVec->y - rVec->y * vVec->x, 0.0};
    const rg_vec_t lVec = {(-mu / r) * rVec->x + vVec->y * cVec.z - vVec->z * cVec.y,
                           (-mu / r) * rVec->y + vVec->z * cVec.x - vVec->x * cVec.z,
                           (-mu / r) * rVec->z + vVec->x * cVec.y - vVec->y * cVec.x, 0.0};
    const double rv = rVec->x * vVec->x + rVec->y * vVec->y + rVec->z * vVec->z;
    const double c = std::sqrt(RG_SQR(cVec.x) + RG_SQR(cVec.y) + RG_SQR(cVec.z));
    const double l = std::sqrt(RG_SQR(lVec.x) + RG_SQR(lVec.y) + RG_SQR(lVec.z));

    double e2 = 1.0 + 2.0 * RG_SQR(c) * h / (mu * mu);
    if (std::fabs(e2) < sq3) e2 = 0.0;
    const double e = std::sqrt(e2);
    const double a = -mu / (2.0 * h);

    const double cosi = cVec.z / c;
    const double sini = std::sqrt(RG_SQR(cVec.x) + RG_SQR(cVec.y)) / c;
    double incl = std::acos(cosi);
    if (incl < sq2)
        incl = 0.0;
    else if (incl > (PI - sq2))
        incl = PI;

    double node = 0.0;
    if (incl != 0.0 && incl != PI) {
        const double tmpx = -cVec.y / (c * sini);
        const double tmpy = cVec.x / (c * sini);
        node = std::atan2(tmpy, tmpx);
        shift_into_range(0.0, 2.0 * PI, node);
    }

    double E = 0.0, H = 0.0, shH = 0.0, peri = 0.0;
    if (e2 != 0.0) {
        double tmpx = (lVec.x * std::cos(node) + lVec.y * std::sin(node)) / l;
        double tmpy = (-lVec.x * std::sin(node) + lVec.y * std::cos(node)) / (l * cosi);
        peri = std::atan2(tmpy, tmpx);
        shift_into_range(0.0, 2.0 * PI, peri);
        if (h >= 0.0) {
            shH = rv / (RG_SQR(a * mu) / RG_CUBE(c) * e * std::pow(e2 - 1, 1.5));
            H = std::asinh(shH);
        } else {
            tmpx = 1.0 / e * (1.0 - r / a);
            tmpy = rv / (std::sqrt(mu * a) * e);
            E = std::atan2(tmpy, tmpx);
            shift_into_range(0.0, 2.0 * PI, E);
        }
    } else {
        peri = 0.0;
        E = std::atan2(rVec->y, rVec->x);
        shift_into_range(0, 2.0 * PI, E);
    }
    double M = 0.0;
    if (h >= 0.0) {
        M = e * shH - H;
    } else {
        M = E - e * std::sin(E);
        shift_into_range(0, 2.0 * PI, M);
    }
    oe->sma = a;
    oe->ecc = e;
    oe->inc = incl;
    oe->peri = peri;
    oe->node = node;
    oe->mean = M;
    return 0;
}

#undef RG_SQR
#undef RG_CUBE

}  // namespace host
}  // namespace redgb
