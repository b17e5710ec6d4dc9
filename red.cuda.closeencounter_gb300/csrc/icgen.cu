// icgen.cu -- seeded synthetic disks generated on the GPU (rg_generate_disks).
//
// The benchmark disks of this project (a star, giant planets on given orbits, a swarm of
// planetesimals or self-gravitating protoplanets, optional test particles), for large
// ensembles: one thread per body, no host loop.  Random numbers come from counter-based
// Philox4x32-10 streams (Salmon, Moraes, Dror & Shaw, "Parallel random numbers: as easy as
// 1, 2, 3", SC 2011): key = the disk's 64-bit seed, counter = (body slot, draw block, 0, 0),
// so every body's draws are independent of the launch shape and of the other disks.
// Distributions: planetesimal masses log-uniform; semi-major axes from a surface density
// Sigma ~ r^-1.5 (dN/da ~ a^-0.5) or uniform; e and i Rayleigh; angles uniform.  Elements go
// to heliocentric positions and velocities (AU, AU/day) by the reference's calculate_phase
// and Kepler solver (tools.cpp:292-359), with mu = k^2 (m_star + m); radii follow from the
// density (tools.cpp:238-243).  The star sits at rest in the origin, as in the reference's
// body files; creating a system moves it to the barycentre (options.cpp:206).
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/redgb.h"
#include "common.cuh"

namespace redgb {

int set_error(int code, const std::string& msg);

namespace {

constexpr double IC_GAUSS2 = 2.959122082855911025e-4;  // k^2 (red_constants.h)
constexpr double IC_FOUR_PI_OVER_THREE = 4.1887902047863909846168578443727;
constexpr double IC_STAR_RADIUS = 0.004649130148;     // AU (the reference's test body lists)
constexpr double IC_STAR_DENSITY = 2375725.607;       // Msun / AU^3
constexpr double IC_GIANT_DENSITY_GCC = 1.33;
constexpr double IC_PI = 3.14159265358979323846;

struct Philox {
    unsigned c[4];
};

// Philox4x32-10: ten rounds of two 32x32 -> 64 multiplications, the key bumped by the Weyl
// constants between rounds (the published multipliers and bumps)
__device__ __forceinline__ Philox philox4x32_10(unsigned c0, unsigned c1, unsigned c2, unsigned c3, unsigned k0,
                                                unsigned k1)
{
    for (int r = 0; r < 10; r++) {
        if (r > 0) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        const unsigned long long p0 = (unsigned long long)0xD2511F53u * c0;
        const unsigned long long p1 = (unsigned long long)0xCD9E8D57u * c2;
        const unsigned hi0 = (unsigned)(p0 >> 32), lo0 = (unsigned)p0;
        const unsigned hi1 = (unsigned)(p1 >> 32), lo1 = (unsigned)p1;
        const unsigned n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
    }
    return Philox{{c0, c1, c2, c3}};
}

// a double in [0, 1) from two 32-bit words (53 random bits)
__device__ __forceinline__ double uniform53(unsigned a, unsigned b)
{
    return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) * (1.0 / 9007199254740992.0);
}

// two uniforms of draw block `blk` of body slot k of a disk
__device__ __forceinline__ void draw2(unsigned long long seed, int k, int blk, double& u0, double& u1)
{
    const Philox x = philox4x32_10((unsigned)k, (unsigned)blk, 0u, 0u, (unsigned)seed, (unsigned)(seed >> 32));
    u0 = uniform53(x.c[0], x.c[1]);
    u1 = uniform53(x.c[2], x.c[3]);
}

__device__ __forceinline__ double rayleigh(double sigma, double u) { return sigma * sqrt(-2.0 * log(1.0 - u)); }

// tools.cpp:292-315; returns 1 when the iteration stopped on its step limit, as the reference
// does
__device__ int kepler_solver(double ecc, double mean, double eps, double* E_out)
{
    if (ecc == 0.0 || mean == 0.0 || mean == IC_PI) {
        *E_out = mean;
        return 0;
    }
    double E = mean + ecc * sin(mean) / (1.0 - sin(mean + ecc) + sin(mean));
    int step = 0;
    while (true) {
        const double E1 = E - (E - ecc * sin(E) - mean) / (1.0 - ecc * cos(E));
        const double error = fabs(E1 - E);
        E = E1;
        bool cont = error > eps;
        if (cont) {
            cont = step <= 15;
            step++;
        }
        if (!cont) break;
    }
    *E_out = E;
    return step > 15 ? 1 : 0;
}

// tools.cpp:317-359: orbital elements -> position and velocity; 1 when the Kepler solver did
// not converge (the reference's return code)
__device__ int calculate_phase(double mu, double sma, double ecc, double inc, double peri, double node,
                               double mean, rg_vec_t* r, rg_vec_t* v)
{
    double E;
    const int status = kepler_solver(ecc, mean, 1.0e-14, &E);
    const double nu = 2.0 * atan(sqrt((1.0 + ecc) / (1.0 - ecc)) * tan(E / 2.0));
    const double p = sma * (1.0 - ecc * ecc);
    const double rr = p / (1.0 + ecc * cos(nu));
    const double kszi = rr * cos(nu), eta = rr * sin(nu);
    const double vkszi = -sqrt(mu / p) * sin(nu);
    const double veta = sqrt(mu / p) * (ecc + cos(nu));
    const double cw = cos(peri), sw = sin(peri), cO = cos(node), sO = sin(node), ci = cos(inc), si = sin(inc);
    const double P[3] = {cw * cO - sw * sO * ci, cw * sO + sw * cO * ci, sw * si};
    const double Q[3] = {-sw * cO - cw * sO * ci, -sw * sO + cw * cO * ci, cw * si};
    *r = rg_vec_t{kszi * P[0] + eta * Q[0], kszi * P[1] + eta * Q[1], kszi * P[2] + eta * Q[2], 0.0};
    *v = rg_vec_t{vkszi * P[0] + veta * Q[0], vkszi * P[1] + veta * Q[1], vkszi * P[2] + veta * Q[2], 0.0};
    return status;
}

__device__ double radius_of(double m, double rho) { return pow(1.0 / IC_FOUR_PI_OVER_THREE * m / rho, 1.0 / 3.0); }

struct GenArgs {
    const rg_disk_spec_t* specs;
    const long long* offset;  // per disk: first record
    const int* disk_of_block; // per CTA: its disk
    const int* block0;        // per disk: its first CTA
    double gram_cc;           // g/cm^3 -> Msun/AU^3
    rg_vec_t* r;
    rg_vec_t* v;
    rg_param_t* p;
    rg_body_metadata_t* md;
};

__global__ void generate_disks_kernel(GenArgs a)
{
    const int s = a.disk_of_block[blockIdx.x];
    const rg_disk_spec_t sp = a.specs[s];
    const int k = (blockIdx.x - a.block0[s]) * blockDim.x + threadIdx.x;  // slot within the disk
    const int n_gp = sp.n_giants;
    const int n_total = 1 + n_gp + sp.n_pl + sp.n_tp;
    if (k >= n_total) return;
    const long long o = a.offset[s] + k;
    const double m_star = 1.0;
    rg_vec_t r{0.0, 0.0, 0.0, 0.0}, v{0.0, 0.0, 0.0, 0.0};
    rg_param_t p{0.0, 0.0, 0.0, 0.0};
    int type;
    if (k == 0) {
        type = RG_BODY_STAR;
        p = rg_param_t{m_star, IC_STAR_RADIUS, IC_STAR_DENSITY, 0.0};
    } else if (k <= n_gp) {
        type = RG_BODY_GIANTPLANET;
        const int g = k - 1;
        const double m = sp.giant_m[g];
        const double rho = IC_GIANT_DENSITY_GCC * a.gram_cc;
        double u_mean, u_peri;
        draw2(sp.seed, k, 0, u_mean, u_peri);
        calculate_phase(IC_GAUSS2 * (m_star + m), sp.giant_a[g], sp.giant_e[g], 0.0, 2.0 * IC_PI * u_peri, 0.0,
                        2.0 * IC_PI * u_mean, &r, &v);
        p = rg_param_t{m, radius_of(m, rho), rho, 0.0};
    } else if (k <= n_gp + sp.n_pl) {
        type = sp.pl_type;
        double um, ua, ue, ui, uw, uO, uM, unused;
        draw2(sp.seed, k, 0, um, ua);
        draw2(sp.seed, k, 1, ue, ui);
        draw2(sp.seed, k, 2, uw, uO);
        draw2(sp.seed, k, 3, uM, unused);
        const double lo = log(sp.m_lo), hi = log(sp.m_hi);
        const double m = exp(lo + um * (hi - lo));
        double sma;
        if (sp.a_mode == 0) {
            const double s0 = sqrt(sp.a_lo), s1 = sqrt(sp.a_hi);
            const double x = s0 + ua * (s1 - s0);
            sma = x * x;
        } else {
            sma = sp.a_lo + ua * (sp.a_hi - sp.a_lo);
        }
        const double ecc = fmin(rayleigh(sp.sigma_e, ue), 0.9);
        const double inc = rayleigh(sp.sigma_i, ui);
        const double rho = sp.rho_pl * a.gram_cc;
        calculate_phase(IC_GAUSS2 * (m_star + m), sma, ecc, inc, 2.0 * IC_PI * uw, 2.0 * IC_PI * uO, 2.0 * IC_PI * uM,
                        &r, &v);
        p = rg_param_t{m, radius_of(m, rho), rho, 0.0};
    } else {
        type = RG_BODY_TESTPARTICLE;
        double ua, ue, ui, uw, uO, uM;
        draw2(sp.seed, k, 0, ua, ue);
        draw2(sp.seed, k, 1, ui, uw);
        draw2(sp.seed, k, 2, uO, uM);
        const double sma = sp.a_lo + ua * (sp.a_hi - sp.a_lo);
        calculate_phase(IC_GAUSS2 * m_star, sma, fmin(rayleigh(sp.sigma_e, ue), 0.9), rayleigh(sp.sigma_i, ui),
                        2.0 * IC_PI * uw, 2.0 * IC_PI * uO, 2.0 * IC_PI * uM, &r, &v);
    }
    a.r[o] = r;
    a.v[o] = v;
    a.p[o] = p;
    rg_body_metadata_t m{};
    m.id = k + 1;
    m.body_type = type;
    m.mig_type = 0;
    m.mig_stop_at = 0.0;
    a.md[o] = m;
}

template <typename T>
int dalloc_t(T** p, size_t n)
{
    if (n == 0) n = 1;
    if (cudaMalloc((void**)p, n * sizeof(T)) != cudaSuccess) return set_error(RG_ERR_NOMEM, "cudaMalloc");
    return RG_OK;
}

}  // namespace

static int generate_impl(int n_sys, const rg_disk_spec_t* specs, rg_counts_t* counts, rg_vec_t* r, rg_vec_t* v,
                         rg_param_t* p, rg_body_metadata_t* md)
{
    constexpr int NT = 256;
    std::vector<long long> offset(n_sys);
    std::vector<int> block0(n_sys), disk_of_block;
    long long total = 0;
    for (int s = 0; s < n_sys; s++) {
        const rg_disk_spec_t& sp = specs[s];
        if (sp.n_pl < 0 || sp.n_tp < 0 || sp.n_giants < 0 || sp.n_giants > 4 ||
            (sp.pl_type != RG_BODY_PROTOPLANET && sp.pl_type != RG_BODY_PLANETESIMAL) || !(sp.m_lo > 0.0) ||
            !(sp.m_hi >= sp.m_lo) || !(sp.a_lo > 0.0) || !(sp.a_hi >= sp.a_lo) || (sp.a_mode != 0 && sp.a_mode != 1))
            return set_error(RG_ERR_ARG, "rg_generate_disks: invalid disk specification " + std::to_string(s));
        const int n = 1 + sp.n_giants + sp.n_pl + sp.n_tp;
        const bool si = sp.pl_type == RG_BODY_PROTOPLANET;
        counts[s] = rg_counts_t{1, sp.n_giants, 0, si ? sp.n_pl : 0, 0, si ? 0 : sp.n_pl, sp.n_tp};
        offset[s] = total;
        block0[s] = (int)disk_of_block.size();
        for (int b = 0; b < (n + NT - 1) / NT; b++) disk_of_block.push_back(s);
        total += n;
    }
    if (total == 0) return RG_OK;
    rg_disk_spec_t* d_specs = nullptr;
    long long* d_off = nullptr;
    int *d_dob = nullptr, *d_b0 = nullptr;
    rg_vec_t *d_r = nullptr, *d_v = nullptr;
    rg_param_t* d_p = nullptr;
    rg_body_metadata_t* d_md = nullptr;
    int rc = dalloc_t(&d_specs, (size_t)n_sys);
    if (!rc) rc = dalloc_t(&d_off, (size_t)n_sys);
    if (!rc) rc = dalloc_t(&d_dob, disk_of_block.size());
    if (!rc) rc = dalloc_t(&d_b0, (size_t)n_sys);
    if (!rc) rc = dalloc_t(&d_r, (size_t)total);
    if (!rc) rc = dalloc_t(&d_v, (size_t)total);
    if (!rc) rc = dalloc_t(&d_p, (size_t)total);
    if (!rc) rc = dalloc_t(&d_md, (size_t)total);
    auto check = [&](cudaError_t e, const char* what) {
        if (!rc && e != cudaSuccess) rc = cuda_fail(e, what, __FILE__, __LINE__);
    };
    if (!rc) {
        check(cudaMemcpy(d_specs, specs, n_sys * sizeof(rg_disk_spec_t), cudaMemcpyHostToDevice), "specs");
        check(cudaMemcpy(d_off, offset.data(), n_sys * sizeof(long long), cudaMemcpyHostToDevice), "offsets");
        check(cudaMemcpy(d_dob, disk_of_block.data(), disk_of_block.size() * sizeof(int), cudaMemcpyHostToDevice),
              "blocks");
        check(cudaMemcpy(d_b0, block0.data(), n_sys * sizeof(int), cudaMemcpyHostToDevice), "blocks");
        // the metadata records have 4 bytes of padding that the kernel's stores may skip
        check(cudaMemset(d_md, 0, total * sizeof(rg_body_metadata_t)), "md");
    }
    if (!rc) {
        // g/cm^3 -> Msun/AU^3 (constants::GramPerCm3ToSolarPerAu3: 1 Msun = 1.98911e33 g,
        // 1 AU = 1.495978707e11 m)
        const double gram_cc = (1.0 / (1.0e3 * 1.98911e30)) / std::pow(1.0e-2 * (1.0 / 1.495978707e11), 3.0);
        GenArgs a{d_specs, d_off, d_dob, d_b0, gram_cc, d_r, d_v, d_p, d_md};
        generate_disks_kernel<<<(unsigned)disk_of_block.size(), NT>>>(a);
        check(cudaGetLastError(), "generate_disks_kernel");
        check(cudaMemcpy(r, d_r, total * sizeof(rg_vec_t), cudaMemcpyDeviceToHost), "r");
        check(cudaMemcpy(v, d_v, total * sizeof(rg_vec_t), cudaMemcpyDeviceToHost), "v");
        check(cudaMemcpy(p, d_p, total * sizeof(rg_param_t), cudaMemcpyDeviceToHost), "p");
        check(cudaMemcpy(md, d_md, total * sizeof(rg_body_metadata_t), cudaMemcpyDeviceToHost), "md");
    }
    cudaFree(d_specs);
    cudaFree(d_off);
    cudaFree(d_dob);
    cudaFree(d_b0);
    cudaFree(d_r);
    cudaFree(d_v);
    cudaFree(d_p);
    cudaFree(d_md);
    return rc;
}

// ------------------------------------------------------------------ rg_populate_disks
namespace {

constexpr int POP_ITEM0 = 16;  // Philox draw block of item t (pp 0-3, oe 4-9): POP_ITEM0 + t

constexpr int POW_MAX_ATTEMPTS = 10000;  // rejection attempts of one power-law draw

// two uniforms of draw block `blk`, attempt `att` of body slot k (attempt 0 = draw2)
__device__ __forceinline__ void draw2a(unsigned long long seed, int k, int blk, int att, double& u0, double& u1)
{
    const Philox x = philox4x32_10((unsigned)k, (unsigned)blk, (unsigned)att, 0u, (unsigned)seed, (unsigned)(seed >> 32));
    u0 = uniform53(x.c[0], x.c[1]);
    u1 = uniform53(x.c[2], x.c[3]);
}

// One value of distribution d for body slot k from draw block blk (distribution.cpp:117-249);
// u = 1 - u0 lies in (0, 1] like the reference's (rand() + 1) / 2^32.  The power law repeats
// the reference's rejection steps (so its density is x^power - min(x_min^power,
// x_max^power), as the reference's is); the lognormal, whose rejection samples the true
// truncated density, is drawn by its inverse distribution function.  *fail is set when the
// rejection loop reaches its attempt limit.
__device__ double sample_dist(const rg_dist_t& d, unsigned long long seed, int k, int blk, int* fail)
{
    double u0, u1;
    draw2(seed, k, blk, u0, u1);
    const double u = 1.0 - u0;
    switch (d.kind) {
    case RG_DIST_UNIFORM: return d.p[0] + (d.p[1] - d.p[0]) * u;
    case RG_DIST_EXPONENTIAL: return -1.0 / d.p[0] * log(u);
    case RG_DIST_RAYLEIGH: return d.p[0] * sqrt(-2.0 * log(u));
    case RG_DIST_NORMAL: return d.p[0] + d.p[1] * sqrt(-2.0 * log(u)) * cos(2.0 * IC_PI * (1.0 - u1));
    case RG_DIST_POWER_LAW: {  // distribution.cpp:187-207
        const double x0 = d.p[0], x1 = d.p[1], pw = d.p[2];
        double y_min = pw == 0.0 ? 0.0 : pow(x0, pw), y_max = pw == 0.0 ? 1.0 : pow(x1, pw);
        if (y_min > y_max) {
            const double t = y_min;
            y_min = y_max;
            y_max = t;
        }
        const double d_y = y_max - y_min, d_x = x1 - x0, area_max = d_x * d_y;
        if (!(d_y > 0.0)) return x0;  // an empty range: the reference would divide 0 by 0
        for (int att = 0; att < POW_MAX_ATTEMPTS; att++) {
            if (att > 0) draw2a(seed, k, blk, att, u0, u1);
            const double x = area_max * (1.0 - u0) / d_y + x0;
            const double y = y_min + (y_max - y_min) * (1.0 - u1);
            if (!(y > pow(x, pw))) return x;
        }
        *fail = 1;
        return x0;
    }
    case RG_DIST_LOGNORMAL: {  // inverse of the truncated distribution function
        const double x0 = d.p[0], x1 = d.p[1], mu = d.p[2], sg = d.p[3];
        const double c0 = normcdf((log(x0) - mu) / sg), c1 = normcdf((log(x1) - mu) / sg);
        const double x = exp(mu + sg * normcdfinv(c0 + u0 * (c1 - c0)));
        return fmin(fmax(x, x0), x1);
    }
    case RG_DIST_LOG_UNIFORM: return exp(log(d.p[0]) + u0 * (log(d.p[1]) - log(d.p[0])));
    default: return 0.0;
    }
}

// tools.cpp:245-261
__device__ double density_of(double m, double R)
{
    if (R == 0.0) return 0.0;
    return m / (IC_FOUR_PI_OVER_THREE * (R * R * R));
}
__device__ double mass_of(double R, double rho) { return IC_FOUR_PI_OVER_THREE * (R * R * R) * rho; }

struct PopArgs {
    const rg_body_disk_t* disks;
    const long long* offset;   // per disk: first record
    const int* n_of;           // per disk: bodies
    const int* disk_of_block;  // per CTA: its disk
    const int* block0;         // per disk: its first CTA
    rg_vec_t* r;
    rg_vec_t* v;
    rg_param_t* p;
    rg_body_metadata_t* md;
    double* oe;                // 6 per body
    int* err;                  // per disk: 1 phase, 2 mass target, 4 rejection limit
};

__device__ int body_type_of(const rg_body_disk_t& D, int k)
{
    int type = 0, first = 0;
    while (type < 6 && k >= first + D.n_body[type]) first += D.n_body[type++];
    return type;
}

// populate_disk (main.cu:29-86): one thread per body
__global__ void populate_draw_kernel(PopArgs a)
{
    const int s = a.disk_of_block[blockIdx.x];
    const rg_body_disk_t& D = a.disks[s];
    const int k = (blockIdx.x - a.block0[s]) * blockDim.x + threadIdx.x;
    if (k >= a.n_of[s]) return;
    const long long o = a.offset[s] + k;
    const int type = body_type_of(D, k);
    double pp[RG_PP_N] = {0.0, 0.0, 0.0, 0.0};
    int fail = 0;
    for (int t = 0; t < RG_PP_N; t++)
        if (D.pp[type][t].kind != RG_DIST_NONE) pp[t] = sample_dist(D.pp[type][t], D.seed, k, POP_ITEM0 + t, &fail);
    if (type != RG_BODY_SUPERPLANETESIMAL) {  // the host has refused any other combination
        const bool hm = D.pp[type][RG_PP_MASS].kind != RG_DIST_NONE;
        const bool hr = D.pp[type][RG_PP_RADIUS].kind != RG_DIST_NONE;
        const bool hd = D.pp[type][RG_PP_DENSITY].kind != RG_DIST_NONE;
        if (!hm && hr && hd)
            pp[RG_PP_MASS] = mass_of(pp[RG_PP_RADIUS], pp[RG_PP_DENSITY]);
        else if (!hr && hm && hd)
            pp[RG_PP_RADIUS] = radius_of(pp[RG_PP_MASS], pp[RG_PP_DENSITY]);
        else if (!hd && hm && hr)
            pp[RG_PP_DENSITY] = density_of(pp[RG_PP_MASS], pp[RG_PP_RADIUS]);
    }
    a.p[o] = rg_param_t{pp[0], pp[1], pp[2], pp[3]};
    for (int e = 0; e < RG_OE_N; e++) {
        double x = 0.0;
        if (type != RG_BODY_STAR && D.oe[type][e].kind != RG_DIST_NONE)
            x = sample_dist(D.oe[type][e], D.seed, k, POP_ITEM0 + RG_PP_N + e, &fail);
        a.oe[6 * o + e] = x;
    }
    if (fail) atomicOr(&a.err[s], 4);
    rg_body_metadata_t m{};
    m.id = k + 1;
    m.body_type = type;
    m.mig_type = 0;
    m.mig_stop_at = 0.0;
    a.md[o] = m;
}

// the protoplanets' total mass, summed from the last body down (tools.cpp:93-107)
__device__ double protoplanet_mass(const PopArgs& a, long long o0, int n)
{
    double tot = 0.0;
    for (int j = n - 1; j >= 0; j--)
        if (a.md[o0 + j].body_type == RG_BODY_PROTOPLANET) tot += a.p[o0 + j].mass;
    return tot;
}

// mass scaling and re-derivation (main.cu:472-509): one thread per disk, serial in the
// reference's order
__global__ void populate_scale_kernel(PopArgs a, int n_sys)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n_sys) return;
    const rg_body_disk_t& D = a.disks[s];
    if (!(D.pp_total_mass > 0.0)) return;
    const long long o0 = a.offset[s];
    const int n = a.n_of[s];
    const double f = D.pp_total_mass / protoplanet_mass(a, o0, n);
    for (int j = 0; j < n; j++)
        if (a.md[o0 + j].body_type == RG_BODY_PROTOPLANET) a.p[o0 + j].mass *= f;
    if (fabs(protoplanet_mass(a, o0, n) - D.pp_total_mass) > 1.0e-15) a.err[s] |= 2;
    for (int j = 0; j < n; j++) {
        rg_param_t& q = a.p[o0 + j];
        const int type = a.md[o0 + j].body_type;
        if (q.mass > 0.0) {
            const bool hr = D.pp[type][RG_PP_RADIUS].kind != RG_DIST_NONE;
            const bool hd = D.pp[type][RG_PP_DENSITY].kind != RG_DIST_NONE;
            if (!hd && hr) q.density = density_of(q.mass, q.radius);
            if (!hr && hd) q.radius = radius_of(q.mass, q.density);
        }
    }
}

// positions and velocities (main.cu:511-536): the first body at rest in the origin
__global__ void populate_phase_kernel(PopArgs a)
{
    const int s = a.disk_of_block[blockIdx.x];
    const int k = (blockIdx.x - a.block0[s]) * blockDim.x + threadIdx.x;
    if (k >= a.n_of[s]) return;
    const long long o0 = a.offset[s], o = o0 + k;
    rg_vec_t r{0.0, 0.0, 0.0, 0.0}, v{0.0, 0.0, 0.0, 0.0};
    if (k > 0) {
        const double mu = IC_GAUSS2 * (a.p[o0].mass + a.p[o].mass);
        const double* e = a.oe + 6 * o;
        if (calculate_phase(mu, e[RG_OE_SMA], e[RG_OE_ECC], e[RG_OE_INC], e[RG_OE_PERI], e[RG_OE_NODE],
                            e[RG_OE_MEAN], &r, &v))
            atomicOr(&a.err[s], 1);
    }
    a.r[o] = r;
    a.v[o] = v;
}

// tools::transform_to_bc (tools.cpp:122-176): one thread per disk, sums from the last body
// down as compute_bc does
__global__ void populate_bc_kernel(PopArgs a, int n_sys)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n_sys || !a.disks[s].to_bc) return;
    const long long o0 = a.offset[s];
    const int n = a.n_of[s];
    double R0[3] = {0.0, 0.0, 0.0}, V0[3] = {0.0, 0.0, 0.0}, M0 = 0.0;
    for (int j = n - 1; j >= 0; j--) {
        const double m = a.p[o0 + j].mass;
        const rg_vec_t r = a.r[o0 + j], v = a.v[o0 + j];
        R0[0] += m * r.x; R0[1] += m * r.y; R0[2] += m * r.z;
        V0[0] += m * v.x; V0[1] += m * v.y; V0[2] += m * v.z;
    }
    for (int j = n - 1; j >= 0; j--) M0 += a.p[o0 + j].mass;
    for (int c = 0; c < 3; c++) {
        R0[c] /= M0;
        V0[c] /= M0;
    }
    for (int j = n - 1; j >= 0; j--) {
        rg_vec_t& r = a.r[o0 + j];
        rg_vec_t& v = a.v[o0 + j];
        r.x -= R0[0]; r.y -= R0[1]; r.z -= R0[2];
        v.x -= V0[0]; v.y -= V0[1]; v.z -= V0[2];
    }
}

bool dist_ok(const rg_dist_t& d)
{
    const double* q = d.p;
    switch (d.kind) {
    case RG_DIST_NONE:
    case RG_DIST_UNIFORM:
    case RG_DIST_NORMAL: return std::isfinite(q[0]) && std::isfinite(q[1]);
    case RG_DIST_EXPONENTIAL: return q[0] > 0.0 && std::isfinite(q[0]);
    case RG_DIST_RAYLEIGH: return q[0] >= 0.0 && std::isfinite(q[0]);
    case RG_DIST_POWER_LAW: return q[0] > 0.0 && q[1] >= q[0] && std::isfinite(q[1]) && std::isfinite(q[2]);
    case RG_DIST_LOGNORMAL:
        return q[0] >= 0.0 && q[1] > q[0] && std::isfinite(q[1]) && std::isfinite(q[2]) && q[3] > 0.0 &&
               std::isfinite(q[3]);
    case RG_DIST_LOG_UNIFORM: return q[0] > 0.0 && q[1] >= q[0] && std::isfinite(q[1]);
    default: return false;
    }
}

}  // namespace

static int populate_impl(int n_sys, const rg_body_disk_t* disks, rg_counts_t* counts, rg_vec_t* r, rg_vec_t* v,
                         rg_param_t* p, rg_body_metadata_t* md)
{
    constexpr int NT = 256;
    std::vector<long long> offset(n_sys);
    std::vector<int> n_of(n_sys), block0(n_sys), disk_of_block;
    long long total = 0;
    for (int s = 0; s < n_sys; s++) {
        const rg_body_disk_t& D = disks[s];
        long long n = 0;
        for (int t = 0; t < 7; t++) {
            if (D.n_body[t] < 0) return set_error(RG_ERR_ARG, "rg_populate_disks: negative body count, disk " + std::to_string(s));
            n += D.n_body[t];
            for (int e = 0; e < RG_OE_N; e++)
                if (!dist_ok(D.oe[t][e]))
                    return set_error(RG_ERR_ARG, "rg_populate_disks: invalid element distribution, disk " + std::to_string(s));
            for (int e = 0; e < RG_PP_N; e++)
                if (!dist_ok(D.pp[t][e]))
                    return set_error(RG_ERR_ARG, "rg_populate_disks: invalid property distribution, disk " + std::to_string(s));
            if (D.n_body[t] > 0 && t != RG_BODY_SUPERPLANETESIMAL) {
                const int missing = (D.pp[t][RG_PP_MASS].kind == RG_DIST_NONE) + (D.pp[t][RG_PP_RADIUS].kind == RG_DIST_NONE) +
                                    (D.pp[t][RG_PP_DENSITY].kind == RG_DIST_NONE);
                if (missing != 1)
                    return set_error(RG_ERR_ARG, "rg_populate_disks: missing physical parameters (exactly one of mass, "
                                                 "radius and density is derived), disk " + std::to_string(s));
            }
        }
        if (n > (1 << 30)) return set_error(RG_ERR_ARG, "rg_populate_disks: disk too large, disk " + std::to_string(s));
        counts[s] = rg_counts_t{D.n_body[0], D.n_body[1], D.n_body[2], D.n_body[3], D.n_body[4], D.n_body[5], D.n_body[6]};
        offset[s] = total;
        n_of[s] = (int)n;
        block0[s] = (int)disk_of_block.size();
        for (long long b = 0; b < (n + NT - 1) / NT; b++) disk_of_block.push_back(s);
        total += n;
    }
    if (total == 0) return RG_OK;
    std::vector<int> err(n_sys, 0);  // host allocations first: nothing after the device ones throws
    rg_body_disk_t* d_disks = nullptr;
    long long* d_off = nullptr;
    int *d_n = nullptr, *d_dob = nullptr, *d_b0 = nullptr, *d_err = nullptr;
    rg_vec_t *d_r = nullptr, *d_v = nullptr;
    rg_param_t* d_p = nullptr;
    rg_body_metadata_t* d_md = nullptr;
    double* d_oe = nullptr;
    int rc = dalloc_t(&d_disks, (size_t)n_sys);
    if (!rc) rc = dalloc_t(&d_off, (size_t)n_sys);
    if (!rc) rc = dalloc_t(&d_n, (size_t)n_sys);
    if (!rc) rc = dalloc_t(&d_dob, disk_of_block.size());
    if (!rc) rc = dalloc_t(&d_b0, (size_t)n_sys);
    if (!rc) rc = dalloc_t(&d_err, (size_t)n_sys);
    if (!rc) rc = dalloc_t(&d_r, (size_t)total);
    if (!rc) rc = dalloc_t(&d_v, (size_t)total);
    if (!rc) rc = dalloc_t(&d_p, (size_t)total);
    if (!rc) rc = dalloc_t(&d_md, (size_t)total);
    if (!rc) rc = dalloc_t(&d_oe, (size_t)total * RG_OE_N);
    auto check = [&](cudaError_t e, const char* what) {
        if (!rc && e != cudaSuccess) rc = cuda_fail(e, what, __FILE__, __LINE__);
    };
    if (!rc) {
        check(cudaMemcpy(d_disks, disks, n_sys * sizeof(rg_body_disk_t), cudaMemcpyHostToDevice), "disks");
        check(cudaMemcpy(d_off, offset.data(), n_sys * sizeof(long long), cudaMemcpyHostToDevice), "offsets");
        check(cudaMemcpy(d_n, n_of.data(), n_sys * sizeof(int), cudaMemcpyHostToDevice), "counts");
        check(cudaMemcpy(d_dob, disk_of_block.data(), disk_of_block.size() * sizeof(int), cudaMemcpyHostToDevice),
              "blocks");
        check(cudaMemcpy(d_b0, block0.data(), n_sys * sizeof(int), cudaMemcpyHostToDevice), "blocks");
        check(cudaMemset(d_err, 0, n_sys * sizeof(int)), "err");
        check(cudaMemset(d_md, 0, total * sizeof(rg_body_metadata_t)), "md");  // padding bytes
    }
    if (!rc) {
        PopArgs a{d_disks, d_off, d_n, d_dob, d_b0, d_r, d_v, d_p, d_md, d_oe, d_err};
        const unsigned nb = (unsigned)disk_of_block.size(), ns = (unsigned)((n_sys + 63) / 64);
        populate_draw_kernel<<<nb, NT>>>(a);
        check(cudaGetLastError(), "populate_draw_kernel");
        populate_scale_kernel<<<ns, 64>>>(a, n_sys);
        check(cudaGetLastError(), "populate_scale_kernel");
        populate_phase_kernel<<<nb, NT>>>(a);
        check(cudaGetLastError(), "populate_phase_kernel");
        populate_bc_kernel<<<ns, 64>>>(a, n_sys);
        check(cudaGetLastError(), "populate_bc_kernel");
        check(cudaMemcpy(err.data(), d_err, n_sys * sizeof(int), cudaMemcpyDeviceToHost), "err");
        check(cudaMemcpy(r, d_r, total * sizeof(rg_vec_t), cudaMemcpyDeviceToHost), "r");
        check(cudaMemcpy(v, d_v, total * sizeof(rg_vec_t), cudaMemcpyDeviceToHost), "v");
        check(cudaMemcpy(p, d_p, total * sizeof(rg_param_t), cudaMemcpyDeviceToHost), "p");
        check(cudaMemcpy(md, d_md, total * sizeof(rg_body_metadata_t), cudaMemcpyDeviceToHost), "md");
    }
    cudaFree(d_disks);
    cudaFree(d_off);
    cudaFree(d_n);
    cudaFree(d_dob);
    cudaFree(d_b0);
    cudaFree(d_err);
    cudaFree(d_r);
    cudaFree(d_v);
    cudaFree(d_p);
    cudaFree(d_md);
    cudaFree(d_oe);
    if (rc) return rc;
    for (int s = 0; s < n_sys; s++) {
        if (err[s] & 1)
            return set_error(RG_ERR_ARG, "rg_populate_disks: could not calculate the phase, disk " + std::to_string(s));
        if (err[s] & 2)
            return set_error(RG_ERR_ARG, "rg_populate_disks: the required mass was not reached, disk " + std::to_string(s));
        if (err[s] & 4)
            return set_error(RG_ERR_ARG, "rg_populate_disks: a power-law draw reached its attempt limit, disk " +
                                             std::to_string(s));
    }
    return RG_OK;
}

// nebula.cpp:23-95 (host arithmetic, as the reference computes it)
static double mmsn_gas(const rg_mmsn_component_t& c)
{
    const double p2 = c.p + 2.0;
    if (p2 != 0.0) return 2.0 * IC_PI * c.f_neb * c.f * c.Sigma_1 / p2 * (std::pow(c.r_2, p2) - std::pow(c.r_1, p2));
    return 2.0 * IC_PI * c.f_neb * c.f * c.Sigma_1 * (std::log(c.r_2) - std::log(c.r_1));
}

static double mmsn_solid(const rg_mmsn_component_t& c)
{
    const double p2 = c.p + 2.0;
    const double C = p2 != 0.0 ? 2.0 * IC_PI * c.f_neb * c.Sigma_1 / p2 : 2.0 * IC_PI * c.f_neb * c.Sigma_1;
    auto I = [&](double a, double b) { return p2 != 0.0 ? std::pow(b, p2) - std::pow(a, p2) : std::log(b) - std::log(a); };
    double integral;
    if (c.r_SL <= c.r_1)
        integral = c.f * I(c.r_1, c.r_2);
    else if (c.r_SL <= c.r_2)
        integral = I(c.r_1, c.r_SL) + c.f * I(c.r_SL, c.r_2);
    else
        integral = I(c.r_1, c.r_2);
    return C * integral;
}

}  // namespace redgb

extern "C" {

RG_API int rg_generate_disks(int n_sys, const rg_disk_spec_t* specs, rg_counts_t* counts, rg_vec_t* r, rg_vec_t* v,
                             rg_param_t* p, rg_body_metadata_t* md)
{
    if (n_sys < 0 || (n_sys > 0 && (!specs || !counts || !r || !v || !p || !md)))
        return redgb::set_error(RG_ERR_ARG, "bad argument");
    try {
        return redgb::generate_impl(n_sys, specs, counts, r, v, p, md);
    } catch (...) {
        return redgb::set_error(RG_ERR_STATE, "unexpected exception");
    }
}

RG_API int rg_populate_disks(int n_sys, const rg_body_disk_t* disks, rg_counts_t* counts, rg_vec_t* r, rg_vec_t* v,
                             rg_param_t* p, rg_body_metadata_t* md)
{
    if (n_sys < 0 || (n_sys > 0 && (!disks || !counts || !r || !v || !p || !md)))
        return redgb::set_error(RG_ERR_ARG, "bad argument");
    try {
        return redgb::populate_impl(n_sys, disks, counts, r, v, p, md);
    } catch (const std::bad_alloc&) {
        return redgb::set_error(RG_ERR_NOMEM, "host allocation failed");
    } catch (...) {
        return redgb::set_error(RG_ERR_STATE, "unexpected exception");
    }
}

RG_API int rg_mmsn_gas_mass(const rg_mmsn_component_t* c, double* m)
{
    if (!c || !m) return redgb::set_error(RG_ERR_ARG, "bad argument");
    *m = redgb::mmsn_gas(*c);
    return RG_OK;
}

RG_API int rg_mmsn_solid_mass(const rg_mmsn_component_t* c, double* m)
{
    if (!c || !m) return redgb::set_error(RG_ERR_ARG, "bad argument");
    *m = redgb::mmsn_solid(*c);
    return RG_OK;
}

}  // extern "C"
