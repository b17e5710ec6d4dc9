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

// tools.cpp:292-315
__device__ double kepler_solver(double ecc, double mean, double eps)
{
    if (ecc == 0.0 || mean == 0.0 || mean == IC_PI) return mean;
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
    return E;
}

// tools.cpp:317-359: orbital elements -> position and velocity
__device__ void calculate_phase(double mu, double sma, double ecc, double inc, double peri, double node,
                                double mean, rg_vec_t* r, rg_vec_t* v)
{
    const double E = kepler_solver(ecc, mean, 1.0e-14);
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

}  // extern "C"
