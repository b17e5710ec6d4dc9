// noalloc.cu -- rg_energy_noalloc: the energy / angular-momentum diagnostic of rg_energy
// for bodies the caller already holds in device memory, computed without allocating
// anything.
//
// rg_energy's kernel writes five per-body partials (kinetic energy, pair potential,
// m r x v) into a scratch buffer that the context allocated with the rest of its state,
// and the host sums them.  Here the scratch is a fixed file-scope device array instead:
// its address on each device is looked up once (cudaGetSymbolAddress, with that device
// current) and cached, the per-body kernel reads the caller's records in the reference's
// device layout, and a second kernel adds the partials on the device in body order, with
// the same Neumaier compensation as the host sum of rg_energy, so both entry points give
// the same numbers for the same state.  The four results come back through a copy into a
// local array followed by a synchronisation of the caller's stream.
//
// Nothing in the scratch has to start at zero: every partial is written before it is
// read within one call, and so are the four results.  There is one scratch per device, so
// calls on the same device must not overlap (two host threads, or two streams with the
// work of both calls in flight) -- they would overwrite each other's partials.
//
// The cached address belongs to the CUDA runtime's primary context of that device, the
// context every runtime-API caller uses.  A caller that makes its own driver-API context
// current, or that calls cudaDeviceReset (which destroys the primary context and with it
// the address), is not supported: the kernels would write through an address that is not
// valid in the current context.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <mutex>
#include <string>

#include "../../include/redgb.h"
#include "abi_guard.h"

namespace redgb {
int set_error(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* what, const char* file, int line);
}  // namespace redgb

namespace {

constexpr int MAX_BODIES = RG_ENERGY_NOALLOC_MAX_BODIES;
constexpr int MAX_DEVICES = 64;

// five rows of MAX_BODIES per-body partials (T, U, Lx, Ly, Lz), then the four results
// (energy, Lx, Ly, Lz): 2.5 MiB per device
static __device__ __align__(256) double g_energy_scratch[5 * MAX_BODIES + 8];

std::mutex g_scratch_mutex;
double* g_scratch_ptr[MAX_DEVICES];  // per device: the scratch's address, once looked up

#define NA_CHECK(call)                                                                  \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess) return redgb::cuda_fail(e_, #call, __FILE__, __LINE__); \
    } while (0)

int scratch_of_current_device(double** out)
{
    int dev = -1;
    NA_CHECK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= MAX_DEVICES)
        return redgb::set_error(RG_ERR_ARG, "rg_energy_noalloc: device index beyond 63");
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        NA_CHECK(cudaGetSymbolAddress(&p, g_energy_scratch));
        g_scratch_ptr[dev] = static_cast<double*>(p);
    }
    *out = g_scratch_ptr[dev];
    return RG_OK;
}

// the per-body partials of energy_kernel (stages.cu), read from the reference's records:
// kinetic energy, the potential of the pairs (i, j < i) the force model couples and
// m r x v, in internal units (G = 1)
__global__ void energy_records_kernel(const rg_vec_t* r, const rg_vec_t* v, const rg_param_t* p,
                                      const rg_body_metadata_t* md, int n, int n_si, int n_massive, double* part)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double T = 0, U = 0, Uc = 0, Lx = 0, Ly = 0, Lz = 0;
    if (md[i].id > 0) {
        const double m = p[i].mass;
        const double xi = r[i].x, yi = r[i].y, zi = r[i].z;
        const double vx = v[i].x, vy = v[i].y, vz = v[i].z;
        T = 0.5 * m * (vx * vx + vy * vy + vz * vz);
        Lx = m * (yi * vz - zi * vy);
        Ly = m * (zi * vx - xi * vz);
        Lz = m * (xi * vy - yi * vx);
        if (i >= 1 && i < n_massive) {
            const int jmax = i < n_si ? i : n_si;
            for (int j = 0; j < jmax; j++) {
                if (md[j].id <= 0) continue;
                const double dx = r[j].x - xi, dy = r[j].y - yi, dz = r[j].z - zi;
                const double d = sqrt(dx * dx + dy * dy + dz * dz);
                const double term = -(m * p[j].mass) / d;
                const double t = U + term;
                if (fabs(U) >= fabs(term))
                    Uc += (U - t) + term;
                else
                    Uc += (term - t) + U;
                U = t;
            }
        }
    }
    part[i] = T;
    part[n + i] = U + Uc;
    part[2 * (long long)n + i] = Lx;
    part[3 * (long long)n + i] = Ly;
    part[4 * (long long)n + i] = Lz;
}

// one thread per quantity: Neumaier sum of its n partials in body order (the order of
// rg_energy's host sum), then energy = T + U and the three components of L
__global__ void energy_sum_kernel(const double* part, int n, double* res)
{
    __shared__ double sum[5], comp[5];
    const int q = threadIdx.x;
    if (q < 5) {
        const double* x = part + (long long)q * n;
        double s = 0.0, c = 0.0;
        for (int i = 0; i < n; i++) {
            const double xi = x[i];
            const double t = s + xi;
            if (fabs(s) >= fabs(xi))
                c += (s - t) + xi;
            else
                c += (xi - t) + s;
            s = t;
        }
        sum[q] = s;
        comp[q] = c;
    }
    __syncthreads();
    if (q == 0) {
        res[0] = (sum[0] + comp[0]) + (sum[1] + comp[1]);
        res[1] = sum[2] + comp[2];
        res[2] = sum[3] + comp[3];
        res[3] = sum[4] + comp[4];
    }
}

int energy_noalloc_impl(const rg_counts_t* counts, const rg_vec_t* r, const rg_vec_t* v, const rg_param_t* p,
                       const rg_body_metadata_t* md, void* stream, double* energy, double* angmom)
{
    if (!counts) return redgb::set_error(RG_ERR_ARG, "rg_energy_noalloc: null counts");
    const int c[7] = {counts->n_s, counts->n_gp, counts->n_rp, counts->n_pp, counts->n_spl, counts->n_pl, counts->n_tp};
    long long total = 0;
    for (int q = 0; q < 7; q++) {
        if (c[q] < 0) return redgb::set_error(RG_ERR_ARG, "rg_energy_noalloc: negative body count");
        total += c[q];
    }
    if (total > MAX_BODIES) {
        char msg[160];
        snprintf(msg, sizeof(msg), "rg_energy_noalloc: %lld bodies exceed its fixed scratch of %d bodies", total,
                 MAX_BODIES);
        return redgb::set_error(RG_ERR_ARG, msg);
    }
    const int n = (int)total;
    const int n_si = c[0] + c[1] + c[2] + c[3];
    const int n_massive = n_si + c[4] + c[5];
    if (n == 0) {
        if (energy) *energy = 0.0;
        if (angmom) angmom[0] = angmom[1] = angmom[2] = 0.0;
        return RG_OK;
    }
    if (!r || !v || !p || !md) return redgb::set_error(RG_ERR_ARG, "rg_energy_noalloc: null body array");
    double* scratch = nullptr;
    int rc = scratch_of_current_device(&scratch);
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    double* part = scratch;
    double* res = scratch + 5LL * MAX_BODIES;
    energy_records_kernel<<<(n + 127) / 128, 128, 0, st>>>(r, v, p, md, n, n_si, n_massive, part);
    NA_CHECK(cudaGetLastError());
    energy_sum_kernel<<<1, 32, 0, st>>>(part, n, res);
    NA_CHECK(cudaGetLastError());
    double h[4];
    NA_CHECK(cudaMemcpyAsync(h, res, sizeof(h), cudaMemcpyDeviceToHost, st));
    NA_CHECK(cudaStreamSynchronize(st));
    if (energy) *energy = h[0];
    if (angmom) {
        angmom[0] = h[1];
        angmom[1] = h[2];
        angmom[2] = h[3];
    }
    return RG_OK;
}

}  // namespace

extern "C" {

int rg_energy_noalloc(const rg_counts_t* counts, const rg_vec_t* r, const rg_vec_t* v, const rg_param_t* p,
                      const rg_body_metadata_t* md, void* stream, double* energy, double angmom[3])
{
    RG_GUARD(energy_noalloc_impl(counts, r, v, p, md, stream, energy, angmom));
}

}  // extern "C"
