// kernels.h -- launch arguments of the stage, error, ejection and energy kernels
// (stages.cu) and of the gravity kernels (gravity_fp64.cu, gravity_mixed.cu).
#pragma once

#include "common.cuh"

namespace redgb {

constexpr int MAXT = 9;  // longest stage row (RKF7(8) stage 12)

// Forms of a stage sum; each is the exact expression of one reference kernel.
enum CombineForm {
    FORM_SUM = 0,     // y + dt * (c0 k0 + c1 k1 + ...)           rk8_kernel::calc_ytemp_for_f*, euler sum_vector
    FORM_SCALED = 1,  // y + (c0 * dt) * k0                        rk4_kernel::sum_vector (int_rungekutta4.cu:37-48)
    FORM_ACC = 2,     // acc = y; acc += dt * c_q * k_q (c_q != 0)  rk5_kernel::calc_ytemp / calc_y_np1
    FORM_RK4_NP1 = 3, // y + (b0 dt)(k0 + k3) + (b1 dt)(k1 + k2)    rk4_kernel::calc_y_np1 (int_rungekutta4.cu:50-61)
    FORM_RK8_NP1 = 4  // y + dt (b0 k0 + b5 k5 + b6 (k6 + k7) + b8 (k8 + k9) + b10 k10)  int_rungekutta8.cu:322-333
};

struct CombineArgs {
    const double* y;           // 6 rows
    const double* k[MAXT];     // stage derivatives used by this row (6 rows each)
    double c[MAXT];            // coefficients
    int nterm;
    int form;
    int n;                     // bodies
    int stride;                // row stride of every buffer (>= n)
    const double* dt;          // device scalar: the trial step (internal units)
    double* out_lo;            // rows 0..2 of the result (positions)
    double* out_hi;            // rows 3..5 of the result (velocities)
};

int launch_combine(const CombineArgs& a, cudaStream_t st);

enum ErrForm { ERR_RK4 = 0, ERR_RK5 = 1, ERR_RK8 = 2 };

struct ErrArgs {
    const double* k[6];
    double c[6];
    int form;
    int stride;  // row stride
    int n_err;   // bodies checked per row
    unsigned long long* max_bits;  // device scalar, zeroed before the launch
};

int launch_error_max(const ErrArgs& a, cudaStream_t st);

// Ejection / hit-star candidate (index, kind, r^2).
struct EjectRec {
    int i;
    int kind;  // RG_EVENT_EJECTION or RG_EVENT_HIT_CENTRUM
    double r2;
};

int launch_ejection(const double* x, const double* y, const double* z, const int* id, const int* type, int n,
                    const double* thr, EjectRec* rec, unsigned int* count, unsigned int cap, cudaStream_t st);

// vec_t records (r, v: 4 doubles per body) <-> the 6 state rows of `stride`; v / k on the way
// in, v * k on the way out when `scale`
int launch_records_to_rows(const double* r, const double* v, int n, int stride, double k, double* y, cudaStream_t st);
// dst[c][k] = src[c][keep[k]] for the 6 state rows (stride doubles apart), k < n
int launch_gather_rows(const double* src, double* dst, int stride, const int* keep, int n, cudaStream_t st);
int launch_rows_to_records(const double* y, int n, int stride, double k, bool scale, double* r, double* v,
                           cudaStream_t st);

struct EnergyArgs {
    const double* y;  // 6 rows of stride
    const double* mass;
    const int* id;
    int n, n_si, n_massive, stride;
    double* part;  // 5 rows of n: T, U, Lx, Ly, Lz
};

int launch_energy(const EnergyArgs& a, cudaStream_t st);

// resident pair-parallel CTAs per SM (the kernels are built for it: 80 registers, 256 threads)
constexpr int RG_PAIRPAR_RESIDENT = 3;
int launch_grav_fp64_pairpar(const GravArgs& g, int S, cudaStream_t st);
int launch_astro_terms(const double* x, const double* y, const double* z, const double* mass, int n, double m_star,
                       double* out, long long stride, cudaStream_t st);
int launch_grav_fp64_rowseq(const GravArgs& g, cudaStream_t st);
constexpr int FEW_SINKS_MAX = 8;  // sinks per few-sink tile
int launch_grav_fp64_few(const GravArgs& g, const int* tile_row0, int max_src, double* terms, int rows,
                         long long pitch, const int* dev_row_sink, const int* dev_row_nsrc, const int* dev_row_sys,
                         int group_row0, int group_rows, cudaStream_t st);
// mixed precision (gravity_mixed.cu): positions split into FP32 (hi, lo) once per evaluation
struct SplitPos;
constexpr int MIXED_SINKS_PER_TILE = 128;
constexpr int MIXED_SOURCE_TILE = 256;  // source-chunk lengths are multiples of this
constexpr size_t SPLIT_POS_BYTES = 32;  // per body
int launch_split_coords(const double* x, const double* y, const double* z, int n, SplitPos* out, cudaStream_t st);
int launch_split_positions(const double* x, const double* y, const double* z, const double* m, const int* id,
                           const int* base_of, const int* screen_slot, const double* radius, int n,
                           SplitPos* out, float* rf, unsigned int* smax, bool hill, cudaStream_t st,
                           float2* mass_f2 = nullptr);
constexpr int SCREEN_MAX_WORDS = 4;  // GravArgs::smax per system: radius, mass, star distance, spare
// hold: test hook -- no tile copies are issued, so the kernel's bounded waits run out
int launch_grav_mixed_tiles(const GravArgs& g, const void* split, const int* heavy_end, float near_ratio,
                            int n_chunks, int chunk, double* partial, int n_part, unsigned int* err, bool hold,
                            cudaStream_t st);
// heavy pairs of the mixed-precision mode in double-float arithmetic (gravity_mixed.cu):
// the row kernel for blocks with a few massive sources, the few-sink kernel for the
// star's and giants' own rows (partial: 3 x rows x pitch doubles, pitch >= source chunks)
int launch_grav_df_rowseq(const GravArgs& g, const void* split, cudaStream_t st);
// chunk_hint: sources per CTA (multiple of 256, 256..2048), or 0 for the automatic choice
int launch_grav_df_few(const GravArgs& g, const void* split, const int* tile_row0, int max_src, int max_sinks,
                       int chunk_hint,
                       double* partial, int rows, long long pitch, const int* row_sink, const int* row_nsrc,
                       const int* row_sys, int group_row0, int group_rows, cudaStream_t st);
// heavy-light pairs once for both rows (grav_df_sym) and the heavy rows' sums: segments (the
// tiles) of light bodies (sinks) against their system's SI bodies (sources, at most
// DF_SYM_MAX_HEAVY), CTA c taking segments [cta_seg[c], cta_seg[c + 1]); Tile::part = the
// segment's part of its heavy rows (1-based; part 1 also takes the heavy-heavy pairs),
// tile_row0 = each segment's first heavy row, row_nparts = parts per heavy row (1 + the
// system's segments), ticket = one counter per system, zero before the first launch; with
// mass_f2 (the split masses, launch_split_positions) the kernel splits the FP64 coordinates
// itself and reads no split records
constexpr int DF_SYM_MAX_HEAVY = 4;
constexpr int DF_SYM_RESIDENT = 3;   // CTAs of 256 threads per SM (the kernel's launch bound)
constexpr int DF_SYM_PASS = 256;             // light bodies per pass of a CTA (one per thread)
constexpr double DF_SYM_SEGMENT_COST = 0.6;  // a segment's reduction and barriers, in passes
int launch_grav_df_sym(const GravArgs& g, const int* cta_seg, int n_cta, const void* split, const int* tile_row0,
                       int max_heavy, double* partial, int rows, long long pitch, const int* row_sink,
                       const int* row_nparts, unsigned int* ticket, cudaStream_t st,
                       const float2* mass_f2 = nullptr);

int launch_star_distance(const double* x, const double* y, const double* z, const int* base_of, int n, double* rho,
                         cudaStream_t st);

int measure_pipe_peak(int kind, double* tflops);

}  // namespace redgb
