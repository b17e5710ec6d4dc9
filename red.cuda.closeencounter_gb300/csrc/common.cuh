// common.cuh -- device data layout and records shared by the kernels and the host driver.
//
// HBM layout of one force evaluation (all FP64, structure of arrays so every kernel reads
// and writes unit-stride, coalesced rows):
//   state y  : 6 rows of n doubles  [rx | ry | rz | vx | vy | vz]
//   stage k_r: 6 rows of n doubles  [v_r (dr/dt) | a_r (dv/dt)]
//   stage positions P: 3 rows of n doubles
//   body data: mass[n], radius[n], id[n] (int32), rho[n] (distance from body 0, Hill test)
// The reference's 4-component vec_t w slot is always 0 and never stored here.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace redgb {

// One rectangular block of the interaction matrix: sinks [sink_begin, sink_end) feel the
// sources [src_begin, src_end) (number_of_bodies::get_bound_SI/NSI/NI,
// number_of_bodies.cpp:196-258).  `sys` is the disk of an ensemble (0 for one disk);
// `base` is the disk's first body.  `block` is 0 for SI, 1 for NSI, 2 for NI sinks.
struct Tile {
    int sink_begin, sink_end;
    int src_begin, src_end;
    int sys, base, block;
    int part;  // a symmetric heavy-light tile (grav_df_sym): its part of the heavy rows, from 1; else 0
};

// A collision / close-encounter / Hill-sphere candidate found by a gravity kernel.
// The host turns it into the reference's 472-byte event_data_t.
struct DevEvent {
    uint32_t seq;   // (attempt << 8) | stage
    int32_t kind;   // 0: radius criterion (pp_disk.cu:265), 1: mutual Hill sphere
    int32_t i, j;   // sink, source (body indices of the whole batch)
    int32_t sys, pad;
    int32_t id1, id2;  // ensembles' device handler: survivor and merger ids, fixed before any merge
    int32_t swap, pad2;  // ... and whether the source is the survivor
    double d;
    double t;  // ensembles: the system's time at the attempt's start (the Hill records' time)
    double ri[3], vi[3], rj[3], vj[3], r0[3], v0[3];
};

struct EventBuf {
    DevEvent* rec;
    unsigned int* count;  // may exceed cap: the host reports RG_ERR_EVENT_OVERFLOW
    unsigned int cap;
};

// Arguments of one force evaluation over a tile list.
struct GravArgs {
    const double* __restrict__ px;  // stage positions, rows of n
    const double* __restrict__ py;
    const double* __restrict__ pz;
    const double* __restrict__ vx;  // stage velocities (event records only)
    const double* __restrict__ vy;
    const double* __restrict__ vz;
    const double* __restrict__ mass;
    const double* __restrict__ radius;
    const int* __restrict__ id;
    const double* __restrict__ rho;  // |r_i - r_0| of the step-start state (Hill test)
    const float* __restrict__ rf;    // mixed mode: radii in FP32 (event screens), else nullptr
    const unsigned int* smax;        // mixed mode with screens: per system (4 words each), FP32 bits
                                     // of the largest radius, mass and |r - r_0| of its light bodies
                                     // (split_positions), else nullptr
    double* ax;  // output rows
    double* ay;
    double* az;
    const Tile* tiles;
    int n_tiles;
    double f_rad;      // THRESHOLD_RADII_ENHANCE_FACTOR
    double hill_f3;    // hill_factor^3
    float f_rad_f;     // the same in FP32 (the mixed kernels' event screens)
    float hill_f3_f;
    int record;        // record radius-criterion candidates
    int hill;          // record Hill candidates
    uint32_t seq;
    EventBuf ev;  // radius-criterion records
    EventBuf hv;  // Hill-sphere records
    // ensembles: tiles of systems whose flag is 0 are skipped; records are counted per system
    // and carry the system's attempt number (collisions) or step-start number (Hill)
    const int* sys_active;
    unsigned int* sys_events;
    const unsigned int* sys_attempt;
    const unsigned int* sys_f0;
    const double* sys_t;  // per system: the time at the attempt's start
    // astrocentric frame (single disks): per body the star's pull -mu / (r^2 |r|) r (rows 0-2,
    // a sink's starting value) and the indirect term m / (r^2 |r|) r (rows 3-5, subtracted
    // after each source's direct term), pp_disk.cu:413-420,447-454; nullptr: barycentric
    const double* astro;
    long long astro_stride;
    // ensembles: per system collision factor (THRESHOLD_RADII_ENHANCE_FACTOR); nullptr: f_rad
    const double* sys_f_rad;
    // the ensemble's mixed form keeps its stage vectors as double-float pairs (float2 per
    // element, hi + lo): acc_f2 -- the output rows are float2 rows; vel_f2 -- so are the
    // velocity rows (stages after the step start)
    int acc_f2;
    int vel_f2;
};

// the collision factor of a tile's system
__device__ __forceinline__ double tile_f_rad(const GravArgs& g, const Tile& t)
{
    return g.sys_f_rad ? g.sys_f_rad[t.sys] : g.f_rad;
}

// sequence tag of a record: (attempt << 8) | stage, or the step-start number for Hill
__device__ __forceinline__ uint32_t record_seq(const GravArgs& g, const Tile& t, int kind)
{
    if (kind == 1 && g.sys_f0) return g.sys_f0[t.sys];
    if (g.sys_attempt) return (g.sys_attempt[t.sys] << 8) | g.seq;
    return g.seq;
}

}  // namespace redgb

#define RG_CUDA_CHECK(expr)                                                   \
    do {                                                                      \
        cudaError_t _e = (expr);                                              \
        if (_e != cudaSuccess) return ::redgb::cuda_fail(_e, #expr, __FILE__, __LINE__); \
    } while (0)

namespace redgb {
int cuda_fail(cudaError_t e, const char* what, const char* file, int line);
// GB300's SM count, for launch-shape choices only (no correctness depends on it)
constexpr int NUM_SMS_HINT = 152;
}
