// ens_events.h -- the ensemble's event handling on the device (ens_events.cu): the raw
// records one attempt's force evaluations produce become the reference's event records,
// merges, ejections and hit-star merges are applied to the disks' state, and the loop
// condition of the graph that runs attempts back to back is set, all without the host.
#pragma once

#include <cuda_runtime.h>

#include "../../include/redgb_types.h"
#include "common.cuh"

namespace redgb {

// one record of an ensemble's event log: the disk, its record number (log order per disk)
// and the reference's 472-byte record
struct EnsLogRec {
    int32_t sys;
    int32_t seqno;
    int64_t pad;
    rg_event_t ev;
};

// error bits of EnsEventArgs::flags (the host turns them into status codes)
enum {
    ENS_FLAG_EVENT_OVERFLOW = 1u,   // more collision records in one attempt than the buffer holds
    ENS_FLAG_HILL_OVERFLOW = 2u,    // more Hill records in one step start than the buffer holds
    ENS_FLAG_LOG_OVERFLOW = 4u,     // the event log is full
    ENS_FLAG_HILL_SET = 8u,         // more pairs inside their Hill spheres than a disk's set holds
    ENS_FLAG_SUPERPLANETESIMAL = 16u,  // collision with a super-planetesimal (not implemented)
    ENS_FLAG_STEP_LOG_OVERFLOW = 32u,  // the attempt log is full
    ENS_FLAG_HIT_OVERFLOW = 64u        // more hit-star records in one check than a disk's list holds
};

struct EnsEventArgs {
    int n_sys;
    const int* base;   // per disk: its first body
    const int* ntot;   // per disk: bodies
    const int* nsi;    // per disk: self-interacting bodies
    long long stride;  // row stride of the state rows
    double* y;         // 6 rows: positions, velocities (internal units)
    double* mass;      // the kernels' mass and radius rows, kept equal to prm
    double* radius;
    rg_param_t* prm;   // authoritative body parameters
    int* id;
    const int* type;
    const double* thr;  // RG_THRESHOLD_N per disk
    int* status;
    int* active;
    int* active_f0;
    const double* t;       // per disk: clock after the attempt
    const double* t_prev;  // per disk: clock at the step's start
    const double* t_stop;
    const double* dt_did;
    const unsigned int* acc_attempt;  // per disk: the accepted attempt's number
    int* ej;
    const DevEvent* ev;  // collision records of this attempt
    const unsigned int* ev_count;
    unsigned int ev_cap;
    const DevEvent* hill;  // Hill records of this attempt's step-start evaluation
    const unsigned int* hill_count;
    long long* hill_set;  // per disk 2 x hill_set_cap pair keys (double buffer)
    int* hill_n;          // per disk: pairs in the current set
    int* hill_which;      // per disk: which half holds the current set
    int hill_set_cap;
    EnsLogRec* log;
    unsigned int* log_count;
    unsigned int log_cap;
    unsigned int* log_seq;  // per disk: records written
    unsigned int* flags;
    unsigned int* hit_slots;  // per disk hit_cap log slots of hit-star records awaiting their merge
    int hit_cap;
    double stage_c[13];  // RKF7(8) stage times c_r (int_rungekutta8.cu:29)
};

struct EnsLoopArgs {
    int n_sys;
    int* status;
    int* active;
    int* active_f0;
    unsigned int* flags;
    const unsigned int* kerr;  // set by a gravity kernel whose tile copy timed out
    const unsigned int* step_log_count;
    unsigned int step_log_cap;
    unsigned int* ev_count;
    unsigned int* hill_count;
    unsigned int ev_cap;  // capacity of both raw record buffers
    long long* attempts;   // [0] attempts run in this advance, [1] its limit (<= 0: none),
                           // [2] the end of this launch's chunk of attempts
    int* keep;             // 1 while another attempt is to run
    cudaGraphConditionalHandle cond;
    int use_cond;  // set the graph's loop condition (inside the graph only)
};

int launch_ens_hill(const EnsEventArgs& a, cudaStream_t st);
int launch_ens_handle(const EnsEventArgs& a, int initial, cudaStream_t st);
int launch_ens_loop(const EnsLoopArgs& a, cudaStream_t st);

}  // namespace redgb
