// context.cu -- host driver of one disk and the C ABI of include/redgb.h.
//
// The context owns the device state (structure-of-arrays rows, common.cuh) on its own
// stream and replays the reference's control flow around the kernels: the step-size
// controllers of rungekutta4/5/8::step (int_rungekutta4.cu:189-273,
// int_rungekutta5.cu:202-282, int_rungekutta8.cu:704-797), the event handling of pp_disk
// (pp_disk.cu:683-1202,1324-1409) and the time loop of main.cu:176-263.  Host-side floating
// point (merges, orbital elements, the controller's pow) is built with -ffp-contract=off so
// it rounds exactly like the reference's CPU path.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/redgb.h"
#include "abi_guard.h"
#include "common.cuh"
#include "host_tools.h"
#include "kernels.h"
#include "plan_tools.h"
#include "rk_tables.h"

namespace redgb {

static thread_local std::string g_last_error;

int set_error(int code, const std::string& msg)
{
    g_last_error = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char* what, const char* file, int line)
{
    char buf[512];
    snprintf(buf, sizeof(buf), "%s: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
    g_last_error = buf;
    return RG_ERR_CUDA;
}

const char* last_error() { return g_last_error.c_str(); }

}  // namespace redgb

using namespace redgb;

// ============================================================================ context
struct rg_ctx {
    int cnt[7] = {};         // n_s, n_gp, n_rp, n_pp, n_spl, n_pl, n_tp
    int n_inactive[7] = {};  // number_of_bodies::n_i_*
    int cap = 0;             // row stride of every device buffer
    int device = 0;
    // device
    cudaStream_t st = nullptr;
    // the double-float rows (star, giants) run on st2 beside the mixed kernel on st
    cudaStream_t st2 = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    double* d_y = nullptr;     // 6 rows: r, v
    double* d_yout = nullptr;  // 6 rows
    double* d_k[13] = {};      // 6 rows each: dr/dt (stage velocities), dv/dt
    double* d_P = nullptr;     // 3 rows: stage positions
    double* d_mass = nullptr;
    double* d_radius = nullptr;
    int* d_id = nullptr;
    int* d_type = nullptr;
    double* d_rho = nullptr;
    Tile* d_tiles = nullptr;
    int* d_heavy = nullptr;  // per mixed tile: end of its heavy sources
    int tiles_cap = 0;
    void* d_split = nullptr;  // FP32 (hi, lo) positions of the mixed kernel
    float* d_rf = nullptr;    // FP32 radii of the mixed kernels' event screens
    unsigned int* d_smax = nullptr;  // the screens' maxima (split_positions)
    int* d_screen_slot = nullptr;    // per body: 0 for a light body, -1 for a heavy one
    DevEvent* d_ev = nullptr;
    DevEvent* d_hill = nullptr;
    // one allocation, read back by one copy per step: [0] events, [1] Hill events, [2] set by
    // a gravity kernel whose tile copy timed out
    unsigned int* d_counters = nullptr;
    unsigned int* d_ev_count = nullptr;    // d_counters + 0
    unsigned int* d_hill_count = nullptr;  // d_counters + 1
    unsigned int* d_kerr = nullptr;        // d_counters + 2
    unsigned int* d_sym_ticket = nullptr;  // d_counters + 3: the symmetric kernel's last-segment ticket
    std::vector<int> sym_cta;              // the symmetric kernel's CTAs: first segments (+ end)
    int* d_sym_cta = nullptr;
    int sym_cta_cap = 0;
    unsigned int ev_cap = 0;
    EjectRec* d_ej = nullptr;
    unsigned int* d_ej_count = nullptr;
    unsigned long long* d_maxbits = nullptr;
    double* d_dt = nullptr;
    double* d_part = nullptr;
    double* d_records = nullptr;  // r and v as vec_t records (state in / out): 8 doubles per body
    double* d_astro = nullptr;    // astrocentric frame: per body the star's pull and indirect term (6 rows)
    int frame = RG_FRAME_BARY;    // pp_disk::frame_center
    double* h_pin = nullptr;  // pinned: [0] dt, [1] max bits, [2..3] counts, [4..5] d_counters
    // host mirrors of the body parameters (authoritative; the state lives on the device)
    std::vector<rg_param_t> p;
    std::vector<rg_body_metadata_t> md;
    std::vector<double> epoch;
    double t = 0.0;
    double thr[RG_THRESHOLD_N] = {};
    int close_encounter = 0, inner_steps = 1, event_time_mode = RG_EVENT_TIME_CPU;
    double hill_factor = 0.0;
    int gravity_mode = RG_GRAVITY_FP64;
    int pairpar_S = 16;
    int rowseq_max_src = 64;
    int mixed_chunk_src = 0;  // sources per grid.y chunk of the mixed kernel, a multiple of
                              // MIXED_SOURCE_TILE (0: from the SM count)
    float near_ratio = 1.0e-5f;
    int hold_tile_copies = 0;  // test hook (rg_test_hold_tile_copies)
    // integrator
    int has_int = 0, int_type = 0, adaptive = 0, ectp = 0, r_max = 0, order = 0;
    double dt_try = 0.0, dt_did = 0.0, tol = 0.0;
    int64_t n_failed = 0, n_passed = 0, n_tried = 0;
    std::vector<double> attempt_dt;
    double t_step = 0.0;  // clock at the start of the step whose events are collected
    // events
    std::vector<rg_event_t> events;  // pp_disk::events of the current step
    int overflow = 0;
    std::vector<rg_event_t> hill;
    std::vector<int64_t> hill_pairs;
    std::vector<rg_event_t> log;
    int64_t n_hit_centrum[3] = {}, n_ejection[3] = {}, n_collision[3] = {}, n_close_encounter[3] = {},
            n_event[3] = {};
    int64_t n_gravity_evals = 0, n_pairs = 0, n_kernels = 0;
    // profiling: event pairs around force evaluations (kind 0) and stage kernels (kind 1)
    int profiling = 0;
    std::vector<cudaEvent_t> ev_pool;
    std::vector<int> ev_kind;  // per recorded pair
    size_t ev_used = 0;
    // tiles for the current body counts
    // launch plan of one force evaluation, per gravity mode (build_plan)
    struct Group {
        int kind;       // GROUP_*
        size_t off;     // first tile in d_tiles
        int n;          // tiles
        int row_base;   // few-sink groups: first row in the terms buffer
        int rows;       // few-sink groups: rows
        int max_src;    // few-sink groups: largest source count of a tile
        int max_sinks;  // few-sink groups: widest tile
    };
    std::vector<Group> plan[2];
    std::vector<Tile> tiles;       // all groups' tiles, uploaded to d_tiles
    std::vector<int> heavy_mx;     // per tile (mixed groups): end of the heavy sources
    std::vector<int> screen_slot;  // per body: 0 light, -1 heavy (the mixed kernels' screen cutoffs)
    std::vector<int> few_row0, few_nsrc;  // per tile (few-sink groups)
    std::vector<int> row_sink, row_nsrc;  // per terms-buffer row
    std::vector<int> row_nparts;          // per terms-buffer row: parts of a symmetric heavy row (else 0)
    int few_rows = 0;
    long long few_pitch = 0;
    double* d_terms = nullptr;
    size_t terms_cap = 0;
    double* d_partial = nullptr;  // mixed kernel: per source chunk partial sums
    size_t partial_cap = 0;
    int n_sm = 152;
    int* d_row_sink = nullptr;
    int* d_row_nsrc = nullptr;
    int* d_row_nparts = nullptr;
    int rows_cap = 0;
    int* d_few_row0 = nullptr;  // per tile
    int64_t pairs_per_eval = 0;
    bool tiles_dirty = true;
    int64_t tiles_version = 0;  // bumped by every upload of the tile plan
    // CUDA graphs of the RKF7(8) step: the step-start evaluation and one attempt, each kept
    // for both parities of the y / y_out swap, rebuilt when anything they freeze changes
    struct StepGraph {
        cudaGraphExec_t exec = nullptr;
        std::vector<double> sig;  // the frozen launch parameters (graph_signature)
        int64_t kernels = 0, evals = 0, pairs = 0;  // host counters one replay advances
    };
    StepGraph g_stage0[2], g_attempt[2];
    bool capturing = false;     // launches are being captured (no allocation may happen)
    bool capture_failed = false;
    unsigned int* d_attempt_no = nullptr;  // the attempt's number for the event records (graphs)
    int use_graphs = 1;

    int n_si() const { return cnt[0] + cnt[1] + cnt[2] + cnt[3]; }
    int n_nsi() const { return cnt[4] + cnt[5]; }
    int n_ni() const { return cnt[6]; }
    int n_massive() const { return n_si() + n_nsi(); }
    int n_total() const { return n_massive() + n_ni(); }
    double* row(double* base, int r) const { return base + (size_t)r * cap; }
};

namespace {

constexpr double GAUSS = 1.720209895e-2;  // red_constants.h:21
constexpr double GAUSS2 = 2.959122082855911025e-4;

template <class T>
int dalloc(T** p, size_t count)
{
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
    if (e != cudaSuccess) {
        *p = nullptr;
        return set_error(RG_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    return RG_OK;
}

void free_all(rg_ctx* c)
{
    cudaFree(c->d_y);
    cudaFree(c->d_yout);
    for (auto& k : c->d_k) cudaFree(k);
    cudaFree(c->d_P);
    cudaFree(c->d_mass);
    cudaFree(c->d_radius);
    cudaFree(c->d_id);
    cudaFree(c->d_type);
    cudaFree(c->d_rho);
    cudaFree(c->d_tiles);
    cudaFree(c->d_heavy);
    cudaFree(c->d_split);
    cudaFree(c->d_rf);
    cudaFree(c->d_smax);
    cudaFree(c->d_screen_slot);
    cudaFree(c->d_terms);
    cudaFree(c->d_partial);
    cudaFree(c->d_row_sink);
    cudaFree(c->d_row_nsrc);
    cudaFree(c->d_row_nparts);
    cudaFree(c->d_sym_cta);
    cudaFree(c->d_few_row0);
    cudaFree(c->d_ev);
    cudaFree(c->d_hill);
    cudaFree(c->d_astro);
    cudaFree(c->d_attempt_no);
    for (int p = 0; p < 2; p++) {
        if (c->g_stage0[p].exec) cudaGraphExecDestroy(c->g_stage0[p].exec);
        if (c->g_attempt[p].exec) cudaGraphExecDestroy(c->g_attempt[p].exec);
    }
    cudaFree(c->d_counters);
    cudaFree(c->d_ej);
    cudaFree(c->d_ej_count);
    cudaFree(c->d_maxbits);
    cudaFree(c->d_dt);
    cudaFree(c->d_part);
    cudaFree(c->d_records);
    if (c->h_pin) cudaFreeHost(c->h_pin);
    for (auto e : c->ev_pool) cudaEventDestroy(e);
    if (c->st2) cudaStreamDestroy(c->st2);
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    if (c->st) cudaStreamDestroy(c->st);
}

// --------------------------------------------------------------------- profiling
constexpr size_t MAX_PROFILE_PAIRS = 1 << 16;

// records the opening event of a timed launch; returns the pair index or -1
long prof_begin(rg_ctx* c, int kind)
{
    if (!c->profiling || c->ev_used / 2 >= MAX_PROFILE_PAIRS) return -1;
    while (c->ev_pool.size() < c->ev_used + 2) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) return -1;
        c->ev_pool.push_back(e);
    }
    cudaEventRecord(c->ev_pool[c->ev_used], c->st);
    c->ev_kind.push_back(kind);
    const long idx = (long)c->ev_used;
    c->ev_used += 2;
    return idx;
}

void prof_end(rg_ctx* c, long idx)
{
    if (idx >= 0) cudaEventRecord(c->ev_pool[(size_t)idx + 1], c->st);
}

// --------------------------------------------------------------------- uploads / downloads
int upload_params(rg_ctx* c)
{
    const int n = c->n_total();
    std::vector<double> m(n), R(n);
    std::vector<int> id(n), ty(n);
    for (int i = 0; i < n; i++) {
        m[i] = c->p[i].mass;
        R[i] = c->p[i].radius;
        id[i] = c->md[i].id;
        ty[i] = c->md[i].body_type;
    }
    if (n > 0) {
        RG_CUDA_CHECK(cudaMemcpyAsync(c->d_mass, m.data(), n * sizeof(double), cudaMemcpyHostToDevice, c->st));
        RG_CUDA_CHECK(cudaMemcpyAsync(c->d_radius, R.data(), n * sizeof(double), cudaMemcpyHostToDevice, c->st));
        RG_CUDA_CHECK(cudaMemcpyAsync(c->d_id, id.data(), n * sizeof(int), cudaMemcpyHostToDevice, c->st));
        RG_CUDA_CHECK(cudaMemcpyAsync(c->d_type, ty.data(), n * sizeof(int), cudaMemcpyHostToDevice, c->st));
    }
    RG_CUDA_CHECK(cudaStreamSynchronize(c->st));
    return RG_OK;
}

// the 6 state rows (internal units) of the first n_total bodies
int download_state(rg_ctx* c, std::vector<double>& h)
{
    const int n = c->n_total();
    h.resize((size_t)6 * n);
    if (n > 0)
        RG_CUDA_CHECK(cudaMemcpy2DAsync(h.data(), n * sizeof(double), c->d_y, c->cap * sizeof(double),
                                        n * sizeof(double), 6, cudaMemcpyDeviceToHost, c->st));
    RG_CUDA_CHECK(cudaStreamSynchronize(c->st));
    return RG_OK;
}

int upload_state(rg_ctx* c, const std::vector<double>& h)
{
    const int n = c->n_total();
    if (n > 0)
        RG_CUDA_CHECK(cudaMemcpy2DAsync(c->d_y, c->cap * sizeof(double), h.data(), n * sizeof(double),
                                        n * sizeof(double), 6, cudaMemcpyHostToDevice, c->st));
    RG_CUDA_CHECK(cudaStreamSynchronize(c->st));
    return RG_OK;
}

int get_body(rg_ctx* c, int i, rg_vec_t* r, rg_vec_t* v)
{
    double h[6];
    RG_CUDA_CHECK(cudaMemcpy2DAsync(h, sizeof(double), c->d_y + i, c->cap * sizeof(double), sizeof(double), 6,
                                    cudaMemcpyDeviceToHost, c->st));
    RG_CUDA_CHECK(cudaStreamSynchronize(c->st));
    *r = rg_vec_t{h[0], h[1], h[2], 0.0};
    *v = rg_vec_t{h[3], h[4], h[5], 0.0};
    return RG_OK;
}

int set_body(rg_ctx* c, int i, const rg_vec_t& r, const rg_vec_t& v)
{
    const double h[6] = {r.x, r.y, r.z, v.x, v.y, v.z};
    RG_CUDA_CHECK(cudaMemcpy2DAsync(c->d_y + i, c->cap * sizeof(double), h, sizeof(double), sizeof(double), 6,
                                    cudaMemcpyHostToDevice, c->st));
    RG_CUDA_CHECK(cudaStreamSynchronize(c->st));
    return RG_OK;
}

int set_param_dev(rg_ctx* c, int i)
{
    RG_CUDA_CHECK(cudaMemcpyAsync(c->d_mass + i, &c->p[i].mass, sizeof(double), cudaMemcpyHostToDevice, c->st));
    RG_CUDA_CHECK(cudaMemcpyAsync(c->d_radius + i, &c->p[i].radius, sizeof(double), cudaMemcpyHostToDevice, c->st));
    RG_CUDA_CHECK(cudaMemcpyAsync(c->d_id + i, &c->md[i].id, sizeof(int), cudaMemcpyHostToDevice, c->st));
    RG_CUDA_CHECK(cudaStreamSynchronize(c->st));
    return RG_OK;
}

// --------------------------------------------------------------------- launch plan
enum {
    GROUP_PAIRPAR = 0,
    GROUP_ROWSEQ = 1,
    GROUP_FEW_SERIAL = 2,
    GROUP_MIXED = 3,
    GROUP_DF_ROWSEQ = 4,  // mixed mode: the row kernel in double-float arithmetic
    GROUP_DF_FEW = 5,     // mixed mode: few heavy sinks in double-float arithmetic
    GROUP_DF_SYM = 6,     // mixed mode: heavy-light pairs once for both rows (grav_df_sym)
};
// light bodies per symmetric tile of one disk, about: one per thread of a 256-thread CTA up to
// a wave of resident CTAs, so that a disk of a thousand bodies spreads over several SMs (the
// evaluation's latency is one tile's)
constexpr int FEW_BLOCK_SINKS = 32;  // blocks with at most this many sinks use the few-sink path

// CTA tiles of the interaction matrix (number_of_bodies::get_bound_SI/NSI/NI,
// number_of_bodies.cpp:196-258, barycentric frame) for both gravity modes.
void build_tiles(rg_ctx* c)
{
    c->tiles.clear();
    c->heavy_mx.clear();
    c->few_row0.clear();
    c->few_nsrc.clear();
    c->row_sink.clear();
    c->row_nsrc.clear();
    c->row_nparts.clear();
    c->few_rows = 0;
    c->few_pitch = 0;
    const int nsi = c->n_si(), nm = c->n_massive(), nt = c->n_total();
    // heavy bodies of the mixed kernel: the leading stars, giant and rocky planets.  As
    // sources of the mixed kernel their terms are exact FP64; as sinks (few rows), and as
    // the sources of row-kernel blocks, they use the double-float kernels.
    const int n_heavy = std::min(nsi, c->cnt[0] + c->cnt[1] + c->cnt[2]);
    struct Blk {
        int s0, s1, src1, block;
    } blks[3] = {{0, nsi, nm, 0}, {nsi, nm, nsi, 1}, {nm, nt, nm, 2}};
    c->pairs_per_eval = (int64_t)nsi * (nm > 0 ? nm - 1 : 0) + (int64_t)(nm - nsi) * nsi + (int64_t)(nt - nm) * nm;
    // the astrocentric frame starts the SI block's sinks and sources at body 1
    // (number_of_bodies.cpp:205-222); only self-interacting systems take it
    const int src0 = c->frame == RG_FRAME_ASTRO ? 1 : 0;
    if (src0) {
        blks[0].s0 = 1;
        c->pairs_per_eval = nsi > 1 ? (int64_t)(nsi - 1) * (nm - 2) : 0;
    }

    // mixed plan: with a few heavy SI bodies (a few-sink block over every massive body) and an
    // NSI block on the row kernel over them, the pairs between the blocks are evaluated once
    // for both rows (grav_df_sym, the heavy-heavy pairs with them): the light bodies in
    // balanced tiles, each one part of the heavy rows
    const bool sym = !src0 && nsi >= 1 && nsi <= DF_SYM_MAX_HEAVY && nm > nsi && nsi <= c->rowseq_max_src &&
                     nm > c->rowseq_max_src && nsi <= FEW_BLOCK_SINKS;
    const int sym_ctas = sym ? std::min((nm - nsi + DF_SYM_PASS - 1) / DF_SYM_PASS, DF_SYM_RESIDENT * c->n_sm) : 0;
    c->sym_cta.clear();
    auto add_group = [&](int mode, int kind, int s0, int s1, int src1, int block, int step) {
        if (s1 <= s0) return;
        rg_ctx::Group gr{kind, c->tiles.size(), 0, c->few_rows, 0, src1, std::min(step, s1 - s0)};
        for (int s = s0; s < s1; s += step) {
            c->tiles.push_back(Tile{s, std::min(s + step, s1), block == 0 ? src0 : 0, src1, 0, 0, block, 0});
            c->heavy_mx.push_back(kind == GROUP_MIXED ? std::min(n_heavy, src1) : 0);
            if (kind == GROUP_FEW_SERIAL || kind == GROUP_DF_FEW) {
                c->few_row0.push_back(c->few_rows);
                c->few_nsrc.push_back(src1);
                for (int i = s; i < std::min(s + step, s1); i++) {
                    c->row_sink.push_back(i);
                    c->row_nsrc.push_back(src1);
                    c->row_nparts.push_back(0);
                    c->few_rows++;
                    gr.rows++;
                }
                c->few_pitch = std::max<long long>(c->few_pitch, src1);
            } else {
                c->few_row0.push_back(0);
                c->few_nsrc.push_back(0);
            }
            gr.n++;
        }
        c->plan[mode].push_back(gr);
    };
    c->plan[0].clear();
    c->plan[1].clear();
    for (const auto& b : blks) {
        if (b.s1 <= b.s0) continue;
        const int ns = b.s1 - b.s0;
        if (src0) {  // the astrocentric terms are in the pair-parallel kernel only
            add_group(0, GROUP_PAIRPAR, b.s0, b.s1, b.src1, b.block, c->pairpar_S);
            continue;
        }
        if (b.src1 <= c->rowseq_max_src) {  // few sources: thread per sink (same tiles in both modes)
            // tiles of up to 128 sinks; narrower ones when that leaves SMs idle (a thread's few
            // serial pair terms are latency-bound, so more SMs beat fuller CTAs)
            const int rs_step = ns >= 2 * 128 * c->n_sm ? 128 : (ns >= 2 * 64 * c->n_sm ? 64 : 32);
            add_group(0, GROUP_ROWSEQ, b.s0, b.s1, b.src1, b.block, rs_step);
            if (sym && b.block == 1) {  // the heavy rows [0, nsi), then one segment per CTA (Tile::part from 1)
                const size_t t0 = c->tiles.size();
                std::vector<int> parts;
                build_sym_segments({Tile{b.s0, b.s1, 0, nsi, 0, 0, b.block, 0}}, sym_ctas, DF_SYM_PASS,
                                   DF_SYM_SEGMENT_COST, c->tiles, c->sym_cta, parts);
                const int nseg = (int)(c->tiles.size() - t0);
                rg_ctx::Group gr{GROUP_DF_SYM, t0, nseg, c->few_rows, nsi, nsi, 0};
                const int row0 = c->few_rows;
                for (int h = 0; h < nsi; h++) {
                    c->row_sink.push_back(h);
                    c->row_nsrc.push_back(nm);
                    c->row_nparts.push_back(parts[0]);
                    c->few_rows++;
                }
                c->few_pitch = std::max<long long>(c->few_pitch, parts[0]);
                for (int k = 0; k < nseg; k++) {
                    c->heavy_mx.push_back(0);
                    c->few_row0.push_back(row0);
                    c->few_nsrc.push_back(0);
                }
                c->plan[1].push_back(gr);
            } else {
                c->plan[1].push_back(c->plan[0].back());
                c->plan[1].back().kind = GROUP_DF_ROWSEQ;
            }
            continue;
        }
        if (ns <= FEW_BLOCK_SINKS) {  // few sinks, many sources: exact serial row sums (same rows)
            add_group(0, GROUP_FEW_SERIAL, b.s0, b.s1, b.src1, b.block, FEW_SINKS_MAX);
            if (!(sym && b.block == 0)) {  // a symmetric plan's heavy rows come with its tiles
                c->plan[1].push_back(c->plan[0].back());
                c->plan[1].back().kind = GROUP_DF_FEW;
            }
            continue;
        }
        add_group(0, GROUP_PAIRPAR, b.s0, b.s1, b.src1, b.block, c->pairpar_S);
        const int light0 = b.block == 0 ? std::max(b.s0, std::min(n_heavy, b.s1)) : b.s0;
        add_group(1, GROUP_DF_FEW, b.s0, light0, b.src1, b.block, FEW_SINKS_MAX);
        add_group(1, GROUP_MIXED, light0, b.s1, b.src1, b.block, MIXED_SINKS_PER_TILE);
    }
    c->screen_slot.assign(nt, 0);
    for (int i = 0; i < n_heavy; i++) c->screen_slot[i] = -1;
    c->tiles_dirty = true;
}

int sync_tiles(rg_ctx* c)
{
    if (!c->tiles_dirty) return RG_OK;
    const int n = (int)c->tiles.size();
    if (n > c->tiles_cap) {
        cudaFree(c->d_tiles);
        cudaFree(c->d_heavy);
        cudaFree(c->d_few_row0);
        c->d_tiles = nullptr;
        c->d_heavy = nullptr;
        c->d_few_row0 = nullptr;
        int rc = dalloc(&c->d_tiles, (size_t)n);
        if (!rc) rc = dalloc(&c->d_heavy, (size_t)n);
        if (!rc) rc = dalloc(&c->d_few_row0, (size_t)n);
        if (rc) return rc;
        c->tiles_cap = n;
    }
    const size_t need = (size_t)3 * c->few_rows * (size_t)c->few_pitch;
    if (need > c->terms_cap) {
        cudaFree(c->d_terms);
        c->d_terms = nullptr;
        int rc = dalloc(&c->d_terms, need);
        if (rc) return rc;
        c->terms_cap = need;
    }
    if (c->few_rows > c->rows_cap) {
        cudaFree(c->d_row_sink);
        cudaFree(c->d_row_nsrc);
        cudaFree(c->d_row_nparts);
        c->d_row_sink = c->d_row_nsrc = c->d_row_nparts = nullptr;
        int rc = dalloc(&c->d_row_sink, (size_t)c->few_rows);
        if (!rc) rc = dalloc(&c->d_row_nsrc, (size_t)c->few_rows);
        if (!rc) rc = dalloc(&c->d_row_nparts, (size_t)c->few_rows);
        if (rc) return rc;
        c->rows_cap = c->few_rows;
    }
    if ((int)c->sym_cta.size() > c->sym_cta_cap) {
        cudaFree(c->d_sym_cta);
        c->d_sym_cta = nullptr;
        int rc = dalloc(&c->d_sym_cta, c->sym_cta.size());
        if (rc) return rc;
        c->sym_cta_cap = (int)c->sym_cta.size();
    }
    if (!c->sym_cta.empty())
        RG_CUDA_CHECK(cudaMemcpyAsync(c->d_sym_cta, c->sym_cta.data(), c->sym_cta.size() * sizeof(int),
                                      cudaMemcpyHostToDevice, c->st));
    if (n > 0) {
        RG_CUDA_CHECK(cudaMemcpyAsync(c->d_tiles, c->tiles.data(), n * sizeof(Tile), cudaMemcpyHostToDevice, c->st));
        RG_CUDA_CHECK(cudaMemcpyAsync(c->d_heavy, c->heavy_mx.data(), n * sizeof(int), cudaMemcpyHostToDevice, c->st));
        RG_CUDA_CHECK(cudaMemcpyAsync(c->d_few_row0, c->few_row0.data(), n * sizeof(int), cudaMemcpyHostToDevice, c->st));
    }
    if (!c->screen_slot.empty())
        RG_CUDA_CHECK(cudaMemcpyAsync(c->d_screen_slot, c->screen_slot.data(), c->screen_slot.size() * sizeof(int),
                                      cudaMemcpyHostToDevice, c->st));
    if (c->few_rows > 0) {
        RG_CUDA_CHECK(cudaMemcpyAsync(c->d_row_sink, c->row_sink.data(), c->few_rows * sizeof(int),
                                      cudaMemcpyHostToDevice, c->st));
        RG_CUDA_CHECK(cudaMemcpyAsync(c->d_row_nsrc, c->row_nsrc.data(), c->few_rows * sizeof(int),
                                      cudaMemcpyHostToDevice, c->st));
        RG_CUDA_CHECK(cudaMemcpyAsync(c->d_row_nparts, c->row_nparts.data(), c->few_rows * sizeof(int),
                                      cudaMemcpyHostToDevice, c->st));
    }
    RG_CUDA_CHECK(cudaStreamSynchronize(c->st));
    c->tiles_dirty = false;
    c->tiles_version++;
    return RG_OK;
}

double mass_of_star(const rg_ctx* c);

// --------------------------------------------------------------------- one force evaluation
// pp_disk::calc_dydx(1, ...) (pp_disk.cu:998-1041): accelerations of the stage positions
// `pos` (3 rows) into `acc` (3 rows); `vel` (3 rows) are the stage velocities, read only
// into event records.
int gravity(rg_ctx* c, const double* pos, const double* vel, double* acc, int stage, int attempt, bool record,
            bool hill)
{
    int rc = sync_tiles(c);
    if (rc) return rc;
    const size_t cap = (size_t)c->cap;
    GravArgs g{};
    g.px = pos;
    g.py = pos + cap;
    g.pz = pos + 2 * cap;
    g.vx = vel;
    g.vy = vel + cap;
    g.vz = vel + 2 * cap;
    g.mass = c->d_mass;
    g.radius = c->d_radius;
    g.id = c->d_id;
    g.rho = c->d_rho;
    g.rf = c->gravity_mode == RG_GRAVITY_MIXED ? c->d_rf : nullptr;
    g.ax = acc;
    g.ay = acc + cap;
    g.az = acc + 2 * cap;
    g.f_rad = c->thr[RG_THRESHOLD_RADII_ENHANCE_FACTOR];
    g.hill_f3 = c->hill_factor * c->hill_factor * c->hill_factor;
    g.f_rad_f = (float)g.f_rad;
    g.hill_f3_f = (float)g.hill_f3;
    g.record = (record && c->inner_steps && g.f_rad > 0.0) ? 1 : 0;
    g.hill = hill ? 1 : 0;
    g.seq = ((uint32_t)attempt << 8) | (uint32_t)stage;
    if (c->capturing && stage > 0) {  // a replayed attempt reads its number from the device
        g.seq = (uint32_t)stage;
        g.sys_attempt = c->d_attempt_no;
    }
    g.ev = EventBuf{c->d_ev, c->d_ev_count, c->ev_cap};
    g.hv = EventBuf{c->d_hill, c->d_hill_count, c->ev_cap};
    if (hill) {
        rc = launch_star_distance(g.px, g.py, g.pz, nullptr, c->n_total(), c->d_rho, c->st);
        if (rc) return rc;
        c->n_kernels++;
    }
    // the screens' maxima serve the mixed kernel's per-sink cutoffs (light sinks x light sources)
    bool mixed_tiles = false;
    for (const auto& gr : c->plan[1]) mixed_tiles = mixed_tiles || gr.kind == GROUP_MIXED;
    if (c->gravity_mode == RG_GRAVITY_MIXED && (g.record || g.hill) && mixed_tiles) {
        RG_CUDA_CHECK(cudaMemsetAsync(c->d_smax, 0, SCREEN_MAX_WORDS * sizeof(unsigned int), c->st));
        g.smax = c->d_smax;
    }
    c->n_gravity_evals++;
    c->n_pairs += c->pairs_per_eval;
    const long prof = prof_begin(c, 0);
    if (c->frame == RG_FRAME_ASTRO) {
        rc = launch_astro_terms(g.px, g.py, g.pz, c->d_mass, c->n_massive(), mass_of_star(c), c->d_astro,
                                (long long)cap, c->st);
        if (rc) return rc;
        c->n_kernels++;
        g.astro = c->d_astro;
        g.astro_stride = (long long)cap;
    }
    bool split_done = false;
    // with a mixed group, the double-float row groups (a few sinks: star, giants) run on a
    // side stream beside it: they write other rows and append events atomically
    bool fork = false;
    if (c->gravity_mode == RG_GRAVITY_MIXED && mixed_tiles)
        for (const auto& gr : c->plan[1])
            fork = fork || gr.kind == GROUP_DF_ROWSEQ || gr.kind == GROUP_DF_FEW || gr.kind == GROUP_DF_SYM;
    if (fork) {
        rc = launch_split_positions(g.px, g.py, g.pz, c->d_mass, c->d_id, nullptr, c->d_screen_slot, c->d_radius,
                                    c->n_total(), (SplitPos*)c->d_split, c->d_rf, g.smax ? c->d_smax : nullptr,
                                    g.hill != 0, c->st);
        if (rc) return rc;
        split_done = true;
        c->n_kernels++;
        RG_CUDA_CHECK(cudaEventRecord(c->ev_fork, c->st));
        RG_CUDA_CHECK(cudaStreamWaitEvent(c->st2, c->ev_fork, 0));
    }
    const cudaStream_t row_st = fork ? c->st2 : c->st;
    // FP64: the few-sink rows (star, giants: their terms, then a long serial sum per row, whose
    // dependent FP64 additions set the evaluation's latency) on the side stream, beside the other
    // groups; they write other rows and append events atomically (collect_events sorts them)
    bool fork_few = false;
    if (c->gravity_mode == RG_GRAVITY_FP64) {
        bool few = false, other = false;
        for (const auto& gr : c->plan[0]) (gr.kind == GROUP_FEW_SERIAL ? few : other) = true;
        fork_few = few && other;
    }
    if (fork_few) {
        RG_CUDA_CHECK(cudaEventRecord(c->ev_fork, c->st));
        RG_CUDA_CHECK(cudaStreamWaitEvent(c->st2, c->ev_fork, 0));
    }
    for (const auto& gr : c->plan[c->gravity_mode == RG_GRAVITY_MIXED ? 1 : 0]) {
        g.tiles = c->d_tiles + gr.off;
        g.n_tiles = gr.n;
        switch (gr.kind) {
        case GROUP_PAIRPAR:
            rc = launch_grav_fp64_pairpar(g, c->pairpar_S, c->st);
            c->n_kernels++;
            break;
        case GROUP_ROWSEQ:
            rc = launch_grav_fp64_rowseq(g, c->st);
            c->n_kernels++;
            break;
        case GROUP_FEW_SERIAL:
            rc = launch_grav_fp64_few(g, c->d_few_row0 + gr.off, gr.max_src, c->d_terms, c->few_rows, c->few_pitch,
                                      c->d_row_sink, c->d_row_nsrc, nullptr, gr.row_base, gr.rows,
                                      fork_few ? c->st2 : c->st);
            c->n_kernels += 2;
            break;
        case GROUP_DF_ROWSEQ:
        case GROUP_DF_FEW:
            if (!split_done) {
                rc = launch_split_positions(g.px, g.py, g.pz, c->d_mass, c->d_id, nullptr, c->d_screen_slot,
                                            c->d_radius, c->n_total(), (SplitPos*)c->d_split, c->d_rf,
                                            g.smax ? c->d_smax : nullptr, g.hill != 0, c->st);
                split_done = true;
                c->n_kernels++;
            }
            if (rc) break;
            if (gr.kind == GROUP_DF_ROWSEQ) {
                rc = launch_grav_df_rowseq(g, c->d_split, row_st);
                c->n_kernels++;
            } else {
                rc = launch_grav_df_few(g, c->d_split, c->d_few_row0 + gr.off, gr.max_src, gr.max_sinks, 0, c->d_terms,
                                        c->few_rows,
                                        c->few_pitch, c->d_row_sink, c->d_row_nsrc, nullptr, gr.row_base, gr.rows,
                                        row_st);
                c->n_kernels += 2;
            }
            break;
        case GROUP_DF_SYM:
            if (!split_done) {
                rc = launch_split_positions(g.px, g.py, g.pz, c->d_mass, c->d_id, nullptr, c->d_screen_slot,
                                            c->d_radius, c->n_total(), (SplitPos*)c->d_split, c->d_rf,
                                            g.smax ? c->d_smax : nullptr, g.hill != 0, c->st);
                split_done = true;
                c->n_kernels++;
            }
            if (!rc)
                rc = launch_grav_df_sym(g, c->d_sym_cta, (int)c->sym_cta.size() - 1, c->d_split,
                                        c->d_few_row0 + gr.off, gr.max_src, c->d_terms, c->few_rows, c->few_pitch,
                                        c->d_row_sink, c->d_row_nparts, c->d_sym_ticket, row_st);
            c->n_kernels++;
            break;
        case GROUP_MIXED:
            if (!split_done) {
                rc = launch_split_positions(g.px, g.py, g.pz, c->d_mass, c->d_id, nullptr, c->d_screen_slot,
                                            c->d_radius, c->n_total(), (SplitPos*)c->d_split, c->d_rf,
                                            g.smax ? c->d_smax : nullptr, g.hill != 0, c->st);
                split_done = true;
                c->n_kernels++;
            }
            if (!rc) {
                // split the sources over grid.y so that about 4 CTAs per SM are in flight
                const int src = c->tiles[gr.off].src_end - c->tiles[gr.off].src_begin;
                const int src_tiles = (src + MIXED_SOURCE_TILE - 1) / MIXED_SOURCE_TILE;
                int chunk;
                if (c->mixed_chunk_src > 0) {
                    chunk = std::min(c->mixed_chunk_src, src_tiles * MIXED_SOURCE_TILE);
                } else {
                    const int n = std::max(1, std::min((4 * c->n_sm + gr.n - 1) / gr.n, src / (4 * MIXED_SOURCE_TILE)));
                    chunk = (src_tiles + n - 1) / n * MIXED_SOURCE_TILE;
                }
                const int chunks = (src + chunk - 1) / chunk;
                if (chunks > 1 && (size_t)chunks * 3 * c->cap > c->partial_cap && c->capturing) {
                    c->capture_failed = true;  // allocate outside a capture (the next direct run)
                    rc = RG_ERR_STATE;
                } else if (chunks > 1 && (size_t)chunks * 3 * c->cap > c->partial_cap) {
                    cudaFree(c->d_partial);
                    c->d_partial = nullptr;
                    c->partial_cap = 0;
                    rc = dalloc(&c->d_partial, (size_t)chunks * 3 * c->cap);
                    if (!rc) c->partial_cap = (size_t)chunks * 3 * c->cap;
                }
                if (!rc)
                    rc = launch_grav_mixed_tiles(g, c->d_split, c->d_heavy + gr.off, c->near_ratio, chunks, chunk,
                                                 c->d_partial, c->cap, c->d_kerr, c->hold_tile_copies != 0, c->st);
                c->n_kernels += chunks > 1;
            }
            c->n_kernels++;
            break;
        }
        if (rc) break;
    }
    if (fork || fork_few) {  // joined on every path, so that no row kernel outlives the call's stream order
        RG_CUDA_CHECK(cudaEventRecord(c->ev_join, c->st2));
        RG_CUDA_CHECK(cudaStreamWaitEvent(c->st, c->ev_join, 0));
    }
    if (rc) return rc;
    prof_end(c, prof);
    return rc;
}

// --------------------------------------------------------------------- events
rg_event_t zero_event()
{
    rg_event_t e;
    std::memset(&e, 0, sizeof(e));
    return e;
}

double mass_of_star(const rg_ctx* c)  // pp_disk::get_mass_of_star (pp_disk.cu:1483-1496)
{
    const int n = c->n_massive();
    for (int j = 0; j < n; j++)
        if (c->md[j].body_type == RG_BODY_STAR) return c->p[j].mass;
    return 0.0;
}

// Astrocentric elements of a recorded body (pp_disk.cu:526-553, tools.cpp:180-236).
void event_elements(const double r[3], const double v[3], const double r0[3], const double v0[3], double mu,
                    rg_orbelem_t* oe)
{
    rg_vec_t ra{r[0] - r0[0], r[1] - r0[1], r[2] - r0[2], 0.0};
    rg_vec_t va{v[0] - v0[0], v[1] - v0[1], v[2] - v0[2], 0.0};
    rg_vec_t vt{va.x * GAUSS, va.y * GAUSS, va.z * GAUSS, 0.0};
    host::calculate_orbital_element(mu, oe, &ra, &vt);
}

double stage_c(const rg_ctx* c, int stage)
{
    switch (c->int_type) {
    case RG_INT_RK4: return rk4_c[stage];
    case RG_INT_RK5: return rk5_c[stage];
    case RG_INT_RKF78: return rk8_c[stage];
    default: return 0.0;
    }
}

// a gravity kernel whose bounded wait for a tile copy ran out leaves d_kerr set; the
// evaluation is then incomplete and the call that read it fails
int kernel_flag_error(rg_ctx* c, unsigned int flag)
{
    if (!flag) return RG_OK;
    RG_CUDA_CHECK(cudaMemsetAsync(c->d_kerr, 0, sizeof(unsigned int), c->st));
    return set_error(RG_ERR_CUDA, "a gravity tile copy did not arrive within the wait limit");
}

// Device candidates -> the reference's raw event records (pp_disk.cu:470-563), in the
// order its CPU loop creates them: stage by stage, sink i, source j ascending.
int collect_events(rg_ctx* c)
{
    // the three counters in one copy to pinned memory: one round trip per step
    unsigned int* const h_counts = reinterpret_cast<unsigned int*>(&c->h_pin[4]);
    RG_CUDA_CHECK(cudaMemcpyAsync(h_counts, c->d_counters, 3 * sizeof(unsigned int), cudaMemcpyDeviceToHost, c->st));
    RG_CUDA_CHECK(cudaStreamSynchronize(c->st));
    const unsigned int counts[3] = {h_counts[0], h_counts[1], h_counts[2]};
    if (int krc = kernel_flag_error(c, counts[2])) return krc;
    const int nsi = c->n_si();
    for (int kind = 0; kind < 2; kind++) {
        unsigned int n = counts[kind];
        if (n > c->ev_cap) {
            c->overflow = 1;
            n = c->ev_cap;
        }
        std::vector<DevEvent> rec(n);
        if (n) {
            RG_CUDA_CHECK(cudaMemcpyAsync(rec.data(), kind == 0 ? c->d_ev : c->d_hill, n * sizeof(DevEvent),
                                          cudaMemcpyDeviceToHost, c->st));
            RG_CUDA_CHECK(cudaStreamSynchronize(c->st));
        }
        std::sort(rec.begin(), rec.end(), [](const DevEvent& a, const DevEvent& b) {
            if (a.seq != b.seq) return a.seq < b.seq;
            if (a.i != b.i) return a.i < b.i;
            return a.j < b.j;
        });
        std::vector<rg_event_t>& out = kind == 0 ? c->events : c->hill;
        out.clear();
        for (const DevEvent& d : rec) {
            rg_event_t e = zero_event();
            const int stage = (int)(d.seq & 0xff), attempt = (int)(d.seq >> 8);
            const double dt = attempt < (int)c->attempt_dt.size() ? c->attempt_dt[attempt] : c->dt_try;
            const double t0 = c->t_step;
            const double curr_t = t0 + stage_c(c, stage) * dt;  // ttemp of the stage (int_rungekutta8.cu:741)
            const bool nsi_ni = d.i >= nsi;
            e.t = (kind == 1) ? t0 : ((nsi_ni && c->event_time_mode == RG_EVENT_TIME_CPU) ? t0 : curr_t);
            e.d = d.d;
            int surv = d.i, merg = d.j;
            const double *rs = d.ri, *vs = d.vi, *rm = d.rj, *vm = d.vj;
            const bool ce = (kind == 1) || c->close_encounter;
            if (!ce && c->p[merg].mass > c->p[surv].mass) {  // pp_disk.cu:472-477
                std::swap(surv, merg);
                std::swap(rs, rm);
                std::swap(vs, vm);
            }
            e.event_name = ce ? RG_EVENT_CLOSE_ENCOUNTER : RG_EVENT_COLLISION;
            e.id1 = c->md[surv].id;
            e.id2 = c->md[merg].id;
            e.idx1 = surv;
            e.idx2 = merg;
            e.r1 = rg_vec_t{rs[0], rs[1], rs[2], 0.0};
            e.v1 = rg_vec_t{vs[0], vs[1], vs[2], 0.0};
            e.r2 = rg_vec_t{rm[0], rm[1], rm[2], 0.0};
            e.v2 = rg_vec_t{vm[0], vm[1], vm[2], 0.0};
            if (ce) {
                e.p1 = c->p[surv];
                e.p2 = c->p[merg];
            }
            if (kind == 0 && c->close_encounter) {
                const double ms = mass_of_star(c);
                // barycentric: relative to the star (transform_to_ac of a copy, pp_disk.cu:529-552);
                // astrocentric: the coordinates as they are (pp_disk.cu:554-560)
                static const double zero[3] = {0.0, 0.0, 0.0};
                const bool astro = c->frame == RG_FRAME_ASTRO;
                event_elements(rs, vs, astro ? zero : d.r0, astro ? zero : d.v0, GAUSS2 * (ms + c->p[surv].mass),
                               &e.oe1);
                event_elements(rm, vm, astro ? zero : d.r0, astro ? zero : d.v0, GAUSS2 * (ms + c->p[merg].mass),
                               &e.oe2);
            }
            out.push_back(e);
        }
    }
    return RG_OK;
}

void increment_event_counter(rg_ctx* c, int64_t* counter)  // pp_disk.cu:1059-1067
{
    for (int i = 0; i < 3; i++) {
        counter[i]++;
        c->n_event[i]++;
    }
}

// pp_disk::handle_collision_pair (pp_disk.cu:1151-1202); the state lives on the device
int handle_collision_pair(rg_ctx* c, rg_event_t* e)
{
    const int surv = e->idx1, merg = e->idx2;
    if (RG_BODY_SUPERPLANETESIMAL == c->md[merg].body_type)
        return set_error(RG_ERR_NOT_IMPLEMENTED,
                         "collision between a massive body and a super-planetesimal is not implemented "
                         "(the reference throws here, pp_disk.cu:1156-1160)");
    e->p1 = c->p[surv];
    e->p2 = c->p[merg];
    host::calc_position_after_collision(e->p1.mass, e->p2.mass, &e->r1, &e->r2, &e->rs);
    host::calc_velocity_after_collision(e->p1.mass, e->p2.mass, &e->v1, &e->v2, &e->vs);
    host::calc_physical_properties(e->p1, e->p2, &e->ps);
    c->p[surv] = e->ps;
    c->md[merg].id *= -1;
    c->p[merg].mass = 0.0;
    c->p[merg].density = 0.0;
    c->p[merg].radius = 0.0;
    int rc = set_body(c, surv, e->rs, e->vs);
    if (!rc) rc = set_body(c, merg, rg_vec_t{1.0e20, 0.0, 0.0, 0.0}, rg_vec_t{0.0, 0.0, 0.0, 0.0});
    if (!rc) rc = set_param_dev(c, surv);
    if (!rc) rc = set_param_dev(c, merg);
    return rc;
}

int log_push(rg_ctx* c, const rg_event_t& e)
{
    try {
        c->log.push_back(e);
    } catch (const std::bad_alloc&) {
        return set_error(RG_ERR_NOMEM, "event log");
    }
    return RG_OK;
}

// New: log the pairs that entered their mutual Hill sphere at the start of the last step.
int handle_hill(rg_ctx* c)
{
    if (c->hill_factor <= 0.0) return RG_OK;
    std::vector<int64_t> cur;
    cur.reserve(c->hill.size());
    for (const rg_event_t& e : c->hill) {
        const int64_t key = ((int64_t)(uint32_t)e.id1 << 32) | (int64_t)(uint32_t)e.id2;
        if (std::find(c->hill_pairs.begin(), c->hill_pairs.end(), key) == c->hill_pairs.end()) {
            int rc = log_push(c, e);
            if (rc) return rc;
            increment_event_counter(c, c->n_close_encounter);
        }
        cur.push_back(key);
    }
    c->hill_pairs.swap(cur);
    c->hill.clear();
    return RG_OK;
}

// --------------------------------------------------------------------- integrator pieces
int set_dt(rg_ctx* c, double dt)
{
    c->h_pin[0] = dt;
    RG_CUDA_CHECK(cudaMemcpyAsync(c->d_dt, &c->h_pin[0], sizeof(double), cudaMemcpyHostToDevice, c->st));
    return RG_OK;
}

int combine(rg_ctx* c, int form, const int* stages, const double* coef, int nterm, double* out_lo, double* out_hi)
{
    CombineArgs a{};
    a.y = c->d_y;
    for (int q = 0; q < nterm; q++) {
        a.k[q] = c->d_k[stages[q]];
        a.c[q] = coef[q];
    }
    a.nterm = nterm;
    a.form = form;
    a.n = c->n_total();
    a.stride = c->cap;
    a.dt = c->d_dt;
    a.out_lo = out_lo;
    a.out_hi = out_hi;
    if (a.n <= 0) return RG_OK;
    const long prof = prof_begin(c, 1);
    int rc = launch_combine(a, c->st);
    prof_end(c, prof);
    c->n_kernels++;
    return rc < 0 && rc != RG_ERR_CUDA ? set_error(RG_ERR_ARG, "bad stage combine") : rc;
}

// a stage r >= 1: combine into (P, k_r.lo), then gravity into k_r.hi
int ytemp_stage(rg_ctx* c, int form, int r, const int* stages, const double* coef, int nterm, int attempt)
{
    int rc = combine(c, form, stages, coef, nterm, c->d_P, c->d_k[r]);
    if (rc) return rc;
    return gravity(c, c->d_P, c->d_k[r], c->d_k[r] + 3 * (size_t)c->cap, r, attempt, true, false);
}

// stage 0: k_0 = (v, a(y)) -- the reference's calc_dydx(0/1, r = 0) on y (pp_disk.cu:1006-1013)
int stage_zero(rg_ctx* c)
{
    const size_t cap = (size_t)c->cap;
    RG_CUDA_CHECK(cudaMemsetAsync(c->d_ev_count, 0, 2 * sizeof(unsigned int), c->st));  // and d_hill_count
    if (c->n_total() > 0)
        RG_CUDA_CHECK(cudaMemcpyAsync(c->d_k[0], c->d_y + 3 * cap, 3 * cap * sizeof(double),
                                      cudaMemcpyDeviceToDevice, c->st));
    return gravity(c, c->d_y, c->d_y + 3 * cap, c->d_k[0] + 3 * cap, 0, 0, true, c->hill_factor > 0.0);
}

// error maximum and event count of this attempt (one synchronisation)
int read_attempt(rg_ctx* c, double* raw, unsigned int* n_events)
{
    RG_CUDA_CHECK(cudaMemcpyAsync(&c->h_pin[1], c->d_maxbits, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                  c->st));
    RG_CUDA_CHECK(cudaMemcpyAsync((unsigned int*)&c->h_pin[2], c->d_ev_count, sizeof(unsigned int),
                                  cudaMemcpyDeviceToHost, c->st));
    RG_CUDA_CHECK(cudaStreamSynchronize(c->st));
    unsigned long long bits;
    std::memcpy(&bits, &c->h_pin[1], sizeof(bits));
    double v;
    std::memcpy(&v, &bits, sizeof(v));
    *raw = v;
    *n_events = *(unsigned int*)&c->h_pin[2];
    return RG_OK;
}

int error_max(rg_ctx* c, int form, const int* stages, const double* coef, int nk)
{
    RG_CUDA_CHECK(cudaMemsetAsync(c->d_maxbits, 0, sizeof(unsigned long long), c->st));
    ErrArgs a{};
    for (int q = 0; q < nk; q++) {
        a.k[q] = c->d_k[stages[q]];
        a.c[q] = coef ? coef[q] : 0.0;
    }
    a.form = form;
    a.stride = c->cap;
    a.n_err = c->ectp ? c->n_total() : c->n_massive();
    a.max_bits = c->d_maxbits;
    const long prof = prof_begin(c, 1);
    const int rc = launch_error_max(a, c->st);
    prof_end(c, prof);
    c->n_kernels += a.n_err > 0;
    return rc;
}

void swap_y(rg_ctx* c) { std::swap(c->d_y, c->d_yout); }

void update_counters(rg_ctx* c, int iter)  // integrator.cu:258-263
{
    c->n_tried += iter;
    c->n_failed += (iter - 1);
    c->n_passed++;
}

// ---- Euler (int_euler.cu:76-141)
int step_euler(rg_ctx* c)
{
    c->attempt_dt.assign(1, c->dt_try);
    int rc = stage_zero(c);
    if (!rc) rc = set_dt(c, c->dt_try);
    const int st0[1] = {0};
    const double one[1] = {1.0};
    if (!rc) rc = combine(c, FORM_SUM, st0, one, 1, c->d_yout, c->d_yout + 3 * (size_t)c->cap);
    if (rc) return rc;
    c->dt_did = c->dt_try;
    update_counters(c, 1);
    c->t += c->dt_did;
    swap_y(c);
    return RG_OK;
}

// ---- RK4 (int_rungekutta4.cu:189-273)
int step_rk4(rg_ctx* c)
{
    const size_t cap = (size_t)c->cap;
    c->attempt_dt.clear();
    int rc = stage_zero(c);
    if (rc) return rc;
    double max_err = 0.0;
    int iter = 0, attempt = 0;
    do {
        c->dt_did = c->dt_try;
        c->attempt_dt.push_back(c->dt_try);
        rc = set_dt(c, c->dt_try);
        for (int r = 1; r < 4 && !rc; r++) {
            const int st[1] = {r - 1};
            const double a[1] = {rk4_a[r]};
            rc = ytemp_stage(c, FORM_SCALED, r, st, a, 1, attempt);
        }
        const int st4[4] = {0, 1, 2, 3};
        const double b[4] = {rk4_b[0], rk4_b[1], 0.0, 0.0};  // the kernel reads c[0], c[1]
        if (!rc) rc = combine(c, FORM_RK4_NP1, st4, b, 4, c->d_yout, c->d_yout + 3 * cap);
        if (rc) return rc;
        if (c->adaptive) {
            // f5 = f(y_{n+1}); dydx[0][4] is v_{n+1}
            RG_CUDA_CHECK(cudaMemcpyAsync(c->d_k[4], c->d_yout + 3 * cap, 3 * cap * sizeof(double),
                                          cudaMemcpyDeviceToDevice, c->st));
            rc = gravity(c, c->d_yout, c->d_yout + 3 * cap, c->d_k[4] + 3 * cap, 4, attempt, true, false);
            const int se[2] = {3, 4};
            if (!rc) rc = error_max(c, ERR_RK4, se, nullptr, 2);
            double raw;
            unsigned int nev;
            if (!rc) rc = read_attempt(c, &raw, &nev);
            if (rc) return rc;
            max_err = std::fabs(c->dt_try * (1.0 / 10.0) * raw);
            c->dt_try *= 0.9 * std::pow(c->tol / max_err, 1.0 / 4.0);
            if (nev > 0) {
                if (c->dt_try < c->dt_did) c->dt_try = c->dt_did;
                break;
            }
        }
        iter++;
        attempt++;
    } while (c->adaptive && max_err > c->tol);
    update_counters(c, iter);
    c->t += c->dt_did;
    swap_y(c);
    return RG_OK;
}

// ---- RKF5, Cash-Karp (restated from int_rungekutta5.cu:41-93,202-282): all six stages
// are evaluated before y_{n+1}, which the reference propagates with the b weights.
int step_rk5(rg_ctx* c)
{
    const size_t cap = (size_t)c->cap;
    c->attempt_dt.clear();
    int rc = stage_zero(c);
    if (rc) return rc;
    double max_err = 0.0;
    int iter = 0, attempt = 0;
    do {
        c->dt_did = c->dt_try;
        c->attempt_dt.push_back(c->dt_try);
        rc = set_dt(c, c->dt_try);
        for (int r = 1; r < 6 && !rc; r++) {
            int st[6];
            double a[6];
            int nt = 0;
            for (int q = 0; q < r; q++) {
                const double aq = rk5_a[rk5_idx[r] + q];
                if (0.0 == aq) continue;
                st[nt] = q;
                a[nt++] = aq;
            }
            rc = ytemp_stage(c, FORM_ACC, r, st, a, nt, attempt);
        }
        if (rc) return rc;
        {
            int st[6];
            double b[6];
            int nt = 0;
            for (int q = 0; q < 6; q++) {
                if (0.0 == rk5_b[q]) continue;
                st[nt] = q;
                b[nt++] = rk5_b[q];
            }
            rc = combine(c, FORM_ACC, st, b, nt, c->d_yout, c->d_yout + 3 * cap);
            if (rc) return rc;
        }
        if (c->adaptive) {
            const int se[6] = {0, 1, 2, 3, 4, 5};
            double ce[6];
            for (int q = 0; q < 6; q++) ce[q] = rk5_bh[q] - rk5_b[q];
            rc = error_max(c, ERR_RK5, se, ce, 6);
            double raw;
            unsigned int nev;
            if (!rc) rc = read_attempt(c, &raw, &nev);
            if (rc) return rc;
            max_err = std::fabs(c->dt_try * raw);
            c->dt_try *= 0.9 * std::pow(c->tol / max_err, 1.0 / 5);
            if (nev > 0) {
                if (c->dt_try < c->dt_did) c->dt_try = c->dt_did;
                break;
            }
        }
        iter++;
        attempt++;
    } while (c->adaptive && max_err > c->tol);
    update_counters(c, iter);
    c->t += c->dt_did;
    swap_y(c);
    return RG_OK;
}

// ---- RKF7(8) (int_rungekutta8.cu:704-797)
// Everything a captured step graph freezes into its launches: buffer addresses, sizes, the
// tile plan, the gravity and event options, the integrator's shape.
std::vector<double> graph_signature(const rg_ctx* c)
{
    return {(double)(uintptr_t)c->d_y,  (double)(uintptr_t)c->d_yout, (double)c->cap,
            (double)c->n_total(),       (double)c->tiles_version,      (double)(uintptr_t)c->d_tiles,
            (double)c->gravity_mode,    c->hill_factor,                c->thr[RG_THRESHOLD_RADII_ENHANCE_FACTOR],
            (double)c->inner_steps,     (double)c->close_encounter,    (double)c->int_type,
            (double)c->adaptive,        (double)c->r_max,              (double)c->ectp,
            (double)c->pairpar_S,       (double)c->rowseq_max_src,     (double)c->mixed_chunk_src,
            (double)c->near_ratio,      (double)(uintptr_t)c->d_partial, (double)c->partial_cap,
            (double)(uintptr_t)c->d_terms, (double)c->few_pitch,       (double)c->few_rows,
            (double)(uintptr_t)c->d_astro};
}

// Captures `body` (launches on the context's stream) into `sg`; false: capture not possible
// now (the body needed an allocation, or CUDA refused), the caller launches directly.
template <class F>
bool capture_step_graph(rg_ctx* c, rg_ctx::StepGraph& sg, F body)
{
    if (sg.exec) cudaGraphExecDestroy(sg.exec);
    sg.exec = nullptr;
    const int64_t k0 = c->n_kernels, e0 = c->n_gravity_evals, p0 = c->n_pairs;
    if (cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    c->capturing = true;
    c->capture_failed = false;
    const int rc = body();
    c->capturing = false;
    cudaGraph_t graph = nullptr;
    const cudaError_t err = cudaStreamEndCapture(c->st, &graph);
    sg.kernels = c->n_kernels - k0;
    sg.evals = c->n_gravity_evals - e0;
    sg.pairs = c->n_pairs - p0;
    c->n_kernels = k0;
    c->n_gravity_evals = e0;
    c->n_pairs = p0;
    bool ok = rc == RG_OK && !c->capture_failed && err == cudaSuccess && graph;
    if (ok && cudaGraphInstantiate(&sg.exec, graph, 0) != cudaSuccess) {
        sg.exec = nullptr;
        ok = false;
    }
    if (graph) cudaGraphDestroy(graph);
    if (!ok) cudaGetLastError();  // a refused capture leaves no sticky error; launch directly
    sg.sig = ok ? graph_signature(c) : std::vector<double>{};
    return ok;
}

// Replays `sg` (capturing it first if its frozen parameters changed); false: launch directly.
template <class F>
bool replay_step_graph(rg_ctx* c, rg_ctx::StepGraph& sg, F body, int* rc)
{
    *rc = RG_OK;
    if (!c->use_graphs || c->profiling || c->hold_tile_copies) return false;
    if ((*rc = sync_tiles(c))) return false;
    if (!sg.exec || sg.sig != graph_signature(c))
        if (!capture_step_graph(c, sg, body)) return false;
    const cudaError_t err = cudaGraphLaunch(sg.exec, c->st);
    if (err != cudaSuccess) {
        *rc = cuda_fail(err, "cudaGraphLaunch", __FILE__, __LINE__);
        return true;
    }
    c->n_kernels += sg.kernels;
    c->n_gravity_evals += sg.evals;
    c->n_pairs += sg.pairs;
    return true;
}

int step_rkf78(rg_ctx* c)
{
    const size_t cap = (size_t)c->cap;
    c->attempt_dt.clear();
    const int parity = c->d_y < c->d_yout ? 0 : 1;
    int rc = RG_OK;
    if (!replay_step_graph(c, c->g_stage0[parity], [&] { return stage_zero(c); }, &rc)) rc = rc ? rc : stage_zero(c);
    if (rc) return rc;
    double max_err = 0.0;
    int iter = 0, attempt = 0;
    // one attempt's device work: stage rows, y_{n+1}, error maximum and the read-back of the
    // error and event count into pinned memory (the attempt's number and trial step come
    // from pinned memory too, so a captured attempt is replayed as it stands)
    auto attempt_body = [&]() {
        // events of a previous attempt (and of stage 0) are dropped (int_rungekutta8.cu:730-733)
        RG_CUDA_CHECK(cudaMemsetAsync(c->d_ev_count, 0, sizeof(unsigned int), c->st));
        RG_CUDA_CHECK(cudaMemcpyAsync(c->d_dt, &c->h_pin[0], sizeof(double), cudaMemcpyHostToDevice, c->st));
        RG_CUDA_CHECK(cudaMemcpyAsync(c->d_attempt_no, &c->h_pin[6], sizeof(unsigned int), cudaMemcpyHostToDevice,
                                      c->st));
        int r2 = RG_OK;
        auto row = [&](int r) {
            double a[9];
            for (int q = 0; q < rk8_nterm[r]; q++) a[q] = rk8_a[rk8_aidx[r][q]];
            return ytemp_stage(c, FORM_SUM, r, rk8_stage[r], a, rk8_nterm[r], attempt);
        };
        for (int r = 1; r <= 10 && !r2; r++) r2 = row(r);
        const int snp[7] = {0, 5, 6, 7, 8, 9, 10};
        const double bnp[7] = {rk8_b[0], rk8_b[5], rk8_b[6], rk8_b[8], rk8_b[10], 0.0, 0.0};  // c[0..4] used
        if (!r2) r2 = combine(c, FORM_RK8_NP1, snp, bnp, 7, c->d_yout, c->d_yout + 3 * cap);
        if (!r2 && c->adaptive) {
            for (int r = 11; r < c->r_max && !r2; r++) r2 = row(r);
            const int se[4] = {0, 10, 11, 12};
            if (!r2) r2 = error_max(c, ERR_RK8, se, nullptr, 4);
            if (!r2) {
                RG_CUDA_CHECK(cudaMemcpyAsync(&c->h_pin[1], c->d_maxbits, sizeof(unsigned long long),
                                              cudaMemcpyDeviceToHost, c->st));
                RG_CUDA_CHECK(cudaMemcpyAsync((unsigned int*)&c->h_pin[2], c->d_ev_count, sizeof(unsigned int),
                                              cudaMemcpyDeviceToHost, c->st));
            }
        }
        return r2;
    };
    do {
        c->dt_did = c->dt_try;
        c->attempt_dt.push_back(c->dt_try);
        c->h_pin[0] = c->dt_try;
        *(unsigned int*)&c->h_pin[6] = (unsigned int)attempt;
        if (!replay_step_graph(c, c->g_attempt[parity], attempt_body, &rc)) rc = rc ? rc : attempt_body();
        if (rc) return rc;
        if (c->adaptive) {
            RG_CUDA_CHECK(cudaStreamSynchronize(c->st));
            unsigned long long bits;
            std::memcpy(&bits, &c->h_pin[1], sizeof(bits));
            double raw;
            std::memcpy(&raw, &bits, sizeof(raw));
            max_err = std::fabs(c->dt_try * (41.0 / 840.0) * raw);
            c->dt_try *= 0.9 * std::pow(c->tol / max_err, 1.0 / (c->order + 1));
        }
        iter++;
        attempt++;
    } while (c->adaptive && max_err > c->tol);
    update_counters(c, iter);
    c->t += c->dt_did;
    swap_y(c);
    return RG_OK;
}

// --------------------------------------------------------------------- pp_disk handlers
// store_event_data, host version (pp_disk.cu:909-932)
int store_event_data(rg_ctx* c, int name, double t, double d, int idx1, int idx2, rg_event_t* e)
{
    *e = zero_event();
    e->event_name = name;
    e->d = d;
    e->t = t;
    e->id1 = c->md[idx1].id;
    e->id2 = c->md[idx2].id;
    e->idx1 = idx1;
    e->idx2 = idx2;
    int rc = get_body(c, idx1, &e->r1, &e->v1);
    if (!rc) rc = get_body(c, idx2, &e->r2, &e->v2);
    if (rc) return rc;
    if (RG_EVENT_EJECTION == name) {
        e->p1 = c->p[idx1];
        e->p2 = c->p[idx2];
        e->rs = e->r1;
        e->vs = e->v1;
        e->ps = e->p1;
    }
    return RG_OK;
}

int check_ejection_hit(rg_ctx* c, int* n_handled)
{
    if (n_handled) *n_handled = 0;
    const int n = c->n_total();
    const bool any = (0.0 < c->thr[RG_THRESHOLD_EJECTION_DISTANCE]) || (0.0 < c->thr[RG_THRESHOLD_HIT_CENTRUM_DISTANCE]);
    if (any && n > 0) {
        RG_CUDA_CHECK(cudaMemsetAsync(c->d_ej_count, 0, sizeof(unsigned int), c->st));
        int rc = launch_ejection(c->d_y, c->d_y + c->cap, c->d_y + 2 * (size_t)c->cap, c->d_id, c->d_type, n, c->thr,
                                 c->d_ej, c->d_ej_count, (unsigned int)c->cap, c->st);
        if (rc) return rc;
        c->n_kernels++;
        unsigned int cnt = 0;
        RG_CUDA_CHECK(cudaMemcpyAsync(&cnt, c->d_ej_count, sizeof(unsigned int), cudaMemcpyDeviceToHost, c->st));
        RG_CUDA_CHECK(cudaStreamSynchronize(c->st));
        if (cnt > 0) {
            std::vector<EjectRec> rec(cnt);
            RG_CUDA_CHECK(cudaMemcpyAsync(rec.data(), c->d_ej, cnt * sizeof(EjectRec), cudaMemcpyDeviceToHost, c->st));
            RG_CUDA_CHECK(cudaStreamSynchronize(c->st));
            std::sort(rec.begin(), rec.end(), [](const EjectRec& a, const EjectRec& b) { return a.i < b.i; });
            for (const EjectRec& r : rec) {
                if (c->events.size() >= c->ev_cap) return set_error(RG_ERR_EVENT_OVERFLOW, "event buffer full");
                rg_event_t e;
                rc = store_event_data(c, r.kind, c->t, std::sqrt(r.r2), 0, r.i, &e);
                if (rc) return rc;
                c->md[r.i].id *= -1;
                c->events.push_back(e);
            }
        }
    }
    const int n_event = (int)c->events.size();
    if (n_handled) *n_handled = n_event;
    if (0 < n_event) {  // pp_disk::handle_ejection_hit_centrum (pp_disk.cu:1091-1109)
        for (int i = 0; i < n_event; i++) {
            rg_event_t e = c->events[i];
            int rc;
            if (e.event_name == RG_EVENT_EJECTION) {
                increment_event_counter(c, c->n_ejection);
                rc = set_param_dev(c, e.idx2);
            } else {
                rc = handle_collision_pair(c, &e);
                increment_event_counter(c, c->n_hit_centrum);
            }
            if (!rc) rc = log_push(c, e);
            if (rc) return rc;
        }
        c->n_ejection[RG_COUNTER_LAST_STEP] = 0;
        c->n_hit_centrum[RG_COUNTER_LAST_STEP] = 0;
        c->events.clear();
    }
    return RG_OK;
}

// pp_disk::check_for_collision -> handle_collision -> create_sp_events (pp_disk.cu:717-738,
// 1078-1149) and the caller's clear_event_counter
int check_collision(rg_ctx* c, int* n_handled)
{
    if (n_handled) *n_handled = 0;
    const int ec = (int)c->events.size();
    if (ec <= 0) return RG_OK;
    std::vector<rg_event_t> sp;
    std::vector<char> processed(ec, 0);
    for (int k = 0; k < ec; k++) {
        if (processed[k]) continue;
        processed[k] = 1;
        rg_event_t cur = c->events[k];
        for (int i = k + 1; i < ec; i++) {
            if (cur.id1 == c->events[i].id1 && cur.id2 == c->events[i].id2) {
                processed[i] = 1;
                if (cur.t > c->events[i].t) cur = c->events[i];
            }
        }
        sp.push_back(cur);
    }
    for (auto& e : sp) {
        int rc = handle_collision_pair(c, &e);
        if (rc) return rc;
        increment_event_counter(c, c->n_collision);
        rc = log_push(c, e);
        if (rc) return rc;
    }
    c->n_collision[RG_COUNTER_LAST_STEP] = 0;
    c->events.clear();
    if (n_handled) *n_handled = (int)sp.size();
    return RG_OK;
}

int check_close_encounter(rg_ctx* c, int* n_handled)  // pp_disk.cu:742-770
{
    const int ec = (int)c->events.size();
    if (n_handled) *n_handled = ec;
    if (ec <= 0) return RG_OK;
    for (const auto& e : c->events) {
        int rc = log_push(c, e);
        if (rc) return rc;
        increment_event_counter(c, c->n_close_encounter);
    }
    c->n_close_encounter[RG_COUNTER_LAST_STEP] = 0;
    c->events.clear();
    return RG_OK;
}

// number_of_bodies::update_numbers + pp_disk::remove_inactive_bodies
// (number_of_bodies.cpp:27-104, pp_disk.cu:1324-1409)
// pp_disk::remove_inactive_bodies (pp_disk.cu:1324-1409): the host records (p, md, epoch)
// are filtered on the host, where they live; the positions and velocities are gathered on the
// device by the list of kept bodies, so the state does not travel to the host and back.
int remove_inactive_bodies(rg_ctx* c)
{
    const int old_n = c->n_total();
    int rc = RG_OK;
    int inactive[7] = {0};
    for (int i = 0; i < old_n; i++) {
        if (!(0 < c->md[i].id && RG_BODY_PADDINGPARTICLE > c->md[i].body_type)) {
            const int ty = c->md[i].body_type;
            if (ty < 0 || ty > 6) return set_error(RG_ERR_ARG, "Undefined body type!");
            inactive[ty]++;
        }
    }
    for (int k = 0; k < 7; k++) {
        c->n_inactive[k] += inactive[k];
        c->cnt[k] -= inactive[k];
    }
    const int n = c->n_total();
    std::vector<int> keep;
    keep.reserve(n);
    int k = 0;
    for (int i = 0; i < old_n; i++) {
        if (0 < c->md[i].id && RG_BODY_PADDINGPARTICLE > c->md[i].body_type) {
            keep.push_back(i);
            c->p[k] = c->p[i];
            c->md[k] = c->md[i];
            c->epoch[k] = c->epoch[i];
            k++;
        }
    }
    if (k != n) return set_error(RG_ERR_STATE, "number of copied bodies does not equal the number of active bodies");
    c->p.resize(n);
    c->md.resize(n);
    c->epoch.resize(n);
    if (n > 0) {
        // the list goes to a temporary device array; the gather writes d_yout (scratch between
        // steps), which is then copied back into d_y
        int* d_keep = nullptr;
        rc = dalloc(&d_keep, (size_t)n);
        if (rc) return rc;
        cudaError_t e = cudaMemcpyAsync(d_keep, keep.data(), (size_t)n * sizeof(int), cudaMemcpyHostToDevice, c->st);
        if (e == cudaSuccess) rc = launch_gather_rows(c->d_y, c->d_yout, c->cap, d_keep, n, c->st);
        if (e == cudaSuccess && !rc)
            e = cudaMemcpy2DAsync(c->d_y, c->cap * sizeof(double), c->d_yout, c->cap * sizeof(double),
                                  n * sizeof(double), 6, cudaMemcpyDeviceToDevice, c->st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);  // keep (host) and d_keep outlive the copies
        cudaFree(d_keep);
        if (e != cudaSuccess) return cuda_fail(e, "compaction", __FILE__, __LINE__);
        if (rc) return rc;
    }
    rc = upload_params(c);
    build_tiles(c);
    return rc;
}

int check_rebuild(rg_ctx* c, int n, int* rebuilt)  // pp_disk.cu:893-907
{
    if (rebuilt) *rebuilt = 0;
    if (c->n_event[RG_COUNTER_LAST_CLEAR] >= n) {
        int rc = remove_inactive_bodies(c);
        if (rc) return rc;
        c->n_hit_centrum[RG_COUNTER_LAST_CLEAR] = 0;
        c->n_ejection[RG_COUNTER_LAST_CLEAR] = 0;
        c->n_collision[RG_COUNTER_LAST_CLEAR] = 0;
        c->n_close_encounter[RG_COUNTER_LAST_CLEAR] = 0;
        c->n_event[RG_COUNTER_LAST_CLEAR] = 0;
        if (rebuilt) *rebuilt = 1;
    }
    return RG_OK;
}

int do_step(rg_ctx* c)
{
    if (!c->has_int) return set_error(RG_ERR_STATE, "no integrator set (rg_set_integrator)");
    c->t_step = c->t;
    int rc;
    switch (c->int_type) {
    case RG_INT_EULER: rc = step_euler(c); break;
    case RG_INT_RK4: rc = step_rk4(c); break;
    case RG_INT_RK5: rc = step_rk5(c); break;
    default: rc = step_rkf78(c); break;
    }
    if (!rc) rc = collect_events(c);
    if (rc) return rc;
    if (c->overflow) {
        c->overflow = 0;
        return set_error(RG_ERR_EVENT_OVERFLOW, "more event records in one step than the event buffer holds");
    }
    return RG_OK;
}

}  // namespace

// ============================================================================ C ABI

extern "C" {

const char* rg_last_error(void) { return redgb::last_error(); }

const char* rg_version(void) { return "redgb 1.0 (sm_103a)"; }

int rg_device_count(void)
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

// The default sinks per pair-parallel CTA: every CTA of the self-interacting block runs all of
// its sources, so a launch takes (waves of resident CTAs) x (one CTA's time, proportional to
// S); the S of the candidate set with the fewest wave-sinks, the larger S on a tie (fewer
// barriers per pair).  16 385 sinks on 152 SMs x 3 CTAs: S = 36, one wave of 456 CTAs.
// rg_autotune times the candidates instead.
static int wave_best_sinks(const rg_ctx* c)
{
    const int ns = c->n_si() - (c->frame == RG_FRAME_ASTRO ? 1 : 0);
    if (ns <= 0) return 16;
    const long long slots = (long long)std::max(c->n_sm, 1) * RG_PAIRPAR_RESIDENT;
    static const int astro_s[] = {8, 16, 32};
    static const int bary_s[] = {8, 12, 16, 18, 24, 32, 36};
    const int* cand = c->frame == RG_FRAME_ASTRO ? astro_s : bary_s;
    const int nc = c->frame == RG_FRAME_ASTRO ? 3 : 7;
    int best = 16;
    long long best_cost = -1;
    for (int k = 0; k < nc; k++) {
        const int S = cand[k];
        const long long ctas = (ns + S - 1) / S;
        const long long cost = (ctas + slots - 1) / slots * S;
        if (best_cost < 0 || cost < best_cost || (cost == best_cost && S > best)) {
            best_cost = cost;
            best = S;
        }
    }
    return best;
}

static int create_impl(const rg_counts_t* n, const rg_vec_t* r, const rg_vec_t* v, const rg_param_t* p,
                       const rg_body_metadata_t* md, const double* epoch, const double thr[RG_THRESHOLD_N],
                       int event_capacity, int frame, rg_ctx** out)
{
    if (!n || !r || !v || !p || !md || !thr || !out) return set_error(RG_ERR_ARG, "null argument");
    *out = nullptr;
    if (frame != RG_FRAME_BARY && frame != RG_FRAME_ASTRO) return set_error(RG_ERR_ARG, "frame_center");
    if (frame == RG_FRAME_ASTRO && (n->n_spl > 0 || n->n_pl > 0 || n->n_tp > 0))
        return set_error(RG_ERR_NOT_IMPLEMENTED,
                         "the astrocentric frame with super-planetesimals, planetesimals or test particles: their "
                         "blocks take the star at the origin as a source, whose indirect term m / (0 sqrt(0)) 0 "
                         "makes the reference's accelerations NaN (pp_disk.cu:447-454)");
    const int32_t* cn = &n->n_s;
    int64_t tot = 0;
    for (int k = 0; k < 7; k++) {
        if (cn[k] < 0) return set_error(RG_ERR_ARG, "negative body count");
        tot += cn[k];
    }
    if (tot <= 0 || tot > (1 << 28)) return set_error(RG_ERR_ARG, "body count out of range");
    if (rg_device_count() <= 0) return set_error(RG_ERR_NO_DEVICE, "no CUDA device");
    if (frame == RG_FRAME_ASTRO && md[0].body_type != RG_BODY_STAR)
        return set_error(RG_ERR_ARG, "the astrocentric frame needs the star as body 0 (\"No star is included!\")");
    rg_ctx* c = new rg_ctx();
    c->frame = frame;
    for (int k = 0; k < 7; k++) c->cnt[k] = cn[k];
    const int nt = (int)tot;
    c->cap = nt;
    cudaGetDevice(&c->device);
    cudaDeviceGetAttribute(&c->n_sm, cudaDevAttrMultiProcessorCount, c->device);
    c->ev_cap = (unsigned int)(event_capacity > 0 ? event_capacity : std::max(nt, 1024));
    int rc = RG_OK;
    auto chk = [&](int x) {
        if (!rc) rc = x;
    };
    if (cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking) != cudaSuccess) chk(set_error(RG_ERR_CUDA, "stream"));
    if (!rc && (cudaStreamCreateWithFlags(&c->st2, cudaStreamNonBlocking) != cudaSuccess ||
                cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
                cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming) != cudaSuccess))
        chk(set_error(RG_ERR_CUDA, "stream"));
    chk(dalloc(&c->d_y, (size_t)6 * nt));
    chk(dalloc(&c->d_yout, (size_t)6 * nt));
    for (auto& k : c->d_k) chk(dalloc(&k, (size_t)6 * nt));
    chk(dalloc(&c->d_P, (size_t)3 * nt));
    chk(dalloc(&c->d_mass, nt));
    chk(dalloc(&c->d_radius, nt));
    chk(dalloc(&c->d_id, nt));
    chk(dalloc(&c->d_type, nt));
    chk(dalloc(&c->d_rho, nt));
    chk(dalloc(&c->d_ev, c->ev_cap));
    chk(dalloc(&c->d_hill, c->ev_cap));
    chk(dalloc(&c->d_counters, 4));
    if (!rc) {
        c->d_ev_count = c->d_counters;
        c->d_hill_count = c->d_counters + 1;
        c->d_kerr = c->d_counters + 2;
        c->d_sym_ticket = c->d_counters + 3;
    }
    if (!rc && cudaMemsetAsync(c->d_counters, 0, 4 * sizeof(unsigned int), c->st) != cudaSuccess)
        chk(set_error(RG_ERR_CUDA, "cudaMemsetAsync"));
    chk(dalloc(&c->d_ej, nt));
    chk(dalloc(&c->d_ej_count, 1));
    chk(dalloc(&c->d_maxbits, 1));
    chk(dalloc(&c->d_dt, 1));
    chk(dalloc(&c->d_attempt_no, 1));
    chk(dalloc(&c->d_part, (size_t)5 * nt));
    chk(dalloc(&c->d_records, (size_t)8 * nt));
    chk(dalloc((char**)&c->d_split, SPLIT_POS_BYTES * (size_t)nt));
    chk(dalloc(&c->d_rf, nt));
    chk(dalloc(&c->d_smax, SCREEN_MAX_WORDS));
    chk(dalloc(&c->d_screen_slot, nt));
    if (!rc && cudaMallocHost((void**)&c->h_pin, 8 * sizeof(double)) != cudaSuccess)
        chk(set_error(RG_ERR_NOMEM, "pinned host buffer"));
    if (frame == RG_FRAME_ASTRO) {
        chk(dalloc(&c->d_astro, (size_t)6 * nt));
        // the star's row of every derivative buffer is never written in this frame
        // (get_bound_SI starts at 1) and stays zero, as the reference's cleared host buffers do
        for (auto& k : c->d_k)
            if (!rc && k && cudaMemsetAsync(k, 0, (size_t)6 * nt * sizeof(double), c->st) != cudaSuccess)
                chk(set_error(RG_ERR_CUDA, "cudaMemsetAsync"));
    }
    if (rc) {
        free_all(c);
        delete c;
        return rc;
    }
    // pp_disk::load + options::create_pp_disk (pp_disk.cu:1576-1683, options.cpp:197-235)
    std::vector<rg_vec_t> rr(r, r + nt), vv(v, v + nt);
    for (int i = 0; i < nt; i++) rr[i].w = vv[i].w = 0.0;
    c->p.assign(p, p + nt);
    c->md.assign(md, md + nt);
    c->epoch.assign(nt, 0.0);
    if (epoch)
        for (int i = 0; i < nt; i++) c->epoch[i] = epoch[i];
    for (int k = 0; k < RG_THRESHOLD_N; k++) c->thr[k] = thr[k];
    const bool at_rest_in_origin = 0 == std::fabs(rr[0].x) && 0 == std::fabs(rr[0].y) && 0 == std::fabs(rr[0].z) &&
                                   0 == std::fabs(vv[0].x) && 0 == std::fabs(vv[0].y) && 0 == std::fabs(vv[0].z);
    if (!at_rest_in_origin && frame == RG_FRAME_ASTRO) {
        // tools.cpp:180-236 get_star_bc_phase + transform_to_ac, loop j = n-1 .. 0
        const rg_vec_t R0 = rr[0], V0 = vv[0];
        for (int j = nt - 1; j >= 0; j--) {
            rr[j].x -= R0.x;
            rr[j].y -= R0.y;
            rr[j].z -= R0.z;
            vv[j].x -= V0.x;
            vv[j].y -= V0.y;
            vv[j].z -= V0.z;
        }
    }
    if (at_rest_in_origin && frame == RG_FRAME_BARY) {
        // tools.cpp:109-178 compute_bc + transform_to_bc, loops j = n-1 .. 0
        rg_vec_t R0{0, 0, 0, 0}, V0{0, 0, 0, 0};
        for (int j = nt - 1; j >= 0; j--) {
            const double m = c->p[j].mass;
            R0.x += m * rr[j].x;
            R0.y += m * rr[j].y;
            R0.z += m * rr[j].z;
            V0.x += m * vv[j].x;
            V0.y += m * vv[j].y;
            V0.z += m * vv[j].z;
        }
        double M0 = 0.0;
        for (int j = nt - 1; j >= 0; j--) M0 += c->p[j].mass;
        R0.x /= M0;
        R0.y /= M0;
        R0.z /= M0;
        V0.x /= M0;
        V0.y /= M0;
        V0.z /= M0;
        for (int j = nt - 1; j >= 0; j--) {
            rr[j].x -= R0.x;
            rr[j].y -= R0.y;
            rr[j].z -= R0.z;
            vv[j].x -= V0.x;
            vv[j].y -= V0.y;
            vv[j].z -= V0.z;
        }
    }
    for (int j = 0; j < nt; j++) c->epoch[j] *= GAUSS;  // pp_disk.cu:1512-1551
    for (int j = 0; j < nt; j++) {
        vv[j].x /= GAUSS;
        vv[j].y /= GAUSS;
        vv[j].z /= GAUSS;
    }
    std::vector<double> h((size_t)6 * nt);
    for (int i = 0; i < nt; i++) {
        h[i] = rr[i].x;
        h[(size_t)nt + i] = rr[i].y;
        h[(size_t)2 * nt + i] = rr[i].z;
        h[(size_t)3 * nt + i] = vv[i].x;
        h[(size_t)4 * nt + i] = vv[i].y;
        h[(size_t)5 * nt + i] = vv[i].z;
    }
    rc = upload_state(c, h);
    if (!rc) rc = upload_params(c);
    if (rc) {
        free_all(c);
        delete c;
        return rc;
    }
    c->pairpar_S = wave_best_sinks(c);
    build_tiles(c);
    *out = c;
    return RG_OK;
}

int rg_create(const rg_counts_t* n, const rg_vec_t* r, const rg_vec_t* v, const rg_param_t* p,
              const rg_body_metadata_t* md, const double* epoch, const double thr[RG_THRESHOLD_N], int event_capacity,
              rg_ctx** out)
{
    RG_GUARD(create_impl(n, r, v, p, md, epoch, thr, event_capacity, RG_FRAME_BARY, out));
}

int rg_create_in_frame(const rg_counts_t* n, const rg_vec_t* r, const rg_vec_t* v, const rg_param_t* p,
                       const rg_body_metadata_t* md, const double* epoch, const double thr[RG_THRESHOLD_N],
                       int event_capacity, int frame_center, rg_ctx** out)
{
    RG_GUARD(create_impl(n, r, v, p, md, epoch, thr, event_capacity, frame_center, out));
}

int rg_destroy(rg_ctx* c)
{
    if (!c) return set_error(RG_ERR_ARG, "null context");
    cudaStreamSynchronize(c->st);
    free_all(c);
    delete c;
    return RG_OK;
}

int rg_set_integrator(rg_ctx* c, int type, double dt_day, int adaptive, double tolerance, int error_check_for_tp)
{
    if (!c || !(dt_day == dt_day)) return set_error(RG_ERR_ARG, "bad argument");
    switch (type) {
    case RG_INT_EULER: c->r_max = 1; c->order = 1; adaptive = 0; break;
    case RG_INT_RK4: c->r_max = adaptive ? 5 : 4; c->order = 4; break;
    case RG_INT_RK5: c->r_max = 6; c->order = 5; break;
    case RG_INT_RKF78: c->r_max = adaptive ? 13 : 11; c->order = 7; break;
    default: return set_error(RG_ERR_ARG, "Requested integrator is not implemented.");
    }
    c->int_type = type;
    c->adaptive = adaptive ? 1 : 0;
    c->tol = tolerance;
    c->ectp = error_check_for_tp ? 1 : 0;
    c->dt_try = dt_day * GAUSS;  // integrator.cu:29
    c->dt_did = 0.0;
    c->n_failed = c->n_passed = c->n_tried = 0;
    c->has_int = 1;
    return RG_OK;
}

int rg_set_event_options(rg_ctx* c, int close_encounter, int inner_steps, double hill_factor, int event_time_mode)
{
    if (!c || !(hill_factor >= 0.0) || (event_time_mode != RG_EVENT_TIME_CPU && event_time_mode != RG_EVENT_TIME_STAGE))
        return set_error(RG_ERR_ARG, "bad event option");
    c->close_encounter = close_encounter ? 1 : 0;
    c->inner_steps = inner_steps ? 1 : 0;
    c->hill_factor = hill_factor;
    c->event_time_mode = event_time_mode;
    return RG_OK;
}

int rg_set_gravity_mode(rg_ctx* c, int mode)
{
    if (!c || (mode != RG_GRAVITY_FP64 && mode != RG_GRAVITY_MIXED)) return set_error(RG_ERR_ARG, "bad gravity mode");
    if (mode == RG_GRAVITY_MIXED && c->frame == RG_FRAME_ASTRO)
        return set_error(RG_ERR_NOT_IMPLEMENTED, "mixed-precision gravity in the astrocentric frame");
    c->gravity_mode = mode;
    return RG_OK;
}

int rg_set_time(rg_ctx* c, double t_day)
{
    if (!c) return set_error(RG_ERR_ARG, "null context");
    c->t = t_day * GAUSS;
    return RG_OK;
}

int rg_step(rg_ctx* c, double* dt_did_day)
{
    if (!c) return set_error(RG_ERR_ARG, "null context");
    int rc;
    try {
        rc = do_step(c);
    } catch (const std::bad_alloc&) {
        rc = set_error(RG_ERR_NOMEM, "host allocation failed");
    }
    if (dt_did_day) *dt_did_day = c->dt_did / GAUSS;
    return rc;
}

int rg_check_for_ejection_hit_centrum(rg_ctx* c, int* n)
{
    if (!c) return set_error(RG_ERR_ARG, "null context");
    RG_GUARD(check_ejection_hit(c, n));
}

int rg_check_for_collision(rg_ctx* c, int* n)
{
    if (!c) return set_error(RG_ERR_ARG, "null context");
    RG_GUARD(check_collision(c, n));
}

int rg_check_for_close_encounter(rg_ctx* c, int* n)
{
    if (!c) return set_error(RG_ERR_ARG, "null context");
    RG_GUARD(check_close_encounter(c, n));
}

int rg_check_for_rebuild_vectors(rg_ctx* c, int n, int* rebuilt)
{
    if (!c) return set_error(RG_ERR_ARG, "null context");
    RG_GUARD(check_rebuild(c, n, rebuilt));
}

static int advance_impl(rg_ctx* c, double t_stop_day, int64_t max_steps, int64_t* n_steps)
{
    if (!c->has_int) return set_error(RG_ERR_STATE, "no integrator set (rg_set_integrator)");
    const double stop = t_stop_day * GAUSS;
    int64_t k = 0;
    int rc = RG_OK;
    while (c->t <= stop && (max_steps <= 0 || k < max_steps)) {  // main.cu:176-263
        rc = check_ejection_hit(c, nullptr);
        if (rc) break;
        rc = do_step(c);
        if (rc) break;
        k++;
        rc = handle_hill(c);
        if (rc) break;
        if (c->close_encounter && c->inner_steps) {
            if (0.0 < c->thr[RG_THRESHOLD_RADII_ENHANCE_FACTOR]) rc = check_close_encounter(c, nullptr);
        } else if (!c->close_encounter && c->inner_steps) {
            if (0.0 < c->thr[RG_THRESHOLD_RADII_ENHANCE_FACTOR]) rc = check_collision(c, nullptr);
            if (!rc) rc = check_rebuild(c, 8, nullptr);
        }
        if (rc) break;
        if (!std::isfinite(c->dt_try) || c->dt_try == 0.0) {
            rc = set_error(RG_ERR_DT_NONFINITE, "the step-size controller produced a non-finite or zero step");
            break;
        }
    }
    if (n_steps) *n_steps = k;
    return rc;
}

int rg_advance(rg_ctx* c, double t_stop_day, int64_t max_steps, int64_t* n_steps)
{
    if (!c) return set_error(RG_ERR_ARG, "null context");
    RG_GUARD(advance_impl(c, t_stop_day, max_steps, n_steps));
}

int rg_events(rg_ctx* c, rg_event_t* out, int cap, int* n)
{
    if (!c || !n || cap < 0 || (cap > 0 && !out)) return set_error(RG_ERR_ARG, "bad argument");
    const int m = std::min<int>((int)c->log.size(), cap);
    if (m > 0) std::memcpy(out, c->log.data(), (size_t)m * sizeof(rg_event_t));
    c->log.erase(c->log.begin(), c->log.begin() + m);
    *n = m;
    return RG_OK;
}

int rg_event_count(rg_ctx* c, int* n)
{
    if (!c || !n) return set_error(RG_ERR_ARG, "bad argument");
    *n = (int)c->log.size();
    return RG_OK;
}

int rg_get_n_total(rg_ctx* c, rg_counts_t* n, int* n_total)
{
    if (!c) return set_error(RG_ERR_ARG, "null context");
    if (n) {
        n->n_s = c->cnt[0];
        n->n_gp = c->cnt[1];
        n->n_rp = c->cnt[2];
        n->n_pp = c->cnt[3];
        n->n_spl = c->cnt[4];
        n->n_pl = c->cnt[5];
        n->n_tp = c->cnt[6];
    }
    if (n_total) *n_total = c->n_total();
    return RG_OK;
}

static int get_state_impl(rg_ctx* c, rg_vec_t* r, rg_vec_t* v, rg_param_t* p, rg_body_metadata_t* md, bool file_units)
{
    const int n = c->n_total();
    if ((r || v) && n > 0) {  // records built on the device, one copy per array
        double* dr = c->d_records;
        double* dv = c->d_records + (size_t)4 * n;
        int rc = launch_rows_to_records(c->d_y, n, c->cap, GAUSS, file_units, dr, dv, c->st);  // pp_disk.cu:1720-1722
        if (rc) return rc;
        if (r) RG_CUDA_CHECK(cudaMemcpyAsync(r, dr, (size_t)n * sizeof(rg_vec_t), cudaMemcpyDeviceToHost, c->st));
        if (v) RG_CUDA_CHECK(cudaMemcpyAsync(v, dv, (size_t)n * sizeof(rg_vec_t), cudaMemcpyDeviceToHost, c->st));
        RG_CUDA_CHECK(cudaStreamSynchronize(c->st));
    }
    if (p) std::memcpy(p, c->p.data(), (size_t)n * sizeof(rg_param_t));
    if (md) std::memcpy(md, c->md.data(), (size_t)n * sizeof(rg_body_metadata_t));
    return RG_OK;
}

int rg_get_state(rg_ctx* c, rg_vec_t* r, rg_vec_t* v, rg_param_t* p, rg_body_metadata_t* md, double* t_day)
{
    if (!c) return set_error(RG_ERR_ARG, "null context");
    if (t_day) *t_day = c->t / GAUSS;
    RG_GUARD(get_state_impl(c, r, v, p, md, true));
}

int rg_get_state_internal(rg_ctx* c, rg_vec_t* r, rg_vec_t* v, rg_param_t* p, rg_body_metadata_t* md, double* t)
{
    if (!c) return set_error(RG_ERR_ARG, "null context");
    if (t) *t = c->t;
    RG_GUARD(get_state_impl(c, r, v, p, md, false));
}

static int set_state_impl(rg_ctx* c, const rg_vec_t* r, const rg_vec_t* v)
{
    const int n = c->n_total();
    if (n > 0) {  // one copy per array, the rows built on the device (v / k as the host would)
        double* dr = c->d_records;
        double* dv = c->d_records + (size_t)4 * n;
        RG_CUDA_CHECK(cudaMemcpyAsync(dr, r, (size_t)n * sizeof(rg_vec_t), cudaMemcpyHostToDevice, c->st));
        RG_CUDA_CHECK(cudaMemcpyAsync(dv, v, (size_t)n * sizeof(rg_vec_t), cudaMemcpyHostToDevice, c->st));
        const int rc = launch_records_to_rows(dr, dv, n, c->cap, GAUSS, c->d_y, c->st);
        if (rc) return rc;
        RG_CUDA_CHECK(cudaStreamSynchronize(c->st));
    }
    return RG_OK;
}

int rg_set_state(rg_ctx* c, const rg_vec_t* r, const rg_vec_t* v)
{
    if (!c || !r || !v) return set_error(RG_ERR_ARG, "bad argument");
    RG_GUARD(set_state_impl(c, r, v));
}

// CUDA-event time of one force evaluation (stage-0 form, no event recording) over `reps`
static int time_evaluations(rg_ctx* c, int reps, double* ms)
{
    const size_t cap = (size_t)c->cap;
    int rc = gravity(c, c->d_y, c->d_y + 3 * cap, c->d_P, 0, 0, false, false);  // warm-up (plan upload)
    if (rc) return rc;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    RG_CUDA_CHECK(cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return set_error(RG_ERR_CUDA, "cudaEventCreate");
    }
    cudaEventRecord(e0, c->st);
    for (int k = 0; k < reps && !rc; k++) rc = gravity(c, c->d_y, c->d_y + 3 * cap, c->d_P, 0, 0, false, false);
    cudaEventRecord(e1, c->st);
    cudaError_t err = cudaEventSynchronize(e1);
    float t = 0.0f;
    if (!rc && err == cudaSuccess) err = cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    if (err != cudaSuccess) return cuda_fail(err, "autotune timing", __FILE__, __LINE__);
    *ms = (double)t / reps;
    return RG_OK;
}

// Mixed mode tunes in two stages: the row-kernel limit with the current chunking, then the
// mixed kernel's chunk size.  Chunk candidates: for every chunk count n up to 24, the
// smallest whole number of source tiles that gives n chunks and one tile less, so that the
// tuner can pick the grid whose last wave of CTAs is best filled.
static int autotune_impl(rg_ctx* c, int reps, rg_tune_t* out)
{
    struct Shape {
        int S, rowseq, chunk_src;
    };
    const int rows[3] = {32, 64, 128};
    // tuning evaluations leave the counters as they were
    const int64_t evals = c->n_gravity_evals, pairs = c->n_pairs, kernels = c->n_kernels;
    const Shape before{c->pairpar_S, c->rowseq_max_src, c->mixed_chunk_src};
    double ms_before = 0.0, best_ms = 0.0;
    int rc = time_evaluations(c, reps, &ms_before);
    Shape best = before;
    best_ms = ms_before;
    int n_cand = 0;
    auto run = [&](const std::vector<Shape>& cand) {
        for (const Shape& sh : cand) {
            if (rc) break;
            c->pairpar_S = sh.S;
            c->rowseq_max_src = sh.rowseq;
            c->mixed_chunk_src = sh.chunk_src;
            build_tiles(c);
            double ms = 0.0;
            rc = time_evaluations(c, reps, &ms);
            n_cand++;
            if (!rc && ms < best_ms) {
                best_ms = ms;
                best = sh;
            }
        }
        c->pairpar_S = best.S;
        c->rowseq_max_src = best.rowseq;
        c->mixed_chunk_src = best.chunk_src;
        build_tiles(c);
    };
    std::vector<Shape> cand;
    if (c->gravity_mode == RG_GRAVITY_MIXED) {
        for (int r : rows) cand.push_back({c->pairpar_S, r, c->mixed_chunk_src});
        run(cand);
        int src_tiles = 0;  // the largest mixed group's sources, in tiles
        for (const auto& gr : c->plan[1])
            if (gr.kind == GROUP_MIXED)
                src_tiles = std::max(src_tiles, (c->tiles[gr.off].src_end - c->tiles[gr.off].src_begin +
                                                 MIXED_SOURCE_TILE - 1) / MIXED_SOURCE_TILE);
        std::vector<int> ks;
        for (int n = 1; n <= 24 && src_tiles > 0; n++) {
            const int k = (src_tiles + n - 1) / n;
            for (int kk : {k, k - 1})
                if (kk >= 1 && std::find(ks.begin(), ks.end(), kk) == ks.end()) ks.push_back(kk);
        }
        cand.clear();
        cand.push_back({best.S, best.rowseq, 0});
        for (int k : ks) cand.push_back({best.S, best.rowseq, k * MIXED_SOURCE_TILE});
        run(cand);
    } else {
        // sinks per pair-parallel CTA (the astrocentric kernel has 8, 16 and 32), then the
        // row-kernel source limit at the best of them
        std::vector<int> ss = {8, 16, 32};
        if (c->frame != RG_FRAME_ASTRO) ss = {8, 12, 16, 18, 24, 32, 36};
        for (int S : ss) cand.push_back({S, c->rowseq_max_src, c->mixed_chunk_src});
        run(cand);
        cand.clear();
        for (int r : rows) cand.push_back({best.S, r, c->mixed_chunk_src});
        run(cand);
    }
    c->n_gravity_evals = evals;
    c->n_pairs = pairs;
    c->n_kernels = kernels;
    if (rc) return rc;
    if (out) {
        out->pairpar_sinks = best.S;
        out->rowseq_max_src = best.rowseq;
        out->mixed_chunks = best.chunk_src;
        out->candidates = (int32_t)n_cand;
        out->ms_per_eval = best_ms;
        out->ms_before = ms_before;
    }
    return RG_OK;
}

static int calc_accel_impl(rg_ctx* c, rg_vec_t* a)
{
    const size_t cap = (size_t)c->cap;
    const int n = c->n_total();
    int rc = gravity(c, c->d_y, c->d_y + 3 * cap, c->d_P, 0, 0, false, false);
    if (rc) return rc;
    std::vector<double> h((size_t)3 * n);
    if (n > 0)
        RG_CUDA_CHECK(cudaMemcpy2DAsync(h.data(), n * sizeof(double), c->d_P, cap * sizeof(double), n * sizeof(double),
                                        3, cudaMemcpyDeviceToHost, c->st));
    unsigned int flag = 0;
    RG_CUDA_CHECK(cudaMemcpyAsync(&flag, c->d_kerr, sizeof(unsigned int), cudaMemcpyDeviceToHost, c->st));
    RG_CUDA_CHECK(cudaStreamSynchronize(c->st));
    if ((rc = kernel_flag_error(c, flag))) return rc;
    for (int i = 0; i < n; i++) a[i] = rg_vec_t{h[i], h[(size_t)n + i], h[(size_t)2 * n + i], 0.0};
    // astrocentric frame: the star's row is not evaluated (its derivative stays zero)
    if (c->frame == RG_FRAME_ASTRO && n > 0) a[0] = rg_vec_t{0.0, 0.0, 0.0, 0.0};
    return RG_OK;
}

int rg_calc_accel(rg_ctx* c, rg_vec_t* a)
{
    if (!c || !a) return set_error(RG_ERR_ARG, "bad argument");
    RG_GUARD(calc_accel_impl(c, a));
}

int rg_test_hold_tile_copies(rg_ctx* c, int on)
{
    if (!c) return set_error(RG_ERR_ARG, "null context");
    c->hold_tile_copies = on ? 1 : 0;
    return RG_OK;
}

int rg_autotune(rg_ctx* c, int reps, rg_tune_t* out)
{
    if (!c || reps <= 0) return set_error(RG_ERR_ARG, "bad argument");
    RG_GUARD(autotune_impl(c, reps, out));
}

static int set_launch_shape_impl(rg_ctx* c, const rg_tune_t* t)
{
    const int S = t->pairpar_sinks;
    const bool astro = c->frame == RG_FRAME_ASTRO;
    const bool s_ok = astro ? (S == 8 || S == 16 || S == 32)
                            : (S == 8 || S == 12 || S == 16 || S == 18 || S == 24 || S == 32 || S == 36);
    if (!s_ok) return set_error(RG_ERR_ARG, "pairpar_sinks: 8, 12, 16, 18, 24, 32 or 36 (8, 16 or 32 in the "
                                            "astrocentric frame)");
    if (t->rowseq_max_src < 1) return set_error(RG_ERR_ARG, "rowseq_max_src must be positive");
    if (t->mixed_chunks < 0 || t->mixed_chunks % MIXED_SOURCE_TILE != 0)
        return set_error(RG_ERR_ARG, "mixed_chunks: 0 or a positive multiple of 256 sources");
    c->pairpar_S = S;
    c->rowseq_max_src = t->rowseq_max_src;
    c->mixed_chunk_src = t->mixed_chunks;
    build_tiles(c);
    return RG_OK;
}

int rg_set_launch_shape(rg_ctx* c, const rg_tune_t* shape)
{
    if (!c || !shape) return set_error(RG_ERR_ARG, "bad argument");
    RG_GUARD(set_launch_shape_impl(c, shape));
}

int rg_get_counters(rg_ctx* c, rg_counters_t* o)
{
    if (!c || !o) return set_error(RG_ERR_ARG, "bad argument");
    std::memset(o, 0, sizeof(*o));
    o->n_failed_step = c->n_failed;
    o->n_passed_step = c->n_passed;
    o->n_tried_step = c->n_tried;
    for (int i = 0; i < 3; i++) {
        o->n_hit_centrum[i] = c->n_hit_centrum[i];
        o->n_ejection[i] = c->n_ejection[i];
        o->n_collision[i] = c->n_collision[i];
        o->n_close_encounter[i] = c->n_close_encounter[i];
        o->n_event[i] = c->n_event[i];
    }
    o->n_gravity_evals = c->n_gravity_evals;
    o->n_pairs = c->n_pairs;
    o->n_kernels = c->n_kernels;
    return RG_OK;
}

int rg_get_stream(rg_ctx* c, void** stream)
{
    if (!c || !stream) return set_error(RG_ERR_ARG, "bad argument");
    *stream = (void*)c->st;
    return RG_OK;
}

int rg_set_profiling(rg_ctx* c, int on)
{
    if (!c) return set_error(RG_ERR_ARG, "null context");
    c->profiling = on ? 1 : 0;
    return RG_OK;
}

int rg_get_profile(rg_ctx* c, rg_profile_t* prof)
{
    if (!c || !prof) return set_error(RG_ERR_ARG, "bad argument");
    std::memset(prof, 0, sizeof(*prof));
    RG_CUDA_CHECK(cudaStreamSynchronize(c->st));
    for (size_t k = 0; k < c->ev_kind.size(); k++) {
        float ms = 0.0f;
        RG_CUDA_CHECK(cudaEventElapsedTime(&ms, c->ev_pool[2 * k], c->ev_pool[2 * k + 1]));
        if (c->ev_kind[k] == 0) {
            prof->gravity_launches++;
            prof->gravity_ms += ms;
        } else if (c->ev_kind[k] == 1) {
            prof->stage_launches++;
            prof->stage_ms += ms;
        } else {
            prof->other_launches++;
            prof->other_ms += ms;
        }
    }
    c->ev_kind.clear();
    c->ev_used = 0;
    return RG_OK;
}

int rg_measure_pipe_peak(int kind, double* tflops)
{
    if ((kind != 0 && kind != 1) || !tflops) return set_error(RG_ERR_ARG, "bad argument");
    if (rg_device_count() <= 0) return set_error(RG_ERR_NO_DEVICE, "no CUDA device");
    return redgb::measure_pipe_peak(kind, tflops);
}

static int energy_impl(rg_ctx* c, double* energy, double* angmom)
{
    const int n = c->n_total();
    EnergyArgs a{c->d_y, c->d_mass, c->d_id, n, c->n_si(), c->n_massive(), c->cap, c->d_part};
    int rc = launch_energy(a, c->st);
    if (rc) return rc;
    c->n_kernels++;
    std::vector<double> h((size_t)5 * n);
    if (n > 0)
        RG_CUDA_CHECK(cudaMemcpyAsync(h.data(), c->d_part, h.size() * sizeof(double), cudaMemcpyDeviceToHost, c->st));
    RG_CUDA_CHECK(cudaStreamSynchronize(c->st));
    double s[5], cc[5];
    for (int q = 0; q < 5; q++) {  // Neumaier sums in body order
        s[q] = 0.0;
        cc[q] = 0.0;
        for (int i = 0; i < n; i++) {
            const double x = h[(size_t)q * n + i];
            const double t = s[q] + x;
            if (std::fabs(s[q]) >= std::fabs(x))
                cc[q] += (s[q] - t) + x;
            else
                cc[q] += (x - t) + s[q];
            s[q] = t;
        }
    }
    if (energy) *energy = (s[0] + cc[0]) + (s[1] + cc[1]);
    if (angmom) {
        angmom[0] = s[2] + cc[2];
        angmom[1] = s[3] + cc[3];
        angmom[2] = s[4] + cc[4];
    }
    return RG_OK;
}

int rg_energy(rg_ctx* c, double* energy, double angmom[3])
{
    if (!c) return set_error(RG_ERR_ARG, "null context");
    RG_GUARD(energy_impl(c, energy, angmom));
}

int rg_get_dt(rg_ctx* c, double* dt_did_day, double* dt_try_day)
{
    if (!c) return set_error(RG_ERR_ARG, "null context");
    if (dt_did_day) *dt_did_day = c->dt_did / GAUSS;
    if (dt_try_day) *dt_try_day = c->dt_try / GAUSS;
    return RG_OK;
}

}  // extern "C"
