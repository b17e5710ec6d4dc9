// ens_events.cu -- the ensemble's event handling on the device, so that attempts run back to
// back without the host (one graph launch per rg_ens_advance).
//
// After every attempt, one thread per disk applies the reference's handlers to its disk:
//  * ens_hill_kernel (after the step-start force evaluation): the pairs found inside their
//    mutual Hill spheres, in body order, are logged when they were not inside at the previous
//    step start (the set of pairs is kept per disk);
//  * ens_handle_kernel (after the step-size controller, for disks whose accepted attempt
//    recorded a collision or left a body beyond the ejection or hit-star radius): the raw
//    collision records in the reference's order become event records, one per pair (the
//    earliest, pp_disk.cu:1111-1149), and each merges its pair (pp_disk.cu:1151-1202,
//    tools.cpp:263-290); then the ejection / hit-star check of the new state
//    (pp_disk.cu:934-976,1091-1109) retires and merges bodies; the disk is released;
//  * ens_loop_kernel: the loop condition -- another attempt while a disk is running, no
//    error bit is set, and neither the caller's attempt limit nor the end of the launch's
//    chunk of attempts is reached (every graph launch is bounded; the host launches the next
//    chunk while disks are running).
//
// The records are the single-disk path's (context.cu) field for field.  One difference from
// the reference: a merged body's radius, pow(3 m / (4 pi rho), 1/3) (tools.cpp:238-243), is
// the device's pow, which may differ from glibc's in the last bit, as the ensemble's step-size
// controller already does (its trial steps use the device's pow).
//
// Built with -fmad=false: the merge formulas keep the reference's operation order.
#include "ens_events.h"

namespace redgb {

namespace {

__device__ __forceinline__ long long pair_key(int id1, int id2)
{
    return ((long long)(unsigned int)id1 << 32) | (long long)(unsigned int)id2;
}

// the record's place in the reference's order: (attempt << 8 | stage, sink, source)
__device__ __forceinline__ bool rec_before(const DevEvent& a, const DevEvent& b)
{
    if (a.seq != b.seq) return a.seq < b.seq;
    if (a.i != b.i) return a.i < b.i;
    return a.j < b.j;
}

__device__ rg_event_t* log_slot(const EnsEventArgs& a, int s)
{
    const unsigned int slot = atomicAdd(a.log_count, 1u);
    if (slot >= a.log_cap) {
        atomicOr(a.flags, ENS_FLAG_LOG_OVERFLOW);
        return nullptr;
    }
    EnsLogRec& r = a.log[slot];
    r.sys = s;
    r.seqno = (int)a.log_seq[s]++;
    r.pad = 0;
    rg_event_t* e = &r.ev;
    memset(e, 0, sizeof(*e));
    return e;
}

__device__ __forceinline__ rg_vec_t row_vec(const EnsEventArgs& a, int row0, int i)
{
    return rg_vec_t{a.y[row0 * a.stride + i], a.y[(row0 + 1) * a.stride + i], a.y[(row0 + 2) * a.stride + i], 0.0};
}

__device__ __forceinline__ void set_state(const EnsEventArgs& a, int i, const rg_vec_t& r, const rg_vec_t& v)
{
    a.y[i] = r.x;
    a.y[a.stride + i] = r.y;
    a.y[2 * a.stride + i] = r.z;
    a.y[3 * a.stride + i] = v.x;
    a.y[4 * a.stride + i] = v.y;
    a.y[5 * a.stride + i] = v.z;
}

__device__ __forceinline__ void set_param(const EnsEventArgs& a, int i, const rg_param_t& p)
{
    a.prm[i] = p;
    a.mass[i] = p.mass;
    a.radius[i] = p.radius;
}

// pp_disk::handle_collision_pair (pp_disk.cu:1151-1202) with tools.cpp:263-290 on a record
// whose idx fields are disk-relative; false for a super-planetesimal (the reference throws)
__device__ bool merge_pair(const EnsEventArgs& a, int b, rg_event_t* c)
{
    const int surv = c->idx1 + b, merg = c->idx2 + b;
    if (a.type[merg] == RG_BODY_SUPERPLANETESIMAL) return false;
    c->p1 = a.prm[surv];
    c->p2 = a.prm[merg];
    const double m1 = c->p1.mass, m2 = c->p2.mass;
    const double M = m1 + m2;
    c->rs = rg_vec_t{(m1 * c->r1.x + m2 * c->r2.x) / M, (m1 * c->r1.y + m2 * c->r2.y) / M,
                     (m1 * c->r1.z + m2 * c->r2.z) / M, 0.0};
    c->vs = rg_vec_t{(m1 * c->v1.x + m2 * c->v2.x) / M, (m1 * c->v1.y + m2 * c->v2.y) / M,
                     (m1 * c->v1.z + m2 * c->v2.z) / M, 0.0};
    set_state(a, surv, c->rs, c->vs);
    const double R1 = c->p1.radius, R2 = c->p2.radius;
    const double volume = 4.188790204786391 * (R1 * R1 * R1 + R2 * R2 * R2);
    rg_param_t ps;
    ps.mass = m1 + m2;
    ps.density = ps.mass / volume;
    ps.radius = pow(1.0 / 4.1887902047863909846168578443727 * ps.mass / ps.density, 1.0 / 3.0);
    ps.cd = c->p1.cd;
    c->ps = ps;
    set_param(a, surv, ps);
    a.id[merg] = -a.id[merg];
    rg_param_t pm = a.prm[merg];
    pm.mass = 0.0;
    pm.density = 0.0;
    pm.radius = 0.0;
    set_param(a, merg, pm);
    set_state(a, merg, rg_vec_t{1.0e20, 0.0, 0.0, 0.0}, rg_vec_t{0.0, 0.0, 0.0, 0.0});
    return true;
}

// the raw collision record d as an event record (pp_disk.cu:262-296 with the CPU path's
// times, pp_disk.cu:576,581), with the orientation and ids fixed by orient_records
__device__ void raw_to_event(const EnsEventArgs& a, int s, const DevEvent& d, rg_event_t* x)
{
    const int b = a.base[s];
    const int stage = (int)(d.seq & 0xff);
    const double curr_t = a.t_prev[s] + a.stage_c[stage] * a.dt_did[s];
    x->t = (d.i - b >= a.nsi[s]) ? a.t_prev[s] : curr_t;
    x->d = d.d;
    x->event_name = RG_EVENT_COLLISION;
    const int surv = d.swap ? d.j : d.i, merg = d.swap ? d.i : d.j;
    const double *rs = d.swap ? d.rj : d.ri, *vs = d.swap ? d.vj : d.vi;
    const double *rm = d.swap ? d.ri : d.rj, *vm = d.swap ? d.vi : d.vj;
    x->id1 = d.id1;
    x->id2 = d.id2;
    x->idx1 = surv - b;
    x->idx2 = merg - b;
    x->r1 = rg_vec_t{rs[0], rs[1], rs[2], 0.0};
    x->v1 = rg_vec_t{vs[0], vs[1], vs[2], 0.0};
    x->r2 = rg_vec_t{rm[0], rm[1], rm[2], 0.0};
    x->v2 = rg_vec_t{vm[0], vm[1], vm[2], 0.0};
}

__device__ __forceinline__ bool mine(const EnsEventArgs& a, int s, const DevEvent& d)
{
    return d.sys == s && d.kind == 0 && (d.seq >> 8) == a.acc_attempt[s];
}

}  // namespace

// ------------------------------------------------------------------- Hill-sphere records
constexpr int HILL_LOCAL = 48;  // a disk's records gathered in one pass (more: repeated scans)

__device__ void log_hill(const EnsEventArgs& a, int s, int b, const DevEvent& d, const long long* prev, int n_prev,
                         long long* next, int& n_next)
{
    const long long key = pair_key(a.id[d.i], a.id[d.j]);
    bool seen = false;
    for (int q = 0; q < n_prev && !seen; q++) seen = prev[q] == key;
    if (!seen) {
        rg_event_t* x = log_slot(a, s);
        if (x) {
            x->event_name = RG_EVENT_CLOSE_ENCOUNTER;
            x->t = d.t;  // the step start, where the pair was found inside the sphere
            x->d = d.d;
            x->id1 = a.id[d.i];
            x->id2 = a.id[d.j];
            x->idx1 = d.i - b;
            x->idx2 = d.j - b;
            x->p1 = a.prm[d.i];
            x->p2 = a.prm[d.j];
            x->r1 = rg_vec_t{d.ri[0], d.ri[1], d.ri[2], 0.0};
            x->v1 = rg_vec_t{d.vi[0], d.vi[1], d.vi[2], 0.0};
            x->r2 = rg_vec_t{d.rj[0], d.rj[1], d.rj[2], 0.0};
            x->v2 = rg_vec_t{d.vj[0], d.vj[1], d.vj[2], 0.0};
        }
    }
    if (n_next < a.hill_set_cap)
        next[n_next++] = key;
    else
        atomicOr(a.flags, ENS_FLAG_HILL_SET);
}

// one CTA per disk: its threads scan the step start's Hill records together and gather the
// disk's (at most HILL_LOCAL of them; a disk with more repeats the scan for the rest, one
// record at a time), then one thread logs them in (sink, source) order
constexpr int HILL_THREADS = 64;

__global__ void __launch_bounds__(HILL_THREADS) ens_hill_kernel(EnsEventArgs a)
{
    const int s = blockIdx.x;
    if (!a.active_f0[s]) return;  // uniform over the CTA
    __shared__ long long key[HILL_LOCAL];
    __shared__ unsigned int idx[HILL_LOCAL];
    __shared__ int m_sh;
    if (threadIdx.x == 0) m_sh = 0;
    __syncthreads();
    const unsigned int n = min(*a.hill_count, a.ev_cap);
    for (unsigned int k = threadIdx.x; k < n; k += HILL_THREADS) {
        const DevEvent& d = a.hill[k];
        if (d.sys != s || d.kind != 1) continue;
        const int p = atomicAdd(&m_sh, 1);
        if (p < HILL_LOCAL) {
            key[p] = ((long long)d.i << 32) | (long long)(unsigned int)d.j;
            idx[p] = k;
        }
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    const int m = m_sh;
    const int b = a.base[s];
    const int cur = a.hill_which[s];
    const long long* prev = a.hill_set + ((long long)s * 2 + cur) * a.hill_set_cap;
    long long* next = a.hill_set + ((long long)s * 2 + (cur ^ 1)) * a.hill_set_cap;
    const int n_prev = a.hill_n[s];
    int n_next = 0;
    if (m <= HILL_LOCAL) {
        // the gathered records in (sink, source) order (the keys are distinct)
        for (int q = 1; q < m; q++) {
            const long long kk = key[q];
            const unsigned int kx = idx[q];
            int p = q;
            while (p > 0 && key[p - 1] > kk) {
                key[p] = key[p - 1];
                idx[p] = idx[p - 1];
                p--;
            }
            key[p] = kk;
            idx[p] = kx;
        }
        for (int q = 0; q < m; q++) log_hill(a, s, b, a.hill[idx[q]], prev, n_prev, next, n_next);
    } else {
        // repeatedly the smallest key above the last
        long long last = -1;
        for (;;) {
            long long best = 0x7fffffffffffffffll;
            unsigned int bk = 0xffffffffu;
            for (unsigned int k = 0; k < n; k++) {
                const DevEvent& d = a.hill[k];
                if (d.sys != s || d.kind != 1) continue;
                const long long kk = ((long long)d.i << 32) | (long long)(unsigned int)d.j;
                if (kk > last && kk < best) {
                    best = kk;
                    bk = k;
                }
            }
            if (bk == 0xffffffffu) break;
            last = best;
            log_hill(a, s, b, a.hill[bk], prev, n_prev, next, n_next);
        }
    }
    a.hill_n[s] = n_next;
    a.hill_which[s] = cur ^ 1;
}

// ------------------------------------------------------------------- collisions, ejections
__global__ void ens_handle_kernel(EnsEventArgs a, int initial)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= a.n_sys) return;
    if (initial ? !a.ej[s] : a.status[s] != RG_SYS_HELD) return;
    const int b = a.base[s], n = a.ntot[s];
    if (!initial) {
        const unsigned int nr = min(*a.ev_count, a.ev_cap);
        DevEvent* ev = const_cast<DevEvent*>(a.ev);
        // every record's survivor (the heavier body) and ids, from the state before any merge,
        // as the reference builds its whole list before handling a record (pp_disk.cu:717-738)
        for (unsigned int k = 0; k < nr; k++) {
            DevEvent& d = ev[k];
            if (!mine(a, s, d)) continue;
            d.swap = a.prm[d.j].mass > a.prm[d.i].mass ? 1 : 0;
            d.id1 = a.id[d.swap ? d.j : d.i];
            d.id2 = a.id[d.swap ? d.i : d.j];
        }
        // the distinct pairs in the order of their first record; of each pair the earliest
        // record merges (pp_disk.cu:1111-1149: a later record replaces an earlier one only
        // with a strictly smaller time)
        int last = -1;
        for (;;) {
            int bk = -1;
            for (unsigned int k = 0; k < nr; k++) {
                const DevEvent& d = ev[k];
                if (!mine(a, s, d)) continue;
                if (last >= 0 && !rec_before(ev[last], d)) continue;
                if (bk < 0 || rec_before(d, ev[bk])) bk = (int)k;
            }
            if (bk < 0) break;
            last = bk;
            const DevEvent& first_rec = ev[bk];
            bool first = true;
            for (unsigned int k = 0; k < nr && first; k++) {
                const DevEvent& d = ev[k];
                if ((int)k != bk && mine(a, s, d) && rec_before(d, first_rec) && d.id1 == first_rec.id1 &&
                    d.id2 == first_rec.id2)
                    first = false;
            }
            if (!first) continue;
            rg_event_t cur;
            memset(&cur, 0, sizeof(cur));
            raw_to_event(a, s, first_rec, &cur);
            // later records of the pair, in order
            int lk = bk;
            for (;;) {
                int nk = -1;
                for (unsigned int k = 0; k < nr; k++) {
                    const DevEvent& d = ev[k];
                    if (!mine(a, s, d) || d.id1 != first_rec.id1 || d.id2 != first_rec.id2) continue;
                    if (!rec_before(ev[lk], d)) continue;
                    if (nk < 0 || rec_before(d, ev[nk])) nk = (int)k;
                }
                if (nk < 0) break;
                lk = nk;
                rg_event_t x;
                memset(&x, 0, sizeof(x));
                raw_to_event(a, s, ev[nk], &x);
                if (cur.t > x.t) cur = x;
            }
            rg_event_t* out = log_slot(a, s);
            rg_event_t tmp;
            rg_event_t* c = out ? out : &tmp;
            *c = cur;
            if (!merge_pair(a, b, c)) atomicOr(a.flags, ENS_FLAG_SUPERPLANETESIMAL);
        }
    }
    // ejection / hit-star check of the new state (pp_disk.cu:934-976,1091-1109): the record of
    // every body beyond a radius first, in body order, from the state after the merges above;
    // then the hit-star merges in that order
    const double* th = a.thr + RG_THRESHOLD_N * s;
    unsigned int* hits = a.hit_slots + (long long)s * a.hit_cap;
    int n_hit = 0;
    for (int i = b; i < b + n; i++) {
        if (!(0 < a.id[i] && RG_BODY_STAR != a.type[i])) continue;
        const rg_vec_t ri = row_vec(a, 0, i);
        const double r2 = ri.x * ri.x + ri.y * ri.y + ri.z * ri.z;
        int name = 0;
        if (0.0 < th[1] && th[4] < r2)
            name = RG_EVENT_EJECTION;
        else if (0.0 < th[0] && th[3] > r2)
            name = RG_EVENT_HIT_CENTRUM;
        if (!name) continue;
        const unsigned int slot = atomicAdd(a.log_count, 1u);
        a.id[i] = -a.id[i];
        if (slot >= a.log_cap) {
            atomicOr(a.flags, ENS_FLAG_LOG_OVERFLOW);
            continue;
        }
        EnsLogRec& lr = a.log[slot];
        lr.sys = s;
        lr.seqno = (int)a.log_seq[s]++;
        lr.pad = 0;
        rg_event_t* x = &lr.ev;
        memset(x, 0, sizeof(*x));
        x->event_name = name;
        x->d = sqrt(r2);
        x->t = a.t[s];
        x->id1 = a.id[b];
        x->id2 = -a.id[i];
        x->idx1 = 0;
        x->idx2 = i - b;
        x->r1 = row_vec(a, 0, b);
        x->v1 = row_vec(a, 3, b);
        x->r2 = ri;
        x->v2 = row_vec(a, 3, i);
        if (name == RG_EVENT_EJECTION) {
            x->p1 = a.prm[b];
            x->p2 = a.prm[i];
            x->rs = x->r1;
            x->vs = x->v1;
            x->ps = x->p1;
        } else if (n_hit < a.hit_cap) {
            hits[n_hit++] = slot;
        } else {
            atomicOr(a.flags, ENS_FLAG_HIT_OVERFLOW);
        }
    }
    for (int q = 0; q < n_hit; q++)
        if (!merge_pair(a, b, &a.log[hits[q]].ev)) atomicOr(a.flags, ENS_FLAG_SUPERPLANETESIMAL);
    a.ej[s] = 0;
    const bool run = a.t[s] <= a.t_stop[s];
    a.status[s] = run ? RG_SYS_RUNNING : RG_SYS_DONE;
    a.active[s] = run;
    a.active_f0[s] = run;
}

// ------------------------------------------------------------------- loop condition
__global__ void ens_loop_kernel(EnsLoopArgs a)
{
    __shared__ int any_run, any_err;
    if (threadIdx.x == 0) {
        any_run = 0;
        any_err = 0;
    }
    __syncthreads();
    for (int s = threadIdx.x; s < a.n_sys; s += blockDim.x) {
        if (a.status[s] == RG_SYS_RUNNING) any_run = 1;
        if (a.status[s] == RG_SYS_ERROR) any_err = 1;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        if (*a.ev_count > a.ev_cap) atomicOr(a.flags, ENS_FLAG_EVENT_OVERFLOW);
        if (*a.hill_count > a.ev_cap) atomicOr(a.flags, ENS_FLAG_HILL_OVERFLOW);
        if (a.step_log_count && *a.step_log_count > a.step_log_cap) atomicOr(a.flags, ENS_FLAG_STEP_LOG_OVERFLOW);
        const long long done = ++a.attempts[0];
        const bool err = any_err || *a.flags != 0u || *a.kerr != 0u;
        const bool limit = (a.attempts[1] > 0 && done >= a.attempts[1]) || done >= a.attempts[2];
        const int keep = any_run && !err && !limit;
        *a.keep = keep;
        *a.ev_count = 0u;
        *a.hill_count = 0u;
        if (a.use_cond) cudaGraphSetConditional(a.cond, keep ? 1u : 0u);
    }
}

int launch_ens_hill(const EnsEventArgs& a, cudaStream_t st)
{
    if (a.n_sys <= 0) return 0;
    ens_hill_kernel<<<a.n_sys, HILL_THREADS, 0, st>>>(a);
    RG_CUDA_CHECK(cudaGetLastError());
    return 0;
}

int launch_ens_handle(const EnsEventArgs& a, int initial, cudaStream_t st)
{
    ens_handle_kernel<<<(a.n_sys + 63) / 64, 64, 0, st>>>(a, initial);
    RG_CUDA_CHECK(cudaGetLastError());
    return 0;
}

int launch_ens_loop(const EnsLoopArgs& a, cudaStream_t st)
{
    ens_loop_kernel<<<1, 256, 0, st>>>(a);
    RG_CUDA_CHECK(cudaGetLastError());
    return 0;
}

}  // namespace redgb
