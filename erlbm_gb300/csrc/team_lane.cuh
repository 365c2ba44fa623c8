// team_lane.cuh -- the request server's resident team loop (server.cu): mixed-size lattices admitted
// on the device by HBM footprint and stepped by the CTAs of one persistent launch.
//
// The reference has no serving path.  This lane takes the lattices too large for one CTA's shared
// memory, up to the server's team_max_nodes (by default D2Q9 Taylor-Green up to 512^2, D3Q19
// Taylor-Green up to 64^3, the obstacle channels scaled by more than 1), and runs them with no host
// launch per run or per step.  One launch per precision stays resident while it has work:
//
//  admitter  thread 0 of the CTA that wins the election.  It claims requests from a ring in mapped
//            pinned memory as the host publishes them, keeps up to TEAM_PEND of them waiting, and
//            admits them shortest estimated run first with aging (an entry's key is its estimate
//            minus the time it has waited).  A request is admitted when one of max_jobs run slots is
//            free and its buffers fit in the arena: a bitmap of TEAM_PAGE pages shared by both
//            precisions' launches, claimed with CAS.  The first request that does not fit stops the
//            pass, so memory frees up for it.
//  workers   every other CTA.  A run is a sequence of work items: the copy of its tables and solid
//            mask from the ring, the initial state in chunks of nodes, each step in the same chunks,
//            the final kinetic energy per node in chunks, its partial sums, the final sum.  A free
//            CTA joins the run with the fewest CTAs for its size, and its members take the next item
//            from the run's counter (claiming it while the previous one runs) until none is left.
//            An item waits until every item of the previous phases is done, which is the step
//            barrier.  When admitted runs have no member, as many CTAs leave runs that have other
//            members, so small runs admitted behind large ones start at once.  The CTA that finishes the last
//            item publishes the result; the last member out frees the pages.
//
// Results do not depend on how many CTAs work on a run, nor on the mix: each node's update reads only
// the previous step, the density check folds with max / or / min, and the energy sum has a fixed
// shape (serial in fluid order up to 65536 nodes, else 1024 blocks of 256 strided partial sums and a
// 256-wide tree, as launch_sum).  They equal the stream lane's bit for bit.
//
// Every wait is bounded: free CTAs leave when the admitter has left or its heartbeat is older than the
// idle limit; the admitter leaves after the idle limit without work; an item that waits longer than
// sync_ns for the previous phase marks the run failed (TeamDone.status TEAM_TIMEOUT, reported to the
// caller as ERLBM_E_TIMEOUT) and goes on without it, so the run still ends.
// Buffers that the launch rewrites (populations, energies, the payload copies) are read with
// L2-coherent loads, the host's ring memory with uncached ones.
#pragma once

#include <climits>
#include <cstdint>

#include "lattice_kernels.cuh"

namespace erlbm {

// threads per CTA (a quarter of an SM's registers at the kernels' 128 registers per thread, so that
// both precisions' loops and a slot loop's CTA fit on one SM)
template <class P>
constexpr int team_threads() { return 128; }
constexpr int TEAM_RB = 256;             // threads of a reduction block of launch_sum (two per CTA thread)
constexpr int TEAM_RG = 1024;            // reduction blocks of launch_sum
constexpr int TEAM_RG_ITEM = 8;          // reduction blocks per work item
constexpr int TEAM_COPY = 8192;          // payload bytes per work item
constexpr long long TEAM_SERIAL = 1 << 16;  // up to this many fluid nodes the energy is summed serially
constexpr int TEAM_MAX_JOBS = 64;
constexpr int TEAM_MAX_GRID = 4096;
constexpr int TEAM_PEND = 64;
constexpr long long TEAM_PAGE = 1LL << 20;  // arena page
constexpr int TEAM_TIMEOUT = 16;            // TeamDone.status: a wait for the previous phase gave up
constexpr int TEAM_CLOSED = 1 << 30;        // TeamJob.members: no item left to hand out

// One request, written by the host before it publishes the ring tail.  Offsets are bytes from the
// run's first page.  The payload (tab_len doubles at 0, solid_len bytes at pay_solid, one int per
// fluid node at pay_nof when solid_len > 0; pay_bytes in all, a multiple of 16) sits in the entry's
// slot of mapped host memory until the result is collected; the run's first items copy it to
// off_pay.
struct TeamEntry {
    CollParams prm;
    double u0, tau, k;
    long long est_ns;
    long long off_buf1, off_scr, off_pay, pay_solid, pay_nof, pay_bytes;
    int q, op, init, n_steps;  // init: 1 D2Q9 Taylor-Green, 4 D3Q19 Taylor-Green, 0 rest
    int nx, ny, nz, n_fluid;
    int check_density, inlet_x, outlet_x, chunk;  // chunk: nodes per work item
    int pages, tab_len, solid_len, pad;
};

// Result of one request, written by the device; seq (ring index + 1) is published last.
struct TeamDone {
    double energy, margin;
    long long t_admit_ns, t_done_ns;
    int label, steps_done, decided_step, status;
    int peak_members, seq, pad[2];
};

// An admitted run (device memory).
struct TeamJob {
    TeamEntry e;
    char *base;
    RunStatus status;
    double energy;
    long long t_admit_ns;
    unsigned long long next, done;  // work items handed out, finished
    long long total;                // work items of the run
    int ring_idx, page0, c_items, n_chunks, f_chunks, e2_items, want;
    int members;                    // CTAs in the run, | TEAM_CLOSED once every item is handed out
    int error, peak, pad;
};

// Control words of one launch (device memory, zeroed before each launch).
struct TeamCtl {
    int admitter;         // blockIdx + 1 of the elected admitter, 0 before
    int closing;          // the admitter has left; free CTAs leave too
    int live, pad;        // worker CTAs in the launch
    long long heartbeat;  // the admitter's clock (ns) at its last pass
};

// State kept across launches (device memory, zeroed once): claimed requests not yet admitted, and
// the admitted runs, which a later launch carries on when a launch leaves with runs unfinished.
struct TeamQueue {
    int head;  // next ring entry to claim
    int n;
    int idx[TEAM_PEND];
    long long claim_ns[TEAM_PEND], est_ns[TEAM_PEND];
    int active, hungry;            // admitted runs not yet freed; of those, runs with no member
    int rescuers, pad;             // CTAs that left a run to join a hungry one and have not joined yet
    int job_state[TEAM_MAX_JOBS];  // 0 free, 1 admitted
};

struct TeamRing {
    const int *tail, *stop;         // host-mapped: entries published; 1 = leave
    const TeamEntry *entries;       // host-mapped ring of `capacity` entries
    const unsigned char *payload;   // host-mapped: payload_stride bytes per entry
    TeamDone *done;                 // host-mapped ring of results
    long long payload_stride;
    int capacity, max_jobs;
    TeamQueue *queue;
    TeamCtl *ctl;
    TeamJob *jobs;
    unsigned *pages;                // arena page bitmap (1 = used), shared by both precisions
    char *arena;                    // page 0
    int n_pages, pad;
    long long idle_ns, sync_ns;
};

int launch_team_server_fp64(const TeamRing &r, int grid, cudaStream_t s);
int launch_team_server_fp32(const TeamRing &r, int grid, cudaStream_t s);
int team_server_occupancy_fp64();
int team_server_occupancy_fp32();
// device clock (globaltimer, ns) into *out (device or mapped memory)
int launch_team_clock(long long *out, cudaStream_t s);

#ifdef __CUDACC__
namespace team {

__device__ __forceinline__ long long now_ns()
{
    long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ int ld_acq_gpu(const int *p)
{
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ unsigned long long ld_acq_gpu64(const unsigned long long *p)
{
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_rel_gpu(int *p, int v)
{
    asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ int ld_acq_sys(const int *p)
{
    int v;
    asm volatile("ld.acquire.sys.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_rel_sys(int *p, int v)
{
    asm volatile("st.release.sys.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ unsigned run_mask(int lo, int hi)
{
    return (hi == 32 ? 0xffffffffu : ((1u << hi) - 1u)) & ~((1u << lo) - 1u);
}

// First fit of n contiguous free pages; returns the first page, or -1.  Each word of the run is
// claimed with CAS (the other precision's admitter allocates from the same bitmap); on a conflict the
// words claimed so far are released and -1 returned, to be tried again on a later pass.
static __device__ int pages_claim(unsigned *bits, int n_pages, int n)
{
    if (n <= 0 || n > n_pages) return -1;
    int start = -1, run = 0;
    for (int p = 0; p < n_pages && run < n; p++) {
        const unsigned w = __ldcg(bits + (p >> 5));
        if (w & (1u << (p & 31))) {
            run = 0;
            start = -1;
        } else {
            if (run == 0) start = p;
            run++;
        }
    }
    if (run < n) return -1;
    int claimed_to = start;  // pages [start, claimed_to) are ours
    for (int p = start; p < start + n;) {
        const int w = p >> 5, lo = p & 31, hi = min(32, lo + (start + n - p));
        const unsigned mask = run_mask(lo, hi);
        bool ok = false;
        for (int tries = 0; tries < 16 && !ok; tries++) {
            const unsigned old = __ldcg(bits + w);
            if (old & mask) break;
            ok = atomicCAS(bits + w, old, old | mask) == old;
        }
        if (!ok) {
            for (int q = start; q < claimed_to;) {
                const int w2 = q >> 5, lo2 = q & 31, hi2 = min(32, lo2 + (claimed_to - q));
                atomicAnd(bits + w2, ~run_mask(lo2, hi2));
                q += hi2 - lo2;
            }
            return -1;
        }
        p += hi - lo;
        claimed_to = p;
    }
    return start;
}

static __device__ void pages_free(unsigned *bits, int start, int n)
{
    for (int p = start; p < start + n;) {
        const int w = p >> 5, lo = p & 31, hi = min(32, lo + (start + n - p));
        atomicAnd(bits + w, ~run_mask(lo, hi));
        p += hi - lo;
    }
}

// Work items of a run, in order: kCOPY (c_items: the payload into the run's pages), kINIT (n_chunks),
// kSTEP (n_steps x n_chunks), kENERGY (f_chunks), kPARTIAL (e2_items: 1 serial sum, or 128 items of 8
// reduction blocks), kFINAL (0 or 1).
enum ItemKind : int { kCOPY = 5, kINIT = 0, kSTEP = 1, kENERGY = 2, kPARTIAL = 3, kFINAL = 4 };

struct Item {
    int kind, step, chunk;
    long long start;  // first item of the phase this one belongs to
};

__device__ __forceinline__ Item item_of(long long k, int c_items, int n_chunks, int f_chunks, int e2_items,
                                        int n_steps)
{
    Item it;
    const long long nc = n_chunks;
    if (k < c_items) {
        it.kind = kCOPY;
        it.step = 0;
        it.chunk = (int)k;
        it.start = 0;
        return it;
    }
    k -= c_items;
    if (k < nc) {
        it.kind = kINIT;
        it.step = 0;
        it.chunk = (int)k;
        it.start = c_items;
        return it;
    }
    long long base = nc;
    const long long steps = (long long)n_steps * nc;
    if (k < base + steps) {
        const long long r = k - base;
        it.kind = kSTEP;
        it.step = (int)(r / nc);
        it.chunk = (int)(r % nc);
        it.start = c_items + base + (long long)it.step * nc;
        return it;
    }
    base += steps;
    if (k < base + f_chunks) {
        it.kind = kENERGY;
        it.step = 0;
        it.chunk = (int)(k - base);
        it.start = c_items + base;
        return it;
    }
    base += f_chunks;
    if (k < base + e2_items) {
        it.kind = kPARTIAL;
        it.step = 0;
        it.chunk = (int)(k - base);
        it.start = c_items + base;
        return it;
    }
    base += e2_items;
    it.kind = kFINAL;
    it.step = 0;
    it.chunk = 0;
    it.start = c_items + base;
    return it;
}

template <class P, int Q, int OP, int NT>
__device__ void chunk_step(const typename P::T *src, typename P::T *dst, const Geo &g, const BCp &bc,
                           const CollParams &prm, int mode, int check, RunStatus *status, int step, long long n_begin,
                           long long n_end)
{
    // n0 is the same in every thread, so every warp runs whole iterations (the density check
    // reduces per warp)
    for (long long n0 = n_begin; n0 < n_end; n0 += NT) {
        const long long node = n0 + threadIdx.x;
        bool active = node < n_end;
        if (active && g.solid != nullptr && __ldcg(g.solid + node)) active = false;
        unsigned long long rho_bits = 0;
        int flag = 0;
        if (active) step_node<P, Q, OP, true>(src, dst, g, bc, prm, mode, check, 10.0, node, rho_bits, flag);
        if (check) report_density(status, step, rho_bits, flag);
    }
}

template <class P, int Q, int NT>
__device__ void chunk_step_op(int op, const typename P::T *src, typename P::T *dst, const Geo &g, const BCp &bc,
                              const CollParams &prm, int mode, int check, RunStatus *status, int step,
                              long long n_begin, long long n_end)
{
    switch (op) {
    case OP_BGK: chunk_step<P, Q, OP_BGK, NT>(src, dst, g, bc, prm, mode, check, status, step, n_begin, n_end); break;
    case OP_REG: chunk_step<P, Q, OP_REG, NT>(src, dst, g, bc, prm, mode, check, status, step, n_begin, n_end); break;
    case OP_MRT:
        if constexpr (Q == 9)
            chunk_step<P, Q, OP_MRT, NT>(src, dst, g, bc, prm, mode, check, status, step, n_begin, n_end);
        break;
    default:
        chunk_step<P, Q, OP_EXTREG, NT>(src, dst, g, bc, prm, mode, check, status, step, n_begin, n_end);
        break;
    }
}

// The result of run J (by the CTA that finished its last item).
static __device__ void publish(const TeamRing &r, TeamJob *J, const TeamEntry &e)
{
    RunStatus st;
    st.flags = ld_acq_gpu(&J->status.flags);
    st.decided_step = ld_acq_gpu(&J->status.decided_step);
    st.max_abs_rho_bits = atomicAdd(&J->status.max_abs_rho_bits, 0ull);
    const int ring_idx = __ldcg(&J->ring_idx);
    TeamDone *d = r.done + (ring_idx % r.capacity);
    double margin = 0.0;
    int label = 0, dec = e.n_steps, steps = e.n_steps;
    if (e.check_density) {
        const double mx = __longlong_as_double((long long)st.max_abs_rho_bits);
        margin = (st.flags & 2) ? __longlong_as_double(0x7ff0000000000000LL) : mx / 10.0;
        if (st.flags) {
            label = 1;
            dec = st.decided_step;
            steps = st.decided_step + 1;
        }
    }
    d->energy = *(volatile double *)&J->energy;
    d->margin = margin;
    d->t_admit_ns = __ldcg(&J->t_admit_ns);
    d->t_done_ns = now_ns();
    d->label = label;
    d->steps_done = steps;
    d->decided_step = dec;
    d->status = ld_acq_gpu(&J->error) ? TEAM_TIMEOUT : 0;
    d->peak_members = ld_acq_gpu(&J->peak);
    __threadfence_system();
    st_rel_sys(&d->seq, ring_idx + 1);
}

// Copy of n ints from device memory that other CTAs of the launch write, through L2.
__device__ __forceinline__ void copy_cg(void *dst, const void *src, int bytes)
{
    const int *s = (const int *)src;
    int *d = (int *)dst;
    for (int i = 0; i < bytes / (int)sizeof(int); i++) d[i] = __ldcg(s + i);
}

// Leaves run jid (thread 0).  The last member out of a closed run frees its pages and slot; a member
// that leaves an open run empty marks it hungry again.
static __device__ void leave_run(const TeamRing &r, int jid, bool close)
{
    TeamJob *J = r.jobs + jid;
    if (close) atomicOr(&J->members, TEAM_CLOSED);
    __threadfence();
    const int old = atomicSub(&J->members, 1);
    if (old == (TEAM_CLOSED | 1)) {
        pages_free(r.pages, __ldcg(&J->page0), __ldcg(&J->e.pages));
        atomicSub(&r.queue->active, 1);
        __threadfence();
        st_rel_gpu(&r.queue->job_state[jid], 0);
    } else if (old == 1) {
        atomicAdd(&r.queue->hungry, 1);
    }
}

// Joins an admitted, open run: the one with the fewest members for what it can use (a run with none
// first).  Returns its slot, or -1.
static __device__ int join_run(const TeamRing &r)
{
    TeamQueue *qu = r.queue;
    for (int tries = 0; tries < 4; tries++) {
        int best = -1;
        long long best_score = LLONG_MAX;
        for (int j = 0; j < r.max_jobs; j++) {
            if (ld_acq_gpu(&qu->job_state[j]) != 1) continue;
            TeamJob *J = r.jobs + j;
            const int m = ld_acq_gpu(&J->members);
            const int want = ld_acq_gpu(&J->want);
            if ((m & TEAM_CLOSED) || m >= want) continue;
            const long long score = ((long long)m << 20) / max(1, want);
            if (score < best_score) {
                best_score = score;
                best = j;
            }
        }
        if (best < 0) return -1;
        TeamJob *J = r.jobs + best;
        const int m = ld_acq_gpu(&J->members);
        if ((m & TEAM_CLOSED) || m >= ld_acq_gpu(&J->want)) continue;
        if (atomicCAS(&J->members, m, m + 1) == m) {
            if (m == 0) atomicSub(&qu->hungry, 1);
            atomicMax(&J->peak, m + 1);
            __threadfence();
            return best;
        }
    }
    return -1;
}

// The work of one CTA in run jid, until no item is left or another run needs it.  Returns true when
// the CTA left to join a hungry run (it holds one of the rescuers' places).
template <class P>
__device__ bool work_run(const TeamRing &r, int jid)
{
    using T = typename P::T;
    constexpr int NT = team_threads<P>();
    __shared__ TeamEntry s_e;
    __shared__ char *s_base;
    __shared__ long long s_total, s_k;
    __shared__ int s_cit, s_nch, s_fch, s_e2, s_ring, s_kind, s_step, s_chunk, s_noop, s_sd, s_leave;
    __shared__ double s_red[TEAM_RB];
    TeamJob *J = r.jobs + jid;
    const int tid = threadIdx.x;
    if (tid == 0) {
        copy_cg(&s_e, &J->e, sizeof(TeamEntry));
        s_base = (char *)__ldcg((const unsigned long long *)&J->base);
        s_total = __ldcg(&J->total);
        s_cit = __ldcg(&J->c_items);
        s_nch = __ldcg(&J->n_chunks);
        s_fch = __ldcg(&J->f_chunks);
        s_e2 = __ldcg(&J->e2_items);
        s_ring = __ldcg(&J->ring_idx);
    }
    __syncthreads();
    const TeamEntry &e = s_e;
    char *base = s_base;
    Geo g;
    g.nx = e.nx;
    g.ny = e.ny;
    g.nz = e.nz;
    g.nbox = (long long)e.nx * e.ny * e.nz;
    g.plane = (g.nbox + 63) / 64 * 64;
    T *buf[2] = {(T *)base, (T *)(base + e.off_buf1)};
    double *scr = (double *)(base + e.off_scr);
    double *part = scr + e.n_fluid;
    const unsigned char *hpl = r.payload + (long long)(s_ring % r.capacity) * r.payload_stride;
    unsigned char *pl = (unsigned char *)base + e.off_pay;  // the payload's copy in the run's pages
    const double *tab = (const double *)pl;
    g.solid = e.solid_len ? pl + e.pay_solid : nullptr;
    const int *nof = e.solid_len ? (const int *)(pl + e.pay_nof) : nullptr;
    BCp bc;
    bc.inlet_x = e.inlet_x;
    bc.outlet_x = e.outlet_x;
    bc.u_in = e.u0;
    bc.rho_out = 1.0;
    bc.inlet_kind = 0;
    bc.outlet_kind = 0;
    bc.open_y = -1;
    bc.profile = nullptr;
    const long long total = s_total, cn = e.chunk, nf = e.n_fluid;
    // thread 0: the next item, claimed while this one is worked on (-1: none claimed), and the last
    // count of finished items it read (the count only grows)
    long long pf = -1, known_done = 0;
    bool last_item = false;  // leaving after the item already claimed
    for (;;) {
        if (tid == 0) {
            const long long k = pf >= 0 ? pf : (long long)atomicAdd(&J->next, 1ull);
            pf = -1;
            s_k = k;
            s_noop = 0;
            if (k < total) {
                const Item it = item_of(k, s_cit, s_nch, s_fch, s_e2, e.n_steps);
                s_kind = it.kind;
                s_step = it.step;
                s_chunk = it.chunk;
                // every item of the previous phases done (the step barrier); bounded
                if (known_done < it.start) {
                    const long long t0 = now_ns();
                    while ((known_done = (long long)ld_acq_gpu64(&J->done)) < it.start) {
                        if (now_ns() - t0 > r.sync_ns) {
                            atomicExch(&J->error, 1);
                            break;
                        }
                        __nanosleep(64);
                    }
                }
                __threadfence();
                // a density check failed in an earlier step: the run stopped there
                int sd = e.n_steps;
                if (e.check_density && ld_acq_gpu(&J->status.flags)) sd = ld_acq_gpu(&J->status.decided_step) + 1;
                s_sd = sd;
                if (it.kind == kSTEP && it.step >= sd) s_noop = 1;
                // claim the next item now: the atomic's round trip overlaps this item's work
                if (!last_item && !s_noop) pf = (long long)atomicAdd(&J->next, 1ull);
            }
        }
        __syncthreads();
        const long long k = s_k;
        if (k >= total) break;
        if (!s_noop) {
            const int kind = s_kind, c = s_chunk;
            if (kind == kCOPY) {
                // host memory that the host rewrites for later requests: read uncached
                const long long b0 = (long long)c * TEAM_COPY, b1 = min(b0 + TEAM_COPY, e.pay_bytes);
                for (long long b = b0 + 16LL * tid; b < b1; b += 16LL * NT)
                    *(int4 *)(pl + b) = __ldcv((const int4 *)(hpl + b));
            } else if (kind == kINIT) {
                const long long nb = (long long)c * cn, ne = min(nb + cn, g.nbox);
                for (long long node = nb + tid; node < ne; node += NT) {
                    if (e.init == 1)
                        init_tg2d_node<P, true>(buf[0], g, tab, e.u0, e.tau, e.k, node);
                    else if (e.init == 4)
                        init_tg3d_node<P, true>(buf[0], g, tab, e.u0, node);
                    else if (e.q == 9)
                        init_rest_node<P, 9>(buf[0], g, 1.0, node);
                    else
                        init_rest_node<P, 19>(buf[0], g, 1.0, node);
                }
            } else if (kind == kSTEP) {
                const int s = s_step;
                const int mode = s == 0 ? 1 : 0;  // the initial state is a post-stream state
                const long long nb = (long long)c * cn, ne = min(nb + cn, g.nbox);
                if (e.q == 9)
                    chunk_step_op<P, 9, NT>(e.op, buf[s & 1], buf[(s + 1) & 1], g, bc, e.prm, mode, e.check_density,
                                        &J->status, s, nb, ne);
                else
                    chunk_step_op<P, 19, NT>(e.op, buf[s & 1], buf[(s + 1) & 1], g, bc, e.prm, mode, e.check_density,
                                         &J->status, s, nb, ne);
            } else if (kind == kENERGY) {
                // kinetic energy of the post-stream state (k_stream_only + k_node_fields)
                const int sd = s_sd;
                const long long pb = (long long)c * cn, pe = min(pb + cn, nf);
                for (long long p = pb + tid; p < pe; p += NT)
                    scr[p] = e.q == 9 ? node_energy_at<P, 9, true>(buf[sd & 1], g, nof, p, sd > 0)
                                      : node_energy_at<P, 19, true>(buf[sd & 1], g, nof, p, sd > 0);
            } else if (kind == kPARTIAL && nf <= TEAM_SERIAL) {
                if (tid == 0) {  // k_sum_serial
                    double sum = 0;
                    for (long long i = 0; i < nf; i++) sum = sum + __ldcg(scr + i);
                    J->energy = sum;
                }
            } else if (kind == kPARTIAL) {
                // k_sum_partial: block b, thread t sums i = b * 256 + t advancing by 1024 * 256, then a
                // tree over the 256 threads; a CTA thread plays threads t, t + NT, ...
                for (int b = c * TEAM_RG_ITEM; b < (c + 1) * TEAM_RG_ITEM && b < TEAM_RG; b++) {
                    for (int h = 0; h < TEAM_RB / NT; h++) {
                        const int t = tid + h * NT;
                        double sum = 0;
                        for (long long i = (long long)b * TEAM_RB + t; i < nf; i += (long long)TEAM_RG * TEAM_RB)
                            sum += __ldcg(scr + i);
                        s_red[t] = sum;
                    }
                    __syncthreads();
                    for (int o = TEAM_RB / 2; o > 0; o >>= 1) {
                        if (tid < o) s_red[tid] += s_red[tid + o];
                        __syncthreads();
                    }
                    if (tid == 0) part[b] = s_red[0];
                    __syncthreads();
                }
            } else {  // kFINAL: k_sum_final
                for (int h = 0; h < TEAM_RB / NT; h++) {
                    const int t = tid + h * NT;
                    double sum = 0;
                    for (int i = t; i < TEAM_RG; i += TEAM_RB) sum += __ldcg(part + i);
                    s_red[t] = sum;
                }
                __syncthreads();
                for (int o = TEAM_RB / 2; o > 0; o >>= 1) {
                    if (tid < o) s_red[tid] += s_red[tid + o];
                    __syncthreads();
                }
                if (tid == 0) J->energy = s_red[0];
            }
        }
        __syncthreads();
        if (tid == 0) {
            unsigned long long add = 1;
            if (s_noop) {
                // skip the remaining steps of a stopped run in one claim
                const long long e1 = (long long)s_cit + s_nch + (long long)e.n_steps * s_nch;
                unsigned long long cur = ld_acq_gpu64(&J->next);
                for (int tries = 0; tries < 16 && (long long)cur < e1; tries++) {
                    const unsigned long long old = atomicCAS(&J->next, cur, (unsigned long long)e1);
                    if (old == cur) {
                        add += (unsigned long long)e1 - cur;
                        break;
                    }
                    cur = old;
                }
            }
            __threadfence();
            const unsigned long long d = atomicAdd(&J->done, add) + add;
            if ((long long)d == total) publish(r, J, e);
            // make room for an admitted run that has no member yet: as many CTAs leave their runs as
            // there are such runs, each taking a rescuer's place first.  A CTA that holds a claimed
            // item works on it before it leaves.
            s_leave = 0;
            if (last_item) {
                s_leave = 1;
            } else if (ld_acq_gpu(&r.queue->hungry) > 0 && (ld_acq_gpu(&J->members) & ~TEAM_CLOSED) > 1) {
                int hungry = ld_acq_gpu(&r.queue->hungry), resc = ld_acq_gpu(&r.queue->rescuers);
                for (int tries = 0; tries < 4 && resc < hungry; tries++) {
                    const int old = atomicCAS(&r.queue->rescuers, resc, resc + 1);
                    if (old == resc) {
                        if (pf >= 0 && pf < total)
                            last_item = true;
                        else
                            s_leave = 1;
                        break;
                    }
                    resc = old;
                    hungry = ld_acq_gpu(&r.queue->hungry);
                }
            }
        }
        __syncthreads();
        if (s_leave) break;
    }
    // a claimed item past the end leaves the run closed; one that ended the loop by leaving was worked on
    const bool rescuer = s_leave != 0 && s_k < total;
    if (tid == 0) leave_run(r, jid, s_k >= total || pf >= total);
    __syncthreads();
    return rescuer;
}

// Admission of ring entry idx: 0 admitted, 1 not now.  Called by the admitter thread only.
static __device__ int try_admit(const TeamRing &r, int grid, int idx, long long now)
{
    TeamQueue *qu = r.queue;
    const TeamEntry *pe = r.entries + (idx % r.capacity);
    if (ld_acq_gpu(&qu->active) >= r.max_jobs) return 1;
    int slot = -1;
    for (int j = 0; j < r.max_jobs; j++)
        if (ld_acq_gpu(&qu->job_state[j]) == 0) {
            slot = j;
            break;
        }
    if (slot < 0) return 1;
    const int pages = __ldcv(&pe->pages);
    const int page0 = pages_claim(r.pages, r.n_pages, pages);
    if (page0 < 0) return 1;
    TeamJob *J = r.jobs + slot;
    {
        const int *src = (const int *)pe;
        int *dst = (int *)&J->e;
        for (int i = 0; i < (int)(sizeof(TeamEntry) / sizeof(int)); i++) dst[i] = __ldcv(src + i);
    }
    const TeamEntry &e = J->e;
    const long long nbox = (long long)e.nx * e.ny * e.nz;
    J->base = r.arena + (long long)page0 * TEAM_PAGE;
    J->status.flags = 0;
    J->status.decided_step = INT_MAX;
    J->status.max_abs_rho_bits = 0ull;
    J->energy = 0.0;
    J->t_admit_ns = now;
    J->next = 0ull;
    J->done = 0ull;
    J->ring_idx = idx;
    J->page0 = page0;
    J->c_items = (int)((e.pay_bytes + TEAM_COPY - 1) / TEAM_COPY);
    J->n_chunks = (int)((nbox + e.chunk - 1) / e.chunk);
    J->f_chunks = (int)(((long long)e.n_fluid + e.chunk - 1) / e.chunk);
    J->e2_items = e.n_fluid <= TEAM_SERIAL ? 1 : TEAM_RG / TEAM_RG_ITEM;
    J->total = J->c_items + (long long)J->n_chunks * (1 + e.n_steps) + J->f_chunks + J->e2_items +
               (e.n_fluid <= TEAM_SERIAL ? 0 : 1);
    J->want = max(1, min(J->n_chunks, grid - 1));
    J->error = 0;
    J->peak = 0;
    __threadfence();
    atomicExch(&J->members, 0);
    atomicAdd(&qu->active, 1);
    atomicAdd(&qu->hungry, 1);
    __threadfence();
    st_rel_gpu(&qu->job_state[slot], 1);
    return 0;
}

// The admitter's loop (thread 0 of the elected CTA).
static __device__ void admit_loop(const TeamRing &r, int grid)
{
    TeamCtl *ctl = r.ctl;
    TeamQueue *qu = r.queue;
    const long long t_start = now_ns();
    long long last = t_start;
    for (;;) {
        const long long now = now_ns();
        atomicExch((unsigned long long *)&ctl->heartbeat, (unsigned long long)now);
        if (ld_acq_sys(r.stop)) break;
        bool busy = false;
        // claim what the host has published
        const int tail = ld_acq_sys(r.tail);
        int head = qu->head, n = qu->n;
        while (head < tail && n < TEAM_PEND) {
            qu->idx[n] = head;
            qu->claim_ns[n] = now;
            qu->est_ns[n] = __ldcv(&r.entries[head % r.capacity].est_ns);
            n++;
            head++;
            busy = true;
        }
        qu->head = head;
        // admit, shortest estimate first with aging
        while (n > 0) {
            int best = 0;
            long long bk = LLONG_MAX;
            for (int k = 0; k < n; k++) {
                const long long key = qu->est_ns[k] - (now - qu->claim_ns[k]);
                if (key < bk) {
                    bk = key;
                    best = k;
                }
            }
            if (try_admit(r, grid, qu->idx[best], now) != 0) break;
            for (int k = best; k + 1 < n; k++) {
                qu->idx[k] = qu->idx[k + 1];
                qu->claim_ns[k] = qu->claim_ns[k + 1];
                qu->est_ns[k] = qu->est_ns[k + 1];
            }
            n--;
            busy = true;
        }
        qu->n = n;
        const int active = ld_acq_gpu(&qu->active);
        if (busy || active > 0) last = now;
        if (n == 0 && active == 0 && now - last > r.idle_ns) break;
        // no worker CTA ever came up in this launch: leave, the host launches again
        if (ld_acq_gpu(&ctl->live) == 0 && now - t_start > r.idle_ns) break;
        if (!busy) __nanosleep(2000);
    }
    __threadfence();
    st_rel_gpu(&ctl->closing, 1);
}

// A worker CTA's loop.
template <class P>
__device__ void work_loop(const TeamRing &r)
{
    __shared__ int s_job;
    TeamCtl *ctl = r.ctl;
    if (threadIdx.x == 0) atomicAdd(&ctl->live, 1);
    const long long t0 = now_ns();
    __shared__ int s_rescuer;
    if (threadIdx.x == 0) s_rescuer = 0;
    for (;;) {
        if (threadIdx.x == 0) {
            int job = -2;
            unsigned nap = 1000;  // ns; doubled after each empty scan up to 64 us, so that idle CTAs
                                  // do not load L2 with scans of the run table
            while (job == -2) {
                const int j = ld_acq_gpu(&r.queue->active) > 0 ? join_run(r) : -1;
                if (s_rescuer) {  // the place is given back whether or not a hungry run was left
                    atomicSub(&r.queue->rescuers, 1);
                    s_rescuer = 0;
                }
                if (j >= 0) {
                    job = j;
                    break;
                }
                const long long hb = (long long)atomicAdd((unsigned long long *)&ctl->heartbeat, 0ull);
                if (ld_acq_gpu(&ctl->closing) || ld_acq_sys(r.stop) || now_ns() - (hb > 0 ? hb : t0) > r.idle_ns) {
                    job = -1;
                } else {
                    __nanosleep(nap);
                    nap = min(nap * 2, 64000u);
                }
            }
            s_job = job;
        }
        __syncthreads();
        if (s_job < 0) break;
        const bool rescuer = work_run<P>(r, s_job);
        if (threadIdx.x == 0) s_rescuer = rescuer ? 1 : 0;
    }
    if (threadIdx.x == 0) atomicSub(&ctl->live, 1);
}

template <class P>
__global__ void __launch_bounds__(team_threads<P>(), 512 / team_threads<P>()) k_team_server(TeamRing r)
{
    __shared__ int s_role;
    if (threadIdx.x == 0) s_role = atomicCAS(&r.ctl->admitter, 0, (int)blockIdx.x + 1) == 0 ? 1 : 0;
    __syncthreads();
    if (s_role) {
        if (threadIdx.x == 0) admit_loop(r, (int)gridDim.x);
        return;
    }
    work_loop<P>(r);
}

}  // namespace team
#endif  // __CUDACC__

}  // namespace erlbm
