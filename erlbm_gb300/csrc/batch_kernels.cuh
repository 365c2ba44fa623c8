// batch_kernels.cuh -- many small independent lattices in one persistent launch.
//
// This replaces the stability-map loops of the reference: "#pragma omp parallel for collapse(2)
// schedule(dynamic)" over map points (main_stability-map_taylor-green.cpp:150-177,
// main_stability-map_obstacle.cpp:161-186), each point running roda_ponto (TG map :41-104,
// obstacle map :75-123) on its own populations.
//
// Layout.  One CTA owns one lattice "slot": the whole lattice (nx * ny <= NPT * blockDim nodes,
// nz = 1) lives in shared memory as SoA, buf[i * NB + node].  A step is
//   gather (pull; bounce-back from the solid mask) into registers -> [barrier] ->
//   [energy check] -> boundary planes -> collide -> [density check] -> write own nodes -> barrier.
// Where two buffers fit (dbl), the step reads one and writes the other, and the barrier after the
// gather is not needed; otherwise one buffer is updated in place.  When a run ends (budget reached, or a check failed), thread 0 claims the
// next run index from a global counter and the slot is refilled: the launch is persistent, with
// grid = SMs x resident CTAs, and the host orders runs longest-first so the tail is short.
//
// Checks (the reference's, per run):
//   energy: E = sum 1/2 |u|^2 of the post-stream populations at step % every == 0 && step > 0;
//           unstable when E > factor * E0 or E is not finite (TG map :69-81).  FP64: per-node
//           energies are summed serially in node order, as kinectic_energy does.
//   density: |rho| > limit or non-finite at any node after its collision; the step is finished
//           and the run stops (obstacle map :98-106, :88).
// Every loop is bounded by the run's step budget; nothing waits on another CTA.
#pragma once

#include <cstdint>

#include "lattice_kernels.cuh"

namespace erlbm {

enum BatchInit : int { INIT_REST = 0, INIT_TG_MAP = 1, INIT_AOS = 2 };

// Geometry and checks shared by every run of a launch.
struct BatchGeo {
    int nx, ny, nb;               // box (nz = 1), nb = nx * ny
    const uint8_t *solid;         // nb bytes, 1 = solid; null = fully periodic
    int inlet_x, outlet_x;        // boundary planes, -1 = none (D3Q19 inlet only)
    double rho0;                  // outlet density and rest density
    int energy_every;             // 0 = off
    double energy_factor;
    int density_check;
    double density_limit;
    int init;                     // BatchInit
    const double *sinx, *cosx;    // INIT_TG_MAP: sin(2 pi x / L), cos(2 pi x / L) for x < nx
    // FP32 path: |1 + drho| > density_limit  <=>  drho > drho_hi || drho < drho_lo for a float drho
    // (bounds limit - 1 and -limit - 1 rounded outward to float on the host; see density_bounds)
    float drho_hi, drho_lo;
};

// Float bounds equivalent to the FP64 test |1 + (double)d| > limit for every float d: 1 + d is exact
// in FP64 near the thresholds, and "d > x" for a double x equals "d > x rounded down to float".
inline void density_bounds(BatchGeo &g)
{
    const double hi = g.density_limit - 1.0, lo = -g.density_limit - 1.0;
    float fh = (float)hi, fl = (float)lo;
    if ((double)fh > hi) fh = nextafterf(fh, -INFINITY);
    if ((double)fl < lo) fl = nextafterf(fl, INFINITY);
    g.drho_hi = fh;
    g.drho_lo = fl;
}

// One run, prepared on the host.
struct BatchRun {
    Relax R;
    shifted::Coef k;
    double u0;          // TG amplitude (INIT_TG_MAP) or inlet velocity (inlet_x >= 0)
    long long aos_off;  // INIT_AOS: offset (in doubles) of this run's initial AoS populations
    int n_steps;
    int op;
    int out;            // result slot
    int pad;
};

struct BatchResult {
    int label;          // 1 unstable
    int decided_step;   // failing step, or n_steps
    int steps_done;
    int status;         // bit 0 density, bit 1 non-finite density, bit 2 energy
    double margin;      // max E/(factor E0) or max |rho|/limit (+inf for non-finite)
    double energy;      // last energy computed (E0 when no check ran)
};

template <class P, int Q>
__device__ __forceinline__ void batch_collide(typename P::T *f, const BatchRun &r)
{
    CollParams prm;
    prm.R = r.R;
    prm.k = r.k;
    if constexpr (Q == 9) {
        if (r.op == OP_MRT) {
            P::template collide<Q, OP_MRT>(f, prm);
            return;
        }
    }
    if (r.op == OP_BGK)
        P::template collide<Q, OP_BGK>(f, prm);
    else if (r.op == OP_REG)
        P::template collide<Q, OP_REG>(f, prm);
    else
        P::template collide<Q, OP_EXTREG>(f, prm);
}

// Two D2Q9 nodes of the FP32 path at once, in the halves of float2 lanes (packed FP32x2
// instructions): the same bits as batch_collide on each.
template <int Q>
__device__ __forceinline__ void batch_collide_pair(float *fa, float *fb, const BatchRun &r)
{
    static_assert(Q == 9, "packed pairs are used for D2Q9");
    float2 g[Q];
#pragma unroll
    for (int i = 0; i < Q; i++) g[i] = make_float2(fa[i], fb[i]);
    if (r.op == OP_MRT)
        shifted::collide9x2<OP_MRT>(g, r.k);
    else if (r.op == OP_BGK)
        shifted::collide9x2<OP_BGK>(g, r.k);
    else if (r.op == OP_REG)
        shifted::collide9x2<OP_REG>(g, r.k);
    else
        shifted::collide9x2<OP_EXTREG>(g, r.k);
#pragma unroll
    for (int i = 0; i < Q; i++) {
        fa[i] = g[i].x;
        fb[i] = g[i].y;
    }
}

// Initial equilibrium of the Taylor-Green map (main_stability-map_taylor-green.cpp:49-61): rho = 1,
// u_x = U0 sin(kx) cos(ky), u_y = -U0 cos(kx) sin(ky), u_z = 0.
template <class P, int Q>
__device__ __forceinline__ void tg_map_init(typename P::T *f, int x, int y, double u0, const BatchGeo &g)
{
    if constexpr (sizeof(typename P::T) == 4) {
        // FP32 path: the shifted equilibrium at rho = 1, g_i = w_i (3 cu + 4.5 cu^2 - 1.5 u^2), formed in
        // FP32 from small quantities (within an ulp or two of the FP64 equilibrium rounded to float)
        const float ux = (float)(u0 * g.sinx[x] * g.cosx[y]);
        const float uy = (float)(-u0 * g.cosx[x] * g.sinx[y]);
        const float mu = -1.5f * fmaf(ux, ux, uy * uy);
#pragma unroll
        for (int i = 0; i < Q; i++) {
            const float cu = (float)Lat<Q>::cx(i) * ux + (float)Lat<Q>::cy(i) * uy;
            f[i] = (float)Lat<Q>::w(i) * fmaf(cu, fmaf(4.5f, cu, 3.f), mu);
        }
        return;
    }
    const double ux = u0 * g.sinx[x] * g.cosx[y];
    const double uy = -u0 * g.cosx[x] * g.sinx[y];
    double feq[Q];
    if constexpr (Q == 19)
        exact::equilibrium19(1.0, ux, uy, 0.0, feq);
    else
        exact::equilibrium9(1.0, ux, uy, feq);
#pragma unroll
    for (int i = 0; i < Q; i++) f[i] = P::template from_f<Q>(feq[i], i);
}

// Deterministic block sum of one double per thread.  Exact path: serial in fluid-index order (slot =
// the thread's fluid index, -1 for a thread without a node), like kinectic_energy; FP32 path: fixed
// shuffle tree + serial over warps.
template <bool SERIAL>
__device__ double block_sum(double v, double *sh, int n_vals, int slot)
{
    const int tid = threadIdx.x;
    double total;
    if (SERIAL) {
        if (slot >= 0) sh[slot] = v;
        __syncthreads();
        if (tid == 0) {
            double s = 0;
            for (int k = 0; k < n_vals; k++) s = s + sh[k];
            sh[blockDim.x] = s;
        }
        __syncthreads();
        total = sh[blockDim.x];
    } else {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((tid & 31) == 0) sh[tid >> 5] = v;
        __syncthreads();
        if (tid == 0) {
            double s = 0;
            for (int k = 0; k < (int)(blockDim.x >> 5); k++) s += sh[k];
            sh[blockDim.x] = s;
        }
        __syncthreads();
        total = sh[blockDim.x];
    }
    __syncthreads();
    return total;
}

__device__ __forceinline__ double block_max(double v, double *sh)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    const int tid = threadIdx.x;
    if ((tid & 31) == 0) sh[tid >> 5] = v;
    __syncthreads();
    if (tid == 0) {
        double s = 0;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) s = fmax(s, sh[k]);
        sh[blockDim.x] = s;
    }
    __syncthreads();
    const double t = sh[blockDim.x];
    __syncthreads();
    return t;
}

// Shared memory: populations Q * NB of T (twice when ping-ponged), reduction scratch, the solid mask
// (NB bytes), the node order (NB shorts), the number of fluid nodes and the Zou-He constants.
template <class P, int Q>
__host__ __device__ inline size_t batch_smem_bytes(int nb, int block, int dbl)
{
    const size_t pop = (size_t)Q * nb * sizeof(typename P::T) * (dbl ? 2 : 1);
    const size_t red = ((size_t)block + 1) * sizeof(double);
    const size_t mask = ((size_t)nb + 15) / 16 * 16;
    const size_t order = ((size_t)nb * sizeof(short) + 15) / 16 * 16;
    return (pop + 15) / 16 * 16 + red + mask + order + 16 + 32;
}

// Register budget: one node per thread (the map lattices: 256 or 264 nodes) wants several
// resident CTAs per SM to overlap their barriers, so it is bounded to 288 threads x 3 CTAs (FP32)
// or x 2 (FP64, whose exact collision needs more registers); larger lattices get 512 x 1.
template <int NPT, int BYTES>
struct BatchBounds {
    static constexpr int MAXT = NPT == 1 ? 288 : 512;
    static constexpr int MINB = NPT == 1 ? (BYTES == 8 ? 2 : 3) : 1;
};

// Shared-memory carve-up of a batched CTA (sizes from batch_smem_bytes).
template <class P, int Q>
struct BatchSmem {
    typename P::T *buf0, *buf1;  // the same buffer unless ping-ponged
    double *red;
    uint8_t *solid;
    short *order;   // node of each thread slot: fluid nodes only, boundary-plane nodes first
    int *n_fluid;
    double *zh;     // the run's Zou-He closure constants (P::ZouHe, <= 32 bytes)
    __device__ BatchSmem(unsigned char *raw, int nb, int dbl)
    {
        const size_t one = (size_t)Q * nb * sizeof(typename P::T);
        buf0 = reinterpret_cast<typename P::T *>(raw);
        buf1 = dbl ? reinterpret_cast<typename P::T *>(raw + one) : buf0;
        red = reinterpret_cast<double *>(raw + (one * (dbl ? 2 : 1) + 15) / 16 * 16);
        solid = reinterpret_cast<uint8_t *>(red + blockDim.x + 1);
        order = reinterpret_cast<short *>(solid + ((size_t)nb + 15) / 16 * 16);
        n_fluid = reinterpret_cast<int *>(order + ((size_t)nb * sizeof(short) + 15) / 16 * 16 / sizeof(short));
        zh = reinterpret_cast<double *>(n_fluid + 4);
    }
};

// Thread slots of a geometry (one thread, after sm.solid is loaded): the fluid nodes in node order,
// except that the nodes of the boundary planes come first.  Those run the inlet and outlet closures
// (with FP64 operations in the FP32 path); packed into the first warp, they no longer put that work
// on every warp of the CTA in every step.  Solid nodes get no thread.
__device__ inline void make_order(const BatchGeo &g, short *order, int *n_fluid, const uint8_t *solid)
{
    int k = 0;
    for (int pass = 0; pass < 2; pass++)
        for (int n = 0; n < g.nb; n++) {
            if (solid[n]) continue;
            const int x = n % g.nx;
            const bool plane = x == g.inlet_x || x == g.outlet_x;
            if (plane == (pass == 0)) order[k++] = (short)n;
        }
    *n_fluid = k;
}

// One run of one lattice by the whole CTA.  sm.solid must hold the geometry's mask.  The result is
// returned to every thread.
template <class P, int Q, int NPT>
__device__ BatchResult batch_one_run(const BatchGeo &g, const BatchRun &r, const BatchSmem<P, Q> &sm,
                                     const double *__restrict__ aos)
{
    using T = typename P::T;
    const int NB = g.nb;
    // populations of the current step are read from cur and the next step's are stored to nxt; with
    // two buffers one barrier per step suffices (a step's stores never touch what it reads)
    T *cur = sm.buf0, *nxt = sm.buf1;
    const bool dbl = sm.buf1 != sm.buf0;
    double *red = sm.red;
    const uint8_t *solid = sm.solid;
    const int tid = threadIdx.x;
    const bool any_solid = g.solid != nullptr;

    int node[NPT], nx_[NPT], ny_[NPT];
    bool fluid[NPT];
    const int n_fluid = *sm.n_fluid;
#pragma unroll
    for (int s = 0; s < NPT; s++) {
        const int slot = tid + s * blockDim.x;
        fluid[s] = slot < n_fluid;
        node[s] = fluid[s] ? sm.order[slot] : 0;
        nx_[s] = node[s] % g.nx;
        ny_[s] = node[s] / g.nx;
    }
    constexpr bool SERIAL = NPT == 1 && sizeof(T) == 8;
    // fluid index of a thread's node (solid nodes before it skipped): the serial energy sum's order
    // and the AoS initial populations' position
    int fidx = -1;
    if (fluid[0] && (g.init == INIT_AOS || (SERIAL && g.energy_every > 0))) {
        fidx = 0;
        for (int k = 0; k < node[0]; k++) fidx += !solid[k];
    }
    // the Zou-He constants live in shared memory: only the boundary threads read them, and keeping
    // them in registers for the whole run would cost every thread
    using ZH = typename P::ZouHe;
    static_assert(sizeof(ZH) <= 32, "ZouHe constants exceed their shared-memory slot");
    if (tid == 0) *reinterpret_cast<ZH *>(sm.zh) = P::zou_he_prep(r.u0);

    // ---- initial populations (post-stream state of step 0) ----
    T f[NPT][Q];
#pragma unroll
    for (int s = 0; s < NPT; s++) {
        if (!fluid[s]) continue;
        if (g.init == INIT_TG_MAP) {
            tg_map_init<P, Q>(f[s], nx_[s], ny_[s], r.u0, g);
        } else if (g.init == INIT_AOS) {
            int p = fidx;
            if (s > 0) {
                p = 0;
                for (int k = 0; k < node[s]; k++) p += !solid[k];
            }
            const double *src = aos + r.aos_off + (long long)p * Q;
#pragma unroll
            for (int i = 0; i < Q; i++) f[s][i] = P::template from_f<Q>(src[i], i);
        } else {
#pragma unroll
            for (int i = 0; i < Q; i++) f[s][i] = P::template from_f<Q>(Lat<Q>::w(i) * g.rho0, i);
        }
#pragma unroll
        for (int i = 0; i < Q; i++) cur[i * NB + node[s]] = f[s][i];
    }
    __syncthreads();

    double E0 = 0.0, E = 0.0, margin = 0.0, max_rho = 0.0;
    float dmax = -INFINITY, dmin = INFINITY;  // FP32 path: extreme drho seen by this thread
    int label = 0, decided = r.n_steps, status = 0, steps_done = r.n_steps;
    if (g.energy_every > 0) {
        double e = 0.0;
#pragma unroll
        for (int s = 0; s < NPT; s++)
            if (fluid[s]) e += P::template energy<Q>(f[s]);
        E0 = block_sum<SERIAL>(e, red, n_fluid, fidx);
        E = E0;
    }

    int until_check = g.energy_every;  // steps to the next energy check (no division in the loop)
    for (int step = 0; step < r.n_steps; step++, until_check--) {
        // ---- stream: post-stream populations of this step ----
        if (step > 0) {
#pragma unroll
            for (int s = 0; s < NPT; s++) {
                if (!fluid[s]) continue;
                int x = nx_[s];
                const int y = ny_[s];
                int me = node[s];
                if (x == g.outlet_x) {  // the outlet copies its inner neighbour (devnull_rho_x)
                    x += (g.outlet_x < g.nx / 2) ? 1 : -1;
                    me = node[s] + (x - nx_[s]);
                }
#pragma unroll
                for (int i = 0; i < Q; i++) {
                    const int xs = wrap1(x - Lat<Q>::cx(i), g.nx);
                    const int ys = wrap1(y - Lat<Q>::cy(i), g.ny);
                    const int src = xs + g.nx * ys;
                    f[s][i] = (any_solid && solid[src]) ? cur[Lat<Q>::opp(i) * NB + me] : cur[i * NB + src];
                }
            }
        } else if (g.outlet_x >= 0) {
#pragma unroll
            for (int s = 0; s < NPT; s++) {
                if (!fluid[s] || nx_[s] != g.outlet_x) continue;
                const int me = node[s] + ((g.outlet_x < g.nx / 2) ? 1 : -1);
#pragma unroll
                for (int i = 0; i < Q; i++) f[s][i] = cur[i * NB + me];
            }
        }
        if (!dbl) __syncthreads();

        // ---- energy check on the post-stream populations ----
        if (g.energy_every > 0 && until_check == 0) {  // step > 0 && step % energy_every == 0
            until_check = g.energy_every;
            double e = 0.0;
#pragma unroll
            for (int s = 0; s < NPT; s++)
                if (fluid[s]) e += P::template energy<Q>(f[s]);
            E = block_sum<SERIAL>(e, red, n_fluid, fidx);
            const double lim = g.energy_factor * E0;
            const double rr = isfinite(E) ? E / lim : INFINITY;
            margin = fmax(margin, rr);
            if (E > lim || !isfinite(E)) {
                label = 1;
                decided = step;
                steps_done = step;
                status |= 4;
                break;
            }
        }

        // ---- boundary planes, collision, density check, store ----
        int flag = 0;
#pragma unroll
        for (int s = 0; s < NPT; s++) {
            if (!fluid[s]) continue;
            const int x = nx_[s];
            if (x == g.outlet_x) {
                const int xn = x + ((g.outlet_x < g.nx / 2) ? 1 : -1);
                if (Q == 19 && xn == g.inlet_x)
                    P::zou_he(f[s], *reinterpret_cast<const ZH *>(sm.zh), g.inlet_x < g.nx / 2);
                if (any_solid && solid[node[s] + (xn - x)])
                    P::template rest<Q>(f[s], g.rho0);
                else
                    P::template outlet<Q>(f[s], g.rho0);
            } else if (Q == 19 && x == g.inlet_x) {
                P::zou_he(f[s], *reinterpret_cast<const ZH *>(sm.zh), g.inlet_x < g.nx / 2);
            }
        }
        // FP32: the nodes of a thread in pairs, in packed FP32x2 instructions (D2Q9).  The D3Q19 pairs
        // collide one after the other: the packed D3Q19 form measured 5 % faster on the Taylor-Green
        // map but did not reproduce the scalar form's bits (final energies 3.5e-7 apart after 1500
        // steps), and the scalar form is the one every other FP32 D3Q19 path uses.
        constexpr bool PAIRS = sizeof(T) == 4 && NPT % 2 == 0 && Q == 9;
        if constexpr (PAIRS) {
#pragma unroll
            for (int s = 0; s < NPT; s += 2) {
                if (fluid[s] && fluid[s + 1]) {
                    batch_collide_pair<Q>(f[s], f[s + 1], r);
                } else {
                    if (fluid[s]) batch_collide<P, Q>(f[s], r);
                    if (fluid[s + 1]) batch_collide<P, Q>(f[s + 1], r);
                }
            }
        }
#pragma unroll
        for (int s = 0; s < NPT; s++) {
            if (!fluid[s]) continue;
            if constexpr (!PAIRS) batch_collide<P, Q>(f[s], r);
            if (g.density_check) {
                if constexpr (sizeof(T) == 4) {
                    const float d = shifted::node_drho<Q>(f[s]);
                    if (!isfinite(d)) {
                        flag |= 2;
                    } else {
                        dmax = fmaxf(dmax, d);
                        dmin = fminf(dmin, d);
                        if (d > g.drho_hi || d < g.drho_lo) flag |= 1;
                    }
                } else {
                    const double rho = P::template density<Q>(f[s]);
                    if (!isfinite(rho)) {
                        flag |= 2;
                    } else {
                        const double a = fabs(rho);
                        max_rho = fmax(max_rho, a);
                        if (a > g.density_limit) flag |= 1;
                    }
                }
            }
#pragma unroll
            for (int i = 0; i < Q; i++) nxt[i * NB + node[s]] = f[s][i];
        }
        if (dbl) {
            T *t = cur;
            cur = nxt;
            nxt = t;
        }
        if (g.density_check) {
            // finish the step everywhere, then stop if any node failed
            const int any = __syncthreads_or(flag);
            if (any) {
                label = 1;
                decided = step;
                steps_done = step + 1;
                status |= __syncthreads_or(flag & 2) ? 3 : 1;
                break;
            }
        } else {
            __syncthreads();
        }
    }
    if (g.density_check) {
        if constexpr (sizeof(T) == 4) {
            if (dmax >= dmin) max_rho = fmax(fabs(1.0 + (double)dmax), fabs(1.0 + (double)dmin));
        }
        max_rho = block_max(max_rho, red);
        margin = (status & 2) ? INFINITY : max_rho / g.density_limit;
    }
    BatchResult o;
    o.label = label;
    o.decided_step = decided;
    o.steps_done = steps_done;
    o.status = status;
    o.margin = margin;
    o.energy = E;
    __syncthreads();
    return o;
}

template <class P, int Q, int NPT>
__global__ void __launch_bounds__(BatchBounds<NPT, sizeof(typename P::T)>::MAXT,
                                  BatchBounds<NPT, sizeof(typename P::T)>::MINB)
    k_batch(BatchGeo g, const BatchRun *__restrict__ runs, int n_runs, int *__restrict__ counter,
            BatchResult *__restrict__ res, const double *__restrict__ aos, int dbl)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const BatchSmem<P, Q> sm(smem_raw, g.nb, dbl);
    __shared__ int s_run;
    const int tid = threadIdx.x;
    for (int k = tid; k < g.nb; k += blockDim.x) sm.solid[k] = g.solid ? g.solid[k] : 0;
    __syncthreads();
    if (tid == 0) make_order(g, sm.order, sm.n_fluid, sm.solid);
    for (;;) {
        __syncthreads();
        if (tid == 0) s_run = atomicAdd(counter, 1);
        __syncthreads();
        const int ri = s_run;
        if (ri >= n_runs) break;
        const BatchRun r = runs[ri];
        const BatchResult o = batch_one_run<P, Q, NPT>(g, r, sm, aos);
        if (tid == 0) res[r.out] = o;
    }
}

// ------------------------------------------------------------------------------------------------
// Device-resident request loop (serving): CTAs claim requests that the host publishes in a ring
// in mapped pinned memory, run them to completion and publish the results.  Every wait is bounded.
// ------------------------------------------------------------------------------------------------

struct SlotEntry {        // written by the host before it publishes the ring tail
    BatchRun run;
    int geo;              // index into the launch's geometry table
    int pad[3];
};

struct SlotDone {         // written by the device; seq is published last
    BatchResult res;
    int seq;              // ring index + 1 once res is valid
    int lane_exit;        // unused by runs
    int pad[2];
};

struct SlotRing {
    const int *tail;             // host-mapped: number of entries published
    const SlotEntry *entries;    // host-mapped ring of `capacity` entries
    SlotDone *done;              // host-mapped ring of results
    const int *stop;             // host-mapped: 1 = stop after the current run
    int *head;                   // device: next entry to claim
    int *exits;                  // device: [0] CTAs that left idle-timed-out, [1] stopped
    int capacity;
    long long idle_polls;        // bounded wait: polls of the tail before a CTA gives up
    const BatchGeo *geos;        // device table of geometries
    int n_geos;
};

__device__ __forceinline__ int ld_acquire_sys(const int *p)
{
    int v;
    asm volatile("ld.acquire.sys.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release_sys(int *p, int v)
{
    asm volatile("st.release.sys.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

template <class P, int Q, int NPT>
__global__ void __launch_bounds__(BatchBounds<NPT, sizeof(typename P::T)>::MAXT,
                                  BatchBounds<NPT, sizeof(typename P::T)>::MINB)
    k_slot_server(SlotRing ring, int max_nb, int dbl)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const BatchSmem<P, Q> sm(smem_raw, max_nb, dbl);
    __shared__ int s_idx;
    __shared__ SlotEntry s_entry;
    const int tid = threadIdx.x;
    for (;;) {
        __syncthreads();
        if (tid == 0) {
            int idx = -1;
            for (long long polls = 0;; polls++) {
                if (ld_acquire_sys(ring.stop)) {
                    idx = -2;
                    break;
                }
                const int t = ld_acquire_sys(ring.tail);
                const int h = *(volatile int *)ring.head;
                if (h < t) {
                    if (atomicCAS(ring.head, h, h + 1) == h) {
                        idx = h;
                        break;
                    }
                    continue;
                }
                if (polls >= ring.idle_polls) {
                    idx = -3;
                    break;
                }
                __nanosleep(2000);
            }
            if (idx >= 0) s_entry = ring.entries[idx % ring.capacity];
            s_idx = idx;
        }
        __syncthreads();
        const int idx = s_idx;
        if (idx < 0) {
            if (tid == 0) atomicAdd(&ring.exits[idx == -3 ? 0 : 1], 1);
            return;
        }
        const SlotEntry e = s_entry;
        const int gi = (e.geo >= 0 && e.geo < ring.n_geos) ? e.geo : 0;
        const BatchGeo g = ring.geos[gi];
        // the launch's shared memory is sized for max_nb nodes; a smaller lattice uses its prefix
        for (int k = tid; k < g.nb && k < max_nb; k += blockDim.x) sm.solid[k] = g.solid ? g.solid[k] : 0;
        __syncthreads();
        if (tid == 0 && g.nb <= max_nb) make_order(g, sm.order, sm.n_fluid, sm.solid);
        __syncthreads();
        BatchResult o;
        if (g.nb > max_nb || g.nb > NPT * (int)blockDim.x) {
            o.label = 0;
            o.decided_step = 0;
            o.steps_done = 0;
            o.status = 8;  // rejected: lattice does not fit this lane
            o.margin = 0;
            o.energy = 0;
        } else {
            o = batch_one_run<P, Q, NPT>(g, e.run, sm, nullptr);
        }
        if (tid == 0) {
            SlotDone *d = ring.done + (idx % ring.capacity);
            d->res = o;
            st_release_sys(&d->seq, idx + 1);
        }
    }
}

}  // namespace erlbm
