// lattice_kernels.cuh -- single-lattice kernels, written once for both precisions.
//
// One launch = one step of the reference's loop for every node: stream (pull) from the
// post-collision populations of the previous step, boundary planes, collision, optional density
// check, store.  The pull form is the push of propag_site (LBM_functions.cpp:3886-3955) through
// the map of def_dir_prop (:1967-2311) read from the receiving side: population i of node x comes
// from x - c_i (periodic wrap) or, when that node is solid, from direction opp(i) of x itself
// (halfway bounce-back).  The buffer between launches therefore holds post-collision populations,
// which is exactly what the reference's drivers measure after the collision of their last step.
//
// Included by k_fp64.cu (P = PrecExact64) and k_fp32.cu (P = PrecShifted32).
#pragma once

#include <cfloat>
#include <climits>
#include <cstdint>

#include "collide_fp32.cuh"
#include "collide_fp64.cuh"
#include "kernels_api.h"
#include "lattice.cuh"

namespace erlbm {

struct CollParams {
    Relax R;
    shifted::Coef k;
};

// ------------------------------------------------------------------------------------------------
// Precision policies
// ------------------------------------------------------------------------------------------------

struct PrecExact64 {
    using T = double;
    template <int Q, int OP>
    __device__ static __forceinline__ void collide(T *f, const CollParams &p)
    {
        exact::collide<Q, OP>(f, p.R);
    }
    template <int Q>
    __device__ static __forceinline__ double density(const T *f)
    {
        return exact::node_density<Q>(f);
    }
    template <int Q>
    __device__ static __forceinline__ double energy(const T *f)
    {
        return exact::node_energy<Q>(f);
    }
    // calcula (LBM_functions.cpp:3518-3589)
    template <int Q>
    __device__ static __forceinline__ void macro(const T *f, double &rho, double &ux, double &uy, double &uz)
    {
        if constexpr (Q == 9) {
            exact::moments9(f, rho, ux, uy);
            uz = 0.0;
        } else {
            exact::moments19(f, rho, ux, uy, uz);
        }
    }
    // Zou-He closure constants of one inlet velocity: the exact path uses vx as the reference does
    struct ZouHe {
        double vx;
    };
    __device__ static __forceinline__ ZouHe zou_he_prep(double vx) { return ZouHe{vx}; }
    __device__ static __forceinline__ void zou_he(T *f, const ZouHe &z, bool left)
    {
        if (left)
            exact::zou_he_left(f, z.vx);
        else
            exact::zou_he_right(f, z.vx);
    }
    // ZouHeD2Q9_vx_x, and the node update of parabolic_D2Q9_x / parabolic_D3Q19_x with a profile velocity
    __device__ static __forceinline__ void zou_he9(T *f, double vx) { exact::zou_he_d2q9(f, vx); }
    template <int Q>
    __device__ static __forceinline__ void parabolic(T *f, double vx)
    {
        if constexpr (Q == 9)
            exact::zou_he_d2q9(f, vx);
        else
            exact::parabolic_d3q19(f, vx);
    }
    // convective_x (Boundary_conditions.cpp:676-703): U = calcula's vx of the inner neighbour a,
    // f = (1 / (1 + U)) (f + U f_a).
    template <int Q>
    __device__ static __forceinline__ void convective(T *f, const T *a)
    {
        double rho, U, vy, vz;
        macro<Q>(a, rho, U, vy, vz);
        const double factor = 1.0 / (1.0 + U);
#pragma unroll
        for (int i = 0; i < Q; i++) f[i] = factor * (f[i] + U * a[i]);
    }
    // devnull_rho_x (Boundary_conditions.cpp:119-125): f = f_adj * (rho / density(f_adj)).
    template <int Q>
    __device__ static __forceinline__ void outlet(T *f, double rho)
    {
        const double fator = rho / exact::node_density<Q>(f);
#pragma unroll
        for (int i = 0; i < Q; i++) f[i] = f[i] * fator;
    }
    // dist_eq(f, rho) (LBM_functions.cpp:3015-3024): f_i = w_i rho.
    template <int Q>
    __device__ static __forceinline__ void rest(T *f, double rho)
    {
#pragma unroll
        for (int i = 0; i < Q; i++) f[i] = Lat<Q>::w(i) * rho;
    }
    template <int Q>
    __device__ static __forceinline__ T from_f(double f, int) { return f; }
    template <int Q>
    __device__ static __forceinline__ double to_f(T v, int) { return v; }
};

struct PrecShifted32 {
    using T = float;
    template <int Q, int OP>
    __device__ static __forceinline__ void collide(T *f, const CollParams &p)
    {
        shifted::collide<Q, OP>(f, p.k);
    }
    template <int Q>
    __device__ static __forceinline__ double density(const T *f)
    {
        return 1.0 + (double)shifted::node_drho<Q>(f);
    }
    template <int Q>
    __device__ static __forceinline__ double energy(const T *f)
    {
        return shifted::node_energy<Q>(f);
    }
    template <int Q>
    __device__ static __forceinline__ void macro(const T *f, double &rho, double &ux, double &uy, double &uz)
    {
        float drho, mx, my, mz = 0.f, fx, fy, fz = 0.f;
        if constexpr (Q == 9)
            shifted::moments9(f, drho, mx, my, fx, fy);
        else
            shifted::moments19(f, drho, mx, my, mz, fx, fy, fz);
        rho = 1.0 + (double)drho;
        ux = fx;
        uy = fy;
        uz = fz;
    }
    using ZouHe = shifted::ZouHe;
    __device__ static __forceinline__ ZouHe zou_he_prep(double vx) { return shifted::zou_he_prep(vx); }
    __device__ static __forceinline__ void zou_he(T *f, const ZouHe &z, bool left) { shifted::zou_he(f, z, left); }
    __device__ static __forceinline__ void zou_he9(T *f, double vx) { shifted::zou_he_d2q9(f, vx); }
    template <int Q>
    __device__ static __forceinline__ void parabolic(T *f, double vx)
    {
        if constexpr (Q == 9)
            shifted::zou_he_d2q9(f, vx);
        else
            shifted::parabolic_d3q19(f, vx);
    }
    // convective_x on shifted populations: (f + U f_a) / (1 + U) - w = (g + U g_a) / (1 + U)
    template <int Q>
    __device__ static __forceinline__ void convective(T *f, const T *a)
    {
        double rho, U, vy, vz;
        macro<Q>(a, rho, U, vy, vz);
        const float u = (float)U, factor = __frcp_rn(1.f + u);
#pragma unroll
        for (int i = 0; i < Q; i++) f[i] = factor * fmaf(u, a[i], f[i]);
    }
    // devnull_rho_x on shifted populations: f = f_adj * (rho / rho_adj) becomes
    // g = g_adj + (s - 1) (g_adj + w),  s - 1 = (rho - rho_adj) / rho_adj = ((rho - 1) - drho) / (1 + drho),
    // all of it small quantities, so FP32 carries it (the error of s - 1, ~1e-7 of a ~1e-3 quantity,
    // stays far below an ulp of g).
    template <int Q>
    __device__ static __forceinline__ void outlet(T *f, double rho)
    {
        const float drho = shifted::node_drho<Q>(f);
        const float sm1 = __fdiv_rn((float)(rho - 1.0) - drho, 1.f + drho);
#pragma unroll
        for (int i = 0; i < Q; i++) f[i] = fmaf(sm1, f[i] + (float)Lat<Q>::w(i), f[i]);
    }
    template <int Q>
    __device__ static __forceinline__ void rest(T *f, double rho)
    {
#pragma unroll
        for (int i = 0; i < Q; i++) f[i] = (float)(Lat<Q>::w(i) * rho - Lat<Q>::w(i));
    }
    template <int Q>
    __device__ static __forceinline__ T from_f(double f, int i) { return (float)(f - Lat<Q>::w(i)); }
    template <int Q>
    __device__ static __forceinline__ double to_f(T v, int i) { return (double)v + Lat<Q>::w(i); }
};

// ------------------------------------------------------------------------------------------------
// Helpers
// ------------------------------------------------------------------------------------------------

__device__ __forceinline__ int wrap1(int a, int n) { return a < 0 ? a + n : (a >= n ? a - n : a); }

// Coordinates of box node `node` (x fastest); 32-bit division when the box index fits in 31 bits.
__device__ __forceinline__ void node_xyz(const Geo &g, long long node, int &x, int &y, int &z)
{
    if (g.nbox < (1LL << 31)) {
        const unsigned n = (unsigned)node, r = n / (unsigned)g.nx;
        x = (int)(n - r * (unsigned)g.nx);
        y = (int)(r % (unsigned)g.ny);
        z = (int)(r / (unsigned)g.ny);
    } else {
        x = (int)(node % g.nx);
        const long long r = node / g.nx;
        y = (int)(r % g.ny);
        z = (int)(r / g.ny);
    }
}

// Loads for kernels that read buffers they (or other CTAs of the same launch) wrote earlier in the
// launch, as the resident team loop does across steps and runs: COH loads go through L2 (ld.global.cg),
// never through the read-only path, whose lines may be stale within a launch.
template <bool COH, class T>
__device__ __forceinline__ T ldx(const T *p)
{
    if constexpr (COH)
        return __ldcg(p);
    else
        return *p;
}

// Post-stream populations of node (x, y, z) gathered from the post-collision buffer.  The source of
// direction i is node (x - c_x, y - c_y, z - c_z) with periodic wrap: its index is the node's plus
// one offset per axis, set once for the node's position.
template <class P, int Q, bool COH = false>
__device__ __forceinline__ void gather(const typename P::T *__restrict__ src, const Geo &g, int mode, int x, int y,
                                       int z, long long node, typename P::T *f)
{
    if (mode == 1) {
#pragma unroll
        for (int i = 0; i < Q; i++) f[i] = ldx<COH>(src + (long long)i * g.plane + node);
        return;
    }
    const long long nx = g.nx, nxy = (long long)g.nx * g.ny;
    // offsets to x - 1 and x + 1 (wrapped), and likewise in y and z
    const long long xm = x == 0 ? nx - 1 : -1, xp = x == g.nx - 1 ? 1 - nx : 1;
    const long long ym = y == 0 ? (long long)(g.ny - 1) * nx : -nx, yp = y == g.ny - 1 ? (long long)(1 - g.ny) * nx : nx;
    long long zm = 0, zp = 0;
    if (Q == 19) {
        zm = z == 0 ? (long long)(g.nz - 1) * nxy : -nxy;
        zp = z == g.nz - 1 ? (long long)(1 - g.nz) * nxy : nxy;
    }
#pragma unroll
    for (int i = 0; i < Q; i++) {
        const int cx = Lat<Q>::cx(i), cy = Lat<Q>::cy(i), cz = Lat<Q>::cz(i);
        const long long s = node + (cx == 1 ? xm : (cx == -1 ? xp : 0)) + (cy == 1 ? ym : (cy == -1 ? yp : 0)) +
                            (cz == 1 ? zm : (cz == -1 ? zp : 0));
        const typename P::T pulled = ldx<COH>(src + (long long)i * g.plane + s);
        if (g.solid != nullptr) {
            // both candidates are loaded before the solid byte is known (every address is a node of
            // the box), so the loads do not wait for the mask
            const typename P::T back = ldx<COH>(src + (long long)Lat<Q>::opp(i) * g.plane + node);
            f[i] = ldx<COH>(g.solid + s) ? back : pulled;
        } else {
            f[i] = pulled;
        }
    }
}

__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    return v;
}

// ------------------------------------------------------------------------------------------------
// Boundary planes.  The reference applies each plane's function to the whole plane in place, in the
// order inlet, outlet, open y plane, before the node loop; a plane that reads its inner neighbour
// sees that neighbour after the planes applied before it.  Here every node builds its own state:
// its post-stream populations (pulled), then the planes that touch it, recomputing a neighbour's
// state where a plane reads one.
// ------------------------------------------------------------------------------------------------

template <class P, int Q>
__device__ __forceinline__ void apply_inlet(typename P::T *f, const Geo &g, const BCp &bc, int y, int z)
{
    if (bc.inlet_kind == 1) {
        P::template parabolic<Q>(f, bc.profile[y + (long long)g.ny * z]);
    } else {
        if constexpr (Q == 19)
            P::zou_he(f, P::zou_he_prep(bc.u_in), bc.inlet_x < g.nx / 2);
        else
            P::zou_he9(f, bc.u_in);
    }
}

// Populations of fluid node (x, y, z) after this step's inlet and outlet planes.
template <class P, int Q, bool COH = false>
__device__ void state_after_x_planes(const typename P::T *__restrict__ src, const Geo &g, const BCp &bc, int mode,
                                     int x, int y, int z, long long node, typename P::T *f)
{
    using T = typename P::T;
    if (x == bc.outlet_x) {
        const int xn = x + ((bc.outlet_x < g.nx / 2) ? 1 : -1);
        const long long nn = node + (xn - x);
        const bool nsolid = g.solid != nullptr && ldx<COH>(g.solid + nn);
        if (bc.outlet_kind == 0) {  // devnull_rho_x: the inner neighbour, rescaled
            if (nsolid) {
                P::template rest<Q>(f, bc.rho_out);
                return;
            }
            gather<P, Q, COH>(src, g, mode, xn, y, z, nn, f);
            if (xn == bc.inlet_x) apply_inlet<P, Q>(f, g, bc, y, z);
            P::template outlet<Q>(f, bc.rho_out);
            return;
        }
        gather<P, Q, COH>(src, g, mode, x, y, z, node, f);
        if (nsolid) return;  // the reference reads no neighbour there (it would read outside the array)
        T a[Q];
        gather<P, Q, COH>(src, g, mode, xn, y, z, nn, a);
        if (xn == bc.inlet_x) apply_inlet<P, Q>(a, g, bc, y, z);
        if (bc.outlet_kind == 1) {
            if constexpr (Q == 9) {  // OpenBoundaryD2Q9_x: the populations entering from outside
                if (xn > x) {
                    f[1] = a[1];
                    f[5] = a[5];
                    f[7] = a[7];
                } else {
                    f[2] = a[2];
                    f[6] = a[6];
                    f[8] = a[8];
                }
            }
        } else {
            P::template convective<Q>(f, a);
        }
        return;
    }
    gather<P, Q, COH>(src, g, mode, x, y, z, node, f);
    if (x == bc.inlet_x) apply_inlet<P, Q>(f, g, bc, y, z);
}

// Post-boundary populations of fluid node (x, y, z): the x planes, then OpenBoundaryD2Q9_y.
template <class P, int Q, bool COH = false>
__device__ void state_after_planes(const typename P::T *__restrict__ src, const Geo &g, const BCp &bc, int mode, int x,
                                   int y, int z, long long node, typename P::T *f)
{
    state_after_x_planes<P, Q, COH>(src, g, bc, mode, x, y, z, node, f);
    if constexpr (Q == 9) {
        if (y != bc.open_y) return;
        const int yn = y + ((bc.open_y < g.ny / 2) ? 1 : -1);
        const long long nn = node + (long long)(yn - y) * g.nx;
        if (g.solid != nullptr && ldx<COH>(g.solid + nn)) return;
        typename P::T a[Q];
        state_after_x_planes<P, Q, COH>(src, g, bc, mode, x, yn, z, nn, a);
        if (yn > y) {
            f[3] = a[3];
            f[5] = a[5];
            f[8] = a[8];
        } else {
            f[4] = a[4];
            f[6] = a[6];
            f[7] = a[7];
        }
    }
}

// ------------------------------------------------------------------------------------------------
// Generic step kernel: any box, solid mask, boundary planes, density check
// ------------------------------------------------------------------------------------------------

// One node of one step: state after the planes, collision, the density check, store.  rho_bits and
// flag return the check's outcome (|rho| as a bit pattern; 1 above the limit, 2 non-finite).  The body
// of k_step, shared with the resident team loop so that both give the same bits.
template <class P, int Q, int OP, bool COH = false>
__device__ __forceinline__ void step_node(const typename P::T *__restrict__ src, typename P::T *__restrict__ dst,
                                          const Geo &g, const BCp &bc, const CollParams &prm, int mode,
                                          int check_density, double density_limit, long long node,
                                          unsigned long long &rho_bits, int &flag)
{
    using T = typename P::T;
    int x, y, z;
    node_xyz(g, node, x, y, z);
    T f[Q];
    state_after_planes<P, Q, COH>(src, g, bc, mode, x, y, z, node, f);
    P::template collide<Q, OP>(f, prm);
    if (check_density) {
        const double rho = P::template density<Q>(f);
        if (!isfinite(rho)) {
            flag = 2;
        } else {
            const double ar = fabs(rho);
            rho_bits = (unsigned long long)__double_as_longlong(ar);
            if (ar > density_limit) flag = 1;
        }
    }
#pragma unroll
    for (int i = 0; i < Q; i++) dst[(long long)i * g.plane + node] = f[i];
}

// The density check's warp reduction: lane 0 folds the warp's outcome into the run status.  Every
// lane of the warp calls it.
__device__ __forceinline__ void report_density(RunStatus *status, int step_index, unsigned long long rho_bits, int flag)
{
    const unsigned long long m = warp_max_u64(rho_bits);
    const int any = __reduce_or_sync(0xffffffffu, flag);
    if ((threadIdx.x & 31) == 0) {
        if (m) atomicMax(&status->max_abs_rho_bits, m);
        if (any) {
            atomicOr(&status->flags, any);
            atomicMin(&status->decided_step, step_index);
        }
    }
}

template <class P, int Q, int OP>
__global__ void __launch_bounds__(256) k_step(const typename P::T *__restrict__ src, typename P::T *__restrict__ dst,
                                              Geo g, BCp bc, CollParams prm, StepArgs a)
{
    if (a.stop_on_flag && a.status != nullptr) {
        // A check failed in an EARLIER step: nothing to do.  (Blocks of the failing step itself
        // still finish it, as the reference finishes the step in which it flags a node.)  One
        // value per warp, so that the warp reductions below see every lane or none.
        const int ds = __shfl_sync(0xffffffffu, *(volatile int *)&a.status->decided_step, 0);
        if (ds < a.step_index) return;
    }
    const long long node = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    bool active = node < g.nbox;
    if (active && g.solid != nullptr && g.solid[node]) active = false;
    unsigned long long rho_bits = 0;
    int flag = 0;
    if (active)
        step_node<P, Q, OP>(src, dst, g, bc, prm, a.mode, a.check_density, a.density_limit, node, rho_bits, flag);
    if (a.check_density) report_density(a.status, a.step_index, rho_bits, flag);
}

template <class P, int Q>
__global__ void __launch_bounds__(256) k_stream_only(const typename P::T *__restrict__ src,
                                                     typename P::T *__restrict__ dst, Geo g)
{
    using T = typename P::T;
    const long long node = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= g.nbox) return;
    if (g.solid != nullptr && g.solid[node]) return;
    int x, y, z;
    node_xyz(g, node, x, y, z);
    T f[Q];
    gather<P, Q>(src, g, 0, x, y, z, node, f);
#pragma unroll
    for (int i = 0; i < Q; i++) dst[(long long)i * g.plane + node] = f[i];
}

// ------------------------------------------------------------------------------------------------
// Layout conversion and per-node fields
// ------------------------------------------------------------------------------------------------

template <class P, int Q>
__global__ void __launch_bounds__(256) k_aos_to_soa(Geo g, long long n_fluid, const int *__restrict__ nof,
                                                    const double *__restrict__ aos, typename P::T *__restrict__ soa)
{
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n_fluid) return;
    const long long node = nof ? nof[p] : p;
#pragma unroll
    for (int i = 0; i < Q; i++) soa[(long long)i * g.plane + node] = P::template from_f<Q>(aos[p * Q + i], i);
}

template <class P, int Q>
__global__ void __launch_bounds__(256) k_soa_to_aos(Geo g, long long n_fluid, const int *__restrict__ nof,
                                                    const typename P::T *__restrict__ soa, double *__restrict__ aos)
{
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n_fluid) return;
    const long long node = nof ? nof[p] : p;
#pragma unroll
    for (int i = 0; i < Q; i++) aos[p * Q + i] = P::template to_f<Q>(soa[(long long)i * g.plane + node], i);
}

// Kinetic energy of fluid index p: of the post-stream state (pull from buf) when `stream`, else of the
// populations in buf.  k_stream_only followed by k_node_fields, for one node.
template <class P, int Q, bool COH = false>
__device__ __forceinline__ double node_energy_at(const typename P::T *buf, const Geo &g, const int *nof, long long p,
                                                 bool stream)
{
    using T = typename P::T;
    const long long node = nof ? ldx<COH>(nof + p) : p;
    T f[Q];
    if (stream) {
        int x, y, z;
        node_xyz(g, node, x, y, z);
        gather<P, Q, COH>(buf, g, 0, x, y, z, node, f);
    } else {
#pragma unroll
        for (int i = 0; i < Q; i++) f[i] = ldx<COH>(buf + (long long)i * g.plane + node);
    }
    return P::template energy<Q>(f);
}

template <class P, int Q>
__global__ void __launch_bounds__(256) k_node_fields(Geo g, long long n_fluid, const int *__restrict__ nof,
                                                     const typename P::T *__restrict__ buf, double *e_out,
                                                     double *rho_out, double *u_out)
{
    using T = typename P::T;
    const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n_fluid) return;
    const long long node = nof ? nof[p] : p;
    T f[Q];
#pragma unroll
    for (int i = 0; i < Q; i++) f[i] = buf[(long long)i * g.plane + node];
    if (e_out) e_out[p] = P::template energy<Q>(f);
    if (rho_out || u_out) {
        double rho, ux, uy, uz;
        P::template macro<Q>(f, rho, ux, uy, uz);
        if (rho_out) rho_out[p] = u_out ? rho : P::template density<Q>(f);
        if (u_out) {
            u_out[3 * p] = ux;
            u_out[3 * p + 1] = uy;
            u_out[3 * p + 2] = uz;
        }
    }
}

// Field of the reference's rec_* writers at every box node, x fastest (LBM_functions.cpp:4218-4470,
// 4979-5241): field 1 = calcula's (vx, vy, vz), 3 values per node; field 3 = density(); solid nodes
// are written as 0.
template <class P, int Q>
__global__ void __launch_bounds__(256) k_box_field(Geo g, const typename P::T *__restrict__ buf, int field,
                                                   double *__restrict__ out)
{
    using T = typename P::T;
    const long long node = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= g.nbox) return;
    const bool solid = g.solid != nullptr && g.solid[node];
    T f[Q];
    if (!solid) {
#pragma unroll
        for (int i = 0; i < Q; i++) f[i] = buf[(long long)i * g.plane + node];
    }
    if (field == 3) {
        out[node] = solid ? 0.0 : P::template density<Q>(f);
        return;
    }
    double rho, ux = 0.0, uy = 0.0, uz = 0.0;
    if (!solid) P::template macro<Q>(f, rho, ux, uy, uz);
    out[3 * node] = ux;
    out[3 * node + 1] = uy;
    out[3 * node + 2] = uz;
}

// ------------------------------------------------------------------------------------------------
// Launch helpers
// ------------------------------------------------------------------------------------------------

inline unsigned blocks_for(long long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

template <class P>
int box_field_any(int q, const Geo &g, const typename P::T *buf, int field, double *out, cudaStream_t s)
{
    const unsigned nb = blocks_for(g.nbox, 256);
    if (q == 9)
        k_box_field<P, 9><<<nb, 256, 0, s>>>(g, buf, field, out);
    else if (q == 19)
        k_box_field<P, 19><<<nb, 256, 0, s>>>(g, buf, field, out);
    else
        return -1;
    return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

template <class P, int Q>
int step_dispatch(int op, const Geo &g, const BCp &bc, const Relax &R, const StepArgs &a,
                  const typename P::T *src, typename P::T *dst, cudaStream_t s)
{
    CollParams prm;
    prm.R = R;
    prm.k = shifted::make_coef(R);
    const unsigned nb = blocks_for(g.nbox, 256);
    switch (op) {
    case OP_BGK:
        k_step<P, Q, OP_BGK><<<nb, 256, 0, s>>>(src, dst, g, bc, prm, a);
        break;
    case OP_MRT:
        if constexpr (Q == 9) {
            k_step<P, Q, OP_MRT><<<nb, 256, 0, s>>>(src, dst, g, bc, prm, a);
            break;
        } else {
            return -1;
        }
    case OP_REG:
        k_step<P, Q, OP_REG><<<nb, 256, 0, s>>>(src, dst, g, bc, prm, a);
        break;
    case OP_EXTREG:
        k_step<P, Q, OP_EXTREG><<<nb, 256, 0, s>>>(src, dst, g, bc, prm, a);
        break;
    default:
        return -1;
    }
    return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

template <class P>
int step_any(int q, int op, const Geo &g, const BCp &bc, const Relax &R, const StepArgs &a,
             const typename P::T *src, typename P::T *dst, cudaStream_t s)
{
    if (q == 9) return step_dispatch<P, 9>(op, g, bc, R, a, src, dst, s);
    if (q == 19) return step_dispatch<P, 19>(op, g, bc, R, a, src, dst, s);
    return -1;
}

template <class P>
int stream_only_any(int q, const Geo &g, const typename P::T *src, typename P::T *dst, cudaStream_t s)
{
    const unsigned nb = blocks_for(g.nbox, 256);
    if (q == 9)
        k_stream_only<P, 9><<<nb, 256, 0, s>>>(src, dst, g);
    else if (q == 19)
        k_stream_only<P, 19><<<nb, 256, 0, s>>>(src, dst, g);
    else
        return -1;
    return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

template <class P>
int aos_to_soa_any(int q, const Geo &g, long long n, const int *nof, const double *aos, typename P::T *soa,
                   cudaStream_t s)
{
    if (n == 0) return 0;
    const unsigned nb = blocks_for(n, 256);
    if (q == 9)
        k_aos_to_soa<P, 9><<<nb, 256, 0, s>>>(g, n, nof, aos, soa);
    else if (q == 19)
        k_aos_to_soa<P, 19><<<nb, 256, 0, s>>>(g, n, nof, aos, soa);
    else
        return -1;
    return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

template <class P>
int soa_to_aos_any(int q, const Geo &g, long long n, const int *nof, const typename P::T *soa, double *aos,
                   cudaStream_t s)
{
    if (n == 0) return 0;
    const unsigned nb = blocks_for(n, 256);
    if (q == 9)
        k_soa_to_aos<P, 9><<<nb, 256, 0, s>>>(g, n, nof, soa, aos);
    else if (q == 19)
        k_soa_to_aos<P, 19><<<nb, 256, 0, s>>>(g, n, nof, soa, aos);
    else
        return -1;
    return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

template <class P>
int node_fields_any(int q, const Geo &g, long long n, const int *nof, const typename P::T *buf, double *e,
                    double *rho, double *u, cudaStream_t s)
{
    if (n == 0) return 0;
    const unsigned nb = blocks_for(n, 256);
    if (q == 9)
        k_node_fields<P, 9><<<nb, 256, 0, s>>>(g, n, nof, buf, e, rho, u);
    else if (q == 19)
        k_node_fields<P, 19><<<nb, 256, 0, s>>>(g, n, nof, buf, e, rho, u);
    else
        return -1;
    return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

}  // namespace erlbm

namespace erlbm {

// ------------------------------------------------------------------------------------------------
// Initial populations written directly into a device SoA buffer (post-stream state of step 0).
// Trig values come from host tables so that the FP64 path reproduces the host programs bit for bit.
// ------------------------------------------------------------------------------------------------

// inicializa_taylor_green (main_taylor-green.cpp:57-100), D2Q9, Poisson density and f_eq + f1.
// tab: [s2 | c2 | c4 | ck] of L doubles each: sin(2 pi x / L), cos(2 pi x / L), cos(4 pi x / L),
// cos(k x) with k = 2 pi / L, evaluated as the reference writes them.
template <class P, bool COH = false>
__device__ __forceinline__ void init_tg2d_node(typename P::T *buf, const Geo &g, const double *tab, double u0,
                                               double tau, double k, long long node)
{
    const int L = g.nx;
    const int x = (int)(node % L), y = (int)(node / L);
    const double *s2 = tab, *c2 = tab + L, *c4 = tab + 2 * L, *ck = tab + 3 * L;
    const double cs2 = 1. / 3.;
    const double rho = 1.0 + 0.75 * u0 * u0 * (ldx<COH>(c4 + x) + ldx<COH>(c4 + y));
    const double ux = u0 * ldx<COH>(s2 + x) * ldx<COH>(c2 + y);
    const double uy = -u0 * ldx<COH>(c2 + x) * ldx<COH>(s2 + y);
    double f[9];
    exact::equilibrium9(rho, ux, uy, f);
    const double Sxx = 2. * u0 * k * ldx<COH>(ck + x) * ldx<COH>(ck + y);
    const double Pxx = -rho * cs2 * tau * Sxx;
    const double Pyy = -Pxx;
#pragma unroll
    for (int i = 0; i < 9; i++) {
        const double cx = Lat<9>::cx(i), cy = Lat<9>::cy(i);
        f[i] += Lat<9>::w(i) / (2. * cs2 * cs2) * ((cx * cx - cs2) * Pxx + (cy * cy - cs2) * Pyy);
    }
#pragma unroll
    for (int i = 0; i < 9; i++) buf[(long long)i * g.plane + node] = P::template from_f<9>(f[i], i);
}

template <class P>
__global__ void __launch_bounds__(256) k_init_tg2d(typename P::T *buf, Geo g, const double *__restrict__ tab,
                                                   double u0, double tau, double k)
{
    const long long node = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= g.nbox) return;
    init_tg2d_node<P>(buf, g, tab, u0, tau, k, node);
}

// Three-dimensional Taylor-Green equilibrium (no driver in the reference; defined here):
// rho = 1, u = U0 (sin kx cos ky cos kz, -cos kx sin ky cos kz, 0).  tab: [s | c] of L doubles.
template <class P, bool COH = false>
__device__ __forceinline__ void init_tg3d_node(typename P::T *buf, const Geo &g, const double *tab, double u0,
                                               long long node)
{
    const int L = g.nx;
    const int x = (int)(node % L);
    const long long r = node / L;
    const int y = (int)(r % g.ny), z = (int)(r / g.ny);
    const double *s = tab, *c = tab + L;
    const double ux = u0 * ldx<COH>(s + x) * ldx<COH>(c + y) * ldx<COH>(c + z);
    const double uy = -u0 * ldx<COH>(c + x) * ldx<COH>(s + y) * ldx<COH>(c + z);
    double f[19];
    exact::equilibrium19(1.0, ux, uy, 0.0, f);
#pragma unroll
    for (int i = 0; i < 19; i++) buf[(long long)i * g.plane + node] = P::template from_f<19>(f[i], i);
}

template <class P>
__global__ void __launch_bounds__(256) k_init_tg3d(typename P::T *buf, Geo g, const double *__restrict__ tab,
                                                   double u0)
{
    const long long node = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= g.nbox) return;
    init_tg3d_node<P>(buf, g, tab, u0, node);
}

// Rest equilibrium f_i = w_i rho on every fluid node (main_stability-map_obstacle.cpp:81-82).
template <class P, int Q>
__device__ __forceinline__ void init_rest_node(typename P::T *buf, const Geo &g, double rho, long long node)
{
#pragma unroll
    for (int i = 0; i < Q; i++) buf[(long long)i * g.plane + node] = P::template from_f<Q>(Lat<Q>::w(i) * rho, i);
}

template <class P, int Q>
__global__ void __launch_bounds__(256) k_init_rest(typename P::T *buf, Geo g, double rho)
{
    const long long node = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= g.nbox) return;
    init_rest_node<P, Q>(buf, g, rho, node);
}

template <class P>
int init_any(int kind, int q, const Geo &g, typename P::T *buf, const double *tab, double u0, double tau, double k,
             double rho, cudaStream_t s)
{
    const unsigned nb = blocks_for(g.nbox, 256);
    if (kind == 1 && q == 9)
        k_init_tg2d<P><<<nb, 256, 0, s>>>(buf, g, tab, u0, tau, k);
    else if (kind == 4 && q == 19)
        k_init_tg3d<P><<<nb, 256, 0, s>>>(buf, g, tab, u0);
    else if (kind == 0 && q == 9)
        k_init_rest<P, 9><<<nb, 256, 0, s>>>(buf, g, rho);
    else if (kind == 0 && q == 19)
        k_init_rest<P, 19><<<nb, 256, 0, s>>>(buf, g, rho);
    else
        return -1;
    return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

}  // namespace erlbm
