// collide_pair.cuh -- the compensated FP32 form: populations stored as an unevaluated sum of two floats.
//
// A population is g = f - w held as (hi, lo) with hi = fl(hi + lo), about 48 significant bits, in
// 8 bytes (the FP64 path's footprint).  The D2Q9 collision is the FP32-shifted one (collide_fp32.cuh,
// the same sequence of operations) with every operation carried in float-float arithmetic on the
// FP32 pipe, and the lattice constants and relaxation coefficients exact to float-float precision.
// Rounding only a part of it to FP32 is not enough: in an under-resolved shear layer the
// non-equilibrium parts and the increments reach ~1e-2, and their FP32 rounding alone is as large as
// that of FP32 storage.
//
// Float-float operations are the error-free transformations of Knuth (two-sum), Dekker (fast
// two-sum, and the product split by an fma), each an explicitly rounded FP32 intrinsic, so the
// sequence is fixed and a CPU restatement in IEEE single precision reproduces it bit for bit.
#pragma once

#include "collide_fp32.cuh"
#include "lattice.cuh"

namespace erlbm {
namespace pair32 {

struct DS {
    float hi, lo;
};

// s + e = a + b exactly (Knuth's two-sum, 6 operations)
__device__ __forceinline__ DS two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}
// s + e = a + b for |a| >= |b| (Dekker's fast two-sum, 3 operations); the renormalisation step
__device__ __forceinline__ DS fast_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ DS add(DS a, DS b)
{
    const DS s = two_sum(a.hi, b.hi);
    return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ DS neg(DS a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ DS sub(DS a, DS b) { return add(a, neg(b)); }
// Lane arithmetic in float-float for shifted::collide9l: the D2Q9 update of the FP32 form, every
// operation of it carried as an unevaluated float pair, with exact lattice constants (kc) and
// relaxation coefficients (ck).  fma(a, b, c) is mul then add (two float-float roundings).
struct LaneDS {
    using V = DS;
    static __device__ __forceinline__ V c(float x) { return {x, 0.f}; }
    static __device__ __forceinline__ V ck(DS x) { return x; }
    static __device__ __forceinline__ V kc(float, double dv)
    {
        const float hi = (float)dv;
        return {hi, (float)(dv - (double)hi)};
    }
    static __device__ __forceinline__ V add(V a, V b) { return pair32::add(a, b); }
    static __device__ __forceinline__ V sub(V a, V b) { return pair32::add(a, pair32::neg(b)); }
    static __device__ __forceinline__ V neg(V a) { return pair32::neg(a); }
    // Dekker's product: the exact hi x hi split by an fma, the cross terms added (lo x lo left out)
    static __device__ __forceinline__ V mul(V a, V b)
    {
        const float p = __fmul_rn(a.hi, b.hi);
        const float e = __fmaf_rn(a.lo, b.hi, __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.hi, b.hi, -p)));
        return fast_two_sum(p, e);
    }
    static __device__ __forceinline__ V fma(V a, V b, V d) { return add(mul(a, b), d); }
    // one Newton step from the FP32 reciprocal: y = y0 + y0 (1 - a y0)
    static __device__ __forceinline__ V rcp(V a)
    {
        const V y0 = c(shifted::rcp_rn(a.hi));
        return add(y0, mul(y0, sub(c(1.f), mul(a, y0))));
    }
};

// Relaxation coefficients of the float-float lane: the values of shifted::Coef formed in FP64 and
// split into float pairs (hi = float, lo = the float of the remainder).
struct CoefDS {
    DS kd, d1, nkc, kh, d1t, nkct;
};

__host__ __device__ inline DS split(double v)
{
    const float hi = (float)v;
    return {hi, (float)(v - (double)hi)};
}

__host__ __device__ inline CoefDS make_coef_ds(const Relax &R)
{
    const double d1 = 2.0 - R.inv_tau;
    double kd = 0.0, nkc = 0.0;
    if (R.op == OP_REG) {
        kd = -1.0;
        nkc = -1.0;
    } else if (R.op == OP_EXTREG) {
        kd = R.omega_gt1 - 1.0;
        nkc = -(1.0 + R.omega_gt1);
    }
    CoefDS k;
    k.kd = split(kd);
    k.d1 = split(d1);
    k.nkc = split(nkc);
    k.kh = split(0.5 * kd);
    k.d1t = split(-2.0 / 3.0 * d1);
    k.nkct = split(-2.0 / 3.0 * nkc);
    return k;
}

template <int OP>
__device__ __forceinline__ void collide9(DS g[9], const CoefDS &k)
{
    static_assert(OP != OP_MRT, "MRT has no compensated form");
    shifted::collide9l<LaneDS, OP, CoefDS>(g, k);
}

}  // namespace pair32

// Precision policy of the compensated form (T = float2: x = hi, y = lo).  Populations cross the
// ABI as FP64 f = w + hi + lo.  Queries (energy, density, velocity) are evaluated in FP64 from
// hi + lo, which is exact in double.
struct PrecPair32 {
    using T = float2;
    template <int Q>
    __device__ static __forceinline__ T from_f(double f, int i)
    {
        const double d = f - Lat<Q>::w(i);
        const float hi = (float)d;
        return make_float2(hi, (float)(d - (double)hi));
    }
    template <int Q>
    __device__ static __forceinline__ double to_f(T v, int i)
    {
        return ((double)v.x + (double)v.y) + Lat<Q>::w(i);
    }
    template <int Q>
    __device__ static __forceinline__ void macro(const T *f, double &rho, double &ux, double &uy, double &uz)
    {
        double s = 0.0, mx = 0.0, my = 0.0, mz = 0.0;
#pragma unroll
        for (int i = 0; i < Q; i++) {
            const double v = to_f<Q>(f[i], i);
            s += v;
            mx += Lat<Q>::cx(i) * v;
            my += Lat<Q>::cy(i) * v;
            mz += Lat<Q>::cz(i) * v;
        }
        rho = s;
        const double inv = s != 0.0 ? 1.0 / s : 0.0;
        ux = mx * inv;
        uy = my * inv;
        uz = mz * inv;
    }
    template <int Q>
    __device__ static __forceinline__ double density(const T *f)
    {
        double s = 0.0;
#pragma unroll
        for (int i = 0; i < Q; i++) s += to_f<Q>(f[i], i);
        return s;
    }
    template <int Q>
    __device__ static __forceinline__ double energy(const T *f)
    {
        double rho, ux, uy, uz;
        macro<Q>(f, rho, ux, uy, uz);
        return 0.5 * (ux * ux + uy * uy + uz * uz);
    }
};

}  // namespace erlbm
