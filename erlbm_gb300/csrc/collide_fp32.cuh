// collide_fp32.cuh -- FP32 collision on shifted populations g_i = f_i - w_i (rho_ref = 1).
//
// Same operators as the reference (coll_Ext_Reg, Collision_operators.cpp:1182-1307; coll_Reg,
// :860-967; coll_BGK, :12-49), rewritten for FP32 storage and arithmetic.  In exact arithmetic
//   f* = f_eq + w_1 f1 + w_gt1 (f - f_eq - f1)  =  f + k_d d + k_f f1,   d = f - f_eq,
// with k_d = w_gt1 - 1, k_f = w_1 - w_gt1 (RLBM: k_d = -1, k_f = w_1; BGK: k_d = -1/tau, k_f = 0).
// The increment form is what keeps FP32 honest: the update adds a small correction to the stored
// population instead of rebuilding it from O(1) pieces.  The viscosity is set by the factor the
// Hermite part f1 is multiplied by, w_1 = 1 - 1/tau = delta_1 - 1 with delta_1 = 2 - 1/tau, and
// at the maps' lowest viscosity delta_1 is ~1e-4: as the sum of two O(1) FP32 coefficients it
// would carry only ~4 significant digits.  So the update is written with delta_1 itself:
//   f* = f + [delta_1 f1 + k_d (d - f1) - 2 f1]            (E-RLBM, RLBM: k_d = w_gt1 - 1)
//      = f + [delta_1 f1 - k_c f1 + k_d d],  k_c = 2 + k_d = 1 + w_gt1 (formed in FP64, rounded once)
//   f* = f + [delta d - 2 d],  delta = 2 - 1/tau           (BGK)
// The second E-RLBM / RLBM form is the one evaluated: for an opposite pair with d = (D +- DO) / 2 the
// part common to both members, delta_1 f1 - k_c f1 + (k_d / 2) D, is formed once and the odd part
// (k_d / 2) DO added and subtracted by one fma each, so delta_1 f1 still enters as its own exactly
// multiplied term.
//
// Each opposite pair (i, j) is split into an even part e = (g_i + g_j)/2 and an odd part
// o = (g_i - g_j)/2 (both exact; the updates carry them, and the non-equilibrium parts, at twice this
// scale, which rounds identically and saves the scalings).  Then
//   drho = g_0 + 2 sum e,   m = 2 sum c o,   u = m / (1 + drho),
//   non-equilibrium even part  de = e - w (drho + 4.5 (c.m)(c.u) - 1.5 m.u),
//   non-equilibrium odd part   do = o - 3 w (c.m),
//   Pi^neq = 2 sum c c de  (odd parts do not enter even moments),  f1 = 4.5 w Q_i : Pi^neq.
// The non-equilibrium part must carry no mass and no momentum.  That holds in exact arithmetic,
// but the rounding of c.m = m_x +- m_y is a fixed function of the local state, so in a region of
// uniform flow it would push momentum the same way every step (a drift linear in time, measured at
// ~1e-8 relative velocity per step on the double shear layer).  So the axis pairs' odd parts and
// the rest population's even part are not computed but closed:
//   do_x = -(sum of the other c_x do),  ...,  de_0 = -2 sum de,
// which makes the update conserve mass and momentum up to the rounding of small quantities; the
// remaining error is the unbiased rounding of the stored populations (growth ~ sqrt(t)).
#pragma once

#include "lattice.cuh"

namespace erlbm {
namespace shifted {

// Increment coefficients, formed in FP64 and rounded once: kd = w_gt1 - 1 (unused by BGK and MRT),
// d1 = 2 - 1/tau (delta_1, or delta for BGK), nkc = -(1 + w_gt1) = -(2 + kd); kh = kd / 2 (exact);
// d1t = -2/3 d1 and nkct = -2/3 nkc, the D2Q9 rest population's factors of the trace (its f1 is
// -2/3 tr).
struct Coef {
    float kd, d1, nkc, kh, d1t, nkct;
};

__host__ __device__ inline Coef make_coef(const Relax &R)
{
    Coef k;
    const double d1 = 2.0 - R.inv_tau;
    double nkc = 0.0;
    k.d1 = (float)d1;
    if (R.op == OP_BGK || R.op == OP_MRT) {
        k.kd = 0.f;
    } else if (R.op == OP_REG) {
        k.kd = -1.f;
        nkc = -1.0;
    } else {
        k.kd = (float)(R.omega_gt1 - 1.0);
        nkc = -(1.0 + R.omega_gt1);
    }
    k.nkc = (float)nkc;
    k.kh = 0.5f * k.kd;
    k.d1t = (float)(-2.0 / 3.0 * d1);
    k.nkct = (float)(-2.0 / 3.0 * nkc);
    return k;
}

// 1 / b rounded to nearest: the hardware's approximate reciprocal refined by one fused correction step
// (Markstein's method: e = 1 - b y, y' = y + y e, both as single roundings).  Checked against
// __frcp_rn on every float whose exponent field lies in [1, 252] (|b| in [2^-126, 2^126)): identical
// bits.  Outside that range (zero, subnormals, |b| >= 2^126, infinities, NaN) the approximation's
// flush-to-zero and overflow would differ, so those take __frcp_rn.  3 FP32 operations instead of
// the ~10 of __frcp_rn in the common case.
__device__ __forceinline__ float rcp_rn(float b)
{
    const unsigned ex = (__float_as_uint(b) >> 23) & 0xffu;
    if (ex - 1u > 251u) return __frcp_rn(b);
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(b));
    const float e = __fmaf_rn(-b, y, 1.0f);
    return __fmaf_rn(y, e, y);
}

// ------------------------------------------------------------------------------------------------
// D2Q9: pairs X = (1,2) c = (1,0); Y = (3,4) c = (0,1); P = (5,6) c = (1,1); M = (7,8) c = (1,-1)
// ------------------------------------------------------------------------------------------------

__device__ __forceinline__ void moments9(const float g[9], float &drho, float &mx, float &my, float &ux, float &uy)
{
    const float eX = g[1] + g[2], eY = g[3] + g[4], eP = g[5] + g[6], eM = g[7] + g[8];
    const float oX = g[1] - g[2], oY = g[3] - g[4], oP = g[5] - g[6], oM = g[7] - g[8];
    drho = g[0] + ((eX + eY) + (eP + eM));
    mx = oX + (oP + oM);
    my = oY + (oP - oM);
    const float inv = __frcp_rn(1.f + drho);
    ux = mx * inv;
    uy = my * inv;
}

// Lane arithmetic of the D2Q9 update, written once for one node (LaneF1: float) and for two nodes
// in the halves of a float2 (LaneF2: Blackwell's packed FP32x2 FFMA2 / FADD2 / FMUL2, which issue
// one instruction for both).  Every operation is an explicitly rounded intrinsic (nothing is left to
// the compiler's contraction), so both forms compute the same bits.
struct LaneF1 {
    using V = float;
    static __device__ __forceinline__ V c(float x) { return x; }
    static __device__ __forceinline__ V ck(float x) { return x; }  // a relaxation coefficient
    // a lattice constant: its FP32 value (fv, as the expression the FP32 update has always used) or,
    // for a wider lane, the exact value dv
    static __device__ __forceinline__ V kc(float fv, double) { return fv; }
    static __device__ __forceinline__ V add(V a, V b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ V sub(V a, V b) { return __fsub_rn(a, b); }
    static __device__ __forceinline__ V mul(V a, V b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ V fma(V a, V b, V d) { return __fmaf_rn(a, b, d); }
    static __device__ __forceinline__ V neg(V a) { return -a; }
    static __device__ __forceinline__ V rcp(V a) { return rcp_rn(a); }
};

struct LaneF2 {
    using V = float2;
    static __device__ __forceinline__ V c(float x) { return make_float2(x, x); }
    static __device__ __forceinline__ V ck(float x) { return make_float2(x, x); }
    static __device__ __forceinline__ V kc(float fv, double) { return make_float2(fv, fv); }
    static __device__ __forceinline__ V add(V a, V b) { return __fadd2_rn(a, b); }
    static __device__ __forceinline__ V sub(V a, V b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); }
    static __device__ __forceinline__ V mul(V a, V b) { return __fmul2_rn(a, b); }
    static __device__ __forceinline__ V fma(V a, V b, V d) { return __ffma2_rn(a, b, d); }
    static __device__ __forceinline__ V neg(V a) { return make_float2(-a.x, -a.y); }
    // rcp_rn on both halves: one range test for the pair, the correction step in packed form
    static __device__ __forceinline__ V rcp(V a)
    {
        const unsigned ex = (__float_as_uint(a.x) >> 23) & 0xffu, ey = (__float_as_uint(a.y) >> 23) & 0xffu;
        if ((ex - 1u > 251u) | (ey - 1u > 251u)) return make_float2(rcp_rn(a.x), rcp_rn(a.y));
        float2 y;
        asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y.x) : "f"(a.x));
        asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y.y) : "f"(a.y));
        const float2 e = __ffma2_rn(make_float2(-a.x, -a.y), y, make_float2(1.f, 1.f));
        return __ffma2_rn(y, e, y);
    }
};

// Update of one opposite pair from twice its even/odd non-equilibrium parts, D = 2 de and DO = 2 do,
// and f1: the increment is formed from the small quantities first and added to the stored population
// once, so only that last addition rounds at the scale of g.  The halving of D and DO is folded into
// the coefficient k_d / 2 (exact), which rounds exactly as the half-scale form would.  The rest
// population (update_rest_l) takes its parts at their own scale.
template <class M, int OP, class K>
__device__ __forceinline__ void update_pair2_l(typename M::V &gi, typename M::V &gj, typename M::V D,
                                               typename M::V DO, typename M::V f1, const K &k)
{
    using V = typename M::V;
    const V d1 = M::ck(k.d1), m2 = M::c(-2.f), half = M::c(0.5f);
    if (OP == OP_BGK) {
        const V DI = M::add(D, DO), DJ = M::sub(D, DO);
        gi = M::fma(half, M::fma(d1, DI, M::mul(m2, DI)), gi);
        gj = M::fma(half, M::fma(d1, DJ, M::mul(m2, DJ)), gj);
    } else {
        // every product here feeds an explicit fma, so there is nothing left for contraction to fuse
        const V kh = M::ck(k.kh);
        const V cm = M::fma(d1, f1, M::fma(M::ck(k.nkc), f1, M::mul(kh, D)));
        gi = M::add(gi, M::fma(kh, DO, cm));
        gj = M::add(gj, M::fma(M::neg(kh), DO, cm));
    }
}

template <class M, int OP, class K>
__device__ __forceinline__ typename M::V update_rest_l(typename M::V g0, typename M::V de0, typename M::V f10,
                                                       const K &k)
{
    const typename M::V d1 = M::ck(k.d1), m2 = M::c(-2.f);
    if (OP == OP_BGK) return M::add(g0, M::fma(d1, de0, M::mul(m2, de0)));
    return M::add(g0, M::fma(d1, f10, M::fma(M::ck(k.nkc), f10, M::mul(M::ck(k.kd), de0))));
}

// The D2Q9 update with the pair sums and differences kept at twice their scale: E = g_i + g_j = 2e,
// O = g_i - g_j = 2o, and the non-equilibrium parts D = 2 de, DO = 2 do.  Scaling by 2 or 1/2 is exact
// in binary floating point (the magnitudes here are far from the subnormal range), so every rounded
// operation below yields exactly twice (or, for the moments, exactly) what the half-scale form yields:
// the same bits with 13 multiplications fewer.  The final 1/2 is folded into the fma that consumes D.
template <class M, int OP, class K = Coef>
__device__ __forceinline__ void collide9l(typename M::V g[9], const K &k)
{
    using V = typename M::V;
    constexpr float W1 = 1.f / 9.f, W2 = 1.f / 36.f, M3W2 = -3.f * (1.f / 36.f);
    const V half = M::c(0.5f), two = M::c(2.f);
    const V EX = M::add(g[1], g[2]), OX = M::sub(g[1], g[2]);
    const V EY = M::add(g[3], g[4]), OY = M::sub(g[3], g[4]);
    const V EP = M::add(g[5], g[6]), OP_ = M::sub(g[5], g[6]);
    const V EM = M::add(g[7], g[8]), OM = M::sub(g[7], g[8]);
    const V drho = M::add(M::add(M::add(EX, EY), M::add(EP, EM)), g[0]);
    const V mx = M::add(OX, M::add(OP_, OM));
    const V my = M::add(OY, M::sub(OP_, OM));
    const V inv = M::rcp(M::add(M::c(1.f), drho));
    const V ux = M::mul(mx, inv), uy = M::mul(my, inv);
    // the equilibrium's quadratic parts 4.5 (c.m)(c.u) - 1.5 m.u from a = m_x u_x, b = m_y u_y and
    // c = m_x u_y + m_y u_x: 4.5 a - 1.5 (a + b) on the x axis, 3 (a + b) +- 4.5 c on the diagonals
    const V a = M::mul(mx, ux), b = M::mul(my, uy);
    const V sab = M::fma(mx, ux, b);  // a + b as one rounding (no product is left to an add)
    const V mu15 = M::mul(M::c(-1.5f), sab);
    const V cxy = M::fma(mx, uy, M::mul(my, ux));
    const V s3 = M::mul(M::c(3.f), sab);
    const V k45 = M::c(4.5f), mw1x2 = M::kc(-2.f * W1, -2.0 / 9.0), mw2x2 = M::kc(-2.f * W2, -2.0 / 36.0);
    // twice the even non-equilibrium parts
    const V DX = M::fma(mw1x2, M::fma(k45, a, mu15), M::fma(mw1x2, drho, EX));
    const V DY = M::fma(mw1x2, M::fma(k45, b, mu15), M::fma(mw1x2, drho, EY));
    const V cmP = M::add(mx, my), cmM = M::sub(mx, my);
    const V DP = M::fma(mw2x2, M::fma(k45, cxy, s3), M::fma(mw2x2, drho, EP));
    const V DM = M::fma(mw2x2, M::fma(M::c(-4.5f), cxy, s3), M::fma(mw2x2, drho, EM));
    // twice the odd non-equilibrium parts; the axis pairs close the momentum
    const V DOP = M::fma(M::kc(2.f * M3W2, -1.0 / 6.0), cmP, OP_);
    const V DOM = M::fma(M::kc(2.f * M3W2, -1.0 / 6.0), cmM, OM);
    const V DOX = M::neg(M::add(DOP, DOM));
    const V DOY = M::neg(M::sub(DOP, DOM));
    if constexpr (OP == OP_MRT) {
        const V deX = M::mul(half, DX), deY = M::mul(half, DY), deP = M::mul(half, DP), deM = M::mul(half, DM);
        const V doP = M::mul(half, DOP), doM = M::mul(half, DOM);
        const V A = M::add(deX, deY), B = M::add(deP, deM);
        const V hE = M::mul(M::c((float)(MRT9_SE / 6.0)), M::fma(two, B, A));
        const V hP = M::mul(M::c((float)(MRT9_SEPS / 6.0)), M::fma(M::c(-2.f), A, M::neg(B)));
        const V sX = M::sub(deX, deY), sP = M::sub(deP, deM);
        const V hd = M::c(-0.5f * k.d1);
        const V vX = M::fma(hd, sX, sX), vP = M::fma(hd, sP, sP);
        const V ax = M::fma(two, hP, hE), ap = M::neg(M::fma(two, hE, hP));
        const V xX = M::sub(ax, vX), xY = M::add(ax, vX), xP = M::sub(ap, vP), xM = M::add(ap, vP);
        const V sq = M::c((float)-MRT9_SQ);
        const V qP = M::mul(sq, doP), qM = M::mul(sq, doM);
        const V qX = M::neg(M::add(qP, qM)), qY = M::neg(M::sub(qP, qM));
        g[0] = M::add(g[0], M::mul(M::c(-2.f), M::add(M::add(xX, xY), M::add(xP, xM))));
        g[1] = M::add(g[1], M::add(xX, qX));
        g[2] = M::add(g[2], M::sub(xX, qX));
        g[3] = M::add(g[3], M::add(xY, qY));
        g[4] = M::add(g[4], M::sub(xY, qY));
        g[5] = M::add(g[5], M::add(xP, qP));
        g[6] = M::add(g[6], M::sub(xP, qP));
        g[7] = M::add(g[7], M::add(xM, qM));
        g[8] = M::add(g[8], M::sub(xM, qM));
        return;
    }
    const V zero = M::c(0.f);
    if constexpr (OP == OP_BGK) {
        const V de0 = M::neg(M::add(M::add(DX, DY), M::add(DP, DM)));
        g[0] = update_rest_l<M, OP>(g[0], de0, zero, k);
        update_pair2_l<M, OP>(g[1], g[2], DX, DOX, zero, k);
        update_pair2_l<M, OP>(g[3], g[4], DY, DOY, zero, k);
        update_pair2_l<M, OP>(g[5], g[6], DP, DOP, zero, k);
        update_pair2_l<M, OP>(g[7], g[8], DM, DOM, zero, k);
        return;
    }
    // Pi^neq (twice) through the sums sxy = D_X + D_Y and sd = D_P + D_M: tr = sxy + 2 sd,
    // pxx - pyy = D_X - D_Y, the rest population's closure de0 = -(sxy + sd); f1 (f1X = pxx / 3 -
    // pyy / 6 written as (pxx - pyy) / 4 + tr / 12; f1_0 = -2/3 tr enters through d1t and nkct)
    const V sxy = M::add(DX, DY), sd = M::add(DP, DM);
    const V tr = M::fma(M::c(2.f), sd, sxy);
    const V de0 = M::neg(M::add(sxy, sd));
    const V t12 = M::mul(tr, M::kc(1.f / 12.f, 1.0 / 12.0));
    const V dxy = M::sub(DX, DY), pxy = M::sub(DP, DM);
    const V f1X = M::fma(dxy, M::c(0.25f), t12);
    const V f1Y = M::fma(dxy, M::c(-0.25f), t12);
    const V f1P = M::fma(pxy, M::c(0.25f), t12);
    const V f1M = M::fma(pxy, M::c(-0.25f), t12);
    g[0] = M::add(g[0], M::fma(M::ck(k.d1t), tr, M::fma(M::ck(k.nkct), tr, M::mul(M::ck(k.kd), de0))));
    update_pair2_l<M, OP>(g[1], g[2], DX, DOX, f1X, k);
    update_pair2_l<M, OP>(g[3], g[4], DY, DOY, f1Y, k);
    update_pair2_l<M, OP>(g[5], g[6], DP, DOP, f1P, k);
    update_pair2_l<M, OP>(g[7], g[8], DM, DOM, f1M, k);
}

template <int OP>
__device__ __forceinline__ void collide9(float g[9], const Coef &k)
{
    collide9l<LaneF1, OP>(g, k);
}

// Two nodes at once, one in each half of a float2: the same bits as collide9 on each.
template <int OP>
__device__ __forceinline__ void collide9x2(float2 g[9], const Coef &k)
{
    collide9l<LaneF2, OP>(g, k);
}

// ------------------------------------------------------------------------------------------------
// D3Q19: pairs X (1,2), Y (3,4), Z (5,6); A (7,8) c = (1,1,0); B (9,10) c = (1,-1,0);
// C (11,12) c = (1,0,1); D (13,14) c = (1,0,-1); E (16,15) c = (0,1,1); F (17,18) c = (0,-1,1)
// ------------------------------------------------------------------------------------------------

__device__ __forceinline__ void moments19(const float g[19], float &drho, float &mx, float &my, float &mz, float &ux,
                                          float &uy, float &uz)
{
    const float oX = g[1] - g[2], oY = g[3] - g[4], oZ = g[5] - g[6], oA = g[7] - g[8], oB = g[9] - g[10];
    const float oC = g[11] - g[12], oD = g[13] - g[14], oE = g[16] - g[15], oF = g[17] - g[18];
    const float e1 = (g[1] + g[2]) + (g[3] + g[4]), e2 = (g[5] + g[6]) + (g[7] + g[8]);
    const float e3 = (g[9] + g[10]) + (g[11] + g[12]), e4 = (g[13] + g[14]) + (g[15] + g[16]);
    drho = (g[0] + (e1 + e2)) + ((e3 + e4) + (g[17] + g[18]));
    mx = (oX + (oA + oB)) + (oC + oD);
    my = (oY + (oA - oB)) + (oE - oF);
    mz = (oZ + (oC - oD)) + (oE + oF);
    const float inv = __frcp_rn(1.f + drho);
    ux = mx * inv;
    uy = my * inv;
    uz = mz * inv;
}

// The D3Q19 update in lane arithmetic (explicitly rounded operations), with the pair sums, differences
// and non-equilibrium parts at twice their scale as in the D2Q9 one: the same bits, 28 multiplications
// fewer.
template <class M, int OP>
__device__ __forceinline__ void collide19l(typename M::V g[19], const Coef &k)
{
    using V = typename M::V;
    constexpr float W1 = 1.f / 18.f, W2 = 1.f / 36.f, M3W2 = -3.f * (1.f / 36.f);
    const V EX = M::add(g[1], g[2]), OX = M::sub(g[1], g[2]);
    const V EY = M::add(g[3], g[4]), OY = M::sub(g[3], g[4]);
    const V EZ = M::add(g[5], g[6]), OZ = M::sub(g[5], g[6]);
    const V EA = M::add(g[7], g[8]), OA = M::sub(g[7], g[8]);
    const V EB = M::add(g[9], g[10]), OB = M::sub(g[9], g[10]);
    const V EC = M::add(g[11], g[12]), OC = M::sub(g[11], g[12]);
    const V ED = M::add(g[13], g[14]), OD = M::sub(g[13], g[14]);
    const V EE = M::add(g[16], g[15]), OE = M::sub(g[16], g[15]);
    const V EF = M::add(g[17], g[18]), OF = M::sub(g[17], g[18]);
    const V drho = M::add(M::add(M::add(M::add(EX, EY), M::add(EZ, EA)),
                                 M::add(M::add(EB, EC), M::add(ED, M::add(EE, EF)))), g[0]);
    const V mx = M::add(M::add(OX, M::add(OA, OB)), M::add(OC, OD));
    const V my = M::add(M::add(OY, M::sub(OA, OB)), M::sub(OE, OF));
    const V mz = M::add(M::add(OZ, M::sub(OC, OD)), M::add(OE, OF));
    const V inv = M::rcp(M::add(M::c(1.f), drho));
    const V ux = M::mul(mx, inv), uy = M::mul(my, inv), uz = M::mul(mz, inv);
    const V mu15 = M::mul(M::c(-1.5f), M::fma(mx, ux, M::fma(my, uy, M::mul(mz, uz))));
    const V mw1x2 = M::c(-2.f * W1), mw2x2 = M::c(-2.f * W2), k45 = M::c(4.5f);
    const V R1 = M::mul(mw1x2, drho), R2 = M::mul(mw2x2, drho);
    const V DX = M::fma(mw1x2, M::fma(M::mul(k45, mx), ux, mu15), M::add(EX, R1));
    const V DY = M::fma(mw1x2, M::fma(M::mul(k45, my), uy, mu15), M::add(EY, R1));
    const V DZ = M::fma(mw1x2, M::fma(M::mul(k45, mz), uz, mu15), M::add(EZ, R1));
    const V cmA = M::add(mx, my), cmB = M::sub(mx, my), cmC = M::add(mx, mz), cmD = M::sub(mx, mz);
    const V cmE = M::add(my, mz), cmF = M::sub(mz, my);
    const V DA = M::fma(mw2x2, M::fma(M::mul(k45, cmA), M::add(ux, uy), mu15), M::add(EA, R2));
    const V DB = M::fma(mw2x2, M::fma(M::mul(k45, cmB), M::sub(ux, uy), mu15), M::add(EB, R2));
    const V DC = M::fma(mw2x2, M::fma(M::mul(k45, cmC), M::add(ux, uz), mu15), M::add(EC, R2));
    const V DD = M::fma(mw2x2, M::fma(M::mul(k45, cmD), M::sub(ux, uz), mu15), M::add(ED, R2));
    const V DE = M::fma(mw2x2, M::fma(M::mul(k45, cmE), M::add(uy, uz), mu15), M::add(EE, R2));
    const V DF = M::fma(mw2x2, M::fma(M::mul(k45, cmF), M::sub(uz, uy), mu15), M::add(EF, R2));
    const V de0 = M::neg(M::add(M::add(M::add(DX, DY), M::add(DZ, DA)),
                                M::add(M::add(DB, DC), M::add(DD, M::add(DE, DF)))));
    const V m3w2x2 = M::c(2.f * M3W2);
    const V DOA = M::fma(m3w2x2, cmA, OA), DOB = M::fma(m3w2x2, cmB, OB);
    const V DOC = M::fma(m3w2x2, cmC, OC), DOD = M::fma(m3w2x2, cmD, OD);
    const V DOE = M::fma(m3w2x2, cmE, OE), DOF = M::fma(m3w2x2, cmF, OF);
    const V DOX = M::neg(M::add(M::add(DOA, DOB), M::add(DOC, DOD)));
    const V DOY = M::neg(M::add(M::sub(DOA, DOB), M::sub(DOE, DOF)));
    const V DOZ = M::neg(M::add(M::sub(DOC, DOD), M::add(DOE, DOF)));
    const V zero = M::c(0.f);
    V f10 = zero, f1X = zero, f1Y = zero, f1Z = zero, f1A = zero, f1B = zero, f1C = zero, f1D = zero, f1E = zero,
      f1F = zero;
    if (OP != OP_BGK) {
        const V pxx = M::add(M::add(DX, M::add(DA, DB)), M::add(DC, DD));
        const V pyy = M::add(M::add(DY, M::add(DA, DB)), M::add(DE, DF));
        const V pzz = M::add(M::add(DZ, M::add(DC, DD)), M::add(DE, DF));
        const V pxy = M::sub(DA, DB), pxz = M::sub(DC, DD);
        const V pyz = M::sub(DE, DF);
        const V tr3 = M::mul(M::add(M::add(pxx, pyy), pzz), M::c(1.f / 3.f));
        const V q4 = M::c(0.25f), q8 = M::c(0.125f), mq4 = M::c(-0.25f);
        f10 = M::mul(M::c(-1.5f), tr3);
        f1X = M::mul(q4, M::sub(pxx, tr3));
        f1Y = M::mul(q4, M::sub(pyy, tr3));
        f1Z = M::mul(q4, M::sub(pzz, tr3));
        const V bxy = M::mul(q8, M::sub(M::add(pxx, pyy), tr3));
        const V bxz = M::mul(q8, M::sub(M::add(pxx, pzz), tr3));
        const V byz = M::mul(q8, M::sub(M::add(pyy, pzz), tr3));
        f1A = M::fma(q4, pxy, bxy);
        f1B = M::fma(mq4, pxy, bxy);
        f1C = M::fma(q4, pxz, bxz);
        f1D = M::fma(mq4, pxz, bxz);
        f1E = M::fma(q4, pyz, byz);
        f1F = M::fma(mq4, pyz, byz);
    }
    g[0] = update_rest_l<M, OP>(g[0], de0, f10, k);
    update_pair2_l<M, OP>(g[1], g[2], DX, DOX, f1X, k);
    update_pair2_l<M, OP>(g[3], g[4], DY, DOY, f1Y, k);
    update_pair2_l<M, OP>(g[5], g[6], DZ, DOZ, f1Z, k);
    update_pair2_l<M, OP>(g[7], g[8], DA, DOA, f1A, k);
    update_pair2_l<M, OP>(g[9], g[10], DB, DOB, f1B, k);
    update_pair2_l<M, OP>(g[11], g[12], DC, DOC, f1C, k);
    update_pair2_l<M, OP>(g[13], g[14], DD, DOD, f1D, k);
    update_pair2_l<M, OP>(g[16], g[15], DE, DOE, f1E, k);
    update_pair2_l<M, OP>(g[17], g[18], DF, DOF, f1F, k);
}

template <int OP>
__device__ __forceinline__ void collide19(float g[19], const Coef &k)
{
    collide19l<LaneF1, OP>(g, k);
}

template <int Q, int OP>
__device__ __forceinline__ void collide(float *g, const Coef &k)
{
    static_assert(Q == 9 || OP != OP_MRT, "MRT is a D2Q9 operator");
    if constexpr (Q == 9)
        collide9<OP>(g, k);
    else
        collide19<OP>(g, k);
}

// 1/2 |u|^2 of a node, from the FP32 velocity in FP32 (one conversion for the FP64 energy reduction:
// on GB300 every FP64 operation and conversion is issued at a small fraction of the FP32 rate)
template <int Q>
__device__ __forceinline__ double node_energy(const float *g)
{
    if constexpr (Q == 9) {
        float drho, mx, my, ux, uy;
        moments9(g, drho, mx, my, ux, uy);
        return (double)(0.5f * fmaf(ux, ux, uy * uy));
    } else {
        float drho, mx, my, mz, ux, uy, uz;
        moments19(g, drho, mx, my, mz, ux, uy, uz);
        return (double)(0.5f * fmaf(ux, ux, fmaf(uy, uy, uz * uz)));
    }
}

// drho of a node
template <int Q>
__device__ __forceinline__ float node_drho(const float *g)
{
    float s = 0.f;
#pragma unroll
    for (int i = 0; i < Q; i++) s += g[i];
    return s;
}

// Zou-He velocity inlet (ZouHeD3Q19_vx_x, Boundary_conditions.cpp:350-436) on shifted
// populations.  With f = w + g the weight sums of the two index sets are 1/6 and 2/3 and the
// transverse corrections carry no weight, so rho = (1 + 2 G_minus + G_zero) / (1 - vx).  The
// closure (rho and rho vx / 3, rho vx / 6) is evaluated in FP64, with 1 / (1 - vx), vx / 3 and
// vx / 6 formed once per run (zou_he_prep); the small population sums and the corrections stay in
// FP32.  That keeps the FP64 work of an inlet node to a handful of multiplies: on GB300 FP64 issues
// at a small fraction of the FP32 rate.
struct ZouHe {
    double inv_1mvx, vx3, vx6;
};

__device__ __forceinline__ ZouHe zou_he_prep(double vx)
{
    ZouHe z;
    z.inv_1mvx = 1.0 / (1.0 - vx);
    z.vx3 = vx / 3.0;
    z.vx6 = vx / 6.0;
    return z;
}

__device__ __forceinline__ void zou_he(float g[19], const ZouHe &z, bool left)
{
    const float ty = ((((g[18] + g[3]) + g[16]) - g[15]) - g[4]) - g[17];
    const float tz = ((((g[17] + g[5]) + g[16]) - g[15]) - g[6]) - g[18];
    const float gz = (((g[0] + g[3]) + (g[4] + g[5])) + ((g[6] + g[15]) + (g[16] + g[17]))) + g[18];
    if (left) {
        const float gm = ((g[1] + g[7]) + (g[9] + g[11])) + g[13];
        const double rho = (1.0 + (2.0 * (double)gm + (double)gz)) * z.inv_1mvx;
        const float a3 = (float)(rho * z.vx3), a6 = (float)(rho * z.vx6);
        g[1] = g[1] + a3;
        g[7] = g[7] + fmaf(-0.5f, ty, a6);
        g[9] = g[9] + fmaf(0.5f, ty, a6);
        g[11] = g[11] + fmaf(-0.5f, tz, a6);
        g[13] = g[13] + fmaf(0.5f, tz, a6);
    } else {
        const float gp = ((g[2] + g[8]) + (g[10] + g[12])) + g[14];
        const double rho = (1.0 + (2.0 * (double)gp + (double)gz)) * z.inv_1mvx;
        const float a3 = (float)(rho * z.vx3), a6 = (float)(rho * z.vx6);
        g[2] = g[2] - a3;
        g[10] = g[10] - fmaf(0.5f, ty, a6);
        g[8] = g[8] - fmaf(-0.5f, ty, a6);
        g[14] = g[14] - fmaf(0.5f, tz, a6);
        g[12] = g[12] - fmaf(-0.5f, tz, a6);
    }
}

// ZouHeD2Q9_vx_x (Boundary_conditions.cpp:710-744) on shifted populations: the weights of the
// closure's index set sum to 1, so rho = (1 + G) / (1 - vx) with G = g0 + g3 + g4 + 2 (g2 + g8 + g6),
// and g_i = w_i (rho P - 1) with P = 1 + 3 vx + 3 vx^2 for the +x movers (rho P - 1 in FP64).  The
// FP64 products and sums are explicitly rounded, so no contraction changes them.
__device__ __forceinline__ void zou_he_d2q9(float g[9], double vx)
{
    const float G = ((g[0] + g[3]) + g[4]) + 2.f * ((g[2] + g[8]) + g[6]);
    const double rho = (1.0 + (double)G) / (1.0 - vx);
    const double vx3 = __dmul_rn(3.0, vx);
    const double P = __dadd_rn(__dadd_rn(1.0, vx3), __dmul_rn(vx3, vx));
    const double e = __dadd_rn(__dmul_rn(rho, P), -1.0);
    g[1] = (float)(e / 9.0);
    g[5] = (float)(e / 36.0);
    g[7] = (float)(e / 36.0);
}

// parabolic_D3Q19_x's node update (:456-530) on shifted populations: an opposite pair has one weight,
// so g_i = g_opp + rho vx / 3 (or / 6) and the transverse corrections carry no weight.
__device__ __forceinline__ void parabolic_d3q19(float g[19], double vx)
{
    const float ty = ((((g[18] + g[3]) + g[16]) - g[15]) - g[4]) - g[17];
    const float tz = ((((g[17] + g[5]) + g[16]) - g[15]) - g[6]) - g[18];
    const float gz = (((g[0] + g[3]) + (g[4] + g[5])) + ((g[6] + g[15]) + (g[16] + g[17]))) + g[18];
    const float gm = ((g[2] + g[8]) + (g[10] + g[12])) + g[14];
    const double rho = (1.0 + (2.0 * (double)gm + (double)gz)) / (1.0 - vx);
    const float a3 = (float)(rho * vx / 3.0), a6 = (float)(rho * vx / 6.0);
    g[1] = g[2] + a3;
    g[7] = g[8] + fmaf(-0.5f, ty, a6);
    g[9] = g[10] + fmaf(0.5f, ty, a6);
    g[11] = g[12] + fmaf(-0.5f, tz, a6);
    g[13] = g[14] + fmaf(0.5f, tz, a6);
}

}  // namespace shifted
}  // namespace erlbm
