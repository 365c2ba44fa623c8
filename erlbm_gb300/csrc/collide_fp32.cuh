// collide_fp32.cuh -- FP32 collision on shifted populations g_i = f_i - w_i (rho_ref = 1).
//
// Same operators as the reference (coll_Ext_Reg, Collision_operators.cpp:1182-1307; coll_Reg,
// :860-967; coll_BGK, :12-49), rewritten for storage and arithmetic in FP32 without losing the
// small quantities to cancellation against the O(w_i) rest populations:
//   drho = sum g,  m = sum c g,  u = m / (1 + drho);
//   Pi^neq_ab = sum c_a c_b g - (drho / 3) delta_ab - m_a u_b      (second moment of f_eq - w:
//               exact for the second-order equilibrium on D2Q9 and D3Q19);
//   geq_i = w_i (drho + 3 c.m + 4.5 (c.m)(c.u) - 1.5 m.u)          (= f_eq_i - w_i);
//   f1_i  = 4.5 w_i Q_i : Pi^neq,  Q_i = c c - delta / 3;
//   E-RLBM: g*_i = (1 - w_gt1) geq_i + w_gt1 g_i + (w_1 - w_gt1) f1_i
//   RLBM:   g*_i = geq_i + w_1 f1_i;   BGK: g*_i = (1 - 1/tau) g_i + geq_i / tau.
// Opposite directions share c.m c.u and f1, which halves that work.
#pragma once

#include "lattice.cuh"

namespace erlbm {
namespace shifted {

// Coefficients of the shifted update, formed in FP64 and rounded once.
struct Coef {
    float a, b, c;  // E-RLBM: a = 1 - w_gt1, b = w_gt1, c = w_1 - w_gt1; RLBM: a = 1, b = 0, c = w_1;
                    // BGK: a = 1/tau, b = 1 - 1/tau, c = 0
};

inline Coef make_coef(const Relax &R)
{
    Coef k;
    if (R.op == OP_BGK) {
        k.a = (float)R.inv_tau;
        k.b = (float)(1.0 - R.inv_tau);
        k.c = 0.f;
    } else if (R.op == OP_REG) {
        k.a = 1.f;
        k.b = 0.f;
        k.c = (float)R.omega_1;
    } else {
        k.a = (float)(1.0 - R.omega_gt1);
        k.b = (float)R.omega_gt1;
        k.c = (float)(R.omega_1 - R.omega_gt1);
    }
    return k;
}

template <int OP>
__device__ __forceinline__ float update(float geq, float g, float f1, const Coef &k)
{
    if (OP == OP_BGK) return fmaf(k.b, g, k.a * geq);
    if (OP == OP_REG) return fmaf(k.c, f1, geq);
    return fmaf(k.a, geq, fmaf(k.b, g, k.c * f1));
}

// Equilibrium deviation of an opposite pair (cm = c.m, cu = c.u of the first member).
__device__ __forceinline__ void geq_pair(float cm, float cu, float base, float w, float &ga, float &gb)
{
    const float s = fmaf(4.5f * cm, cu, base);
    const float ws = w * s;
    ga = fmaf(3.f * w, cm, ws);
    gb = fmaf(-3.f * w, cm, ws);
}

// Moments of the shifted populations; returns drho, u and the node's kinetic energy 1/2 |u|^2.
template <int Q>
struct Mom;

// ------------------------------------------------------------------------------------------------
// D2Q9
// ------------------------------------------------------------------------------------------------

__device__ __forceinline__ void moments9(const float g[9], float &drho, float &mx, float &my, float &ux, float &uy)
{
    drho = ((g[0] + (g[1] + g[2])) + (g[3] + g[4])) + ((g[5] + g[6]) + (g[7] + g[8]));
    mx = ((g[1] - g[2]) + (g[5] - g[6])) + (g[7] - g[8]);
    my = ((g[3] - g[4]) + (g[5] - g[6])) + (g[8] - g[7]);
    const float inv = __frcp_rn(1.f + drho);
    ux = mx * inv;
    uy = my * inv;
}

template <int OP>
__device__ __forceinline__ void collide9(float g[9], const Coef &k)
{
    float drho, mx, my, ux, uy;
    moments9(g, drho, mx, my, ux, uy);
    const float base = fmaf(-1.5f, fmaf(mx, ux, my * uy), drho);
    float geq[9];
    geq[0] = (4.f / 9.f) * base;
    geq_pair(mx, ux, base, 1.f / 9.f, geq[1], geq[2]);
    geq_pair(my, uy, base, 1.f / 9.f, geq[3], geq[4]);
    geq_pair(mx + my, ux + uy, base, 1.f / 36.f, geq[5], geq[6]);
    geq_pair(mx - my, ux - uy, base, 1.f / 36.f, geq[7], geq[8]);
    float f1[9];
    if (OP != OP_BGK) {
        const float a56 = g[5] + g[6], a78 = g[7] + g[8];
        const float dd = a56 + a78;
        const float c3 = drho * (1.f / 3.f);
        const float pxx = fmaf(-mx, ux, ((g[1] + g[2]) + dd) - c3);
        const float pyy = fmaf(-my, uy, ((g[3] + g[4]) + dd) - c3);
        const float pxy = fmaf(-mx, uy, a56 - a78);
        const float tr = pxx + pyy;
        f1[0] = (-2.f / 3.f) * tr;
        f1[1] = f1[2] = fmaf(pxx, 1.f / 3.f, pyy * (-1.f / 6.f));
        f1[3] = f1[4] = fmaf(pyy, 1.f / 3.f, pxx * (-1.f / 6.f));
        const float t12 = tr * (1.f / 12.f);
        f1[5] = f1[6] = fmaf(pxy, 0.25f, t12);
        f1[7] = f1[8] = fmaf(pxy, -0.25f, t12);
    }
#pragma unroll
    for (int i = 0; i < 9; i++) g[i] = update<OP>(geq[i], g[i], OP != OP_BGK ? f1[i] : 0.f, k);
}

// ------------------------------------------------------------------------------------------------
// D3Q19
// ------------------------------------------------------------------------------------------------

__device__ __forceinline__ void moments19(const float g[19], float &drho, float &mx, float &my, float &mz, float &ux,
                                          float &uy, float &uz)
{
    const float s12 = g[1] + g[2], s34 = g[3] + g[4], s56 = g[5] + g[6];
    const float s78 = g[7] + g[8], s910 = g[9] + g[10], s1112 = g[11] + g[12], s1314 = g[13] + g[14];
    const float s1516 = g[15] + g[16], s1718 = g[17] + g[18];
    drho = ((g[0] + (s12 + s34)) + (s56 + s78)) + ((s910 + s1112) + ((s1314 + s1516) + s1718));
    const float d12 = g[1] - g[2], d34 = g[3] - g[4], d56 = g[5] - g[6];
    const float d78 = g[7] - g[8], d910 = g[9] - g[10], d1112 = g[11] - g[12], d1314 = g[13] - g[14];
    const float d1615 = g[16] - g[15], d1718 = g[17] - g[18];
    mx = (d12 + (d78 + d910)) + (d1112 + d1314);
    my = (d34 + (d78 - d910)) + (d1615 - d1718);
    mz = (d56 + (d1112 - d1314)) + (d1615 + d1718);
    const float inv = __frcp_rn(1.f + drho);
    ux = mx * inv;
    uy = my * inv;
    uz = mz * inv;
}

template <int OP>
__device__ __forceinline__ void collide19(float g[19], const Coef &k)
{
    float drho, mx, my, mz, ux, uy, uz;
    moments19(g, drho, mx, my, mz, ux, uy, uz);
    const float base = fmaf(-1.5f, fmaf(mx, ux, fmaf(my, uy, mz * uz)), drho);
    float geq[19];
    constexpr float W1 = 1.f / 18.f, W2 = 1.f / 36.f;
    geq[0] = (1.f / 3.f) * base;
    geq_pair(mx, ux, base, W1, geq[1], geq[2]);
    geq_pair(my, uy, base, W1, geq[3], geq[4]);
    geq_pair(mz, uz, base, W1, geq[5], geq[6]);
    geq_pair(mx + my, ux + uy, base, W2, geq[7], geq[8]);
    geq_pair(mx - my, ux - uy, base, W2, geq[9], geq[10]);
    geq_pair(mx + mz, ux + uz, base, W2, geq[11], geq[12]);
    geq_pair(mx - mz, ux - uz, base, W2, geq[13], geq[14]);
    geq_pair(my + mz, uy + uz, base, W2, geq[16], geq[15]);
    geq_pair(mz - my, uz - uy, base, W2, geq[17], geq[18]);
    float f1[19];
    if (OP != OP_BGK) {
        const float s78 = g[7] + g[8], s910 = g[9] + g[10], s1112 = g[11] + g[12], s1314 = g[13] + g[14];
        const float s1516 = g[15] + g[16], s1718 = g[17] + g[18];
        const float c3 = drho * (1.f / 3.f);
        const float sxx = ((g[1] + g[2]) + (s78 + s910)) + (s1112 + s1314);
        const float syy = ((g[3] + g[4]) + (s78 + s910)) + (s1516 + s1718);
        const float szz = ((g[5] + g[6]) + (s1112 + s1314)) + (s1516 + s1718);
        const float pxx = fmaf(-mx, ux, sxx - c3);
        const float pyy = fmaf(-my, uy, syy - c3);
        const float pzz = fmaf(-mz, uz, szz - c3);
        const float pxy = fmaf(-mx, uy, s78 - s910);
        const float pxz = fmaf(-mx, uz, s1112 - s1314);
        const float pyz = fmaf(-my, uz, s1516 - s1718);
        const float tr3 = (pxx + pyy + pzz) * (1.f / 3.f);
        f1[0] = -0.5f * (3.f * tr3);
        f1[1] = f1[2] = 0.25f * (pxx - tr3);
        f1[3] = f1[4] = 0.25f * (pyy - tr3);
        f1[5] = f1[6] = 0.25f * (pzz - tr3);
        const float bxy = 0.125f * ((pxx + pyy) - tr3);
        f1[7] = f1[8] = fmaf(0.25f, pxy, bxy);
        f1[9] = f1[10] = fmaf(-0.25f, pxy, bxy);
        const float bxz = 0.125f * ((pxx + pzz) - tr3);
        f1[11] = f1[12] = fmaf(0.25f, pxz, bxz);
        f1[13] = f1[14] = fmaf(-0.25f, pxz, bxz);
        const float byz = 0.125f * ((pyy + pzz) - tr3);
        f1[15] = f1[16] = fmaf(0.25f, pyz, byz);
        f1[17] = f1[18] = fmaf(-0.25f, pyz, byz);
    }
#pragma unroll
    for (int i = 0; i < 19; i++) g[i] = update<OP>(geq[i], g[i], OP != OP_BGK ? f1[i] : 0.f, k);
}

template <int Q, int OP>
__device__ __forceinline__ void collide(float *g, const Coef &k)
{
    if constexpr (Q == 9)
        collide9<OP>(g, k);
    else
        collide19<OP>(g, k);
}

// 1/2 |u|^2 of a node (FP32 velocity, returned in FP64 for the FP64 energy reduction)
template <int Q>
__device__ __forceinline__ double node_energy(const float *g)
{
    if constexpr (Q == 9) {
        float drho, mx, my, ux, uy;
        moments9(g, drho, mx, my, ux, uy);
        return 0.5 * ((double)ux * ux + (double)uy * uy);
    } else {
        float drho, mx, my, mz, ux, uy, uz;
        moments19(g, drho, mx, my, mz, ux, uy, uz);
        return 0.5 * (((double)ux * ux + (double)uy * uy) + (double)uz * uz);
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
// populations, closed in FP64.  With f = w + g the weight sums of the two index sets are 1/6
// and 2/3 and the transverse corrections carry no weight, so
//   rho = (1 + 2 G_minus + G_zero) / (1 - vx).
__device__ __forceinline__ void zou_he(float g[19], double vx, bool left)
{
    const double ty = ((((double)g[18] + g[3]) + g[16]) - g[15] - g[4]) - g[17];
    const double tz = ((((double)g[17] + g[5]) + g[16]) - g[15] - g[6]) - g[18];
    const double gz = (double)g[0] + g[3] + g[4] + g[5] + g[6] + g[15] + g[16] + g[17] + g[18];
    if (left) {
        const double gm = (double)g[1] + g[7] + g[9] + g[11] + g[13];
        const double rho = (1.0 + 2.0 * gm + gz) / (1.0 - vx);
        const double a3 = rho * vx / 3.0, a6 = rho * vx / 6.0;
        g[1] = (float)(g[1] + a3);
        g[7] = (float)(g[7] + a6 - 0.5 * ty);
        g[9] = (float)(g[9] + a6 + 0.5 * ty);
        g[11] = (float)(g[11] + a6 - 0.5 * tz);
        g[13] = (float)(g[13] + a6 + 0.5 * tz);
    } else {
        const double gp = (double)g[2] + g[8] + g[10] + g[12] + g[14];
        const double rho = (1.0 + 2.0 * gp + gz) / (1.0 - vx);
        const double a3 = rho * vx / 3.0, a6 = rho * vx / 6.0;
        g[2] = (float)(g[2] - a3);
        g[10] = (float)(g[10] - a6 - 0.5 * ty);
        g[8] = (float)(g[8] - a6 + 0.5 * ty);
        g[14] = (float)(g[14] - a6 - 0.5 * tz);
        g[12] = (float)(g[12] - a6 + 0.5 * tz);
    }
}

}  // namespace shifted
}  // namespace erlbm
