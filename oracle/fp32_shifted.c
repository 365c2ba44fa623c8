/*
 * fp32_shifted.c -- test infrastructure: the GPU engine's FP32-shifted periodic update (D2Q9 and
 * D3Q19) restated for the CPU, operation for operation.
 *
 * This is not the reference's algorithm (that is erlbm_oracle.c, in FP64).  It is the checker for the
 * engine's own FP32 formulation.  The populations are stored as g_i = (float)(f_i - w_i).  The collision
 * is E-RLBM / RLBM / BGK / MRT written as an increment on g, with the pair sums, differences and
 * non-equilibrium parts carried at twice their scale.  Every operation below is one IEEE
 * single-precision operation, rounded to nearest: the CPU's float +, -, * and /, and C99 fmaf.  The
 * GPU forms use the same operations as explicitly rounded intrinsics (__fadd_rn, __fmul_rn,
 * __fmaf_rn, __frcp_rn), so the two agree bit for bit.  This file is compiled with
 * -ffp-contract=off, so the compiler fuses nothing.
 *
 * Step semantics are those of the engine's erlbm_step on a periodic box, optionally with solid nodes:
 *   - the first step after setting the populations collides them in place;
 *   - every later step pulls g_i from node (x - c_ix, y - c_iy, z - c_iz) (periodic) and collides;
 *     when that node is solid, g_i is the population of the opposite direction that this node sent
 *     towards it in the previous step (halfway bounce-back);
 *   - solid nodes are never updated;
 *   - optionally (orc32_channel) boundary planes, applied after the pull and before the collision, in
 *     the same FP32 / FP64 split as the engine: a Zou-He velocity inlet (D3Q19 or D2Q9); an outlet
 *     that is the inner neighbour rescaled to rho_out (devnull_rho_x), open (OpenBoundaryD2Q9_x) or
 *     convective (convective_x); and the open y plane of D2Q9 (OpenBoundaryD2Q9_y).
 * The result is the post-collision populations, returned as f = (double)g + w for every node of the box
 * in x-fastest order (solid nodes carry their input).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "erlbm_oracle.h"

static const int CX9[9] = {0, 1, -1, 0, 0, 1, -1, 1, -1};
static const int CY9[9] = {0, 0, 0, 1, -1, 1, -1, -1, 1};

static double w9(int i) { return i == 0 ? 4. / 9. : (i < 5 ? 1. / 9. : 1. / 36.); }

/* Increment coefficients, formed in double and rounded once (the engine's shifted::Coef): d1 = 2 - 1/tau,
 * kd = w_gt1 - 1, nkc = -(1 + w_gt1), kh = kd / 2, d1t = -2/3 d1, nkct = -2/3 nkc. */
typedef struct {
    float d1, kd, nkc, kh, d1t, nkct;
} Coef32;

/* one opposite pair from D = 2 de, DO = 2 do and f1: the increment delta_1 f1 - k_c f1 + k_d d with
 * d = (D +- DO) / 2, the part common to both members formed once */
static void pair_update(float *gi, float *gj, float D, float DO, float f1, const Coef32 *k, int op)
{
    if (op == ORC_OP_BGK) {
        const float d1 = k->d1, DI = D + DO, DJ = D - DO;
        *gi = fmaf(0.5f, fmaf(d1, DI, -2.f * DI), *gi);
        *gj = fmaf(0.5f, fmaf(d1, DJ, -2.f * DJ), *gj);
    } else {
        const float cm = fmaf(k->d1, f1, fmaf(k->nkc, f1, k->kh * D));
        *gi = *gi + fmaf(k->kh, DO, cm);
        *gj = *gj + fmaf(-k->kh, DO, cm);
    }
}

static float rest_update(float g0, float de0, float f10, const Coef32 *k, int op)
{
    if (op == ORC_OP_BGK) return g0 + fmaf(k->d1, de0, -2.f * de0);
    return g0 + fmaf(k->d1, f10, fmaf(k->nkc, f10, k->kd * de0));
}

static void collide9_f32(float g[9], const Coef32 *k, int op)
{
    const float d1 = k->d1;
    const float W1 = 1.f / 9.f, W2 = 1.f / 36.f, M3W2 = -3.f * (1.f / 36.f);
    const float EX = g[1] + g[2], OX = g[1] - g[2];
    const float EY = g[3] + g[4], OY = g[3] - g[4];
    const float EP = g[5] + g[6], OP = g[5] - g[6];
    const float EM = g[7] + g[8], OM = g[7] - g[8];
    const float drho = ((EX + EY) + (EP + EM)) + g[0];
    const float mx = OX + (OP + OM);
    const float my = OY + (OP - OM);
    const float inv = 1.f / (1.f + drho);
    const float ux = mx * inv, uy = my * inv;
    const float a = mx * ux, b = my * uy;
    const float sab = fmaf(mx, ux, b);
    const float mu15 = -1.5f * sab;
    const float cxy = fmaf(mx, uy, my * ux);
    const float s3 = 3.f * sab;
    const float k45 = 4.5f, mw1x2 = -2.f * W1, mw2x2 = -2.f * W2;
    const float DX = fmaf(mw1x2, fmaf(k45, a, mu15), fmaf(mw1x2, drho, EX));
    const float DY = fmaf(mw1x2, fmaf(k45, b, mu15), fmaf(mw1x2, drho, EY));
    const float cmP = mx + my, cmM = mx - my;
    const float DP = fmaf(mw2x2, fmaf(k45, cxy, s3), fmaf(mw2x2, drho, EP));
    const float DM = fmaf(mw2x2, fmaf(-4.5f, cxy, s3), fmaf(mw2x2, drho, EM));
    const float DOP = fmaf(2.f * M3W2, cmP, OP);
    const float DOM = fmaf(2.f * M3W2, cmM, OM);
    const float DOX = -(DOP + DOM);
    const float DOY = -(DOP - DOM);
    if (op == ORC_OP_MRT) {
        const float deX = 0.5f * DX, deY = 0.5f * DY, deP = 0.5f * DP, deM = 0.5f * DM;
        const float doP = 0.5f * DOP, doM = 0.5f * DOM;
        const float A = deX + deY, B = deP + deM;
        const float hE = (float)(1.6 / 6.0) * fmaf(2.f, B, A);
        const float hP = (float)(1.8 / 6.0) * fmaf(-2.f, A, -B);
        const float sX = deX - deY, sP = deP - deM;
        const float hd = -0.5f * d1;
        const float vX = fmaf(hd, sX, sX), vP = fmaf(hd, sP, sP);
        const float ax = fmaf(2.f, hP, hE), ap = -fmaf(2.f, hE, hP);
        const float xX = ax - vX, xY = ax + vX, xP = ap - vP, xM = ap + vP;
        const float sq = (float)-1.9;
        const float qP = sq * doP, qM = sq * doM;
        const float qX = -(qP + qM), qY = -(qP - qM);
        g[0] = g[0] + -2.f * ((xX + xY) + (xP + xM));
        g[1] = g[1] + (xX + qX);
        g[2] = g[2] + (xX - qX);
        g[3] = g[3] + (xY + qY);
        g[4] = g[4] + (xY - qY);
        g[5] = g[5] + (xP + qP);
        g[6] = g[6] + (xP - qP);
        g[7] = g[7] + (xM + qM);
        g[8] = g[8] + (xM - qM);
        return;
    }
    float f1X = 0.f, f1Y = 0.f, f1P = 0.f, f1M = 0.f;
    if (op == ORC_OP_BGK) {
        const float de0 = -((DX + DY) + (DP + DM));
        g[0] = rest_update(g[0], de0, 0.f, k, op);
    } else {
        const float sxy = DX + DY, sd = DP + DM;
        const float tr = fmaf(2.f, sd, sxy);
        const float de0 = -(sxy + sd);
        const float t12 = tr * (1.f / 12.f);
        const float dxy = DX - DY, pxy = DP - DM;
        f1X = fmaf(dxy, 0.25f, t12);
        f1Y = fmaf(dxy, -0.25f, t12);
        f1P = fmaf(pxy, 0.25f, t12);
        f1M = fmaf(pxy, -0.25f, t12);
        g[0] = g[0] + fmaf(k->d1t, tr, fmaf(k->nkct, tr, k->kd * de0));
    }
    pair_update(&g[1], &g[2], DX, DOX, f1X, k, op);
    pair_update(&g[3], &g[4], DY, DOY, f1Y, k, op);
    pair_update(&g[5], &g[6], DP, DOP, f1P, k, op);
    pair_update(&g[7], &g[8], DM, DOM, f1M, k, op);
}

/* D3Q19: pairs X = (1,2), Y = (3,4), Z = (5,6), A = (7,8) c = (1,1,0), B = (9,10) c = (1,-1,0),
 * C = (11,12) c = (1,0,1), D = (13,14) c = (1,0,-1), E = (16,15) c = (0,1,1), F = (17,18) c = (0,-1,1) */
static const int CX19[19] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0};
static const int CY19[19] = {0, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, -1, 1, -1, 1};
static const int CZ19[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, -1, 1, -1, 1, 1, -1};

static double w19(int i) { return i == 0 ? 1. / 3. : (i < 7 ? 1. / 18. : 1. / 36.); }

static void collide19_f32(float g[19], const Coef32 *k, int op)
{
    const float W1 = 1.f / 18.f, W2 = 1.f / 36.f, M3W2 = -3.f * (1.f / 36.f);
    const float EX = g[1] + g[2], OX = g[1] - g[2];
    const float EY = g[3] + g[4], OY = g[3] - g[4];
    const float EZ = g[5] + g[6], OZ = g[5] - g[6];
    const float EA = g[7] + g[8], OA = g[7] - g[8];
    const float EB = g[9] + g[10], OB = g[9] - g[10];
    const float EC = g[11] + g[12], OC = g[11] - g[12];
    const float ED = g[13] + g[14], OD = g[13] - g[14];
    const float EE = g[16] + g[15], OE = g[16] - g[15];
    const float EF = g[17] + g[18], OF = g[17] - g[18];
    const float drho = (((EX + EY) + (EZ + EA)) + ((EB + EC) + (ED + (EE + EF)))) + g[0];
    const float mx = (OX + (OA + OB)) + (OC + OD);
    const float my = (OY + (OA - OB)) + (OE - OF);
    const float mz = (OZ + (OC - OD)) + (OE + OF);
    const float inv = 1.f / (1.f + drho);
    const float ux = mx * inv, uy = my * inv, uz = mz * inv;
    const float mu15 = -1.5f * fmaf(mx, ux, fmaf(my, uy, mz * uz));
    const float mw1x2 = -2.f * W1, mw2x2 = -2.f * W2, k45 = 4.5f;
    const float R1 = mw1x2 * drho, R2 = mw2x2 * drho;
    const float DX = fmaf(mw1x2, fmaf(k45 * mx, ux, mu15), EX + R1);
    const float DY = fmaf(mw1x2, fmaf(k45 * my, uy, mu15), EY + R1);
    const float DZ = fmaf(mw1x2, fmaf(k45 * mz, uz, mu15), EZ + R1);
    const float cmA = mx + my, cmB = mx - my, cmC = mx + mz, cmD = mx - mz;
    const float cmE = my + mz, cmF = mz - my;
    const float DA = fmaf(mw2x2, fmaf(k45 * cmA, ux + uy, mu15), EA + R2);
    const float DB = fmaf(mw2x2, fmaf(k45 * cmB, ux - uy, mu15), EB + R2);
    const float DC = fmaf(mw2x2, fmaf(k45 * cmC, ux + uz, mu15), EC + R2);
    const float DD = fmaf(mw2x2, fmaf(k45 * cmD, ux - uz, mu15), ED + R2);
    const float DE = fmaf(mw2x2, fmaf(k45 * cmE, uy + uz, mu15), EE + R2);
    const float DF = fmaf(mw2x2, fmaf(k45 * cmF, uz - uy, mu15), EF + R2);
    const float de0 = -(((DX + DY) + (DZ + DA)) + ((DB + DC) + (DD + (DE + DF))));
    const float m3w2x2 = 2.f * M3W2;
    const float DOA = fmaf(m3w2x2, cmA, OA), DOB = fmaf(m3w2x2, cmB, OB);
    const float DOC = fmaf(m3w2x2, cmC, OC), DOD = fmaf(m3w2x2, cmD, OD);
    const float DOE = fmaf(m3w2x2, cmE, OE), DOF = fmaf(m3w2x2, cmF, OF);
    const float DOX = -((DOA + DOB) + (DOC + DOD));
    const float DOY = -((DOA - DOB) + (DOE - DOF));
    const float DOZ = -((DOC - DOD) + (DOE + DOF));
    float f10 = 0.f, f1X = 0.f, f1Y = 0.f, f1Z = 0.f, f1A = 0.f, f1B = 0.f, f1C = 0.f, f1D = 0.f, f1E = 0.f,
          f1F = 0.f;
    if (op != ORC_OP_BGK) {
        const float pxx = (DX + (DA + DB)) + (DC + DD);
        const float pyy = (DY + (DA + DB)) + (DE + DF);
        const float pzz = (DZ + (DC + DD)) + (DE + DF);
        const float pxy = DA - DB, pxz = DC - DD, pyz = DE - DF;
        const float tr3 = ((pxx + pyy) + pzz) * (1.f / 3.f);
        f10 = -1.5f * tr3;
        f1X = 0.25f * (pxx - tr3);
        f1Y = 0.25f * (pyy - tr3);
        f1Z = 0.25f * (pzz - tr3);
        const float bxy = 0.125f * ((pxx + pyy) - tr3);
        const float bxz = 0.125f * ((pxx + pzz) - tr3);
        const float byz = 0.125f * ((pyy + pzz) - tr3);
        f1A = fmaf(0.25f, pxy, bxy);
        f1B = fmaf(-0.25f, pxy, bxy);
        f1C = fmaf(0.25f, pxz, bxz);
        f1D = fmaf(-0.25f, pxz, bxz);
        f1E = fmaf(0.25f, pyz, byz);
        f1F = fmaf(-0.25f, pyz, byz);
    }
    g[0] = rest_update(g[0], de0, f10, k, op);
    pair_update(&g[1], &g[2], DX, DOX, f1X, k, op);
    pair_update(&g[3], &g[4], DY, DOY, f1Y, k, op);
    pair_update(&g[5], &g[6], DZ, DOZ, f1Z, k, op);
    pair_update(&g[7], &g[8], DA, DOA, f1A, k, op);
    pair_update(&g[9], &g[10], DB, DOB, f1B, k, op);
    pair_update(&g[11], &g[12], DC, DOC, f1C, k, op);
    pair_update(&g[13], &g[14], DD, DOD, f1D, k, op);
    pair_update(&g[16], &g[15], DE, DOE, f1E, k, op);
    pair_update(&g[17], &g[18], DF, DOF, f1F, k, op);
}

static int opp(int i) { return i == 0 ? 0 : (i % 2 ? i + 1 : i - 1); }

typedef struct {
    int inlet_x, outlet_x, outlet_kind, open_y;
    double u_in, rho_out;
    double inv_1mvx, vx3, vx6; /* formed once per run, as the engine's zou_he_prep */
    const double *prof;        /* parabolic inlet: the x velocity per (y, z), else NULL */
} Planes;

enum { OUTLET_DENSITY = 0, OUTLET_OPEN = 1, OUTLET_CONVECTIVE = 2 };

/* ZouHeD2Q9_vx_x on shifted populations: rho = (1 + G) / (1 - vx), g_i = w_i (rho P - 1) for the +x
 * movers with P = (1 + 3 vx) + (3 vx) vx, in FP64 with every operation rounded separately. */
static void zou_he9(float g[9], double vx)
{
    const float G = ((g[0] + g[3]) + g[4]) + 2.f * ((g[2] + g[8]) + g[6]);
    const double rho = (1.0 + (double)G) / (1.0 - vx);
    const double vx3 = 3.0 * vx;
    const double P = (1.0 + vx3) + vx3 * vx;
    const double e = rho * P - 1.0;
    g[1] = (float)(e / 9.0);
    g[5] = (float)(e / 36.0);
    g[7] = (float)(e / 36.0);
}

/* x velocity of a node in FP32, as the engine's moments: u_x = m_x / (1 + drho) */
static float node_ux(const float *g, int q)
{
    float drho, mx;
    if (q == 9) {
        const float eX = g[1] + g[2], eY = g[3] + g[4], eP = g[5] + g[6], eM = g[7] + g[8];
        drho = g[0] + ((eX + eY) + (eP + eM));
        mx = (g[1] - g[2]) + ((g[5] - g[6]) + (g[7] - g[8]));
    } else {
        const float e1 = (g[1] + g[2]) + (g[3] + g[4]), e2 = (g[5] + g[6]) + (g[7] + g[8]);
        const float e3 = (g[9] + g[10]) + (g[11] + g[12]), e4 = (g[13] + g[14]) + (g[15] + g[16]);
        drho = (g[0] + (e1 + e2)) + ((e3 + e4) + (g[17] + g[18]));
        mx = ((g[1] - g[2]) + ((g[7] - g[8]) + (g[9] - g[10]))) + ((g[11] - g[12]) + (g[13] - g[14]));
    }
    const float inv = 1.f / (1.f + drho);
    return mx * inv;
}

/* convective_x on shifted populations: g = (g + U g_a) / (1 + U), U the inner neighbour's u_x */
static void convective(float *g, const float *a, int q)
{
    const float u = node_ux(a, q), factor = 1.f / (1.f + u);
    for (int i = 0; i < q; i++) g[i] = factor * fmaf(u, a[i], g[i]);
}

/* Zou-He velocity inlet on shifted D3Q19 populations: rho = (1 + 2 G_minus + G_zero) / (1 - vx) in
 * FP64, the population sums and the transverse corrections in FP32 (ZouHeD3Q19_vx_x's closure). */
static void zou_he19(float g[19], const Planes *pl, int left)
{
    const float ty = ((((g[18] + g[3]) + g[16]) - g[15]) - g[4]) - g[17];
    const float tz = ((((g[17] + g[5]) + g[16]) - g[15]) - g[6]) - g[18];
    const float gz = (((g[0] + g[3]) + (g[4] + g[5])) + ((g[6] + g[15]) + (g[16] + g[17]))) + g[18];
    if (left) {
        const float gm = ((g[1] + g[7]) + (g[9] + g[11])) + g[13];
        const double rho = (1.0 + (2.0 * (double)gm + (double)gz)) * pl->inv_1mvx;
        const float a3 = (float)(rho * pl->vx3), a6 = (float)(rho * pl->vx6);
        g[1] = g[1] + a3;
        g[7] = g[7] + fmaf(-0.5f, ty, a6);
        g[9] = g[9] + fmaf(0.5f, ty, a6);
        g[11] = g[11] + fmaf(-0.5f, tz, a6);
        g[13] = g[13] + fmaf(0.5f, tz, a6);
    } else {
        const float gp = ((g[2] + g[8]) + (g[10] + g[12])) + g[14];
        const double rho = (1.0 + (2.0 * (double)gp + (double)gz)) * pl->inv_1mvx;
        const float a3 = (float)(rho * pl->vx3), a6 = (float)(rho * pl->vx6);
        g[2] = g[2] - a3;
        g[10] = g[10] - fmaf(0.5f, ty, a6);
        g[8] = g[8] - fmaf(-0.5f, ty, a6);
        g[14] = g[14] - fmaf(0.5f, tz, a6);
        g[12] = g[12] - fmaf(-0.5f, tz, a6);
    }
}

/* devnull_rho_x on shifted populations: g = g_adj + (s - 1)(g_adj + w) with
 * s - 1 = ((rho_out - 1) - drho) / (1 + drho), all in FP32. */
static void outlet_rescale(float *g, int q, double rho_out)
{
    float drho = 0.f;
    for (int i = 0; i < q; i++) drho += g[i];
    const float sm1 = ((float)(rho_out - 1.0) - drho) / (1.f + drho);
    for (int i = 0; i < q; i++) g[i] = fmaf(sm1, g[i] + (float)(q == 9 ? w9(i) : w19(i)), g[i]);
}

/* populations of node (x, y, z) after the pull (or in place on the first step) */
static void pull_node(const float *a, int q, int nx, int ny, int nz, const uint8_t *solid, int first, int x, int y,
                      int z, float *g)
{
    const int *cx = q == 9 ? CX9 : CX19, *cy = q == 9 ? CY9 : CY19, *cz = q == 9 ? NULL : CZ19;
    const size_t node = ((size_t)z * ny + y) * nx + x;
    for (int i = 0; i < q; i++) {
        if (first) {
            g[i] = a[node * q + i];
            continue;
        }
        const int xs = (x - cx[i] + nx) % nx, ys = (y - cy[i] + ny) % ny;
        const int zs = cz ? (z - cz[i] + nz) % nz : z;
        const size_t src = ((size_t)zs * ny + ys) * nx + xs;
        g[i] = (solid && solid[src]) ? a[node * q + opp(i)] : a[src * q + i];
    }
}

/* parabolic_D3Q19_x's node update on shifted populations: an opposite pair has one weight, so
 * g_i = g_opp + rho vx / 3 (or / 6), rho in FP64 */
static void parabolic19(float g[19], double vx)
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

static void apply_inlet(float *g, int q, int nx, int ny, int y, int z, const Planes *pl)
{
    if (pl->prof) { /* parabolic_D2Q9_x is the D2Q9 Zou-He closure with the profile's velocity */
        const double vx = pl->prof[y + (size_t)ny * z];
        if (q == 19)
            parabolic19(g, vx);
        else
            zou_he9(g, vx);
        return;
    }
    if (q == 19)
        zou_he19(g, pl, pl->inlet_x < nx / 2);
    else
        zou_he9(g, pl->u_in);
}

/* populations of fluid node (x, y, z) after this step's inlet and outlet planes */
static void after_x_planes(const float *a, int q, int nx, int ny, int nz, const uint8_t *solid, const Planes *pl,
                           int first, int x, int y, int z, float *g)
{
    const size_t node = ((size_t)z * ny + y) * nx + x;
    if (pl && x == pl->outlet_x) {
        const int xn = x + (pl->outlet_x < nx / 2 ? 1 : -1);
        const int nsolid = solid && solid[node + (size_t)(xn - x)];
        if (pl->outlet_kind == OUTLET_DENSITY) {
            if (nsolid) { /* the rest state w rho_out */
                for (int i = 0; i < q; i++) {
                    const double w = q == 9 ? w9(i) : w19(i);
                    g[i] = (float)(w * pl->rho_out - w);
                }
                return;
            }
            pull_node(a, q, nx, ny, nz, solid, first, xn, y, z, g);
            if (xn == pl->inlet_x) apply_inlet(g, q, nx, ny, y, z, pl);
            outlet_rescale(g, q, pl->rho_out);
            return;
        }
        pull_node(a, q, nx, ny, nz, solid, first, x, y, z, g);
        if (nsolid) return;
        float an[19];
        pull_node(a, q, nx, ny, nz, solid, first, xn, y, z, an);
        if (xn == pl->inlet_x) apply_inlet(an, q, nx, ny, y, z, pl);
        if (pl->outlet_kind == OUTLET_OPEN) { /* the populations entering from outside */
            if (xn > x) {
                g[1] = an[1];
                g[5] = an[5];
                g[7] = an[7];
            } else {
                g[2] = an[2];
                g[6] = an[6];
                g[8] = an[8];
            }
        } else {
            convective(g, an, q);
        }
        return;
    }
    pull_node(a, q, nx, ny, nz, solid, first, x, y, z, g);
    if (pl && x == pl->inlet_x) apply_inlet(g, q, nx, ny, y, z, pl);
}

/* the x planes, then the open y plane (D2Q9): the populations entering through it are the inner
 * neighbour's, taken after that neighbour's own x planes */
static void after_planes(const float *a, int q, int nx, int ny, int nz, const uint8_t *solid, const Planes *pl,
                         int first, int x, int y, int z, float *g)
{
    after_x_planes(a, q, nx, ny, nz, solid, pl, first, x, y, z, g);
    if (!pl || q != 9 || y != pl->open_y) return;
    const int yn = y + (pl->open_y < ny / 2 ? 1 : -1);
    if (solid && solid[(size_t)yn * nx + x]) return;
    float an[9];
    after_x_planes(a, q, nx, ny, nz, solid, pl, first, x, yn, z, an);
    if (yn > y) {
        g[3] = an[3];
        g[5] = an[5];
        g[8] = an[8];
    } else {
        g[4] = an[4];
        g[6] = an[6];
        g[7] = an[7];
    }
}

/* The stepping loop shared by both lattices: q populations per node, AoS, x fastest. */
static int run_periodic(int q, int nx, int ny, int nz, const uint8_t *solid, const Planes *pl, int op, double tau,
                        double tau_nh, const double *f_in, int n_steps, double *f_out)
{
    if (nx < 1 || ny < 1 || nz < 1 || n_steps < 0 || !f_in || !f_out) return -1;
    if (op != ORC_OP_BGK && op != ORC_OP_REG && op != ORC_OP_EXTREG && !(op == ORC_OP_MRT && q == 9)) return -1;
    const size_t n = (size_t)nx * ny * nz;
    float *a = malloc(n * q * sizeof(float)), *b = malloc(n * q * sizeof(float));
    if (!a || !b) {
        free(a);
        free(b);
        return -2;
    }
    Coef32 k;
    const double d1 = 2.0 - 1.0 / tau;
    double nkc = 0.0;
    k.d1 = (float)d1;
    if (op == ORC_OP_BGK || op == ORC_OP_MRT) {
        k.kd = 0.f;
    } else if (op == ORC_OP_REG) {
        k.kd = -1.f;
        nkc = -1.0;
    } else {
        const double omega_gt1 = 1.0 - 1.0 / tau_nh;
        k.kd = (float)(omega_gt1 - 1.0);
        nkc = -(1.0 + omega_gt1);
    }
    k.nkc = (float)nkc;
    k.kh = 0.5f * k.kd;
    k.d1t = (float)(-2.0 / 3.0 * d1);
    k.nkct = (float)(-2.0 / 3.0 * nkc);
    for (size_t p = 0; p < n; p++)
        for (int i = 0; i < q; i++) a[p * q + i] = (float)(f_in[p * q + i] - (q == 9 ? w9(i) : w19(i)));
    for (int s = 0; s < n_steps; s++) {
        for (int z = 0; z < nz; z++)
            for (int y = 0; y < ny; y++)
                for (int x = 0; x < nx; x++) {
                    const size_t node = ((size_t)z * ny + y) * nx + x;
                    float g[19];
                    if (solid && solid[node]) {
                        memcpy(&b[node * q], &a[node * q], (size_t)q * sizeof(float));
                        continue;
                    }
                    after_planes(a, q, nx, ny, nz, solid, pl, s == 0, x, y, z, g);
                    if (q == 9)
                        collide9_f32(g, &k, op);
                    else
                        collide19_f32(g, &k, op);
                    memcpy(&b[node * q], g, (size_t)q * sizeof(float));
                }
        float *t = a;
        a = b;
        b = t;
    }
    for (size_t p = 0; p < n; p++)
        for (int i = 0; i < q; i++) f_out[p * q + i] = (double)a[p * q + i] + (q == 9 ? w9(i) : w19(i));
    free(a);
    free(b);
    return 0;
}

int orc32_periodic_d2q9(int nx, int ny, int op, double tau, double tau_nh, const double *f_in, int n_steps,
                        double *f_out)
{
    return run_periodic(9, nx, ny, 1, NULL, NULL, op, tau, tau_nh, f_in, n_steps, f_out);
}

int orc32_periodic_d3q19(int nx, int ny, int nz, int op, double tau, double tau_nh, const double *f_in,
                         int n_steps, double *f_out)
{
    return run_periodic(19, nx, ny, nz, NULL, NULL, op, tau, tau_nh, f_in, n_steps, f_out);
}

int orc32_periodic_solid(int q, int nx, int ny, int nz, const uint8_t *solid, int op, double tau, double tau_nh,
                         const double *f_in, int n_steps, double *f_out)
{
    if ((q != 9 && q != 19) || (q == 9 && nz != 1)) return -1;
    return run_periodic(q, nx, ny, nz, solid, NULL, op, tau, tau_nh, f_in, n_steps, f_out);
}

int orc32_channel(int q, int nx, int ny, int nz, const uint8_t *solid, int op, double tau, double tau_nh,
                  int inlet_x, double u_in, int outlet_x, int outlet_kind, double rho_out, int open_y,
                  const double *f_in, int n_steps, double *f_out)
{
    return orc32_channel_ex(q, nx, ny, nz, solid, op, tau, tau_nh, inlet_x, u_in, 0, 0, outlet_x, outlet_kind, rho_out,
                            open_y, f_in, n_steps, f_out);
}

/* the parabolic profile of parabolic_D2Q9_x / parabolic_D3Q19_x (Boundary_conditions.cpp :759-764,
 * :467-472) at the h-th fluid node of a column, counted from 1 */
static double parabolic_vel32(int h, double vx_max, int Lw)
{
    const double d_h = (double)h - 0.5;
    return -4.0 * vx_max / (Lw * Lw) * (d_h) * (d_h - Lw);
}

int orc32_channel_ex(int q, int nx, int ny, int nz, const uint8_t *solid, int op, double tau, double tau_nh,
                     int inlet_x, double u_in, int inlet_kind, int parabolic_L, int outlet_x, int outlet_kind,
                     double rho_out, int open_y, const double *f_in, int n_steps, double *f_out)
{
    if ((q != 9 && q != 19) || (q == 9 && nz != 1)) return -1;
    if (inlet_kind != 0 && inlet_kind != 1) return -1;
    if (inlet_x >= nx || outlet_x >= nx || open_y >= ny) return -1;
    if (outlet_kind < OUTLET_DENSITY || outlet_kind > OUTLET_CONVECTIVE) return -1;
    if (q == 19 && ((outlet_x >= 0 && outlet_kind == OUTLET_OPEN) || open_y >= 0)) return -1; /* D2Q9 planes */
    if (outlet_x >= 0) {
        const int xn = outlet_x + (outlet_x < nx / 2 ? 1 : -1);
        if (xn < 0 || xn >= nx) return -1;
    }
    if (open_y >= 0) {
        const int yn = open_y + (open_y < ny / 2 ? 1 : -1);
        if (yn < 0 || yn >= ny) return -1;
    }
    Planes pl;
    pl.inlet_x = inlet_x < 0 ? -1 : inlet_x;
    pl.outlet_x = outlet_x < 0 ? -1 : outlet_x;
    pl.outlet_kind = outlet_kind;
    pl.open_y = open_y < 0 ? -1 : open_y;
    pl.u_in = u_in;
    pl.rho_out = rho_out;
    pl.inv_1mvx = 1.0 / (1.0 - u_in);
    pl.vx3 = u_in / 3.0;
    pl.vx6 = u_in / 6.0;
    pl.prof = NULL;
    double *prof = NULL;
    if (inlet_kind == 1 && inlet_x >= 0) { /* the fluid nodes of each inlet column, counted up from y = 0 */
        if (parabolic_L < 1 || parabolic_L >= ny) return -1;
        prof = calloc((size_t)ny * nz, sizeof(double));
        if (!prof) return -2;
        for (int z = 0; z < nz; z++) {
            int h = 0;
            for (int y = 0; y < ny; y++) {
                if (solid && solid[((size_t)z * ny + y) * nx + inlet_x]) continue;
                if (++h > parabolic_L) {
                    free(prof);
                    return -1;
                }
                prof[y + (size_t)ny * z] = parabolic_vel32(h, u_in, parabolic_L);
            }
        }
        pl.prof = prof;
    }
    const int rc = run_periodic(q, nx, ny, nz, solid, &pl, op, tau, tau_nh, f_in, n_steps, f_out);
    free(prof);
    return rc;
}

/* ------------------------------------------------------------------------------------------------
 * One run of the engine's batched FP32 map kernel (k_batch over PrecShifted32; a D3Q19 or D2Q9 lattice
 * of nx x ny x 1 nodes held by one CTA of `block` threads with `npt` nodes each), restated with every
 * operation of the kernel in the kernel's order, so that label, decided step, steps done, status,
 * margin and energy agree bit for bit:
 *   - thread slots: the fluid nodes in node order, the boundary-plane nodes first; thread t holds
 *     slots t, t + block, ..., t + (npt - 1) block;
 *   - initial state: the Taylor-Green map's equilibrium formed in FP32 from the FP64 velocity
 *     (init 1), or the rest state w rho0 (init 0);
 *   - a step: pull (in place on the first step) with bounce-back and the outlet's copy of its inner
 *     neighbour; the energy check on those post-stream populations when step > 0 and step % every == 0;
 *     the inlet and outlet closures; the collision; the density check drho > hi or drho < lo (float
 *     bounds equivalent to |1 + drho| > limit) or non-finite at any node, the step finished first;
 *   - energy: per node (double)(0.5f |u|^2) from FP32 moments, summed per thread over its slots
 *     (0.0 + ...), then across each warp by the xor butterfly (strides 16, 8, 4, 2, 1), then over the
 *     warps in order;
 *   - margin: max over checks of E / (factor E0) (+inf for a non-finite E), or max |1 + drho| / limit
 *     over every node and step seen (+inf when a density was non-finite).
 * ------------------------------------------------------------------------------------------------ */

#define ORC32_PI 3.14159265358979323846 /* the value of M_PI, which strict C11 does not declare */

static double node_energy32(const float *g, int q)
{
    float drho, mx, my, mz = 0.f;
    if (q == 9) {
        const float eX = g[1] + g[2], eY = g[3] + g[4], eP = g[5] + g[6], eM = g[7] + g[8];
        const float oX = g[1] - g[2], oY = g[3] - g[4], oP = g[5] - g[6], oM = g[7] - g[8];
        drho = g[0] + ((eX + eY) + (eP + eM));
        mx = oX + (oP + oM);
        my = oY + (oP - oM);
    } else {
        const float oX = g[1] - g[2], oY = g[3] - g[4], oZ = g[5] - g[6], oA = g[7] - g[8], oB = g[9] - g[10];
        const float oC = g[11] - g[12], oD = g[13] - g[14], oE = g[16] - g[15], oF = g[17] - g[18];
        const float e1 = (g[1] + g[2]) + (g[3] + g[4]), e2 = (g[5] + g[6]) + (g[7] + g[8]);
        const float e3 = (g[9] + g[10]) + (g[11] + g[12]), e4 = (g[13] + g[14]) + (g[15] + g[16]);
        drho = (g[0] + (e1 + e2)) + ((e3 + e4) + (g[17] + g[18]));
        mx = (oX + (oA + oB)) + (oC + oD);
        my = (oY + (oA - oB)) + (oE - oF);
        mz = (oZ + (oC - oD)) + (oE + oF);
    }
    const float inv = 1.f / (1.f + drho);
    const float ux = mx * inv, uy = my * inv, uz = mz * inv;
    if (q == 9) return (double)(0.5f * fmaf(ux, ux, uy * uy));
    return (double)(0.5f * fmaf(ux, ux, fmaf(uy, uy, uz * uz)));
}

static float node_drho32(const float *g, int q)
{
    float s = 0.f;
    for (int i = 0; i < q; i++) s += g[i];
    return s;
}

/* the kernel's block sum: per-thread values v[0 .. block-1], xor butterfly per warp, warps in order */
static double block_sum32(double *v, int block)
{
    double s = 0.0;
    for (int w = 0; w < block / 32; w++) {
        double *l = v + 32 * w;
        for (int o = 16; o > 0; o >>= 1) {
            double t[32];
            for (int k = 0; k < 32; k++) t[k] = l[k] + l[k ^ o];
            memcpy(l, t, sizeof(t));
        }
        s += l[0];
    }
    return s;
}

int orc32_batch_run(int q, int nx, int ny, const uint8_t *solid, int inlet_x, int outlet_x, double rho0,
                    int energy_every, double energy_factor, int density_check, double density_limit, int init,
                    int op, double tau, double tau_nh, double u0, int n_steps, int block, int npt, int *out4,
                    double *out2)
{
    if ((q != 9 && q != 19) || nx < 1 || ny < 1 || block < 32 || block % 32 || npt < 1 || n_steps < 0) return -1;
    if (op != ORC_OP_BGK && op != ORC_OP_REG && op != ORC_OP_EXTREG && !(op == ORC_OP_MRT && q == 9)) return -1;
    if (inlet_x >= 0 && q != 19) return -1;
    const int nb = nx * ny;
    if (nb > block * npt) return -1;
    float *a = malloc((size_t)nb * q * sizeof(float)), *b = malloc((size_t)nb * q * sizeof(float));
    float *f = malloc((size_t)nb * q * sizeof(float));
    int *order = malloc((size_t)nb * sizeof(int));
    double *tv = malloc((size_t)block * sizeof(double));
    if (!a || !b || !f || !order || !tv) {
        free(a), free(b), free(f), free(order), free(tv);
        return -2;
    }
    /* thread slots */
    int n_fluid = 0;
    for (int pass = 0; pass < 2; pass++)
        for (int n = 0; n < nb; n++) {
            if (solid && solid[n]) continue;
            const int x = n % nx;
            const int plane = x == inlet_x || x == outlet_x;
            if (plane == (pass == 0)) order[n_fluid++] = n;
        }
    /* coefficients (as the host prepares a run) and the planes */
    Coef32 k;
    const double d1 = 2.0 - 1.0 / tau;
    double nkc = 0.0;
    k.d1 = (float)d1;
    if (op == ORC_OP_BGK || op == ORC_OP_MRT) {
        k.kd = 0.f;
    } else if (op == ORC_OP_REG) {
        k.kd = -1.f;
        nkc = -1.0;
    } else {
        const double omega_gt1 = 1.0 - 1.0 / tau_nh;
        k.kd = (float)(omega_gt1 - 1.0);
        nkc = -(1.0 + omega_gt1);
    }
    k.nkc = (float)nkc;
    k.kh = 0.5f * k.kd;
    k.d1t = (float)(-2.0 / 3.0 * d1);
    k.nkct = (float)(-2.0 / 3.0 * nkc);
    Planes pl;
    memset(&pl, 0, sizeof(pl)); /* no parabolic profile */
    pl.inlet_x = inlet_x;
    pl.outlet_x = outlet_x;
    pl.outlet_kind = OUTLET_DENSITY;
    pl.open_y = -1;
    pl.u_in = u0;
    pl.rho_out = rho0;
    pl.inv_1mvx = 1.0 / (1.0 - u0);
    pl.vx3 = u0 / 3.0;
    pl.vx6 = u0 / 6.0;
    const Planes *plp = (inlet_x >= 0 || outlet_x >= 0) ? &pl : NULL;
    /* density bounds: |1 + (double)d| > limit  <=>  d > hi or d < lo for a float d */
    const double hi = density_limit - 1.0, lo = -density_limit - 1.0;
    float fh = (float)hi, fl = (float)lo;
    if ((double)fh > hi) fh = nextafterf(fh, -INFINITY);
    if ((double)fl < lo) fl = nextafterf(fl, INFINITY);
    /* initial populations */
    const double L = (double)nx;
    for (int n = 0; n < nb; n++) {
        float *g = &a[(size_t)n * q];
        const int x = n % nx, y = n / nx;
        for (int i = 0; i < q; i++) {
            const double w = q == 9 ? w9(i) : w19(i);
            if (init == 1) {
                const double sx = sin(2. * ORC32_PI * (double)x / L), cx_ = cos(2. * ORC32_PI * (double)x / L);
                const double sy = sin(2. * ORC32_PI * (double)y / L), cy_ = cos(2. * ORC32_PI * (double)y / L);
                const float ux = (float)(u0 * sx * cy_), uy = (float)(-u0 * cx_ * sy);
                const float mu = -1.5f * fmaf(ux, ux, uy * uy);
                const int ci = q == 9 ? CX9[i] : CX19[i], cj = q == 9 ? CY9[i] : CY19[i];
                const float cu = (float)ci * ux + (float)cj * uy;
                g[i] = (float)w * fmaf(cu, fmaf(4.5f, cu, 3.f), mu);
            } else {
                g[i] = (float)(w * rho0 - w);
            }
        }
    }
    /* per-thread energy of a population set (f: every node's populations) */
#define THREAD_ENERGY(POP)                                                                        \
    do {                                                                                          \
        for (int t = 0; t < block; t++) {                                                         \
            double e = 0.0;                                                                       \
            for (int s = 0; s < npt; s++) {                                                       \
                const int slot = t + s * block;                                                   \
                if (slot < n_fluid) e += node_energy32(&(POP)[(size_t)order[slot] * q], q);      \
            }                                                                                     \
            tv[t] = e;                                                                            \
        }                                                                                         \
    } while (0)
    double E0 = 0.0, E = 0.0, margin = 0.0, max_rho = 0.0;
    float dmax = -INFINITY, dmin = INFINITY;
    int label = 0, decided = n_steps, status = 0, steps_done = n_steps;
    if (energy_every > 0) {
        THREAD_ENERGY(a);
        E0 = block_sum32(tv, block);
        E = E0;
    }
    for (int step = 0; step < n_steps; step++) {
        /* post-stream populations (the outlet node holds its inner neighbour's) */
        for (int n = 0; n < nb; n++) {
            if (solid && solid[n]) continue;
            const int x = n % nx, y = n / nx;
            int xp = x;
            if (x == outlet_x) xp = x + (outlet_x < nx / 2 ? 1 : -1);
            pull_node(a, q, nx, ny, 1, solid, step == 0, xp, y, 0, &f[(size_t)n * q]);
        }
        if (energy_every > 0 && step > 0 && step % energy_every == 0) {
            THREAD_ENERGY(f);
            E = block_sum32(tv, block);
            const double lim = energy_factor * E0;
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
        int flag = 0;
        for (int n = 0; n < nb; n++) {
            if (solid && solid[n]) {
                memcpy(&b[(size_t)n * q], &a[(size_t)n * q], (size_t)q * sizeof(float));
                continue;
            }
            float g[19];
            const int x = n % nx, y = n / nx;
            after_planes(a, q, nx, ny, 1, solid, plp, step == 0, x, y, 0, g);
            if (q == 9)
                collide9_f32(g, &k, op);
            else
                collide19_f32(g, &k, op);
            if (density_check) {
                const float d = node_drho32(g, q);
                if (!isfinite(d)) {
                    flag |= 2;
                } else {
                    dmax = fmaxf(dmax, d);
                    dmin = fminf(dmin, d);
                    if (d > fh || d < fl) flag |= 1;
                }
            }
            memcpy(&b[(size_t)n * q], g, (size_t)q * sizeof(float));
        }
        float *t = a;
        a = b;
        b = t;
        if (density_check && flag) {
            label = 1;
            decided = step;
            steps_done = step + 1;
            status |= (flag & 2) ? 3 : 1;
            break;
        }
    }
#undef THREAD_ENERGY
    if (density_check) {
        if (dmax >= dmin) max_rho = fmax(fabs(1.0 + (double)dmax), fabs(1.0 + (double)dmin));
        margin = (status & 2) ? INFINITY : max_rho / density_limit;
    }
    out4[0] = label;
    out4[1] = decided;
    out4[2] = steps_done;
    out4[3] = status;
    out2[0] = margin;
    out2[1] = E;
    free(a), free(b), free(f), free(order), free(tv);
    return 0;
}

/* ------------------------------------------------------------------------------------------------
 * The engine's compensated FP32 form (ERLBM_FP32_PAIR) restated: g = f - w held as an unevaluated
 * float pair (hi + lo); the D2Q9 collision with the pair sums and differences, the momentum, c.m on
 * the diagonals, the diagonals' odd non-equilibrium parts and the increment's addition in float-float
 * arithmetic (Knuth's two-sum, Dekker's fast two-sum, the fma-split product), the rest in FP32; every
 * step of it as the engine's collide_pair.cuh orders it.
 * ------------------------------------------------------------------------------------------------ */
typedef struct {
    float hi, lo;
} DS32;

static DS32 ds_two_sum(float a, float b)
{
    const float s = a + b;
    const float bb = s - a;
    DS32 r = {s, (a - (s - bb)) + (b - bb)};
    return r;
}
static DS32 ds_fast_two_sum(float a, float b)
{
    const float s = a + b;
    DS32 r = {s, b - (s - a)};
    return r;
}
static DS32 ds_add(DS32 a, DS32 b)
{
    const DS32 s = ds_two_sum(a.hi, b.hi);
    return ds_fast_two_sum(s.hi, s.lo + (a.lo + b.lo));
}
static DS32 ds_neg(DS32 a)
{
    DS32 r = {-a.hi, -a.lo};
    return r;
}
static DS32 ds_sub(DS32 a, DS32 b) { return ds_add(a, ds_neg(b)); }
static DS32 ds_c(float x)
{
    DS32 r = {x, 0.f};
    return r;
}
static DS32 ds_split(double v)
{
    const float hi = (float)v;
    DS32 r = {hi, (float)(v - (double)hi)};
    return r;
}
/* Dekker's product: hi x hi split by an fma, the cross terms added */
static DS32 ds_mul(DS32 a, DS32 b)
{
    const float p = a.hi * b.hi;
    const float e = fmaf(a.lo, b.hi, fmaf(a.hi, b.lo, fmaf(a.hi, b.hi, -p)));
    return ds_fast_two_sum(p, e);
}
static DS32 ds_fma(DS32 a, DS32 b, DS32 d) { return ds_add(ds_mul(a, b), d); }
static DS32 ds_rcp(DS32 a)
{
    const DS32 y0 = ds_c(1.f / a.hi);
    return ds_add(y0, ds_mul(y0, ds_sub(ds_c(1.f), ds_mul(a, y0))));
}

typedef struct {
    DS32 kd, d1, nkc, kh, d1t, nkct;
} CoefDS32;

static void ds_pair_update(DS32 *gi, DS32 *gj, DS32 D, DS32 DO, DS32 f1, const CoefDS32 *k, int op)
{
    const DS32 d1 = k->d1, m2 = ds_c(-2.f), half = ds_c(0.5f);
    if (op == ORC_OP_BGK) {
        const DS32 DI = ds_add(D, DO), DJ = ds_sub(D, DO);
        *gi = ds_fma(half, ds_fma(d1, DI, ds_mul(m2, DI)), *gi);
        *gj = ds_fma(half, ds_fma(d1, DJ, ds_mul(m2, DJ)), *gj);
    } else {
        const DS32 kh = k->kh;
        const DS32 cm = ds_fma(d1, f1, ds_fma(k->nkc, f1, ds_mul(kh, D)));
        *gi = ds_add(*gi, ds_fma(kh, DO, cm));
        *gj = ds_add(*gj, ds_fma(ds_neg(kh), DO, cm));
    }
}

/* shifted::collide9l over the float-float lane (BGK, RLBM, E-RLBM), operation for operation */
static void collide9_pair(DS32 g[9], const CoefDS32 *k, int op)
{
    const float W1 = 1.f / 9.f, W2 = 1.f / 36.f, M3W2 = -3.f * (1.f / 36.f);
    (void)W1, (void)W2, (void)M3W2;
    const DS32 EX = ds_add(g[1], g[2]), OX = ds_sub(g[1], g[2]);
    const DS32 EY = ds_add(g[3], g[4]), OY = ds_sub(g[3], g[4]);
    const DS32 EP = ds_add(g[5], g[6]), OP = ds_sub(g[5], g[6]);
    const DS32 EM = ds_add(g[7], g[8]), OM = ds_sub(g[7], g[8]);
    const DS32 drho = ds_add(ds_add(ds_add(EX, EY), ds_add(EP, EM)), g[0]);
    const DS32 mx = ds_add(OX, ds_add(OP, OM));
    const DS32 my = ds_add(OY, ds_sub(OP, OM));
    const DS32 inv = ds_rcp(ds_add(ds_c(1.f), drho));
    const DS32 ux = ds_mul(mx, inv), uy = ds_mul(my, inv);
    const DS32 a = ds_mul(mx, ux), b = ds_mul(my, uy);
    const DS32 sab = ds_fma(mx, ux, b);
    const DS32 mu15 = ds_mul(ds_c(-1.5f), sab);
    const DS32 cxy = ds_fma(mx, uy, ds_mul(my, ux));
    const DS32 s3 = ds_mul(ds_c(3.f), sab);
    const DS32 k45 = ds_c(4.5f), mw1x2 = ds_split(-2.0 / 9.0), mw2x2 = ds_split(-2.0 / 36.0);
    const DS32 DX = ds_fma(mw1x2, ds_fma(k45, a, mu15), ds_fma(mw1x2, drho, EX));
    const DS32 DY = ds_fma(mw1x2, ds_fma(k45, b, mu15), ds_fma(mw1x2, drho, EY));
    const DS32 cmP = ds_add(mx, my), cmM = ds_sub(mx, my);
    const DS32 DP = ds_fma(mw2x2, ds_fma(k45, cxy, s3), ds_fma(mw2x2, drho, EP));
    const DS32 DM = ds_fma(mw2x2, ds_fma(ds_c(-4.5f), cxy, s3), ds_fma(mw2x2, drho, EM));
    const DS32 DOP = ds_fma(ds_split(-1.0 / 6.0), cmP, OP);
    const DS32 DOM = ds_fma(ds_split(-1.0 / 6.0), cmM, OM);
    const DS32 DOX = ds_neg(ds_add(DOP, DOM));
    const DS32 DOY = ds_neg(ds_sub(DOP, DOM));
    const DS32 zero = ds_c(0.f);
    if (op == ORC_OP_BGK) {
        const DS32 de0 = ds_neg(ds_add(ds_add(DX, DY), ds_add(DP, DM)));
        const DS32 d1 = k->d1, m2 = ds_c(-2.f);
        g[0] = ds_add(g[0], ds_fma(d1, de0, ds_mul(m2, de0)));
        ds_pair_update(&g[1], &g[2], DX, DOX, zero, k, op);
        ds_pair_update(&g[3], &g[4], DY, DOY, zero, k, op);
        ds_pair_update(&g[5], &g[6], DP, DOP, zero, k, op);
        ds_pair_update(&g[7], &g[8], DM, DOM, zero, k, op);
        return;
    }
    const DS32 sxy = ds_add(DX, DY), sd = ds_add(DP, DM);
    const DS32 tr = ds_fma(ds_c(2.f), sd, sxy);
    const DS32 de0 = ds_neg(ds_add(sxy, sd));
    const DS32 t12 = ds_mul(tr, ds_split(1.0 / 12.0));
    const DS32 dxy = ds_sub(DX, DY), pxy = ds_sub(DP, DM);
    const DS32 f1X = ds_fma(dxy, ds_c(0.25f), t12), f1Y = ds_fma(dxy, ds_c(-0.25f), t12);
    const DS32 f1P = ds_fma(pxy, ds_c(0.25f), t12), f1M = ds_fma(pxy, ds_c(-0.25f), t12);
    g[0] = ds_add(g[0], ds_fma(k->d1t, tr, ds_fma(k->nkct, tr, ds_mul(k->kd, de0))));
    ds_pair_update(&g[1], &g[2], DX, DOX, f1X, k, op);
    ds_pair_update(&g[3], &g[4], DY, DOY, f1Y, k, op);
    ds_pair_update(&g[5], &g[6], DP, DOP, f1P, k, op);
    ds_pair_update(&g[7], &g[8], DM, DOM, f1M, k, op);
}

int orc32p_periodic_d2q9(int nx, int ny, int op, double tau, double tau_nh, const double *f_in, int n_steps,
                         double *f_out)
{
    if (nx < 1 || ny < 1 || n_steps < 0 || !f_in || !f_out) return -1;
    if (op != ORC_OP_BGK && op != ORC_OP_REG && op != ORC_OP_EXTREG) return -1;
    const size_t n = (size_t)nx * ny;
    DS32 *a = malloc(n * 9 * sizeof(DS32)), *b = malloc(n * 9 * sizeof(DS32));
    if (!a || !b) {
        free(a), free(b);
        return -2;
    }
    CoefDS32 k;
    const double d1 = 2.0 - 1.0 / tau;
    double kd = 0.0, nkc = 0.0;
    if (op == ORC_OP_REG) {
        kd = -1.0;
        nkc = -1.0;
    } else if (op == ORC_OP_EXTREG) {
        const double omega_gt1 = 1.0 - 1.0 / tau_nh;
        kd = omega_gt1 - 1.0;
        nkc = -(1.0 + omega_gt1);
    }
    k.kd = ds_split(kd);
    k.d1 = ds_split(d1);
    k.nkc = ds_split(nkc);
    k.kh = ds_split(0.5 * kd);
    k.d1t = ds_split(-2.0 / 3.0 * d1);
    k.nkct = ds_split(-2.0 / 3.0 * nkc);
    for (size_t p = 0; p < n; p++)
        for (int i = 0; i < 9; i++) {
            const double d = f_in[p * 9 + i] - w9(i);
            const float hi = (float)d;
            a[p * 9 + i].hi = hi;
            a[p * 9 + i].lo = (float)(d - (double)hi);
        }
    for (int s = 0; s < n_steps; s++) {
        for (int y = 0; y < ny; y++)
            for (int x = 0; x < nx; x++) {
                const size_t node = (size_t)y * nx + x;
                DS32 g[9];
                for (int i = 0; i < 9; i++) {
                    if (s == 0) {
                        g[i] = a[node * 9 + i];
                    } else {
                        const int xs = (x - CX9[i] + nx) % nx, ys = (y - CY9[i] + ny) % ny;
                        g[i] = a[((size_t)ys * nx + xs) * 9 + i];
                    }
                }
                collide9_pair(g, &k, op);
                memcpy(&b[node * 9], g, sizeof(g));
            }
        DS32 *t = a;
        a = b;
        b = t;
    }
    for (size_t p = 0; p < n; p++)
        for (int i = 0; i < 9; i++) f_out[p * 9 + i] = ((double)a[p * 9 + i].hi + (double)a[p * 9 + i].lo) + w9(i);
    free(a), free(b);
    return 0;
}
