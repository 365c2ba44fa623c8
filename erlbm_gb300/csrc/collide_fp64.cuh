// collide_fp64.cuh -- the plain FP64 collision, operation for operation as the reference.
//
// Bit-for-bit parity with the reference's FP64 CPU build rests on three facts:
//  (1) the reference is compiled by GCC in ISO C++17 mode, which does not contract a*b+c into an
//      FMA; every file that includes this header is compiled with nvcc --fmad=false, so each
//      multiply and add below is one correctly rounded IEEE operation as on the CPU;
//  (2) the sequence of rounded operations is the reference's:
//        calcula         LBM_functions.cpp:3518-3589
//        dist_eq         LBM_functions.cpp:2945-3000
//        coll_Ext_Reg    Collision_operators.cpp:1182-1307  (Pi accumulation, f1, f_gt1, update)
//        coll_Reg        Collision_operators.cpp:860-967
//        coll_BGK        Collision_operators.cpp:12-49
//        coll_MRT        Collision_operators.cpp:583-699 (D2Q9)
//  (3) the only operations left out are exact ones: products by the velocity components
//      c in {-1, 0, +1}, sums with +-0 (the terms whose coefficient is zero), and the source
//      term S of source() (LBM_functions.cpp:5646-5716), which is +-0 for every finite state
//      because all programs pass zero acceleration.  Leaving these out can change only the sign
//      of an exactly zero intermediate, which no later operation turns into a different
//      non-zero value, so finite results are identical.  A non-finite state may carry Inf where
//      the reference carries NaN; both are "non-finite" to every stability check.
//
// Sharing between opposite directions is exact too: c.u of direction opp(i) is the exact negation
// of that of i, so (0.5 cv) cv is identical and 1 + 3 cv becomes 1 - 3 cv.
#pragma once

#include "lattice.cuh"

namespace erlbm {
namespace exact {

// Reference constants, formed with the reference's own operations (calc_Q: Q = c c - c_s^2 delta;
// one_over_2cs4 = 0.5 * 3 * 3; f1 prefactor one_over_2cs4 * w_i).
constexpr double CS2 = 1. / 3.;
constexpr double QA = 1.0 * 1.0 - CS2;  // Q_aa for c_a = +-1
constexpr double QB = 0.0 * 0.0 - CS2;  // Q_aa for c_a = 0
constexpr double O2CS4 = 0.5 * 3. * 3.;

// Equilibrium of one opposite pair from cv = c_i.u of its first member.
__device__ __forceinline__ void feq_pair(double cv, double wr, double C, double &fa, double &fb)
{
    const double t3 = cv * 3.;
    const double B = ((0.5 * cv) * cv * 3.) * 3.;
    fa = wr * (((1.0 + t3) + B) - C);
    fb = wr * (((1.0 - t3) + B) - C);
}

// ------------------------------------------------------------------------------------------------
// D2Q9
// ------------------------------------------------------------------------------------------------

// calcula: rho summed in velocity order from 0.0; momenta summed in velocity order.
__device__ __forceinline__ void moments9(const double f[9], double &rho, double &ux, double &uy)
{
    double r = 0.0;
#pragma unroll
    for (int i = 0; i < 9; i++) r = r + f[i];
    const double mx = ((((f[1] - f[2]) + f[5]) - f[6]) + f[7]) - f[8];
    const double my = ((((f[3] - f[4]) + f[5]) - f[6]) - f[7]) + f[8];
    if (r != 0.0) {
        const double inv = 1.0 / r;
        ux = mx * inv;
        uy = my * inv;
    } else {
        ux = 0.;
        uy = 0.;
    }
    rho = r;
}

// dist_eq for D2Q9 (vz = 0).
__device__ __forceinline__ void equilibrium9(double rho, double ux, double uy, double feq[9])
{
    const double vq = ux * ux + uy * uy;
    const double C = (0.5 * vq) * 3.;
    const double wr0 = (4. / 9.) * rho, wr1 = (1. / 9.) * rho, wr2 = (1. / 36.) * rho;
    feq[0] = wr0 * (1.0 - C);
    feq_pair(ux, wr1, C, feq[1], feq[2]);
    feq_pair(uy, wr1, C, feq[3], feq[4]);
    feq_pair(ux + uy, wr2, C, feq[5], feq[6]);
    feq_pair(ux - uy, wr2, C, feq[7], feq[8]);
}

// Row ROW of the MRT transform applied to f: the reference sums M[ROW][i] * f[i] from 0.0 in
// column order.  Terms with M = 0 add +-0 and are left out; products by +-1 are exact.
template <int ROW>
__device__ __forceinline__ double mrt9_row(const double f[9])
{
    double acc = 0.0;
    bool first = true;
#pragma unroll
    for (int i = 0; i < 9; i++) {
        const int m = mrt9_m(ROW, i);
        if (m == 0) continue;
        const double t = m == 1 ? f[i] : (m == -1 ? -f[i] : (double)m * f[i]);
        acc = first ? t : acc + t;
        first = false;
    }
    return acc;
}

// Population I from the moments: sum over c of M^-1[I][c] * m[c] from 0.0, M^-1[I][c] =
// M[c][I] / |row c|^2 (a correctly rounded quotient, the value of the reference's literal).
template <int I>
__device__ __forceinline__ double mrt9_back(const double m[9])
{
    double acc = 0.0;
    bool first = true;
#pragma unroll
    for (int c = 0; c < 9; c++) {
        const int a = mrt9_m(c, I);
        if (a == 0) continue;
        const double t = ((double)a / (double)mrt9_norm2(c)) * m[c];
        acc = first ? t : acc + t;
        first = false;
    }
    return acc;
}

// coll_MRT, D2Q9: moments m = M f and m_eq = M f_eq; m <- m - s (m - m_eq) on the non-conserved
// rows (the conserved rows have s = 0, and the force moments are those of a zero force); f = M^-1 m.
__device__ __forceinline__ void collide9_mrt(double f[9], const Relax &R, const double feq[9])
{
    double m[9];
    m[0] = mrt9_row<0>(f);
    m[3] = mrt9_row<3>(f);
    m[5] = mrt9_row<5>(f);
    m[1] = mrt9_row<1>(f);
    m[1] = m[1] - MRT9_SE * (m[1] - mrt9_row<1>(feq));
    m[2] = mrt9_row<2>(f);
    m[2] = m[2] - MRT9_SEPS * (m[2] - mrt9_row<2>(feq));
    m[4] = mrt9_row<4>(f);
    m[4] = m[4] - MRT9_SQ * (m[4] - mrt9_row<4>(feq));
    m[6] = mrt9_row<6>(f);
    m[6] = m[6] - MRT9_SQ * (m[6] - mrt9_row<6>(feq));
    m[7] = mrt9_row<7>(f);
    m[7] = m[7] - R.inv_tau * (m[7] - mrt9_row<7>(feq));
    m[8] = mrt9_row<8>(f);
    m[8] = m[8] - R.inv_tau * (m[8] - mrt9_row<8>(feq));
    f[0] = mrt9_back<0>(m);
    f[1] = mrt9_back<1>(m);
    f[2] = mrt9_back<2>(m);
    f[3] = mrt9_back<3>(m);
    f[4] = mrt9_back<4>(m);
    f[5] = mrt9_back<5>(m);
    f[6] = mrt9_back<6>(m);
    f[7] = mrt9_back<7>(m);
    f[8] = mrt9_back<8>(m);
}

template <int OP>
__device__ __forceinline__ void collide9(double f[9], const Relax &R)
{
    double rho, ux, uy, feq[9];
    moments9(f, rho, ux, uy);
    equilibrium9(rho, ux, uy, feq);
    if constexpr (OP == OP_MRT) {
        collide9_mrt(f, R, feq);
        return;
    }
    if (OP == OP_BGK) {
#pragma unroll
        for (int i = 0; i < 9; i++) f[i] = f[i] + (feq[i] - f[i]) * R.inv_tau;
        return;
    }
    double d[9];
#pragma unroll
    for (int i = 0; i < 9; i++) d[i] = f[i] - feq[i];
    const double pxx = ((((d[1] + d[2]) + d[5]) + d[6]) + d[7]) + d[8];
    const double pyy = ((((d[3] + d[4]) + d[5]) + d[6]) + d[7]) + d[8];
    const double pxy = ((d[5] + d[6]) - d[7]) - d[8];
    const double xa = QA * pxx, xb = QB * pxx, ya = QA * pyy, yb = QB * pyy;
    const double p2 = 2. * pxy;
    const double dd = xa + ya;
    double f1[9];
    f1[0] = (O2CS4 * (4. / 9.)) * (xb + yb);
    f1[1] = f1[2] = (O2CS4 * (1. / 9.)) * (xa + yb);
    f1[3] = f1[4] = (O2CS4 * (1. / 9.)) * (xb + ya);
    f1[5] = f1[6] = (O2CS4 * (1. / 36.)) * (dd + p2);
    f1[7] = f1[8] = (O2CS4 * (1. / 36.)) * (dd - p2);
    if (OP == OP_REG) {
#pragma unroll
        for (int i = 0; i < 9; i++) f[i] = feq[i] + R.omega_1 * f1[i];
        return;
    }
#pragma unroll
    for (int i = 0; i < 9; i++) {
        const double gt1 = d[i] - f1[i];
        f[i] = (feq[i] + R.omega_1 * f1[i]) + R.omega_gt1 * gt1;
    }
}

// ------------------------------------------------------------------------------------------------
// D3Q19
// ------------------------------------------------------------------------------------------------

__device__ __forceinline__ void moments19(const double f[19], double &rho, double &ux, double &uy, double &uz)
{
    double r = 0.0;
#pragma unroll
    for (int i = 0; i < 19; i++) r = r + f[i];
    const double mx = ((((((((f[1] - f[2]) + f[7]) - f[8]) + f[9]) - f[10]) + f[11]) - f[12]) + f[13]) - f[14];
    const double my = ((((((((f[3] - f[4]) + f[7]) - f[8]) - f[9]) + f[10]) - f[15]) + f[16]) - f[17]) + f[18];
    const double mz = ((((((((f[5] - f[6]) + f[11]) - f[12]) - f[13]) + f[14]) - f[15]) + f[16]) + f[17]) - f[18];
    if (r != 0.0) {
        const double inv = 1.0 / r;
        ux = mx * inv;
        uy = my * inv;
        uz = mz * inv;
    } else {
        ux = 0.;
        uy = 0.;
        uz = 0.;
    }
    rho = r;
}

__device__ __forceinline__ void equilibrium19(double rho, double ux, double uy, double uz, double feq[19])
{
    const double vq = (ux * ux + uy * uy) + uz * uz;
    const double C = (0.5 * vq) * 3.;
    const double wr0 = (1. / 3.) * rho, wr1 = (1. / 18.) * rho, wr2 = (1. / 36.) * rho;
    feq[0] = wr0 * (1.0 - C);
    feq_pair(ux, wr1, C, feq[1], feq[2]);
    feq_pair(uy, wr1, C, feq[3], feq[4]);
    feq_pair(uz, wr1, C, feq[5], feq[6]);
    feq_pair(ux + uy, wr2, C, feq[7], feq[8]);
    feq_pair(ux - uy, wr2, C, feq[9], feq[10]);
    feq_pair(ux + uz, wr2, C, feq[11], feq[12]);
    feq_pair(ux - uz, wr2, C, feq[13], feq[14]);
    // direction 16 is (0,1,1) and 15 its opposite; 17 is (0,-1,1) and 18 its opposite
    feq_pair(uy + uz, wr2, C, feq[16], feq[15]);
    feq_pair(uz - uy, wr2, C, feq[17], feq[18]);
}

template <int OP>
__device__ __forceinline__ void collide19(double f[19], const Relax &R)
{
    double rho, ux, uy, uz, feq[19];
    moments19(f, rho, ux, uy, uz);
    equilibrium19(rho, ux, uy, uz, feq);
    if (OP == OP_BGK) {
#pragma unroll
        for (int i = 0; i < 19; i++) f[i] = f[i] + (feq[i] - f[i]) * R.inv_tau;
        return;
    }
    double d[19];
#pragma unroll
    for (int i = 0; i < 19; i++) d[i] = f[i] - feq[i];
    const double pxx = ((((((((d[1] + d[2]) + d[7]) + d[8]) + d[9]) + d[10]) + d[11]) + d[12]) + d[13]) + d[14];
    const double pyy = ((((((((d[3] + d[4]) + d[7]) + d[8]) + d[9]) + d[10]) + d[15]) + d[16]) + d[17]) + d[18];
    const double pzz = ((((((((d[5] + d[6]) + d[11]) + d[12]) + d[13]) + d[14]) + d[15]) + d[16]) + d[17]) + d[18];
    const double pxy = ((d[7] + d[8]) - d[9]) - d[10];
    const double pxz = ((d[11] + d[12]) - d[13]) - d[14];
    const double pyz = ((d[15] + d[16]) - d[17]) - d[18];
    const double xa = QA * pxx, xb = QB * pxx;
    const double ya = QA * pyy, yb = QB * pyy;
    const double za = QA * pzz, zb = QB * pzz;
    const double kr = O2CS4 * (1. / 3.), k1 = O2CS4 * (1. / 18.), k2 = O2CS4 * (1. / 36.);
    double f1[19];
    f1[0] = kr * ((xb + yb) + zb);
    f1[1] = f1[2] = k1 * ((xa + yb) + zb);
    f1[3] = f1[4] = k1 * ((xb + ya) + zb);
    f1[5] = f1[6] = k1 * ((xb + yb) + za);
    const double bxy = (xa + ya) + zb, pxy2 = 2. * pxy;
    f1[7] = f1[8] = k2 * (bxy + pxy2);
    f1[9] = f1[10] = k2 * (bxy - pxy2);
    const double bxz = (xa + yb) + za, pxz2 = 2. * pxz;
    f1[11] = f1[12] = k2 * (bxz + pxz2);
    f1[13] = f1[14] = k2 * (bxz - pxz2);
    const double byz = (xb + ya) + za, pyz2 = 2. * pyz;
    f1[15] = f1[16] = k2 * (byz + pyz2);
    f1[17] = f1[18] = k2 * (byz - pyz2);
    if (OP == OP_REG) {
#pragma unroll
        for (int i = 0; i < 19; i++) f[i] = feq[i] + R.omega_1 * f1[i];
        return;
    }
#pragma unroll
    for (int i = 0; i < 19; i++) {
        const double gt1 = d[i] - f1[i];
        f[i] = (feq[i] + R.omega_1 * f1[i]) + R.omega_gt1 * gt1;
    }
}

template <int Q, int OP>
__device__ __forceinline__ void collide(double *f, const Relax &R)
{
    static_assert(Q == 9 || OP != OP_MRT, "MRT is a D2Q9 operator");
    if constexpr (Q == 9)
        collide9<OP>(f, R);
    else
        collide19<OP>(f, R);
}

// calcula velocity of one node (for kinectic_energy, Other_functions.cpp:100-115):
// returns 0.5 * (vx*vx + vy*vy + vz*vz) with vz = 0 for D2Q9.
template <int Q>
__device__ __forceinline__ double node_energy(const double *f)
{
    if constexpr (Q == 9) {
        double rho, ux, uy;
        moments9(f, rho, ux, uy);
        return 0.5 * ((ux * ux + uy * uy) + 0.0 * 0.0);
    } else {
        double rho, ux, uy, uz;
        moments19(f, rho, ux, uy, uz);
        return 0.5 * ((ux * ux + uy * uy) + uz * uz);
    }
}

// density (LBM_functions.cpp:5544-5552)
template <int Q>
__device__ __forceinline__ double node_density(const double *f)
{
    double r = 0.0;
#pragma unroll
    for (int i = 0; i < Q; i++) r = r + f[i];
    return r;
}

// ZouHeD3Q19_vx_x, left-plane branch (Boundary_conditions.cpp:370-403) with vy = vz = 0, applied
// to one node's post-stream populations.  The right-plane branch (:404-436) mirrors it.
__device__ __forceinline__ void zou_he_left(double f[19], double vx)
{
    const double vy = 0.0, vz = 0.0;
    const double s_minus = (((f[1] + f[7]) + f[9]) + f[11]) + f[13];
    const double s_zero = (((((((f[0] + f[3]) + f[4]) + f[5]) + f[6]) + f[15]) + f[16]) + f[17]) + f[18];
    const double rho = (2.0 * s_minus + s_zero) / (1.0 - vx);
    const double ty = (((((f[18] + f[3]) + f[16]) - f[15]) - f[4]) - f[17]);
    const double tz = (((((f[17] + f[5]) + f[16]) - f[15]) - f[6]) - f[18]);
    const double a3 = rho * vx / 3.0, a6 = rho * vx / 6.0;
    f[1] = f[1] + a3;
    f[7] = ((f[7] + a6) + 0.5 * rho * vy) - 0.5 * ty;
    f[9] = ((f[9] + a6) - 0.5 * rho * vy) + 0.5 * ty;
    f[11] = ((f[11] + a6) + 0.5 * rho * vz) - 0.5 * tz;
    f[13] = ((f[13] + a6) - 0.5 * rho * vz) + 0.5 * tz;
}

__device__ __forceinline__ void zou_he_right(double f[19], double vx)
{
    const double vy = 0.0, vz = 0.0;
    const double s_plus = (((f[2] + f[8]) + f[10]) + f[12]) + f[14];
    const double s_zero = (((((((f[0] + f[3]) + f[4]) + f[5]) + f[6]) + f[15]) + f[16]) + f[17]) + f[18];
    const double rho = (2.0 * s_plus + s_zero) / (1.0 - vx);
    const double ty = (((((f[18] + f[3]) + f[16]) - f[15]) - f[4]) - f[17]);
    const double tz = (((((f[17] + f[5]) + f[16]) - f[15]) - f[6]) - f[18]);
    const double a3 = rho * vx / 3.0, a6 = rho * vx / 6.0;
    f[2] = f[2] - a3;
    f[10] = ((f[10] - a6) + 0.5 * rho * vy) - 0.5 * ty;
    f[8] = ((f[8] - a6) - 0.5 * rho * vy) + 0.5 * ty;
    f[14] = ((f[14] - a6) + 0.5 * rho * vz) - 0.5 * tz;
    f[12] = ((f[12] - a6) - 0.5 * rho * vz) + 0.5 * tz;
}

// ZouHeD2Q9_vx_x (Boundary_conditions.cpp:710-744), also the node update of parabolic_D2Q9_x
// (:748-800) with the profile's velocity: the +x movers from the closure density.
__device__ __forceinline__ void zou_he_d2q9(double f[9], double vx)
{
    const double rho = (((f[0] + f[3]) + f[4]) + 2 * ((f[2] + f[8]) + f[6])) / (1. - vx);
    const double p = (1.0 + 3.0 * vx) + 3.0 * vx * vx;
    f[1] = (rho / 9.0) * p;
    f[5] = (rho / 36.0) * p;
    f[7] = (rho / 36.0) * p;
}

// Node update of parabolic_D3Q19_x (Boundary_conditions.cpp:456-530): the +x movers from their
// opposites, rho from the closure (vy = vz = 0).
__device__ __forceinline__ void parabolic_d3q19(double f[19], double vx)
{
    const double vy = 0.0, vz = 0.0;
    const double s_minus = (((f[2] + f[8]) + f[10]) + f[12]) + f[14];
    const double s_zero = (((((((f[0] + f[3]) + f[4]) + f[5]) + f[6]) + f[15]) + f[16]) + f[17]) + f[18];
    const double rho = (2.0 * s_minus + s_zero) / (1.0 - vx);
    const double ty = (((((f[18] + f[3]) + f[16]) - f[15]) - f[4]) - f[17]);
    const double tz = (((((f[17] + f[5]) + f[16]) - f[15]) - f[6]) - f[18]);
    const double a3 = rho * vx / 3.0, a6 = rho * vx / 6.0;
    f[1] = f[2] + a3;
    f[7] = ((f[8] + a6) + 0.5 * rho * vy) - 0.5 * ty;
    f[9] = ((f[10] + a6) - 0.5 * rho * vy) + 0.5 * ty;
    f[11] = ((f[12] + a6) + 0.5 * rho * vz) - 0.5 * tz;
    f[13] = ((f[14] + a6) - 0.5 * rho * vz) + 0.5 * tz;
}

}  // namespace exact
}  // namespace erlbm
