// lattice.cuh -- compile-time D2Q9 / D3Q19 velocity sets.
//
// Velocity order and weights are the reference's (def_lattice_d2q9, LBM_functions.cpp:1437-1501;
// def_lattice_d3q19, LBM_functions.cpp:577-708): populations exchanged with callers use that
// order, and opposite directions are the adjacent pairs (2k-1, 2k).
#pragma once

#include <cstdint>

namespace erlbm {

template <int Q>
struct Lat;

template <>
struct Lat<9> {
    static constexpr int Q = 9;
    static constexpr int D = 2;
    __host__ __device__ static constexpr int cx(int i)
    {
        return i == 1 || i == 5 || i == 7 ? 1 : (i == 2 || i == 6 || i == 8 ? -1 : 0);
    }
    __host__ __device__ static constexpr int cy(int i)
    {
        return i == 3 || i == 5 || i == 8 ? 1 : (i == 4 || i == 6 || i == 7 ? -1 : 0);
    }
    __host__ __device__ static constexpr int cz(int) { return 0; }
    __host__ __device__ static constexpr double w(int i) { return i == 0 ? 4. / 9. : (i < 5 ? 1. / 9. : 1. / 36.); }
    __host__ __device__ static constexpr int opp(int i) { return i == 0 ? 0 : (i % 2 ? i + 1 : i - 1); }
};

template <>
struct Lat<19> {
    static constexpr int Q = 19;
    static constexpr int D = 3;
    __host__ __device__ static constexpr int cx(int i)
    {
        return (i == 1 || i == 7 || i == 9 || i == 11 || i == 13) ? 1
               : (i == 2 || i == 8 || i == 10 || i == 12 || i == 14) ? -1
                                                                     : 0;
    }
    __host__ __device__ static constexpr int cy(int i)
    {
        return (i == 3 || i == 7 || i == 10 || i == 16 || i == 18) ? 1
               : (i == 4 || i == 8 || i == 9 || i == 15 || i == 17) ? -1
                                                                    : 0;
    }
    __host__ __device__ static constexpr int cz(int i)
    {
        return (i == 5 || i == 11 || i == 14 || i == 16 || i == 17) ? 1
               : (i == 6 || i == 12 || i == 13 || i == 15 || i == 18) ? -1
                                                                      : 0;
    }
    __host__ __device__ static constexpr double w(int i) { return i == 0 ? 1. / 3. : (i < 7 ? 1. / 18. : 1. / 36.); }
    __host__ __device__ static constexpr int opp(int i) { return i == 0 ? 0 : (i % 2 ? i + 1 : i - 1); }
};

// Collision operators, numbered like COLISAO (src/erlbm_common.h:42).
enum Op : int { OP_BGK = 1, OP_MRT = 2, OP_REG = 3, OP_EXTREG = 4 };

// Relaxation parameters of one run, as the reference derives them (Collision_operators.cpp:1192-1194,
// 870, 20): omega_1 = 1 - 1/tau, omega_gt1 = 1 - 1/tau_nh, inv_tau = 1/tau.
struct Relax {
    double omega_1, omega_gt1, inv_tau;
    int op;
};

// d'Humieres' MRT moment basis for D2Q9 (coll_MRT, Collision_operators.cpp:459-470): moments rho, e,
// eps, jx, qx, jy, qy, pxx, pxy.  Each row of the transform M is a polynomial in c evaluated on the
// velocity set; the rows are orthogonal, so M^-1 = M^T diag(1 / |row|^2).
__host__ __device__ constexpr int mrt9_m(int row, int i)
{
    const int cx = Lat<9>::cx(i), cy = Lat<9>::cy(i), c2 = cx * cx + cy * cy;
    return row == 0   ? 1
           : row == 1 ? 3 * c2 - 4
           : row == 2 ? (9 * c2 * c2 - 21 * c2 + 8) / 2
           : row == 3 ? cx
           : row == 4 ? (3 * c2 - 5) * cx
           : row == 5 ? cy
           : row == 6 ? (3 * c2 - 5) * cy
           : row == 7 ? cx * cx - cy * cy
                      : cx * cy;
}

__host__ __device__ constexpr int mrt9_norm2(int row)
{
    int n = 0;
    for (int i = 0; i < 9; i++) n += mrt9_m(row, i) * mrt9_m(row, i);
    return n;
}

// MRT relaxation rates of the D2Q9 ghost moments (Collision_operators.cpp:586-594); the shear rates
// s_7 = s_8 are 1/tau.
constexpr double MRT9_SE = 1.6, MRT9_SEPS = 1.8, MRT9_SQ = 1.9;

__host__ __device__ inline Relax make_relax(double tau, double tau_nh, int op)
{
    Relax r;
    r.omega_1 = 1.0 - 1.0 / tau;
    r.omega_gt1 = 1.0 - 1.0 / tau_nh;
    r.inv_tau = 1.0 / tau;
    r.op = op;
    return r;
}

}  // namespace erlbm
