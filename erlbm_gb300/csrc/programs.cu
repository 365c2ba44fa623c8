// programs.cu -- host-side initial conditions, geometries and metrics of the reference's programs.
//
// These replace the parts of src/main_*.cpp that sit around the node loops, so that a caller of
// the ABI gets the same inputs the reference programs build.  Host code only, compiled without
// FMA contraction; every expression keeps the reference's operand order.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>

#include "../../include/erlbm_gb300.h"
#include "abi_internal.h"

namespace {

const int C9[9][3] = {{0, 0, 0}, {1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {1, 1, 0}, {-1, -1, 0}, {1, -1, 0}, {-1, 1, 0}};
const int C19[19][3] = {{0, 0, 0},  {1, 0, 0},  {-1, 0, 0}, {0, 1, 0},  {0, -1, 0}, {0, 0, 1},  {0, 0, -1},
                        {1, 1, 0},  {-1, -1, 0}, {1, -1, 0}, {-1, 1, 0}, {1, 0, 1},  {-1, 0, -1}, {1, 0, -1},
                        {-1, 0, 1}, {0, -1, -1}, {0, 1, 1},  {0, -1, 1}, {0, 1, -1}};

double weight(int q, int i)
{
    if (q == 9) return i == 0 ? 4. / 9. : (i < 5 ? 1. / 9. : 1. / 36.);
    return i == 0 ? 1. / 3. : (i < 7 ? 1. / 18. : 1. / 36.);
}

int cc(int q, int i, int a) { return q == 9 ? C9[i][a] : C19[i][a]; }

// dist_eq (LBM_functions.cpp:2945-3000) with the reference's dot_product order
void equilibrium(int q, double vx, double vy, double vz, double rho, double *feq)
{
    const int d = q == 9 ? 2 : 3;
    const double o = 3.;
    double vquad = vx * vx + vy * vy;
    if (d == 3) vquad = vquad + vz * vz;
    const double v[3] = {vx, vy, vz};
    for (int i = 0; i < q; i++) {
        double cv = 0.0;
        for (int a = 0; a < d; a++) cv = cv + (double)cc(q, i, a) * v[a];
        feq[i] = weight(q, i) * rho * (1.0 + cv * o + 0.5 * cv * cv * o * o - 0.5 * vquad * o);
    }
}

// calcula (LBM_functions.cpp:3518-3589)
void moments(int q, const double *f, double &ux, double &uy, double &uz, double &rho)
{
    const int d = q == 9 ? 2 : 3;
    double m[3] = {0.0, 0.0, 0.0}, r = 0.0;
    for (int i = 0; i < q; i++) {
        r = r + f[i];
        for (int a = 0; a < d; a++) m[a] = m[a] + (double)cc(q, i, a) * f[i];
    }
    ux = uy = uz = 0.0;
    if (r != 0.0) {
        const double inv = 1.0 / r;
        ux = m[0] * inv;
        uy = m[1] * inv;
        if (d == 3) uz = m[2] * inv;
    }
    rho = r;
}

}  // namespace

extern "C" {

int erlbm_init_taylor_green(int q, int L_, int nz, double u_0, double tau, int poisson, int neq, int variant,
                            double *aos)
{
    if ((q != 9 && q != 19) || L_ < 1 || nz < 1 || (q == 9 && nz != 1) || !aos) return ERLBM_E_INVAL;
    const double L = (double)L_;
    const double k = 2. * M_PI / L;
    const double cs2 = 1. / 3.;
    for (int z = 0; z < nz; z++)
        for (int y = 0; y < L_; y++)
            for (int x = 0; x < L_; x++) {
                double rho = 1.0, u_x, u_y, Sxx;
                if (variant == 0) {  // inicializa_taylor_green, main_taylor-green.cpp:57-100
                    if (poisson) rho = 1.0 + 0.75 * u_0 * u_0 * (cos(4. * M_PI * x / L) + cos(4. * M_PI * y / L));
                    u_x = u_0 * sin(2. * M_PI * x / L) * cos(2. * M_PI * y / L);
                    u_y = -u_0 * cos(2. * M_PI * x / L) * sin(2. * M_PI * y / L);
                    Sxx = 2. * u_0 * k * cos(k * x) * cos(k * y);
                } else {  // the same vortex translated by (L/4, L/4)
                    if (poisson) rho = 1.0 - 0.75 * u_0 * u_0 * (cos(4. * M_PI * x / L) + cos(4. * M_PI * y / L));
                    u_x = -u_0 * cos(2. * M_PI * x / L) * sin(2. * M_PI * y / L);
                    u_y = u_0 * sin(2. * M_PI * x / L) * cos(2. * M_PI * y / L);
                    Sxx = 2. * u_0 * k * sin(k * x) * sin(k * y);
                }
                double *f = aos + ((size_t)x + (size_t)y * L_ + (size_t)z * L_ * L_) * q;
                equilibrium(q, u_x, u_y, 0.0, rho, f);
                if (!neq) continue;
                const double Pxx = -rho * cs2 * tau * Sxx;
                const double Pyy = -Pxx;
                for (int i = 0; i < q; i++) {
                    const double cx = cc(q, i, 0), cy = cc(q, i, 1);
                    f[i] += weight(q, i) / (2. * cs2 * cs2) * ((cx * cx - cs2) * Pxx + (cy * cy - cs2) * Pyy);
                }
            }
    return ERLBM_OK;
}

int erlbm_init_double_shear(int L_, double rho_ini, double *aos)
{
    if (L_ < 1 || !aos) return ERLBM_E_INVAL;
    const double U_0 = 1. / 32., LAMBDA = 80., EPSILON = 0.05;  // main_double-shear-layer.cpp:259-261
    const double L = (double)L_;
    for (int y = 0; y < L_; y++)
        for (int x = 0; x < L_; x++) {
            double u_x = U_0 * tanh(LAMBDA * ((double)y / L - 1. / 4.));
            if (y > L_ / 2) u_x = U_0 * tanh(LAMBDA * (3. / 4. - (double)y / L));  // integer ny / 2 (:278)
            const double u_y = EPSILON * U_0 * sin(2. * M_PI * ((double)x / L + 1. / 4.));
            equilibrium(9, u_x, u_y, 0.0, rho_ini, aos + ((size_t)x + (size_t)y * L_) * 9);
        }
    return ERLBM_OK;
}

int erlbm_equilibrium(int q, double ux, double uy, double uz, double rho, double *feq)
{
    if ((q != 9 && q != 19) || !feq) return ERLBM_E_INVAL;
    equilibrium(q, ux, uy, uz, rho, feq);
    return ERLBM_OK;
}

int erlbm_obstacle_geometry(int sx, int sy, int *nx, int *ny, uint8_t *solid)
{
    if (sx < 1 || sy < 1 || !nx || !ny) return ERLBM_E_INVAL;
    // geometria_obstaculo (main_stability-map_obstacle.cpp:42-70), scaled by (sx, sy)
    const int NX = 20 * sx + 2, NY = 12 * sy;
    *nx = NX;
    *ny = NY;
    if (!solid) return ERLBM_OK;
    for (int y = 0; y < NY; y++)
        for (int x = 0; x < NX; x++) {
            int s = 0;
            if (x == 0 || x == NX - 1) s = 1;
            if (x >= 7 * sx && x <= 9 * sx - 1 && y >= 4 * sy && y <= 8 * sy - 1) s = 1;
            solid[x + y * NX] = (uint8_t)s;
        }
    return ERLBM_OK;
}

int erlbm_taylor_green_error(int q, int L_, const double *aos, double u_0, double visc, int step, int variant,
                             double *out)
{
    if ((q != 9 && q != 19) || !aos || !out) return ERLBM_E_INVAL;
    // main_taylor-green.cpp:178-213
    const double L = (double)L_;
    const double k = 2. * M_PI / L;
    double s_mag = 0, s_vec = 0, s_r = 0, s_proj = 0, s_phi = 0;
    const double e = exp(-2. * visc * k * k * step);
    for (int y = 0; y < L_; y++)
        for (int x = 0; x < L_; x++) {
            double vx, vy, vz, rho;
            moments(q, aos + ((size_t)x + (size_t)y * L_) * q, vx, vy, vz, rho);
            double rx, ry, px, py;
            if (variant == 0) {
                rx = u_0 * e * sin(k * x) * cos(k * y);
                ry = -u_0 * e * cos(k * x) * sin(k * y);
                px = sin(k * x) * cos(k * y);
                py = -cos(k * x) * sin(k * y);
            } else {
                rx = -u_0 * e * cos(k * x) * sin(k * y);
                ry = u_0 * e * sin(k * x) * cos(k * y);
                px = -cos(k * x) * sin(k * y);
                py = sin(k * x) * cos(k * y);
            }
            const double us = sqrt(vx * vx + vy * vy + vz * vz), ur = sqrt(rx * rx + ry * ry);
            s_mag += (us - ur) * (us - ur);
            s_vec += (vx - rx) * (vx - rx) + (vy - ry) * (vy - ry) + vz * vz;
            s_r += ur * ur;
            s_proj += vx * px + vy * py;
            s_phi += px * px + py * py;
        }
    const double A = s_proj / s_phi / u_0;
    const double nu_ef = -log(A) / (2. * k * k * step);
    out[0] = sqrt(s_vec / s_r);
    out[1] = sqrt(s_mag / s_r);
    out[2] = nu_ef / visc - 1.;
    return ERLBM_OK;
}

// Map axes (main_stability-map_taylor-green.cpp:134-164)
int erlbm_tg_map_params(int i, int j, int n_ma, int n_nu, int op, double tau_nh_in, double *u0, double *tau,
                        double *tau_nh)
{
    if (!u0 || !tau || !tau_nh || n_ma < 1 || n_nu < 1) return ERLBM_E_INVAL;
    const double c_s = 1. / sqrt(3.);
    const double u_min = 0.05 * c_s;
    const double log_nu_min = -5., log_nu_max = -2.;
    *u0 = u_min + (i + 1) * (c_s - u_min) / n_ma;
    const double log_nu = log_nu_min + j * (log_nu_max - log_nu_min) / n_nu;
    *tau = 3. * pow(10., log_nu) + 0.5;
    *tau_nh = (op == ERLBM_OP_REG) ? 1.0 : tau_nh_in;
    return ERLBM_OK;
}

// Map axes (main_stability-map_obstacle.cpp:147-173)
int erlbm_obstacle_map_params(int i, int j, int n_tau, int n_nu, double ma, double *u_imp, double *tau,
                              double *tau_nh)
{
    if (!u_imp || !tau || !tau_nh || n_tau < 1 || n_nu < 1) return ERLBM_E_INVAL;
    const double tau_nh_min = 0.5, tau_nh_max = 1.1;
    const double log_nu_min = -5., log_nu_max = -0.7;
    const double log_nu = log_nu_min + j * (log_nu_max - log_nu_min) / n_nu;
    *tau = 3. * pow(10., log_nu) + 0.5;
    *tau_nh = tau_nh_min + (double)i * (tau_nh_max - tau_nh_min) / n_tau;
    *u_imp = ma / sqrt(3.);
    return ERLBM_OK;
}

// read_geo (LBM_functions.cpp:282-353): skip four header lines, read "DIMENSIONS nx ny nz", skip five
// more, then one integer per node of the file's box (x fastest, nonzero = fluid).  pts_in / pts_out
// layers of fluid are added before and after in x; with `wall` the first and last x planes of the
// widened box are solid (the reference's overload without the flag always adds them).
int erlbm_read_geo(const char *path, int pts_in, int pts_out, int wall, int *nx, int *ny, int *nz, uint8_t *solid,
                   size_t n)
{
    if (!path || !nx || !ny || !nz || pts_in < 0 || pts_out < 0) return ERLBM_E_INVAL;
    std::ifstream fm(path);
    if (!fm) {
        erlbm::set_error("cannot open %s%s", path, "");
        return ERLBM_E_INVAL;
    }
    std::string line, dump;
    for (int i = 0; i < 4; i++) std::getline(fm, dump);
    std::getline(fm, line);
    std::stringstream dados(line);
    int fx = 0, fy = 0, fz = 0;
    dados >> dump >> fx >> fy >> fz;
    for (int i = 0; i < 5; i++) std::getline(fm, dump);
    if (!fm || fx < 1 || fy < 1 || fz < 1) {
        erlbm::set_error("%s is not a legacy VTK geometry file%s", path, "");
        return ERLBM_E_INVAL;
    }
    const int X = fx + pts_in + pts_out;
    *nx = X;
    *ny = fy;
    *nz = fz;
    const size_t total = (size_t)X * fy * fz;
    if (!solid) return ERLBM_OK;  // dimensions only
    if (n != total) return ERLBM_E_INVAL;
    for (int z = 0; z < fz; z++)
        for (int y = 0; y < fy; y++)
            for (int x = 0; x < X; x++) {
                const size_t pos = x + (size_t)y * X + (size_t)z * fy * X;
                bool fluid;
                if (x >= pts_in && x < X - pts_out) {
                    int v = 0;
                    fm >> v;
                    if (!fm) {
                        erlbm::set_error("%s ends before its last node%s", path, "");
                        return ERLBM_E_INVAL;
                    }
                    fluid = v != 0;
                } else {
                    fluid = !((x == 0 || x == X - 1) && wall);
                }
                solid[pos] = fluid ? 0 : 1;
            }
    return ERLBM_OK;
}

}  // extern "C"
