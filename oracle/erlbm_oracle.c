/*
 * erlbm_oracle.c -- TEST INFRASTRUCTURE, NOT THE PRODUCT.
 *
 * A plain-C, FP64, CPU restatement of the reference's E-RLBM collide-stream path (SimBoltz as
 * shipped with ERLBM).  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
 * load it, and only as the checker or the timed CPU baseline.  The CUDA library never calls it.
 *
 * Layout and arithmetic follow the reference on purpose, so that the CUDA FP64 path can be
 * checked bit for bit and so that timing this file is a fair stand-in for the reference's own
 * OpenMP loops:
 *   - populations are AoS in fluid-index order, f[pto*Q + i] (src/erlbm_common.h:86-99,144-148);
 *   - streaming is a push through an int map built like def_dir_prop
 *     (SimBoltz_Functions/LBM_functions.cpp:1967-2311) and applied like propag_site (:3886-3955);
 *   - every floating-point expression keeps the reference's operand order, and the file is
 *     compiled with -ffp-contract=off, as GCC does for the reference's -std=c++17 build.
 *
 * Pinning: tests check this file against (1) the reference's published tables
 * (data/fig3_taylor_green_Re50*.csv, data/kappa4_check_L64.csv) and (2) golden vectors produced
 * by the reference library itself compiled from its own sources (oracle/ref_harness.cpp), kept
 * in tests/golden/ together with the script that made them.
 */
#define _DEFAULT_SOURCE /* M_PI, as the reference gets it from <cmath> */
#include <math.h>
#include <stdio.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "erlbm_oracle.h"

/* ------------------------------------------------------------------------------------------ */
/* Lattice tables: def_lattice_d2q9 (LBM_functions.cpp:1437-1501), def_lattice_d3q19 (577-708), */
/* calc_Q (5815-5829).  Velocity order, weights and c_s^2 = 1/3 are those of the reference.     */
/* ------------------------------------------------------------------------------------------ */

typedef struct {
    int q, dim;
    double c[19 * 3];
    double w[19];
    double Qt[19 * 9];
    int opp[19];
    double cs2, ocs2;
} tables_t;

static const int D2Q9_C[9][2] = {{0, 0}, {1, 0}, {-1, 0}, {0, 1}, {0, -1}, {1, 1}, {-1, -1}, {1, -1}, {-1, 1}};
static const int D3Q19_C[19][3] = {{0, 0, 0},  {1, 0, 0},   {-1, 0, 0}, {0, 1, 0},  {0, -1, 0},
                                   {0, 0, 1},  {0, 0, -1},  {1, 1, 0},  {-1, -1, 0}, {1, -1, 0},
                                   {-1, 1, 0}, {1, 0, 1},   {-1, 0, -1}, {1, 0, -1}, {-1, 0, 1},
                                   {0, -1, -1}, {0, 1, 1},  {0, -1, 1}, {0, 1, -1}};

static void make_tables(tables_t *t, int q)
{
    memset(t, 0, sizeof(*t));
    t->q = q;
    t->dim = (q == 9) ? 2 : 3;
    for (int i = 0; i < q; i++)
        for (int a = 0; a < t->dim; a++)
            t->c[i * t->dim + a] = (double)(q == 9 ? D2Q9_C[i][a] : D3Q19_C[i][a]);
    if (q == 9) {
        t->w[0] = 4. / 9.;
        for (int i = 1; i < 5; i++) t->w[i] = 1. / 9.;
        for (int i = 5; i < 9; i++) t->w[i] = 1. / 36.;
    } else {
        t->w[0] = 1. / 3.;
        for (int i = 1; i < 7; i++) t->w[i] = 1. / 18.;
        for (int i = 7; i < 19; i++) t->w[i] = 1. / 36.;
    }
    t->cs2 = 1. / 3.;
    t->ocs2 = 3.;
    const int d = t->dim;
    for (int i = 0; i < q; i++)
        for (int a = 0; a < d; a++)
            for (int b = 0; b < d; b++)
                t->Qt[a + b * d + i * d * d] = t->c[i * d + a] * t->c[i * d + b] - (t->cs2) * (double)(a == b);
    for (int i = 0; i < q; i++) {
        t->opp[i] = 0;
        for (int j = 0; j < q; j++) {
            int same = 1;
            for (int a = 0; a < d; a++)
                if (t->c[j * d + a] != -t->c[i * d + a]) same = 0;
            if (same) t->opp[i] = j;
        }
    }
}

static tables_t T9, T19;
static int tables_ready = 0;

static const tables_t *tables_for(int q)
{
    if (!tables_ready) {
        make_tables(&T9, 9);
        make_tables(&T19, 19);
        tables_ready = 1;
    }
    return q == 9 ? &T9 : &T19;
}

/* ------------------------------------------------------------------------------------------ */
/* Per-site functions                                                                          */
/* ------------------------------------------------------------------------------------------ */

/* dot_product (LBM_functions.cpp:2865-2876): left-to-right sum starting from 0.0 */
static inline double dotv(const double *a, const double *b, int d)
{
    double r = 0.0;
    for (int k = 0; k < d; k++) r = r + a[k] * b[k];
    return r;
}

/* calcula (LBM_functions.cpp:3518-3589): rho = sum f, m = sum c f, u = m * (1/rho), u = 0 if rho == 0 */
static inline void moments(const tables_t *t, const double *f, double *u, double *rho)
{
    const int d = t->dim;
    double m[3] = {0.0, 0.0, 0.0};
    double r = 0.0;
    u[0] = u[1] = u[2] = 0.0;
    for (int i = 0; i < t->q; i++) {
        r = r + f[i];
        for (int a = 0; a < d; a++) m[a] = m[a] + t->c[i * d + a] * f[i];
    }
    if (r != 0.0) {
        const double inv = 1.0 / (r);
        for (int a = 0; a < d; a++) u[a] = m[a] * inv;
    } else {
        for (int a = 0; a < d; a++) u[a] = 0.;
    }
    *rho = r;
}

/* dist_eq (LBM_functions.cpp:2945-3000): w rho (1 + cu/cs2 + (cu)^2/(2cs4) - u^2/(2cs2)) */
static inline void equilibrium(const tables_t *t, const double *u, double rho, double *feq)
{
    const int d = t->dim;
    const double o = t->ocs2;
    double vq = u[0] * u[0] + u[1] * u[1];
    if (d == 3) vq = vq + u[2] * u[2];
    for (int i = 0; i < t->q; i++) {
        const double cv = dotv(&t->c[i * d], u, d);
        feq[i] = t->w[i] * rho * (1.0 + cv * o + 0.5 * cv * cv * o * o - 0.5 * vq * o);
    }
}

/* source (LBM_functions.cpp:5646-5716).  Every program passes zero acceleration, so S is +0.0
 * for finite states; it is kept so that the oracle's non-finite payloads match the reference. */
static inline void forcing(const tables_t *t, const double *F, const double *u, double tau, double *S)
{
    const int d = t->dim;
    const double o = t->ocs2;
    const double factor = (1. - 1. / (2. * tau));
    const double vF = dotv(F, u, d);
    for (int i = 0; i < t->q; i++) {
        const double cF = dotv(&t->c[i * d], F, d);
        const double cv = dotv(&t->c[i * d], u, d);
        S[i] = factor * t->w[i] * o * (cF + o * cF * cv - vF);
    }
}

/* Common front part of coll_BGK / coll_Reg / coll_Ext_Reg: moments, forcing-shifted velocity,
 * source and equilibrium (Collision_operators.cpp:12-36, 860-888, 1182-1213). */
static inline void collide_front(const tables_t *t, const double *f, double tau, double *feq, double *S)
{
    double u[3], rho;
    moments(t, f, u, &rho);
    const double acc[3] = {0., 0., 0.};
    double ua[3], F[3];
    for (int a = 0; a < 3; a++) ua[a] = u[a] + 0.5 * acc[a];
    for (int a = 0; a < 3; a++) F[a] = acc[a] * rho;
    forcing(t, F, ua, tau, S);
    equilibrium(t, ua, rho, feq);
}

/* Second-order Hermite projection f1 = w/(2cs^4) Q_i : Pi^neq (Collision_operators.cpp:1216-1245 for
 * D2Q9, 1259-1295 for D3Q19).  Pi accumulates ((f - feq) c_a) c_b in velocity order. */
static inline void hermite_f1(const tables_t *t, const double *f, const double *feq, double *f1)
{
    const int d = t->dim;
    const double o2cs4 = 0.5 * t->ocs2 * t->ocs2;
    if (d == 2) {
        double pxx = 0.0, pyy = 0.0, pxy = 0.0;
        for (int i = 0; i < t->q; i++) {
            const double cx = t->c[i * 2], cy = t->c[i * 2 + 1];
            pxx = pxx + (f[i] - feq[i]) * cx * cx;
            pyy = pyy + (f[i] - feq[i]) * cy * cy;
            pxy = pxy + (f[i] - feq[i]) * cx * cy;
        }
        for (int i = 0; i < t->q; i++) {
            const double *Q = &t->Qt[i * 4];
            f1[i] = o2cs4 * t->w[i] * (Q[0] * pxx + Q[3] * pyy + 2 * Q[1] * pxy);
        }
    } else {
        double pxx = 0.0, pyy = 0.0, pzz = 0.0, pxy = 0.0, pxz = 0.0, pyz = 0.0;
        for (int i = 0; i < t->q; i++) {
            const double cx = t->c[i * 3], cy = t->c[i * 3 + 1], cz = t->c[i * 3 + 2];
            pxx = pxx + (f[i] - feq[i]) * cx * cx;
            pyy = pyy + (f[i] - feq[i]) * cy * cy;
            pzz = pzz + (f[i] - feq[i]) * cz * cz;
            pxy = pxy + (f[i] - feq[i]) * cx * cy;
            pxz = pxz + (f[i] - feq[i]) * cx * cz;
            pyz = pyz + (f[i] - feq[i]) * cy * cz;
        }
        for (int i = 0; i < t->q; i++) {
            const double *Q = &t->Qt[i * 9];
            f1[i] = o2cs4 * t->w[i] *
                    (Q[0] * pxx + Q[4] * pyy + Q[8] * pzz + 2 * Q[1] * pxy + 2 * Q[2] * pxz + 2 * Q[5] * pyz);
        }
    }
}

/* MRT transform of d'Humieres (D2Q9; moments rho, e, eps, jx, qx, jy, qy, pxx, pxy), as used by
 * coll_MRT (Collision_operators.cpp:459-470).  Each row of M is a polynomial in c evaluated on the
 * velocity set; the rows are orthogonal, so M^-1 = M^T diag(1 / |row|^2), every entry a correctly
 * rounded quotient of two integers, which is what the reference's literals (1./9., -1./36., ...)
 * evaluate to. */
static int mrt9_row(int row, int cx, int cy)
{
    const int c2 = cx * cx + cy * cy;
    switch (row) {
    case 0: return 1;
    case 1: return 3 * c2 - 4;
    case 2: return (9 * c2 * c2 - 21 * c2 + 8) / 2;
    case 3: return cx;
    case 4: return (3 * c2 - 5) * cx;
    case 5: return cy;
    case 6: return (3 * c2 - 5) * cy;
    case 7: return cx * cx - cy * cy;
    default: return cx * cy;
    }
}

static double MRT9_M[9][9], MRT9_MINV[9][9];
static int mrt9_ready = 0;

static void mrt9_tables(void)
{
    if (mrt9_ready) return;
    for (int r = 0; r < 9; r++) {
        int n2 = 0;
        for (int i = 0; i < 9; i++) {
            const int m = mrt9_row(r, D2Q9_C[i][0], D2Q9_C[i][1]);
            MRT9_M[r][i] = (double)m;
            n2 += m * m;
        }
        for (int i = 0; i < 9; i++) MRT9_MINV[i][r] = MRT9_M[r][i] / (double)n2;
    }
    mrt9_ready = 1;
}

/* coll_MRT, D2Q9 branch (Collision_operators.cpp:583-699): moments of f and f_eq by M (sums from
 * 0.0 in column order), relaxation m - s (m - m_eq) + (1 - s/2) F_m with the rates of :586-594,
 * back-transform by M^-1.  F_m is the transform of a zero force term. */
static void collide_mrt9(const tables_t *t, double *f, double tau)
{
    const double s[9] = {0.0, 1.6, 1.8, 0.0, 1.9, 0.0, 1.9, 1. / tau, 1. / tau};
    double u[3], rho, feq[9];
    mrt9_tables();
    moments(t, f, u, &rho);
    equilibrium(t, u, rho, feq);
    double m[9], meq[9], fm[9];
    const double Sf[9] = {0.0};
    for (int r = 0; r < 9; r++) {
        m[r] = 0.0;
        meq[r] = 0.0;
        fm[r] = 0.0;
        for (int c = 0; c < 9; c++) {
            m[r] = m[r] + MRT9_M[r][c] * f[c];
            meq[r] = meq[r] + MRT9_M[r][c] * feq[c];
            fm[r] = fm[r] + MRT9_M[r][c] * Sf[c];
        }
    }
    for (int r = 0; r < 9; r++) m[r] = m[r] - s[r] * (m[r] - meq[r]) + (1.0 - 0.5 * s[r]) * fm[r];
    for (int i = 0; i < 9; i++) {
        f[i] = 0.0;
        for (int c = 0; c < 9; c++) f[i] = f[i] + MRT9_MINV[i][c] * m[c];
    }
}

/* One node's collision, in place.  op: ORC_OP_BGK (coll_BGK, Collision_operators.cpp:12-49),
 * ORC_OP_MRT (coll_MRT, :487-701), ORC_OP_REG (coll_Reg, :860-967), ORC_OP_EXTREG (coll_Ext_Reg,
 * :1182-1307).  The reference's dispatch (src/erlbm_common.h:69-80) compiles coll_MRT only into
 * D2Q9 builds; in a D3Q19 build it matches no case and the site is not collided, as here. */
static void collide_site(const tables_t *t, double *f, int op, double tau, double tau_nh)
{
    double feq[19], S[19];
    if (op == ORC_OP_MRT) {
        if (t->q == 9) collide_mrt9(t, f, tau);
        return;
    }
    collide_front(t, f, tau, feq, S);
    if (op == ORC_OP_BGK) {
        const double one_over_tau = 1.0 / tau;
        for (int i = 0; i < t->q; i++) {
            const double opc = (feq[i] - f[i]) * one_over_tau;
            f[i] = f[i] + opc + S[i];
        }
        return;
    }
    double f1[19];
    hermite_f1(t, f, feq, f1);
    if (op == ORC_OP_REG) {
        const double one_over_tau = 1.0 / tau;
        for (int i = 0; i < t->q; i++) f[i] = feq[i] + (1.0 - one_over_tau) * f1[i] + S[i];
        return;
    }
    const double omega_1 = 1.0 - 1.0 / tau;
    const double omega_gt1 = 1.0 - 1.0 / tau_nh;
    double fgt1[19];
    for (int i = 0; i < t->q; i++) fgt1[i] = f[i] - feq[i] - f1[i];
    for (int i = 0; i < t->q; i++) f[i] = feq[i] + omega_1 * f1[i] + omega_gt1 * fgt1[i] + S[i];
}

/* density (LBM_functions.cpp:5544-5552) */
static inline double site_density(const double *f, int q)
{
    double r = 0.0;
    for (int i = 0; i < q; i++) r = r + f[i];
    return r;
}

/* ------------------------------------------------------------------------------------------ */
/* Lattice object                                                                              */
/* ------------------------------------------------------------------------------------------ */

struct orc_lattice {
    const tables_t *t;
    int q, nx, ny, nz, n_fluid;
    int *ini;     /* geometry.ini: 0 solid, else 1-based fluid index (erlbm_common.h:86-99) */
    int *stream;  /* ini_stream push map (def_dir_prop) */
    double *f, *fnew;
    double tau, tau_nh;
    int op;
};

static inline int wrapi(int a, int n) { return ((a % n) + n) % n; }

/* def_dir_prop for unit-speed lattices (LBM_functions.cpp:1967-2311): the push target of direction
 * i is the periodic neighbour x + c_i; if that node is solid the population returns to its own
 * node in the opposite direction (halfway bounce-back, :2099-2128 / :2270-2300). */
static void build_stream_map(orc_lattice *L)
{
    const tables_t *t = L->t;
    const int d = t->dim;
    for (int z = 0; z < L->nz; z++)
        for (int y = 0; y < L->ny; y++)
            for (int x = 0; x < L->nx; x++) {
                const int self = L->ini[x + y * L->nx + z * L->nx * L->ny];
                if (!self) continue;
                int *dir = L->stream + (size_t)(self - 1) * L->q;
                dir[0] = (self - 1) * L->q;
                for (int i = 1; i < L->q; i++) {
                    const int cx = (int)t->c[i * d], cy = (int)t->c[i * d + 1];
                    const int cz = (d == 3) ? (int)t->c[i * d + 2] : 0;
                    const int xn = wrapi(x + cx, L->nx), yn = wrapi(y + cy, L->ny), zn = wrapi(z + cz, L->nz);
                    const int nb = L->ini[xn + yn * L->nx + zn * L->nx * L->ny];
                    if (nb)
                        dir[i] = i + (nb - 1) * L->q;
                    else
                        dir[i] = t->opp[i] + (self - 1) * L->q;
                }
            }
}

orc_lattice *orc_create(int q, int nx, int ny, int nz, const uint8_t *solid, double tau, double tau_nh, int op)
{
    if ((q != 9 && q != 19) || nx <= 0 || ny <= 0 || nz <= 0) return NULL;
    if (q == 9 && nz != 1) return NULL;
    orc_lattice *L = (orc_lattice *)calloc(1, sizeof(orc_lattice));
    L->t = tables_for(q);
    L->q = q;
    L->nx = nx;
    L->ny = ny;
    L->nz = nz;
    L->tau = tau;
    L->tau_nh = tau_nh;
    L->op = op;
    const size_t nb = (size_t)nx * ny * nz;
    L->ini = (int *)malloc(nb * sizeof(int));
    int n = 0;
    for (size_t k = 0; k < nb; k++) L->ini[k] = (solid && solid[k]) ? 0 : ++n; /* numera_fluido */
    L->n_fluid = n;
    L->stream = (int *)malloc((size_t)n * q * sizeof(int));
    L->f = (double *)calloc((size_t)n * q, sizeof(double));
    L->fnew = (double *)calloc((size_t)n * q, sizeof(double));
    build_stream_map(L);
    return L;
}

void orc_destroy(orc_lattice *L)
{
    if (!L) return;
    free(L->ini);
    free(L->stream);
    free(L->f);
    free(L->fnew);
    free(L);
}

int orc_fluid_count(const orc_lattice *L) { return L->n_fluid; }

void orc_set_params(orc_lattice *L, double tau, double tau_nh, int op)
{
    L->tau = tau;
    L->tau_nh = tau_nh;
    L->op = op;
}

void orc_set_populations(orc_lattice *L, const double *aos)
{
    memcpy(L->f, aos, (size_t)L->n_fluid * L->q * sizeof(double));
}

/* stage 0: populations the next step starts from (post-stream; lattice.inif after the swap).
 * stage 1: post-collision populations of the last step, before streaming: after the swap they
 *          sit in lattice.inif_new, which is what main_taylor-green.cpp:164-214 and
 *          main_double-shear-layer.cpp:402-428 measure. */
void orc_get_populations(const orc_lattice *L, double *aos, int stage)
{
    memcpy(aos, stage ? L->fnew : L->f, (size_t)L->n_fluid * L->q * sizeof(double));
}

/* ZouHeD3Q19_vx_x, left-plane branch (Boundary_conditions.cpp:350-403): velocity inlet on plane x. */
static void zou_he_inlet(orc_lattice *L, int px, double vx)
{
    if (L->q != 19) return;
    const int left = px < L->nx / 2;
    for (int y = 0; y < L->ny; y++)
        for (int z = 0; z < L->nz; z++) {
            const int m = L->ini[px + y * L->nx + z * L->ny * L->nx];
            if (!m) continue;
            double *f = L->f + (size_t)(m - 1) * 19;
            const double vy = 0.0, vz = 0.0;
            if (left) {
                const double s_minus = f[1] + f[7] + f[9] + f[11] + f[13];
                const double s_zero = f[0] + f[3] + f[4] + f[5] + f[6] + f[15] + f[16] + f[17] + f[18];
                const double rho = (2.0 * s_minus + s_zero) / (1.0 - vx);
                f[1] = f[1] + rho * vx / 3.0;
                f[7] = f[7] + rho * vx / 6.0 + 0.5 * rho * vy - 0.5 * (f[18] + f[3] + f[16] - f[15] - f[4] - f[17]);
                f[9] = f[9] + rho * vx / 6.0 - 0.5 * rho * vy + 0.5 * (f[18] + f[3] + f[16] - f[15] - f[4] - f[17]);
                f[11] = f[11] + rho * vx / 6.0 + 0.5 * rho * vz - 0.5 * (f[17] + f[5] + f[16] - f[15] - f[6] - f[18]);
                f[13] = f[13] + rho * vx / 6.0 - 0.5 * rho * vz + 0.5 * (f[17] + f[5] + f[16] - f[15] - f[6] - f[18]);
            } else { /* right-plane branch (Boundary_conditions.cpp:404-436) */
                const double s_plus = f[2] + f[8] + f[10] + f[12] + f[14];
                const double s_zero = f[0] + f[3] + f[4] + f[5] + f[6] + f[15] + f[16] + f[17] + f[18];
                const double rho = (2.0 * s_plus + s_zero) / (1.0 - vx);
                f[2] = f[2] - rho * vx / 3.0;
                f[10] = f[10] - rho * vx / 6.0 + 0.5 * rho * vy - 0.5 * (f[18] + f[3] + f[16] - f[15] - f[4] - f[17]);
                f[8] = f[8] - rho * vx / 6.0 - 0.5 * rho * vy + 0.5 * (f[18] + f[3] + f[16] - f[15] - f[4] - f[17]);
                f[14] = f[14] - rho * vx / 6.0 + 0.5 * rho * vz - 0.5 * (f[17] + f[5] + f[16] - f[15] - f[6] - f[18]);
                f[12] = f[12] - rho * vx / 6.0 - 0.5 * rho * vz + 0.5 * (f[17] + f[5] + f[16] - f[15] - f[6] - f[18]);
            }
        }
}

/* ZouHeD2Q9_vx_x (Boundary_conditions.cpp:710-744): the +x movers set from the closure density */
static void zou_he_d2q9(orc_lattice *L, int px, double vx)
{
    for (int y = 0; y < L->ny; y++) {
        const int m = L->ini[px + y * L->nx];
        if (!m) continue;
        double *f = L->f + (size_t)(m - 1) * 9;
        const double rho = (f[0] + f[3] + f[4] + 2 * (f[2] + f[8] + f[6])) / (1. - vx);
        f[1] = (rho / 9.0) * (1.0 + 3.0 * vx + 3.0 * vx * vx);
        f[5] = (rho / 36.0) * (1.0 + 3.0 * vx + 3.0 * vx * vx);
        f[7] = (rho / 36.0) * (1.0 + 3.0 * vx + 3.0 * vx * vx);
    }
}

/* the parabolic profile of parabolic_D3Q19_x / parabolic_D2Q9_x (:467-472, :759-764) at the h-th
 * fluid node of a column (h from 1) */
static double parabolic_vel(int h, double vx_max, int Lw)
{
    const double d_h = (double)h - 0.5;
    return -4.0 * vx_max / (Lw * Lw) * (d_h) * (d_h - Lw);
}

/* parabolic_D3Q19_x (:456-530) and parabolic_D2Q9_x (:748-800): a Zou-He closure with the profile's
 * velocity, the h-th fluid node of each column (per z) taking the h-th value; D3Q19 sets the +x
 * movers from their opposites */
static void parabolic_inlet(orc_lattice *L, int px, double vx_max, int Lw)
{
    for (int z = 0; z < L->nz; z++) {
        int h = 0;
        for (int y = 0; y < L->ny; y++) {
            const int m = L->ini[px + y * L->nx + z * L->ny * L->nx];
            if (!m) continue;
            h++;
            const double vx = parabolic_vel(h, vx_max, Lw);
            double *f = L->f + (size_t)(m - 1) * L->q;
            if (L->q == 9) {
                const double rho = (f[0] + f[3] + f[4] + 2 * (f[2] + f[8] + f[6])) / (1. - vx);
                f[1] = (rho / 9.0) * (1.0 + 3.0 * vx + 3.0 * vx * vx);
                f[5] = (rho / 36.0) * (1.0 + 3.0 * vx + 3.0 * vx * vx);
                f[7] = (rho / 36.0) * (1.0 + 3.0 * vx + 3.0 * vx * vx);
                continue;
            }
            const double sum_f_xminus = f[2] + f[8] + f[10] + f[12] + f[14];
            const double sum_f_xzero = f[0] + f[3] + f[4] + f[5] + f[6] + f[15] + f[16] + f[17] + f[18];
            const double rho = (2.0 * sum_f_xminus + sum_f_xzero) / (1.0 - vx);
            const double vy = 0.0, vz = 0.0;
            f[1] = f[2] + rho * vx / 3.0;
            f[7] = f[8] + rho * vx / 6.0 + 0.5 * rho * vy - 0.5 * (f[18] + f[3] + f[16] - f[15] - f[4] - f[17]);
            f[9] = f[10] + rho * vx / 6.0 - 0.5 * rho * vy + 0.5 * (f[18] + f[3] + f[16] - f[15] - f[4] - f[17]);
            f[11] = f[12] + rho * vx / 6.0 + 0.5 * rho * vz - 0.5 * (f[17] + f[5] + f[16] - f[15] - f[6] - f[18]);
            f[13] = f[14] + rho * vx / 6.0 - 0.5 * rho * vz + 0.5 * (f[17] + f[5] + f[16] - f[15] - f[6] - f[18]);
        }
    }
}

/* OpenBoundaryD2Q9_x (:584-621): the populations entering from outside copied from the inner
 * neighbour (solid nodes, which the reference does not test for, are skipped) */
static void open_x(orc_lattice *L, int px)
{
    const int d = (px < L->nx / 2) ? 1 : -1;
    for (int y = 0; y < L->ny; y++) {
        const int m = L->ini[px + y * L->nx], ma = L->ini[px + d + y * L->nx];
        if (!m || !ma) continue;
        double *f = L->f + (size_t)(m - 1) * 9;
        const double *fa = L->f + (size_t)(ma - 1) * 9;
        if (d > 0) {
            f[1] = fa[1];
            f[5] = fa[5];
            f[7] = fa[7];
        } else {
            f[2] = fa[2];
            f[6] = fa[6];
            f[8] = fa[8];
        }
    }
}

/* OpenBoundaryD2Q9_y (:542-580) */
static void open_y(orc_lattice *L, int py)
{
    const int d = (py < L->ny / 2) ? 1 : -1;
    for (int x = 0; x < L->nx; x++) {
        const int m = L->ini[x + py * L->nx], ma = L->ini[x + (py + d) * L->nx];
        if (!m || !ma) continue;
        double *f = L->f + (size_t)(m - 1) * 9;
        const double *fa = L->f + (size_t)(ma - 1) * 9;
        if (d > 0) {
            f[3] = fa[3];
            f[5] = fa[5];
            f[8] = fa[8];
        } else {
            f[4] = fa[4];
            f[6] = fa[6];
            f[7] = fa[7];
        }
    }
}

/* convective_x (:627-706): f = (f + U f_A) / (1 + U), U = the x velocity (calcula) of the inner
 * neighbour A (solid neighbours, which the reference does not test for, are skipped) */
static void convective_outlet(orc_lattice *L, int px)
{
    const int infx = (px < L->nx / 2) ? 1 : -1;
    for (int y = 0; y < L->ny; y++)
        for (int z = 0; z < L->nz; z++) {
            const int m = L->ini[px + y * L->nx + z * L->ny * L->nx];
            const int ma = L->ini[(px + infx) + y * L->nx + z * L->ny * L->nx];
            if (!m || !ma) continue;
            const double *fa = L->f + (size_t)(ma - 1) * L->q;
            double u[3], rho;
            moments(L->t, fa, u, &rho);
            const double U = u[0];
            double *f = L->f + (size_t)(m - 1) * L->q;
            const double factor = 1.0 / (1.0 + U);
            for (int i = 0; i < L->q; i++) f[i] = factor * (f[i] + U * fa[i]);
        }
}

/* devnull_rho_x (Boundary_conditions.cpp:68-141): outlet plane copied from its inner neighbour
 * and rescaled to rho; rest equilibrium w_i rho when the neighbour is solid. */
static void outlet_rescale(orc_lattice *L, int px, double rho)
{
    const int infx = (px < L->nx / 2) ? 1 : -1;
    for (int y = 0; y < L->ny; y++)
        for (int z = 0; z < L->nz; z++) {
            const int m = L->ini[px + y * L->nx + z * L->ny * L->nx];
            if (!m) continue;
            double *fp = L->f + (size_t)(m - 1) * L->q;
            const int ma = L->ini[(px + infx) + y * L->nx + z * L->ny * L->nx];
            if (ma) {
                const double *fa = L->f + (size_t)(ma - 1) * L->q;
                const double rho_adj = site_density(fa, L->q);
                const double fator = rho / rho_adj;
                for (int i = 0; i < L->q; i++) fp[i] = fa[i] * fator;
            } else {
                for (int i = 0; i < L->q; i++) fp[i] = L->t->w[i] * rho;
            }
        }
}

/* One reference step: boundary planes, then collide + push every fluid node, then swap
 * (main_stability-map_obstacle.cpp:88-118; the periodic programs skip the boundary calls).
 * Returns the running max |rho| / flags when density checking is requested. */
static void one_step(orc_lattice *L, const orc_bc *bc, int nthreads, double *max_abs_rho, int *nonfinite)
{
    if (bc && bc->inlet_x >= 0) {
        if (bc->inlet_kind == 1)
            parabolic_inlet(L, bc->inlet_x, bc->u_in, bc->parabolic_L);
        else if (L->q == 9)
            zou_he_d2q9(L, bc->inlet_x, bc->u_in);
        else
            zou_he_inlet(L, bc->inlet_x, bc->u_in);
    }
    if (bc && bc->outlet_x >= 0) {
        if (bc->outlet_kind == 1 && L->q == 9)
            open_x(L, bc->outlet_x);
        else if (bc->outlet_kind == 2)
            convective_outlet(L, bc->outlet_x);
        else
            outlet_rescale(L, bc->outlet_x, bc->rho_out);
    }
    if (bc && bc->open_y >= 0 && L->q == 9) open_y(L, bc->open_y);
    const int q = L->q;
    const tables_t *t = L->t;
    double mx = 0.0;
    int nf = 0;
    const int check = (max_abs_rho != NULL);
#pragma omp parallel for num_threads(nthreads > 0 ? nthreads : 1) reduction(max : mx) reduction(| : nf) schedule(static) if (nthreads > 1)
    for (int pto = 0; pto < L->n_fluid; pto++) {
        double *f = L->f + (size_t)pto * q;
        collide_site(t, f, L->op, L->tau, L->tau_nh);
        if (check) {
            const double dens = site_density(f, q);
            if (!isfinite(dens))
                nf = 1;
            else if (fabs(dens) > mx)
                mx = fabs(dens);
        }
        const int *dir = L->stream + (size_t)pto * q;
        for (int i = 0; i < q; i++) L->fnew[dir[i]] = f[i];
    }
    double *tmp = L->f;
    L->f = L->fnew;
    L->fnew = tmp;
    if (check) {
        if (mx > *max_abs_rho) *max_abs_rho = mx;
        *nonfinite |= nf;
    }
}

void orc_step(orc_lattice *L, int n_steps, const orc_bc *bc, int nthreads)
{
    for (int s = 0; s < n_steps; s++) one_step(L, bc, nthreads, NULL, NULL);
}

/* kinectic_energy (Other_functions.cpp:100-115): serial sum of 1/2 |u|^2 in fluid-index order.
 * stage selects the populations as in orc_get_populations. */
double orc_kinetic_energy(const orc_lattice *L, int stage)
{
    const double *F = stage ? L->fnew : L->f;
    double e = 0;
    for (int pto = 0; pto < L->n_fluid; pto++) {
        double u[3], rho;
        moments(L->t, F + (size_t)pto * L->q, u, &rho);
        e = e + 0.5 * (u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
    }
    return e;
}

/* max |rho| over fluid nodes of the chosen stage, and a non-finite flag */
double orc_max_abs_density(const orc_lattice *L, int stage, int *nonfinite)
{
    const double *F = stage ? L->fnew : L->f;
    double mx = 0.0;
    int nf = 0;
    for (int pto = 0; pto < L->n_fluid; pto++) {
        const double r = site_density(F + (size_t)pto * L->q, L->q);
        if (!isfinite(r))
            nf = 1;
        else if (fabs(r) > mx)
            mx = fabs(r);
    }
    if (nonfinite) *nonfinite = nf;
    return mx;
}

void orc_equilibrium(int q, double ux, double uy, double uz, double rho, double *feq)
{
    const double u[3] = {ux, uy, uz};
    equilibrium(tables_for(q), u, rho, feq);
}

void orc_collide_site(int q, double *f, int op, double tau, double tau_nh)
{
    collide_site(tables_for(q), f, op, tau, tau_nh);
}

/* ------------------------------------------------------------------------------------------ */
/* Program initial conditions                                                                  */
/* ------------------------------------------------------------------------------------------ */

/* Taylor-Green initial populations on a periodic L x L (x nz) box in fluid-index order.
 * variant 0: inicializa_taylor_green (main_taylor-green.cpp:57-100):
 *            u = U0 ( sin kx cos ky, -cos kx sin ky ), rho = 1 + 3/4 U0^2 (cos 2kx + cos 2ky).
 * variant 1: the same vortex translated by (L/4, L/4):
 *            u = U0 (-cos kx sin ky, sin kx cos ky), rho = 1 - 3/4 U0^2 (cos 2kx + cos 2ky),
 *            and Sxx = 2 U0 k sin kx sin ky.
 * poisson = 0 gives rho = 1; neq = 0 gives f_eq only.  For D3Q19 every z layer gets the same
 * populations (the reference's -DLATT=19 build uses nz = 1). */
void orc_init_taylor_green(int q, int L_, int nz, double u_0, double tau, int poisson, int neq, int variant,
                           double *aos)
{
    const tables_t *t = tables_for(q);
    const int d = t->dim;
    const double L = (double)L_;
    const double k = 2. * M_PI / L;
    const double cs2 = 1. / 3.;
    for (int z = 0; z < nz; z++)
        for (int y = 0; y < L_; y++)
            for (int x = 0; x < L_; x++) {
                double rho = 1.0;
                double u_x, u_y, Sxx;
                if (variant == 0) {
                    if (poisson) rho = 1.0 + 0.75 * u_0 * u_0 * (cos(4. * M_PI * x / L) + cos(4. * M_PI * y / L));
                    u_x = u_0 * sin(2. * M_PI * x / L) * cos(2. * M_PI * y / L);
                    u_y = -u_0 * cos(2. * M_PI * x / L) * sin(2. * M_PI * y / L);
                    Sxx = 2. * u_0 * k * cos(k * x) * cos(k * y);
                } else {
                    if (poisson) rho = 1.0 - 0.75 * u_0 * u_0 * (cos(4. * M_PI * x / L) + cos(4. * M_PI * y / L));
                    u_x = -u_0 * cos(2. * M_PI * x / L) * sin(2. * M_PI * y / L);
                    u_y = u_0 * sin(2. * M_PI * x / L) * cos(2. * M_PI * y / L);
                    Sxx = 2. * u_0 * k * sin(k * x) * sin(k * y);
                }
                double *f = aos + ((size_t)x + (size_t)y * L_ + (size_t)z * L_ * L_) * q;
                const double u[3] = {u_x, u_y, 0.0};
                equilibrium(t, u, rho, f);
                if (!neq) continue;
                const double Pxx = -rho * cs2 * tau * Sxx;
                const double Pyy = -Pxx;
                for (int i = 0; i < q; i++) {
                    const double cx = t->c[i * d];
                    const double cy = t->c[i * d + 1];
                    f[i] += t->w[i] / (2. * cs2 * cs2) * ((cx * cx - cs2) * Pxx + (cy * cy - cs2) * Pyy);
                }
            }
}

/* Error of a Taylor-Green field against the analytic decay, computed like
 * main_taylor-green.cpp:178-213 on the given populations (post-collision of step `step`).
 * out[0] = E_vector, out[1] = E_magnitude, out[2] = nu_ef/nu - 1. */
void orc_taylor_green_error(int q, int L_, const double *aos, double u_0, double visc, int step, int variant,
                            double *out)
{
    const tables_t *t = tables_for(q);
    const double L = (double)L_;
    const double k = 2. * M_PI / L;
    double s_mag = 0, s_vec = 0, s_r = 0, s_proj = 0, s_phi = 0;
    const double e = exp(-2. * visc * k * k * step);
    for (int y = 0; y < L_; y++)
        for (int x = 0; x < L_; x++) {
            double u[3], rho;
            moments(t, aos + ((size_t)x + (size_t)y * L_) * q, u, &rho);
            const double vx = u[0], vy = u[1], vz = u[2];
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
}

/* Whole Taylor-Green program (main_taylor-green.cpp:103-218): returns the output line's numbers.
 * tau_mode != 0 uses the given tau (--tau); otherwise Re (diffusive scaling).  u_0 <= 0 means 2/L.
 * out: [tau, tau_nh, u0, steps, E_vector, E_magnitude, nu_rel]. */
void orc_taylor_green_program(int q, int L_, int op, double tau_nh_in, double Re, double u_0, int tau_mode,
                              double tau_in, int neq, int poisson, int variant, int nthreads, double *out)
{
    if (u_0 <= 0) u_0 = 2. / L_;
    double tau, visc;
    if (tau_mode) {
        tau = tau_in;
        visc = (tau - 0.5) / 3.;
    } else {
        visc = u_0 * L_ / Re;
        tau = 0.5 + 3. * visc;
    }
    const double tau_nh = (op == ORC_OP_REG) ? 1.0 : (op == ORC_OP_BGK ? tau : tau_nh_in);
    orc_lattice *lat = orc_create(q, L_, L_, 1, NULL, tau, tau_nh, op);
    double *f0 = (double *)malloc((size_t)L_ * L_ * q * sizeof(double));
    orc_init_taylor_green(q, L_, 1, u_0, tau, poisson, neq, variant, f0);
    orc_set_populations(lat, f0);
    const double L = L_;
    const double k = 2. * M_PI / L;
    const int nT = tau_mode ? (int)round(1. / (2. * visc * k * k)) : (int)round(L / u_0);
    orc_step(lat, nT + 1, NULL, nthreads);
    orc_get_populations(lat, f0, 1);
    double err[3];
    orc_taylor_green_error(q, L_, f0, u_0, visc, nT, variant, err);
    out[0] = tau;
    out[1] = tau_nh;
    out[2] = u_0;
    out[3] = nT;
    out[4] = err[0];
    out[5] = err[1];
    out[6] = err[2];
    free(f0);
    orc_destroy(lat);
}

/* Double shear layer initial populations (main_double-shear-layer.cpp:48-66), U0 = 1/32,
 * lambda = 80, epsilon = 0.05; note the integer division ny/2 in the branch test. */
void orc_init_double_shear(int L_, double rho_ini, double *aos)
{
    const tables_t *t = tables_for(9);
    const double U_0 = 1. / 32., LAMBDA = 80., EPSILON = 0.05;
    const double L = (double)L_;
    for (int y = 0; y < L_; y++)
        for (int x = 0; x < L_; x++) {
            double u_x = U_0 * tanh(LAMBDA * ((double)y / L - 1. / 4.));
            if (y > L_ / 2) u_x = U_0 * tanh(LAMBDA * (3. / 4. - (double)y / L));
            const double u_y = EPSILON * U_0 * sin(2. * M_PI * ((double)x / L + 1. / 4.));
            const double u[3] = {u_x, u_y, 0.0};
            equilibrium(t, u, rho_ini, aos + ((size_t)x + (size_t)y * L_) * 9);
        }
}

/* ------------------------------------------------------------------------------------------ */
/* Stability-map runs                                                                          */
/* ------------------------------------------------------------------------------------------ */

/* Map axes of main_stability-map_taylor-green.cpp:134-164 */
void orc_tg_map_params(int i, int j, int n_ma, int n_nu, int op, double tau_nh_in, double *u0, double *tau,
                       double *tau_nh)
{
    const double c_s = 1. / sqrt(3.);
    const double u_min = 0.05 * c_s;
    const double log_nu_min = -5., log_nu_max = -2.;
    *u0 = u_min + (i + 1) * (c_s - u_min) / n_ma;
    const double log_nu = log_nu_min + j * (log_nu_max - log_nu_min) / n_nu;
    *tau = 3. * pow(10., log_nu) + 0.5;
    *tau_nh = (op == ORC_OP_REG) ? 1.0 : tau_nh_in;
}

/* Map axes of main_stability-map_obstacle.cpp:147-173 */
void orc_obstacle_map_params(int i, int j, int n_tau, int n_nu, double ma, double *u_imp, double *tau,
                             double *tau_nh)
{
    const double tau_nh_min = 0.5, tau_nh_max = 1.1;
    const double log_nu_min = -5., log_nu_max = -0.7;
    const double log_nu = log_nu_min + j * (log_nu_max - log_nu_min) / n_nu;
    *tau = 3. * pow(10., log_nu) + 0.5;
    *tau_nh = tau_nh_min + (double)i * (tau_nh_max - tau_nh_min) / n_tau;
    *u_imp = ma / sqrt(3.);
}

/* roda_ponto of the Taylor-Green map (main_stability-map_taylor-green.cpp:41-104) on an L x L x 1
 * D3Q19 box.  Equilibrium start with rho = 1; n_steps = (int)(100 ny / U0) unless max_steps > 0
 * caps it; the energy of the
 * post-stream populations is checked when step % 100 == 0 && step > 0.
 * Outputs: label (1 unstable), decided step (the failing check, or n_steps), and the margin
 * max over checks of E / (2 E0) (non-finite E gives +inf). */
int orc_tg_map_point(int L_, int op, double tau, double tau_nh, double u_0, int max_steps, int *decided_step,
                     double *margin)
{
    orc_lattice *lat = orc_create(19, L_, L_, 1, NULL, tau, tau_nh, op);
    const double L = (double)L_;
    const double rho_ini = 1.0;
    for (int y = 0; y < L_; y++)
        for (int x = 0; x < L_; x++) {
            const double u_x = u_0 * sin(2. * M_PI * (double)x / L) * cos(2. * M_PI * (double)y / L);
            const double u_y = -u_0 * cos(2. * M_PI * (double)x / L) * sin(2. * M_PI * (double)y / L);
            const double u[3] = {u_x, u_y, 0.0};
            equilibrium(lat->t, u, rho_ini, lat->f + (size_t)(lat->ini[x + y * L_] - 1) * 19);
        }
    int n_steps = (int)((double)(100 * L_) / u_0);
    if (max_steps > 0 && max_steps < n_steps) n_steps = max_steps;
    const double energy_ini = orc_kinetic_energy(lat, 0);
    int unstable = 0, dstep = n_steps;
    double mg = 0.0;
    for (int step = 0; step < n_steps; step++) {
        if (step % 100 == 0 && step > 0) {
            const double energy = orc_kinetic_energy(lat, 0);
            const double r = isfinite(energy) ? energy / (2. * energy_ini) : INFINITY;
            if (r > mg) mg = r;
            if (energy > 2. * energy_ini || !isfinite(energy)) {
                unstable = 1;
                dstep = step;
                break;
            }
        }
        one_step(lat, NULL, 1, NULL, NULL);
    }
    orc_destroy(lat);
    if (decided_step) *decided_step = dstep;
    if (margin) *margin = mg;
    return unstable;
}

/* Obstacle channel geometry (main_stability-map_obstacle.cpp:42-70), scaled by (sx, sy):
 * nx = 20 sx + 2 with solid end columns, ny = 12 sy, a 2 sx x 4 sy block at x in [7 sx, 9 sx - 1]
 * (for sx = 1: x = 7, 8) and y in [4 sy, 8 sy - 1].  sx = sy = 1 is the reference's channel. */
void orc_obstacle_geometry(int sx, int sy, int *nx, int *ny, uint8_t *solid)
{
    const int NX = 20 * sx + 2, NY = 12 * sy;
    *nx = NX;
    *ny = NY;
    if (!solid) return;
    for (int y = 0; y < NY; y++)
        for (int x = 0; x < NX; x++) {
            int s = 0;
            if (x == 0 || x == NX - 1) s = 1;
            if (x >= 7 * sx && x <= 9 * sx - 1 && y >= 4 * sy && y <= 8 * sy - 1) s = 1;
            solid[x + y * NX] = (uint8_t)s;
        }
}

/* roda_ponto of the obstacle map (main_stability-map_obstacle.cpp:75-123): rest equilibrium,
 * n_steps = (int)(200 ny / u_imp) unless max_steps > 0 caps it; each step applies the Zou-He
 * inlet at x = 1 and the outlet at x = nx - 2, then collides, checks |rho| > 10 rho0 or
 * non-finite on the post-collision node, and streams.  Margin = max |rho| / (10 rho0). */
int orc_obstacle_map_point(int sx, int sy, double tau, double tau_nh, double u_imp, int max_steps, int *decided_step,
                           double *margin)
{
    int nx, ny;
    orc_obstacle_geometry(sx, sy, &nx, &ny, NULL);
    uint8_t *solid = (uint8_t *)malloc((size_t)nx * ny);
    orc_obstacle_geometry(sx, sy, &nx, &ny, solid);
    orc_lattice *lat = orc_create(19, nx, ny, 1, solid, tau, tau_nh, ORC_OP_EXTREG);
    free(solid);
    const double rho_ini = 1.0;
    for (int pto = 0; pto < lat->n_fluid; pto++)
        for (int i = 0; i < 19; i++) lat->f[(size_t)pto * 19 + i] = lat->t->w[i] * rho_ini;
    int n_steps = (int)((double)(200 * ny) / u_imp);
    if (max_steps > 0 && max_steps < n_steps) n_steps = max_steps;
    orc_bc bc = {1, u_imp, nx - 2, rho_ini};
    int unstable = 0, dstep = n_steps;
    double mx = 0.0;
    int nf = 0;
    for (int step = 0; step < n_steps && !unstable; step++) {
        double smx = 0.0;
        int snf = 0;
        one_step(lat, &bc, 1, &smx, &snf);
        if (smx > mx) mx = smx;
        nf |= snf;
        if (snf || smx > 10. * rho_ini) {
            unstable = 1;
            dstep = step;
        }
    }
    orc_destroy(lat);
    if (decided_step) *decided_step = dstep;
    if (margin) *margin = nf ? INFINITY : mx / (10. * rho_ini);
    return unstable;
}

/* Map sweeps over a list of grid points, OpenMP dynamic over points like the reference
 * (main_stability-map_taylor-green.cpp:150-177, main_stability-map_obstacle.cpp:161-186). */
void orc_tg_map(int L_, int op, double tau_nh, int n_ma, int n_nu, int n_pts, const int *pi, const int *pj,
                int max_steps, int nthreads, int *labels, int *decided, double *margins)
{
#pragma omp parallel for schedule(dynamic) num_threads(nthreads > 0 ? nthreads : 1)
    for (int k = 0; k < n_pts; k++) {
        double u0, tau, tnh;
        orc_tg_map_params(pi[k], pj[k], n_ma, n_nu, op, tau_nh, &u0, &tau, &tnh);
        int ds;
        double mg;
        labels[k] = orc_tg_map_point(L_, op, tau, tnh, u0, max_steps, &ds, &mg);
        if (decided) decided[k] = ds;
        if (margins) margins[k] = mg;
    }
}

void orc_obstacle_map(int n_tau, int n_nu, double ma, int n_pts, const int *pi, const int *pj, int max_steps,
                      int nthreads, int *labels, int *decided, double *margins)
{
#pragma omp parallel for schedule(dynamic) num_threads(nthreads > 0 ? nthreads : 1)
    for (int k = 0; k < n_pts; k++) {
        double u_imp, tau, tnh;
        orc_obstacle_map_params(pi[k], pj[k], n_tau, n_nu, ma, &u_imp, &tau, &tnh);
        int ds;
        double mg;
        labels[k] = orc_obstacle_map_point(1, 1, tau, tnh, u_imp, max_steps, &ds, &mg);
        if (decided) decided[k] = ds;
        if (margins) margins[k] = mg;
    }
}

int orc_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------------------------------ */
/* Fields and VTK output (LBM_functions.cpp:3761-3872 vorticity; rec_velocity :4218,            */
/* rec_vorticity :4302, rec_density :4416; rec_velocity_bin :4979, rec_vorticity_bin :5061,     */
/* rec_density_bin :5179 with the helpers of :4795-4883), and tools/error_calculator.cpp.       */
/* ------------------------------------------------------------------------------------------ */

/* geometry.ini of a box with an optional solid mask: 0 solid, else the 1-based fluid index */
static int *box_ini(int nx, int ny, int nz, const uint8_t *solid)
{
    const long long n = (long long)nx * ny * nz;
    int *ini = (int *)malloc((size_t)n * sizeof(int));
    int k = 0;
    for (long long i = 0; i < n; i++) ini[i] = (solid && solid[i]) ? 0 : ++k;
    return ini;
}

/* calcula's velocity at every box node, 3 values per node, 0 at solid nodes */
static void box_velocity(const tables_t *t, int nx, int ny, int nz, const int *ini, const double *aos, double *v)
{
    const long long n = (long long)nx * ny * nz;
    for (long long i = 0; i < n; i++) {
        double u[3] = {0.0, 0.0, 0.0}, rho;
        if (ini[i]) moments(t, aos + (size_t)(ini[i] - 1) * t->q, u, &rho);
        v[3 * i] = u[0];
        v[3 * i + 1] = u[1];
        v[3 * i + 2] = u[2];
    }
}

void orc_field(int q, int nx, int ny, int nz, const uint8_t *solid, const double *aos, int field, double *out)
{
    const tables_t *t = tables_for(q);
    const long long n = (long long)nx * ny * nz;
    int *ini = box_ini(nx, ny, nz, solid);
    if (field == 3) {
        for (long long i = 0; i < n; i++) out[i] = ini[i] ? site_density(aos + (size_t)(ini[i] - 1) * q, q) : 0.0;
    } else if (field == 1) {
        box_velocity(t, nx, ny, nz, ini, aos, out);
    } else {
        /* vorticity (:3761-3872): central differences of the neighbours' calcula velocities with
         * periodic wrap; a solid neighbour contributes 0; solid nodes are written as 0 */
        double *v = (double *)malloc((size_t)n * 3 * sizeof(double));
        box_velocity(t, nx, ny, nz, ini, aos, v);
        for (int z = 0; z < nz; z++)
            for (int y = 0; y < ny; y++)
                for (int x = 0; x < nx; x++) {
                    const long long i = x + (long long)nx * (y + (long long)ny * z);
                    if (!ini[i]) {
                        out[3 * i] = out[3 * i + 1] = out[3 * i + 2] = 0.0;
                        continue;
                    }
                    const long long xp = (x + 1) % nx + (long long)nx * (y + (long long)ny * z);
                    const long long xm = (x - 1 + nx) % nx + (long long)nx * (y + (long long)ny * z);
                    const long long yp = x + (long long)nx * ((y + 1) % ny + (long long)ny * z);
                    const long long ym = x + (long long)nx * ((y - 1 + ny) % ny + (long long)ny * z);
                    const long long zp = x + (long long)nx * (y + (long long)ny * ((z + 1) % nz));
                    const long long zm = x + (long long)nx * (y + (long long)ny * ((z - 1 + nz) % nz));
                    const double *a = v + 3 * xp, *b = v + 3 * xm, *c = v + 3 * yp, *d = v + 3 * ym;
                    const double *e = v + 3 * zp, *g = v + 3 * zm;
                    const double dvz_y = (c[2] - d[2]) / 2.0, dvy_z = (e[1] - g[1]) / 2.0;
                    const double dvx_z = (e[0] - g[0]) / 2.0, dvz_x = (a[2] - b[2]) / 2.0;
                    const double dvy_x = (a[1] - b[1]) / 2.0, dvx_y = (c[0] - d[0]) / 2.0;
                    out[3 * i] = dvz_y - dvy_z;
                    out[3 * i + 1] = dvx_z - dvz_x;
                    out[3 * i + 2] = dvy_x - dvx_y;
                }
        free(v);
    }
    free(ini);
}

/* value in big-endian byte order, as vtk_push does on a little-endian host */
static void put_be(FILE *fp, double v, int as_double)
{
    unsigned char b[8];
    if (as_double) {
        uint64_t u;
        memcpy(&u, &v, 8);
        for (int k = 0; k < 8; k++) b[k] = (unsigned char)(u >> (56 - 8 * k));
        fwrite(b, 1, 8, fp);
    } else {
        const float f = (float)v;
        uint32_t u;
        memcpy(&u, &f, 4);
        for (int k = 0; k < 4; k++) b[k] = (unsigned char)(u >> (24 - 8 * k));
        fwrite(b, 1, 4, fp);
    }
}

int orc_write_vtk(int q, int nx, int ny, int nz, const uint8_t *solid, const double *aos, int field, int format,
                  const char *path)
{
    const long long n = (long long)nx * ny * nz;
    const int nc = field == 3 ? 1 : 3;
    double *val = (double *)malloc((size_t)n * nc * sizeof(double));
    orc_field(q, nx, ny, nz, solid, aos, field, val);
    FILE *fp = fopen(path, "wb");
    if (!fp) {
        free(val);
        return -1;
    }
    static const char *ascii_title[] = {"", "Velocidade", "Velocidade", "Densidade"};
    static const char *bin_title[] = {"", "Velocidade", "Vorticidade", "Densidade"};
    static const char *name[] = {"", "velocidade", "vorticity", "densidade"};
    fprintf(fp, "# vtk DataFile Version 2.0\n%s\n%s\nDATASET STRUCTURED_POINTS\n", format ? bin_title[field] : ascii_title[field],
            format ? "BINARY" : "ASCII");
    fprintf(fp, "DIMENSIONS %d %d %d\nASPECT_RATIO 1 1 1\nORIGIN 0 0 0\n", nx, ny, nz);
    if (format)
        fprintf(fp, "POINT_DATA %lld\n", n);
    else
        fprintf(fp, "POINT_DATA %d\n", nx * ny * nz);
    const char *type = format == 1 ? "float" : "double";
    if (field == 3)
        fprintf(fp, "SCALARS %s %s\nLOOKUP_TABLE default\n", name[field], type);
    else
        fprintf(fp, "VECTORS %s %s\n", name[field], type);
    if (format == 0) {
        /* ostream << double with the default precision: printf's %g with 6 significant digits */
        for (long long r = 0; r < (long long)ny * nz; r++) {
            for (int x = 0; x < nx; x++)
                for (int c = 0; c < nc; c++) fprintf(fp, "%g ", val[(r * nx + x) * nc + c]);
            fputc('\n', fp);
        }
    } else {
        for (long long i = 0; i < n * nc; i++) put_be(fp, val[i], format == 2);
        fputc('\n', fp);
    }
    fclose(fp);
    free(val);
    return 0;
}

/* a value written as text with `digits` significant digits and read back (ostream << / >>) */
static double text_round(double v, int digits)
{
    char buf[64];
    snprintf(buf, sizeof buf, "%.*g", digits, v);
    return strtod(buf, NULL);
}

/* tools/error_calculator.cpp:60-105: the reference field sampled at (s x, s y), s = nx_ref / nx;
 * E_vec = sqrt(sum |u_s - u_r|^2 / sum |u_r|^2), E_mod = sqrt(sum (|u_s| - |u_r|)^2 / sum |u_r|^2).
 * vel and vel_ref hold 3 values per node; text_digits > 0 first rounds every value as the tool's
 * ASCII input files carry it (rec_velocity writes 6 significant digits). */
int orc_velocity_error(int nx, int ny, const double *vel, int nx_ref, int ny_ref, const double *vel_ref,
                       int text_digits, double *e_vec, double *e_mod)
{
    if (nx_ref % nx != 0 || ny_ref % ny != 0 || nx_ref / nx != ny_ref / ny) return -1;
    const int amost = nx_ref / nx;
    double sum_dif2 = 0.0, sum_vec2 = 0.0, sum_ur2 = 0.0;
    for (int y = 0; y < ny; y++)
        for (int x = 0; x < nx; x++) {
            const size_t pc = 3 * ((size_t)x + (size_t)y * nx);
            const size_t pr = 3 * ((size_t)x * amost + (size_t)y * amost * nx_ref);
            double vx_ref = vel_ref[pr], vy_ref = vel_ref[pr + 1], vx_cal = vel[pc], vy_cal = vel[pc + 1];
            if (text_digits > 0) {
                vx_ref = text_round(vx_ref, text_digits);
                vy_ref = text_round(vy_ref, text_digits);
                vx_cal = text_round(vx_cal, text_digits);
                vy_cal = text_round(vy_cal, text_digits);
            }
            const double u_r = sqrt(vx_ref * vx_ref + vy_ref * vy_ref);
            const double u_s = sqrt(vx_cal * vx_cal + vy_cal * vy_cal);
            sum_dif2 = sum_dif2 + (u_s - u_r) * (u_s - u_r);
            sum_vec2 = sum_vec2 + (vx_cal - vx_ref) * (vx_cal - vx_ref) + (vy_cal - vy_ref) * (vy_cal - vy_ref);
            sum_ur2 = sum_ur2 + u_r * u_r;
        }
    *e_mod = sqrt(sum_dif2 / sum_ur2);
    *e_vec = sqrt(sum_vec2 / sum_ur2);
    return 0;
}

/* read_geo (LBM_functions.cpp:282-353): four header lines, "DIMENSIONS nx ny nz", five more header
 * lines, then one integer per node of the file's box, x fastest; the added layers are fluid, except
 * that with `wall` the planes x = 0 and x = nx - 1 of the widened box are solid. */
int orc_read_geo(const char *path, int pts_in, int pts_out, int wall, int *nx_out, int *ny_out, int *nz_out,
                 uint8_t *solid)
{
    FILE *fp = fopen(path, "r");
    if (!fp) return -1;
    char line[4096];
    for (int i = 0; i < 4; i++)
        if (!fgets(line, sizeof line, fp)) {
            fclose(fp);
            return -1;
        }
    int nx, ny, nz;
    if (!fgets(line, sizeof line, fp) || sscanf(line, "%*s %d %d %d", &nx, &ny, &nz) != 3) {
        fclose(fp);
        return -1;
    }
    for (int i = 0; i < 5; i++)
        if (!fgets(line, sizeof line, fp)) {
            fclose(fp);
            return -1;
        }
    nx = nx + pts_in + pts_out;
    *nx_out = nx;
    *ny_out = ny;
    *nz_out = nz;
    int poros = 0;
    for (int z = 0; z < nz; z++)
        for (int y = 0; y < ny; y++)
            for (int x = 0; x < nx; x++) {
                const long long pos = x + (long long)y * nx + (long long)z * ny * nx;
                int fluid;
                if (x >= pts_in && x < nx - pts_out) {
                    int v = 0;
                    if (fscanf(fp, "%d", &v) != 1) v = 0;
                    fluid = v != 0;
                } else if ((x == 0 || x == nx - 1) && wall) {
                    fluid = 0;
                } else {
                    fluid = 1;
                }
                poros += fluid;
                if (solid) solid[pos] = (uint8_t)!fluid;
            }
    fclose(fp);
    return poros;
}
