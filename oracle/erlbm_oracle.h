/*
 * erlbm_oracle.h -- TEST INFRASTRUCTURE, NOT THE PRODUCT.
 * C interface of the CPU oracle (erlbm_oracle.c).  Loaded by tests/, smoke() and bench.py's
 * CPU-baseline leg only.
 */
#ifndef ERLBM_ORACLE_H
#define ERLBM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* operator numbers of COLISAO (src/erlbm_common.h:42) */
#define ORC_OP_BGK 1
#define ORC_OP_MRT 2
#define ORC_OP_REG 3
#define ORC_OP_EXTREG 4

typedef struct orc_lattice orc_lattice;

typedef struct orc_bc {
    int inlet_x;     /* velocity inlet plane, -1 = none */
    double u_in;     /* imposed x velocity (the profile maximum for a parabolic inlet) */
    int outlet_x;    /* outlet plane, -1 = none */
    double rho_out;  /* density a copy-and-rescale outlet is rescaled to */
    int inlet_kind;  /* 0 Zou-He (ZouHeD3Q19_vx_x / ZouHeD2Q9_vx_x), 1 parabolic (parabolic_D3Q19_x / _D2Q9_x) */
    int parabolic_L; /* channel width of the parabolic profile */
    int outlet_kind; /* 0 devnull_rho_x, 1 OpenBoundaryD2Q9_x, 2 convective_x */
    int open_y;      /* OpenBoundaryD2Q9_y plane, -1 = none */
} orc_bc;

orc_lattice *orc_create(int q, int nx, int ny, int nz, const uint8_t *solid, double tau, double tau_nh, int op);
void orc_destroy(orc_lattice *L);
int orc_fluid_count(const orc_lattice *L);
void orc_set_params(orc_lattice *L, double tau, double tau_nh, int op);
void orc_set_populations(orc_lattice *L, const double *aos);
void orc_get_populations(const orc_lattice *L, double *aos, int stage);
void orc_step(orc_lattice *L, int n_steps, const orc_bc *bc, int nthreads);
double orc_kinetic_energy(const orc_lattice *L, int stage);
double orc_max_abs_density(const orc_lattice *L, int stage, int *nonfinite);
void orc_equilibrium(int q, double ux, double uy, double uz, double rho, double *feq);
void orc_collide_site(int q, double *f, int op, double tau, double tau_nh);

void orc_init_taylor_green(int q, int L, int nz, double u_0, double tau, int poisson, int neq, int variant,
                           double *aos);
void orc_taylor_green_error(int q, int L, const double *aos, double u_0, double visc, int step, int variant,
                            double *out);
void orc_taylor_green_program(int q, int L, int op, double tau_nh, double Re, double u_0, int tau_mode,
                              double tau_in, int neq, int poisson, int variant, int nthreads, double *out);
void orc_init_double_shear(int L, double rho_ini, double *aos);

void orc_tg_map_params(int i, int j, int n_ma, int n_nu, int op, double tau_nh_in, double *u0, double *tau,
                       double *tau_nh);
void orc_obstacle_map_params(int i, int j, int n_tau, int n_nu, double ma, double *u_imp, double *tau,
                             double *tau_nh);
int orc_tg_map_point(int L, int op, double tau, double tau_nh, double u_0, int max_steps, int *decided_step,
                     double *margin);
void orc_obstacle_geometry(int sx, int sy, int *nx, int *ny, uint8_t *solid);
int orc_obstacle_map_point(int sx, int sy, double tau, double tau_nh, double u_imp, int max_steps,
                           int *decided_step, double *margin);
void orc_tg_map(int L, int op, double tau_nh, int n_ma, int n_nu, int n_pts, const int *pi, const int *pj,
                int max_steps, int nthreads, int *labels, int *decided, double *margins);
void orc_obstacle_map(int n_tau, int n_nu, double ma, int n_pts, const int *pi, const int *pj, int max_steps,
                      int nthreads, int *labels, int *decided, double *margins);
int orc_max_threads(void);

/* Fields, VTK files and the error calculator (LBM_functions.cpp rec_* writers and vorticity,
 * tools/error_calculator.cpp).  field: 1 velocity, 2 vorticity (3 values per node), 3 density;
 * format: 0 ASCII, 1 binary float, 2 binary double. */
void orc_field(int q, int nx, int ny, int nz, const uint8_t *solid, const double *aos, int field, double *out);
int orc_write_vtk(int q, int nx, int ny, int nz, const uint8_t *solid, const double *aos, int field, int format,
                  const char *path);
/* read_geo (LBM_functions.cpp:282-353): the solid mask (1 = solid) of a legacy ASCII VTK geometry
 * file (nonzero = fluid) with pts_in / pts_out layers added in x; with `wall` the first and last x
 * planes of the added layers are solid.  solid may be NULL to read the dimensions only; returns the
 * fluid count, -1 if the file cannot be read. */
int orc_read_geo(const char *path, int pts_in, int pts_out, int wall, int *nx, int *ny, int *nz, uint8_t *solid);
int orc_velocity_error(int nx, int ny, const double *vel, int nx_ref, int ny_ref, const double *vel_ref,
                       int text_digits, double *e_vec, double *e_mod);

/* fp32_shifted.c: the engine's own FP32-shifted periodic update restated on the CPU (the checker of
 * the GPU FP32 kernels' bits): n_steps steps from the AoS populations f_in (post-stream), the first
 * colliding in place; f_out = the post-collision populations.  Returns 0, or -1 / -2 on bad arguments
 * (MRT is D2Q9 only) / allocation failure. */
int orc32_periodic_d2q9(int nx, int ny, int op, double tau, double tau_nh, const double *f_in, int n_steps,
                        double *f_out);
int orc32_periodic_d3q19(int nx, int ny, int nz, int op, double tau, double tau_nh, const double *f_in,
                         int n_steps, double *f_out);
/* the same with a solid mask (nx * ny * nz bytes, NULL = none; halfway bounce-back at solid nodes):
 * f_in and f_out hold every node of the box, solid nodes included (left as given) */
int orc32_periodic_solid(int q, int nx, int ny, int nz, const uint8_t *solid, int op, double tau, double tau_nh,
                         const double *f_in, int n_steps, double *f_out);
/* the same with boundary planes (-1 = none): a Zou-He velocity inlet u_in at inlet_x; an outlet at
 * outlet_x of kind 0 (devnull_rho_x to rho_out), 1 (OpenBoundaryD2Q9_x) or 2 (convective_x); the
 * open y plane open_y of D2Q9 (OpenBoundaryD2Q9_y) */
int orc32_channel(int q, int nx, int ny, int nz, const uint8_t *solid, int op, double tau, double tau_nh,
                  int inlet_x, double u_in, int outlet_x, int outlet_kind, double rho_out, int open_y,
                  const double *f_in, int n_steps, double *f_out);
int orc32_channel_ex(int q, int nx, int ny, int nz, const uint8_t *solid, int op, double tau, double tau_nh,
                     int inlet_x, double u_in, int inlet_kind, int parabolic_L, int outlet_x, int outlet_kind,
                     double rho_out, int open_y, const double *f_in, int n_steps, double *f_out);

/* one run of the engine's batched FP32 map kernel restated (fp32_shifted.c): a block of `block` threads
 * with npt nodes each; init 0 = rest state w rho0, 1 = the Taylor-Green map equilibrium with amplitude u0
 * (u0 is also the Zou-He inlet velocity); out4 = label, decided step, steps done, status; out2 = margin,
 * energy */
int orc32_batch_run(int q, int nx, int ny, const uint8_t *solid, int inlet_x, int outlet_x, double rho0,
                    int energy_every, double energy_factor, int density_check, double density_limit, int init,
                    int op, double tau, double tau_nh, double u0, int n_steps, int block, int npt, int *out4,
                    double *out2);

/* the compensated FP32 form (float-pair populations, fp32_shifted.c) on a periodic D2Q9 box: the same
 * contract as orc32_periodic_d2q9; BGK, RLBM and E-RLBM */
int orc32p_periodic_d2q9(int nx, int ny, int op, double tau, double tau_nh, const double *f_in, int n_steps,
                         double *f_out);

#ifdef __cplusplus
}
#endif
#endif
