// ref_harness.cpp -- TEST INFRASTRUCTURE, NOT THE PRODUCT.
//
// Compiles the reference's own SimBoltz library and program functions, from their sources where
// they lie (the reference tree is passed with -I by oracle/Makefile; nothing is copied), into a
// shared library with a small C interface.  It is built only where the reference tree exists and
// is used to (1) check the C oracle bit for bit and (2) generate the golden vectors in
// tests/golden/ (tests/golden/make_golden.py).  REF_Q selects the lattice, because the reference
// fixes it with the nvel/dim macros (src/erlbm_common.h:3-6).
//
// The program files are included with their main() renamed, so that their own helper functions
// (inicializa_taylor_green, initial_double_shear_layer, both roda_ponto, geometria_obstaculo) are
// the ones exercised.

#if REF_Q == 9
#define main erlbm_ref_main_taylor_green
#include "main_taylor-green.cpp"
#undef main
#define main erlbm_ref_main_double_shear
#include "main_double-shear-layer.cpp"
#undef main
#define REF_PREFIX(name) ref9_##name
#elif REF_Q == 19
#define main erlbm_ref_main_tg_map
#include "main_stability-map_taylor-green.cpp"
#undef main
#define main erlbm_ref_main_obstacle_map
#include "main_stability-map_obstacle.cpp"
#undef main
#define REF_PREFIX(name) ref19_##name
#else
#error "REF_Q must be 9 or 19"
#endif

#include <cstdint>

namespace {

struct RefCase {
    GEOMETRY geometry;
    LATTICE lattice;
};

// Geometry like geometria_periodica / numera_fluido (src/erlbm_common.h:89-114), but with an
// optional solid mask (1 = solid), x fastest.
void make_case(RefCase &c, int nx, int ny, int nz, const uint8_t *solid)
{
    c.geometry.file = "";
    c.geometry.ftesc = 1.0;
    c.geometry.nx = nx;
    c.geometry.ny = ny;
    c.geometry.nz = nz;
    c.geometry.ini = new int[(size_t)nx * ny * nz];
    for (int i = 0; i < nx * ny * nz; i++) c.geometry.ini[i] = (solid && solid[i]) ? 0 : 1;
    numera_fluido(c.geometry);
    define_rede(c.geometry, c.lattice);
    aloca_populacoes(c.geometry, c.lattice);
}

void free_case(RefCase &c)
{
    libera_populacoes(c.lattice);
    delete[] c.lattice.c_i;
    delete[] c.lattice.Q_i;
    delete[] c.lattice.ini_stream;
    delete[] c.geometry.ini;
}

}  // namespace

extern "C" {

int REF_PREFIX(q)(void) { return nvel; }

// Runs n_steps steps of a driver loop built from the library calls: boundary planes
// (ZouHeD3Q19_vx_x / devnull_rho_x, D3Q19 only), colisao_sitio and propag_site at every fluid
// node, pointer swap.  f_in: post-stream AoS populations (n_fluid * nvel).  Outputs (nullable):
// post-stream populations after the last step, post-collision populations of the last step, and
// the kinetic energy (kinectic_energy) of the post-stream populations.
int REF_PREFIX(run_threads)(int nx, int ny, int nz, const uint8_t *solid, int col, double tau, double tau_nh,
                            const double *f_in, int n_steps, int inlet_x, double u_in, int outlet_x, double rho_out,
                            double *f_post_stream, double *f_post_collision, double *energy, int threads);

int REF_PREFIX(run)(int nx, int ny, int nz, const uint8_t *solid, int col, double tau, double tau_nh,
                    const double *f_in, int n_steps, int inlet_x, double u_in, int outlet_x, double rho_out,
                    double *f_post_stream, double *f_post_collision, double *energy)
{
    return REF_PREFIX(run_threads)(nx, ny, nz, solid, col, tau, tau_nh, f_in, n_steps, inlet_x, u_in, outlet_x,
                                   rho_out, f_post_stream, f_post_collision, energy, 1);
}

// threads > 1: the node loop runs under "omp parallel for", as in main_double-shear-layer.cpp:389
int REF_PREFIX(run_threads)(int nx, int ny, int nz, const uint8_t *solid, int col, double tau, double tau_nh,
                            const double *f_in, int n_steps, int inlet_x, double u_in, int outlet_x, double rho_out,
                            double *f_post_stream, double *f_post_collision, double *energy, int threads)
{
    RefCase c;
    make_case(c, nx, ny, nz, solid);
    const int n = c.geometry.fluid * nvel;
    for (int k = 0; k < n; k++) c.lattice.inif[k] = f_in[k];
    for (int k = 0; k < n; k++) c.lattice.inif_new[k] = 0.0;
    PARAMETERS p;
    p.tau = tau;
    p.tau_nh = tau_nh;
    p.visc = (tau - 0.5) / 3.;
    p.rho_ini = 1.0;
    for (int step = 0; step < n_steps; step++) {
#if REF_Q == 19
        if (inlet_x >= 0) ZouHeD3Q19_vx_x(inlet_x, u_in, c.geometry, c.lattice);
#endif
        if (outlet_x >= 0) devnull_rho_x(outlet_x, rho_out, c.geometry, c.lattice);
#pragma omp parallel for num_threads(threads > 1 ? threads : 1) if (threads > 1)
        for (int pto = 0; pto < c.geometry.fluid; pto++) {
            double *f = c.lattice.inif + pto * nvel;
            colisao_sitio(f, 0., 0., 0., c.lattice, p, col);
            double mx, my, mz;
            propag_site(c.lattice, pto, mx, my, mz);
        }
        double *t = c.lattice.inif;
        c.lattice.inif = c.lattice.inif_new;
        c.lattice.inif_new = t;
    }
    if (f_post_stream)
        for (int k = 0; k < n; k++) f_post_stream[k] = c.lattice.inif[k];
    if (f_post_collision)
        for (int k = 0; k < n; k++) f_post_collision[k] = c.lattice.inif_new[k];
    if (energy) *energy = kinectic_energy(c.geometry, c.lattice);
    const int nf = c.geometry.fluid;
    free_case(c);
    return nf;
}

#if REF_Q == 9
// inicializa_taylor_green (main_taylor-green.cpp:57-100) on a periodic L x L box.
void ref9_init_taylor_green(int L, double u_0, double tau, int poisson, int neq, double *f_out)
{
    RefCase c;
    make_case(c, L, L, 1, nullptr);
    inicializa_taylor_green(c.geometry, c.lattice, u_0, tau, poisson != 0, neq != 0);
    for (int k = 0; k < L * L * nvel; k++) f_out[k] = c.lattice.inif[k];
    free_case(c);
}

// initial_double_shear_layer (main_double-shear-layer.cpp:48-66).
void ref9_init_double_shear(int L, double rho_ini, double *f_out)
{
    RefCase c;
    make_case(c, L, L, 1, nullptr);
    initial_double_shear_layer(c.geometry, c.lattice, (double)L, rho_ini);
    for (int k = 0; k < L * L * nvel; k++) f_out[k] = c.lattice.inif[k];
    free_case(c);
}

// The Taylor-Green program's measurement (main_taylor-green.cpp:103-218) by calling its main()
// with the given command line; the program prints its one output line to stdout.
int ref9_taylor_green_main(int argc, char **argv) { return erlbm_ref_main_taylor_green(argc, argv); }
#endif

// A driver loop with the channel boundaries of the library (Boundary_conditions.cpp), called before
// the node loop in this order: inlet (bci[1] = 0: ZouHeD3Q19_vx_x or ZouHeD2Q9_vx_x; 1: parabolic_D3Q19_x
// or parabolic_D2Q9_x with width bci[2]), outlet (bci[4] = 0: devnull_rho_x; 1: OpenBoundaryD2Q9_x;
// 2: convective_x), then OpenBoundaryD2Q9_y.  bci = {inlet_x, inlet_kind, L, outlet_x, outlet_kind,
// open_y} (-1 = none), bcd = {u_in, rho_out}.  Outputs as in run().
int REF_PREFIX(run_bc)(int nx, int ny, int nz, const uint8_t *solid, int col, double tau, double tau_nh,
                       const double *f_in, int n_steps, const int *bci, const double *bcd, double *f_post_stream,
                       double *f_post_collision)
{
    RefCase c;
    make_case(c, nx, ny, nz, solid);
    const int n = c.geometry.fluid * nvel;
    for (int k = 0; k < n; k++) c.lattice.inif[k] = f_in[k];
    for (int k = 0; k < n; k++) c.lattice.inif_new[k] = 0.0;
    PARAMETERS p;
    p.tau = tau;
    p.tau_nh = tau_nh;
    p.visc = (tau - 0.5) / 3.;
    p.rho_ini = 1.0;
    for (int step = 0; step < n_steps; step++) {
        if (bci[0] >= 0) {
#if REF_Q == 19
            if (bci[1] == 1) parabolic_D3Q19_x(bci[0], bcd[0], bci[2], c.geometry, c.lattice);
            else ZouHeD3Q19_vx_x(bci[0], bcd[0], c.geometry, c.lattice);
#else
            if (bci[1] == 1) parabolic_D2Q9_x(bci[0], bcd[0], bci[2], c.geometry, c.lattice);
            else ZouHeD2Q9_vx_x(bci[0], bcd[0], c.geometry, c.lattice);
#endif
        }
        if (bci[3] >= 0) {
            if (bci[4] == 2) convective_x(bci[3], c.geometry, c.lattice);
#if REF_Q == 9
            else if (bci[4] == 1) OpenBoundaryD2Q9_x(bci[3], c.geometry, c.lattice);
#endif
            else devnull_rho_x(bci[3], bcd[1], c.geometry, c.lattice);
        }
#if REF_Q == 9
        if (bci[5] >= 0) OpenBoundaryD2Q9_y(bci[5], c.geometry, c.lattice);
#endif
        for (int pto = 0; pto < c.geometry.fluid; pto++) {
            double *f = c.lattice.inif + pto * nvel;
            colisao_sitio(f, 0., 0., 0., c.lattice, p, col);
            double mx, my, mz;
            propag_site(c.lattice, pto, mx, my, mz);
        }
        double *t = c.lattice.inif;
        c.lattice.inif = c.lattice.inif_new;
        c.lattice.inif_new = t;
    }
    if (f_post_stream)
        for (int k = 0; k < n; k++) f_post_stream[k] = c.lattice.inif[k];
    if (f_post_collision)
        for (int k = 0; k < n; k++) f_post_collision[k] = c.lattice.inif_new[k];
    free_case(c);
    return 0;
}

// read_geo (LBM_functions.cpp:282-353, the overload with the wall flag): geometry.ini of a legacy
// VTK geometry file with pts_in / pts_out layers added in x.  meio must hold (nx + pts_in + pts_out)
// * ny * nz ints; returns the number of fluid nodes.
int REF_PREFIX(read_geo)(const char *path, int pts_in, int pts_out, int wall, int *meio)
{
    return read_geo(std::string(path), meio, pts_in, pts_out, wall != 0);
}

// The reference's field writers (LBM_functions.cpp: rec_velocity :4218, rec_vorticity :4302,
// rec_density :4416 in ASCII; rec_velocity_bin :4979, rec_vorticity_bin :5061, rec_density_bin
// :5179 in big-endian binary) on the given AoS populations.  field: 1 velocity, 2 vorticity,
// 3 density; format: 0 ASCII, 1 binary float, 2 binary double.  The file is written into the current
// directory under the reference's own name (vel_<tempo>.vtk, vor_<passo>.vtk, rho_<passo>.vtk).
int REF_PREFIX(rec_field)(int nx, int ny, int nz, const uint8_t *solid, const double *f_aos, int field, int format,
                          double tempo, unsigned passo)
{
    RefCase c;
    make_case(c, nx, ny, nz, solid);
    const int n = c.geometry.fluid * nvel;
    for (int k = 0; k < n; k++) c.lattice.inif[k] = f_aos[k];
    const bool dp = format == 2;
    if (field == 1) {
        if (format == 0) rec_velocity(c.geometry, c.lattice, tempo);
        else rec_velocity_bin(c.geometry, c.lattice, tempo, dp);
    } else if (field == 2) {
        if (format == 0) rec_vorticity(c.geometry, c.lattice, passo);
        else rec_vorticity_bin(c.geometry, c.lattice, passo, dp);
    } else {
        if (format == 0) rec_density(c.geometry, c.lattice, passo);
        else rec_density_bin(c.geometry, c.lattice, passo, dp);
    }
    free_case(c);
    return 0;
}

#if REF_Q == 19
// roda_ponto of the Taylor-Green map (main_stability-map_taylor-green.cpp:41-104).
int ref19_tg_map_point(int L, int col, double tau, double tau_nh, double u_0)
{
    GEOMETRY geometry;
    geometria_periodica(geometry, L, L, 1);
    LATTICE lattice;
    define_rede(geometry, lattice);
    PARAMETERS p;
    p.tau = tau;
    p.visc = (tau - 0.5) / 3.;
    p.tau_nh = tau_nh;
    p.rho_ini = 1.0;
    const int r = roda_ponto(geometry, lattice, p, col, u_0);
    delete[] lattice.c_i;
    delete[] lattice.Q_i;
    delete[] lattice.ini_stream;
    delete[] geometry.ini;
    return r;
}

// roda_ponto of the obstacle map (main_stability-map_obstacle.cpp:75-123) on geometria_obstaculo.
int ref19_obstacle_map_point(double tau, double tau_nh, double u_imp)
{
    GEOMETRY geometry;
    geometria_obstaculo(geometry);
    LATTICE lattice;
    define_rede(geometry, lattice);
    PARAMETERS p;
    p.tau = tau;
    p.visc = (tau - 0.5) / 3.;
    p.tau_nh = tau_nh;
    p.rho_ini = 1.0;
    const int r = roda_ponto(geometry, lattice, p, u_imp);
    delete[] lattice.c_i;
    delete[] lattice.Q_i;
    delete[] lattice.ini_stream;
    delete[] geometry.ini;
    return r;
}
#endif

}  // extern "C"
