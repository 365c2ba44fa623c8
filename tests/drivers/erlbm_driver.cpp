// erlbm_driver.cpp -- a compiled C++ caller of liberlbm_gb300.so through include/erlbm_gb300.h, written
// as the reference's programs would call it in place of their node loops.
//
//   obstacle <i> <j>      roda_ponto of main_stability-map_obstacle.cpp:75-123 for map point (i, j) of the
//                         400 x 400 grid: rest equilibrium, then per step the boundary planes, the
//                         collision and the density check of every node, and the stream, until the step
//                         budget (int)(200 ny / u_imp) or the first unstable step.  Here each step is
//                         erlbm_step(1) (Zou-He inlet, density outlet) followed by
//                         erlbm_max_abs_density of the post-collision populations.
//   dsl <L> <interval> <n> the double shear layer loop of main_double-shear-layer.cpp:162-230 in FP64:
//                         initial_double_shear_layer, then n intervals of `interval` steps, each followed
//                         by kinectic_energy of the post-collision populations.
// Output: one JSON object per line.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "erlbm_gb300.h"

static int fail(const char *what, int rc)
{
    std::fprintf(stderr, "%s failed: %d (%s) %s\n", what, rc, erlbm_strerror(rc), erlbm_last_error());
    return 1;
}

static int obstacle(int i, int j)
{
    double u_imp = 0, tau = 0, tau_nh = 0;
    int rc = erlbm_obstacle_map_params(i, j, 400, 400, 0.1, &u_imp, &tau, &tau_nh);
    if (rc) return fail("erlbm_obstacle_map_params", rc);
    int nx = 0, ny = 0;
    if ((rc = erlbm_obstacle_geometry(1, 1, &nx, &ny, nullptr))) return fail("erlbm_obstacle_geometry", rc);
    std::vector<uint8_t> solid((size_t)nx * ny);
    if ((rc = erlbm_obstacle_geometry(1, 1, &nx, &ny, solid.data()))) return fail("erlbm_obstacle_geometry", rc);
    const erlbm_desc d = {19, nx, ny, 1, solid.data(), tau, tau_nh, ERLBM_OP_EXTREG, ERLBM_FP64};
    erlbm_handle *h = nullptr;
    if ((rc = erlbm_create(&d, &h))) return fail("erlbm_create", rc);
    int64_t n_fluid = 0;
    erlbm_fluid_count(h, &n_fluid);
    // dist_eq(0, 0, 0, rho_ini) at every fluid node
    const double rho_ini = 1.0;
    double feq[19];
    erlbm_equilibrium(19, 0., 0., 0., rho_ini, feq);
    std::vector<double> f((size_t)n_fluid * 19);
    for (int64_t p = 0; p < n_fluid; p++) std::memcpy(&f[(size_t)p * 19], feq, sizeof(feq));
    if ((rc = erlbm_set_populations(h, f.data(), f.size()))) return fail("erlbm_set_populations", rc);
    const int n_steps = (int)((double)(200 * ny) / u_imp);
    erlbm_bc bc;
    std::memset(&bc, 0, sizeof(bc));
    bc.inlet_x = 1;          // ZouHeD3Q19_vx_x(1, u_imp, ...)
    bc.u_in = u_imp;
    bc.outlet_x = nx - 2;    // devnull_rho_x(nx - 2, rho_ini, ...)
    bc.rho_out = rho_ini;
    int instavel = 0, step = 0;
    for (; step < n_steps && !instavel; step++) {
        if ((rc = erlbm_step(h, 1, &bc))) return fail("erlbm_step", rc);
        double max_rho = 0;
        int nonfinite = 0;
        if ((rc = erlbm_max_abs_density(h, ERLBM_STAGE_POST_COLLISION, &max_rho, &nonfinite)))
            return fail("erlbm_max_abs_density", rc);
        if (max_rho > 10. * rho_ini || nonfinite) instavel = 1;
    }
    erlbm_destroy(h);
    std::printf("{\"program\": \"obstacle\", \"i\": %d, \"j\": %d, \"label\": %d, \"steps\": %d, \"n_steps\": %d}\n", i,
                j, instavel, step, n_steps);
    return 0;
}

static int dsl(int L, int interval, int n)
{
    const double tau = 0.5 + 3.0 * (1.0 / 32.0) * L / 80000.0;  // main_double-shear-layer.cpp: Re = 80000
    const erlbm_desc d = {9, L, L, 1, nullptr, tau, 0.65, ERLBM_OP_EXTREG, ERLBM_FP64};
    erlbm_handle *h = nullptr;
    int rc = erlbm_create(&d, &h);
    if (rc) return fail("erlbm_create", rc);
    std::vector<double> f((size_t)L * L * 9);
    if ((rc = erlbm_init_double_shear(L, 1.0, f.data()))) return fail("erlbm_init_double_shear", rc);
    if ((rc = erlbm_set_populations(h, f.data(), f.size()))) return fail("erlbm_set_populations", rc);
    for (int k = 1; k <= n; k++) {
        if ((rc = erlbm_step(h, interval, nullptr))) return fail("erlbm_step", rc);
        double e = 0;
        if ((rc = erlbm_kinetic_energy(h, ERLBM_STAGE_POST_COLLISION, &e))) return fail("erlbm_kinetic_energy", rc);
        std::printf("{\"program\": \"dsl\", \"L\": %d, \"step\": %d, \"energy\": %.17g}\n", L, k * interval, e);
    }
    erlbm_destroy(h);
    return 0;
}

int main(int argc, char **argv)
{
    if (argc >= 4 && !std::strcmp(argv[1], "obstacle")) return obstacle(std::atoi(argv[2]), std::atoi(argv[3]));
    if (argc >= 5 && !std::strcmp(argv[1], "dsl")) return dsl(std::atoi(argv[2]), std::atoi(argv[3]), std::atoi(argv[4]));
    std::fprintf(stderr, "usage: %s obstacle <i> <j> | dsl <L> <interval> <n>\n", argv[0]);
    return 2;
}
