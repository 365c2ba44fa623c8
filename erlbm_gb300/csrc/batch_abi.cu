// batch_abi.cu -- C ABI of the batched runs and stability maps (include/erlbm_gb300.h).
//
// erlbm_batch_run: any set of independent small runs on one geometry in one persistent launch.
// erlbm_map_run:   the reference's two stability maps (main_stability-map_taylor-green.cpp,
//                  main_stability-map_obstacle.cpp) built on it, with the reference's map axes.
// The launch sequence (counter reset, persistent kernel, result copy) is captured once into a
// CUDA graph and replayed.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/erlbm_gb300.h"
#include "abi_internal.h"
#include "batch_kernels.cuh"
#include "kernels_api.h"

using namespace erlbm;

namespace {

#define CK(call)                                              \
    do {                                                      \
        cudaError_t e_ = (call);                              \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call);   \
    } while (0)

static_assert(sizeof(BatchResult) == sizeof(erlbm_batch_result), "result layouts differ");

int sm_count()
{
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
}

// Device buffers of one call; freed on every exit path.
struct Scratch {
    std::vector<void *> p;
    ~Scratch()
    {
        for (void *q : p) cudaFree(q);
    }
    template <class T>
    cudaError_t alloc(T **out, size_t bytes)
    {
        void *q = nullptr;
        cudaError_t e = cudaMalloc(&q, bytes ? bytes : 16);
        if (e == cudaSuccess) {
            p.push_back(q);
            *out = (T *)q;
        }
        return e;
    }
};

}  // namespace

namespace erlbm {

int pick_shape(int prec, int q, int nb, int slots, int n_runs, LaunchShape *out)
{
    static const int NPT_64[] = {1, 2, 4};
    // FP32 prefers two nodes per thread (more independent work per thread; D2Q9 pairs also collide in
    // packed FP32x2 instructions): Taylor-Green map on GB300 42.2 k runs/s against 33.9 k with one
    // node per thread
    static const int NPT_32[] = {2, 1, 4, 8};
    const int *list = prec == ERLBM_FP64 ? NPT_64 : NPT_32;
    const int nl = prec == ERLBM_FP64 ? 3 : 4;
    for (int k = 0; k < nl; k++) {
        const int npt = list[k];
        if (q == 19 && npt > (prec == ERLBM_FP64 ? 2 : 4)) continue;
        int block = ((nb + npt - 1) / npt + 31) / 32 * 32;
        if (block < 32) block = 32;
        if (block > (npt == 1 ? 288 : 512)) continue;
        // two population buffers (one barrier per step) when they fit, else one
        for (int dbl = 1; dbl >= 0; dbl--) {
            const size_t smem = batch_smem(prec, q, nb, block, dbl);
            const int occ = batch_occupancy(prec, q, npt, block, smem);
            if (occ <= 0) continue;
            const int per_sm = slots > 0 ? std::min(slots, occ) : occ;
            out->npt = npt;
            out->block = block;
            out->smem = smem;
            out->dbl = dbl;
            out->grid = std::max(1, std::min(n_runs, per_sm * sm_count()));
            return ERLBM_OK;
        }
    }
    set_error("lattice of %s nodes does not fit one CTA's shared memory%s", std::to_string(nb).c_str(), "");
    return ERLBM_E_UNSUPPORTED;
}

int check_desc(const erlbm_batch_desc *d)
{
    if (!d) return ERLBM_E_INVAL;
    if ((d->q != 9 && d->q != 19) || d->nx < 1 || d->ny < 1 || (long long)d->nx * d->ny > 4096) {
        set_error("batched lattices are D2Q9 or D3Q19 with nx * ny <= 4096 nodes%s%s", "", "");
        return ERLBM_E_INVAL;
    }
    if (d->precision != ERLBM_FP64 && d->precision != ERLBM_FP32_SHIFTED) return ERLBM_E_INVAL;
    if (d->inlet_x >= d->nx || d->outlet_x >= d->nx) return ERLBM_E_INVAL;
    if (d->inlet_x >= 0 && d->q != 19) {
        set_error("the Zou-He inlet is a D3Q19 boundary%s%s", "", "");
        return ERLBM_E_UNSUPPORTED;
    }
    if (d->outlet_x >= 0) {
        const int nb = d->outlet_x + (d->outlet_x < d->nx / 2 ? 1 : -1);
        if (nb < 0 || nb >= d->nx) return ERLBM_E_INVAL;
    }
    if (d->init != ERLBM_INIT_REST && d->init != ERLBM_INIT_TG_MAP && d->init != ERLBM_INIT_AOS) return ERLBM_E_INVAL;
    return ERLBM_OK;
}

// Shared by erlbm_batch_run and the server: run a prepared batch on `stream` (synchronous).
int run_batch(const erlbm_batch_desc *d, int n_runs, const erlbm_run_spec *runs, const double *aos, size_t n_aos,
              erlbm_batch_result *out, cudaStream_t stream)
{
    int rc = check_desc(d);
    if (rc) return rc;
    if (n_runs < 0 || (n_runs > 0 && (!runs || !out))) return ERLBM_E_INVAL;
    if (n_runs == 0) return ERLBM_OK;
    const int nb = d->nx * d->ny;
    std::vector<BatchRun> hr(n_runs);
    std::vector<int> order(n_runs);
    std::iota(order.begin(), order.end(), 0);
    // longest budgets first: the persistent slots then finish together
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return runs[a].n_steps > runs[b].n_steps; });
    long long n_fluid = nb;
    if (d->solid) {
        n_fluid = 0;
        for (int k = 0; k < nb; k++) n_fluid += !d->solid[k];
    }
    for (int k = 0; k < n_runs; k++) {
        const erlbm_run_spec &s = runs[order[k]];
        if (s.op != ERLBM_OP_BGK && s.op != ERLBM_OP_REG && s.op != ERLBM_OP_EXTREG &&
            !(s.op == ERLBM_OP_MRT && d->q == 9)) {
            set_error("run %s: unknown collision operator, or MRT on D3Q19%s", std::to_string(order[k]).c_str(), "");
            return s.op == ERLBM_OP_MRT ? ERLBM_E_UNSUPPORTED : ERLBM_E_INVAL;
        }
        if (!(s.tau > 0) || !std::isfinite(s.tau) || !std::isfinite(s.tau_nh) || s.tau_nh == 0 || s.n_steps < 0)
            return ERLBM_E_INVAL;
        if (d->init == ERLBM_INIT_AOS &&
            (!aos || s.aos_offset < 0 || (size_t)s.aos_offset + (size_t)n_fluid * d->q > n_aos)) {
            set_error("run %s: initial populations outside the given array%s", std::to_string(order[k]).c_str(), "");
            return ERLBM_E_INVAL;
        }
        BatchRun &r = hr[k];
        memset(&r, 0, sizeof(r));
        r.R = make_relax(s.tau, s.tau_nh, s.op);
        r.k = shifted::make_coef(r.R);
        r.u0 = s.u0;
        r.aos_off = s.aos_offset;
        r.n_steps = s.n_steps;
        r.op = s.op;
        r.out = order[k];
    }
    LaunchShape sh;
    if ((rc = pick_shape(d->precision, d->q, nb, d->slots, n_runs, &sh))) return rc;

    Scratch m;
    BatchRun *d_runs;
    BatchResult *d_res;
    int *d_counter;
    double *d_tab = nullptr, *d_aos = nullptr;
    uint8_t *d_solid = nullptr;
    CK(m.alloc(&d_runs, hr.size() * sizeof(BatchRun)));
    CK(m.alloc(&d_res, (size_t)n_runs * sizeof(BatchResult)));
    CK(m.alloc(&d_counter, sizeof(int)));
    CK(cudaMemcpyAsync(d_runs, hr.data(), hr.size() * sizeof(BatchRun), cudaMemcpyHostToDevice, stream));
    BatchGeo g;
    memset(&g, 0, sizeof(g));
    g.nx = d->nx;
    g.ny = d->ny;
    g.nb = nb;
    g.inlet_x = d->inlet_x;
    g.outlet_x = d->outlet_x;
    g.rho0 = d->rho0;
    g.energy_every = d->energy_every;
    g.energy_factor = d->energy_factor;
    g.density_check = d->density_check;
    g.density_limit = d->density_limit;
    g.init = d->init;
    density_bounds(g);
    std::vector<double> tab;
    if (d->init == ERLBM_INIT_TG_MAP) {
        // sin(2 pi x / L) and cos(2 pi x / L) as main_stability-map_taylor-green.cpp:55-57 evaluates them
        const int n = std::max(d->nx, d->ny);
        const double L = (double)d->nx;
        tab.resize(2 * n);
        for (int x = 0; x < n; x++) {
            tab[x] = sin(2. * M_PI * (double)x / L);
            tab[n + x] = cos(2. * M_PI * (double)x / L);
        }
        CK(m.alloc(&d_tab, tab.size() * sizeof(double)));
        CK(cudaMemcpyAsync(d_tab, tab.data(), tab.size() * sizeof(double), cudaMemcpyHostToDevice, stream));
        g.sinx = d_tab;
        g.cosx = d_tab + n;
    }
    if (d->solid) {
        CK(m.alloc(&d_solid, nb));
        CK(cudaMemcpyAsync(d_solid, d->solid, nb, cudaMemcpyHostToDevice, stream));
        g.solid = d_solid;
    }
    if (d->init == ERLBM_INIT_AOS) {
        CK(m.alloc(&d_aos, n_aos * sizeof(double)));
        CK(cudaMemcpyAsync(d_aos, aos, n_aos * sizeof(double), cudaMemcpyHostToDevice, stream));
    }
    // counter reset + persistent kernel, captured into a CUDA graph and launched as one unit
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    cudaMemsetAsync(d_counter, 0, sizeof(int), stream);
    const int lrc = d->precision == ERLBM_FP64
                        ? launch_batch_fp64(d->q, sh.npt, g, d_runs, n_runs, d_counter, d_res, d_aos, sh.grid,
                                            sh.block, sh.smem, sh.dbl, stream)
                        : launch_batch_fp32(d->q, sh.npt, g, d_runs, n_runs, d_counter, d_res, d_aos, sh.grid,
                                            sh.block, sh.smem, sh.dbl, stream);
    cudaError_t ce = cudaStreamEndCapture(stream, &graph);
    if (lrc != 0 || ce != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();
        if (lrc == -1) {
            set_error("no batched kernel for this lattice shape%s%s", "", "");
            return ERLBM_E_UNSUPPORTED;
        }
        return cuda_fail(ce != cudaSuccess ? ce : cudaErrorLaunchFailure, "batched launch capture");
    }
    ce = cudaGraphInstantiate(&exec, graph, 0);
    if (ce == cudaSuccess) ce = cudaGraphLaunch(exec, stream);
    if (ce == cudaSuccess)
        ce = cudaMemcpyAsync(out, d_res, (size_t)n_runs * sizeof(BatchResult), cudaMemcpyDeviceToHost, stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(stream);
    if (exec) cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
    if (ce != cudaSuccess) return cuda_fail(ce, "batched run");
    return ERLBM_OK;
}

}  // namespace erlbm

// The run table of a stability map: one erlbm_run_spec per point (per operator, RLBM first when
// op = 0), the batch descriptor, and the obstacle's solid mask (bd->solid points into it).
static int build_map_runs(const erlbm_map_desc *d, erlbm_batch_desc *bd, std::vector<erlbm_run_spec> *runs,
                          std::vector<uint8_t> *solid, int *n_ops)
{
    if (d->n_i < 1 || d->n_j < 1) return ERLBM_E_INVAL;
    const int npts = d->n_points > 0 ? d->n_points : d->n_i * d->n_j;
    if (d->n_points > 0 && (!d->pi || !d->pj)) return ERLBM_E_INVAL;
    std::vector<int> ops;
    if (d->kind == ERLBM_MAP_TAYLOR_GREEN) {
        if (d->op == 0) ops = {ERLBM_OP_REG, ERLBM_OP_EXTREG};
        else if (d->op == ERLBM_OP_REG || d->op == ERLBM_OP_EXTREG || d->op == ERLBM_OP_BGK) ops = {d->op};
        else return d->op == ERLBM_OP_MRT ? ERLBM_E_UNSUPPORTED : ERLBM_E_INVAL;
    } else if (d->kind == ERLBM_MAP_OBSTACLE) {
        ops = {ERLBM_OP_EXTREG};  // the obstacle program always uses coll_Ext_Reg (:102)
    } else {
        return ERLBM_E_INVAL;
    }
    *n_ops = (int)ops.size();
    const int n_runs = npts * (int)ops.size();
    runs->assign(n_runs, erlbm_run_spec{});
    memset(bd, 0, sizeof(*bd));
    bd->precision = d->precision;
    bd->slots = d->slots;
    if (d->kind == ERLBM_MAP_TAYLOR_GREEN) {
        const int L = d->L > 0 ? d->L : 16;
        bd->q = 19;
        bd->nx = bd->ny = L;
        bd->inlet_x = bd->outlet_x = -1;
        bd->rho0 = 1.0;
        bd->energy_every = 100;    // :71
        bd->energy_factor = 2.0;   // :75
        bd->init = ERLBM_INIT_TG_MAP;
        for (size_t o = 0; o < ops.size(); o++)
            for (int k = 0; k < npts; k++) {
                const int i = d->n_points > 0 ? d->pi[k] : k % d->n_i;
                const int j = d->n_points > 0 ? d->pj[k] : k / d->n_i;
                double u0, tau, tau_nh;
                erlbm_tg_map_params(i, j, d->n_i, d->n_j, ops[o], d->tau_nh, &u0, &tau, &tau_nh);
                erlbm_run_spec &r = (*runs)[o * npts + k];
                r.op = ops[o];
                r.tau = tau;
                r.tau_nh = tau_nh;
                r.u0 = u0;
                r.n_steps = (int)((double)(100 * L) / u0);  // :63, 100 T
                if (d->max_steps > 0 && r.n_steps > d->max_steps) r.n_steps = d->max_steps;
                r.aos_offset = 0;
            }
    } else {
        int nx, ny;
        erlbm_obstacle_geometry(1, 1, &nx, &ny, nullptr);
        solid->resize((size_t)nx * ny);
        erlbm_obstacle_geometry(1, 1, &nx, &ny, solid->data());
        bd->q = 19;
        bd->nx = nx;
        bd->ny = ny;
        bd->solid = solid->data();
        bd->inlet_x = 1;            // :92
        bd->outlet_x = nx - 2;      // :94
        bd->rho0 = 1.0;
        bd->density_check = 1;      // :104-106
        bd->density_limit = 10.0;
        bd->init = ERLBM_INIT_REST; // :81-82
        const double ma = d->ma > 0 ? d->ma : 0.1;
        for (int k = 0; k < npts; k++) {
            const int i = d->n_points > 0 ? d->pi[k] : k % d->n_i;
            const int j = d->n_points > 0 ? d->pj[k] : k / d->n_i;
            double u_imp, tau, tau_nh;
            erlbm_obstacle_map_params(i, j, d->n_i, d->n_j, ma, &u_imp, &tau, &tau_nh);
            erlbm_run_spec &r = (*runs)[k];
            r.op = ERLBM_OP_EXTREG;
            r.tau = tau;
            r.tau_nh = tau_nh;
            r.u0 = u_imp;
            r.n_steps = (int)((double)(200 * ny) / u_imp);  // :84
            if (d->max_steps > 0 && r.n_steps > d->max_steps) r.n_steps = d->max_steps;
            r.aos_offset = 0;
        }
    }
    return ERLBM_OK;
}

extern "C" {

int erlbm_batch_run(const erlbm_batch_desc *d, int n_runs, const erlbm_run_spec *runs, const double *aos,
                    size_t n_aos, erlbm_batch_result *out)
{
    cudaStream_t s;
    CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    const int rc = run_batch(d, n_runs, runs, aos, n_aos, out, s);
    cudaStreamDestroy(s);
    return rc;
}

int erlbm_map_run(const erlbm_map_desc *d, int32_t *labels, int32_t *decided_step, double *margins)
{
    if (!d || !labels) return ERLBM_E_INVAL;
    erlbm_batch_desc bd;
    std::vector<erlbm_run_spec> runs;
    std::vector<uint8_t> solid;
    int n_ops = 0;
    int rc = build_map_runs(d, &bd, &runs, &solid, &n_ops);
    if (rc) return rc;
    const int n_runs = (int)runs.size();
    std::vector<erlbm_batch_result> res(n_runs);
    rc = erlbm_batch_run(&bd, n_runs, runs.data(), nullptr, 0, res.data());
    if (rc) return rc;
    for (int k = 0; k < n_runs; k++) {
        labels[k] = res[k].label;
        if (decided_step) decided_step[k] = res[k].decided_step;
        if (margins) margins[k] = res[k].margin;
    }
    return ERLBM_OK;
}

int erlbm_map_run_refined(const erlbm_map_desc *d, const erlbm_refine_desc *r, int32_t *labels,
                          int32_t *decided_step, double *margins, uint8_t *refined, int *n_passes)
{
    if (!d || !r || !labels) return ERLBM_E_INVAL;
    if (d->n_points != 0) {
        set_error("a refined map needs the whole n_i x n_j grid (n_points = 0)%s%s", "", "");
        return ERLBM_E_INVAL;
    }
    if (r->radius < 0 || r->radius > 64 || !(r->late_fraction <= 1.0) || r->probe_stride < 0 ||
        r->max_passes < 0) {
        set_error("refine radius must lie in [0, 64], late_fraction be at most 1, probe_stride and "
                  "max_passes be non-negative%s%s", "", "");
        return ERLBM_E_INVAL;
    }
    erlbm_batch_desc bd;
    std::vector<erlbm_run_spec> runs;
    std::vector<uint8_t> solid;
    int n_ops = 0;
    int rc = build_map_runs(d, &bd, &runs, &solid, &n_ops);
    if (rc) return rc;
    const int ni = d->n_i, nj = d->n_j, n_runs = (int)runs.size(), rad = r->radius;
    const size_t plane_n = (size_t)ni * nj;
    // pass 0: every point in FP32-shifted
    std::vector<erlbm_batch_result> res(n_runs);
    bd.precision = ERLBM_FP32_SHIFTED;
    rc = erlbm_batch_run(&bd, n_runs, runs.data(), nullptr, 0, res.data());
    if (rc) return rc;
    std::vector<uint8_t> done(n_runs, 0), change(plane_n);
    std::vector<int32_t> lab(plane_n), hi(plane_n), lo(plane_n);
    // change[k] = 1 when the window of half-width rad around k (clipped to the grid) holds two labels;
    // the max and min filters are taken along i and then along j
    auto find_changes = [&](const erlbm_batch_result *plane) {
        for (size_t k = 0; k < plane_n; k++) lab[k] = plane[k].label;
        for (int j = 0; j < nj; j++)
            for (int i = 0; i < ni; i++) {
                int32_t a = lab[(size_t)j * ni + i], b = a;
                for (int ii = std::max(0, i - rad); ii <= std::min(ni - 1, i + rad); ii++) {
                    a = std::max(a, lab[(size_t)j * ni + ii]);
                    b = std::min(b, lab[(size_t)j * ni + ii]);
                }
                hi[(size_t)j * ni + i] = a;
                lo[(size_t)j * ni + i] = b;
            }
        for (int j = 0; j < nj; j++)
            for (int i = 0; i < ni; i++) {
                int32_t a = hi[(size_t)j * ni + i], b = lo[(size_t)j * ni + i];
                for (int jj = std::max(0, j - rad); jj <= std::min(nj - 1, j + rad); jj++) {
                    a = std::max(a, hi[(size_t)jj * ni + i]);
                    b = std::min(b, lo[(size_t)jj * ni + i]);
                }
                change[(size_t)j * ni + i] = a != b;
            }
    };
    const int s = r->probe_stride;
    int passes = 0;
    std::vector<int> pick;
    for (;;) {
        pick.clear();
        for (int o = 0; o < n_ops; o++) {
            const size_t base = (size_t)o * plane_n;
            find_changes(res.data() + base);
            for (int j = 0; j < nj; j++)
                for (int i = 0; i < ni; i++) {
                    const size_t k = (size_t)j * ni + i;
                    if (done[base + k]) continue;
                    bool sel = change[k] != 0;
                    if (passes == 0) {
                        sel = sel || (s > 0 && i % s == s / 2 && j % s == s / 2) ||
                              (r->late_fraction > 0.0 && res[base + k].label == 1 &&
                               res[base + k].decided_step > r->late_fraction * runs[base + k].n_steps);
                    }
                    if (sel) pick.push_back((int)(base + k));
                }
        }
        if (pick.empty() || (r->max_passes > 0 && passes == r->max_passes)) break;
        // the selected runs again in FP64, whose results are the reference's
        std::vector<erlbm_run_spec> sub(pick.size());
        for (size_t m = 0; m < pick.size(); m++) sub[m] = runs[pick[m]];
        std::vector<erlbm_batch_result> r64(pick.size());
        bd.precision = ERLBM_FP64;
        rc = erlbm_batch_run(&bd, (int)sub.size(), sub.data(), nullptr, 0, r64.data());
        if (rc) return rc;
        for (size_t m = 0; m < pick.size(); m++) {
            res[pick[m]] = r64[m];
            done[pick[m]] = 1;
        }
        passes++;
    }
    if (refined) memcpy(refined, done.data(), (size_t)n_runs);
    if (n_passes) *n_passes = passes;
    for (int k = 0; k < n_runs; k++) {
        labels[k] = res[k].label;
        if (decided_step) decided_step[k] = res[k].decided_step;
        if (margins) margins[k] = res[k].margin;
    }
    return ERLBM_OK;
}

}  // extern "C"
