// erlbm_abi.cu -- C ABI of the single-lattice engine (include/erlbm_gb300.h).
//
// A handle owns one lattice on the device: two SoA population buffers (ping-pong), an optional
// solid mask and fluid-index map, a staging buffer for the caller's AoS arrays, reduction
// scratch, a run-status block and its own CUDA stream.
//
// State machine.  The reference's drivers hold post-stream populations at the top of each step.
// The kernels here fuse "stream of step s-1" with "boundary + collision of step s", so between
// launches the buffer holds post-collision populations with the stream still pending:
//   after erlbm_set_populations: kind = PRE   (buffer = post-stream populations, as given)
//   after >= 1 step:             kind = POST  (buffer = post-collision populations of the last step)
// The first step after a set collides the given populations in place (mode 1); every later step
// pulls (mode 0).  Post-stream populations of a POST state are produced on demand by a stream-only
// pass into the spare buffer, so nothing the caller can observe differs from the reference loop.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/erlbm_gb300.h"
#include "abi_internal.h"
#include "kernels_api.h"

using namespace erlbm;

namespace erlbm {

static thread_local std::string g_last_error;

void set_error(const char *fmt, const char *a, const char *b)
{
    char buf[512];
    snprintf(buf, sizeof(buf), fmt, a ? a : "", b ? b : "");
    g_last_error = buf;
}

int cuda_fail(cudaError_t e, const char *where)
{
    set_error("CUDA error in %s: %s", where, cudaGetErrorString(e));
    return ERLBM_E_CUDA;
}

}  // namespace erlbm

#define CK(call)                                              \
    do {                                                      \
        cudaError_t e_ = (call);                              \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call);   \
    } while (0)

#define CKL(rc, what)                                                                  \
    do {                                                                               \
        int r_ = (rc);                                                                 \
        if (r_ != 0) {                                                                 \
            cudaError_t e_ = cudaGetLastError();                                       \
            if (e_ != cudaSuccess) return cuda_fail(e_, what);                         \
            set_error("launch of %s rejected its arguments%s", what, "");              \
            return ERLBM_E_INVAL;                                                      \
        }                                                                              \
    } while (0)

struct erlbm_handle {
    int q = 0, prec = 0, op = 0, device = 0;
    double tau = 0, tau_nh = 0;
    Relax R{};
    Geo g{};
    long long n_fluid = 0;
    uint8_t *d_solid = nullptr;
    uint8_t *d_segflag = nullptr;    // D2Q9, nx % 128 == 0, solids: per 128-column segment, a solid in its stencil
    uint8_t *d_nodeflag = nullptr;   // and per node, a solid among its eight neighbours
    int *d_fix = nullptr;            // the fluid nodes with a solid neighbour (n_fix)
    int n_fix = 0;
    int *d_nof = nullptr;            // node of fluid index (null for periodic boxes)
    void *d_buf[2] = {nullptr, nullptr};
    int cur = 0;
    int kind = 0;                    // 0 PRE (post-stream), 1 POST (post-collision, stream pending)
    long long steps_done = 0;
    double *d_aos = nullptr;         // staging: n_fluid * q doubles
    double *d_scr = nullptr;         // n_fluid doubles of per-node values + 4096 reduction scratch
    double *d_out = nullptr;         // small device result block
    RunStatus *d_status = nullptr;
    cudaStream_t stream = nullptr;
    cudaStream_t own_stream = nullptr;  // the stream created at erlbm_create
    int shape = 0;                      // launch shape of the fused periodic kernel (erlbm_set_launch)
    bool two_step = false;              // pairs of fused periodic steps as one launch (erlbm_set_launch)
    bool three_step = false;            // triples of fused periodic steps as one launch (erlbm_set_launch)
    bool wide_strips = false;           // the three-step launches use 64-column strips over column pairs
    std::vector<uint8_t> h_solid;       // host copy of the solid mask (empty for periodic boxes)
    std::vector<double> h_profile;      // parabolic inlet velocity per (y, z) of the inlet plane
    double *d_profile = nullptr;
    double profile_key[3] = {-1, 0, 0}; // inlet_x, u_in, L of the uploaded profile
    // CUDA graphs of a block of plain fused periodic steps, one per buffer parity, for the launch
    // shape and parameters in graph_key (rebuilt when erlbm_set_launch or erlbm_set_params changes them)
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    long long graph_key = -1;
    // the same for blocks of D2Q9 FP32 steps with solids or planes (k_d2q9_hybrid), for the planes in
    // bc_graph_bc (rebuilt when a call brings other planes)
    cudaGraphExec_t bc_graph[2] = {nullptr, nullptr};
    BCp bc_graph_bc{};
    cudaStream_t capture_stream = nullptr;
    size_t elem() const { return prec == ERLBM_FP32_SHIFTED ? sizeof(float) : 8; }  // FP64 or a float pair
};

namespace {

int check_handle(const erlbm_handle *h)
{
    if (!h) {
        set_error("null handle%s%s", "", "");
        return ERLBM_E_INVAL;
    }
    return ERLBM_OK;
}

// MRT exists for D2Q9 only: the reference's dispatch compiles coll_MRT into D2Q9 builds alone
// (src/erlbm_common.h:74-76), and a D3Q19 build given "mrt" collides nothing.
int check_op(int op, int q)
{
    if (op == ERLBM_OP_BGK || op == ERLBM_OP_REG || op == ERLBM_OP_EXTREG) return ERLBM_OK;
    if (op == ERLBM_OP_MRT) {
        if (q == 9) return ERLBM_OK;
        set_error("collision operator MRT is a D2Q9 operator%s%s", "", "");
        return ERLBM_E_UNSUPPORTED;
    }
    set_error("unknown collision operator (use BGK=1, MRT=2, REG=3, EXTREG=4)%s%s", "", "");
    return ERLBM_E_INVAL;
}

void drop_bc_graphs(erlbm_handle *h)
{
    for (cudaGraphExec_t &x : h->bc_graph) {
        if (x) cudaGraphExecDestroy(x);
        x = nullptr;
    }
}

void drop_graphs(erlbm_handle *h)
{
    for (cudaGraphExec_t &x : h->graph) {
        if (x) cudaGraphExecDestroy(x);
        x = nullptr;
    }
    h->graph_key = -1;
    drop_bc_graphs(h);
}

void free_handle(erlbm_handle *h)
{
    if (!h) return;
    cudaFree(h->d_solid);
    cudaFree(h->d_segflag);
    cudaFree(h->d_nodeflag);
    cudaFree(h->d_fix);
    cudaFree(h->d_profile);
    cudaFree(h->d_nof);
    cudaFree(h->d_buf[0]);
    cudaFree(h->d_buf[1]);
    cudaFree(h->d_aos);
    cudaFree(h->d_scr);
    cudaFree(h->d_out);
    cudaFree(h->d_status);
    drop_graphs(h);
    if (h->capture_stream) cudaStreamDestroy(h->capture_stream);
    if (h->own_stream) cudaStreamDestroy(h->own_stream);
    delete h;
}

// Buffer holding the populations of `stage`; may run the stream-only pass into the spare buffer.
int stage_buffer(erlbm_handle *h, int stage, const void **out)
{
    if (stage != ERLBM_STAGE_POST_STREAM && stage != ERLBM_STAGE_POST_COLLISION) {
        set_error("unknown stage%s%s", "", "");
        return ERLBM_E_INVAL;
    }
    if (h->kind == 0) {
        if (stage == ERLBM_STAGE_POST_COLLISION) {
            set_error("no collision has run since the populations were set%s%s", "", "");
            return ERLBM_E_STATE;
        }
        *out = h->d_buf[h->cur];
        return ERLBM_OK;
    }
    if (stage == ERLBM_STAGE_POST_COLLISION) {
        *out = h->d_buf[h->cur];
        return ERLBM_OK;
    }
    void *spare = h->d_buf[h->cur ^ 1];
    if (h->prec == ERLBM_FP64)
        CKL(launch_stream_only_fp64(h->q, h->g, (const double *)h->d_buf[h->cur], (double *)spare, h->stream),
            "stream_only");
    else if (h->prec == ERLBM_FP32_PAIR)
        CKL(launch_stream_only_pair(h->q, h->g, (const float2 *)h->d_buf[h->cur], (float2 *)spare, h->stream),
            "stream_only");
    else
        CKL(launch_stream_only_fp32(h->q, h->g, (const float *)h->d_buf[h->cur], (float *)spare, h->stream),
            "stream_only");
    *out = spare;
    return ERLBM_OK;
}

int node_fields(erlbm_handle *h, const void *buf, double *e, double *rho, double *u)
{
    if (h->prec == ERLBM_FP64)
        CKL(launch_node_fields_fp64(h->q, h->g, h->n_fluid, h->d_nof, (const double *)buf, e, rho, u, h->stream),
            "node_fields");
    else if (h->prec == ERLBM_FP32_PAIR)
        CKL(launch_node_fields_pair(h->q, h->g, h->n_fluid, h->d_nof, (const float2 *)buf, e, rho, u, h->stream),
            "node_fields");
    else
        CKL(launch_node_fields_fp32(h->q, h->g, h->n_fluid, h->d_nof, (const float *)buf, e, rho, u, h->stream),
            "node_fields");
    return ERLBM_OK;
}

int ensure_aos(erlbm_handle *h)
{
    if (h->d_aos) return ERLBM_OK;
    const size_t bytes = (size_t)h->n_fluid * h->q * sizeof(double);
    if (cudaMalloc(&h->d_aos, bytes ? bytes : 8) != cudaSuccess) {
        cudaGetLastError();
        set_error("out of device memory for the staging buffer%s%s", "", "");
        return ERLBM_E_OOM;
    }
    return ERLBM_OK;
}

// The reference's parabolic profile (Boundary_conditions.cpp:467-472): the h-th fluid node of a column
double parabolic_vel(int hh, double vx_max, int L)
{
    const double d_h = (double)hh - 0.5;
    return -4.0 * vx_max / (L * L) * (d_h) * (d_h - L);
}

int validate_bc(erlbm_handle *h, const erlbm_bc *bc, BCp *out)
{
    out->inlet_x = -1;
    out->outlet_x = -1;
    out->u_in = 0;
    out->rho_out = 1;
    out->inlet_kind = ERLBM_INLET_ZOUHE;
    out->outlet_kind = ERLBM_OUTLET_DENSITY;
    out->open_y = -1;
    out->profile = nullptr;
    if (!bc) return ERLBM_OK;
    const Geo &g = h->g;
    auto solid = [h](long long n) { return !h->h_solid.empty() && h->h_solid[n]; };
    if (bc->inlet_x >= 0) {
        if (bc->inlet_x >= g.nx) {
            set_error("inlet plane outside the box%s%s", "", "");
            return ERLBM_E_INVAL;
        }
        if (bc->inlet_kind != ERLBM_INLET_ZOUHE && bc->inlet_kind != ERLBM_INLET_PARABOLIC) {
            set_error("unknown inlet kind%s%s", "", "");
            return ERLBM_E_INVAL;
        }
        out->inlet_x = bc->inlet_x;
        out->u_in = bc->u_in;
        out->inlet_kind = bc->inlet_kind;
        if (bc->inlet_kind == ERLBM_INLET_PARABOLIC) {
            const int L = bc->parabolic_L;
            if (L < 1 || L >= g.ny) {
                set_error("parabolic_L must lie in [1, ny) (the reference's profile table has ny entries)%s%s", "",
                          "");
                return ERLBM_E_INVAL;
            }
            const double key[3] = {(double)bc->inlet_x, bc->u_in, (double)L};
            if (!h->d_profile || memcmp(key, h->profile_key, sizeof(key)) != 0) {
                std::vector<double> prof((size_t)g.ny * g.nz, 0.0);
                for (int z = 0; z < g.nz; z++) {
                    int hh = 0;
                    for (int y = 0; y < g.ny; y++) {
                        if (solid(bc->inlet_x + (long long)g.nx * (y + (long long)g.ny * z))) continue;
                        if (++hh > L) {
                            set_error("a column of the inlet plane holds more than parabolic_L fluid nodes%s%s", "",
                                      "");
                            return ERLBM_E_INVAL;
                        }
                        prof[y + (size_t)g.ny * z] = parabolic_vel(hh, bc->u_in, L);
                    }
                }
                if (!h->d_profile) CK(cudaMalloc(&h->d_profile, prof.size() * sizeof(double)));
                CK(cudaStreamSynchronize(h->stream));  // the previous profile may still be in use
                h->h_profile.swap(prof);
                CK(cudaMemcpyAsync(h->d_profile, h->h_profile.data(), h->h_profile.size() * sizeof(double),
                                   cudaMemcpyHostToDevice, h->stream));
                memcpy(h->profile_key, key, sizeof(key));
            }
            out->profile = h->d_profile;
        }
    }
    if (bc->outlet_x >= 0) {
        if (bc->outlet_x >= g.nx || g.nx < 2) {
            set_error("outlet plane outside the box%s%s", "", "");
            return ERLBM_E_INVAL;
        }
        const int nb = bc->outlet_x + (bc->outlet_x < g.nx / 2 ? 1 : -1);
        if (nb < 0 || nb >= g.nx) {
            set_error("outlet plane has no inner neighbour%s%s", "", "");
            return ERLBM_E_INVAL;
        }
        if (bc->outlet_kind < ERLBM_OUTLET_DENSITY || bc->outlet_kind > ERLBM_OUTLET_CONVECTIVE ||
            bc->outlet_x == bc->inlet_x) {
            set_error("unknown outlet kind, or outlet and inlet on one plane%s%s", "", "");
            return ERLBM_E_INVAL;
        }
        if (bc->outlet_kind == ERLBM_OUTLET_OPEN && h->q != 9) {
            set_error("the open outlet is a D2Q9 boundary (OpenBoundaryD2Q9_x)%s%s", "", "");
            return ERLBM_E_UNSUPPORTED;
        }
        out->outlet_x = bc->outlet_x;
        out->rho_out = bc->rho_out;
        out->outlet_kind = bc->outlet_kind;
    }
    if (bc->open_y_on) {
        if (h->q != 9) {
            set_error("the open y plane is a D2Q9 boundary (OpenBoundaryD2Q9_y)%s%s", "", "");
            return ERLBM_E_UNSUPPORTED;
        }
        const int yn = bc->open_y + (bc->open_y < g.ny / 2 ? 1 : -1);
        if (bc->open_y < 0 || bc->open_y >= g.ny || yn < 0 || yn >= g.ny) {
            set_error("open y plane outside the box or without an inner neighbour%s%s", "", "");
            return ERLBM_E_INVAL;
        }
        out->open_y = bc->open_y;
    }
    return ERLBM_OK;
}

// Enqueue one step.  status/check_density are used by erlbm_run.
int enqueue_step(erlbm_handle *h, const BCp &bc, int check_density, double density_limit, bool stop_on_flag)
{
    StepArgs a;
    a.mode = h->kind == 0 ? 1 : 0;
    a.step_index = (int)h->steps_done;
    a.check_density = check_density;
    a.density_limit = density_limit;
    a.status = (check_density || stop_on_flag) ? h->d_status : nullptr;
    a.stop_on_flag = stop_on_flag ? 1 : 0;
    void *src = h->d_buf[h->cur], *dst = h->d_buf[h->cur ^ 1];
    const bool plain =
        bc.inlet_x < 0 && bc.outlet_x < 0 && bc.open_y < 0 && !check_density && !stop_on_flag && a.mode == 0;
    if (h->prec == ERLBM_FP32_PAIR) {
        if (!plain && !(a.mode == 1 && bc.inlet_x < 0 && bc.outlet_x < 0 && bc.open_y < 0 && !check_density &&
                        !stop_on_flag)) {
            set_error("the compensated FP32 form runs periodic lattices without boundary planes or per-step "
                      "density checks%s%s", "", "");
            return ERLBM_E_UNSUPPORTED;
        }
        CKL(launch_step_pair(h->q, h->op, h->g, h->R, a.mode, (const float2 *)src, (float2 *)dst, h->stream),
            "step_pair");
    } else if (h->prec == ERLBM_FP32_SHIFTED && h->q == 9 && plain && periodic_d2q9_fp32_ok(h->g)) {
        CKL(launch_periodic_d2q9_fp32(h->op, h->g, h->R, (const float *)src, (float *)dst, h->stream, h->shape),
            "periodic_d2q9");
    } else if (h->prec == ERLBM_FP32_SHIFTED && h->q == 9 && a.mode == 0 && !check_density && !stop_on_flag &&
               d2q9_hybrid_ok(h->g)) {
        CKL(launch_step_fp32_hybrid(h->op, h->g, bc, h->R, (const float *)src, (float *)dst, h->d_segflag,
                                    h->d_nodeflag, h->d_fix, h->n_fix, h->stream),
            "d2q9_hybrid");
    } else if (h->prec == ERLBM_FP64) {
        CKL(launch_step_fp64(h->q, h->op, h->g, bc, h->R, a, (const double *)src, (double *)dst, h->stream), "step");
    } else {
        CKL(launch_step_fp32(h->q, h->op, h->g, bc, h->R, a, (const float *)src, (float *)dst, h->stream), "step");
    }
    h->cur ^= 1;
    h->kind = 1;
    h->steps_done++;
    return ERLBM_OK;
}

// A block of plain periodic steps of the fused FP32 D2Q9 kernels (per_launch steps per launch) as one
// CUDA graph launch: the launches of a block are captured once per buffer parity and replayed, so a
// small lattice is not bound by the host's launch rate.  An even number of launches leaves the
// buffer parity unchanged.
// steps per graph: an even number of launches of every shape (1, 2 or 3 steps each)
int graph_steps_of(int per_launch) { return per_launch == 3 ? 66 : 64; }

int graph_steps(erlbm_handle *h, int per_launch)
{
    const int n_steps = graph_steps_of(per_launch);
    const long long key = per_launch | ((long long)h->shape << 2);
    if (h->graph_key != key) {
        drop_graphs(h);
        h->graph_key = key;
    }
    cudaGraphExec_t &x = h->graph[h->cur];
    if (!x) {
        if (!h->capture_stream) CK(cudaStreamCreateWithFlags(&h->capture_stream, cudaStreamNonBlocking));
        CK(cudaStreamBeginCapture(h->capture_stream, cudaStreamCaptureModeRelaxed));
        int c = h->cur, lrc = 0;
        for (int k = 0; k < n_steps / per_launch && lrc == 0; k++) {
            const float *src = (const float *)h->d_buf[c];
            float *dst = (float *)h->d_buf[c ^ 1];
            lrc = per_launch == 3   ? launch_periodic_d2q9_fp32_x3(h->op, h->g, h->R, src, dst, h->capture_stream,
                                                                 h->wide_strips)
                  : per_launch == 2 ? launch_periodic_d2q9_fp32_x2(h->op, h->g, h->R, src, dst, h->capture_stream)
                                    : launch_periodic_d2q9_fp32(h->op, h->g, h->R, src, dst, h->capture_stream,
                                                                h->shape);
            c ^= 1;
        }
        cudaGraph_t graph = nullptr;
        const cudaError_t e = cudaStreamEndCapture(h->capture_stream, &graph);
        if (lrc != 0 || e != cudaSuccess || !graph) {
            if (graph) cudaGraphDestroy(graph);
            const cudaError_t le = cudaGetLastError();
            return cuda_fail(e != cudaSuccess ? e : (le != cudaSuccess ? le : cudaErrorInvalidValue),
                             "capture of the periodic step graph");
        }
        const cudaError_t ie = cudaGraphInstantiate(&x, graph, 0);
        cudaGraphDestroy(graph);
        if (ie != cudaSuccess) {
            x = nullptr;
            return cuda_fail(ie, "cudaGraphInstantiate");
        }
    }
    CK(cudaGraphLaunch(x, h->stream));
    h->steps_done += n_steps;
    h->kind = 1;
    return ERLBM_OK;
}

bool same_planes(const BCp &a, const BCp &b)
{
    return a.inlet_x == b.inlet_x && a.u_in == b.u_in && a.outlet_x == b.outlet_x && a.rho_out == b.rho_out &&
           a.inlet_kind == b.inlet_kind && a.outlet_kind == b.outlet_kind && a.open_y == b.open_y &&
           a.profile == b.profile;
}

// A block of BC_GRAPH_STEPS steps of k_d2q9_hybrid as one CUDA graph launch, captured once per buffer
// parity for the planes b.  The parabolic profile is read from h->d_profile when the graph runs, and
// validate_bc rewrites it only after the stream has drained.
constexpr int BC_GRAPH_STEPS = 64;

int bc_graph_steps(erlbm_handle *h, const BCp &b)
{
    if (!same_planes(h->bc_graph_bc, b)) {
        drop_bc_graphs(h);
        h->bc_graph_bc = b;
    }
    cudaGraphExec_t &x = h->bc_graph[h->cur];
    if (!x) {
        if (!h->capture_stream) CK(cudaStreamCreateWithFlags(&h->capture_stream, cudaStreamNonBlocking));
        CK(cudaStreamBeginCapture(h->capture_stream, cudaStreamCaptureModeRelaxed));
        int c = h->cur, lrc = 0;
        for (int k = 0; k < BC_GRAPH_STEPS && lrc == 0; k++) {
            lrc = launch_step_fp32_hybrid(h->op, h->g, b, h->R, (const float *)h->d_buf[c], (float *)h->d_buf[c ^ 1],
                                          h->d_segflag, h->d_nodeflag, h->d_fix, h->n_fix, h->capture_stream);
            c ^= 1;
        }
        cudaGraph_t graph = nullptr;
        const cudaError_t e = cudaStreamEndCapture(h->capture_stream, &graph);
        if (lrc != 0 || e != cudaSuccess || !graph) {
            if (graph) cudaGraphDestroy(graph);
            const cudaError_t le = cudaGetLastError();
            return cuda_fail(e != cudaSuccess ? e : (le != cudaSuccess ? le : cudaErrorInvalidValue),
                             "capture of the boundary step graph");
        }
        const cudaError_t ie = cudaGraphInstantiate(&x, graph, 0);
        cudaGraphDestroy(graph);
        if (ie != cudaSuccess) {
            x = nullptr;
            return cuda_fail(ie, "cudaGraphInstantiate");
        }
    }
    CK(cudaGraphLaunch(x, h->stream));
    h->steps_done += BC_GRAPH_STEPS;
    h->kind = 1;
    return ERLBM_OK;
}

int energy_now(erlbm_handle *h, int stage, double *E)
{
    const void *buf;
    int rc = stage_buffer(h, stage, &buf);
    if (rc) return rc;
    if ((rc = node_fields(h, buf, h->d_scr, nullptr, nullptr))) return rc;
    // serial order (the reference's) up to 2^16 nodes, fixed-shape tree above
    CKL(launch_sum(h->d_scr, h->n_fluid, 1 << 16, h->d_scr + h->n_fluid, h->d_out, h->stream), "sum");
    CK(cudaMemcpyAsync(E, h->d_out, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return ERLBM_OK;
}

}  // namespace

extern "C" {

int erlbm_version(void) { return 10000; }

const char *erlbm_strerror(int code)
{
    switch (code) {
    case ERLBM_OK: return "ok";
    case ERLBM_E_INVAL: return "invalid argument";
    case ERLBM_E_OOM: return "out of memory";
    case ERLBM_E_CUDA: return "CUDA error";
    case ERLBM_E_TIMEOUT: return "timeout";
    case ERLBM_E_NONFINITE: return "non-finite value";
    case ERLBM_E_UNSUPPORTED: return "unsupported";
    case ERLBM_E_STATE: return "invalid state";
    default: return "unknown error";
    }
}

const char *erlbm_last_error(void) { return g_last_error.c_str(); }

int erlbm_create(const erlbm_desc *d, erlbm_handle **out)
{
    if (!d || !out) {
        set_error("null argument%s%s", "", "");
        return ERLBM_E_INVAL;
    }
    *out = nullptr;
    if (d->q != 9 && d->q != 19) {
        set_error("q must be 9 (D2Q9) or 19 (D3Q19)%s%s", "", "");
        return ERLBM_E_INVAL;
    }
    if (d->nx < 1 || d->ny < 1 || d->nz < 1 || (d->q == 9 && d->nz != 1)) {
        set_error("bad lattice extent (D2Q9 needs nz = 1)%s%s", "", "");
        return ERLBM_E_INVAL;
    }
    if ((long long)d->nx * d->ny * d->nz > (1LL << 31) - 1) {
        set_error("lattice too large for 32-bit node indices%s%s", "", "");
        return ERLBM_E_INVAL;
    }
    if (d->precision != ERLBM_FP64 && d->precision != ERLBM_FP32_SHIFTED && d->precision != ERLBM_FP32_PAIR) {
        set_error("unknown precision%s%s", "", "");
        return ERLBM_E_INVAL;
    }
    int rc = check_op(d->op, d->q);
    if (rc) return rc;
    if (d->precision == ERLBM_FP32_PAIR && (d->q != 9 || d->solid || d->op == ERLBM_OP_MRT)) {
        set_error("the compensated FP32 form runs periodic D2Q9 lattices with BGK, RLBM or E-RLBM%s%s", "", "");
        return ERLBM_E_UNSUPPORTED;
    }
    if (!(d->tau > 0) || !std::isfinite(d->tau) || !std::isfinite(d->tau_nh) || d->tau_nh == 0) {
        set_error("tau and tau_nh must be finite and non-zero%s%s", "", "");
        return ERLBM_E_INVAL;
    }
    erlbm_handle *h = new (std::nothrow) erlbm_handle();
    if (!h) return ERLBM_E_OOM;
    h->q = d->q;
    h->prec = d->precision;
    h->op = d->op;
    h->tau = d->tau;
    h->tau_nh = d->tau_nh;
    h->R = make_relax(d->tau, d->tau_nh, d->op);
    h->g.nx = d->nx;
    h->g.ny = d->ny;
    h->g.nz = d->nz;
    h->g.nbox = (long long)d->nx * d->ny * d->nz;
    h->g.plane = (h->g.nbox + 63) / 64 * 64;
    h->g.solid = nullptr;
    cudaError_t e;
    if ((e = cudaGetDevice(&h->device)) != cudaSuccess) {
        free_handle(h);
        return cuda_fail(e, "cudaGetDevice");
    }
    if ((e = cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking)) != cudaSuccess) {
        free_handle(h);
        return cuda_fail(e, "cudaStreamCreate");
    }
    h->stream = h->own_stream;
    std::vector<int> nof;
    h->n_fluid = h->g.nbox;
    if (d->solid) {
        bool any = false;
        for (long long k = 0; k < h->g.nbox; k++) any |= d->solid[k] != 0;
        if (any) {
            nof.reserve(h->g.nbox);
            for (long long k = 0; k < h->g.nbox; k++)
                if (!d->solid[k]) nof.push_back((int)k);
            h->n_fluid = (long long)nof.size();
            h->h_solid.assign(d->solid, d->solid + h->g.nbox);
        }
    }
    const size_t pop_bytes = (size_t)h->q * h->g.plane * h->elem();
    bool ok = cudaMalloc(&h->d_buf[0], pop_bytes) == cudaSuccess && cudaMalloc(&h->d_buf[1], pop_bytes) == cudaSuccess &&
              cudaMalloc(&h->d_scr, ((size_t)h->n_fluid + 4096) * sizeof(double)) == cudaSuccess &&
              cudaMalloc(&h->d_out, 64 * sizeof(double)) == cudaSuccess &&
              cudaMalloc(&h->d_status, sizeof(RunStatus)) == cudaSuccess;
    if (ok && !nof.empty()) {
        ok = cudaMalloc(&h->d_solid, h->g.nbox) == cudaSuccess &&
             cudaMalloc(&h->d_nof, nof.size() * sizeof(int)) == cudaSuccess;
        if (ok) {
            ok = cudaMemcpy(h->d_solid, d->solid, h->g.nbox, cudaMemcpyHostToDevice) == cudaSuccess &&
                 cudaMemcpy(h->d_nof, nof.data(), nof.size() * sizeof(int), cudaMemcpyHostToDevice) == cudaSuccess;
            h->g.solid = h->d_solid;
        }
        if (ok && h->q == 9 && h->prec == ERLBM_FP32_SHIFTED && d2q9_hybrid_ok(h->g)) {
            std::vector<uint8_t> flags((size_t)h->g.ny * (h->g.nx / 128)), nflags((size_t)h->g.nbox);
            d2q9_segment_flags(h->g, d->solid, flags.data(), nflags.data());
            std::vector<int> fix;
            for (long long k = 0; k < h->g.nbox; k++)
                if (nflags[k] && !d->solid[k]) fix.push_back((int)k);
            h->n_fix = (int)fix.size();
            ok = cudaMalloc(&h->d_fix, std::max<size_t>(fix.size(), 1) * sizeof(int)) == cudaSuccess &&
                 (fix.empty() || cudaMemcpy(h->d_fix, fix.data(), fix.size() * sizeof(int), cudaMemcpyHostToDevice) ==
                                     cudaSuccess) &&
                 cudaMalloc(&h->d_segflag, flags.size()) == cudaSuccess &&
                 cudaMalloc(&h->d_nodeflag, nflags.size()) == cudaSuccess &&
                 cudaMemcpy(h->d_segflag, flags.data(), flags.size(), cudaMemcpyHostToDevice) == cudaSuccess &&
                 cudaMemcpy(h->d_nodeflag, nflags.data(), nflags.size(), cudaMemcpyHostToDevice) == cudaSuccess;
        }
    }
    if (!ok) {
        cudaError_t le = cudaGetLastError();
        free_handle(h);
        if (le == cudaErrorMemoryAllocation) {
            set_error("out of device memory%s%s", "", "");
            return ERLBM_E_OOM;
        }
        return cuda_fail(le, "erlbm_create");
    }
    // populations start as zeros (new double[] of the reference is uninitialised; callers set them)
    if ((e = cudaMemsetAsync(h->d_buf[0], 0, pop_bytes, h->stream)) != cudaSuccess ||
        (e = cudaMemsetAsync(h->d_buf[1], 0, pop_bytes, h->stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(h->stream)) != cudaSuccess) {
        free_handle(h);
        return cuda_fail(e, "erlbm_create");
    }
    *out = h;
    return ERLBM_OK;
}

int erlbm_destroy(erlbm_handle *h)
{
    if (!h) return ERLBM_OK;
    cudaStreamSynchronize(h->stream);
    free_handle(h);
    return ERLBM_OK;
}

int erlbm_fluid_count(const erlbm_handle *h, int64_t *n)
{
    int rc = check_handle(h);
    if (rc) return rc;
    if (!n) return ERLBM_E_INVAL;
    *n = h->n_fluid;
    return ERLBM_OK;
}

int erlbm_set_params(erlbm_handle *h, double tau, double tau_nh, int op)
{
    int rc = check_handle(h);
    if (rc) return rc;
    if ((rc = check_op(op, h->q))) return rc;
    if (h->prec == ERLBM_FP32_PAIR && op == ERLBM_OP_MRT) {
        set_error("MRT has no compensated FP32 form%s%s", "", "");
        return ERLBM_E_UNSUPPORTED;
    }
    if (!(tau > 0) || !std::isfinite(tau) || !std::isfinite(tau_nh) || tau_nh == 0) {
        set_error("tau and tau_nh must be finite and non-zero%s%s", "", "");
        return ERLBM_E_INVAL;
    }
    h->tau = tau;
    h->tau_nh = tau_nh;
    h->op = op;
    h->R = make_relax(tau, tau_nh, op);
    drop_graphs(h);  // a graph in flight finishes with the parameters it was captured with
    return ERLBM_OK;
}

int erlbm_set_populations(erlbm_handle *h, const double *aos, size_t n)
{
    int rc = check_handle(h);
    if (rc) return rc;
    if (!aos || n != (size_t)h->n_fluid * h->q) {
        set_error("population array must hold n_fluid * q doubles%s%s", "", "");
        return ERLBM_E_INVAL;
    }
    if ((rc = ensure_aos(h))) return rc;
    CK(cudaMemcpyAsync(h->d_aos, aos, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    if (h->prec == ERLBM_FP64)
        CKL(launch_aos_to_soa_fp64(h->q, h->g, h->n_fluid, h->d_nof, h->d_aos, (double *)h->d_buf[h->cur], h->stream),
            "aos_to_soa");
    else if (h->prec == ERLBM_FP32_PAIR)
        CKL(launch_aos_to_soa_pair(h->q, h->g, h->n_fluid, h->d_nof, h->d_aos, (float2 *)h->d_buf[h->cur], h->stream),
            "aos_to_soa");
    else
        CKL(launch_aos_to_soa_fp32(h->q, h->g, h->n_fluid, h->d_nof, h->d_aos, (float *)h->d_buf[h->cur], h->stream),
            "aos_to_soa");
    h->kind = 0;
    h->steps_done = 0;
    // the caller may reuse its buffer as soon as we return
    CK(cudaStreamSynchronize(h->stream));
    return ERLBM_OK;
}

int erlbm_get_populations(erlbm_handle *h, double *aos, size_t n, int stage)
{
    int rc = check_handle(h);
    if (rc) return rc;
    if (!aos || n != (size_t)h->n_fluid * h->q) {
        set_error("population array must hold n_fluid * q doubles%s%s", "", "");
        return ERLBM_E_INVAL;
    }
    if ((rc = ensure_aos(h))) return rc;
    const void *buf;
    if ((rc = stage_buffer(h, stage, &buf))) return rc;
    if (h->prec == ERLBM_FP64)
        CKL(launch_soa_to_aos_fp64(h->q, h->g, h->n_fluid, h->d_nof, (const double *)buf, h->d_aos, h->stream),
            "soa_to_aos");
    else if (h->prec == ERLBM_FP32_PAIR)
        CKL(launch_soa_to_aos_pair(h->q, h->g, h->n_fluid, h->d_nof, (const float2 *)buf, h->d_aos, h->stream),
            "soa_to_aos");
    else
        CKL(launch_soa_to_aos_fp32(h->q, h->g, h->n_fluid, h->d_nof, (const float *)buf, h->d_aos, h->stream),
            "soa_to_aos");
    CK(cudaMemcpyAsync(aos, h->d_aos, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return ERLBM_OK;
}

int erlbm_step(erlbm_handle *h, int n_steps, const erlbm_bc *bc)
{
    int rc = check_handle(h);
    if (rc) return rc;
    if (n_steps < 0) return ERLBM_E_INVAL;
    BCp b;
    if ((rc = validate_bc(h, bc, &b))) return rc;
    const bool plain = h->prec == ERLBM_FP32_SHIFTED && h->q == 9 && b.inlet_x < 0 && b.outlet_x < 0 &&
                       b.open_y < 0 && periodic_d2q9_fp32_ok(h->g);
    const bool fused3 = plain && h->three_step && periodic_d2q9_x2_ok(h->g) &&
                        (!h->wide_strips || periodic_d2q9_x3a_ok(h->g));
    const bool fused2 = plain && h->two_step && periodic_d2q9_x2_ok(h->g);
    const int per_launch = fused3 ? 3 : (fused2 ? 2 : 1);
    const bool hybrid = !plain && h->prec == ERLBM_FP32_SHIFTED && h->q == 9 && d2q9_hybrid_ok(h->g);
    for (int s = 0; s < n_steps;) {
        if (hybrid && h->kind == 1 && n_steps - s >= BC_GRAPH_STEPS) {
            if ((rc = bc_graph_steps(h, b))) return rc;
            s += BC_GRAPH_STEPS;
            continue;
        }
        if (plain && h->kind == 1 && n_steps - s >= graph_steps_of(per_launch)) {
            if ((rc = graph_steps(h, per_launch))) return rc;
            s += graph_steps_of(per_launch);
            continue;
        }
        if (fused3 && h->kind == 1 && n_steps - s >= 3) {
            // three plain periodic steps in one launch
            CKL(launch_periodic_d2q9_fp32_x3(h->op, h->g, h->R, (const float *)h->d_buf[h->cur],
                                             (float *)h->d_buf[h->cur ^ 1], h->stream, h->wide_strips),
                "periodic_d2q9_x3");
            h->cur ^= 1;
            h->steps_done += 3;
            s += 3;
            continue;
        }
        if (fused2 && h->kind == 1 && n_steps - s >= 2) {
            // two plain periodic steps in one launch: step s and s + 1
            CKL(launch_periodic_d2q9_fp32_x2(h->op, h->g, h->R, (const float *)h->d_buf[h->cur],
                                             (float *)h->d_buf[h->cur ^ 1], h->stream),
                "periodic_d2q9_x2");
            h->cur ^= 1;
            h->steps_done += 2;
            s += 2;
            continue;
        }
        if ((rc = enqueue_step(h, b, 0, 0.0, false))) return rc;
        s++;
    }
    return ERLBM_OK;
}

int erlbm_set_launch(erlbm_handle *h, int block_threads, int flags)
{
    int rc = check_handle(h);
    if (rc) return rc;
    if (block_threads != 0 && block_threads != 128 && block_threads != 256 && block_threads != 512) {
        set_error("block_threads must be 0, 128, 256 or 512%s%s", "", "");
        return ERLBM_E_INVAL;
    }
    if (flags & ~(ERLBM_LAUNCH_STREAMING_STORES | ERLBM_LAUNCH_TWO_STEP | ERLBM_LAUNCH_THREE_STEP |
                  ERLBM_LAUNCH_WIDE_STRIPS))
        return ERLBM_E_INVAL;
    if ((flags & ERLBM_LAUNCH_WIDE_STRIPS) && !(flags & ERLBM_LAUNCH_THREE_STEP)) {
        set_error("set_launch: ERLBM_LAUNCH_WIDE_STRIPS applies to ERLBM_LAUNCH_THREE_STEP%s%s", "", "");
        return ERLBM_E_INVAL;
    }
    if ((flags & ERLBM_LAUNCH_TWO_STEP) && (flags & ERLBM_LAUNCH_THREE_STEP)) {
        set_error("set_launch: at most one of ERLBM_LAUNCH_TWO_STEP and ERLBM_LAUNCH_THREE_STEP%s%s", "", "");
        return ERLBM_E_INVAL;
    }
    h->shape = block_threads | ((flags & ERLBM_LAUNCH_STREAMING_STORES) ? 0x1000 : 0) |
               ((flags & ERLBM_LAUNCH_WIDE_STRIPS) ? 0x2000 : 0);  // part of the graph key
    h->two_step = (flags & ERLBM_LAUNCH_TWO_STEP) != 0;
    h->three_step = (flags & ERLBM_LAUNCH_THREE_STEP) != 0;
    h->wide_strips = (flags & ERLBM_LAUNCH_WIDE_STRIPS) != 0;
    return ERLBM_OK;  // graphs of another shape are rebuilt on their next use (graph_key)
}

int erlbm_set_stream(erlbm_handle *h, void *stream)
{
    int rc = check_handle(h);
    if (rc) return rc;
    CK(cudaStreamSynchronize(h->stream));
    h->stream = stream ? (cudaStream_t)stream : h->own_stream;
    return ERLBM_OK;
}

int erlbm_fp64_rate(double *ops_per_s)
{
    if (!ops_per_s) return ERLBM_E_INVAL;
    if (measure_fp64_rate(ops_per_s)) return cuda_fail(cudaGetLastError(), "FP64 rate probe");
    return ERLBM_OK;
}

int erlbm_sync(erlbm_handle *h)
{
    int rc = check_handle(h);
    if (rc) return rc;
    CK(cudaStreamSynchronize(h->stream));
    return ERLBM_OK;
}

int erlbm_kinetic_energy(erlbm_handle *h, int stage, double *E)
{
    int rc = check_handle(h);
    if (rc) return rc;
    if (!E) return ERLBM_E_INVAL;
    return energy_now(h, stage, E);
}

int erlbm_max_abs_density(erlbm_handle *h, int stage, double *m, int *nonfinite)
{
    int rc = check_handle(h);
    if (rc) return rc;
    const void *buf;
    if ((rc = stage_buffer(h, stage, &buf))) return rc;
    if ((rc = node_fields(h, buf, nullptr, h->d_scr, nullptr))) return rc;
    CKL(launch_maxabs(h->d_scr, h->n_fluid, h->d_scr + h->n_fluid, h->d_out, h->stream), "maxabs");
    double r[2];
    CK(cudaMemcpyAsync(r, h->d_out, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    if (m) *m = r[0];
    if (nonfinite) *nonfinite = r[1] != 0.0;
    return ERLBM_OK;
}

int erlbm_macroscopic(erlbm_handle *h, int stage, double *rho, double *u)
{
    int rc = check_handle(h);
    if (rc) return rc;
    if ((rc = ensure_aos(h))) return rc;
    const void *buf;
    if ((rc = stage_buffer(h, stage, &buf))) return rc;
    // d_aos holds n_fluid * q >= 4 * n_fluid doubles: rho first, then u
    double *d_rho = h->d_aos, *d_u = h->d_aos + h->n_fluid;
    if ((rc = node_fields(h, buf, nullptr, rho ? d_rho : nullptr, u ? d_u : nullptr))) return rc;
    if (rho) CK(cudaMemcpyAsync(rho, d_rho, h->n_fluid * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    if (u) CK(cudaMemcpyAsync(u, d_u, 3 * h->n_fluid * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return ERLBM_OK;
}

int erlbm_run(erlbm_handle *h, int n_steps, const erlbm_bc *bc, const erlbm_checks *chk, erlbm_run_result *res)
{
    int rc = check_handle(h);
    if (rc) return rc;
    if (n_steps < 0 || !res) return ERLBM_E_INVAL;
    BCp b;
    if ((rc = validate_bc(h, bc, &b))) return rc;
    erlbm_checks c{};
    if (chk) c = *chk;
    if (c.energy_every < 0) return ERLBM_E_INVAL;
    res->label = 0;
    res->decided_step = n_steps;
    res->steps_done = 0;
    res->margin = 0.0;
    RunStatus st0{0, 0x7fffffff, 0ull};
    CK(cudaMemcpyAsync(h->d_status, &st0, sizeof(st0), cudaMemcpyHostToDevice, h->stream));
    const long long base = h->steps_done;
    const int cur0 = h->cur;
    double E0 = 0.0;
    if (c.energy_every > 0)
        if ((rc = energy_now(h, ERLBM_STAGE_POST_STREAM, &E0))) return rc;
    // Steps are enqueued in chunks ending at the next energy check; with density checks the
    // kernels stop themselves one step after a failing step, and the host reads the status
    // once per chunk.
    const int chunk = c.energy_every > 0 ? c.energy_every : 512;
    int s = 0;
    while (s < n_steps) {
        if (c.energy_every > 0 && s % c.energy_every == 0 && s > 0) {
            double E;
            if ((rc = energy_now(h, ERLBM_STAGE_POST_STREAM, &E))) return rc;
            const double r = std::isfinite(E) ? E / (c.energy_factor * E0) : INFINITY;
            if (r > res->margin) res->margin = r;
            if (E > c.energy_factor * E0 || !std::isfinite(E)) {
                res->label = 1;
                res->decided_step = s;
                res->steps_done = s;
                return ERLBM_OK;
            }
        }
        int m = chunk - (s % chunk);
        if (s + m > n_steps) m = n_steps - s;
        // keep the step numbering of the run itself in the kernels' step index
        for (int k = 0; k < m; k++) {
            h->steps_done = base + s + k;
            if ((rc = enqueue_step(h, b, c.density_check, c.density_limit, c.density_check != 0))) return rc;
        }
        h->steps_done = base + s + m;
        s += m;
        if (c.density_check) {
            RunStatus st;
            CK(cudaMemcpyAsync(&st, h->d_status, sizeof(st), cudaMemcpyDeviceToHost, h->stream));
            CK(cudaStreamSynchronize(h->stream));
            if (st.flags) {
                double mx;
                memcpy(&mx, &st.max_abs_rho_bits, sizeof(mx));
                res->label = 1;
                res->decided_step = st.decided_step - (int)base;
                res->steps_done = res->decided_step + 1;
                res->margin = (st.flags & 2) ? INFINITY : mx / c.density_limit;
                h->steps_done = base + res->steps_done;
                // launches after the failing step did nothing: the last written buffer is the one
                // of step decided_step
                h->cur = cur0 ^ (res->steps_done & 1);
                CK(cudaStreamSynchronize(h->stream));
                return ERLBM_OK;
            }
        }
    }
    if (c.density_check) {
        RunStatus st;
        CK(cudaMemcpyAsync(&st, h->d_status, sizeof(st), cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
        double mx;
        memcpy(&mx, &st.max_abs_rho_bits, sizeof(mx));
        res->margin = mx / c.density_limit;
    }
    res->steps_done = n_steps;
    CK(cudaStreamSynchronize(h->stream));
    return ERLBM_OK;
}

}  // extern "C"

// ---- fields, VTK output, error calculator --------------------------------------------------------

namespace {

// A device buffer allocated and freed in the order of one stream (no device-wide synchronisation).
struct StreamBuf {
    void *p = nullptr;
    cudaStream_t s = nullptr;
    ~StreamBuf()
    {
        if (p) cudaFreeAsync(p, s);
    }
    int alloc(size_t bytes, cudaStream_t stream)
    {
        s = stream;
        if (cudaMallocAsync(&p, bytes ? bytes : 16, stream) != cudaSuccess) {
            cudaGetLastError();
            p = nullptr;
            set_error("out of device memory for a field buffer%s%s", "", "");
            return ERLBM_E_OOM;
        }
        return ERLBM_OK;
    }
};

size_t field_values(const erlbm_handle *h, int field) { return (size_t)h->g.nbox * (field == 3 ? 1 : 3); }

// The field of the chosen stage at every box node into out (device, field_values doubles).
int field_on_device(erlbm_handle *h, int stage, int field, double *out)
{
    if (field < 1 || field > 3) {
        set_error("unknown field (1 velocity, 2 vorticity, 3 density)%s%s", "", "");
        return ERLBM_E_INVAL;
    }
    const void *buf;
    int rc = stage_buffer(h, stage, &buf);
    if (rc) return rc;
    StreamBuf vel;
    double *target = out;
    if (field == 2) {
        if ((rc = vel.alloc(field_values(h, 1) * sizeof(double), h->stream))) return rc;
        target = (double *)vel.p;
    }
    const int kind = field == 3 ? 3 : 1;
    if (h->prec == ERLBM_FP64)
        CKL(launch_box_field_fp64(h->q, h->g, (const double *)buf, kind, target, h->stream), "box_field");
    else if (h->prec == ERLBM_FP32_PAIR)
        CKL(launch_box_field_pair(h->q, h->g, (const float2 *)buf, kind, target, h->stream), "box_field");
    else
        CKL(launch_box_field_fp32(h->q, h->g, (const float *)buf, kind, target, h->stream), "box_field");
    if (field == 2) CKL(launch_vorticity(h->g, target, out, h->stream), "vorticity");
    return ERLBM_OK;
}

}  // namespace

extern "C" {

int erlbm_field(erlbm_handle *h, int stage, int field, double *out, size_t n)
{
    int rc = check_handle(h);
    if (rc) return rc;
    if (!out || field < 1 || field > 3 || n != field_values(h, field)) {
        set_error("field: out must hold nx*ny*nz (density) or 3*nx*ny*nz (velocity, vorticity) doubles%s%s", "",
                  "");
        return ERLBM_E_INVAL;
    }
    StreamBuf d;
    if ((rc = d.alloc(n * sizeof(double), h->stream))) return rc;
    if ((rc = field_on_device(h, stage, field, (double *)d.p))) return rc;
    CK(cudaMemcpyAsync(out, d.p, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return ERLBM_OK;
}

int erlbm_write_vtk(erlbm_handle *h, int stage, int field, int format, const char *path)
{
    int rc = check_handle(h);
    if (rc) return rc;
    if (!path || field < 1 || field > 3 || format < ERLBM_VTK_ASCII || format > ERLBM_VTK_BINARY_DOUBLE) {
        set_error("write_vtk: bad field, format or path%s%s", "", "");
        return ERLBM_E_INVAL;
    }
    const size_t n = field_values(h, field);
    StreamBuf d, enc;
    if ((rc = d.alloc(n * sizeof(double), h->stream))) return rc;
    if ((rc = field_on_device(h, stage, field, (double *)d.p))) return rc;
    std::vector<double> vals;
    std::vector<unsigned char> bytes;
    if (format == ERLBM_VTK_ASCII) {
        vals.resize(n);
        CK(cudaMemcpyAsync(vals.data(), d.p, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    } else {
        const size_t w = format == ERLBM_VTK_BINARY_DOUBLE ? 8 : 4;
        if ((rc = enc.alloc(n * w, h->stream))) return rc;
        CKL(launch_encode_be((const double *)d.p, (long long)n, w == 8, (unsigned char *)enc.p, h->stream), "encode");
        bytes.resize(n * w);
        CK(cudaMemcpyAsync(bytes.data(), enc.p, n * w, cudaMemcpyDeviceToHost, h->stream));
    }
    CK(cudaStreamSynchronize(h->stream));
    if (write_vtk_file(path, field, format, h->g.nx, h->g.ny, h->g.nz, vals.data(), bytes.data(), bytes.size())) {
        set_error("cannot write %s%s", path, "");
        return ERLBM_E_INVAL;
    }
    return ERLBM_OK;
}

int erlbm_velocity_error(erlbm_handle *sim, int sim_stage, erlbm_handle *ref, int ref_stage, int text_digits,
                         double *e_vec, double *e_mod)
{
    int rc = check_handle(sim);
    if (rc || (rc = check_handle(ref))) return rc;
    if (!e_vec || !e_mod || text_digits < 0 || text_digits > 17) return ERLBM_E_INVAL;
    const Geo &a = sim->g, &b = ref->g;
    if (a.nz != 1 || b.nz != 1 || b.nx % a.nx != 0 || b.ny % a.ny != 0 || b.nx / a.nx != b.ny / a.ny) {
        set_error("the reference grid must refine the simulation grid by one integer factor (nz = 1)%s%s", "", "");
        return ERLBM_E_INVAL;
    }
    if (sim->device != ref->device) {
        set_error("both lattices must live on the same GPU%s%s", "", "");
        return ERLBM_E_INVAL;
    }
    const int stride = b.nx / a.nx;
    StreamBuf vr, vs;
    if ((rc = vr.alloc(field_values(ref, 1) * sizeof(double), ref->stream))) return rc;
    if ((rc = field_on_device(ref, ref_stage, 1, (double *)vr.p))) return rc;
    CK(cudaStreamSynchronize(ref->stream));
    if ((rc = vs.alloc(field_values(sim, 1) * sizeof(double), sim->stream))) return rc;
    if ((rc = field_on_device(sim, sim_stage, 1, (double *)vs.p))) return rc;
    double sums[3];
    if (text_digits == 0) {
        StreamBuf scr;
        if ((rc = scr.alloc((3 * 1024 + 3) * sizeof(double), sim->stream))) return rc;
        double *d_out = (double *)scr.p + 3 * 1024;
        CKL(launch_velocity_error_sums((const double *)vs.p, a.nx, a.ny, (const double *)vr.p, b.nx, stride,
                                       (double *)scr.p, d_out, sim->stream),
            "velocity_error");
        CK(cudaMemcpyAsync(sums, d_out, sizeof(sums), cudaMemcpyDeviceToHost, sim->stream));
        CK(cudaStreamSynchronize(sim->stream));
    } else {
        std::vector<double> hs(field_values(sim, 1)), hr(field_values(ref, 1));
        CK(cudaMemcpyAsync(hs.data(), vs.p, hs.size() * sizeof(double), cudaMemcpyDeviceToHost, sim->stream));
        CK(cudaMemcpyAsync(hr.data(), vr.p, hr.size() * sizeof(double), cudaMemcpyDeviceToHost, sim->stream));
        CK(cudaStreamSynchronize(sim->stream));
        error_sums_host(hs.data(), a.nx, a.ny, hr.data(), b.nx, stride, text_digits, sums);
    }
    *e_mod = std::sqrt(sums[0] / sums[2]);
    *e_vec = std::sqrt(sums[1] / sums[2]);
    return ERLBM_OK;
}

}  // extern "C"
