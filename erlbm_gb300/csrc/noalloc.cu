// noalloc.cu -- erlbm_batch_run_noalloc: batched runs for callers that cannot allocate device memory.
//
// Some callers of this library must not allocate GPU memory themselves or let a library do it:
// code that owns every byte of the device through its own allocator (a host framework handing out
// device buffers), loops that may not take the cost or the implicit synchronisation of cudaMalloc /
// cudaFree, or code whose memory plan is fixed in advance.  erlbm_batch_run allocates its per-call
// scratch (run table, work counter, trig tables) with cudaMalloc; this entry point keeps that scratch
// in one file-scope device array instead, and takes the runs and the results as device pointers
// that the caller already owns.  It calls no cudaMalloc, cudaFree or other allocating routine.
//
// The array is NOALLOC_SCRATCH_BYTES (about 1.2 MB) on every GPU that loads the library, for as
// long as the process lives.  Host code must not use its name as a device address: the address is
// taken with cudaGetSymbolAddress by the first call on a device (and again after that device's
// context was replaced, e.g. by cudaDeviceReset) and passed to the kernels.
#include <cuda.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/erlbm_gb300.h"
#include "abi_internal.h"
#include "batch_kernels.cuh"
#include "kernels_api.h"

using namespace erlbm;

namespace {

// Scratch layout (bytes): work counter | sin/cos tables (2 x 4096 doubles) | refused-run flags |
// prepared runs.
constexpr size_t OFF_COUNTER = 0;
constexpr size_t OFF_TAB = 256;
constexpr int MAX_SIDE = 4096;
constexpr size_t OFF_FLAGS = OFF_TAB + 2 * MAX_SIDE * sizeof(double);
constexpr size_t OFF_RUNS = OFF_FLAGS + (size_t)ERLBM_NOALLOC_MAX_RUNS;
constexpr size_t NOALLOC_SCRATCH_BYTES = OFF_RUNS + (size_t)ERLBM_NOALLOC_MAX_RUNS * sizeof(BatchRun);
static_assert(OFF_RUNS % 256 == 0, "runs must stay aligned");

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

std::mutex g_mu;
constexpr int MAX_DEVICES = 64;
struct ScratchSlot {
    void *addr;
    unsigned long long ctx_id;  // context the address belongs to (0: not looked up yet)
};
ScratchSlot g_scratch[MAX_DEVICES] = {};

// Identity of the current context (0 when none is current yet).  The driver API is reached through
// the runtime's entry-point query, so the library does not link libcuda itself.
int current_context_id(unsigned long long *id)
{
    using GetCurrent = CUresult (*)(CUcontext *);
    using GetId = CUresult (*)(CUcontext, unsigned long long *);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    if (!get_current || !get_id) {
        cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSuccess, q2 = cudaDriverEntryPointSuccess;
        void *a = nullptr, *b = nullptr;
        cudaError_t e1 = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &q1);
        cudaError_t e2 = cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &q2);
        if (e1 != cudaSuccess || e2 != cudaSuccess || q1 != cudaDriverEntryPointSuccess ||
            q2 != cudaDriverEntryPointSuccess || !a || !b) {
            set_error("the driver's context queries (cuCtxGetCurrent, cuCtxGetId) are unavailable%s%s", "", "");
            return ERLBM_E_CUDA;
        }
        get_current = (GetCurrent)a;
        get_id = (GetId)b;
    }
    CUcontext ctx = nullptr;
    *id = 0;
    if (get_current(&ctx) != CUDA_SUCCESS) {
        set_error("cuCtxGetCurrent failed in erlbm_batch_run_noalloc%s%s", "", "");
        return ERLBM_E_CUDA;
    }
    if (ctx && get_id(ctx, id) != CUDA_SUCCESS) {
        set_error("cuCtxGetId failed in erlbm_batch_run_noalloc%s%s", "", "");
        return ERLBM_E_CUDA;
    }
    return ERLBM_OK;
}

// Device address of the scratch array on the current device.  Looked up by the first call on a
// device (cudaGetSymbolAddress, with that device current; it also brings up the runtime's context if
// none is current), and again if the current context is not the one the address was taken in.
int scratch_address(unsigned char **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    if (dev < 0 || dev >= MAX_DEVICES) {
        set_error("device index %s beyond the supported range%s", std::to_string(dev).c_str(), "");
        return ERLBM_E_UNSUPPORTED;
    }
    unsigned long long id = 0;
    int rc = current_context_id(&id);
    if (rc) return rc;
    std::lock_guard<std::mutex> lk(g_mu);
    ScratchSlot &slot = g_scratch[dev];
    if (!slot.addr || id == 0 || slot.ctx_id != id) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress");
        if ((rc = current_context_id(&id))) return rc;
        slot.addr = p;
        slot.ctx_id = id;
    }
    *out = (unsigned char *)slot.addr;
    return ERLBM_OK;
}

// Turns the caller's run descriptions (device memory) into the kernel's prepared runs, in the
// caller's order.  A run with refused parameters becomes an empty run (no steps) and is flagged, so
// that its result can be marked afterwards (status 8).
__global__ void k_prepare_runs(const erlbm_run_spec *__restrict__ specs, int n, int q, BatchRun *__restrict__ runs,
                               uint8_t *__restrict__ refused)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const erlbm_run_spec s = specs[i];
    BatchRun r;
    memset(&r, 0, sizeof(r));
    const bool ok = (s.op == ERLBM_OP_BGK || s.op == ERLBM_OP_REG || s.op == ERLBM_OP_EXTREG ||
                     (s.op == ERLBM_OP_MRT && q == 9)) && s.tau > 0 &&
                    isfinite(s.tau) && isfinite(s.tau_nh) && s.tau_nh != 0 && s.n_steps >= 0;
    r.R = make_relax(ok ? s.tau : 1.0, ok ? s.tau_nh : 1.0, ok ? s.op : ERLBM_OP_EXTREG);
    r.k = shifted::make_coef(r.R);
    r.u0 = s.u0;
    r.n_steps = ok ? s.n_steps : 0;
    r.op = ok ? s.op : ERLBM_OP_EXTREG;
    r.out = i;
    runs[i] = r;
    refused[i] = ok ? 0 : 1;
}

__global__ void k_mark_refused(const uint8_t *__restrict__ refused, int n, BatchResult *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && refused[i]) out[i].status = 8;
}

}  // namespace

extern "C" int erlbm_batch_run_noalloc(const erlbm_batch_desc *d, int n_runs, const erlbm_run_spec *runs,
                                       erlbm_batch_result *out, void *stream)
{
    int rc = check_desc(d);
    if (rc) return rc;
    if (n_runs < 0 || n_runs > ERLBM_NOALLOC_MAX_RUNS) {
        set_error("erlbm_batch_run_noalloc takes at most %s runs per call%s",
                  std::to_string(ERLBM_NOALLOC_MAX_RUNS).c_str(), "");
        return ERLBM_E_INVAL;
    }
    if (d->init == ERLBM_INIT_AOS) {
        set_error("erlbm_batch_run_noalloc starts runs from ERLBM_INIT_REST or ERLBM_INIT_TG_MAP only%s%s", "", "");
        return ERLBM_E_UNSUPPORTED;
    }
    if (n_runs == 0) return ERLBM_OK;
    if (!runs || !out) return ERLBM_E_INVAL;
    unsigned char *scr = nullptr;
    if ((rc = scratch_address(&scr))) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    int *counter = (int *)(scr + OFF_COUNTER);
    double *tab = (double *)(scr + OFF_TAB);
    BatchRun *prepared = (BatchRun *)(scr + OFF_RUNS);
    uint8_t *refused = scr + OFF_FLAGS;

    BatchGeo g;
    memset(&g, 0, sizeof(g));
    g.nx = d->nx;
    g.ny = d->ny;
    g.nb = d->nx * d->ny;
    g.solid = d->solid;  // a device pointer here
    g.inlet_x = d->inlet_x;
    g.outlet_x = d->outlet_x;
    g.rho0 = d->rho0;
    g.energy_every = d->energy_every;
    g.energy_factor = d->energy_factor;
    g.density_check = d->density_check;
    g.density_limit = d->density_limit;
    g.init = d->init;
    density_bounds(g);
    cudaError_t e;
    if (d->init == ERLBM_INIT_TG_MAP) {
        // The same tables erlbm_batch_run builds, copied from host memory.  A pageable copy cannot be
        // recorded into a graph, so a stream under capture is refused here rather than left with a
        // broken capture.
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if ((e = cudaStreamIsCapturing(s, &cs)) != cudaSuccess) return cuda_fail(e, "cudaStreamIsCapturing");
        if (cs != cudaStreamCaptureStatusNone) {
            set_error("erlbm_batch_run_noalloc with ERLBM_INIT_TG_MAP copies its tables from host memory and "
                      "cannot run on a stream under capture%s%s", "", "");
            return ERLBM_E_UNSUPPORTED;
        }
        const int n = d->nx > d->ny ? d->nx : d->ny;
        const double L = (double)d->nx;
        double h[2 * MAX_SIDE];
        for (int x = 0; x < n; x++) {
            h[x] = sin(2. * M_PI * (double)x / L);
            h[n + x] = cos(2. * M_PI * (double)x / L);
        }
        if ((e = cudaMemcpyAsync(tab, h, 2 * n * sizeof(double), cudaMemcpyHostToDevice, s)) != cudaSuccess)
            return cuda_fail(e, "noalloc tables");
        g.sinx = tab;
        g.cosx = tab + n;
    }
    // the array keeps the previous call's contents: the work counter must start at zero
    if ((e = cudaMemsetAsync(counter, 0, sizeof(int), s)) != cudaSuccess) return cuda_fail(e, "noalloc counter");
    k_prepare_runs<<<(n_runs + 255) / 256, 256, 0, s>>>(runs, n_runs, d->q, prepared, refused);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "noalloc prepare");
    LaunchShape sh;
    if ((rc = pick_shape(d->precision, d->q, g.nb, d->slots, n_runs, &sh))) return rc;
    const int lrc = d->precision == ERLBM_FP64
                        ? launch_batch_fp64(d->q, sh.npt, g, prepared, n_runs, counter, (BatchResult *)out, nullptr,
                                            sh.grid, sh.block, sh.smem, sh.dbl, s)
                        : launch_batch_fp32(d->q, sh.npt, g, prepared, n_runs, counter, (BatchResult *)out, nullptr,
                                            sh.grid, sh.block, sh.smem, sh.dbl, s);
    if (lrc == -1) {
        set_error("no batched kernel for this lattice shape%s%s", "", "");
        return ERLBM_E_UNSUPPORTED;
    }
    if (lrc) return cuda_fail(cudaGetLastError(), "noalloc batched launch");
    k_mark_refused<<<(n_runs + 255) / 256, 256, 0, s>>>(refused, n_runs, (BatchResult *)out);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "noalloc results");
    return ERLBM_OK;
}
