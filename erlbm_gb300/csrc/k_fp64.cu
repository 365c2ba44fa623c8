// k_fp64.cu -- plain FP64 kernels.  This translation unit is compiled with --fmad=false so that
// every multiply and add is rounded on its own, as in the reference's GCC -std=c++17 build.
#include "lattice_kernels.cuh"

namespace erlbm {

int launch_step_fp64(int q, int op, const Geo &g, const BCp &bc, const Relax &R, const StepArgs &a, const double *src,
                     double *dst, cudaStream_t s)
{
    return step_any<PrecExact64>(q, op, g, bc, R, a, src, dst, s);
}

int launch_stream_only_fp64(int q, const Geo &g, const double *src, double *dst, cudaStream_t s)
{
    return stream_only_any<PrecExact64>(q, g, src, dst, s);
}

int launch_aos_to_soa_fp64(int q, const Geo &g, long long n, const int *nof, const double *aos, double *soa,
                           cudaStream_t s)
{
    return aos_to_soa_any<PrecExact64>(q, g, n, nof, aos, soa, s);
}

int launch_soa_to_aos_fp64(int q, const Geo &g, long long n, const int *nof, const double *soa, double *aos,
                           cudaStream_t s)
{
    return soa_to_aos_any<PrecExact64>(q, g, n, nof, soa, aos, s);
}

int launch_node_fields_fp64(int q, const Geo &g, long long n, const int *nof, const double *buf, double *e,
                            double *rho, double *u, cudaStream_t s)
{
    return node_fields_any<PrecExact64>(q, g, n, nof, buf, e, rho, u, s);
}

int launch_box_field_fp64(int q, const Geo &g, const double *buf, int field, double *out, cudaStream_t s)
{
    return box_field_any<PrecExact64>(q, g, buf, field, out, s);
}

// ------------------------------------------------------------------------------------------------
// Reductions (FP64; deterministic)
// ------------------------------------------------------------------------------------------------

namespace {

// Serial sum in index order: the reference's kinectic_energy loop (Other_functions.cpp:100-115).
__global__ void k_sum_serial(const double *__restrict__ x, long long n, double *out)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double s = 0;
    for (long long i = 0; i < n; i++) s = s + x[i];
    *out = s;
}

constexpr int RB = 256;   // threads per reduction block
constexpr int RG = 1024;  // reduction blocks (fixed, so the tree shape does not depend on the GPU)

__global__ void __launch_bounds__(RB) k_sum_partial(const double *__restrict__ x, long long n, double *part)
{
    __shared__ double sh[RB];
    double s = 0;
    for (long long i = (long long)blockIdx.x * RB + threadIdx.x; i < n; i += (long long)RG * RB) s += x[i];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = RB / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void __launch_bounds__(RB) k_sum_final(const double *__restrict__ part, double *out)
{
    __shared__ double sh[RB];
    double s = 0;
    for (int i = threadIdx.x; i < RG; i += RB) s += part[i];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = RB / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sh[0];
}

__global__ void __launch_bounds__(RB) k_maxabs_partial(const double *__restrict__ x, long long n, double *part)
{
    __shared__ double sm[RB];
    __shared__ int snf[RB];
    double m = 0;
    int nf = 0;
    for (long long i = (long long)blockIdx.x * RB + threadIdx.x; i < n; i += (long long)RG * RB) {
        const double v = x[i];
        if (!isfinite(v))
            nf = 1;
        else
            m = fmax(m, fabs(v));
    }
    sm[threadIdx.x] = m;
    snf[threadIdx.x] = nf;
    __syncthreads();
    for (int o = RB / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            sm[threadIdx.x] = fmax(sm[threadIdx.x], sm[threadIdx.x + o]);
            snf[threadIdx.x] |= snf[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = sm[0];
        part[2 * blockIdx.x + 1] = snf[0] ? 1.0 : 0.0;
    }
}

__global__ void k_maxabs_final(const double *__restrict__ part, double *out)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double m = 0, nf = 0;
    for (int i = 0; i < RG; i++) {
        m = fmax(m, part[2 * i]);
        nf = fmax(nf, part[2 * i + 1]);
    }
    out[0] = m;
    out[1] = nf;
}

}  // namespace

int launch_sum(const double *x, long long n, long long serial_limit, double *scratch, double *out, cudaStream_t s)
{
    if (n <= serial_limit) {
        k_sum_serial<<<1, 32, 0, s>>>(x, n, out);
    } else {
        k_sum_partial<<<RG, RB, 0, s>>>(x, n, scratch);
        k_sum_final<<<1, RB, 0, s>>>(scratch, out);
    }
    return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

int launch_maxabs(const double *x, long long n, double *scratch, double *out, cudaStream_t s)
{
    k_maxabs_partial<<<RG, RB, 0, s>>>(x, n, scratch);
    k_maxabs_final<<<1, 32, 0, s>>>(scratch, out);
    return cudaGetLastError() == cudaSuccess ? 0 : -3;
}


// Initial fields on the device (lattice_kernels.cuh): kind 1 = D2Q9 Taylor-Green program init,
// 4 = D3Q19 3-D Taylor-Green equilibrium, 0 = rest equilibrium.
int launch_init_fp64(int kind, int q, const Geo &g, double *buf, const double *tab, double u0, double tau, double k,
                     double rho, cudaStream_t s)
{
    return init_any<PrecExact64>(kind, q, g, buf, tab, u0, tau, k, rho, s);
}

}  // namespace erlbm

// ------------------------------------------------------------------------------------------------
// FP64 add / multiply issue rate (the roofline of the exact path, which issues them unfused)
// ------------------------------------------------------------------------------------------------

namespace erlbm {
namespace {

constexpr int RATE_CHAINS = 8;

// Eight independent multiply-then-add chains per thread; with --fmad=false each is one DMUL and one
// DADD.  The values stay bounded (x -> a x + b with a < 1); the final test keeps the work alive.
__global__ void __launch_bounds__(256) k_fp64_rate(double *out, int iters, double a, double b)
{
    double x[RATE_CHAINS];
#pragma unroll
    for (int k = 0; k < RATE_CHAINS; k++) x[k] = 1.0 + 1e-9 * (double)(threadIdx.x + 37 * k);
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < RATE_CHAINS; k++) x[k] = x[k] * a + b;
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < RATE_CHAINS; k++) s = s + x[k];
    if (s == -1.0 && out) out[blockIdx.x] = s;  // never true: every x stays near 1
}

}  // namespace

// FP64 operations (each DADD and DMUL counted once, per thread) per second over one full wave of
// resident CTAs, timed with events on a private stream after one warm-up launch.
int measure_fp64_rate(double *ops_per_s)
{
    int dev = 0, sms = 0, occ = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_fp64_rate, 256, 0);
    if (e != cudaSuccess) return -3;
    if (occ < 1) occ = 1;
    const int grid = sms * occ, iters = 4096;
    cudaStream_t s = nullptr;
    cudaEvent_t a = nullptr, b = nullptr;
    int rc = -3;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) == cudaSuccess && cudaEventCreate(&a) == cudaSuccess &&
        cudaEventCreate(&b) == cudaSuccess) {
        k_fp64_rate<<<grid, 256, 0, s>>>(nullptr, iters / 8, 0.999999, 1e-6);
        cudaEventRecord(a, s);
        k_fp64_rate<<<grid, 256, 0, s>>>(nullptr, iters, 0.999999, 1e-6);
        cudaEventRecord(b, s);
        float ms = 0.f;
        if (cudaEventSynchronize(b) == cudaSuccess && cudaEventElapsedTime(&ms, a, b) == cudaSuccess && ms > 0.f) {
            *ops_per_s = (double)grid * 256.0 * iters * RATE_CHAINS * 2.0 / (ms * 1e-3);
            rc = 0;
        }
    }
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    if (s) cudaStreamDestroy(s);
    return rc == 0 && cudaGetLastError() == cudaSuccess ? 0 : -3;
}

}  // namespace erlbm
