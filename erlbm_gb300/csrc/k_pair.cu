// k_pair.cu -- kernels of the compensated FP32 form (populations as float pairs; collide_pair.cuh).
// Compiled with --fmad=false: every float-float step is an explicitly rounded intrinsic, and the
// FP64 queries round each operation on its own.
#include "collide_pair.cuh"
#include "lattice_kernels.cuh"

namespace erlbm {
namespace {

// One step of a periodic D2Q9 lattice: pull (mode 0) or the populations in place (mode 1, the first
// step after they were set), then the compensated collision.  One node per thread.
template <int OP>
__global__ void __launch_bounds__(256) k_step_pair(const float2 *__restrict__ src, float2 *__restrict__ dst, Geo g,
                                                   int mode, pair32::CoefDS k)
{
    const long long node = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= g.nbox) return;
    int x, y, z;
    node_xyz(g, node, x, y, z);
    float2 f[9];
    gather<PrecPair32, 9>(src, g, mode, x, y, z, node, f);
    pair32::DS d[9];
#pragma unroll
    for (int i = 0; i < 9; i++) d[i] = {f[i].x, f[i].y};
    pair32::collide9<OP>(d, k);
#pragma unroll
    for (int i = 0; i < 9; i++) dst[(long long)i * g.plane + node] = make_float2(d[i].hi, d[i].lo);
}

}  // namespace

bool step_pair_ok(int q, int op, const Geo &g)
{
    return q == 9 && g.nz == 1 && g.solid == nullptr && (op == OP_BGK || op == OP_REG || op == OP_EXTREG);
}

int launch_step_pair(int q, int op, const Geo &g, const Relax &R, int mode, const float2 *src, float2 *dst,
                     cudaStream_t s)
{
    if (!step_pair_ok(q, op, g)) return -1;
    const pair32::CoefDS k = pair32::make_coef_ds(R);
    const unsigned nb = blocks_for(g.nbox, 256);
    switch (op) {
    case OP_BGK: k_step_pair<OP_BGK><<<nb, 256, 0, s>>>(src, dst, g, mode, k); break;
    case OP_REG: k_step_pair<OP_REG><<<nb, 256, 0, s>>>(src, dst, g, mode, k); break;
    default: k_step_pair<OP_EXTREG><<<nb, 256, 0, s>>>(src, dst, g, mode, k); break;
    }
    return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

int launch_stream_only_pair(int q, const Geo &g, const float2 *src, float2 *dst, cudaStream_t s)
{
    return stream_only_any<PrecPair32>(q, g, src, dst, s);
}

int launch_aos_to_soa_pair(int q, const Geo &g, long long n, const int *nof, const double *aos, float2 *soa,
                           cudaStream_t s)
{
    return aos_to_soa_any<PrecPair32>(q, g, n, nof, aos, soa, s);
}

int launch_soa_to_aos_pair(int q, const Geo &g, long long n, const int *nof, const float2 *soa, double *aos,
                           cudaStream_t s)
{
    return soa_to_aos_any<PrecPair32>(q, g, n, nof, soa, aos, s);
}

int launch_node_fields_pair(int q, const Geo &g, long long n, const int *nof, const float2 *buf, double *e,
                            double *rho, double *u, cudaStream_t s)
{
    return node_fields_any<PrecPair32>(q, g, n, nof, buf, e, rho, u, s);
}

int launch_box_field_pair(int q, const Geo &g, const float2 *buf, int field, double *out, cudaStream_t s)
{
    return box_field_any<PrecPair32>(q, g, buf, field, out, s);
}

}  // namespace erlbm
