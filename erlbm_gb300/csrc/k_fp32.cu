// k_fp32.cu -- FP32 shifted-population kernels (compiled with FMA contraction on).
//
// Besides the generic single-lattice kernels of lattice_kernels.cuh, this file holds the fused
// periodic D2Q9 kernel used for the double-shear-layer lattices (L = 512 ... 2048): one warp
// owns 128 consecutive nodes of a row, every lane four of them, so each direction plane is read
// and written with 128-bit accesses.  The pull from x - c_x needs one neighbour column per
// lane; it comes from the adjacent lane by a warp shuffle, and only the two warp-edge lanes
// issue an extra 4-byte load (an L2 hit: the neighbouring warp reads that line too).
// Algorithmic traffic is 2 * 9 * 4 = 72 bytes per lattice update.
#include "lattice_kernels.cuh"

namespace erlbm {

namespace {

constexpr unsigned FULL = 0xffffffffu;

// Pull one direction plane for the four nodes x0..x0+3 of row y (periodic in x and y).
template <int CX>
__device__ __forceinline__ float4 pull4(const float *__restrict__ row, int x0, int xl, int xr, int lane)
{
    const float4 a = __ldg(reinterpret_cast<const float4 *>(row + x0));
    if (CX == 0) return a;
    if (CX == 1) {  // values at x0-1 .. x0+2
        const float e = (lane == 0) ? __ldg(row + xl) : 0.f;
        float p = __shfl_up_sync(FULL, a.w, 1);
        if (lane == 0) p = e;
        return make_float4(p, a.x, a.y, a.z);
    }
    // CX == -1: values at x0+1 .. x0+4
    const float e = (lane == 31) ? __ldg(row + xr) : 0.f;
    float n = __shfl_down_sync(FULL, a.x, 1);
    if (lane == 31) n = e;
    return make_float4(a.y, a.z, a.w, n);
}

__device__ __forceinline__ float comp(const float4 &v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : (k == 2 ? v.z : v.w)); }

__device__ __forceinline__ void setc(float4 &v, int k, float x)
{
    if (k == 0)
        v.x = x;
    else if (k == 1)
        v.y = x;
    else if (k == 2)
        v.z = x;
    else
        v.w = x;
}

// Store of one direction plane's four nodes: plain, or streaming (evict-first: the next launch
// reads these lines back, but the lattice is larger than L2, so keeping them there only displaces
// lines still to be read in this launch).
template <bool STREAMING>
__device__ __forceinline__ void store4(float *p, const float4 &v)
{
    if (STREAMING)
        __stcs(reinterpret_cast<float4 *>(p), v);
    else
        *reinterpret_cast<float4 *>(p) = v;
}

template <int OP, int BLOCK, bool STREAMING>
__global__ void __launch_bounds__(BLOCK) k_periodic_d2q9(const float *__restrict__ src, float *__restrict__ dst, int nx,
                                                          int ny, long long plane, shifted::Coef k)
{
    const int lane = threadIdx.x & 31;
    const int wpr = nx >> 7;  // warps per row
    const long long gw = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (gw >= (long long)wpr * ny) return;  // whole warps only
    const int y = (int)(gw / wpr);
    const int xw = (int)(gw % wpr) << 7;
    const int x0 = xw + 4 * lane;
    const int ym = (y == 0) ? ny - 1 : y - 1;  // row of populations moving +y
    const int yp = (y == ny - 1) ? 0 : y + 1;  // row of populations moving -y
    const int xl = (xw == 0) ? nx - 1 : xw - 1;
    const int xr = (xw + 128 == nx) ? 0 : xw + 128;
    const long long ry = (long long)y * nx, rm = (long long)ym * nx, rp = (long long)yp * nx;

    float4 v[9];
    v[0] = pull4<0>(src + 0 * plane + ry, x0, xl, xr, lane);
    v[1] = pull4<1>(src + 1 * plane + ry, x0, xl, xr, lane);
    v[2] = pull4<-1>(src + 2 * plane + ry, x0, xl, xr, lane);
    v[3] = pull4<0>(src + 3 * plane + rm, x0, xl, xr, lane);
    v[4] = pull4<0>(src + 4 * plane + rp, x0, xl, xr, lane);
    v[5] = pull4<1>(src + 5 * plane + rm, x0, xl, xr, lane);
    v[6] = pull4<-1>(src + 6 * plane + rp, x0, xl, xr, lane);
    v[7] = pull4<1>(src + 7 * plane + rp, x0, xl, xr, lane);
    v[8] = pull4<-1>(src + 8 * plane + rm, x0, xl, xr, lane);

#pragma unroll
    for (int c = 0; c < 4; c++) {
        float g[9];
#pragma unroll
        for (int i = 0; i < 9; i++) g[i] = comp(v[i], c);
        shifted::collide9<OP>(g, k);
#pragma unroll
        for (int i = 0; i < 9; i++) setc(v[i], c, g[i]);
    }
#pragma unroll
    for (int i = 0; i < 9; i++) store4<STREAMING>(dst + i * plane + ry + x0, v[i]);
}

}  // namespace

bool periodic_d2q9_fp32_ok(const Geo &g)
{
    return g.solid == nullptr && g.nz == 1 && g.nx % 128 == 0 && g.ny >= 2 && g.plane % 4 == 0;
}

namespace {

template <int OP, int BLOCK, bool ST>
void go_periodic(const Geo &g, const shifted::Coef &k, const float *src, float *dst, cudaStream_t s)
{
    const long long warps = (long long)(g.nx / 128) * g.ny;
    const unsigned nb = (unsigned)((warps * 32 + BLOCK - 1) / BLOCK);
    k_periodic_d2q9<OP, BLOCK, ST><<<nb, BLOCK, 0, s>>>(src, dst, g.nx, g.ny, g.plane, k);
}

template <int OP>
int periodic_shape(int block, bool st, const Geo &g, const shifted::Coef &k, const float *src, float *dst,
                   cudaStream_t s)
{
    if (block == 128 && !st) go_periodic<OP, 128, false>(g, k, src, dst, s);
    else if (block == 128 && st) go_periodic<OP, 128, true>(g, k, src, dst, s);
    else if (block == 256 && !st) go_periodic<OP, 256, false>(g, k, src, dst, s);
    else if (block == 256 && st) go_periodic<OP, 256, true>(g, k, src, dst, s);
    else if (block == 512 && !st) go_periodic<OP, 512, false>(g, k, src, dst, s);
    else if (block == 512 && st) go_periodic<OP, 512, true>(g, k, src, dst, s);
    else return -1;
    return 0;
}

// Two steps per launch (temporal blocking).  A CTA owns a strip of W columns and a chunk of HC rows
// and walks down it with a rolling window: four rows of the input populations P (W + 4 columns: the
// two-step pull reaches two columns out) and four rows of the intermediate step P' (W + 2 columns),
// both in shared memory.  Per iteration two output rows j, j + 1 are made: rows j + 2, j + 3 of P
// enter the window (their global loads were issued one iteration ahead), rows j + 1, j + 2 of P' are
// collided from P, and rows j, j + 1 of the output from P'; only the output goes back to HBM.  The
// two rows of each stage are collided together as the two halves of float2 lanes (packed FP32x2
// instructions), with the same bits as the one-step kernel.  Each node is read once and written once
// per two steps, plus a margin for the window's start (four rows per chunk) and the strip edges.
template <int W>
struct X2 {
    static constexpr int T = W + 32;  // threads: W + 4 loaders, W + 2 for P', W for the output
    static constexpr int WA = W + 4;
    static constexpr int WB = W + 2;
    static constexpr size_t SMEM = (size_t)4 * 9 * (WA + WB) * sizeof(float);
};

__device__ __forceinline__ int slot4(int r) { return (r + 8) & 3; }  // rows from y0 - 8 up


template <int OP, int W>
__global__ void __launch_bounds__(X2<W>::T) k_periodic_d2q9_x2(const float *__restrict__ src, float *__restrict__ dst,
                                                               int nx, int ny, long long plane, int hc,
                                                               shifted::Coef k)
{
    constexpr int WA = X2<W>::WA, WB = X2<W>::WB;
    extern __shared__ float x2_smem[];
    float *A = x2_smem;              // [4][9][WA]
    float *B = x2_smem + 4 * 9 * WA;  // [4][9][WB]
    const int t = threadIdx.x;
    const int strips = nx / W;
    const int x0 = (blockIdx.x % strips) * W;
    const int y0 = (blockIdx.x / strips) * hc;
    const int y1 = min(y0 + hc, ny);
    int cw = x0 - 2 + t;  // this thread's column of the P window (periodic in x)
    cw = cw < 0 ? cw + nx : (cw >= nx ? cw - nx : cw);

    auto load_row = [&](int r, float v[9]) {
        const int rr = ((r % ny) + ny) % ny;
        const float *p = src + (long long)rr * nx + cw;
#pragma unroll
        for (int i = 0; i < 9; i++) v[i] = __ldg(p + i * plane);
    };
    auto put_row = [&](int r, const float v[9]) {
        float *a = A + slot4(r) * 9 * WA + t;
#pragma unroll
        for (int i = 0; i < 9; i++) a[i * WA] = v[i];
    };
    // P' rows r and r + 1 at column x0 - 1 + t, from the P window
    auto mid2 = [&](int r) {
        if (t >= WB) return;
        float2 g[9];
#pragma unroll
        for (int i = 0; i < 9; i++) {
            const int c = (t + 1) - Lat<9>::cx(i);
            g[i].x = A[(slot4(r - Lat<9>::cy(i)) * 9 + i) * WA + c];
            g[i].y = A[(slot4(r + 1 - Lat<9>::cy(i)) * 9 + i) * WA + c];
        }
        shifted::collide9x2<OP>(g, k);
        float *b0 = B + slot4(r) * 9 * WB + t, *b1 = B + slot4(r + 1) * 9 * WB + t;
#pragma unroll
        for (int i = 0; i < 9; i++) {
            b0[i * WB] = g[i].x;
            b1[i * WB] = g[i].y;
        }
    };
    // output rows r and r + 1 at column x0 + t, from the P' window
    auto out2 = [&](int r) {
        if (t >= W) return;
        float2 g[9];
#pragma unroll
        for (int i = 0; i < 9; i++) {
            const int c = (t + 1) - Lat<9>::cx(i);
            g[i].x = B[(slot4(r - Lat<9>::cy(i)) * 9 + i) * WB + c];
            g[i].y = B[(slot4(r + 1 - Lat<9>::cy(i)) * 9 + i) * WB + c];
        }
        shifted::collide9x2<OP>(g, k);
        float *d0 = dst + (long long)r * nx + x0 + t, *d1 = d0 + nx;
#pragma unroll
        for (int i = 0; i < 9; i++) {
            d0[i * plane] = g[i].x;
            d1[i * plane] = g[i].y;
        }
    };

    const bool loader = t < WA;
    float va[9], vb[9];
    // prologue: P rows y0 - 2 .. y0 + 1 and P' rows y0 - 1, y0; va, vb hold P rows y0 + 2, y0 + 3
    if (loader) {
        load_row(y0 - 2, va);
        put_row(y0 - 2, va);
        load_row(y0 - 1, va);
        put_row(y0 - 1, va);
        load_row(y0, va);
        put_row(y0, va);
        load_row(y0 + 1, va);
        put_row(y0 + 1, va);
    }
    __syncthreads();
    mid2(y0 - 1);
    if (loader) {
        load_row(y0 + 2, va);
        load_row(y0 + 3, vb);
    }
    __syncthreads();  // mid2 has read P rows y0 - 2, y0 - 1, whose slots rows y0 + 2, y0 + 3 take
    for (int j = y0; j < y1; j += 2) {
        if (loader) {
            put_row(j + 2, va);
            put_row(j + 3, vb);
            if (j + 2 < y1) {  // one iteration ahead
                load_row(j + 4, va);
                load_row(j + 5, vb);
            }
        }
        __syncthreads();
        mid2(j + 1);
        __syncthreads();
        out2(j);
    }
}


}  // namespace

// Chunk height of the two-step kernel: one wave of CTAs (resident CTAs per SM x SMs) over the
// (nx / W) x ny lattice, so that no second, partial wave runs, and even (two rows per iteration).
static int x2_chunk(int nx, int ny, int W, int resident_per_sm, int sms)
{
    const long long slots = (long long)(resident_per_sm > 0 ? resident_per_sm : 1) * (sms > 0 ? sms : 1);
    const long long strips = nx / W;
    long long hc = (ny * strips + slots - 1) / slots;
    if (hc < 8) hc = 8;
    hc += hc & 1;
    if (hc > ny) hc = ny;
    return (int)hc;
}

bool periodic_d2q9_x2_ok(const Geo &g)
{
    return periodic_d2q9_fp32_ok(g) && g.ny >= 4 && g.ny % 2 == 0;  // nx % 128 == 0 from the one-step check
}

template <int OP, int W>
static void go_x2w(const Geo &g, const shifted::Coef &k, const float *src, float *dst, cudaStream_t s)
{
    auto kern = k_periodic_d2q9_x2<OP, W>;
    // shared-memory attribute, occupancy and SM count once per device and instantiation (settings
    // are per device; concurrent first calls set the same values)
    constexpr int MAXDEV = 64;
    static int occ[MAXDEV], sms[MAXDEV];
    int dev = 0;
    cudaGetDevice(&dev);
    const int d = dev >= 0 && dev < MAXDEV ? dev : 0;
    if (occ[d] <= 0) {
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)X2<W>::SMEM);
        int o = 0, n = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, kern, X2<W>::T, X2<W>::SMEM) != cudaSuccess || o < 1)
            o = 1;
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        sms[d] = n > 0 ? n : 1;
        occ[d] = o;
    }
    const int hc = x2_chunk(g.nx, g.ny, W, occ[d], sms[d]);
    const unsigned nb = (unsigned)((g.nx / W) * ((g.ny + hc - 1) / hc));
    kern<<<nb, X2<W>::T, X2<W>::SMEM, s>>>(src, dst, g.nx, g.ny, g.plane, hc, k);
}

template <int OP>
static void go_x2(const Geo &g, const shifted::Coef &k, const float *src, float *dst, cudaStream_t s)
{
    // 128-column strips: 160-thread CTAs, five resident per SM.  On GB300 at L = 2048: 113.8 G LU/s,
    // against 110.7 with 256-column strips (two 288-thread CTAs per SM) and 110.4 with 512
    go_x2w<OP, 128>(g, k, src, dst, s);
}

// Two steps of the fused periodic D2Q9 FP32 update in one launch (periodic_d2q9_x2_ok(g) required).
int launch_periodic_d2q9_fp32_x2(int op, const Geo &g, const Relax &R, const float *src, float *dst, cudaStream_t s)
{
    if (!periodic_d2q9_x2_ok(g)) return -1;
    const shifted::Coef k = shifted::make_coef(R);
    switch (op) {
    case OP_BGK: go_x2<OP_BGK>(g, k, src, dst, s); break;
    case OP_MRT: go_x2<OP_MRT>(g, k, src, dst, s); break;
    case OP_REG: go_x2<OP_REG>(g, k, src, dst, s); break;
    case OP_EXTREG: go_x2<OP_EXTREG>(g, k, src, dst, s); break;
    default: return -1;
    }
    return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

// shape: threads per block (128, 256 or 512; 0 = 256) and bit 0x1000 for streaming stores.
int launch_periodic_d2q9_fp32(int op, const Geo &g, const Relax &R, const float *src, float *dst, cudaStream_t s,
                              int shape)
{
    if (!periodic_d2q9_fp32_ok(g)) return -1;
    const shifted::Coef k = shifted::make_coef(R);
    const int block = (shape & 0xfff) ? (shape & 0xfff) : 256;
    const bool st = (shape & 0x1000) != 0;
    int rc;
    switch (op) {
    case OP_BGK:
        rc = periodic_shape<OP_BGK>(block, st, g, k, src, dst, s);
        break;
    case OP_MRT:
        rc = periodic_shape<OP_MRT>(block, st, g, k, src, dst, s);
        break;
    case OP_REG:
        rc = periodic_shape<OP_REG>(block, st, g, k, src, dst, s);
        break;
    case OP_EXTREG:
        rc = periodic_shape<OP_EXTREG>(block, st, g, k, src, dst, s);
        break;
    default:
        return -1;
    }
    if (rc) return rc;
    return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

int launch_step_fp32(int q, int op, const Geo &g, const BCp &bc, const Relax &R, const StepArgs &a, const float *src,
                     float *dst, cudaStream_t s)
{
    return step_any<PrecShifted32>(q, op, g, bc, R, a, src, dst, s);
}

int launch_stream_only_fp32(int q, const Geo &g, const float *src, float *dst, cudaStream_t s)
{
    return stream_only_any<PrecShifted32>(q, g, src, dst, s);
}

int launch_aos_to_soa_fp32(int q, const Geo &g, long long n, const int *nof, const double *aos, float *soa,
                           cudaStream_t s)
{
    return aos_to_soa_any<PrecShifted32>(q, g, n, nof, aos, soa, s);
}

int launch_soa_to_aos_fp32(int q, const Geo &g, long long n, const int *nof, const float *soa, double *aos,
                           cudaStream_t s)
{
    return soa_to_aos_any<PrecShifted32>(q, g, n, nof, soa, aos, s);
}

int launch_node_fields_fp32(int q, const Geo &g, long long n, const int *nof, const float *buf, double *e,
                            double *rho, double *u, cudaStream_t s)
{
    return node_fields_any<PrecShifted32>(q, g, n, nof, buf, e, rho, u, s);
}

int launch_box_field_fp32(int q, const Geo &g, const float *buf, int field, double *out, cudaStream_t s)
{
    return box_field_any<PrecShifted32>(q, g, buf, field, out, s);
}


// Initial fields on the device (lattice_kernels.cuh): kind 1 = D2Q9 Taylor-Green program init,
// 4 = D3Q19 3-D Taylor-Green equilibrium, 0 = rest equilibrium.
int launch_init_fp32(int kind, int q, const Geo &g, float *buf, const double *tab, double u0, double tau, double k,
                     double rho, cudaStream_t s)
{
    return init_any<PrecShifted32>(kind, q, g, buf, tab, u0, tau, k, rho, s);
}

}  // namespace erlbm
