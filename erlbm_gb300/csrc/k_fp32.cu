// k_fp32.cu -- FP32 shifted-population kernels (compiled with FMA contraction on).
//
// Besides the generic single-lattice kernels of lattice_kernels.cuh, this file holds the fused
// periodic D2Q9 kernel used for the double-shear-layer lattices (L = 512 ... 2048): one warp
// owns 128 consecutive nodes of a row, every lane four of them, so each direction plane is read
// and written with 128-bit accesses.  The pull from x - c_x needs one neighbour column per
// lane; it comes from the adjacent lane by a warp shuffle, and only the two warp-edge lanes
// issue an extra 4-byte load (an L2 hit: the neighbouring warp reads that line too).
// Algorithmic traffic is 2 * 9 * 4 = 72 bytes per lattice update.  The two- and three-step kernels
// (k_periodic_d2q9_x2s, k_periodic_d2q9_x3s, and k_periodic_d2q9_x3a over column pairs) advance every
// node by two or three steps per launch in independent warp strips: 36 and 24 bytes per lattice update.
#include <atomic>

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

// Two steps per launch with warp strips: each warp owns XS_W = 30 output columns and a chunk of rows
// and walks down it on its own (no shared memory, no block barrier).  Lane l holds column
// xs - 1 + l.  A population that comes from the next column over reaches a lane through a warp
// shuffle; lanes 0 and 31, whose neighbour column lies outside the warp, load those three populations
// themselves.  All 32 lanes collide the intermediate step P' (columns xs - 1 .. xs + 30); lanes 1 .. 30
// collide and store the output.  Per iteration two output rows j, j + 1 are made from P' rows j - 1 ..
// j + 2, and P' rows j + 1, j + 2 from P rows j .. j + 3, of which rows j + 2, j + 3 were loaded one
// iteration ahead.  Every value is carried in registers already moved to the lane that pulls it, and
// only the populations a later row still needs are kept: the cy = +1 group of the older row and the
// cy = 0 and cy = +1 groups of the newer one.  The two rows of each stage are collided together in
// packed FP32x2 lanes with the same bits as the one-step kernel.
constexpr int XS_W = 30;
constexpr unsigned XS_FULL = 0xffffffffu;

template <int OP>
__global__ void __launch_bounds__(128) k_periodic_d2q9_x2s(const float *__restrict__ src, float *__restrict__ dst,
                                                          int nx, int ny, long long plane, int hc, int strips,
                                                          int n_warps, shifted::Coef k)
{
    const int lane = threadIdx.x & 31;
    const int wid = (int)blockIdx.x * (int)(blockDim.x >> 5) + (int)(threadIdx.x >> 5);
    if (wid >= n_warps) return;  // the whole warp leaves together
    const int xs = (wid % strips) * XS_W;
    const int y0 = (wid / strips) * hc;
    const int y1 = min(y0 + hc, ny);
    int c = xs - 1 + lane;  // in [-1, nx + 29]
    const bool store = lane >= 1 && lane <= XS_W && c < nx;
    c = c < 0 ? c + nx : (c >= nx ? c - nx : c);
    // halo: lane 0 pulls populations 1, 5, 7 (cx = +1) from column xs - 2, lane 31 pulls 2, 6, 8
    // (cx = -1) from column xs + 31
    const bool halo = lane == 0 || lane == 31;
    int hcol = lane == 0 ? xs - 2 : xs + 31;
    hcol = hcol < 0 ? hcol + nx : (hcol >= nx ? hcol - nx : hcol);
    const long long h0 = hcol + (lane == 0 ? 1 : 2) * plane, h1 = hcol + (lane == 0 ? 5 : 6) * plane,
                    h2 = hcol + (lane == 0 ? 7 : 8) * plane;

    auto load = [&](int r, float v[9], float h[3]) {
        r = r < 0 ? r + ny : (r >= ny ? r - ny : r);
        const float *p = src + (long long)r * nx;
#pragma unroll
        for (int i = 0; i < 9; i++) v[i] = __ldg(p + c + i * plane);
        if (halo) {
            h[0] = __ldg(p + h0);
            h[1] = __ldg(p + h1);
            h[2] = __ldg(p + h2);
        }
    };
    // a[i] = P(column - cx_i) of the loaded row
    auto align = [&](const float v[9], const float h[3], float a[9]) {
        a[0] = v[0];
        a[3] = v[3];
        a[4] = v[4];
        float u;
        u = __shfl_up_sync(XS_FULL, v[1], 1);
        a[1] = lane == 0 ? h[0] : u;
        u = __shfl_up_sync(XS_FULL, v[5], 1);
        a[5] = lane == 0 ? h[1] : u;
        u = __shfl_up_sync(XS_FULL, v[7], 1);
        a[7] = lane == 0 ? h[2] : u;
        u = __shfl_down_sync(XS_FULL, v[2], 1);
        a[2] = lane == 31 ? h[0] : u;
        u = __shfl_down_sync(XS_FULL, v[6], 1);
        a[6] = lane == 31 ? h[1] : u;
        u = __shfl_down_sync(XS_FULL, v[8], 1);
        a[8] = lane == 31 ? h[2] : u;
    };
    // the same for both rows of a collided pair; lanes 0 and 31 get values no stored output uses
    auto align2 = [&](float2 g[9]) {
        g[1].x = __shfl_up_sync(XS_FULL, g[1].x, 1);
        g[1].y = __shfl_up_sync(XS_FULL, g[1].y, 1);
        g[5].x = __shfl_up_sync(XS_FULL, g[5].x, 1);
        g[5].y = __shfl_up_sync(XS_FULL, g[5].y, 1);
        g[7].x = __shfl_up_sync(XS_FULL, g[7].x, 1);
        g[7].y = __shfl_up_sync(XS_FULL, g[7].y, 1);
        g[2].x = __shfl_down_sync(XS_FULL, g[2].x, 1);
        g[2].y = __shfl_down_sync(XS_FULL, g[2].y, 1);
        g[6].x = __shfl_down_sync(XS_FULL, g[6].x, 1);
        g[6].y = __shfl_down_sync(XS_FULL, g[6].y, 1);
        g[8].x = __shfl_down_sync(XS_FULL, g[8].x, 1);
        g[8].y = __shfl_down_sync(XS_FULL, g[8].y, 1);
    };
    // the pulled populations of rows m (x) and m + 1 (y) from the aligned rows m - 1 (o: cy = +1
    // group), m (n: cy = 0 and +1 groups), m + 1 (all) and m + 2 (cy = -1 group)
    auto gather = [](float2 g[9], const float o[9], const float n[9], const float p[9], const float q[9]) {
        g[3] = make_float2(o[3], n[3]);
        g[5] = make_float2(o[5], n[5]);
        g[8] = make_float2(o[8], n[8]);
        g[0] = make_float2(n[0], p[0]);
        g[1] = make_float2(n[1], p[1]);
        g[2] = make_float2(n[2], p[2]);
        g[4] = make_float2(p[4], q[4]);
        g[6] = make_float2(p[6], q[6]);
        g[7] = make_float2(p[7], q[7]);
    };

    float va[9], vb[9], ha[3] = {0.f, 0.f, 0.f}, hb[3] = {0.f, 0.f, 0.f};
    float aA[9], aB[9], aC[9], aD[9];  // aligned P rows
    float bA[9], bB[9];                // aligned P' rows j - 1 (cy = +1 group) and j (cy = 0, +1 groups)
    float2 g[9];
    // prologue: P rows y0 - 2 .. y0 + 1, P' rows y0 - 1, y0
    load(y0 - 2, va, ha);
    load(y0 - 1, vb, hb);
    align(va, ha, aA);
    align(vb, hb, aB);
    load(y0, va, ha);
    load(y0 + 1, vb, hb);
    align(va, ha, aC);
    align(vb, hb, aD);
    load(y0 + 2, va, ha);
    load(y0 + 3, vb, hb);
    gather(g, aA, aB, aC, aD);
    shifted::collide9x2<OP>(g, k);
    align2(g);
#pragma unroll
    for (int i = 0; i < 9; i++) {
        bA[i] = g[i].x;
        bB[i] = g[i].y;
        aA[i] = aC[i];
        aB[i] = aD[i];
    }
    for (int j = y0; j < y1; j += 2) {
        align(va, ha, aC);  // P row j + 2
        align(vb, hb, aD);  // P row j + 3
        if (j + 2 < y1) {   // one iteration ahead
            load(j + 4, va, ha);
            load(j + 5, vb, hb);
        }
        gather(g, aA, aB, aC, aD);  // P' rows j + 1, j + 2
        shifted::collide9x2<OP>(g, k);
        align2(g);
        float nA[9], nB[9];
#pragma unroll
        for (int i = 0; i < 9; i++) {
            nA[i] = g[i].x;
            nB[i] = g[i].y;
        }
        gather(g, bA, bB, nA, nB);  // output rows j, j + 1
        shifted::collide9x2<OP>(g, k);
        if (store) {
            float *d0 = dst + (long long)j * nx + c, *d1 = d0 + nx;
#pragma unroll
            for (int i = 0; i < 9; i++) {
                d0[i * plane] = g[i].x;
                d1[i * plane] = g[i].y;
            }
        }
#pragma unroll
        for (int i = 0; i < 9; i++) {
            aA[i] = aC[i];
            aB[i] = aD[i];
            bA[i] = nA[i];
            bB[i] = nB[i];
        }
    }
}

// Three steps per launch in the same warp-strip form, with strips of 28 output columns: lane l holds
// column xs - 2 + l; the first stage P' is valid in every lane (lanes 0 and 31 load their halo
// populations), the second P'' in lanes 1 .. 30, the output in lanes 2 .. 29.  Per iteration the
// output rows j, j + 1 come from P'' rows j - 1 .. j + 2, P'' rows j + 1, j + 2 from P' rows j .. j + 3,
// and P' rows j + 2, j + 3 from P rows j + 1 .. j + 4, of which rows j + 3, j + 4 were loaded one
// iteration ahead.  Each node is read and written once per three steps (24 bytes per update).
constexpr int X3_W = 28;

// Four resident CTAs per SM: the register cap (128) spills 8 bytes, and 16 warps per SM instead of
// 12 run 4 % faster on GB300 (158.6 against 151.9 G LU/s at L = 2048).
template <int OP>
__global__ void __launch_bounds__(128, 4) k_periodic_d2q9_x3s(const float *__restrict__ src, float *__restrict__ dst,
                                                          int nx, int ny, long long plane, int hc, int strips,
                                                          int n_warps, shifted::Coef k)
{
    const int lane = threadIdx.x & 31;
    const int wid = (int)blockIdx.x * (int)(blockDim.x >> 5) + (int)(threadIdx.x >> 5);
    if (wid >= n_warps) return;
    const int xs = (wid % strips) * X3_W;
    const int y0 = (wid / strips) * hc;
    const int y1 = min(y0 + hc, ny);
    int c = xs - 2 + lane;  // in [-2, nx + 28]
    const bool store = lane >= 2 && lane <= X3_W + 1 && c < nx;
    c = c < 0 ? c + nx : (c >= nx ? c - nx : c);
    const bool halo = lane == 0 || lane == 31;
    int hcol = lane == 0 ? xs - 3 : xs + 30;
    hcol = hcol < 0 ? hcol + nx : (hcol >= nx ? hcol - nx : hcol);
    const long long h0 = hcol + (lane == 0 ? 1 : 2) * plane, h1 = hcol + (lane == 0 ? 5 : 6) * plane,
                    h2 = hcol + (lane == 0 ? 7 : 8) * plane;
    auto load = [&](int r, float v[9], float h[3]) {
        r = r < 0 ? r + ny : (r >= ny ? r - ny : r);
        const float *p = src + (long long)r * nx;
#pragma unroll
        for (int i = 0; i < 9; i++) v[i] = __ldg(p + c + i * plane);
        if (halo) {
            h[0] = __ldg(p + h0);
            h[1] = __ldg(p + h1);
            h[2] = __ldg(p + h2);
        }
    };
    auto align = [&](const float v[9], const float h[3], float a[9]) {
        a[0] = v[0];
        a[3] = v[3];
        a[4] = v[4];
        float u;
        u = __shfl_up_sync(XS_FULL, v[1], 1);
        a[1] = lane == 0 ? h[0] : u;
        u = __shfl_up_sync(XS_FULL, v[5], 1);
        a[5] = lane == 0 ? h[1] : u;
        u = __shfl_up_sync(XS_FULL, v[7], 1);
        a[7] = lane == 0 ? h[2] : u;
        u = __shfl_down_sync(XS_FULL, v[2], 1);
        a[2] = lane == 31 ? h[0] : u;
        u = __shfl_down_sync(XS_FULL, v[6], 1);
        a[6] = lane == 31 ? h[1] : u;
        u = __shfl_down_sync(XS_FULL, v[8], 1);
        a[8] = lane == 31 ? h[2] : u;
    };
    auto align2 = [&](float2 g[9]) {
        g[1].x = __shfl_up_sync(XS_FULL, g[1].x, 1);
        g[1].y = __shfl_up_sync(XS_FULL, g[1].y, 1);
        g[5].x = __shfl_up_sync(XS_FULL, g[5].x, 1);
        g[5].y = __shfl_up_sync(XS_FULL, g[5].y, 1);
        g[7].x = __shfl_up_sync(XS_FULL, g[7].x, 1);
        g[7].y = __shfl_up_sync(XS_FULL, g[7].y, 1);
        g[2].x = __shfl_down_sync(XS_FULL, g[2].x, 1);
        g[2].y = __shfl_down_sync(XS_FULL, g[2].y, 1);
        g[6].x = __shfl_down_sync(XS_FULL, g[6].x, 1);
        g[6].y = __shfl_down_sync(XS_FULL, g[6].y, 1);
        g[8].x = __shfl_down_sync(XS_FULL, g[8].x, 1);
        g[8].y = __shfl_down_sync(XS_FULL, g[8].y, 1);
    };
    auto gather = [](float2 g[9], const float o[9], const float n[9], const float p[9], const float q[9]) {
        g[3] = make_float2(o[3], n[3]);
        g[5] = make_float2(o[5], n[5]);
        g[8] = make_float2(o[8], n[8]);
        g[0] = make_float2(n[0], p[0]);
        g[1] = make_float2(n[1], p[1]);
        g[2] = make_float2(n[2], p[2]);
        g[4] = make_float2(p[4], q[4]);
        g[6] = make_float2(p[6], q[6]);
        g[7] = make_float2(p[7], q[7]);
    };
    auto split = [](const float2 g[9], float x[9], float y[9]) {
#pragma unroll
        for (int i = 0; i < 9; i++) {
            x[i] = g[i].x;
            y[i] = g[i].y;
        }
    };

    float va[9], vb[9], ha[3] = {0.f, 0.f, 0.f}, hb[3] = {0.f, 0.f, 0.f};
    float aA[9], aB[9], aC[9], aD[9];  // aligned P rows
    float bA[9], bB[9];                // aligned P' rows (carried)
    float cA[9], cB[9];                // aligned P'' rows (carried)
    float2 g[9];
    // prologue: P rows y0 - 3 .. y0 + 2; P' rows y0 - 2 .. y0 + 1; P'' rows y0 - 1, y0
    {
        float p0[9], p1[9], p2[9], p3[9], p4[9], p5[9];
        load(y0 - 3, va, ha);
        load(y0 - 2, vb, hb);
        align(va, ha, p0);
        align(vb, hb, p1);
        load(y0 - 1, va, ha);
        load(y0, vb, hb);
        align(va, ha, p2);
        align(vb, hb, p3);
        load(y0 + 1, va, ha);
        load(y0 + 2, vb, hb);
        align(va, ha, p4);
        align(vb, hb, p5);
        load(y0 + 3, va, ha);
        load(y0 + 4, vb, hb);
        float q0[9], q1[9], q2[9], q3[9];
        gather(g, p0, p1, p2, p3);  // P' rows y0 - 2, y0 - 1
        shifted::collide9x2<OP>(g, k);
        align2(g);
        split(g, q0, q1);
        gather(g, p2, p3, p4, p5);  // P' rows y0, y0 + 1
        shifted::collide9x2<OP>(g, k);
        align2(g);
        split(g, q2, q3);
        gather(g, q0, q1, q2, q3);  // P'' rows y0 - 1, y0
        shifted::collide9x2<OP>(g, k);
        align2(g);
        split(g, cA, cB);
#pragma unroll
        for (int i = 0; i < 9; i++) {
            aA[i] = p4[i];
            aB[i] = p5[i];
            bA[i] = q2[i];
            bB[i] = q3[i];
        }
    }
    for (int j = y0; j < y1; j += 2) {
        align(va, ha, aC);  // P row j + 3
        align(vb, hb, aD);  // P row j + 4
        if (j + 2 < y1) {
            load(j + 5, va, ha);
            load(j + 6, vb, hb);
        }
        float nA[9], nB[9], mA[9], mB[9];
        gather(g, aA, aB, aC, aD);  // P' rows j + 2, j + 3
        shifted::collide9x2<OP>(g, k);
        align2(g);
        split(g, nA, nB);
        gather(g, bA, bB, nA, nB);  // P'' rows j + 1, j + 2
        shifted::collide9x2<OP>(g, k);
        align2(g);
        split(g, mA, mB);
        gather(g, cA, cB, mA, mB);  // output rows j, j + 1
        shifted::collide9x2<OP>(g, k);
        if (store) {
            float *d0 = dst + (long long)j * nx + c, *d1 = d0 + nx;
#pragma unroll
            for (int i = 0; i < 9; i++) {
                d0[i * plane] = g[i].x;
                d1[i * plane] = g[i].y;
            }
        }
#pragma unroll
        for (int i = 0; i < 9; i++) {
            aA[i] = aC[i];
            aB[i] = aD[i];
            bA[i] = nA[i];
            bB[i] = nB[i];
            cA[i] = mA[i];
            cB[i] = mB[i];
        }
    }
}


// Three steps per launch over column pairs (k_periodic_d2q9_x3a).  Lane l holds the columns xs - 2 + 2l
// and xs - 1 + 2l of a 64-column strip as the two halves of a float2, so each packed FP32x2 operation
// of the collision works on two neighbouring nodes of one row and every operand pair is formed where it
// is produced.  The strip walks down its chunk one row per iteration:
//   - the first stage P' is valid in all 64 columns, P'' in columns 1 .. 62, the output in columns
//     2 .. 61: 60 output columns per 64 (the x3s strips: 28 per 32);
//   - the x pull of a collided row's direction with c_x = +1 takes the left half from the lane below
//     (one shuffle) and the right half from the lane's own left half, and the reverse for c_x = -1;
//   - the y pull of row r takes the c_y = +1 group (3, 5, 8) from row r - 1, the c_y = 0 group (0, 1,
//     2) from row r and the c_y = -1 group (4, 6, 7) from row r + 1.
// The two later stages carry the c_y = +1 groups of their two newest input rows and the c_y = 0 group
// of the newest one in registers; the groups of a row stay in the register slot they arrive in (three
// slots per group, used in turn), so the loop body is unrolled three times and no group is copied
// between iterations.  Per iteration P' row j + 2, P'' row j + 1 and output row j are collided; the
// first four iterations of a chunk are its prologue, in which only the stages whose inputs exist run.
// Bit-identical to three one-step launches: every node is collided by collide9x2 as by collide9.
constexpr int XP_W = 60;   // output columns per strip
constexpr int XP_SPAN = 3; // rows per unrolled group: one turn of the three register slots

template <int I>
struct IntC {
    static constexpr int value = I;
};

// Its first-stage inputs are brought in ahead by asynchronous copies into a per-warp ring of shared
// memory (XA_DEPTH slots), not into registers, which keeps the kernel at 122 registers (16 warps per
// SM) and two rows of loads in flight.  A slot holds, for each of the
// nine populations, the 68 columns xs - 4 .. xs + 63 of the input row its c_y group comes from (c_y =
// +1: row r - 1, 0: row r, -1: row r + 1 for P' row r), as 153 aligned 16-byte pieces spread over the
// lanes.  The x pull is then a shifted shared-memory read: a lane's nodes sit at slot columns 2l + 2,
// 2l + 3; c_x = +1 populations are read at 2l + 1, 2l + 2 and c_x = -1 ones at 2l + 3, 2l + 4, which
// also covers the strip's edge columns, so the first stage needs no shuffle, select or edge load.  The
// copies for P' row r + 2 are issued while row r is collided.
constexpr int XA_DEPTH = 3;                // ring slots (two rows of copies in flight)
constexpr int XA_ROW = 68;                 // columns per population row in a slot
constexpr int XA_SLOT = 9 * XA_ROW;        // floats per slot
constexpr int XA_PIECES = 9 * XA_ROW / 4;  // 16-byte pieces per slot (153)
constexpr size_t XA_SMEM_PER_WARP = (size_t)XA_DEPTH * XA_SLOT * sizeof(float);

__device__ __forceinline__ void cp_async16(float *dst_smem, const float *src)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst_smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

template <int OP, int MINB>
__global__ void __launch_bounds__(128, MINB) k_periodic_d2q9_x3a(const float *__restrict__ src, float *__restrict__ dst,
                                                                int nx, int ny, int plane, int hc, int strips,
                                                                int n_warps, shifted::Coef k)
{
    extern __shared__ __align__(16) float xa_smem[];
    const int lane = threadIdx.x & 31;
    const int wib = (int)(threadIdx.x >> 5);
    const int wid = (int)blockIdx.x * (int)(blockDim.x >> 5) + wib;
    if (wid >= n_warps) return;  // the whole warp leaves together
    float *ring = xa_smem + (size_t)wib * (XA_DEPTH * XA_SLOT);
    const int xs = (wid % strips) * XP_W;
    const int y0 = (wid / strips) * hc;
    const int y1 = min(y0 + hc, ny);
    int c = xs - 2 + 2 * lane;  // even, in [-2, nx + 60]
    const bool store = lane >= 1 && lane <= 30 && c < nx;
    c = c < 0 ? c + nx : (c >= nx ? c - nx : c);
    auto wrap = [&](int r) { return r < 0 ? r + ny : (r >= ny ? r - ny : r); };

    // this lane's pieces q = lane + 32 m (q < 153): population q / 17, columns xs - 4 + 4 (q % 17) .. + 3
    // (a piece never straddles the periodic seam: nx and the piece start are multiples of 4), offset
    // within the population's plane, and the row of its c_y group (0: r - 1, 1: r, 2: r + 1)
    int off[5];
    unsigned rowsel = 0;  // 2 bits per piece
#pragma unroll
    for (int m = 0; m < 5; m++) {
        const int q = lane + 32 * m;
        const int pop = q / 17;
        int col = xs - 4 + 4 * (q % 17);
        col = col < 0 ? col + nx : (col >= nx ? col - nx : col);
        off[m] = pop * plane + col;
        const unsigned sel = (pop == 3 || pop == 5 || pop == 8) ? 0u : ((pop <= 2) ? 1u : 2u);
        rowsel |= sel << (2 * m);
    }
    // copies of P' row r's inputs into a slot
    auto issue = [&](int r, float *slot) {
        const int ra = wrap(r - 1) * nx, rb = wrap(r) * nx, rc = wrap(r + 1) * nx;
#pragma unroll
        for (int m = 0; m < 5; m++) {
            if (m == 4 && lane + 128 >= XA_PIECES) break;
            const unsigned sel = (rowsel >> (2 * m)) & 3u;
            const int ro = sel == 0 ? ra : (sel == 1 ? rb : rc);
            cp_async16(slot + 4 * (lane + 32 * m), src + (unsigned)(ro + off[m]));
        }
        cp_async_commit();
    };
    // first-stage input of the lane's two nodes from a slot (x pull by the read offsets)
    auto read = [&](const float *S, float2 g[9]) {
        const int b = 2 * lane;
        g[0] = *reinterpret_cast<const float2 *>(S + 0 * XA_ROW + b + 2);
        g[3] = *reinterpret_cast<const float2 *>(S + 3 * XA_ROW + b + 2);
        g[4] = *reinterpret_cast<const float2 *>(S + 4 * XA_ROW + b + 2);
        g[1] = make_float2(S[1 * XA_ROW + b + 1], S[1 * XA_ROW + b + 2]);
        g[5] = make_float2(S[5 * XA_ROW + b + 1], S[5 * XA_ROW + b + 2]);
        g[7] = make_float2(S[7 * XA_ROW + b + 1], S[7 * XA_ROW + b + 2]);
        g[2] = make_float2(S[2 * XA_ROW + b + 3], S[2 * XA_ROW + b + 4]);
        g[6] = make_float2(S[6 * XA_ROW + b + 3], S[6 * XA_ROW + b + 4]);
        g[8] = make_float2(S[8 * XA_ROW + b + 3], S[8 * XA_ROW + b + 4]);
    };
    auto pull_p = [&](float2 v) { return make_float2(__shfl_up_sync(XS_FULL, v.y, 1), v.x); };
    auto pull_m = [&](float2 v) { return make_float2(v.y, __shfl_down_sync(XS_FULL, v.x, 1)); };

    float2 s1[2][3][3], s0[2][3][3];
    float2 g[9], nm[3];

    // one iteration at rotation phase T (P' row j + 2 from ring slot (T + 1) % 3; the copies for P' row
    // j + 4 go to slot T, which every lane finished reading one iteration earlier)
    auto step = [&](auto T, auto C1, auto C2, int j) {
        constexpr int t = decltype(T)::value % 3;
        constexpr int a = t, b = (t + 1) % 3, n = (t + 2) % 3;
        constexpr bool c1 = decltype(C1)::value, c2 = decltype(C2)::value;
        cp_async_wait<XA_DEPTH - 2>();
        __syncwarp();
        read(ring + ((t + 1) % 3) * XA_SLOT, g);
        issue(j + 4, ring + t * XA_SLOT);
#pragma unroll
        for (int s = 0; s < 3; s++) {
            if (s == 1 && !c1) break;
            if (s == 2 && !c2) break;
            if (s > 0) {
                g[3] = s1[s - 1][a][0];
                g[5] = s1[s - 1][a][1];
                g[8] = s1[s - 1][a][2];
                g[0] = s0[s - 1][b][0];
                g[1] = s0[s - 1][b][1];
                g[2] = s0[s - 1][b][2];
                g[4] = nm[0];
                g[6] = nm[1];
                g[7] = nm[2];
            }
            shifted::collide9x2<OP>(g, k);
            if (s == 2) {
                if (store && j < y1) {
                    float *d = dst + (long long)j * nx + c;
#pragma unroll
                    for (int i = 0; i < 9; i++) *reinterpret_cast<float2 *>(d + (long long)i * plane) = g[i];
                }
            } else {
                s1[s][n][0] = g[3];
                s1[s][n][1] = pull_p(g[5]);
                s1[s][n][2] = pull_m(g[8]);
                s0[s][n][0] = g[0];
                s0[s][n][1] = pull_p(g[1]);
                s0[s][n][2] = pull_m(g[2]);
                nm[0] = g[4];
                nm[1] = pull_m(g[6]);
                nm[2] = pull_p(g[7]);
            }
        }
    };
    using F = IntC<0>;
    using N = IntC<1>;
    // P' rows y0 - 2 and y0 - 1 go to slots 0 and 1; the prologue runs phases 2, 0, 1, 2
    issue(y0 - 2, ring);
    issue(y0 - 1, ring + XA_SLOT);
    step(IntC<2>{}, F{}, F{}, y0 - 4);
    step(IntC<0>{}, F{}, F{}, y0 - 3);
    step(IntC<1>{}, N{}, F{}, y0 - 2);
    step(IntC<2>{}, N{}, F{}, y0 - 1);
    for (int j = y0; j < y1; j += XP_SPAN) {
        step(IntC<0>{}, N{}, N{}, j);
        step(IntC<1>{}, N{}, N{}, j + 1);
        step(IntC<2>{}, N{}, N{}, j + 2);
    }
    cp_async_wait_all();  // the copies issued for rows past the chunk land before the warp leaves
}

}  // namespace

bool periodic_d2q9_x2_ok(const Geo &g)
{
    return periodic_d2q9_fp32_ok(g) && g.ny >= 4 && g.ny % 2 == 0;  // nx % 128 == 0 from the one-step check
}

// Two-step launch: 128-thread CTAs of four independent warps, and rows per chunk such that one wave
// of resident warps covers the ceil(nx / 30) x (ny / hc) warp strips (no second, partial wave).
template <int OP>
static void go_x2(const Geo &g, const shifted::Coef &k, const float *src, float *dst, cudaStream_t s)
{
    auto kern = k_periodic_d2q9_x2s<OP>;
    // resident warps per device, found once per device and instantiation (handles on several host
    // threads may launch concurrently; they store the same value)
    constexpr int MAXDEV = 64;
    static std::atomic<int> warps_cache[MAXDEV];
    int dev = 0;
    cudaGetDevice(&dev);
    const int d = dev >= 0 && dev < MAXDEV ? dev : 0;
    int resident = warps_cache[d].load(std::memory_order_relaxed);
    if (resident <= 0) {
        int o = 0, n = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, kern, 128, 0) != cudaSuccess || o < 1) o = 1;
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        resident = o * 4 * (n > 0 ? n : 1);
        warps_cache[d].store(resident, std::memory_order_relaxed);
    }
    const int strips = (g.nx + XS_W - 1) / XS_W;
    const long long slots = resident;
    long long chunks = slots / strips;
    if (chunks < 1) chunks = 1;
    long long hc = (g.ny + chunks - 1) / chunks;
    if (hc < 8) hc = 8;
    hc += hc & 1;
    if (hc > g.ny) hc = g.ny;
    const int n_warps = strips * (int)((g.ny + hc - 1) / hc);
    const unsigned nb = (unsigned)((n_warps + 3) / 4);
    kern<<<nb, 128, 0, s>>>(src, dst, g.nx, g.ny, g.plane, (int)hc, strips, n_warps, k);
}

// Three-step launch: as go_x2, over ceil(nx / 28) strips.
template <int OP>
static void go_x3(const Geo &g, const shifted::Coef &k, const float *src, float *dst, cudaStream_t s)
{
    auto kern = k_periodic_d2q9_x3s<OP>;
    constexpr int MAXDEV = 64;
    static std::atomic<int> warps_cache[MAXDEV];
    int dev = 0;
    cudaGetDevice(&dev);
    const int d = dev >= 0 && dev < MAXDEV ? dev : 0;
    int resident = warps_cache[d].load(std::memory_order_relaxed);
    if (resident <= 0) {
        int o = 0, n = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, kern, 128, 0) != cudaSuccess || o < 1) o = 1;
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        resident = o * 4 * (n > 0 ? n : 1);
        warps_cache[d].store(resident, std::memory_order_relaxed);
    }
    const int strips = (g.nx + X3_W - 1) / X3_W;
    const long long slots = resident;
    long long chunks = slots / strips;
    if (chunks < 1) chunks = 1;
    long long hc = (g.ny + chunks - 1) / chunks;
    if (hc < 8) hc = 8;
    hc += hc & 1;
    if (hc > g.ny) hc = g.ny;
    const int n_warps = strips * (int)((g.ny + hc - 1) / hc);
    kern<<<(unsigned)((n_warps + 3) / 4), 128, 0, s>>>(src, dst, g.nx, g.ny, g.plane, (int)hc, strips, n_warps, k);
}

// Three-step launch over column pairs: ceil(nx / 60) strips, chunks of whole unrolled groups, as many
// chunks per strip as one wave of resident warps holds (no second, partial wave).
constexpr int XA_MINB = 4;  // resident 128-thread CTAs per SM (122 registers, no spills)

template <int OP>
static void go_x3a(const Geo &g, const shifted::Coef &k, const float *src, float *dst, cudaStream_t s)
{
    auto kern = k_periodic_d2q9_x3a<OP, XA_MINB>;
    const size_t smem = 4 * XA_SMEM_PER_WARP;
    constexpr int MAXDEV = 64;
    static std::atomic<int> warps_cache[MAXDEV];
    int dev = 0;
    cudaGetDevice(&dev);
    const int d = dev >= 0 && dev < MAXDEV ? dev : 0;
    int resident = warps_cache[d].load(std::memory_order_relaxed);
    if (resident <= 0) {
        int o = 0, n = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, kern, 128, smem) != cudaSuccess || o < 1) o = 1;
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        resident = o * 4 * (n > 0 ? n : 1);
        warps_cache[d].store(resident, std::memory_order_relaxed);
    }
    const int strips = (g.nx + XP_W - 1) / XP_W;
    long long chunks = resident / strips;
    if (chunks < 1) chunks = 1;
    long long hc = (g.ny + chunks - 1) / chunks;
    hc = (hc + XP_SPAN - 1) / XP_SPAN * XP_SPAN;
    if (hc < 2 * XP_SPAN) hc = 2 * XP_SPAN;
    const int n_warps = strips * (int)((g.ny + hc - 1) / hc);
    kern<<<(unsigned)((n_warps + 3) / 4), 128, smem, s>>>(src, dst, g.nx, g.ny, (int)g.plane, (int)hc, strips, n_warps,
                                                         k);
}

bool periodic_d2q9_x3a_ok(const Geo &g)
{
    // 64-column strips need ny >= 16; the nine planes are addressed with 32-bit offsets
    return periodic_d2q9_fp32_ok(g) && g.ny >= 16 && g.nx >= 128 && 9 * g.plane < (1LL << 31);
}

// Three steps of the fused periodic D2Q9 FP32 update in one launch (periodic_d2q9_x2_ok(g) required;
// wide = the column-pair kernel, which needs periodic_d2q9_x3a_ok(g)).
int launch_periodic_d2q9_fp32_x3(int op, const Geo &g, const Relax &R, const float *src, float *dst, cudaStream_t s,
                                 bool wide)
{
    if (!periodic_d2q9_x2_ok(g) || (wide && !periodic_d2q9_x3a_ok(g))) return -1;
    const shifted::Coef k = shifted::make_coef(R);
    if (wide) {
        switch (op) {
        case OP_BGK: go_x3a<OP_BGK>(g, k, src, dst, s); break;
        case OP_MRT: go_x3a<OP_MRT>(g, k, src, dst, s); break;
        case OP_REG: go_x3a<OP_REG>(g, k, src, dst, s); break;
        case OP_EXTREG: go_x3a<OP_EXTREG>(g, k, src, dst, s); break;
        default: return -1;
        }
        return cudaGetLastError() == cudaSuccess ? 0 : -3;
    }
    switch (op) {
    case OP_BGK: go_x3<OP_BGK>(g, k, src, dst, s); break;
    case OP_MRT: go_x3<OP_MRT>(g, k, src, dst, s); break;
    case OP_REG: go_x3<OP_REG>(g, k, src, dst, s); break;
    case OP_EXTREG: go_x3<OP_EXTREG>(g, k, src, dst, s); break;
    default: return -1;
    }
    return cudaGetLastError() == cudaSuccess ? 0 : -3;
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

namespace {

// One step of a D2Q9 lattice with solids and boundary planes, FP32-shifted.  Two kinds of blocks:
//  - fix-up blocks (the first n_fix_blocks): one thread per node that needs the generic per-node update
//    (pull with bounce-back, the planes, the collision): the fluid nodes next to a solid (the list
//    `fix`, n_fix entries) and the nodes of the inlet column, the outlet column and the open y row;
//  - fused blocks (the rest): k_periodic_d2q9's update, a warp per 128 columns of a row, four per lane,
//    float4 accesses, x neighbours by shuffle.  It is the right update for every fluid node whose eight
//    neighbours are fluid and which lies on no plane.  A segment whose stencil holds a solid (segflag)
//    or which a plane crosses stores only its other nodes (nodeflag marks the nodes next to a solid).
// The fix-up blocks come first, so their scattered loads overlap the fused stream instead of
// lengthening its last wave.  No node is written by both kinds, and a node on a plane that is also
// next to a solid is computed twice with the same result.  A solid node's storage is written by the
// fused update but never read (the pull of a fluid node that faces a solid takes its own opposite
// population), so what it holds does not matter.  Both updates give the generic kernel's bits.
template <int OP>
__global__ void __launch_bounds__(256) k_d2q9_hybrid(const float *__restrict__ src, float *__restrict__ dst, Geo g,
                                                     BCp bc, CollParams prm, const uint8_t *__restrict__ segflag,
                                                     const uint8_t *__restrict__ nodeflag,
                                                     const int *__restrict__ fix, int n_fix, int n_fix_blocks)
{
    const int nx = g.nx, ny = g.ny;
    const long long plane = g.plane;
    if ((int)blockIdx.x < n_fix_blocks) {
        int t = (int)(blockIdx.x * blockDim.x + threadIdx.x);
        int x, y;
        if (t < n_fix) {
            const int node = fix[t];
            y = node / nx;
            x = node - y * nx;
        } else {
            t -= n_fix;
            if (bc.inlet_x >= 0) {
                if (t < ny) { x = bc.inlet_x; y = t; goto have; }
                t -= ny;
            }
            if (bc.outlet_x >= 0) {
                if (t < ny) { x = bc.outlet_x; y = t; goto have; }
                t -= ny;
            }
            if (bc.open_y >= 0 && t < nx) { x = t; y = bc.open_y; goto have; }
            return;
        }
    have:
        const long long node = (long long)y * nx + x;
        if (g.solid != nullptr && g.solid[node]) return;
        float f[9];
        state_after_planes<PrecShifted32, 9>(src, g, bc, 0, x, y, 0, node, f);
        shifted::collide<9, OP>(f, prm.k);
#pragma unroll
        for (int i = 0; i < 9; i++) dst[(long long)i * plane + node] = f[i];
        return;
    }
    const int lane = threadIdx.x & 31;
    const int wpr = nx >> 7;
    const long long gw = ((long long)(blockIdx.x - n_fix_blocks) * blockDim.x + threadIdx.x) >> 5;
    if (gw >= (long long)wpr * ny) return;  // whole warps only
    const int y = (int)(gw / wpr);
    const int xw = (int)(gw % wpr) << 7;
    const int x0 = xw + 4 * lane;
    const int ym = (y == 0) ? ny - 1 : y - 1;
    const int yp = (y == ny - 1) ? 0 : y + 1;
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
        float gg[9];
#pragma unroll
        for (int i = 0; i < 9; i++) gg[i] = comp(v[i], c);
        shifted::collide9<OP>(gg, prm.k);
#pragma unroll
        for (int i = 0; i < 9; i++) setc(v[i], c, gg[i]);
    }
    const bool planes = (bc.inlet_x >= xw && bc.inlet_x < xw + 128) || (bc.outlet_x >= xw && bc.outlet_x < xw + 128) ||
                        y == bc.open_y;
    if (!planes && !(segflag != nullptr && segflag[gw])) {
#pragma unroll
        for (int i = 0; i < 9; i++) *reinterpret_cast<float4 *>(dst + i * plane + ry + x0) = v[i];
        return;
    }
    const uchar4 nf = nodeflag != nullptr ? *reinterpret_cast<const uchar4 *>(nodeflag + ry + x0) : make_uchar4(0, 0, 0, 0);
    const bool open_row = y == bc.open_y;
    const bool k0 = !(nf.x || open_row || x0 == bc.inlet_x || x0 == bc.outlet_x);
    const bool k1 = !(nf.y || open_row || x0 + 1 == bc.inlet_x || x0 + 1 == bc.outlet_x);
    const bool k2 = !(nf.z || open_row || x0 + 2 == bc.inlet_x || x0 + 2 == bc.outlet_x);
    const bool k3 = !(nf.w || open_row || x0 + 3 == bc.inlet_x || x0 + 3 == bc.outlet_x);
#pragma unroll
    for (int i = 0; i < 9; i++) {
        float *p = dst + i * plane + ry + x0;
        if (k0 && k1 && k2 && k3) {
            *reinterpret_cast<float4 *>(p) = v[i];
        } else {
            if (k0) p[0] = v[i].x;
            if (k1) p[1] = v[i].y;
            if (k2) p[2] = v[i].z;
            if (k3) p[3] = v[i].w;
        }
    }
}

}  // namespace

bool d2q9_hybrid_ok(const Geo &g)
{
    // node indices of the fix-up list and the fix-up thread index are 32-bit
    return g.nz == 1 && g.nx % 128 == 0 && g.ny >= 2 && g.plane % 4 == 0 && g.nbox + 3LL * (g.nx + g.ny) < (1LL << 31);
}

// Solid flags of a D2Q9 box for k_d2q9_hybrid (host).  segflags: ny * nx / 128 bytes, one per fused
// warp in launch order, 1 where the 128-column segment's pull stencil holds a solid node.  nodeflags:
// nx * ny bytes, 1 where one of the node's eight neighbours (periodic wrap) is solid; the fluid nodes
// among those are the kernel's fix-up list.
void d2q9_segment_flags(const Geo &g, const uint8_t *solid, uint8_t *flags, uint8_t *nodeflags)
{
    for (int y = 0; y < g.ny; y++)
        for (int x = 0; x < g.nx; x++) {
            uint8_t f = 0;
            for (int dy = -1; dy <= 1; dy++)
                for (int dx = -1; dx <= 1; dx++) {
                    if (!dx && !dy) continue;
                    const int xx = (x + dx + g.nx) % g.nx, yy = (y + dy + g.ny) % g.ny;
                    f |= solid[(size_t)yy * g.nx + xx] ? 1 : 0;
                }
            nodeflags[(size_t)y * g.nx + x] = f;
        }
    const int wpr = g.nx / 128;
    for (int y = 0; y < g.ny; y++)
        for (int w = 0; w < wpr; w++) {
            uint8_t f = 0;
            for (int dy = -1; dy <= 1 && !f; dy++) {
                const int yy = (y + dy + g.ny) % g.ny;
                for (int x = w * 128 - 1; x <= w * 128 + 128 && !f; x++) {
                    const int xx = (x + g.nx) % g.nx;
                    f = solid[(size_t)yy * g.nx + xx] ? 1 : 0;
                }
            }
            flags[(size_t)y * wpr + w] = f;
        }
}

int launch_step_fp32_hybrid(int op, const Geo &g, const BCp &bc, const Relax &R, const float *src, float *dst,
                            const uint8_t *segflag, const uint8_t *nodeflag, const int *fix, int n_fix, cudaStream_t s)
{
    if (!d2q9_hybrid_ok(g) || n_fix < 0) return -1;
    CollParams prm;
    prm.R = R;
    prm.k = shifted::make_coef(R);
    const long long warps = (long long)(g.nx / 128) * g.ny;
    const long long n_generic =
        (long long)n_fix + (bc.inlet_x >= 0 ? g.ny : 0) + (bc.outlet_x >= 0 ? g.ny : 0) + (bc.open_y >= 0 ? g.nx : 0);
    const long long fix_blocks = (n_generic + 255) / 256;
    const long long nb = fix_blocks + (warps * 32 + 255) / 256;
    if (nb > 0x7fffffffLL) return -1;
    const int fb = (int)fix_blocks;
    switch (op) {
    case OP_BGK: k_d2q9_hybrid<OP_BGK><<<(unsigned)nb, 256, 0, s>>>(src, dst, g, bc, prm, segflag, nodeflag, fix, n_fix, fb); break;
    case OP_MRT: k_d2q9_hybrid<OP_MRT><<<(unsigned)nb, 256, 0, s>>>(src, dst, g, bc, prm, segflag, nodeflag, fix, n_fix, fb); break;
    case OP_REG: k_d2q9_hybrid<OP_REG><<<(unsigned)nb, 256, 0, s>>>(src, dst, g, bc, prm, segflag, nodeflag, fix, n_fix, fb); break;
    case OP_EXTREG:
        k_d2q9_hybrid<OP_EXTREG><<<(unsigned)nb, 256, 0, s>>>(src, dst, g, bc, prm, segflag, nodeflag, fix, n_fix, fb);
        break;
    default: return -1;
    }
    return cudaGetLastError() == cudaSuccess ? 0 : -3;
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
