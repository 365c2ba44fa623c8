// fields.cu -- the reference's field outputs and its error calculator, on the device.
//
//   vorticity()                 LBM_functions.cpp:3761-3872
//   rec_velocity / rec_vorticity / rec_density (ASCII)        LBM_functions.cpp:4218, 4302, 4416
//   rec_velocity_bin / rec_vorticity_bin / rec_density_bin    LBM_functions.cpp:4979, 5061, 5179
//     with the header and big-endian helpers of :4795-4883
//   tools/error_calculator.cpp:60-105 (E_vec, E_mod)
//
// The fields are computed where the populations live; only the finished field (or its encoded
// bytes) crosses to the host.  Compiled with --fmad=false: the vorticity differences and the error
// terms round like the reference's GCC build.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <thread>
#include <vector>

#include "kernels_api.h"

namespace erlbm {

namespace {

__device__ __forceinline__ long long wrap_index(int x, int y, int z, const Geo &g)
{
    return (long long)x + (long long)g.nx * ((long long)y + (long long)g.ny * z);
}

// vort = curl u by central differences of the neighbours' velocities, periodic wrap, a solid
// neighbour counting as u = 0; solid nodes are written as 0.
__global__ void __launch_bounds__(256) k_vorticity(Geo g, const double *__restrict__ v, double *__restrict__ w)
{
    const long long node = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (node >= g.nbox) return;
    if (g.solid != nullptr && g.solid[node]) {
        w[3 * node] = w[3 * node + 1] = w[3 * node + 2] = 0.0;
        return;
    }
    const int x = (int)(node % g.nx);
    const int y = (int)((node / g.nx) % g.ny);
    const int z = (int)(node / ((long long)g.nx * g.ny));
    const double *a = v + 3 * wrap_index((x + 1) % g.nx, y, z, g);
    const double *b = v + 3 * wrap_index((x - 1 + g.nx) % g.nx, y, z, g);
    const double *c = v + 3 * wrap_index(x, (y + 1) % g.ny, z, g);
    const double *d = v + 3 * wrap_index(x, (y - 1 + g.ny) % g.ny, z, g);
    const double *e = v + 3 * wrap_index(x, y, (z + 1) % g.nz, g);
    const double *h = v + 3 * wrap_index(x, y, (z - 1 + g.nz) % g.nz, g);
    const double dvz_y = (c[2] - d[2]) / 2.0, dvy_z = (e[1] - h[1]) / 2.0;
    const double dvx_z = (e[0] - h[0]) / 2.0, dvz_x = (a[2] - b[2]) / 2.0;
    const double dvy_x = (a[1] - b[1]) / 2.0, dvx_y = (c[0] - d[0]) / 2.0;
    w[3 * node] = dvz_y - dvy_z;
    w[3 * node + 1] = dvx_z - dvz_x;
    w[3 * node + 2] = dvy_x - dvx_y;
}

__global__ void __launch_bounds__(256) k_encode_be(const double *__restrict__ in, long long n, int as_double,
                                                   unsigned char *__restrict__ out)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (as_double) {
        const unsigned long long u = (unsigned long long)__double_as_longlong(in[i]);
        const unsigned hi = (unsigned)(u >> 32), lo = (unsigned)u;
        // bytes of u from the most significant one: swap each half, then the halves
        const unsigned long long be =
            ((unsigned long long)__byte_perm(lo, 0, 0x0123) << 32) | (unsigned long long)__byte_perm(hi, 0, 0x0123);
        reinterpret_cast<unsigned long long *>(out)[i] = be;
    } else {
        const unsigned u = __float_as_uint(__double2float_rn(in[i]));
        reinterpret_cast<unsigned *>(out)[i] = __byte_perm(u, 0, 0x0123);
    }
}

constexpr int EB = 256;   // threads per block of the error sums
constexpr int EG = 1024;  // blocks (fixed, so the tree does not depend on the GPU)

__device__ __forceinline__ void tree3(double (*sh)[EB], double a, double b, double c)
{
    sh[0][threadIdx.x] = a;
    sh[1][threadIdx.x] = b;
    sh[2][threadIdx.x] = c;
    __syncthreads();
    for (int o = EB / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o)
            for (int k = 0; k < 3; k++) sh[k][threadIdx.x] = sh[k][threadIdx.x] + sh[k][threadIdx.x + o];
        __syncthreads();
    }
}

__global__ void __launch_bounds__(EB) k_error_partial(const double *__restrict__ vs, int nx, int ny,
                                                      const double *__restrict__ vr, int nx_ref, int stride,
                                                      double *__restrict__ part)
{
    __shared__ double sh[3][EB];
    double s_dif = 0.0, s_vec = 0.0, s_ur = 0.0;
    const long long n = (long long)nx * ny;
    for (long long i = (long long)blockIdx.x * EB + threadIdx.x; i < n; i += (long long)EG * EB) {
        const int x = (int)(i % nx), y = (int)(i / nx);
        const double *c = vs + 3 * i;
        const double *r = vr + 3 * ((long long)x * stride + (long long)y * stride * nx_ref);
        const double u_r = sqrt(r[0] * r[0] + r[1] * r[1]);
        const double u_s = sqrt(c[0] * c[0] + c[1] * c[1]);
        s_dif = s_dif + (u_s - u_r) * (u_s - u_r);
        s_vec = s_vec + (c[0] - r[0]) * (c[0] - r[0]) + (c[1] - r[1]) * (c[1] - r[1]);
        s_ur = s_ur + u_r * u_r;
    }
    tree3(sh, s_dif, s_vec, s_ur);
    if (threadIdx.x == 0)
        for (int k = 0; k < 3; k++) part[k * EG + blockIdx.x] = sh[k][0];
}

__global__ void __launch_bounds__(EB) k_error_final(const double *__restrict__ part, double *__restrict__ out)
{
    __shared__ double sh[3][EB];
    double a[3];
    for (int k = 0; k < 3; k++) {
        a[k] = 0.0;
        for (int j = threadIdx.x; j < EG; j += EB) a[k] = a[k] + part[k * EG + j];
    }
    tree3(sh, a[0], a[1], a[2]);
    if (threadIdx.x == 0)
        for (int k = 0; k < 3; k++) out[k] = sh[k][0];
}

unsigned blocks(long long n) { return (unsigned)((n + 255) / 256); }

}  // namespace

int launch_vorticity(const Geo &g, const double *vel, double *vor, cudaStream_t s)
{
    k_vorticity<<<blocks(g.nbox), 256, 0, s>>>(g, vel, vor);
    return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

int launch_encode_be(const double *in, long long n, int as_double, unsigned char *out, cudaStream_t s)
{
    if (n == 0) return 0;
    k_encode_be<<<blocks(n), 256, 0, s>>>(in, n, as_double, out);
    return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

int launch_velocity_error_sums(const double *vel, int nx, int ny, const double *vel_ref, int nx_ref, int stride,
                               double *scratch, double *out, cudaStream_t s)
{
    k_error_partial<<<EG, EB, 0, s>>>(vel, nx, ny, vel_ref, nx_ref, stride, scratch);
    k_error_final<<<1, EB, 0, s>>>(scratch, out);
    return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

// ------------------------------------------------------------------------------------------------
// Host side
// ------------------------------------------------------------------------------------------------

namespace {

int n_threads(size_t work)
{
    const unsigned hw = std::thread::hardware_concurrency();
    const size_t t = std::min<size_t>(hw ? hw : 4, std::max<size_t>(1, work / 65536));
    return (int)std::max<size_t>(1, t);
}

// Rows [r0, r1) of nx nodes with nc values each, as rec_velocity writes them: "%g " per value and
// a newline per row.
void format_rows(const double *v, int nx, int nc, long long r0, long long r1, std::string *out)
{
    char buf[40];
    for (long long r = r0; r < r1; r++) {
        const double *p = v + r * nx * nc;
        for (long long k = 0; k < (long long)nx * nc; k++) {
            const int m = snprintf(buf, sizeof buf, "%g ", p[k]);
            out->append(buf, (size_t)m);
        }
        out->push_back('\n');
    }
}

}  // namespace

int write_vtk_file(const char *path, int field, int format, int nx, int ny, int nz, const double *vals,
                   const unsigned char *bytes, size_t n_bytes)
{
    FILE *fp = fopen(path, "wb");
    if (!fp) return -1;
    // titles and names of the reference's writers (the ASCII vorticity writer reuses "Velocidade")
    static const char *ascii_title[] = {"", "Velocidade", "Velocidade", "Densidade"};
    static const char *bin_title[] = {"", "Velocidade", "Vorticidade", "Densidade"};
    static const char *name[] = {"", "velocidade", "vorticity", "densidade"};
    const long long n = (long long)nx * ny * nz;
    fprintf(fp, "# vtk DataFile Version 2.0\n%s\n%s\nDATASET STRUCTURED_POINTS\n",
            format ? bin_title[field] : ascii_title[field], format ? "BINARY" : "ASCII");
    fprintf(fp, "DIMENSIONS %d %d %d\nASPECT_RATIO 1 1 1\nORIGIN 0 0 0\n", nx, ny, nz);
    if (format)
        fprintf(fp, "POINT_DATA %lld\n", n);
    else
        fprintf(fp, "POINT_DATA %d\n", nx * ny * nz);  // an int product, as the ASCII writers print it
    const char *type = format == 1 ? "float" : "double";
    if (field == 3)
        fprintf(fp, "SCALARS %s %s\nLOOKUP_TABLE default\n", name[field], type);
    else
        fprintf(fp, "VECTORS %s %s\n", name[field], type);
    int rc = 0;
    if (format == 0) {
        const int nc = field == 3 ? 1 : 3;
        const long long rows = (long long)ny * nz;
        const int t = n_threads((size_t)n * nc);
        std::vector<std::string> parts(t);
        std::vector<std::thread> th;
        for (int k = 0; k < t; k++)
            th.emplace_back(format_rows, vals, nx, nc, rows * k / t, rows * (k + 1) / t, &parts[k]);
        for (auto &x : th) x.join();
        for (auto &p : parts)
            if (fwrite(p.data(), 1, p.size(), fp) != p.size()) rc = -1;
    } else {
        if (fwrite(bytes, 1, n_bytes, fp) != n_bytes) rc = -1;
        fputc('\n', fp);
    }
    if (fclose(fp) != 0) rc = -1;
    return rc;
}

void error_sums_host(const double *vs, int nx, int ny, const double *vr, int nx_ref, int stride, int digits,
                     double out[3])
{
    // the values the tool reads: vx, vy of every simulation node and of every sampled reference node
    std::vector<double> c((size_t)nx * ny * 2), r((size_t)nx * ny * 2);
    for (long long y = 0; y < ny; y++)
        for (long long x = 0; x < nx; x++) {
            const size_t k = 2 * (size_t)(x + y * nx);
            const double *p = vs + 3 * (x + y * nx);
            const double *q = vr + 3 * (x * stride + y * stride * (long long)nx_ref);
            c[k] = p[0];
            c[k + 1] = p[1];
            r[k] = q[0];
            r[k + 1] = q[1];
        }
    if (digits > 0) {
        text_round(c.data(), c.size(), digits);
        text_round(r.data(), r.size(), digits);
    }
    double sum_dif2 = 0.0, sum_vec2 = 0.0, sum_ur2 = 0.0;
    for (size_t k = 0; k < c.size(); k += 2) {
        const double vx_ref = r[k], vy_ref = r[k + 1], vx_cal = c[k], vy_cal = c[k + 1];
        const double u_r = std::sqrt(vx_ref * vx_ref + vy_ref * vy_ref);
        const double u_s = std::sqrt(vx_cal * vx_cal + vy_cal * vy_cal);
        sum_dif2 = sum_dif2 + (u_s - u_r) * (u_s - u_r);
        sum_vec2 = sum_vec2 + (vx_cal - vx_ref) * (vx_cal - vx_ref) + (vy_cal - vy_ref) * (vy_cal - vy_ref);
        sum_ur2 = sum_ur2 + u_r * u_r;
    }
    out[0] = sum_dif2;
    out[1] = sum_vec2;
    out[2] = sum_ur2;
}

void text_round(double *v, size_t n, int digits)
{
    auto work = [v, digits](size_t a, size_t b) {
        char buf[64];
        for (size_t i = a; i < b; i++) {
            snprintf(buf, sizeof buf, "%.*g", digits, v[i]);
            v[i] = strtod(buf, nullptr);
        }
    };
    const int t = n_threads(n);
    std::vector<std::thread> th;
    for (int k = 0; k < t; k++) th.emplace_back(work, n * k / t, n * (k + 1) / t);
    for (auto &x : th) x.join();
}

}  // namespace erlbm
