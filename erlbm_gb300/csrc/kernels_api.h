// kernels_api.h -- host-side launchers of the single-lattice and batched kernels.
//
// The FP64 kernels live in k_fp64.cu (compiled with --fmad=false, the reference's rounding) and
// the FP32-shifted kernels in k_fp32.cu.  Everything here is internal to liberlbm_gb300.so.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "lattice.cuh"

namespace erlbm {

// Box geometry of one lattice on the device.  Populations are SoA: direction plane i starts at
// i * plane, node index = x + nx (y + ny z).  solid is null for a fully periodic box.
struct Geo {
    int nx, ny, nz;
    long long nbox, plane;
    const uint8_t *solid;
};

// Boundary planes of one step; -1 disables a plane.  inlet_kind 0: ZouHeD3Q19_vx_x / ZouHeD2Q9_vx_x,
// 1: parabolic_D3Q19_x / parabolic_D2Q9_x with the per-node velocity profile[y + ny z];
// outlet_kind 0: devnull_rho_x, 1: OpenBoundaryD2Q9_x, 2: convective_x; open_y: OpenBoundaryD2Q9_y.
struct BCp {
    int inlet_x;
    double u_in;
    int outlet_x;
    double rho_out;
    int inlet_kind, outlet_kind, open_y;
    const double *profile;
};

// Per-run device status used by the stability checks and early stop.
struct RunStatus {
    int flags;            // bit 0: |rho| above limit, bit 1: non-finite density, bit 2: energy check failed
    int decided_step;     // first step that set a flag (INT32_MAX when none)
    unsigned long long max_abs_rho_bits;  // max |rho| seen, as the bit pattern of a non-negative double
};

struct StepArgs {
    int mode;             // 0: stream (pull) + BC + collide;  1: BC + collide on local populations
    int step_index;       // reference step number of this launch
    int check_density;    // per-node |rho| > density_limit or non-finite, post-collision
    double density_limit;
    RunStatus *status;    // may be null when no check and no early stop
    int stop_on_flag;     // return without work when a check failed in an earlier step
};

// FP64 (exact) and FP32-shifted launchers.  src/dst are device SoA buffers of the precision.
int launch_step_fp64(int q, int op, const Geo &g, const BCp &bc, const Relax &R, const StepArgs &a, const double *src,
                     double *dst, cudaStream_t s);
int launch_step_fp32(int q, int op, const Geo &g, const BCp &bc, const Relax &R, const StepArgs &a, const float *src,
                     float *dst, cudaStream_t s);

// Fused periodic D2Q9 FP32 kernel (nx % 128 == 0, no solids, no boundary planes).  shape: threads
// per block (128, 256, 512; 0 = 256), plus 0x1000 for streaming (evict-first) stores.
int launch_periodic_d2q9_fp32(int op, const Geo &g, const Relax &R, const float *src, float *dst, cudaStream_t s,
                              int shape = 0);
bool periodic_d2q9_fp32_ok(const Geo &g);
// Two steps per launch of the same update (temporal blocking; nx % 128 == 0, ny even and >= 4).
int launch_periodic_d2q9_fp32_x2(int op, const Geo &g, const Relax &R, const float *src, float *dst, cudaStream_t s);
bool periodic_d2q9_x2_ok(const Geo &g);
// Three steps per launch: 32-column warp strips (wide = false) or 64-column strips over column pairs
// (wide = true, also needs periodic_d2q9_x3a_ok: ny >= 16, nine planes within 32-bit offsets).
int launch_periodic_d2q9_fp32_x3(int op, const Geo &g, const Relax &R, const float *src, float *dst, cudaStream_t s,
                                 bool wide);
bool periodic_d2q9_x3a_ok(const Geo &g);

// Stream only: dst = post-stream populations of the post-collision state src (no BC, no collision).
int launch_stream_only_fp64(int q, const Geo &g, const double *src, double *dst, cudaStream_t s);
int launch_stream_only_fp32(int q, const Geo &g, const float *src, float *dst, cudaStream_t s);

// Layout conversion between the caller's AoS fluid-index populations (double, reference order)
// and the device SoA box layout.  node_of_fluid is null for a periodic box (identity).
int launch_aos_to_soa_fp64(int q, const Geo &g, long long n_fluid, const int *node_of_fluid, const double *aos,
                           double *soa, cudaStream_t s);
int launch_soa_to_aos_fp64(int q, const Geo &g, long long n_fluid, const int *node_of_fluid, const double *soa,
                           double *aos, cudaStream_t s);
int launch_aos_to_soa_fp32(int q, const Geo &g, long long n_fluid, const int *node_of_fluid, const double *aos,
                           float *soa, cudaStream_t s);
int launch_soa_to_aos_fp32(int q, const Geo &g, long long n_fluid, const int *node_of_fluid, const float *soa,
                           double *aos, cudaStream_t s);

// Per-fluid-node kinetic energy 1/2 |u|^2, density and velocity of the populations in buf,
// written in fluid-index order into e_out / rho_out / u_out (3 per node); any may be null.
int launch_node_fields_fp64(int q, const Geo &g, long long n_fluid, const int *node_of_fluid, const double *buf,
                            double *e_out, double *rho_out, double *u_out, cudaStream_t s);
int launch_node_fields_fp32(int q, const Geo &g, long long n_fluid, const int *node_of_fluid, const float *buf,
                            double *e_out, double *rho_out, double *u_out, cudaStream_t s);

// Box fields of the reference's rec_* writers (every node, x fastest, solid nodes 0): field 1 =
// velocity (3 doubles per node), 3 = density (1 per node).
int launch_box_field_fp64(int q, const Geo &g, const double *buf, int field, double *out, cudaStream_t s);
int launch_box_field_fp32(int q, const Geo &g, const float *buf, int field, double *out, cudaStream_t s);
// vorticity() (LBM_functions.cpp:3761-3872) at every box node from the box velocity field vel.
int launch_vorticity(const Geo &g, const double *vel, double *vor, cudaStream_t s);
// n doubles as big-endian float (as_double = 0) or double bytes, vtk_push_real's encoding.
int launch_encode_be(const double *in, long long n, int as_double, unsigned char *out, cudaStream_t s);
// tools/error_calculator.cpp sums over an nx x ny velocity field against a reference field of
// nx_ref columns sampled with stride `stride`: out[0..2] = sum (|u_s| - |u_r|)^2, sum |u_s - u_r|^2,
// sum |u_r|^2 (fixed-shape tree, deterministic).  scratch holds >= 3 * 1024 doubles.
int launch_velocity_error_sums(const double *vel, int nx, int ny, const double *vel_ref, int nx_ref, int stride,
                               double *scratch, double *out, cudaStream_t s);

// Host side of the VTK writers (fields.cu): the reference's header text, then ASCII values (printf
// %g with `digits` significant digits, as an ostream writes them) or the given big-endian bytes.
int write_vtk_file(const char *path, int field, int format, int nx, int ny, int nz, const double *vals,
                   const unsigned char *bytes, size_t n_bytes);
// Each value of v rounded as text with `digits` significant digits and read back (threads).
void text_round(double *v, size_t n, int digits);
// tools/error_calculator.cpp's loop on the host, in its order: out = {sum (|u_s| - |u_r|)^2,
// sum |u_s - u_r|^2, sum |u_r|^2}; digits > 0 first rounds each value read as its text input does.
void error_sums_host(const double *vs, int nx, int ny, const double *vr, int nx_ref, int stride, int digits,
                     double out[3]);

// Sum of n doubles: serial in index order when n <= serial_limit (the reference's order), else a
// fixed-shape tree (deterministic).  scratch holds >= 1024 doubles.  Result in *out (device).
int launch_sum(const double *x, long long n, long long serial_limit, double *scratch, double *out, cudaStream_t s);
// max |x| over n doubles and a non-finite flag: out[0] = max, out[1] = 1.0 if any non-finite.
int launch_maxabs(const double *x, long long n, double *scratch, double *out, cudaStream_t s);

}  // namespace erlbm

namespace erlbm {

struct BatchGeo;
struct BatchRun;
struct BatchResult;

// Persistent batched launch (batch_kernels.cuh).  block = threads per CTA, npt = nodes per thread,
// grid = CTAs; smem = dynamic shared bytes.  Returns 0, -1 (no such instantiation) or -3.
// dbl: two population buffers in shared memory (one barrier per step) instead of one.
int launch_batch_fp64(int q, int npt, const BatchGeo &g, const BatchRun *runs, int n_runs, int *counter,
                      BatchResult *res, const double *aos, int grid, int block, size_t smem, int dbl,
                      cudaStream_t s);
int launch_batch_fp32(int q, int npt, const BatchGeo &g, const BatchRun *runs, int n_runs, int *counter,
                      BatchResult *res, const double *aos, int grid, int block, size_t smem, int dbl,
                      cudaStream_t s);
// Launch shape of a batch: nodes per thread, threads per CTA, CTAs, dynamic shared bytes.
struct LaunchShape {
    int npt, block, grid, dbl;
    size_t smem;
};
int pick_shape(int prec, int q, int nb, int slots, int n_runs, LaunchShape *out);

// Resident CTAs per SM for a configuration (0 if it cannot run).
int batch_occupancy(int prec, int q, int npt, int block, size_t smem);
size_t batch_smem(int prec, int q, int nb, int block, int dbl);

}  // namespace erlbm

namespace erlbm {

struct SlotRing;

// Device-resident request loop for D3Q19 lattices of <= 288 nodes (batch_kernels.cuh).
int launch_slot_server_fp64(const SlotRing &ring, int max_nb, int grid, int block, size_t smem, int dbl,
                            cudaStream_t s);
int launch_slot_server_fp32(const SlotRing &ring, int max_nb, int grid, int block, size_t smem, int dbl,
                            cudaStream_t s);
int slot_server_occupancy_fp64(int block, size_t smem);
int slot_server_occupancy_fp32(int block, size_t smem);

}  // namespace erlbm

namespace erlbm {

// Initial populations on the device: kind 1 = D2Q9 Taylor-Green program (tab = 4 L doubles),
// 4 = D3Q19 3-D Taylor-Green (tab = 2 L doubles), 0 = rest equilibrium with density rho.
int launch_init_fp64(int kind, int q, const Geo &g, double *buf, const double *tab, double u0, double tau, double k,
                     double rho, cudaStream_t s);
int launch_init_fp32(int kind, int q, const Geo &g, float *buf, const double *tab, double u0, double tau, double k,
                     double rho, cudaStream_t s);

// FP64 add / multiply rate of the current GPU (operations per second), k_fp64.cu
int measure_fp64_rate(double *ops_per_s);

// The compensated FP32 form (k_pair.cu): populations as float pairs (hi, lo); periodic D2Q9 lattices
// without boundary planes, BGK / RLBM / E-RLBM.
bool step_pair_ok(int q, int op, const Geo &g);
int launch_step_pair(int q, int op, const Geo &g, const Relax &R, int mode, const float2 *src, float2 *dst,
                     cudaStream_t s);
int launch_stream_only_pair(int q, const Geo &g, const float2 *src, float2 *dst, cudaStream_t s);
int launch_aos_to_soa_pair(int q, const Geo &g, long long n_fluid, const int *node_of_fluid, const double *aos,
                           float2 *soa, cudaStream_t s);
int launch_soa_to_aos_pair(int q, const Geo &g, long long n_fluid, const int *node_of_fluid, const float2 *soa,
                           double *aos, cudaStream_t s);
int launch_node_fields_pair(int q, const Geo &g, long long n_fluid, const int *node_of_fluid, const float2 *buf,
                            double *e, double *rho, double *u, cudaStream_t s);
int launch_box_field_pair(int q, const Geo &g, const float2 *buf, int field, double *out, cudaStream_t s);

// D2Q9 FP32-shifted steps with solids and boundary planes, fused where a 128-column segment touches
// neither (k_fp32.cu): nx % 128 == 0; segflag and nodeflag from d2q9_segment_flags (null: no solids);
// fix: the n_fix fluid nodes with nodeflag set, in node order.
bool d2q9_hybrid_ok(const Geo &g);
void d2q9_segment_flags(const Geo &g, const uint8_t *solid, uint8_t *flags, uint8_t *nodeflags);
int launch_step_fp32_hybrid(int op, const Geo &g, const BCp &bc, const Relax &R, const float *src, float *dst,
                            const uint8_t *segflag, const uint8_t *nodeflag, const int *fix, int n_fix, cudaStream_t s);

}  // namespace erlbm
