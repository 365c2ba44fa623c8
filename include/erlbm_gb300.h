/*
 * erlbm_gb300.h -- C ABI of the GB300 E-RLBM collide-stream engine (liberlbm_gb300.so).
 *
 * Plain C: pointers, sizes and PODs only; no C++ or CUDA types cross this boundary, and nothing
 * depends on the reference's nvel/dim macros.  Every function returns an int status
 * (ERLBM_OK = 0, negative on error) and never throws.  The caller owns every host buffer; the
 * library owns device memory.  A handle is used by one host thread at a time; different handles
 * may be driven from different threads (each has its own CUDA stream).
 *
 * Granularity.  The reference's interface is per site -- coll_Ext_Reg(f, ax, ay, az, LATTICE,
 * PARAMETERS) (SimBoltz_Functions/Definitions.cpp:697), propag_site (:509), ZouHeD3Q19_vx_x
 * (:922), devnull_rho_x (:907), kinectic_energy (:1005), density (:582) -- called by the
 * drivers' node loops (src/main_*.cpp).  A per-site call cannot run on a GPU, so this ABI sits
 * one level up, at sweep and run granularity: one erlbm_step() replaces one pass of a driver's
 * "for pto: colisao_sitio; propag_site" loop plus the pointer swap, and erlbm_map_run() replaces
 * a whole OpenMP map loop.  Population arrays crossing the ABI use the reference layout:
 * AoS in fluid-index order, f[pto * q + i], velocity order of def_lattice_d2q9 / def_lattice_d3q19.
 */
#ifndef ERLBM_GB300_H
#define ERLBM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------------------------- */
#define ERLBM_OK 0
#define ERLBM_E_INVAL (-1)       /* bad argument (the reference exit(1)s on a bad operator name) */
#define ERLBM_E_OOM (-2)         /* device or host allocation failed */
#define ERLBM_E_CUDA (-3)        /* CUDA error; erlbm_last_error() has the text */
#define ERLBM_E_TIMEOUT (-4)     /* a bounded device wait ran out */
#define ERLBM_E_NONFINITE (-5)   /* non-finite value where a finite one was required */
#define ERLBM_E_UNSUPPORTED (-6) /* valid request this build does not provide */
#define ERLBM_E_STATE (-7)       /* call not valid in the handle's current state */

/* ---- collision operators: same numbers as COLISAO (src/erlbm_common.h:42) ------------------- */
#define ERLBM_OP_BGK 1    /* coll_BGK     Collision_operators.cpp:12-49 */
#define ERLBM_OP_MRT 2    /* coll_MRT     Collision_operators.cpp:487-701 (D2Q9 only, as in the reference) */
#define ERLBM_OP_REG 3    /* coll_Reg     Collision_operators.cpp:860-967 (E-RLBM with tau_nh = 1) */
#define ERLBM_OP_EXTREG 4 /* coll_Ext_Reg Collision_operators.cpp:1182-1307 */

/* ---- precisions --------------------------------------------------------------------------- */
#define ERLBM_FP64 0         /* plain path: bit-identical to the reference's FP64 CPU results */
#define ERLBM_FP32_SHIFTED 1 /* populations stored and collided in FP32 as f_i - w_i */
#define ERLBM_FP32_PAIR 2    /* compensated: f_i - w_i stored as a pair of floats (hi + lo, 8 bytes), the
                                momentum and the pair differences collided in float-float arithmetic on
                                the FP32 pipe, the small parts in FP32; periodic D2Q9 lattices without
                                boundary planes or per-step density checks, BGK / RLBM / E-RLBM (others
                                return ERLBM_E_UNSUPPORTED); no counterpart in the reference */

/* ---- population stages (which populations a query reads) ---------------------------------- */
#define ERLBM_STAGE_POST_STREAM 0    /* lattice.inif at the top of a driver's step loop */
#define ERLBM_STAGE_POST_COLLISION 1 /* lattice.inif after the last step's collision, before the swap
                                        (what main_taylor-green.cpp and main_double-shear-layer.cpp
                                        measure) */

typedef struct erlbm_handle erlbm_handle;

/* Lattice description; replaces GEOMETRY + LATTICE + PARAMETERS of define_rede / aloca_populacoes
 * (src/erlbm_common.h:123-157).  solid: nx*ny*nz bytes, x fastest, 1 = solid, NULL = all fluid
 * (geometria_periodica, src/erlbm_common.h:101-114).  Fluid indices number the non-solid nodes
 * in that order, as numera_fluido does (src/erlbm_common.h:89-99). */
typedef struct erlbm_desc {
    int q;              /* 9 (D2Q9, nz must be 1) or 19 (D3Q19) */
    int nx, ny, nz;
    const uint8_t *solid;
    double tau, tau_nh; /* PARAMETERS.tau, PARAMETERS.tau_nh */
    int op;             /* ERLBM_OP_* */
    int precision;      /* ERLBM_FP64 or ERLBM_FP32_SHIFTED */
} erlbm_desc;

/* Boundary planes applied to the post-stream populations at the start of each step, in this
 * order: inlet, outlet (main_stability-map_obstacle.cpp:92-94), then the open y plane.  -1 disables
 * a plane.  The first four fields are the obstacle program's; a zero-initialised remainder keeps
 * its boundaries (Zou-He inlet, density outlet, no open y plane). */
#define ERLBM_INLET_ZOUHE 0         /* ZouHeD3Q19_vx_x (Boundary_conditions.cpp:350-442) or, on D2Q9,
                                       ZouHeD2Q9_vx_x (:710-744) */
#define ERLBM_INLET_PARABOLIC 1     /* parabolic_D3Q19_x (:456-530) / parabolic_D2Q9_x (:748-800) */
#define ERLBM_OUTLET_DENSITY 0      /* devnull_rho_x (:68-141): copy of the inner plane rescaled to rho_out */
#define ERLBM_OUTLET_OPEN 1         /* OpenBoundaryD2Q9_x (:584-621), D2Q9 only */
#define ERLBM_OUTLET_CONVECTIVE 2   /* convective_x (:627-706) */
typedef struct erlbm_bc {
    int inlet_x;     /* velocity inlet plane */
    double u_in;     /* its x velocity; the profile's maximum for ERLBM_INLET_PARABOLIC */
    int outlet_x;    /* outlet plane */
    double rho_out;  /* ERLBM_OUTLET_DENSITY's density */
    int inlet_kind;  /* ERLBM_INLET_* */
    int parabolic_L; /* profile width L: the h-th fluid node of a column (from y = 0, per z) gets
                        u = -4 u_in / L^2 (h - 1/2) (h - 1/2 - L); each column may hold at most L fluid
                        nodes and L < ny, as the reference's profile table requires */
    int outlet_kind; /* ERLBM_OUTLET_* */
    int open_y_on;   /* 1: OpenBoundaryD2Q9_y (:542-580) on plane open_y (D2Q9) */
    int open_y;
} erlbm_bc;

/* Stability checks of a run (roda_ponto, main_stability-map_taylor-green.cpp:41-104 and
 * main_stability-map_obstacle.cpp:75-123). */
typedef struct erlbm_checks {
    int energy_every;     /* E of the post-stream populations at step % energy_every == 0 && step > 0;
                             unstable when E > energy_factor * E0 or E non-finite; 0 = off */
    double energy_factor; /* 2 in the reference */
    int density_check;    /* |rho| > density_limit or non-finite at any node, post-collision, every step */
    double density_limit; /* 10 rho0 in the reference */
} erlbm_checks;

typedef struct erlbm_run_result {
    int label;        /* 1 unstable, 0 stable */
    int decided_step; /* step of the failing check, or the step count when stable */
    int steps_done;   /* steps executed */
    double margin;    /* max over checks of E / (factor E0), or max |rho| / density_limit; +inf if non-finite */
} erlbm_run_result;

/* ---- library ------------------------------------------------------------------------------ */
int erlbm_version(void);
const char *erlbm_strerror(int code);
const char *erlbm_last_error(void); /* text of the last error on this host thread */

/* ---- single lattice ------------------------------------------------------------------------ */
/* define_rede + aloca_populacoes (src/erlbm_common.h:123-148) */
int erlbm_create(const erlbm_desc *d, erlbm_handle **h);
/* libera_populacoes (src/erlbm_common.h:150-157) */
int erlbm_destroy(erlbm_handle *h);
int erlbm_fluid_count(const erlbm_handle *h, int64_t *n_fluid);
/* new PARAMETERS for the next steps (colisao_sitio's parameters argument, src/erlbm_common.h:69) */
int erlbm_set_params(erlbm_handle *h, double tau, double tau_nh, int op);
/* writes lattice.inif: n = n_fluid * q post-stream populations (the state a step starts from) */
int erlbm_set_populations(erlbm_handle *h, const double *aos, size_t n);
/* reads the populations of the chosen stage into aos (n = n_fluid * q) */
int erlbm_get_populations(erlbm_handle *h, double *aos, size_t n, int stage);
/* n_steps driver steps: [boundary planes] -> colisao_sitio at every node -> propag_site -> swap
 * (replaces e.g. main_double-shear-layer.cpp:382-449 without the output block).  bc may be NULL. */
int erlbm_step(erlbm_handle *h, int n_steps, const erlbm_bc *bc);
/* kinectic_energy (Other_functions.cpp:100-115) of the chosen stage */
int erlbm_kinetic_energy(erlbm_handle *h, int stage, double *energy);
/* max over fluid nodes of |density| (LBM_functions.cpp:5544-5552) and a non-finite flag */
int erlbm_max_abs_density(erlbm_handle *h, int stage, double *max_abs_rho, int *nonfinite);
/* per-fluid-node density and velocity (calcula, LBM_functions.cpp:3518-3589) of the chosen stage:
 * rho[n_fluid] and u[3 * n_fluid] (ux, uy, uz per node); either may be NULL */
int erlbm_macroscopic(erlbm_handle *h, int stage, double *rho, double *u);
/* Fields of the reference's writers (SimBoltz_Functions/LBM_functions.cpp) computed on the device
 * for the chosen stage, at every node of the box, x fastest, solid nodes 0:
 *   ERLBM_FIELD_VELOCITY   calcula's (vx, vy, vz), 3 values per node (rec_velocity :4218)
 *   ERLBM_FIELD_VORTICITY  vorticity(): central differences of the neighbours' velocities, periodic
 *                          wrap, a solid neighbour counting as 0 (:3761-3872), 3 values per node
 *   ERLBM_FIELD_DENSITY    density(), 1 value per node (rec_density :4416)
 * Only the field crosses to the host, not the populations. */
#define ERLBM_FIELD_VELOCITY 1
#define ERLBM_FIELD_VORTICITY 2
#define ERLBM_FIELD_DENSITY 3
int erlbm_field(erlbm_handle *h, int stage, int field, double *out, size_t n);
/* The same field written as a legacy VTK file, byte for byte what the reference's writers produce:
 * ERLBM_VTK_ASCII as rec_velocity / rec_vorticity / rec_density (values printed with 6 significant
 * digits); ERLBM_VTK_BINARY_FLOAT / _DOUBLE as rec_*_bin (:4979, :5061, :5179; big-endian, encoded
 * on the device).  The caller chooses the path (the reference names files vel_<t*>.vtk,
 * vor_<step>.vtk, rho_<step>.vtk). */
#define ERLBM_VTK_ASCII 0
#define ERLBM_VTK_BINARY_FLOAT 1
#define ERLBM_VTK_BINARY_DOUBLE 2
int erlbm_write_vtk(erlbm_handle *h, int stage, int field, int format, const char *path);
/* tools/error_calculator.cpp:60-105 on two lattices of one GPU: the velocity of `sim` (nx x ny, nz = 1)
 * against that of `ref` sampled at (s x, s y), s = ref nx / sim nx (an integer, the same in y):
 * E_vec = sqrt(sum |u_s - u_r|^2 / sum |u_r|^2), E_mod = sqrt(sum (|u_s| - |u_r|)^2 / sum |u_r|^2).
 * text_digits = 0: full precision, summed on the device (fixed-shape tree).  text_digits > 0: every
 * value is first rounded to that many significant digits, as the tool reads it from the ASCII files
 * rec_velocity writes (6), and summed in the tool's order: the tool's own result. */
int erlbm_velocity_error(erlbm_handle *sim, int sim_stage, erlbm_handle *ref, int ref_stage, int text_digits,
                         double *e_vec, double *e_mod);
/* roda_ponto on this lattice: up to n_steps steps with the given checks; stops at the first
 * failing check as the reference does */
int erlbm_run(erlbm_handle *h, int n_steps, const erlbm_bc *bc, const erlbm_checks *chk, erlbm_run_result *res);
/* wait for the handle's queued work */
int erlbm_sync(erlbm_handle *h);
/* FP64 add and multiply operations per second that the current GPU issues (independent unfused chains
 * over one wave of resident blocks): the roofline of the plain FP64 path, which issues its operations
 * unfused to round as the reference's build does.  No counterpart in the reference. */
int erlbm_fp64_rate(double *ops_per_s);
/* launch shape of the fused periodic D2Q9 FP32 kernel (the double-shear-layer lattices): threads per
 * block of the one-step kernel (128, 256, 512; 0 = default 256) and flags
 *   ERLBM_LAUNCH_STREAMING_STORES  evict-first stores (one-step kernel);
 *   ERLBM_LAUNCH_TWO_STEP          two consecutive steps per launch, the intermediate step kept on
 *                                  chip (nx % 128 == 0, ny even): half the HBM traffic per update;
 *   ERLBM_LAUNCH_THREE_STEP        three steps per launch (same conditions): a third of the traffic;
 *   ERLBM_LAUNCH_WIDE_STRIPS       with ERLBM_LAUNCH_THREE_STEP: 64-column warp strips in which a lane
 *                                  holds two neighbouring columns (60 outputs per 64 columns instead
 *                                  of 28 per 32; ny >= 16 and 9 nx ny < 2^31, else one step per
 *                                  launch).
 * The results are the same bits in every shape; at most one of the two multi-step flags.  Steps left
 * over (fewer than a launch takes) run one at a time.  Chosen by erlbm_gb300.autotune; no
 * counterpart in the reference. */
#define ERLBM_LAUNCH_STREAMING_STORES 1
#define ERLBM_LAUNCH_TWO_STEP 2
#define ERLBM_LAUNCH_THREE_STEP 4
#define ERLBM_LAUNCH_WIDE_STRIPS 8
int erlbm_set_launch(erlbm_handle *h, int block_threads, int flags);
/* run the handle's work on the caller's CUDA stream (a cudaStream_t; NULL = the handle's own
 * stream).  Waits for the work queued so far first.  No counterpart in the reference, whose loops
 * are synchronous; it lets a caller order the engine with its own GPU work and time it with events. */
int erlbm_set_stream(erlbm_handle *h, void *stream);

/* ---- batched independent runs (stability maps) ------------------------------------------- */
/* Many small lattices of one geometry, each its own run, in one persistent GPU launch: the
 * replacement for the maps' "#pragma omp parallel for collapse(2) schedule(dynamic)" loops over
 * roda_ponto (main_stability-map_taylor-green.cpp:150-177, main_stability-map_obstacle.cpp:161-186).
 * nx * ny <= 4096 nodes (the lattice lives in one CTA's shared memory), nz = 1. */
#define ERLBM_INIT_REST 0     /* f_i = w_i rho0 (main_stability-map_obstacle.cpp:81-82) */
#define ERLBM_INIT_TG_MAP 1   /* equilibrium, rho = 1, u = u0 (sin kx cos ky, -cos kx sin ky)
                                 (main_stability-map_taylor-green.cpp:49-61) */
#define ERLBM_INIT_AOS 2      /* each run's initial post-stream populations from aos[aos_offset...] */

typedef struct erlbm_batch_desc {
    int q, nx, ny;
    const uint8_t *solid;       /* nx*ny bytes, 1 = solid; NULL = periodic */
    int inlet_x, outlet_x;      /* boundary planes as in erlbm_bc (-1 = none); inlet velocity = run's u0 */
    double rho0;                /* outlet and rest density */
    int energy_every;           /* energy check period (0 = off) */
    double energy_factor;
    int density_check;          /* per-step density check (0 = off) */
    double density_limit;
    int init;                   /* ERLBM_INIT_* */
    int precision;
    int slots;                  /* resident lattices per SM; 0 = as many as fit */
} erlbm_batch_desc;

typedef struct erlbm_run_spec {
    int op;                     /* ERLBM_OP_* of this run */
    double tau, tau_nh;
    double u0;                  /* TG amplitude (ERLBM_INIT_TG_MAP) or inlet velocity */
    int n_steps;                /* step budget */
    int64_t aos_offset;         /* ERLBM_INIT_AOS: offset in doubles of n_fluid * q populations */
} erlbm_run_spec;

typedef struct erlbm_batch_result {
    int label;                  /* 1 unstable */
    int decided_step;           /* failing step, or n_steps */
    int steps_done;
    int status;                 /* bit 0 |rho| > limit, bit 1 non-finite density, bit 2 energy check;
                                   bit 3 (value 8, erlbm_batch_run_noalloc only): the run was refused
                                   (bad op, tau, tau_nh or n_steps) and not stepped, its label means
                                   nothing */
    double margin;              /* as in erlbm_run_result */
    double energy;              /* last kinetic energy computed (E0 if no check ran) */
} erlbm_batch_result;

int erlbm_batch_run(const erlbm_batch_desc *d, int n_runs, const erlbm_run_spec *runs, const double *aos,
                    size_t n_aos, erlbm_batch_result *out);

/* Batched runs without any allocation.  No counterpart in the reference.  For callers that cannot
 * let a library allocate GPU memory (their own allocator owns the device, or their loop may not pay
 * for cudaMalloc / cudaFree and the synchronisation cudaFree implies): the per-call scratch that
 * erlbm_batch_run allocates lives here in one static device array of about 1.2 MB per GPU, held
 * until the process exits, and nothing is allocated.  runs and out are DEVICE arrays of n_runs
 * entries owned by the caller; d->solid, when set, is a DEVICE pointer; d->init must be
 * ERLBM_INIT_REST or ERLBM_INIT_TG_MAP.  At most ERLBM_NOALLOC_MAX_RUNS runs per call (more is
 * ERLBM_E_INVAL).  The work is queued on `stream` (a cudaStream_t; NULL = the default stream) and
 * the call does not wait for the runs; with ERLBM_INIT_TG_MAP it copies its sin/cos tables from
 * pageable host memory, which may wait for the stream's earlier work, and it returns
 * ERLBM_E_UNSUPPORTED when `stream` is being captured.  Runs are taken in the caller's order
 * (erlbm_batch_run starts the longest first); results are the same.  The run table is read on the
 * device, so a run with a bad operator, tau, tau_nh or n_steps cannot fail the call as it fails
 * erlbm_batch_run (ERLBM_E_INVAL / ERLBM_E_UNSUPPORTED for the whole call): it is refused on its
 * own, not stepped, and its result has status 8 and label 0.  The first call on a device looks up
 * the array's device address (and again after that device's context was replaced, e.g. by
 * cudaDeviceReset): make that first call before any stream capture.  Every call shares the one
 * array, so calls that overlap on the GPU (different streams, or several host threads) race: order
 * them on one stream. */
#define ERLBM_NOALLOC_MAX_RUNS 16384
int erlbm_batch_run_noalloc(const erlbm_batch_desc *d, int n_runs, const erlbm_run_spec *runs,
                            erlbm_batch_result *out, void *stream);

/* The reference's stability maps with their axes (main_stability-map_taylor-green.cpp:134-166,
 * main_stability-map_obstacle.cpp:147-175). */
#define ERLBM_MAP_TAYLOR_GREEN 1
#define ERLBM_MAP_OBSTACLE 2

typedef struct erlbm_map_desc {
    int kind;                   /* ERLBM_MAP_* */
    int precision;
    int op;                     /* TG map: ERLBM_OP_REG or ERLBM_OP_EXTREG, or 0 for both (results
                                   of all RLBM runs first, then all E-RLBM runs); obstacle: ignored */
    double tau_nh;              /* TG map E-RLBM tau_nh (0.65) */
    int L;                      /* TG map lattice side (16) */
    double ma;                  /* obstacle Mach number (0.1) */
    int n_i, n_j;               /* map axes (400 x 400) */
    int n_points;               /* 0: the whole n_i x n_j grid, i fastest; else the points pi[k], pj[k] */
    const int32_t *pi, *pj;
    int max_steps;              /* cap on each run's budget, 0 = the reference's count */
    int slots;                  /* as in erlbm_batch_desc */
} erlbm_map_desc;

/* labels (and optionally decided steps and margins) of n_points (x 2 when op = 0) runs */
int erlbm_map_run(const erlbm_map_desc *d, int32_t *labels, int32_t *decided_step, double *margins);

/* Which points of an FP32-screened map are run again in FP64 (erlbm_map_run_refined). */
typedef struct erlbm_refine_desc {
    int radius;            /* half-width in map steps (i and j) of the window searched for a label change */
    double late_fraction;  /* FP32 runs that turned unstable after this fraction of their budget; <= 0: off */
    int probe_stride;      /* FP64 probes at i, j = stride/2 + m*stride (finds unstable islands the FP32
                              map misses entirely); 0: none */
    int max_passes;        /* FP64 passes; 0: until no label change is left with an FP32 point near it */
} erlbm_refine_desc;

/* A stability map screened in FP32-shifted and refined in FP64.  No counterpart in the reference,
 * whose maps (main_stability-map_*.cpp) run every point in FP64.  Every point runs first in
 * ERLBM_FP32_SHIFTED (d->precision is ignored).  Points are then run again in ERLBM_FP64, whose results
 * replace the FP32 ones and equal the reference's, in passes:
 *   pass 1: points within r->radius of a label change of the FP32 map (the stability boundary, same
 *           operator), FP32 runs that turned unstable late, and the probe points;
 *   pass n: the FP32 points within r->radius of a label change of the map as it stands (FP64 labels where
 *           refined), so that the refinement follows the FP64 boundary where it lies away from the FP32
 *           one, and spreads over an island that a probe found.
 * The whole grid only (d->n_points = 0).  refined (optional, one byte per result) is set to 1 for the
 * results that came from FP64; n_passes (optional) receives the number of FP64 passes.  Arrays are
 * laid out as in erlbm_map_run. */
int erlbm_map_run_refined(const erlbm_map_desc *d, const erlbm_refine_desc *r, int32_t *labels,
                          int32_t *decided_step, double *margins, uint8_t *refined, int *n_passes);

/* read_geo (SimBoltz_Functions/LBM_functions.cpp:282-353): the solid mask (1 = solid, the layout of
 * erlbm_desc.solid) of a legacy ASCII VTK geometry file, nonzero values fluid, with pts_in / pts_out
 * fluid layers added in x and, with `wall`, the first and last x planes of the widened box solid.
 * solid = NULL returns the dimensions only; otherwise n must be nx * ny * nz. */
int erlbm_read_geo(const char *path, int pts_in, int pts_out, int wall, int *nx, int *ny, int *nz, uint8_t *solid,
                   size_t n);

/* ---- request server (continuous batching) ---------------------------------------------------- */
/* No counterpart in the reference, which runs one program per invocation.  A server owns a fixed
 * slice of device memory and a scheduler thread; requests are admitted while others run:
 *  - D3Q19 lattices of <= 288 nodes (Taylor-Green map points, the obstacle channel at scale 1) go to
 *    a device-resident loop whose CTAs claim them from a ring as soon as they are published;
 *  - D2Q9 and D3Q19 Taylor-Green lattices and the scaled obstacle channels of up to team_max_nodes
 *    nodes go to a second device-resident loop (one per precision) that claims them from its own ring
 *    and admits them on the device by memory footprint (pages of half the budget); its CTAs join the
 *    admitted runs and work through their steps in chunks of nodes (lane 2);
 *  - larger lattices are admitted by memory footprint and advanced on their own CUDA streams.
 * The lane a request takes depends only on the request, so its result does not depend on the mix.
 * While a server runs, avoid calls that synchronise the whole device (erlbm_destroy frees memory)
 * on the same GPU: they wait until the resident loop idles out (about a second).  The resident loops
 * run on their own streams; set CUDA_DEVICE_MAX_CONNECTIONS=32 in the environment before the process
 * creates its CUDA context, or work on a stream that shares a hardware queue with a resident loop
 * waits until that loop leaves (the Python package sets it when imported). */
#define ERLBM_REQ_TG2D 1          /* D2Q9 Taylor-Green L x L, inicializa_taylor_green init (main_taylor-green.cpp:57-100) */
#define ERLBM_REQ_TG_MAP_POINT 2  /* D3Q19 16 x 16 x 1 map point, energy checks every 100 steps (TG map roda_ponto) */
#define ERLBM_REQ_OBSTACLE 3      /* D3Q19 obstacle channel scaled (sx, sy), Zou-He inlet with u0, density checks */
#define ERLBM_REQ_TG3D 4          /* D3Q19 L^3 periodic Taylor-Green equilibrium, rho = 1,
                                     u = u0 (sin kx cos ky cos kz, -cos kx sin ky cos kz, 0) */

typedef struct erlbm_server erlbm_server;

typedef struct erlbm_server_desc {
    int64_t hbm_budget_bytes;   /* device memory for admitted lattices (default 8 GiB) */
    int slot_ctas;              /* CTAs of each resident loop (one per precision); 0 = SMs / 2 */
    int max_streams;            /* concurrent stream-lane runs, and team-loop runs per precision; 0 = 16
                                   stream-lane runs and 64 team-loop runs */
    int queue_capacity;         /* ring entries per resident loop; 0 = 65536 */
    int team_ctas;              /* CTAs of each team loop (one per precision); 0 = SMs; < 0: no team
                                   loop, its requests take the stream lane */
    int team_max_nodes;         /* largest lattice (nodes) the team loops take; 0 = 2^19 (D2Q9 512^2,
                                   D3Q19 64^3).  Larger ones take the stream lane.  A lower limit (65536)
                                   sends the large FP64 lattices to the stream lane's whole-GPU launches,
                                   which run them faster: more runs/s on FP64-heavy streams, higher p50 */
    int team_wait_us;           /* longest wait of a team-loop run for the previous phase of its steps
                                   before the run is reported failed (status ERLBM_E_TIMEOUT); 0 = 5 s */
} erlbm_server_desc;

typedef struct erlbm_request {
    int kind;                   /* ERLBM_REQ_* */
    int precision, op;
    int L;                      /* side: TG2D 2..4096, TG3D 2..512 (ERLBM_E_INVAL otherwise) */
    int sx, sy;                 /* obstacle scale */
    double tau, tau_nh, u0;
    int n_steps;                /* step budget */
} erlbm_request;

typedef struct erlbm_result {
    int status;                 /* ERLBM_OK or an error code */
    int label, steps_done, decided_step;
    double energy;              /* kinetic energy: post-stream state after the run (stream lane) or at
                                   the last energy check (map points) */
    double margin;
    double t_submit, t_admit, t_done; /* seconds on the server clock (t_admit < 0: resident loop) */
    int lane;                   /* 0 resident loop, 1 stream lane, 2 resident team loop */
} erlbm_result;

int erlbm_server_start(const erlbm_server_desc *d, erlbm_server **s);
int erlbm_server_submit(erlbm_server *s, const erlbm_request *req, int64_t *ticket);
/* ERLBM_OK and *res filled when the request is done, 1 while it is pending */
int erlbm_server_poll(erlbm_server *s, int64_t ticket, erlbm_result *res);
int erlbm_server_wait(erlbm_server *s, int64_t ticket, erlbm_result *res, double timeout_s);
double erlbm_server_clock(erlbm_server *s);
/* finishes every accepted request, then stops */
int erlbm_server_stop(erlbm_server *s);

/* ---- program inputs (host functions; what the reference's drivers build around their loops) --- */
/* inicializa_taylor_green (main_taylor-green.cpp:57-100) on an L x L (x nz) periodic box, AoS in
 * fluid-index order.  variant 1 is the same vortex translated by (L/4, L/4):
 * u = U0 (-cos kx sin ky, sin kx cos ky), rho = 1 - 3/4 U0^2 (cos 2kx + cos 2ky). */
int erlbm_init_taylor_green(int q, int L, int nz, double u0, double tau, int poisson, int neq, int variant,
                            double *aos);
/* initial_double_shear_layer (main_double-shear-layer.cpp:48-66), U0 = 1/32, lambda = 80, epsilon = 0.05 */
int erlbm_init_double_shear(int L, double rho_ini, double *aos);
/* dist_eq (LBM_functions.cpp:2945-3000) of one node */
int erlbm_equilibrium(int q, double ux, double uy, double uz, double rho, double *feq);
/* geometria_obstaculo (main_stability-map_obstacle.cpp:42-70) scaled by (sx, sy): nx = 20 sx + 2,
 * ny = 12 sy; solid may be NULL to query the extent */
int erlbm_obstacle_geometry(int sx, int sy, int *nx, int *ny, uint8_t *solid);
/* E_vector, E_magnitude and nu_ef/nu - 1 of a Taylor-Green field (main_taylor-green.cpp:178-213) */
int erlbm_taylor_green_error(int q, int L, const double *aos, double u0, double visc, int step, int variant,
                             double *out3);
/* map axes of main_stability-map_taylor-green.cpp:134-164 and main_stability-map_obstacle.cpp:147-173 */
int erlbm_tg_map_params(int i, int j, int n_ma, int n_nu, int op, double tau_nh_in, double *u0, double *tau,
                        double *tau_nh);
int erlbm_obstacle_map_params(int i, int j, int n_tau, int n_nu, double ma, double *u_imp, double *tau,
                              double *tau_nh);

#ifdef __cplusplus
}
#endif
#endif /* ERLBM_GB300_H */
