/*
 * jp.h - C ABI of the GB300 lattice Boltzmann engine (libjpsolver.so).
 *
 * The reference (josepedro/jp-solver) has no library interface: its "API" is the command line of
 * two programs, src/tgv3d_uniform.cu and src/tgv3d_amr.cu, whose main() parses flags, allocates the
 * populations, runs the time loop and prints diagnostics. Every entry point below replaces one piece
 * of those main() functions (cited per entry), so that the drop-in `uniform` / `amr` programs and any
 * other host (Python ctypes, cgo, JNI) drive the same device code through plain pointers and sizes.
 *
 * Conventions
 *   - Every call returns jp_status; JP_OK is 0.  On failure jp_last_error() gives a message (per
 *     host thread).  No entry point calls exit().
 *   - A solver owns all of its device memory and one CUDA stream; host buffers belong to the caller.
 *   - One solver is driven by one host thread at a time.
 *   - Populations cross the boundary in the reference's D3Q19 velocity order
 *     (q: 0 rest, 1..6 faces +x -x +y -y +z -z, 7..18 edges; src/tgv3d_uniform.cu:28-33) and either
 *     in the flat layout [q][z][y][x] or in the reference's blocked layout [block][q][cell]
 *     (block = (bz*gx+by)*gx+bx, cell = (k*MB+j)*MB+i; src/tgv3d_uniform.cu:43-53).
 */
#ifndef JP_H
#define JP_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define JP_ABI_VERSION 1

typedef enum jp_status {
    JP_OK = 0,
    JP_ERR_INVALID = 1,     /* bad argument: the reference exits 2 on N%MB (src/tgv3d_uniform.cu:148) */
    JP_ERR_CUDA = 2,        /* a CUDA runtime error: the reference's CK() exits 2 (src/tgv3d_uniform.cu:25) */
    JP_ERR_CAPACITY = 3,    /* a block pool or a fixed-size buffer would overflow */
    JP_ERR_NOMEM = 4,       /* the device or the HBM budget cannot hold the request */
    JP_ERR_STATE = 5,       /* call not valid in the solver's current state */
    JP_ERR_TIMEOUT = 6,     /* a bounded device wait gave up */
    JP_ERR_UNSUPPORTED = 7  /* valid request this build does not implement */
} jp_status;

typedef enum jp_kind { JP_UNIFORM = 0, JP_AMR = 1 } jp_kind;

/* Population storage.  FP32 is the reference's format.  FP16/BF16 store the shifted value f - w_q
 * (w_q the lattice weight) and collide in FP32; FP64 stores and computes in double. */
typedef enum jp_storage { JP_FP32 = 0, JP_FP16 = 1, JP_BF16 = 2, JP_FP64 = 3 } jp_storage;

typedef enum jp_layout { JP_LAYOUT_FLAT = 0, JP_LAYOUT_BLOCKED = 1 } jp_layout;

/* Host element type of a population copy. */
typedef enum jp_dtype { JP_F32 = 0, JP_F64 = 1 } jp_dtype;

/* Refinement mode of one AMR level (--l1/--l2 all|slab|sensor, src/tgv3d_amr.cu:651). */
typedef enum jp_refine { JP_REFINE_ALL = 0, JP_REFINE_SLAB = 1, JP_REFINE_SENSOR = 2 } jp_refine;

/* Solver configuration.  Defaults (jp_config_default) are the reference's flag defaults:
 * uniform --n 128 --re 1600 --u0 0.05 --tstar 12 (src/tgv3d_uniform.cu:143-147);
 * amr --n 32 --re 800 --frac1 0.35 --frac2 0.35 --l1 all --l2 all --adapt 100 --maxgb 0
 * (src/tgv3d_amr.cu:644-656,674,685). */
typedef struct jp_config {
    int32_t kind;            /* jp_kind */
    int32_t n;               /* uniform edge, or AMR coarse edge; a multiple of mb */
    double re;               /* Reynolds number */
    double u0;               /* TGV velocity amplitude (lattice units) */
    double tstar;            /* end time in t* = s * u0 * 2pi/n */
    int32_t storage;         /* jp_storage */
    int32_t mb;              /* block edge (4, 8 or 16); the reference's -DMB */
    int32_t l1_mode;         /* jp_refine, AMR only */
    int32_t l2_mode;         /* jp_refine, AMR only */
    double frac1, frac2;     /* target refined fractions (sensor mode) */
    int32_t adapt_every;     /* regrid period in coarse steps (sensor mode) */
    int32_t develop_steps;   /* uncounted coarse steps before the first sensor build (300) */
    double max_gb;           /* HBM ceiling for the fine pools in GiB; 0 = 75% of free memory */
    int32_t device;          /* CUDA device ordinal */
    int32_t threads_per_block; /* 0 = default; uniform: 64..512; AMR steps: 64 (MB=4), 128/256/512 */
    int32_t vec;             /* cells per thread along x in the uniform step; 0 = tuned default */
    int32_t flags;           /* JP_FLAG_* */
    int32_t buffer;          /* AMR sensor modes: dilate the refinement marks by this many block layers
                                (--buffer; parsed but unused by the reference, src/tgv3d_amr.cu:648) */
    int32_t reserved[6];
} jp_config;

/* jp_config.flags */
#define JP_FLAG_SKIP_PREP 1      /* AMR profiling: skip prep + ghost fill (breaks physics; --skipprep, src/tgv3d_amr.cu:654) */
#define JP_FLAG_SKIP_RESTRICT 2  /* AMR profiling: skip restriction (breaks physics; --skiprestr, :655) */
#define JP_FLAG_GRAPH 4          /* replay the step from captured CUDA graphs (--graph, :656) */
#define JP_FLAG_DEFER_INIT 8     /* jp_create allocates only: set a sensor override (or populations) and
                                    call jp_init_tgv before the first step, so that even the first
                                    AMR build uses the supplied sensor */
#define JP_FLAG_INPLACE 16       /* uniform: in-place (AA pattern) streaming in one population array,
                                    half the state's HBM, bit-identical results; no reference counterpart */

/* Derived quantities of a solver (src/tgv3d_uniform.cu:151-153, src/tgv3d_amr.cu:658-664). */
typedef struct jp_info {
    int32_t kind, n, mb, storage;
    int64_t cells;           /* uniform: n^3; AMR: coarse n^3 */
    int64_t steps;           /* round(tstar / (u0 * 2pi/n)) */
    double nu, tau, omega;   /* level-0 viscosity, relaxation time, 1/tau */
    double tau1, tau2;       /* AMR level 1/2 relaxation times */
    double kf;               /* 2pi/n */
    int64_t bytes_state;     /* device bytes of the populations (two arrays; one in place) */
    int64_t step_count;      /* time steps taken so far */
    int32_t reserved[8];
} jp_info;

typedef struct jp_solver jp_solver;

/* ---- lifecycle ---------------------------------------------------------------------------- */

/* Fill *cfg with the reference's defaults for `kind`. */
void jp_config_default(jp_config* cfg, int32_t kind);

/* Allocate a solver and put the Taylor-Green initial state in it.
 * Replaces the allocation and k_init_tgv3d launch of src/tgv3d_uniform.cu:157-161
 * (AMR: src/tgv3d_amr.cu:669-670 and the initial build gpurce_init, :776-816). */
jp_status jp_create(const jp_config* cfg, jp_solver** out);

/* Free all device memory of a solver.  Accepts NULL. */
void jp_destroy(jp_solver* s);

/* Last error message of the calling host thread ("" if none). */
const char* jp_last_error(void);

/* ABI version and build description. */
int32_t jp_abi_version(void);
const char* jp_build_info(void);

/* sizeof of the ABI structs: 0 jp_config, 1 jp_info, 2 jp_amr_counts, 3 jp_server_config,
 * 4 jp_request, 5 jp_result, 6 jp_server_stats; else 0.  Lets an FFI binding check its struct mirrors against the
 * library it loaded. */
size_t jp_sizeof(int32_t which);

/* Derived quantities (nu, tau, steps...). */
jp_status jp_get_info(const jp_solver* s, jp_info* out);

/* Re-initialise the populations with the Taylor-Green state and reset the step counter
 * (src/tgv3d_uniform.cu:63-77, src/tgv3d_amr.cu:431-440). */
jp_status jp_init_tgv(jp_solver* s);

/* ---- time stepping ------------------------------------------------------------------------ */

/* Advance `nsteps` time steps (uniform: the k_step launch of src/tgv3d_uniform.cu:194;
 * AMR: base_step, src/tgv3d_amr.cu:821-837, one coarse step each).  Asynchronous on the solver's
 * stream; errors of the launches are reported here or by the next synchronising call. */
jp_status jp_step(jp_solver* s, int64_t nsteps);

/* Wait for all work of the solver. */
jp_status jp_sync(jp_solver* s);

/* Mean kinetic energy 1/2|u|^2, mean enstrophy 1/2|omega|^2 (central differences, periodic) and
 * mean density of the current state, computed on the device with a deterministic reduction: per-cell
 * terms of a float field in double-float (within ~1e-13 relative of FP64), sums in FP64.  A uniform
 * cube in FP32/FP16/BF16 storage is reduced in one pass over its populations (no macro field); its
 * kernel's waits between warps are bounded, and JP_ERR_TIMEOUT reports one that gave up (never seen
 * in practice; out then holds NaN).  out[0]=E, out[1]=enstrophy, out[2]=mass.  Replaces k_macro +
 * the host loop of src/tgv3d_uniform.cu:169-189 and k_composite + k_diag_reduce of
 * src/tgv3d_amr.cu:882-888. */
jp_status jp_diag(jp_solver* s, double out[3]);

/* ---- population I/O (parity checks, checkpoint/restart, host-resident workloads) ----------- */

/* Number of population values (19 per cell) of AMR level `level` (0 for uniform). */
jp_status jp_population_count(const jp_solver* s, int32_t level, int64_t* count);

/* Copy the populations of `level` to a host buffer of `count` values of type `dtype`, in `layout`.
 * Shifted FP16/BF16 storage is returned unshifted (f = w_q + stored). */
jp_status jp_get_populations(jp_solver* s, int32_t level, int32_t layout, int32_t dtype,
                             void* host, int64_t count);

/* Overwrite the populations of `level` from a host buffer (the inverse of jp_get_populations).
 * From pinned memory in the native layout and type the copy is one asynchronous DMA. */
jp_status jp_set_populations(jp_solver* s, int32_t level, int32_t layout, int32_t dtype,
                             const void* host, int64_t count);

/* Upload the populations for the solver's next step while the work already queued runs: the copy
 * goes on a copy stream into a second state buffer (allocated by the first call, counted in
 * bytes_state), and the next jp_step (or ensemble step) waits for it on the device and takes it as
 * the state before its first step.  Calls in between (jp_diag, jp_get_populations, ...) still see the
 * current state, so a caller can stage call i+1's input right after call i's jp_step and overlap the
 * upload with those steps and their diagnostics.  Uniform solvers without JP_FLAG_INPLACE, flat
 * layout in the storage's own type (JP_F32 for FP32, JP_F64 for FP64; else JP_ERR_UNSUPPORTED).
 * `host` (pinned, for an asynchronous copy) must stay valid and unchanged until the step that takes
 * it has been synchronised (jp_sync, jp_diag).  JP_ERR_STATE if populations are already staged.
 * jp_init_tgv, jp_set_populations and jp_load_state set the state explicitly and discard populations
 * staged before them.  No reference counterpart: the reference uploads nothing after its initial
 * state. */
jp_status jp_stage_populations(jp_solver* s, int32_t layout, int32_t dtype, const void* host, int64_t count);

/* Macroscopic field of the current uniform state: `host` receives n^3 float4 (rho, ux, uy, uz) in
 * the linear order (z*n+y)*n+x, as k_macro writes it (src/tgv3d_uniform.cu:80-90). */
jp_status jp_get_macro(jp_solver* s, float* host, int64_t count);

/* Output fields for VTK frames, computed on the device: Q-criterion -1/2 g_ab g_ba of the central-
 * difference velocity gradient, speed |u| and (optional, may be NULL) the velocity vector, in the
 * linear order (z*n+y)*n+x.  Uniform: n = N, as write_vti computes them on the host
 * (src/tgv3d_uniform.cu:110-121); AMR: n = 4*N0 on the composite field, as k_qspeed
 * (src/tgv3d_amr.cu:553-564).  `count` = n^3. */
jp_status jp_get_output_fields(jp_solver* s, float* q, float* speed, float* velocity, int64_t count);

/* Free and total bytes of the solver's device (cudaMemGetInfo). */
jp_status jp_memory_info(jp_solver* s, int64_t* free_bytes, int64_t* total_bytes);

/* Diagnostics of a caller-owned macro field with no device allocation.  No counterpart in the
 * reference: it exists for callers that cannot call cudaMalloc when they need the numbers (a host
 * framework that owns all device memory through its own pool, a loop that must not allocate after
 * start-up).  `field_dev` holds n^3 float4 (rho, ux, uy, uz) in the order of jp_get_macro; `out_dev`
 * receives 3 doubles (mean E, mean enstrophy, mean rho), written on `stream` (a cudaStream_t; NULL =
 * default stream) without host synchronisation.  Both must be device (or managed) memory of the
 * current device, else JP_ERR_INVALID.  float_diff = 1 takes velocity differences in float (the
 * uniform solver's jp_diag), 0 exactly (the AMR composite).  Scratch lives in a fixed 384 KiB device
 * array inside the library, so fields above 268,435,456 cells (n > 645) are rejected with
 * JP_ERR_CAPACITY.  The first call on each device looks up that array's address (again after the
 * device's context was replaced, e.g. by cudaDeviceReset).
 * Calls share the array: calls that overlap on the GPU race and must be serialised by the caller. */
jp_status jp_diag_field_noalloc(const float* field_dev, int32_t n, int32_t float_diff, double* out_dev,
                                void* stream);

/* Pinned host memory for asynchronous copies (cudaMallocHost / cudaFreeHost). */
jp_status jp_host_alloc(void** ptr, size_t bytes);
void jp_host_free(void* ptr);

/* ---- AMR: adaptation and block tables ----------------------------------------------------------- */

/* Block tables of the three-level AMR, int32 with -1 = absent (src/tgv3d_amr.cu:695-701). */
typedef enum jp_table {
    JP_TABLE_REF0 = 0,   /* [cnb0] coarse block refined to level 1 */
    JP_TABLE_FOF0 = 1,   /* [cnb0] first level-1 block of a coarse block, -1 */
    JP_TABLE_RL0 = 2,    /* [nref0] refined coarse blocks in rank order */
    JP_TABLE_L1PCB = 3,  /* [nf1] parent coarse block of a level-1 block */
    JP_TABLE_L1OCT = 4,  /* [nf1] octant of a level-1 block in its parent */
    JP_TABLE_F1POS = 5,  /* [nf1] level-1 grid position of a level-1 block */
    JP_TABLE_L1GRID = 6, /* [(2N/MB)^3] level-1 block at a grid position, -1 */
    JP_TABLE_REF1 = 7,   /* [nf1] level-1 block refined to level 2 */
    JP_TABLE_FOF1 = 8,   /* [nf1] first level-2 block of a level-1 block, -1 */
    JP_TABLE_RL1 = 9,    /* [nref1] refined level-1 blocks in rank order */
    JP_TABLE_L2PL1 = 10, /* [nf2] parent level-1 block of a level-2 block */
    JP_TABLE_L2OCT = 11, /* [nf2] octant of a level-2 block */
    JP_TABLE_SKIN0 = 12, /* [n_skin0] coarse blocks refined or next to a refined one, ascending */
    JP_TABLE_SKIN1 = 13, /* [n_skin1] level-1 blocks refined or next to a refined one, ascending */
    JP_TABLE_DEEP = 14   /* [nf1] level-1 block whose 6 face neighbours exist (2:1 balance) */
} jp_table;

typedef struct jp_amr_counts {
    int32_t nref0, nf1, nref1, nf2, n_skin0, n_skin1, ndeep;
    int32_t cnb0, ng1, cap_nref0, cap1, cap_nref1, cap2;
    int32_t pad;
    int64_t hw_nf1, hw_nf2;   /* pool high-water marks (src/tgv3d_amr.cu:901-902) */
    int32_t reserved[8];
} jp_amr_counts;

/* Rebuild the refinement from the current state: sensor, exact threshold, marks, tables, migration of
 * the fine payloads, skin lists (gpurce_regrid, src/tgv3d_amr.cu:722-764).  Synchronous; only block
 * counts cross to the host.  JP_ERR_CAPACITY if a pool would overflow. */
jp_status jp_regrid(jp_solver* s);

/* Block counts, capacities and high-water marks of an AMR solver. */
jp_status jp_amr_get_counts(jp_solver* s, jp_amr_counts* out);

/* Copy one block table to `host` (capacity entries); *count receives its length. */
jp_status jp_get_table(jp_solver* s, int32_t table, int32_t* host, int64_t capacity, int64_t* count);

/* The refinement sensor of the last adaptation: level 0 per coarse block (cnb0 values), level 1 per
 * level-1 block (nf1 values); block max of |f - feq|_2 / rho (k_sensor, src/tgv3d_amr.cu:442-453). */
jp_status jp_get_sensor(jp_solver* s, int32_t level, float* host, int64_t capacity, int64_t* count);

/* Replace the computed sensor by supplied values in every later adaptation (initial build by
 * jp_init_tgv, regrid): sen0 per coarse block (cnb0 values), sen1_by_pos per level-1 grid position
 * ((2N/MB)^3 values, so a level-1 block takes the value of its position).  NULL, NULL clears.  Feeds
 * two implementations the same sensor field for bit-exact table comparisons. */
jp_status jp_set_sensor_override(jp_solver* s, const float* sen0, const float* sen1_by_pos);

/* ---- state files (extension; the reference always starts from the initial state) -------- */

/* Write the whole state of a solve to `path`: a header (kind, n, mb, storage, Re, u0, refinement
 * modes, step count) and for a uniform cube its stored populations, for an AMR solve its block
 * counts, capacities, block tables and the populations of the blocks in use.  jp_load_state into a
 * solver created with the same kind, n, mb, storage, Re, u0 and refinement modes (t*, diagnostic
 * and regrid cadence may differ) continues bit for bit where the saved solve was, including later
 * regrids.  JP_ERR_INVALID for a file of another configuration, ABI or a truncated file. */
jp_status jp_save_state(jp_solver* s, const char* path);
jp_status jp_load_state(jp_solver* s, const char* path);

/* ---- ensembles and serving (extensions; no counterpart in the reference) ------------- */

/* An ensemble steps many solvers of the same device together, on the ensemble's stream, ordered
 * after each member's pending work and before its later work.  Uniform members: one batched
 * stream-collide launch per storage format per lattice step (up to 48 cubes of any sizes per
 * launch).  AMR members: one coarse step (the 1:2:4 subcycle) with one launch per stage over the
 * blocks of all members of the same block edge, storage and step threads (up to 48 per launch);
 * jp_ensemble_step(e, k) advances AMR members by k coarse steps.  Regrids and diagnostics stay
 * per solver (jp_regrid, jp_diag) between ensemble steps. */
typedef struct jp_ensemble jp_ensemble;
jp_status jp_ensemble_create(int32_t device, jp_ensemble** out);
void jp_ensemble_destroy(jp_ensemble* e);
jp_status jp_ensemble_add(jp_ensemble* e, jp_solver* s);
jp_status jp_ensemble_remove(jp_ensemble* e, jp_solver* s);
jp_status jp_ensemble_step(jp_ensemble* e, int64_t nsteps);
/* Persistent AMR coarse steps (no counterpart in the reference; its base_step issues 18 launches per
 * coarse step, src/tgv3d_amr.cu:821-837).  mode 1: jp_ensemble_step(e, k) runs the k coarse steps of
 * up to 48 AMR members (block edge 8, rows of four cells, restrictions fused; others keep the
 * per-stage launches) in ONE cooperative launch that walks every member's per-level block and
 * cell lists stage by stage, with grid barriers between dependent stages; mode 0 (the default):
 * one launch per stage and coarse step.  Results are the same bits either way.  wait_limit_ns
 * bounds each barrier wait (0: 2 s); past it the launch stops and the next jp_ensemble_sync
 * returns JP_ERR_TIMEOUT (the members' states are then undefined).  grid: CTAs of the launch (0:
 * every CTA that can be resident). */
jp_status jp_ensemble_set_persistent(jp_ensemble* e, int32_t mode, int64_t wait_limit_ns, int32_t grid);
/* Wait for the ensemble's queued steps; JP_ERR_TIMEOUT if a persistent launch gave up at a grid
 * barrier since the last jp_ensemble_sync (the message names the phase and coarse step). */
jp_status jp_ensemble_sync(jp_ensemble* e);

/* A server runs whole Taylor-Green solves (the `uniform` / `amr` programs' runs) for a stream of
 * requests with continuous batching: requests wait in a queue until their HBM estimate fits the
 * pool budget and a slot is free, are admitted between ticks while others run, advance together
 * in batched launches issued by jp_server_tick (uniform solves: one stream-collide launch over all
 * cubes; AMR solves: one launch per stage of the coarse step over the blocks of all of them, on a
 * second stream), and leave a result with their diagnostics summary and timestamps when they
 * finish.  Diagnostics are launched in the batch and read back one tick late.  AMR creation and
 * regrids, which need read-backs, run on worker threads on each solve's own stream while the batch
 * goes on without that solve.  Device memory of served solves comes from one stream-ordered pool,
 * so solves come and go without synchronising the device. */
typedef struct jp_server jp_server;
typedef struct jp_server_config {
    int32_t device;
    int32_t max_active;      /* slots; 0 = unlimited */
    double pool_gb;          /* HBM budget for admitted solves, GiB (0 = 75% of free memory) */
    int32_t tick_steps;      /* lattice steps the uniform solves advance per tick (default 64) */
    int32_t workers;         /* host threads that create and regrid AMR solves (0 = one per core, 4..32) */
    int32_t uniform_first;   /* 1: the uniform batches' stream at the highest priority and the AMR
                                lanes at the lowest (the batches are the HBM-bound bulk); 0: equal */
    int32_t reserved[5];
} jp_server_config;
typedef struct jp_request {
    int64_t id;
    jp_config cfg;           /* kind, n, re, tstar, storage, refinement... as for jp_create */
    int32_t diag_every;      /* 0 = the programs' cadence: steps/240 (uniform), steps/160 (AMR) */
    int32_t reserved[7];
} jp_request;
typedef struct jp_result {
    int64_t id;
    int32_t status;          /* jp_status of the solve */
    int32_t valid;           /* the programs' VALID gate (src/tgv3d_uniform.cu:199) */
    int64_t steps;
    int32_t samples;         /* diagnostic samples taken */
    int32_t pad;
    double peak_tstar, peak_enstrophy, energy_ratio, mass_drift;  /* energy_ratio = E_end / E0 */
    double t_submit, t_start, t_end;   /* seconds on the server clock */
    int64_t bytes;           /* HBM estimate the solve was admitted with */
    int32_t reserved[8];
} jp_result;
jp_status jp_server_create(const jp_server_config* cfg, jp_server** out);
void jp_server_destroy(jp_server* sv);
jp_status jp_server_submit(jp_server* sv, const jp_request* req);  /* never blocks */
/* One scheduling round: retire finished solves, admit queued ones that fit, advance the active ones. */
jp_status jp_server_tick(jp_server* sv, int32_t* active, int32_t* queued);
/* Move up to `max` finished results to `out`; returns how many. */
int32_t jp_server_poll(jp_server* sv, jp_result* out, int32_t max);
/* Seconds since the server was created (the clock of jp_result timestamps). */
double jp_server_clock(const jp_server* sv);
/* Where the server's host time went: cumulative seconds of the calls made for solves, summed over
 * the tick thread and the AMR workers (so they can exceed the wall clock), and event counts. */
typedef struct jp_server_stats {
    double create_s;         /* solver creation: allocation, initial state, initial build */
    double step_s;           /* issuing lattice steps (uniform batches, AMR steps / graph replays) */
    double regrid_s;         /* AMR regrids, including their read-backs */
    double diag_s;           /* diagnostics, including the wait for the result */
    double destroy_s;        /* retiring solves */
    double tick_s;           /* inside jp_server_tick */
    int64_t solves, regrids, diags, coarse_steps;
    double uniform_gpu_s;    /* device time of the batched uniform launches (CUDA events) */
    double amr_gpu_s;        /* device time of the batched AMR launches (CUDA events) */
    int64_t reserved[6];
} jp_server_stats;
jp_status jp_server_get_stats(const jp_server* sv, jp_server_stats* out);

/* ---- autotuning (extension; no counterpart in the reference) ------------------------- */

/* Time `steps` steps of each candidate and write the fastest into *cfg: for a uniform solver the
 * thread mapping (cells per thread `vec` x `threads_per_block`), for an AMR solver the block edge
 * `mb` in {4, 8, 16} dividing n and the threads per CTA of its level steps (`threads_per_block`
 * 64 at MB=4, else 128, 256 or 512; the reference fixes MB at compile time and MB=16 cannot run
 * there, its kernels would need 4096 threads per block).  *best receives the winner's lattice
 * updates per second (AMR: work-normalised, (cnb0 + 2 nf1 + 4 nf2) MB^3 per coarse step). */
jp_status jp_autotune(jp_config* cfg, int32_t steps, double* best);

/* ---- measurement ---------------------------------------------------------------------------- */

/* Advance `nsteps` steps and return the device time of those launches, measured with CUDA events
 * recorded on the solver's own stream (the stream the kernels run on). */
jp_status jp_step_timed(jp_solver* s, int64_t nsteps, float* ms);

/* Number of kernel launches this library has issued in this process. */
int64_t jp_launch_count(void);

#ifdef __cplusplus
}
#endif

#endif /* JP_H */
