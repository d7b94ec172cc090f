/* dugks_gpu.h -- C ABI of the GB300 DUGKS time-step library (libdugks_gpu.so).
 *
 * The library replaces the body of the reference solver's time loop,
 * DUGKS2DSolver() (Ark/Cpp/DUGKS2DSolver.cpp:148-337), for Cartesian meshes
 * of unit cells that are periodic in x and either periodic or bounce-back
 * walls in y.  One handle owns one case: its distributions and macroscopic
 * fields stay resident in GPU memory between calls.  Every call returns a
 * dugks_status; no C++ exception crosses this ABI.  A handle is used by one
 * host thread at a time; kernels run asynchronously on the stream given to
 * dugks_gpu_step (NULL = the legacy default stream) and every call that
 * returns host data synchronises that stream first.
 *
 * Layouts: cell fields are [ny][nx] row-major doubles, cell (i,j) at
 * j*nx+i with x = i+0.5, y = j+0.5.  Distributions are [Q][ny][nx], the
 * discrete-velocity order of the reference model (D2Q9: 0,E,NE,N,NW,W,SW,S,SE,
 * Ark/Lib/D2Q9.h:86-88; D2V16: Ark/Lib/D2V16.cpp:53-66).
 */
#ifndef DUGKS_GPU_H
#define DUGKS_GPU_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum dugks_status {
    DUGKS_OK = 0,
    DUGKS_EINVAL = 1,   /* bad argument or unsupported combination */
    DUGKS_ENOMEM = 2,   /* device or host allocation failed */
    DUGKS_ECUDA = 3,    /* a CUDA call failed; see dugks_gpu_last_error */
    DUGKS_ETIMEOUT = 4, /* a bounded device wait gave up */
    DUGKS_ENAN = 5      /* a NaN/Inf was found in the state */
} dugks_status;

/* Velocity model + multiphase model (Ark/Makefile:7 QModel + ZeroFlip.h flips). */
typedef enum dugks_model {
    DUGKS_MODEL_AC = 0,   /* D2Q9AC: Allen-Cahn, u forced to 0 (Ark/Lib/D2Q9AC.cpp) */
    DUGKS_MODEL_HCZ = 1,  /* D2Q9HCZ: Allen-Cahn, pressure-based f (Ark/Lib/D2Q9HCZ.cpp) */
    DUGKS_MODEL_PP9 = 2,  /* D2Q9PP: pseudopotential (Ark/Lib/D2Q9PP.cpp, Ark/Cpp/PseudoP.cpp) */
    DUGKS_MODEL_PP16 = 3  /* D2V16 pseudopotential (Ark/Lib/D2V16.cpp restated) */
} dugks_model;

typedef enum dugks_precision {
    DUGKS_FP64 = 0,       /* plain FP64 drop-in: every operation rounded like the
                             reference (no FMA contraction), bit-identical results */
    DUGKS_FP32_DEV = 1,   /* FP32 storage of small deviations and remainders (the
                             phase field as a float-float pair; the pseudopotential
                             density in FP64).  Pseudopotential models: the multi-pass
                             step, or with DUGKS_PP_PASSES=1 in the environment at
                             create time the single-pass streaming step (same results) */
    DUGKS_FP64_FMA = 2,   /* FP64 with FMA contraction and reciprocal multiplies:
                             equal to the reference to rounding, fewer FP64 ops */
    DUGKS_FP64_FUSED = 3  /* the fused one-kernel deviation-form step of
                             DUGKS_FP32_DEV, carried out in FP64 */
} dugks_precision;

/* Case parameters: the primary inputs of Ark/Constant/ZeroReference.h and
 * Ark/Constant/ZeroNamespace.h; every derived constant (dt, tau0, beta,
 * kappa, ...) is computed inside the library with the reference's formulas.
 * ChLength = NL = nx, MinL = 1, R0 = 1, T0 = 1/3, Rho0 = 1, p0 = 1, CFL 0.5. */
typedef struct dugks_case {
    int model;          /* dugks_model */
    int precision;      /* dugks_precision */
    double Mu0;         /* reference dynamic viscosity (nu0 = Mu0 / Rho0) */
    double M_Phi;       /* phase-field mobility */
    double W;           /* interface width (Cn = W / ChLength) */
    double Sigma;       /* surface tension */
    double RhoL, RhoV;  /* densities of phi = 1 and phi = 0 */
    double Gy;          /* gravity: Fy -= Gy*(rho - RhoL); 0 = off */
    double Tr;          /* pseudopotential: T / Tc */
    double aCS;         /* Carnahan-Starling attraction a (b = 4, R = 1) */
    double Tc_CS;       /* Carnahan-Starling critical temperature (0.3773 a / b) */
    double d2v16_c;     /* D2V16 lattice speed c (1.2 in the reference) */
    int flux_scheme;    /* dugks_flux_scheme: the face reconstruction (Case.ark "Flux Scheme") */
    int wall_scheme;    /* dugks_wall_scheme: the treatment of y_walls */
} dugks_case_t;

/* Wall faces (Ark/Constant/ZeroFlip.h _Wall_3_BCs_*).  BB (the default):
 * the face computed like an interior face from the extrapolated ghost row,
 * then bounce-back of the entering directions (Flux_2D + Wall_3_BB,
 * Ark/Cpp/Boundary.cpp:118-139).  NEE: the face equilibrium at the owner's
 * extrapolated phi and rho, its pressure and zero velocity, plus the owner's
 * non-equilibrium part, then bounce-back (Wall_3_NEE,
 * Ark/Cpp/Boundary.cpp:140-184).  NEE runs with DUGKS_FP64 / DUGKS_FP64_FMA
 * (bit-identical to the reference) and DUGKS_FP32_DEV (grids of at least 8
 * rows; within 1e-5 of FP64) for the Allen-Cahn models. */
typedef enum dugks_wall_scheme {
    DUGKS_WALL_BB = 0,
    DUGKS_WALL_NEE = 1
} dugks_wall_scheme;

/* Half-step face reconstruction (Ark/Constant/ZeroFlip.h _FLUX_SCHEME_*_ARK).
 * CD (the reference's default): central value and gradients of the two cells
 * at the face (CD_Interior_phi_Bh, Ark/Cpp/DUGKS2DSolver.cpp:604-687).  UW:
 * the upwind cell's value extrapolated with its 6-point isotropic gradient
 * (Grad_VS_6points, Ark/Lib/GradSchemeBasic.h:95-126; UW_Interior_phi_Bh,
 * Ark/Cpp/DUGKS2DSolver.cpp:558-603,689-706), both cells averaged for
 * velocities along the face.  UW runs with the plain FP64 precisions
 * (DUGKS_FP64, DUGKS_FP64_FMA) and with DUGKS_FP32_DEV (four launches a step:
 * collision, gradients, faces, update), the Allen-Cahn models and periodic y:
 * the reference's UW with walls reads the gradients of its wall shadow cells,
 * which it never writes (uninitialised memory).  Serving runs UW cases in solo
 * lanes.  UW_LS and UW_4P are UW with the reference's other cell gradients, the
 * least-squares one (Grad_VS_LS, Ark/Cpp/GradScheme.cpp:219-231 ->
 * Ark/Lib/GradSchemeBasic.h:127-152, weights from Grad_LSMatrix :49-75) and the
 * 4-point central one (Grad_VS_4points :191-204 -> GradSchemeBasic.h:76-94), which
 * the reference selects by editing the gradient call at
 * Ark/Cpp/DUGKS2DSolver.cpp:201-203; same precisions and restrictions as UW. */
typedef enum dugks_flux_scheme {
    DUGKS_FLUX_CD = 0,
    DUGKS_FLUX_UW = 1,
    DUGKS_FLUX_UW_LS = 2,
    DUGKS_FLUX_UW_4P = 3
} dugks_flux_scheme;

typedef struct dugks_grid {
    int nx, ny;         /* cells; nx, ny >= 3 */
    int y_walls;        /* 0: periodic in y; 1: bounce-back walls top and bottom */
} dugks_grid_t;

typedef struct dugks_handle dugks_handle_t;

/* Field ids for dugks_gpu_set_field / dugks_gpu_get_field.  The first group
 * is the macroscopic state the reference keeps in MacroQuantity
 * (Ark/Header/Macroscopic.h:32-44): DUGKS_F_PHIX/PHIY hold the phase-field
 * source vector after MacroSource (Ark/Cpp/SourceM.cpp:47-58). */
typedef enum dugks_field {
    DUGKS_F_RHO = 0, DUGKS_F_U, DUGKS_F_V, DUGKS_F_P, DUGKS_F_PHI, DUGKS_F_TAU,
    DUGKS_F_PHIX, DUGKS_F_PHIY, DUGKS_F_RHOX, DUGKS_F_RHOY, DUGKS_F_FX, DUGKS_F_FY,
    DUGKS_F_PREVPHIU, DUGKS_F_PREVPHIV, DUGKS_F_PSI, DUGKS_F_SCG,
    DUGKS_F_NFIELDS
} dugks_field;

typedef struct dugks_reductions {
    double sum_rho;     /* sum of rho over cells (Ark/Cpp/DUGKS2DSolver.cpp:793-806) */
    double sum_phi;     /* sum of phi: phase-field mass */
    double residual;    /* ||rho - rho_last||2 / ||rho||2 since the previous call
                           (Ark/Cpp/DUGKS2DSolver.cpp:807-820); 1.0 on the first call */
    int64_t steps;      /* steps done since upload */
} dugks_reductions_t;

/* Create a solver; allocates all device memory.  replaces the reference's
 * mesh construction + AllocateResource (Ark/Cpp/main.cpp:106-131). */
int dugks_gpu_create(const dugks_case_t *c, const dugks_grid_t *g, dugks_handle_t **out);

/* Number of discrete velocities of the handle's model (9 or 16). */
int dugks_gpu_nq(const dugks_handle_t *h);

/* Upload a full state: f and hdist are [Q][ny][nx] (hdist ignored for the
 * pseudopotential models, may be NULL); aux is [DUGKS_F_NFIELDS][ny][nx] in
 * dugks_field order.  The next step uses aux as-is (like the reference's
 * first step after an initialisation function).  Host arrays in pinned, mapped
 * memory (cudaHostAlloc) are read in place by the DUGKS_FP32_DEV and
 * DUGKS_FP64_FUSED conversion kernels; other memory is copied through staging
 * planes.  The results are the same either way. */
int dugks_gpu_upload(dugks_handle_t *h, const double *f, const double *hdist, const double *aux);

/* Initialise on the host like the reference initialisation functions and
 * upload.  kind: 0 AC_Drop (Ark/Cpp/Preprocess.cpp:705-760, light phase
 * inside), 1 droplet with the heavy phase inside, 2 Rayleigh-Taylor
 * interface y = Lx(2 + 0.1 cos(2 pi x/Lx)) (heavy above), 3 SCMP_Drop
 * (Ark/Cpp/Preprocess.cpp:337-401), 4 seeded density noise
 * rho = p0 (1 + p1 U(-1,1)) with a 64-bit LCG.  params: kind 0/1: radius
 * (<0: 0.36 ChLength); kind 2: interface height and cosine amplitude in
 * units of nx (default 2, 0.1) and white-noise amplitude on phi (default 0);
 * kind 3: rho_l, rho_v, radius (<0: 0.25 ChLength); kind 4: rho0, amplitude;
 * seed used by kinds 2 (noise) and 4. */
int dugks_gpu_init(dugks_handle_t *h, int kind, const double *params, int nparams, uint64_t seed);

/* Advance nsteps time steps on `stream` (a cudaStream_t, NULL = default). */
int dugks_gpu_step(dugks_handle_t *h, int nsteps, void *stream);

/* Same as dugks_gpu_step, with CUDA events recorded between the kernels of
 * every step; ms_per_phase[k] receives the summed device time of phase k
 * (0 collision, 1 faces (both passes), 2 update) and *nphases = 3.  Used by
 * the benchmark to time the dominant kernel live; synchronises the stream. */
int dugks_gpu_step_profiled(dugks_handle_t *h, int nsteps, void *stream, double *ms_per_phase, int *nphases);

/* Sum of rho, sum of phi and the density residual (FP64 device reductions).
 * DUGKS_ETIMEOUT: a step of a DUGKS_FP32_DEV handle had a TMA row load that did
 * not complete within its bounded wait (the state is then not valid). */
int dugks_gpu_reduce(dugks_handle_t *h, dugks_reductions_t *r);

/* Download the macroscopic fields (any pointer may be NULL): [ny][nx] each. */
int dugks_gpu_download(dugks_handle_t *h, double *rho, double *u, double *v, double *phi, double *p);

/* Single field / distribution access.  which: 0 = f, 1 = h. */
int dugks_gpu_get_field(dugks_handle_t *h, int field, double *out);
int dugks_gpu_set_field(dugks_handle_t *h, int field, const double *in);
int dugks_gpu_get_dist(dugks_handle_t *h, int which, double *out);

/* Scan the state for NaN/Inf: DUGKS_OK or DUGKS_ENAN (DUGKS_ETIMEOUT as for
 * dugks_gpu_reduce). */
int dugks_gpu_check_finite(dugks_handle_t *h);

/* Output quantities of the Allen-Cahn models.
 * dugks_gpu_drop_l2 replaces AC_Drop_L2Norm (Ark/Cpp/Output.cpp:226-238): the
 * relative L2 distance sqrt(sum (phi - phi_A)^2 / sum phi_A^2) of the phase field
 * to the analytic drop profile (Ark/Cpp/Preprocess.cpp:402-438) of the radius and
 * phase orientation the last dugks_gpu_init (kind 0 or 1) placed, centred at
 * (nx/2, nx/2), summed on the host in the reference's cell order (the value the
 * reference prints).  DUGKS_EINVAL for a handle not initialised as a drop.
 * dugks_gpu_thermo_pressure replaces thermoPressure (Ark/Cpp/Output.cpp:146-163)
 * for every cell, out [ny][nx]: pZero(phi) - kappa phi lap(phi) + kappa |grad phi|^2 / 2 + p,
 * from the state the last step's MacroSource saw. */
int dugks_gpu_drop_l2(dugks_handle_t *h, double *l2);
int dugks_gpu_thermo_pressure(dugks_handle_t *h, double *out);

/* Last error message of the handle (or of the last failed create if h is NULL). */
int dugks_gpu_last_error(const dugks_handle_t *h, char *buf, size_t len);

/* Kernel launches issued by this handle so far (for launch accounting). */
int64_t dugks_gpu_launch_count(const dugks_handle_t *h);

int dugks_gpu_destroy(dugks_handle_t *h);

/* Checkpoint / restart (no reference counterpart: its FlowField files hold the
 * macroscopic fields only, Ark/Cpp/Output.cpp:537-606, so a reference run
 * cannot restart).  dugks_gpu_checkpoint writes the handle's whole device state
 * (distributions, macroscopic and auxiliary fields, ping-pong orientation,
 * step counter and the constants an upload derives) into buf, which must hold
 * dugks_gpu_checkpoint_bytes(h) bytes; it synchronises the handle's stream.
 * dugks_gpu_restore loads such a buffer into a handle created with the same
 * case and grid (DUGKS_EINVAL otherwise); the handle then continues bit for bit
 * as the saved one would have. */
int dugks_gpu_checkpoint_bytes(const dugks_handle_t *h, size_t *bytes);
/* Steps done since the upload (after a restore: since the saved run's upload). */
int dugks_gpu_step_count(const dugks_handle_t *h, int64_t *steps);
int dugks_gpu_checkpoint(dugks_handle_t *h, void *buf, size_t len);
int dugks_gpu_restore(dugks_handle_t *h, const void *buf, size_t len);

/* No counterpart in the reference.  For callers that must not allocate
 * device memory themselves or through this library -- a host that hands out
 * a fixed memory budget or its own pool, a plugin running inside another
 * runtime, a loop that may not allocate once running -- this advances a
 * caller-owned device state by nsteps with no cudaMalloc/cudaFree: all scratch
 * (f-bar-plus, face fluxes, ghost rows) lives in one fixed file-scope device
 * array of about 2 MB that every GPU loading the library keeps until exit.
 * d_f, d_h: device [9][ny][nx]; d_aux: device [DUGKS_F_NFIELDS][ny][nx], the
 * same contents dugks_gpu_upload takes; all three are updated in place and
 * are complete on return (the last step's MacroSource is applied).  Limits:
 * models DUGKS_MODEL_AC/HCZ, precision DUGKS_FP64 or DUGKS_FP64_FMA,
 * nx*ny <= 4096 cells (larger grids return DUGKS_EINVAL with a message in
 * dugks_gpu_last_error(NULL, ...)).  Every call outside a stream capture
 * looks up the array's device address (cudaGetSymbolAddress), so a device
 * reset between calls is safe; a call on a capturing stream reuses the address
 * the last uncaptured call found: make one call before the first capture, and
 * one again after a device reset before capturing.  All calls share the one array: calls whose
 * work overlaps on the GPU (other streams, other host threads) race on it
 * and must be serialised by the caller.  Asynchronous on `stream`. */
int dugks_gpu_step_noalloc(const dugks_case_t *c, const dugks_grid_t *g, double *d_f, double *d_h,
                           double *d_aux, int nsteps, void *stream);

/* ---- Serving: a request loop that solves many cases on one GPU.
 *
 * No reference counterpart (the reference solves one case per process,
 * Ark/Cpp/main.cpp:134).  Cases are admitted first-in first-out while their
 * device footprint fits the byte budget; each case's state stays resident
 * until it finishes.  FP32-storage Allen-Cahn cases (AC, HCZ) run together:
 * every chunk of `chunk_steps` steps is one captured CUDA graph of persistent
 * launches over a table of (case, tile) entries, so cases that arrive while
 * others run join at the next chunk and finished cases leave.  Other cases
 * (FP64, pseudopotential) run on `solo_lanes` lanes, one case per lane at a
 * time, each lane on its own stream, overlapping one another and the
 * batched work.  A case's result does not depend on the other cases
 * (bit-identical alone and in a mix).
 *
 * Like the reference's time loop (Ark/Cpp/DUGKS2DSolver.cpp:164 with
 * Update_Residual at :807-835 every ResidualControl steps,
 * Ark/Constant/ZeroNamespace.h:173-177), a case is checked every
 * `check_every` steps: it stops converged when the density residual is at or
 * below `residual_tol`, and fails (DUGKS_SRV_STOP_DIVERGED) when its state is
 * no longer finite.  With `out_dir` set, the state at step 0, every
 * `snapshot_every` steps and at the end is written there as FlowField files
 * in the layout and names of the reference's Output_Flowfield
 * (Ark/Cpp/Output.cpp:537-606); the fields are copied to pinned host buffers
 * and a writer thread formats and writes them while the case runs on. */
typedef struct dugks_srv dugks_srv_t;

typedef struct dugks_srv_config {
    size_t max_bytes;  /* device bytes for resident cases; 0: 85% of the free memory */
    int chunk_steps;   /* steps per captured graph launch; 0: 64 */
    int solo_lanes;    /* lanes for the cases that are not batched; 0: 4 */
    int reserved[5];
} dugks_srv_config_t;

/* One case for dugks_srv_submit_request. */
typedef struct dugks_srv_request {
    dugks_case_t cs;
    dugks_grid_t grid;
    int init_kind;         /* dugks_gpu_init kind, params and seed */
    int nparams;
    const double *params;
    uint64_t seed;
    int64_t nsteps;        /* step limit (the reference's End_Step) */
    double residual_tol;   /* stop once the residual at a check is <= this (RESIDUAL); 0: never */
    int check_every;       /* steps between residual / finiteness checks (ResidualControl); 0: 1000 */
    int snapshot_every;    /* steps between FlowField files (writeFileControl); 0: step 0 and the end only */
    const char *out_dir;   /* existing directory for the FlowField files; NULL: no files */
} dugks_srv_request_t;

typedef enum dugks_srv_stop {
    DUGKS_SRV_STOP_NONE = 0,      /* running, or reached its step limit */
    DUGKS_SRV_STOP_CONVERGED = 1, /* residual at or below residual_tol */
    DUGKS_SRV_STOP_DIVERGED = 2   /* non-finite state at a check (state DUGKS_SRV_FAILED) */
} dugks_srv_stop_t;

typedef enum dugks_srv_state {
    DUGKS_SRV_QUEUED = 0,
    DUGKS_SRV_RUNNING = 1,
    DUGKS_SRV_DONE = 2,
    DUGKS_SRV_CANCELLED = 3,
    DUGKS_SRV_FAILED = 4
} dugks_srv_state_t;

typedef struct dugks_srv_status {
    int state;         /* dugks_srv_state_t */
    int batched;       /* 1: runs in the batched lane */
    int64_t nsteps, steps_done;
    size_t bytes;      /* device footprint */
    double t_submit, t_start, t_done;  /* seconds since dugks_srv_create */
    int stop_reason;   /* dugks_srv_stop_t */
    int files;         /* FlowField files written so far */
    double residual;   /* residual at the last check; -1 before the first */
} dugks_srv_status_t;

typedef struct dugks_srv_stats {
    int64_t submitted, completed, cancelled, failed;
    int64_t cell_updates;     /* steps x cells of the cases that ended (done or stopped) */
    int64_t chunks, graphs_captured, launches;
    int max_resident;         /* most cases resident at once */
    size_t bytes_in_use, bytes_peak, max_bytes;
    double busy_s;            /* batched lane: time with work on the device */
    int64_t converged, diverged;  /* cases stopped by the residual rule / as non-finite */
    int64_t files_written;
    int64_t solo_steps;       /* steps run by the solo lanes */
} dugks_srv_stats_t;

int dugks_srv_create(const dugks_srv_config_t *cfg, dugks_srv_t **out);
/* Queue a case: initialise it like dugks_gpu_init(kind, params, nparams,
 * seed) and run nsteps steps.  Returns at once with the case id. */
int dugks_srv_submit(dugks_srv_t *s, const dugks_case_t *c, const dugks_grid_t *g, int init_kind,
                     const double *params, int nparams, uint64_t seed, int64_t nsteps, int64_t *id);
/* Queue a case with the stopping rule and FlowField output of `rq`
 * (dugks_srv_submit is this with residual_tol 0, check_every 0, no files). */
int dugks_srv_submit_request(dugks_srv_t *s, const dugks_srv_request_t *rq, int64_t *id);
int dugks_srv_poll(dugks_srv_t *s, int64_t id, dugks_srv_status_t *st);
/* Block until the case is done, cancelled or failed, or timeout_s passes
 * (DUGKS_ETIMEOUT; timeout_s < 0: no limit). */
int dugks_srv_wait(dugks_srv_t *s, int64_t id, double timeout_s, dugks_srv_status_t *st);
/* Fields of a finished case ([ny][nx] each, like dugks_gpu_download); any
 * pointer may be NULL.  The result is kept until dugks_srv_release. */
int dugks_srv_result(dugks_srv_t *s, int64_t id, double *rho, double *u, double *v, double *phi, double *p);
int dugks_srv_release(dugks_srv_t *s, int64_t id);
int dugks_srv_cancel(dugks_srv_t *s, int64_t id);
int dugks_srv_stats(dugks_srv_t *s, dugks_srv_stats_t *out);
int dugks_srv_last_error(dugks_srv_t *s, char *buf, size_t len);
/* Cancels what has not finished and waits for the device work to end. */
int dugks_srv_destroy(dugks_srv_t *s);

/* ---- Slab decomposition: one FP32-storage Allen-Cahn case split along y into
 * partitions (on one or several devices), each with two halo rows per side
 * exchanged after every step; bit-identical to the undivided case.  No
 * reference counterpart (the reference runs one OpenMP process per case). */
typedef struct dugks_slabs dugks_slabs_t;

/* Host-only plan: partition p owns rows [row0[p], row0[p] + nrows[p]); lo[p] /
 * hi[p] is the partition below / above (-1: the grid's wall).  Needs at least
 * 8 rows per partition. */
int dugks_slabs_plan(int ny, int y_walls, int nparts, int *row0, int *nrows, int *lo, int *hi);
/* devices: the CUDA device of each partition (NULL: all on the current one). */
int dugks_slabs_create(const dugks_case_t *c, const dugks_grid_t *g, int nparts, const int *devices,
                       dugks_slabs_t **out);
int dugks_slabs_init(dugks_slabs_t *s, int kind, const double *params, int nparams, uint64_t seed);
/* The halo copies issued after every step, in issue order (host-only, the same
 * list dugks_slabs_step executes): `rows` rows of all state planes from local row
 * src_row of partition src to local row dst_row of partition dst (local row 0 =
 * the partition's first owned row; -2, -1 = its lower halo, nrows, nrows + 1 = its
 * upper halo).  *count = the number of copies; out may be NULL to ask only that,
 * else it holds max entries. */
typedef struct dugks_halo_copy {
    int src, src_row, dst, dst_row, rows;
} dugks_halo_copy_t;
int dugks_slabs_schedule(int ny, int y_walls, int nparts, dugks_halo_copy_t *out, int max, int *count);
int dugks_slabs_step(dugks_slabs_t *s, int nsteps);
/* Sum of rho, sum of phi and the density residual over the whole grid, as
 * dugks_gpu_reduce: each partition reduces its rows on its device, the host adds
 * the partitions in order (equal to the undivided case's sums to rounding). */
int dugks_slabs_reduce(dugks_slabs_t *s, dugks_reductions_t *r);
/* the whole grid's fields ([ny][nx] each); any pointer may be NULL */
int dugks_slabs_download(dugks_slabs_t *s, double *rho, double *u, double *v, double *phi, double *p);
int64_t dugks_slabs_launch_count(const dugks_slabs_t *s);
int dugks_slabs_destroy(dugks_slabs_t *s);

#ifdef __cplusplus
}
#endif
#endif
