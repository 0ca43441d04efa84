/*
 * gbfwi — GB300-native drop-in for the hot path of libccy/inv.cu.
 *
 * C ABI of libgbfwi.so: plain pointers, sizes and opaque handles. Every call
 * returns a status (GB_OK == 0) unless it returns a handle or pointer (NULL on
 * error); gb_last_error() describes the last failure on the calling thread.
 * Calls are synchronous, like the reference's default-stream code: when a
 * call returns, its device results are visible to the next call and to any
 * other CUDA user of the device.
 *
 * Device buffers returned by gb_solver_ptr() use the reference layout
 * float[nx*nz] with k = i*nz + j (z contiguous) for grids, and
 * float[nrec*nt] with k = ir*nt + it for traces. They stay valid for the
 * solver's lifetime and may be updated in place between calls (the
 * reference's optimizer aliases lambda/mu/rho and k_* this way).
 *
 * Each declaration names the reference interface it replaces.
 */
#ifndef GBFWI_H
#define GBFWI_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GB_VERSION 1

/* status codes */
#define GB_OK 0
#define GB_ERR_ARG 1    /* invalid argument or size */
#define GB_ERR_CUDA 2   /* CUDA runtime or launch failure */
#define GB_ERR_IO 3     /* file missing or malformed */
#define GB_ERR_BUDGET 4 /* request does not fit the HBM budget */
#define GB_ERR_STATE 5  /* call not valid in the current state */
#define GB_ERR_MODEL 6  /* model size does not match the grid */

/* gb_solver_ptr() selectors */
enum gb_buffer {
    GB_OUT_X = 0, GB_OUT_Y, GB_OUT_Z,
    GB_ADSTF_X, GB_ADSTF_Y, GB_ADSTF_Z,
    GB_LAMBDA, GB_MU, GB_RHO,
    GB_K_LAMBDA, GB_K_MU, GB_K_RHO,
    GB_STF_X, GB_STF_Y, GB_STF_Z
};

/* Last error message of the calling thread (never NULL). */
const char *gb_last_error(void);
/* ABI version (GB_VERSION). */
int gb_version(void);

/* ------------------------------------------------------------------ Config
 * Replaces class Config (lib/config.h:86-108) and the argument handling of
 * main (inv.cu:12-30). */
typedef struct gb_config gb_config;

/* Config(map&) (lib/config.h:92-108): overrides are "-key=value" or
 * "key=value" strings that win over config.ini; reads sources.dat and
 * stations.dat; honours `clean` and creates dir/output. */
gb_config *gb_config_load(const char *dir, int noverrides, const char *const *overrides);
/* Empty configuration rooted at dir (for callers without files). */
gb_config *gb_config_new(const char *dir);
void gb_config_free(gb_config *cfg);
/* Sets one key as if read from config.ini with the highest priority. */
int gb_config_set(gb_config *cfg, const char *key, const char *value);
/* config->f / config->i lookups; missing keys read as 0. */
int gb_config_has(const gb_config *cfg, const char *key);
float gb_config_f(const gb_config *cfg, const char *key);
int gb_config_i(const gb_config *cfg, const char *key);
const char *gb_config_path(const gb_config *cfg);
/* config->src (7 floats: x z type f0 t0 angle amp) and config->rec (x z). */
int gb_config_nsrc(const gb_config *cfg);
int gb_config_nrec(const gb_config *cfg);
int gb_config_source(const gb_config *cfg, int is, float out[7]);
int gb_config_station(const gb_config *cfg, int ir, float out[2]);
int gb_config_add_source(gb_config *cfg, const float src[7]);
int gb_config_add_station(gb_config *cfg, const float rec[2]);

/* ------------------------------------------------------------------ Solver
 * Replaces class Solver (solver/solver.h:7-268) and FdmSolver
 * (solver/fdm.h:222-613), selected by solver = 0 (lib/index.h:33-38). */
typedef struct gb_solver gb_solver;

/* Solver::init + FdmSolver::init (solver/solver.h:158-224,
 * solver/fdm.h:350-462): grid inferred from model_true/proc000000_{x,z}.bin. */
gb_solver *gb_solver_create(const gb_config *cfg);
/* The grid gb_solver_create infers, on the host (no device work): nx, nz,
 * xmax, zmax and the point count from <dir>/model_true/proc000000_{x,z}.bin
 * as FdmSolver::init does (solver/fdm.h:354-391). */
int gb_infer_grid(const char *dir, int *nx, int *nz, float *xmax, float *zmax, int *npt);
/* Same, with the grid given instead of read from model files:
 * dx = xmax/(nx-1), dz = zmax/(nz-1). */
gb_solver *gb_solver_create_grid(const gb_config *cfg, int nx, int nz, float xmax, float zmax);
void gb_solver_destroy(gb_solver *s);

/* Solver::importModel + FdmSolver::importModel (solver/solver.h:225-252,
 * solver/fdm.h:463-476): reads model_true (model_true != 0) or model_init,
 * maps the points onto the grid (mesh2grid, nearest point, first wins) and
 * converts vp/vs to lambda/mu when model_type == 0. */
int gb_import_model(gb_solver *s, int model_true);
/* The same from host arrays of npt model points (x, z, vp|lambda, vs|mu, rho). */
int gb_set_model_points(gb_solver *s, int npt, const float *x, const float *z, const float *a, const float *b,
                        const float *rho);
/* Host lambda, mu, rho already on the grid (reference layout). */
int gb_set_model_grid(gb_solver *s, const float *lambda, const float *mu, const float *rho);

/* FdmSolver::runForward (solver/fdm.h:515-570). isrc < 0 fires every source
 * at once. trace != 0 writes output/{v|u}{x,y,z}_NNNNNN.su; snapshot != 0
 * writes wavefield snapshots every wfe steps. */
int gb_run_forward(gb_solver *s, int isrc, int trace, int snapshot);
/* FdmSolver::runAdjoint (solver/fdm.h:571-612): adjoint sources from
 * GB_ADSTF_*, kernels accumulated into GB_K_*. snapshot uses wae. */
int gb_run_adjoint(gb_solver *s, int isrc, int snapshot);
/* FdmSolver::initKernels (solver/fdm.h:495-499). */
int gb_init_kernels(gb_solver *s);
/* FdmSolver::exportAxis (solver/fdm.h:500-514). */
int gb_export_axis(gb_solver *s);
/* FdmSolver::exportModel (solver/fdm.h:477-494). */
int gb_export_model(gb_solver *s, int n);
/* Solver::exportKernel (solver/solver.h:255-259). */
int gb_export_kernel(gb_solver *s, int n);
/* Solver::exportTraces (solver/solver.h:38-108) of the last forward run. */
int gb_export_traces(gb_solver *s, int isrc);
/* The SU files alone, on the host (no device work): nrec traces of nt
 * samples in host memory with Solver::exportTraces' 240-byte headers
 * (solver/solver.h:38-108; source at xs, zs, receivers at rec_x, rec_z), and
 * their reading as Misfit::importTraces (misfit/misfit.h:52-90), headers
 * skipped. */
int gb_su_write(const char *file, const float *traces, int nrec, int nt, float dt, float xs, float zs,
                const float *rec_x, const float *rec_z);
int gb_su_read(const char *file, float *traces, int nrec, int nt);

/* Public device buffers (Solver's public members, solver/solver.h:122-156). */
float *gb_solver_ptr(gb_solver *s, int which);
int gb_solver_dims(const gb_solver *s, int *nx, int *nz, int *nt, int *nsrc, int *nrec);
int gb_solver_steps(const gb_solver *s, float *dx, float *dz, float *dt);

/* Batched extension of runForward/runAdjoint: n shots propagate together in
 * one launch per time step (CUDA-graph captured). Shot b of the call uses
 * batch slot b; its traces/adjoint sources are gb_slot_ptr(s, b, GB_OUT_*),
 * gb_slot_ptr(s, b, GB_ADSTF_*). n must not exceed the batch capacity. The
 * adjoint batch accumulates every slot into GB_K_*. */
int gb_run_forward_batch(gb_solver *s, const int *isrc, int n);
int gb_run_adjoint_batch(gb_solver *s, const int *isrc, int n);
float *gb_slot_ptr(gb_solver *s, int slot, int which);
int gb_solver_batch_capacity(gb_solver *s);
/* Runtime options: "batch" (slots, 0 = from the HBM budget), "graphs" (0/1),
 * "ckpt" (0 FP32, 1 BF16, 2 FP16), "tile" (0 autotune, 1..20 fixed),
 * "cluster" (1: run whole passes in thread-block clusters when a shot's
 * state fits in their shared memory, with the cluster size chosen by
 * occupancy; 2..16: that cluster size; 0: never), "tma" (1: the marching
 * kernel loads grid columns with bulk tensor copies when nz % 4 == 0,
 * default; 0: per-thread cp.async), "cluster_stage" (1: a cluster adjoint
 * stages each checkpoint in shared memory before the kernel accumulation when
 * it fits; 0: reads it from HBM, default), "cluster_kacc" (1: a cluster
 * adjoint keeps each shot's kernels in shared memory for the whole pass when
 * they fit, default; 0: adds into an HBM buffer), "cluster_shift" (1: the
 * cluster pass shifts the rows of each thread group's columns in shared
 * memory so that no warp meets bank conflicts, when it fits, default; 0:
 * unshifted rows), "cluster_snap" (1: a cluster adjoint stores its state at
 * every accumulation step and a separate kernel accumulates the kernels
 * after the pass, when that state fits in a quarter of the free device
 * memory, default; 0: accumulates in the pass), "pipeline" (1: a gradient
 * whose cluster passes run in more than one round of resident clusters
 * overlaps each round's misfit with the next forward round and the previous
 * adjoint round, default; 0: forward, misfit and adjoint one after another),
 * "cluster_qm" (columns per
 * thread of the cluster pass: 0 = chosen with the cluster size, or 4, 8, 10,
 * 12, 16, 20, 24), "snap_async" (1: wavefield snapshots are copied on the
 * device into a ring of staging buffers and written to their files by a
 * writer thread while the time loop goes on, default; 0: a blocking copy and
 * write per field, as the reference does; either way every file is written
 * when the call returns), "hbm_budget_gb". Options
 * change no forward result; "ckpt" changes kernels by the checkpoint
 * rounding and "cluster" by the order in which shots are summed. */
int gb_solver_set_option(gb_solver *s, const char *key, double value);

/* Timing of the solver since the last reset (CUDA events on the solver's
 * stream). step_ms / step_launches: fused step kernels timed in windows of
 * consecutive launches; launches: kernels (or graph kernel nodes) enqueued.
 * tile_tz, tile_tx: kernel configuration of the last pass (tile_tz = -R for
 * a cluster-resident pass of R-CTA clusters); march_bulk: 1 when the last
 * marching-kernel pass loaded its columns with bulk tensor copies;
 * cluster_adj: shared-memory use of the last cluster-resident adjoint pass,
 * bit 0 checkpoints staged, bit 1 kernels accumulated there, bit 2 adjoint
 * state stored and the kernels accumulated after the pass; cluster_shift:
 * row shift between thread groups in the last cluster-resident pass's
 * shared-memory layout (0: unshifted). */
typedef struct {
    double forward_ms, adjoint_ms, misfit_ms, filter_ms;
    double step_ms;
    long long step_launches;
    long long launches;
    long long cell_updates;
    int tile_tz, tile_tx, batch_capacity;
    int march_bulk;
    int cluster_adj, cluster_shift;
} gb_stats;
int gb_solver_stats(gb_solver *s, gb_stats *out, int reset);

/* ------------------------------------------------------------------ Filter
 * Replaces class Filter / GaussianFilter (filter/filter.h:3-15,
 * filter/gaussian.h:37-61), selected by filter = 0. The smoothing is the
 * reference's: one-sided (causal) Gaussian weights, normalised by their own
 * partial sums (filter/gaussian.h:4-36). */
typedef struct gb_filter gb_filter;
gb_filter *gb_filter_create(int nx, int nz, int sigma);
/* GaussianFilter::apply on a device array float[nx*nz]. */
int gb_filter_apply(gb_filter *f, float *d_data);
void gb_filter_destroy(gb_filter *f);

/* Allocation-free Gaussian smoothing. No counterpart in the reference: an
 * addition for callers that cannot allocate device memory when they smooth a
 * gradient. Two kinds of caller need it: a host application that hands all
 * device memory to its own pool allocator and lets no library call
 * cudaMalloc (a second allocator would fragment or overrun the pool), and a
 * caller that keeps other streams busy and cannot take the device-wide
 * synchronisation that cudaMalloc/cudaFree may imply. It gives the same
 * result as gb_filter_create + gb_filter_apply on d_data (float[nx*nz] on the
 * current device): the same kernels sum the same terms in the same order.
 * Its scratch is a fixed array inside the library, so the grid is limited:
 * nx*nz <= GB_NOALLOC_MAX_CELLS and max(nx, nz) <= GB_NOALLOC_MAX_SIDE, else
 * GB_ERR_ARG. That array (about 16.1 MB) stays reserved on every device that
 * loads the library until the process exits. The first call on a device looks
 * up the array's device address (with that device current); make that first
 * call before any stream capture. Every call on a device shares that
 * device's one array and leaves its contents behind, so calls that overlap
 * on the GPU (several host threads calling at once) race. The call launches
 * on the legacy default stream and returns once its kernels have finished. */
#define GB_NOALLOC_MAX_CELLS 4194304
#define GB_NOALLOC_MAX_SIDE 8192
int gb_filter_apply_noalloc(int nx, int nz, int sigma, float *d_data);

/* ------------------------------------------------------------------ Misfit
 * Replaces class Misfit (misfit/misfit.h:3-153) with WaveformMisfit
 * (misfit = 0, misfit/waveform.h) and EnvelopeMisfit (misfit = 1,
 * misfit/envelope.h). Sums are FP64. */
typedef struct gb_misfit gb_misfit;
/* Misfit::init (misfit/misfit.h:91-151): filter may be NULL (then one is made
 * from filter_sigma when filter == 0); observed traces are read from
 * the traces/ SU files when trace_file != 0, else generated on model_true; finally
 * model_init is imported. */
gb_misfit *gb_misfit_create(const gb_config *cfg, gb_solver *s, gb_filter *f);
/* Same without files: observed traces from host arrays [nsrc][nrec][nt] per
 * component (NULL for unused components); the current model is kept. */
gb_misfit *gb_misfit_create_obs(int type, gb_solver *s, gb_filter *f, const float *obs_x, const float *obs_y,
                                const float *obs_z);
/* Replaces the observed traces of every shot, host arrays as above. */
int gb_misfit_set_obs(gb_misfit *m, const float *obs_x, const float *obs_y, const float *obs_z);
/* The same copies, queued on an upload stream of the misfit's own: the call
 * returns at once, and the next gb_misfit_run overlaps them with its forward
 * pass (only its misfit stage waits for them). The host arrays must stay
 * unchanged until that run returns; pinned memory (cudaMallocHost) makes the
 * copies asynchronous. No counterpart in the reference, whose observed traces
 * are read once at Misfit::init (misfit/misfit.h:91-151). */
int gb_misfit_set_obs_async(gb_misfit *m, const float *obs_x, const float *obs_y, const float *obs_z);
/* Misfit::run (misfit/misfit.h:15-51): all shots, batched; with kernel != 0
 * also the adjoint kernels, then the filter on k_lambda, k_mu, k_rho. */
int gb_misfit_run(gb_misfit *m, int kernel, int snapshot, double *value);
/* Per-trace misfit values of the last run, [nsrc][nrec][ncomp]. */
int gb_misfit_trace_values(gb_misfit *m, double *out, size_t n);
/* Frees the misfit; it may come before or after gb_solver_destroy of its solver. */
void gb_misfit_destroy(gb_misfit *m);

/* --------------------------------------------------------------- Optimizer
 * Replaces class Optimizer (optimizer/optimizer.h) with NLCG (optimizer = 0,
 * optimizer/nlcg.h) and L-BFGS (optimizer = 1, optimizer/lbfgs.h). Dot
 * products and norms are FP64 on the GPU; the line search keeps its steps
 * and history in float, as the reference does; the L-BFGS
 * history stays in device memory, rotated as the reference rotates it
 * (optimizer/lbfgs.h:29-36: once full, its oldest slot shares the newest
 * pair's buffer). */
typedef struct gb_optimizer gb_optimizer;
gb_optimizer *gb_optimizer_create(const gb_config *cfg, gb_solver *s, gb_misfit *m);
/* Optimizer::run (optimizer/optimizer.h:428-467), same stdout lines. */
int gb_optimizer_run(gb_optimizer *o);
/* Misfit history of the last run: value of each accepted iteration. */
int gb_optimizer_history(gb_optimizer *o, double *out, int n);
/* Every misfit evaluation of the last run, in order, as (kind, alpha,
 * value) triples into out[3*n]: kind 1 = the gradient evaluation that starts
 * an iteration (misfit->run(true), optimizer/optimizer.h:433), 0 = a
 * line-search step alpha (optimizer.h:383-389), 2 = the final misfit
 * (optimizer.h:454). Returns the number of evaluations. */
int gb_optimizer_evaluations(gb_optimizer *o, double *out, int n);
/* The line-search step rule alone, on the host (no device work): the next
 * step and status (1 accept, 0 continue, -1 failed; -2 invalid input) that
 * Optimizer::bracket (optimizer = 0, NLCG) or backtrack (1, L-BFGS),
 * optimizer/optimizer.h:267-357, give for a search history: lens/vals the
 * ls_count entries of ls_lens/ls_vals, gtg/gtp the inv_count entries of
 * ls_gtg/ls_gtp, step_count steps taken in the current search. The rule of
 * gb_optimizer_run: history, slopes and steps in float, as the reference
 * keeps them (the inputs are rounded to float). */
double gb_linesearch_step(int optimizer, const double *lens, const double *vals, int ls_count, const double *gtg,
                          const double *gtp, int inv_count, int step_count, int ls_step, double ls_thresh,
                          double step_max, int *status);
/* Frees the optimizer; it may come before or after gb_solver_destroy of its solver. */
void gb_optimizer_destroy(gb_optimizer *o);

/* ----------------------------------------------------------------- Serving
 * No counterpart in the reference, which solves one shot at a time; each
 * request is the per-shot body of Misfit::run (misfit/misfit.h:29-44):
 * forward with checkpoints, waveform misfit, adjoint with kernels. Requests
 * have their own model, grid, step count and wave system; the engine admits
 * them in arrival order while their device footprint fits the HBM budget,
 * advances all admitted requests together (one launch per step), and frees
 * each request's memory when its adjoint ends. A request's result does not
 * depend on the other requests in flight. */
typedef struct gb_server gb_server;
typedef struct {
    int psv;                  /* 1: P-SV, 0: SH */
    int nx, nz;
    float dx, dz, dt;
    int nt;                   /* multiple of the server's sfe */
    const float *lambda, *mu, *rho; /* host, nx*nz, reference layout; kept until the request ends */
    float src[7];             /* x z type f0 t0 angle amp (one Ricker source) */
    int nrec;
    const float *rec;         /* host, nrec x (x, z) */
    const float *obs;         /* host, [comp][nrec][nt] (x, z or y) or NULL for zeros */
    int abs_width;
    float abs_alpha;
    int abs_left, abs_right, abs_bottom, abs_top;
    int inv_lambda, inv_mu, inv_rho;
    double arrival;           /* seconds after gb_server_run starts */
} gb_request_desc;
typedef struct {
    int completed;
    double wall_s, p50_s, p99_s; /* latency = completion - arrival */
    int max_concurrent;
    long long rounds, launches, cell_updates;
} gb_server_stats;
gb_server *gb_server_create(int sfe, int ckpt_precision, double hbm_budget_gb, int max_slots);
/* Options, set before gb_server_run: "tile" (step kernel configuration 1..20,
 * as gb_solver_set_option; default 9, marching strips of 120 rows), "tma"
 * (1: the marching kernel loads grid columns with bulk tensor copies, each
 * request's arrays stored at a pitch of nz rounded up to a multiple of 4,
 * default; 0: per-row cp.async; the results are the same), "streams" (4:
 * each wave system's requests split into two groups, each group's steps of a
 * round on its own stream, default; 2: the SH requests' steps on a second
 * stream beside the P-SV ones; 1: one stream; the results are the same),
 * "compact" (1: a
 * marching launch runs exactly the tiles of its requests, through a block
 * map built each round, default; 0: as many blocks per request as the
 * largest request has tiles, the surplus exiting at once; the results are
 * the same). */
int gb_server_set_option(gb_server *srv, const char *key, double value);
/* Queues a request; returns its id (>= 0) or -1. */
long long gb_server_submit(gb_server *srv, const gb_request_desc *req);
/* Replays every queued request against the wall clock until all are done. */
int gb_server_run(gb_server *srv);
/* Kernels (host arrays of nx*nz, NULL to skip), misfit and latency. */
int gb_server_result(gb_server *srv, long long id, float *k_lambda, float *k_mu, float *k_rho, double *misfit,
                     double *latency_s);
int gb_server_report(gb_server *srv, gb_server_stats *out);
void gb_server_destroy(gb_server *srv);

/* -------------------------------------------------------------- utilities */
/* FP64 reductions over device float arrays (replace cublasSdot/Isamax/Snrm2
 * of lib/device.h:178-192). */
int gb_dot64(const float *d_a, const float *d_b, size_t n, double *out);
int gb_amax64(const float *d_a, size_t n, double *out);
/* Plain device memory and copies for FFI callers that hold no CUDA runtime
 * of their own (the reference allocates with device::create,
 * lib/device.h:99-111). */
void *gb_device_malloc(size_t bytes);
int gb_device_free(void *d_ptr);
int gb_memcpy_d2h(void *dst, const void *src, size_t bytes);
int gb_memcpy_h2d(void *dst, const void *src, size_t bytes);
int gb_device_sync(void);
int gb_device_count(void);
/* Pinned host memory (cudaMallocHost) for staging host<->device copies. */
void *gb_host_malloc(size_t bytes);
int gb_host_free(void *h_ptr);
/* Makes `device` current for the calling thread (one process per GPU). */
int gb_device_select(int device);
/* CUDA-event timer on the solver's stream: begin != 0 records the start;
 * begin == 0 records the stop, waits for it and writes the elapsed ms. */
int gb_solver_timer(gb_solver *s, int begin, double *ms);

#ifdef __cplusplus
}
#endif

#endif /* GBFWI_H */
