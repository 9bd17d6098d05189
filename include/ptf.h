/*
 * ptf.h -- C ABI of libptf.so, the GB300 (sm_103a) implementation of the
 * PassiveTracerFlows.jl TracerAdvectionDiffusion time step.
 *
 * Every entry point replaces one piece of the reference's path; the
 * reference location is cited beside each declaration (paths are relative
 * to the PassiveTracerFlows.jl repository).  FourierFlows.jl 0.10.5 is the
 * framework the reference plugs into (Project.toml:23); its functions are
 * named where the reference calls them.
 *
 * Conventions
 *  - Every function returns 0 on success or a positive PTF_ERR_* code; it
 *    never aborts.  ptf_last_error() gives the message of the last failure
 *    on a handle (or of the last ptf_create failure for NULL).
 *  - The handle owns all of its device memory and one CUDA stream.  A handle
 *    is not thread-safe; distinct handles are independent.
 *  - Array arguments are FP64 in the reference's column-major layout (x
 *    fastest): physical fields are nx*ny[*nz] doubles, spectral fields are
 *    (nx/2+1)*ny[*nz] complex doubles stored (re, im) interleaved.  With
 *    batch > 1 the solves follow one another.  `where` says whether a
 *    pointer is host (PTF_HOST) or device (PTF_DEVICE) memory.
 *  - Calls taking a host pointer return after the copy is complete; calls on
 *    device pointers and ptf_step are ordered on the handle's stream and may
 *    return before the GPU is done (ptf_synchronize waits).
 */
#ifndef PTF_H
#define PTF_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PTF_ABI_VERSION 4

enum ptf_status {
  PTF_OK = 0,
  PTF_ERR_ARG = 1,         /* invalid argument (reference: ArgumentError) */
  PTF_ERR_CUDA = 2,        /* CUDA runtime error */
  PTF_ERR_STATE = 3,       /* call out of order (e.g. step before set_c) */
  PTF_ERR_UNSUPPORTED = 4, /* valid for the reference, not built here */
  PTF_ERR_MEMORY = 5       /* device memory budget exceeded */
};

/* FourierFlows steppers; the Filtered ones multiply the state by the
 * FourierFlows spectral filter after every step (the MultiLayerQG-coupled
 * Problem's default is FilteredRK4, src/traceradvectiondiffusion.jl:228). */
enum ptf_stepper { PTF_RK4 = 0, PTF_ETDRK4 = 1, PTF_FILTERED_RK4 = 2, PTF_FILTERED_ETDRK4 = 3 };
enum ptf_precision { PTF_FP64 = 0, PTF_FP32 = 1 };
/* PTF_CLOCK_T evaluates a time-varying flow at clock.t for all four stages
 * of a step, as the reference does (src/traceradvectiondiffusion.jl:718,737);
 * PTF_STAGE_T evaluates it at each stage time (an extension). */
enum ptf_time_mode { PTF_CLOCK_T = 0, PTF_STAGE_T = 1 };
enum ptf_where { PTF_HOST = 0, PTF_DEVICE = 1 };

/* Mirrors the keyword arguments of TracerAdvectionDiffusion.Problem
 * (src/traceradvectiondiffusion.jl:165-216).  kappah / nkappah are the
 * hyperdiffusion of ConstDiffSteadyFlowParams (:436-452), which the
 * reference reaches only through its low-level constructor. */
typedef struct ptf_config {
  int32_t dim;        /* 1, 2 or 3 */
  int32_t nx, ny, nz; /* powers of two, 16..4096 (ny, nz ignored below their dim) */
  double Lx, Ly, Lz;
  double kappa, eta, iota; /* x, y, z diffusivities */
  double kappah;           /* hyperdiffusivity */
  int32_t nkappah;         /* hyperdiffusivity order (0: none) */
  double dt;
  int32_t stepper;   /* ptf_stepper */
  int32_t precision; /* ptf_precision */
  int32_t time_mode; /* ptf_time_mode */
  int32_t batch;     /* independent solves sharing grid, parameters and flow */
  int32_t k0_mode;   /* FP32 only: 1 (default) carries the conserved (0,0[,0])
                        mode -- its state and stage combinations -- in FP64,
                        with N(0,0) a compensated FP64 sum; 0: all FP32 */
} ptf_config;

typedef struct ptf_handle ptf_handle;

/* Fill a config with the reference's defaults: nx=ny=nz=128, L=2pi,
 * kappa=0.1, eta=iota=kappa, dt=0.01, RK4, FP64, batch 1, k0_mode 1. */
void ptf_config_default(ptf_config* cfg, int32_t dim);

/* TracerAdvectionDiffusion.Problem(dev, flow; ...) construction:
 * 1D (:143-163), 2D (:165-188), 3D (:190-216); grid (:158,:177,:205),
 * Equation L (:538-554), Vars (:652-668) and the FourierFlows time stepper
 * state (FourierFlows.Problem, :162,:187,:215).  1D problems step a batch
 * of solves in pairs (an odd batch carries one zero solve on the device). */
int ptf_create(const ptf_config* cfg, ptf_handle** out);
void ptf_destroy(ptf_handle* h);
const char* ptf_last_error(const ptf_handle* h);

/* Steady flow arrays u.(x[,y,z]), v, w on the grid (v from 2D, w in 3D): the precomputation of
 * ConstDiffSteadyFlowParams (:436-452).  Also used for a time-varying flow
 * re-evaluated by the caller at clock.t before each step (:715-718). */
int ptf_set_flow_arrays(ptf_handle* h, const double* u, const double* v, const double* w, int32_t where);
/* A flow given by formula and evaluated on the device: PTF_FLOW_CELLULAR
 * (2D; Kx, Ky integer wavenumbers in units of 2 pi / L; time-dependent when
 * eps and omega are non-zero) or PTF_FLOW_ABC (3D; A, B, C).  A
 * time-dependent flow is re-evaluated at clock.t before every step, inside
 * ptf_step, as the reference's time-varying calcN! evaluates it at clock.t
 * for all four stages (:715-718) -- without a host evaluation or a copy per
 * step.  No reference counterpart as an entry point: the reference takes
 * flows as Julia functions; this covers the analytic flows of its examples
 * and tests.  ptf_set_flow_arrays / ptf_set_flow_layers replace it. */
typedef struct ptf_flow_desc {
  int32_t kind;        /* PTF_FLOW_CELLULAR or PTF_FLOW_ABC */
  double U, eps, omega;
  int32_t Kx, Ky;
  double A, B, C;
} ptf_flow_desc;
int ptf_set_flow_analytic(ptf_handle* h, const ptf_flow_desc* d);

/* One flow per solve of a 2D batch -- the layers of the MultiLayerQG-coupled
 * tracer (Problem(MQGprob), :225-250; calcN!, :788-804): solve j is advected
 * by u_j + U[j], v_j, with u, v holding batch*nx*ny values (layer-major) and
 * U batch values (host; NULL: zero).  Called before each step with the
 * MultiLayerQG state's velocities, as calcN! reads MQGprob.vars.u, v. */
int ptf_set_flow_layers(ptf_handle* h, const double* u, const double* v, const double* U, int32_t where);

/* set_c!(prob, c) (:844-852, :872): sol = rfft(c). */
int ptf_set_c(ptf_handle* h, const double* c, int32_t where);
/* updatevars!(prob) then copy vars.c out (:815-821, :837). */
int ptf_get_c(ptf_handle* h, double* c, int32_t where);
/* prob.sol out / in (complex, (nx/2+1)*ny[*nz] per solve).  For FP32
 * handles with k0_mode, get_sol reports the FP64 k = 0 mode and set_sol
 * seeds it.  An FP32 2D/3D handle holds its state as a compensated pair of
 * FP32 values; get_sol returns their sum (exact in FP64) and set_sol splits
 * its input the same way.  So get_sol then set_sol (with ptf_clock /
 * ptf_set_clock) saves and resumes a solve exactly -- the state a
 * FourierFlows snapshot of sol and clock holds. */
int ptf_get_sol(ptf_handle* h, double* sol, int32_t where);
int ptf_set_sol(ptf_handle* h, const double* sol, int32_t where);

/* stepforward!(prob, nsteps) (FourierFlows; called at
 * test/test_traceradvectiondiffusion.jl:29): nsteps RK4/ETDRK4 steps, each
 * followed by clock.t += dt, clock.step += 1. */
int ptf_step(ptf_handle* h, int64_t nsteps);
/* prob.clock.t, prob.clock.step */
int ptf_clock(const ptf_handle* h, double* t, int64_t* step);
int ptf_set_clock(ptf_handle* h, double t, int64_t step);

/* calcN!(N, sol, t, clock, vars, params, grid) (:744-754 / :756-769 / :771-786): the
 * FourierFlows Equation plugin on its own: N = rfft(-(u.grad c)) for the
 * spectral field `sol`, with the flow set on the handle.  Complex arrays. */
int ptf_calcN(ptf_handle* h, const double* sol, double* N, int32_t where);

int ptf_synchronize(ptf_handle* h);
/* The handle's CUDA stream (cudaStream_t) and an override of it. */
int ptf_get_stream(const ptf_handle* h, void** stream);
int ptf_set_stream(ptf_handle* h, void* stream);
/* Bytes of device memory held by the handle. */
int ptf_device_bytes(const ptf_handle* h, int64_t* bytes);
/* Step schedule (no reference counterpart).  A batched handle runs each step
 * in groups of solves_per_group solves (0: the whole batch, or batch/branches
 * with several branches); groups are dealt to `branches` (1..4) concurrent
 * stream branches that fork from and join back to the handle's stream.  With
 * use_graph != 0, ptf_step(h, n > 1) captures one step as a CUDA graph and
 * replays it.  The schedule does not change results. */
int ptf_set_schedule(ptf_handle* h, int32_t solves_per_group, int32_t branches, int32_t use_graph);
/* Launch shapes of a handle (no reference counterpart).  col_lines: columns
 * per column-pass block of the main column pass (y in 2D, z in 3D);
 * col_lines_y: the same for the 3D y passes (0 in 2D); row_pairs: row pairs
 * per row-pass block; branches / solves_per_group: as ptf_set_schedule;
 * row_staged: 2D RHS row pass staging its rows in shared memory with bulk
 * copies (falls back to the direct kernel where that does not fit);
 * col_carveout: the share of the SM's L1/shared storage the column passes
 * ask to be shared memory (the rest caches, among others, register spills;
 * set by hand -- measured no better than the CUDA driver's choice, so the tuner
 * leaves it at -1);
 * ms_per_step: the time measured by ptf_autotune (0 when not tuned).  Line
 * counts are powers of two dividing the lines of the pass, within the
 * block's resource limit.  Shapes do not change results. */
typedef struct ptf_tuning {
  int32_t col_lines, col_lines_y, row_pairs, branches, solves_per_group, row_staged;
  int32_t col_carveout; /* column passes' preferred shared-memory carve-out, percent (-1: CUDA driver's choice) */
  double ms_per_step;
} ptf_tuning;
enum { PTF_TUNE_FORCE = 1 };
int ptf_get_tuning(const ptf_handle* h, ptf_tuning* out);
int ptf_set_tuning(ptf_handle* h, const ptf_tuning* t);
/* Pick the launch shapes by timing trial_steps steps per candidate on this
 * handle, one shape at a time (columns per block, 3D y columns, row pairs,
 * branches, staged row pass), keeping the fastest.  The solution, clock and
 * step count are saved and restored, so the solve is unchanged.  Choices are
 * cached per (precision, grid, batch, stepper, k0_mode) for the process and
 * reused unless flags has PTF_TUNE_FORCE.  Needs the flow to be set. */
int ptf_autotune(ptf_handle* h, int32_t trial_steps, int32_t flags);
/* Per-pass timing: with enable != 0 every pass launch is bracketed by CUDA
 * events on the handle's stream (enabling or disabling clears the record).
 * ptf_profile_read sums, for kind 0 (column passes: y transforms + stepper
 * stage) or 1 (row passes: x transforms + advection product), the event
 * time in ms, the launch count and the algorithmic bytes of those launches
 * (the minimum HBM traffic of the pass design).  No reference counterpart:
 * the reference has no profiling hooks. */
int ptf_profile(ptf_handle* h, int32_t enable);
int ptf_profile_read(ptf_handle* h, int32_t kind, double* total_ms, int64_t* launches, double* bytes);
/* Kernels launched by this handle since creation (for launch accounting). */
int ptf_kernel_launches(const ptf_handle* h, int64_t* count);
int32_t ptf_abi_version(void);
/* Arithmetic throughput of the current device (no reference counterpart):
 * FMA flops per second (2 per FMA) of a bounded probe kernel in precision
 * PTF_FP64 or PTF_FP32 -- the roof that bounds the FP64 path, whose FFT
 * butterflies issue on this chip's narrow FP64 pipe, not on HBM. */
int ptf_measure_fma_peak(int32_t precision, double* flops_per_s);

/* ---------------------------------------------------------------------------
 * Batched form.  No single reference counterpart: the reference runs one
 * Problem at a time; this steps many independent TracerAdvectionDiffusion
 * problems (each with its own grid size, diffusivity, dt, clock, step count
 * and flow) together.  Square 2D grids n in {64, 128, 256, 512, 1024}, RK4
 * (FourierFlows RK4 on the same L and calcN! as ptf_step).  Each stage of
 * all solves is a row launch and a column launch over every solve's work
 * items (or one persistent launch, ptf_batch_config.persistent); a step is
 * replayed from a captured CUDA graph.
 * ------------------------------------------------------------------------- */
enum ptf_flow_kind {
  PTF_FLOW_ARRAYS = 0,   /* steady flow given as grid arrays u, v */
  PTF_FLOW_CELLULAR = 1, /* psi = U cos(Kx x + eps sin(omega t)) cos(Ky y), u = -dpsi/dy, v = dpsi/dx,
                            evaluated on the device at clock.t (PTF_CLOCK_T) or at stage times */
  PTF_FLOW_ABC = 2       /* 3D handles only: u = A sin z + C cos y, v = B sin x + A cos z,
                            w = C sin y + B cos x (steady) */
};

typedef struct ptf_solve_desc {
  int32_t dim;       /* 2 (batched) or 3 (served through a single-solve handle) */
  int32_t n;         /* grid points per axis (square / cubic grid) */
  double L;          /* domain length per axis */
  double kappa, eta; /* x and y (and z) diffusivities */
  double kappah;
  int32_t nkappah;
  double dt;
  int64_t nsteps;    /* steps this solve takes */
  int32_t flow_kind; /* ptf_flow_kind */
  int32_t time_mode; /* ptf_time_mode (PTF_FLOW_CELLULAR) */
  double U, eps, omega;
  int32_t Kx, Ky;    /* integer wavenumbers of the cellular flow (in units of 2 pi / L) */
} ptf_solve_desc;

typedef struct ptf_batch_config {
  int32_t precision;        /* ptf_precision */
  int64_t memory_budget;    /* device bytes the batch may hold (0: unlimited) */
  int32_t slots_per_bucket; /* solves per same-size bucket (0: about 1 GB of fields per bucket) */
  int32_t use_graph;        /* replay steps from a captured CUDA graph */
  int32_t max_slots;        /* total slots over all buckets */
  int32_t persistent;       /* 1: one persistent kernel per stage (items from an atomic counter, a
                               bounded wait between a bucket's row and column items); 0 (default):
                               a row launch and a column launch per stage, one block per item */
  int32_t k0_mode;          /* FP32 only: 1 (default) carries each solve's conserved (0,0) mode in
                               FP64 (seeded from a compensated sum of c0, stage combinations in
                               FP64, N(0,0) a compensated FP64 sum; readback shifted so that the
                               field's sum is that mode), as ptf_config.k0_mode; 0: all FP32 */
} ptf_batch_config;

typedef struct ptf_batch ptf_batch;

void ptf_batch_config_default(ptf_batch_config* cfg);
void ptf_solve_desc_default(ptf_solve_desc* d);
int ptf_batch_create(const ptf_batch_config* cfg, ptf_batch** out);
void ptf_batch_destroy(ptf_batch* b);
const char* ptf_batch_last_error(const ptf_batch* b);
/* 1 when a solve of this description fits (free slot or budget for a new bucket). */
int ptf_batch_can_admit(ptf_batch* b, const ptf_solve_desc* d);
/* set_c! for a new solve (host arrays: c0, and u, v for PTF_FLOW_ARRAYS). */
int ptf_batch_add(ptf_batch* b, const ptf_solve_desc* d, const double* c0, const double* u, const double* v,
                  int64_t* id);
/* stepforward! of every active solve by up to nsteps (each stops at its own nsteps). */
int ptf_batch_step(ptf_batch* b, int64_t nsteps);
int ptf_batch_synchronize(ptf_batch* b);
int ptf_batch_status(ptf_batch* b, int64_t id, int64_t* step, double* t, int32_t* active);
/* updatevars! + vars.c of one solve (n*n doubles to host). */
int ptf_batch_get_c(ptf_batch* b, int64_t id, double* c);
int ptf_batch_remove(ptf_batch* b, int64_t id);
int ptf_batch_info(ptf_batch* b, int64_t* device_bytes, int64_t* solves, int64_t* kernel_launches);
int ptf_batch_get_stream(const ptf_batch* b, void** stream);
/* Failure-detection test hook (no reference counterpart), persistent form
 * only: from the next step, a column item of the persistent stage kernel
 * waits for extra_row_items more row items of its bucket than exist, so its
 * bounded wait runs out after spin_limit sleeps of about 128 ns (0: the
 * default limit, about 2 s); the item is skipped, the kernel ends, and
 * ptf_batch_synchronize returns PTF_ERR_CUDA.  Nothing traps or faults and
 * the CUDA context stays usable; the batch's results are invalid from then
 * on.  extra_row_items = 0 restores the normal wait. */
int ptf_batch_inject_wait_timeout(ptf_batch* b, int32_t extra_row_items, int64_t spin_limit);

/* ---------------------------------------------------------------------------
 * Request server (no reference counterpart): continuous batching.  A worker
 * thread admits submitted solves by device-memory budget between chunks of
 * steps, runs everything admitted together, and returns each result when its
 * own step count is reached.  2D requests run in the batched form, 3D
 * requests (dim 3, flow arrays) on single-solve handles in the same loop.
 * ------------------------------------------------------------------------- */
typedef struct ptf_server_config {
  int32_t precision;
  int64_t memory_budget;    /* device bytes for admitted solves (0: unlimited) */
  int32_t chunk_steps;      /* steps between admission points */
  int32_t slots_per_bucket;
} ptf_server_config;

typedef struct ptf_server_stats {
  int64_t completed, failed, queued, active;
  double p50_s, p99_s, mean_s;  /* latency from submission to result */
  double grid_point_steps;      /* sum over completed requests of points x steps */
  double wall_s;                /* first submission to last completion */
  int64_t device_bytes;
  double mass_drift_max_abs;    /* max over completed requests of |sum(c_end) / sum(c0) - 1| */
  int64_t batch_solves;         /* solves holding a slot of the batched form (2D) */
  int64_t handles;              /* single-solve handles alive (3D) */
  double admit_s;               /* worker time admitting requests (copies in, set_c, plan) */
  double chunk_s;               /* worker time from launching a chunk of steps to its completion */
  int64_t chunks;               /* chunks stepped */
} ptf_server_stats;

typedef struct ptf_server ptf_server;
enum ptf_request_state { PTF_REQ_QUEUED = 0, PTF_REQ_ACTIVE = 1, PTF_REQ_DONE = 2, PTF_REQ_FAILED = 3 };

void ptf_server_config_default(ptf_server_config* cfg);
int ptf_server_create(const ptf_server_config* cfg, ptf_server** out);
void ptf_server_destroy(ptf_server* s);
const char* ptf_server_last_error(const ptf_server* s);
/* Copies the inputs; w only for 3D.  Returns immediately.  A request that
 * could not be admitted even into an empty server under its memory budget
 * is refused here with PTF_ERR_MEMORY (as the reference refuses invalid
 * Problem arguments at construction, src/traceradvectiondiffusion.jl:234),
 * instead of queueing for ever. */
int ptf_server_submit(ptf_server* s, const ptf_solve_desc* d, const double* c0, const double* u, const double* v,
                      const double* w, int64_t* id);
/* state: ptf_request_state; copies the tracer field into c when done. */
int ptf_server_poll(ptf_server* s, int64_t id, int32_t* state, double* c);
int ptf_server_release(ptf_server* s, int64_t id);
int ptf_server_wait_all(ptf_server* s, double timeout_s);
int ptf_server_get_stats(ptf_server* s, ptf_server_stats* out);
/* Per-request result record (no reference counterpart): latency from
 * submission to result, and the tracer mass (sum of c, compensated FP64)
 * of the initial condition and of the result -- the mass drift of every
 * result is mass_end / mass0 - 1.  The request must be done. */
int ptf_server_result_info(ptf_server* s, int64_t id, double* latency_s, double* mass0, double* mass_end);
/* Host-side fault injection for tests (no reference counterpart): the chunk
 * of steps `chunks_from_now` chunks after the next one (0: the next) reports
 * a step failure as if the batched step had returned PTF_ERR_CUDA.  Nothing
 * is faulted on the GPU; the server fails the requests in flight, releases
 * their slots and handles, and keeps serving.  A negative value cancels. */
int ptf_server_inject_step_failure(ptf_server* s, int32_t chunks_from_now);

/* Size of the fixed device scratch used by ptf_calcN2d_noalloc (16 MiB). */
#define PTF_NOALLOC_SCRATCH_BYTES (16u << 20)

/* No counterpart in the reference: the reference's calcN! always works in
 * the Vars buffers its Problem allocated.  This is the same advective term
 * as ptf_calcN (N = rfft(-(u c_x + v c_y)) for one 2D FP64 spectral field)
 * for callers that must not have a library allocate device memory: a host
 * whose own memory pool owns the whole device (a Julia process under
 * CUDA.jl's pool, for instance) or a time-critical loop that cannot take
 * the device-wide synchronisation of cudaFree.  It calls no cudaMalloc,
 * cudaFree or allocating library routine.
 *   sol, N: device, (nx/2+1)*ny complex doubles, column-major (x fastest)
 *   u, v:   device, nx*ny doubles (the flow on the grid, unscaled)
 *   stream: cudaStream_t the work is ordered on (NULL: legacy default stream)
 * Intermediates live in one file-scope device array of
 * PTF_NOALLOC_SCRATCH_BYTES that every GPU loading the library keeps until
 * exit; grids needing more (1024x1024 and larger) are rejected with
 * PTF_ERR_MEMORY.  The first call on a device does a one-time set-up (symbol
 * address lookup and a synchronous twiddle upload); make it before any
 * stream capture.  All calls share that array and it keeps the last call's
 * contents, so calls that overlap on the GPU race.  The set-up is kept per
 * device for the life of the process: resetting a device (cudaDeviceReset)
 * after its first call is not supported, since the kept address belongs to
 * the context the reset destroyed.  Errors: ptf_last_error(NULL). */
int ptf_calcN2d_noalloc(int32_t nx, int32_t ny, double Lx, double Ly, const double* sol, const double* u,
                        const double* v, double* N, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* PTF_H */
