/* cthermal.h - C ABI of libcthermal, a GB300 (sm_103a) solver for the steady
 * and backward-Euler heat equation of a layered 3D chip stack: matrix-free
 * PCG preconditioned by one geometric x-y semi-coarsening multigrid V-cycle
 * with a red-black vertical-column (tridiagonal) line smoother, on the 7-point
 * harmonic-mean conductance operator with a heat-sink boundary.
 *
 * This is the drop-in boundary for cuda-thermal's solver layer. Each entry
 * point names the reference interface it replaces (file:line in cuda-thermal).
 * Plain C: pointers, sizes and status codes, no C++ or framework types.
 *
 * Conventions
 *  - Every call returns a ct_status; nothing calls exit(). ct_last_error()
 *    gives the message of the last failure on the calling thread.
 *  - Arrays are in the reference's natural layout: cell (i, j, l) at
 *    (l * ny + j) * nx + i (src/stack3d.h:73). Temperatures are rises above
 *    ambient (K), powers in W, conductances in W/K, capacities in J/K.
 *  - A solver owns its device memory and one CUDA stream. The model arrays are
 *    copied at creation, so the caller may free them afterwards. A solver is
 *    not thread-safe; distinct solvers may be used from distinct threads.
 */
#ifndef CTHERMAL_H
#define CTHERMAL_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CT_MAXZ 64 /* most z-planes a model may have (src/stack3d.h:34) */

typedef enum ct_status {
    CT_OK = 0,
    CT_NOT_CONVERGED = 1, /* maxit reached (PcgStats.converged = false) */
    CT_BREAKDOWN = 2,     /* p.Ap <= 0 or a NaN/Inf in the recurrence */
    CT_CUDA_ERROR = 3,
    CT_TIMEOUT = 4,       /* a bounded device wait ran out */
    CT_BAD_ARG = 5,
    CT_NOT_FINALIZED = 6, /* model arrays missing (finalize() not called) */
    CT_NO_DEVICE = 7,
    CT_OUT_OF_MEMORY = 8,
    CT_IO_ERROR = 9
} ct_status;

/* Precond (src/pcg3d.h:54). */
typedef enum ct_precond { CT_JACOBI = 0, CT_MULTIGRID = 1 } ct_precond;

/* Precision of the V-cycle and form of beta. The outer PCG (residual, iterate
 * updates, dot products, alpha, beta) is FP64 in the first three modes.
 *  CT_MG_FP64      V-cycle in double, beta = rz_new / rz: the reference built
 *                  with -DMG_DOUBLE (src/pcg3d.h:30-34), the plain FP64 method.
 *  CT_MG_FP32      V-cycle in float, same beta: the reference's default build.
 *  CT_MG_FP32_FLEX V-cycle in float inside flexible PCG, beta =
 *                  -(z_new . Ap) / (p . Ap) (Polak-Ribiere form).
 *  CT_MG_FP32_FLEX_DW  as CT_MG_FP32_FLEX, but the outer iterate updates,
 *                  operator apply and dot products run in double-word
 *                  (float-pair, ~48-bit) arithmetic on the FP32 pipes, with
 *                  the residual recomputed once in FP64 when ||r||/||b|| first
 *                  drops below 1e-5 (residual replacement), so the FP64 true
 *                  residual still meets tol. The FP64 residual, alpha, beta,
 *                  dot-product totals and energy balance stay FP64. */
typedef enum ct_precision {
    CT_MG_FP64 = 0,
    CT_MG_FP32 = 1,
    CT_MG_FP32_FLEX = 2,
    CT_MG_FP32_FLEX_DW = 3
} ct_precision;

/* A finalized Model3D's arrays (src/stack3d.h:45-79): gE, gN, gU, cap have
 * nx*ny*nz entries, gB nx*ny, P nx*ny*nz. dx, dy (m) are the lateral cell
 * sizes, which the multigrid coarsening needs (src/mg3d.h:139-166). */
typedef struct ct_model {
    int nx, ny, nz;
    double dx, dy;
    const float* gE;
    const float* gN;
    const float* gU;
    const float* gB;
    const float* cap;
    const double* P;
} ct_model;

/* PcgStats (src/pcg3d.h:45-49), plus the breakdown flag. */
typedef struct ct_stats {
    int iters;
    double relres; /* ||r|| / ||b|| from the PCG recurrence */
    int converged;
    int breakdown;
} ct_stats;

/* GpuSetupTimes (src/pcg3d.h:102-108), in ms. */
typedef struct ct_setup_times {
    double alloc_ms, upload_ms, levels_ms, factor_ms, graphs_ms;
} ct_setup_times;

/* One backward Euler step's bookkeeping (StepRecord, src/transient3d.h:29-35),
 * computed on the device from the current x and the x that
 * ct_set_rhs_transient saw. */
typedef struct ct_step_record {
    double T_max;    /* hottest cell (K above ambient) */
    double q_out;    /* heat leaving through top and bottom (W), heat_out */
    double q_stored; /* sum C (T_new - T_old) / dt (W), heat_stored */
} ct_step_record;

typedef struct ct_solver ct_solver;

/* ---- library ------------------------------------------------------------ */
const char* ct_version(void);
const char* ct_status_string(ct_status s);
const char* ct_last_error(void);
/* gpu_use_graphs (src/pcg3d_gpu.cu:84-85): solvers created afterwards replay
 * each solve as one CUDA graph (on, the default) or launch every kernel
 * directly with a host check per iteration (off). */
void ct_use_graphs(int on);

/* Self-test of the device-side failure detection: one warp waits `polls`
 * polls (1..2^22) on an mbarrier that nothing completes, through the bounded
 * wait every staged kernel uses, and *timed_out = 1 when the wait ran out and
 * the kernel returned (as it must; the solvers then report CT_TIMEOUT). The
 * context stays usable. */
ct_status ct_selftest_bounded_wait(unsigned polls, int* timed_out);
/* No counterpart in the reference. The FP64 outer kernels convert between
 * float and double with integer operations instead of the hardware
 * conversions, which issue at the FP64 rate on GB300; this runs both on n
 * bit patterns (every float exponent, doubles around the float range with
 * mantissas at and beside the rounding tie, then hashed patterns) and
 * returns the number of results that differ in *mismatches (0 expected).
 * n in 1..2^32; synchronises the device. */
ct_status ct_selftest_conversions(unsigned long long n, unsigned long long seed,
                                  unsigned long long* mismatches);
/* No counterpart in the reference. The device's FP64 fused multiply-add
 * rate (instructions per second over every SM, independent chains; about
 * 0.53e12 on GB300): the denominator of the FP64-pipe roofline reported for
 * the FP64 outer kernels. Synchronises the device. */
ct_status ct_probe_fp64_rate(double* dfma_per_s);
/* No counterpart in the reference. Microseconds per phase of `phases`
 * dependent phases run over SMs x blocks_per_sm blocks of 256 threads (capped
 * at what can be resident; *blocks returns the count), separated (a) by a
 * grid-wide barrier inside one persistent cooperative kernel and (b) by one
 * dependently launched kernel per phase in a CUDA graph, the way the solver's
 * graphs separate stages. CT_TIMEOUT if a barrier wait gave up (bounded).
 * Synchronises the device. */
ct_status ct_probe_sync_costs(int phases, int blocks_per_sm, double* us_grid_barrier,
                              double* us_dependent_launch, int* blocks);
/* gpu_last_setup (src/pcg3d_gpu.cu:87-88): setup times of the last solver
 * created on any thread. */
ct_status ct_last_setup(ct_setup_times* out);

/* ---- single solver: GpuPcg (src/pcg3d.h:115-163) ------------------------- */
/* GpuPcg::GpuPcg (src/pcg3d_gpu.cu:346-493): uploads the model, builds the
 * multigrid levels on the device, factors for dt = 0, records the graphs. */
ct_status ct_solver_create(const ct_model* m, ct_precond pc, ct_precision prec, ct_solver** out);
/* GpuPcg::~GpuPcg (src/pcg3d_gpu.cu:495-509). */
ct_status ct_solver_destroy(ct_solver* s);
/* No single counterpart in the reference: build_case_model
 * (src/case3d.h:157-166) followed by the solver's construction, with the
 * model built on the device (power blocks, TSV regions and the face
 * conductances computed by kernels straight into the solver's layout; the
 * same arrays, bit for bit, as ct_model_* on the host), so a floorplan sweep
 * pays neither the host build nor the upload. */
typedef struct ct_case ct_case;
ct_status ct_solver_create_case(const ct_case* c, int nx, int ny, int with_tsv, ct_precond pc,
                                ct_precision prec, ct_solver** out);
/* GpuPcg::set_dt (src/pcg3d_gpu.cu:511-524): 0 = steady state. */
ct_status ct_set_dt(ct_solver* s, double dt);
/* GpuPcg::set_x_zero (src/pcg3d_gpu.cu:526). */
ct_status ct_set_x_zero(ct_solver* s);
/* No reference counterpart beyond get_x: loads x (natural layout, host),
 * e.g. to warm-start or resume a transient. */
ct_status ct_set_x(ct_solver* s, const double* T);
/* GpuPcg::set_rhs_steady (src/pcg3d_gpu.cu:528-530): b = P. */
ct_status ct_set_rhs_steady(ct_solver* s);
/* GpuPcg::set_rhs_transient (src/pcg3d_gpu.cu:532-536): b = P + C/dt x. */
ct_status ct_set_rhs_transient(ct_solver* s);
/* GpuPcg::set_power (src/pcg3d_gpu.cu:538-546): P from host memory. */
ct_status ct_set_power(ct_solver* s, const double* P);
/* Same, from device memory (natural layout). */
ct_status ct_set_power_device(ct_solver* s, const double* P_dev);
/* GpuPcg::solve (src/pcg3d_gpu.cu:640-682): PCG from the current x until
 * ||r|| / ||b|| < tol or maxit. Blocks until done. Returns CT_OK,
 * CT_NOT_CONVERGED or CT_BREAKDOWN, with the statistics in *st. */
ct_status ct_solve(ct_solver* s, double tol, int maxit, ct_stats* st);
/* No counterpart in the reference (its solve always blocks). Queues the same
 * solve on the solver's stream and returns at once, so that a caller running
 * many solves in a row (a power-map sweep: ct_set_power_device or
 * ct_set_rhs_steady, then ct_solve_async, again and again) keeps the GPU busy
 * while the host does other work or is held up. Each queued solve overwrites
 * the previous one's statistics; ct_solve_wait blocks until the last queued
 * solve is done and returns its status and statistics as ct_solve would. A
 * solve that finds no heat in still sets x = 0. Where the solver has no
 * single-graph solve (ct_use_graphs(0)), the solve runs before the call
 * returns and ct_solve_wait reports it. */
ct_status ct_solve_async(ct_solver* s, double tol, int maxit);
ct_status ct_solve_wait(ct_solver* s, ct_stats* st);
/* No counterpart in the reference. The host copies of a power-map sweep,
 * queued beside the solves: ct_set_power_async copies P (host memory, pinned
 * for the copy to overlap) into one of two device staging buffers on a copy
 * stream of its own, and the solver's stream converts it into the solver's P
 * once it has landed; ct_get_x_async converts x on the solver's stream (after
 * the solves queued so far) into one of two staging buffers and copies it to
 * T on a second copy stream. So the copy in of the next step and the copy
 * out of the previous one run while the current step solves. The caller
 * keeps P unchanged and reads T only after ct_copies_wait, which blocks until
 * every queued copy (and the solver's stream) is done. */
ct_status ct_set_power_async(ct_solver* s, const double* P);
ct_status ct_get_x_async(ct_solver* s, double* T);
ct_status ct_copies_wait(ct_solver* s);
/* GpuPcg::get_x (src/pcg3d_gpu.cu:548-552): x to host memory. */
ct_status ct_get_x(ct_solver* s, double* T);
/* GpuPcg::device_x (src/pcg3d.h:130): device pointer to x in the natural
 * layout, valid until the next call on this solver. */
ct_status ct_device_x(ct_solver* s, const double** T_dev);
/* GpuPcg::setup_ (src/pcg3d_gpu.cu:369-492) of this solver. */
ct_status ct_solver_setup_times(const ct_solver* s, ct_setup_times* out);
/* The solver's CUDA stream (cudaStream_t), for callers that time or order
 * work around it. */
ct_status ct_solver_stream(const ct_solver* s, void** stream);
/* true_relres (src/pcg3d_cpu.cpp:207-220) of the current x, recomputed from
 * scratch in FP64 on the device: ||P - A x|| / ||P|| (steady operator). */
ct_status ct_true_relres(ct_solver* s, double* out);
/* T_max, heat_out and heat_stored (src/stack3d.h:252-273, as used by
 * run_transient, src/transient3d.h:72-80) on the device, for the step of
 * length dt that the last ct_set_rhs_transient started. */
ct_status ct_solver_step_record(ct_solver* s, double dt, ct_step_record* out);
/* No counterpart in the reference. The same record queued on the solver's
 * stream, with the statistics of the solve queued before it, into entry
 * `slot` (>= 0) of a table on the device, so that a transient run of
 * ct_set_dt, ct_set_rhs_transient, ct_solve_async and this call per step
 * never waits on the host; ct_solver_step_records waits for the solver's
 * stream and copies entries first .. first + count - 1 out (stats may be
 * NULL). Growing the table past its largest slot so far synchronises. */
ct_status ct_solver_step_record_async(ct_solver* s, double dt, int slot);
ct_status ct_solver_step_records(ct_solver* s, int first, int count, ct_step_record* out, ct_stats* stats);
/* Multigrid hierarchy: number of levels, and level k's size. */
ct_status ct_num_levels(const ct_solver* s, int* n);
ct_status ct_level_dims(const ct_solver* s, int k, int* nx, int* ny, int* nz);
/* Level k's operator (natural layout, host arrays as in MgLevelHost,
 * src/mg3d.h:88-93) as built on the device. gB has nx*ny entries. */
ct_status ct_level_operator(ct_solver* s, int k, float* gE, float* gN, float* gU, float* gB,
                            float* cap);
/* Level k's column factors for the current dt, widened to double. */
ct_status ct_level_factors(ct_solver* s, int k, double* fcp, double* finv);

/* ---- allocation-free residual check -------------------------------------- */
/* No counterpart in the reference. The steady true residual
 * ||P - A T|| / ||P|| of a temperature field, like ct_true_relres, for
 * callers that may not allocate device memory: a per-frame loop that must
 * not stall the GPU (cudaMalloc can synchronise the device), or a host
 * framework that holds the device memory in its own pool and hands out
 * buffers but no allocator. It takes caller-owned DEVICE arrays and allocates
 * nothing: m_dev->gE, gN, gU, gB and P, and T_dev, are device pointers in the
 * natural layout (cap is not read), and the ratio is written to out_dev[0]
 * (device memory) on `stream` (a cudaStream_t, or NULL for the default
 * stream); the call does not synchronise.
 * Its scratch is a fixed CT_NOALLOC_SCRATCH_BYTES array in the library's
 * device memory, held on every GPU that loads the library until exit, which
 * limits a model to CT_NOALLOC_MAX_COLUMNS columns (nx * ny); larger models
 * get CT_BAD_ARG. The first call on each device looks up that array's device
 * address (cudaGetSymbolAddress, no allocation), so make the first call on a
 * device before any stream capture; the address is kept per CUDA context,
 * and the first call in a new context (after a device reset) looks it up
 * again, so make that call before any capture too. All calls share the one scratch array:
 * calls whose work can overlap on the GPU (other streams, other threads)
 * race on it and must be serialised by the caller. */
#define CT_NOALLOC_SCRATCH_BYTES 131072
#define CT_NOALLOC_MAX_COLUMNS 2096640
ct_status ct_true_relres_noalloc(const ct_model* m_dev, const double* T_dev, double* out_dev,
                                 void* stream);

/* ---- batched solver -------------------------------------------------------- */
/* No single counterpart in the reference, which solves one stack per GpuPcg
 * (src/pcg3d.h:115-163); a batch is N independent GpuPcg-style solves of
 * stacks of uneven size (nx, ny, nz per instance), advanced together: every
 * stage of the iteration is one launch for all instances, each instance with
 * its own scalars and convergence test, and the loop of each size bucket is
 * one CUDA graph. The V-cycle is FP32 inside the flexible PCG; the outer
 * iteration is FP64 (CT_MG_FP32_FLEX) or double words on the FP32 pipes with
 * an FP64 residual replacement (CT_MG_FP32_FLEX_DW). Instances are numbered
 * 0..n-1 in the order of `models`, which are copied at creation.
 * Per-instance calls mirror the single-solver calls (ct_set_power, ct_get_x,
 * ...). ct_batch_create: CT_MG_FP32_FLEX_DW; ct_batch_create_prec: either,
 * anything else is CT_BAD_ARG. */
typedef struct ct_batch ct_batch;
ct_status ct_batch_create(int n, const ct_model* const* models, ct_batch** out);
ct_status ct_batch_create_prec(int n, const ct_model* const* models, ct_precision prec, ct_batch** out);
/* The same with every instance's model built on the device from a case on
 * an nx[i] x ny[i] grid (with_tsv may be NULL: all with TSVs), as
 * ct_solver_create_case builds it. */
ct_status ct_batch_create_cases(int n, const ct_case* const* cases, const int* nx, const int* ny,
                                const int* with_tsv, ct_batch** out);
ct_status ct_batch_create_cases_prec(int n, const ct_case* const* cases, const int* nx, const int* ny,
                                     const int* with_tsv, ct_precision prec, ct_batch** out);
ct_status ct_batch_destroy(ct_batch* b);
ct_status ct_batch_size(const ct_batch* b, int* n);
/* Per-instance time step (dt[i] = 0: steady); NULL: all steady. */
ct_status ct_batch_set_dt(ct_batch* b, const double* dt);
ct_status ct_batch_set_x_zero(ct_batch* b);
ct_status ct_batch_set_x(ct_batch* b, int i, const double* T);
ct_status ct_batch_set_rhs_steady(ct_batch* b);
ct_status ct_batch_set_rhs_transient(ct_batch* b);
ct_status ct_batch_set_power(ct_batch* b, int i, const double* P);
/* The same from device memory (natural layout, ncells doubles), ordered on
 * the batch's stream (ct_batch_stream). */
ct_status ct_batch_set_power_device(ct_batch* b, int i, const double* P_dev);
/* Solves every instance to its own relres < tol (or maxit); stats[i] per
 * instance (stats may be NULL). Returns CT_BREAKDOWN / CT_NOT_CONVERGED if
 * any instance did. */
ct_status ct_batch_solve(ct_batch* b, double tol, int maxit, ct_stats* stats);
/* One backward-Euler step of every instance (step_once,
 * src/transient3d.h:52-69): set_dt(dt), b = P + C/dt T, solve from T. */
ct_status ct_batch_step_transient(ct_batch* b, const double* dt, double tol, int maxit,
                                  ct_stats* stats);
ct_status ct_batch_get_x(ct_batch* b, int i, double* T);
ct_status ct_batch_true_relres(ct_batch* b, int i, double* out);
ct_status ct_batch_step_record(ct_batch* b, int i, double dt, ct_step_record* out);
/* The step records of every instance in one launch (out[i] for the step of
 * length dt[i] that the last ct_batch_set_rhs_transient started). */
ct_status ct_batch_step_records(ct_batch* b, const double* dt, ct_step_record* out);
/* Size buckets and the tiles the autotuner picked for each of their depths
 * (arrays of depth entries, each may be NULL): staged[d] = 1 where the
 * sweeps of depth d are staged by bulk tensor copies, 2 where only the
 * instances whose level holds a full tile row are (the others run the grid
 * sweep), 0 where none is; sweep_tiles[d] the 32 x 8-column tiles per block
 * of the staged part, else the columns per block of the grid sweep;
 * restrict_tiles[d] the coarse cells per block of the restriction. */
ct_status ct_batch_num_buckets(const ct_batch* b, int* nbuckets);
/* The batch's stream (a cudaStream_t): every ct_batch_* call is ordered on it,
 * and a solve's work on the buckets' own streams is joined back into it. */
ct_status ct_batch_stream(const ct_batch* b, void** stream);
ct_status ct_batch_bucket_info(const ct_batch* b, int k, int* ninst, int* depth,
                               unsigned* sweep_tiles, unsigned* restrict_tiles, int* staged);

/* ---- field products on the device ------------------------------------------ */
/* The live view's die map without a window (k_colorize, src/viewer.cu:52-87):
 * for every column the hottest of planes l0..l1 of the current solution (K
 * above ambient), as RGBA on the scale [0, rise_hi] (black - purple - red -
 * orange - pale yellow) into rgba_dev (nx*ny uchar4, device, row j = y), and
 * as float into map_dev (nx*ny, device; the tmap_layer*.csv values,
 * src/main3d.cu:303-323, before adding the ambient); either may be NULL. The
 * hottest column's value and position come back through the 64-bit packed
 * key (float bits, then the cell index; the later index wins a tie). */
ct_status ct_colorize(ct_solver* s, int l0, int l1, float rise_hi, void* rgba_dev, void* map_dev,
                      double* max_rise, int* max_i, int* max_j);
/* block_temps (src/main3d.cu:286-300): the maximum and the area-weighted
 * mean of the current solution over the rectangle [x0, x0+w] x [y0, y0+h]
 * (m) in planes l0..l1, cells covered as for_each_overlap counts them. */
ct_status ct_block_temps(ct_solver* s, int l0, int l1, double x0, double y0, double w, double h,
                         double* tmax, double* tavg);

/* ---- per-kernel timing --------------------------------------------------- */
typedef struct ct_kernel_time {
    char name[32];     /* kernel family, e.g. "mg_sweep_l0" */
    int launches;
    double total_ms;   /* sum of CUDA-event durations on the solver's stream */
    double bytes;      /* algorithmic bytes, summed over the launches */
} ct_kernel_time;
/* Runs one solve like ct_solve, but launches every kernel directly with a
 * CUDA event pair around each launch; fills up to max entries of out, one per
 * kernel family, and *n with the count. */
ct_status ct_profile_solve(ct_solver* s, double tol, int maxit, ct_stats* st,
                           ct_kernel_time* out, int max, int* n);
/* The same for a batch: every launch direct, the buckets one after another,
 * per kernel family ("b_sweep_d0", "b_apply", ...) over all buckets. */
ct_status ct_batch_profile_solve(ct_batch* b, double tol, int maxit, ct_stats* stats,
                                 ct_kernel_time* out, int max, int* n);

#ifdef __cplusplus
}
#endif
#endif /* CTHERMAL_H */
