/* oracle.h - CPU oracle for the steady / backward-Euler MG-PCG thermal solve.
 *
 * TEST INFRASTRUCTURE ONLY. This is a plain-C restatement of the reference's
 * CPU solver (cuda-thermal: src/pcg3d_cpu.cpp, src/mg3d.h, src/operator3d.h,
 * src/transient3d.h, src/stack3d.h:252-273). Only the tests, the smoke check
 * and the CPU baseline leg of the benchmark load it, to check results and to
 * time the CPU reference arithmetic. The product path (the CUDA library)
 * never links, loads or calls it.
 *
 * Arithmetic follows the reference operation by operation, in the same order,
 * so that with FMA contraction disabled (-ffp-contract=off) the results are
 * bit-identical to the reference CPU build with the same precision choice:
 *   mg_double = 1  <->  reference built with -DMG_DOUBLE (plain FP64 MG-PCG)
 *   mg_double = 0  <->  reference default build (float V-cycle, double PCG)
 * One addition that the reference does not have: flexible = 1 replaces the
 * Fletcher-Reeves beta (rz_new / rz, src/pcg3d_cpu.cpp:179) with the flexible
 * (Polak-Ribiere) beta  -(z_new . Ap) / (p . Ap), the form the GPU library uses
 * for its FP32 V-cycle path.
 *
 * Layout: natural, cell (i, j, l) at (l * ny + j) * nx + i, as in
 * src/stack3d.h:73.
 */
#ifndef CT_ORACLE_H
#define CT_ORACLE_H
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same fields as the reference's finalized Model3D (src/stack3d.h:45-79). */
typedef struct oracle_model {
    int nx, ny, nz;
    double dx, dy;
    const float *gE, *gN, *gU, *gB, *cap;
    const double* P;
} oracle_model;

typedef struct oracle_solver oracle_solver;

/* precond: 0 = Jacobi, 1 = multigrid. Returns NULL on bad input. */
oracle_solver* oracle_create(const oracle_model* m, int precond, int mg_double, int flexible);
void oracle_destroy(oracle_solver* s);
void oracle_set_dt(oracle_solver* s, double dt);
void oracle_set_x_zero(oracle_solver* s);
void oracle_set_x(oracle_solver* s, const double* x);
void oracle_set_rhs_steady(oracle_solver* s);
void oracle_set_rhs_transient(oracle_solver* s);
void oracle_set_power(oracle_solver* s, const double* P);
/* Returns 1 when converged. iters / relres as the reference's PcgStats. */
int oracle_solve(oracle_solver* s, double tol, int maxit, int* iters, double* relres);
void oracle_get_x(const oracle_solver* s, double* T);
/* Outer iteration in double-float (float pairs on FP32 arithmetic) instead of
 * double: the arithmetic of the GPU library's FP32-pipe outer mode. Not in
 * the reference. */
void oracle_set_outer_df(oracle_solver* s, int on);

/* Multigrid hierarchy (natural layout, as src/mg3d.h:147-183). */
int oracle_num_levels(const oracle_solver* s);
void oracle_level_dims(const oracle_solver* s, int k, int* nx, int* ny, int* nz);
void oracle_level_operator(const oracle_solver* s, int k, float* gE, float* gN, float* gU,
                           float* gB, float* cap);
/* Column factors of level k for the current dt, widened to double. */
void oracle_level_factors(const oracle_solver* s, int k, double* fcp, double* finv);

/* Model-level checks (src/pcg3d_cpu.cpp:207-220, src/stack3d.h:252-273). */
double oracle_true_relres(const oracle_model* m, const double* T);
double oracle_heat_out(const oracle_model* m, const double* T);
double oracle_heat_stored(const oracle_model* m, const double* T_old, const double* T_new,
                          double dt);
/* y = (A + C inv_dt) x in double, natural layout (src/operator3d.h:110). */
void oracle_apply(const oracle_model* m, double inv_dt, const double* x, double* y);

/* Backward Euler run (src/transient3d.h:48-90). With nsteps > 0 the run is
 * driven by step count instead of t_end. Step records go to rec (6 doubles per
 * step: t, dt, iters, T_max, q_out, q_stored) when rec is not NULL, at most
 * max_rec steps. Returns the number of steps taken; T_end gets the final
 * field; *total_iters and *all_converged summarise the run. */
int oracle_run_transient(const oracle_model* m, int precond, int mg_double, int flexible,
                         double dt0, double growth, double dt_max, double t_end, int nsteps,
                         double tol, int maxit, double* rec, int max_rec, double* T_end,
                         long* total_iters, int* all_converged);

#ifdef __cplusplus
}
#endif
#endif
