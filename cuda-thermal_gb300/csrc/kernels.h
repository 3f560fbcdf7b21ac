// kernels.h - host-side launchers of the solver kernels (k_outer.cu, k_mg.cu).
// Every launcher enqueues on the given stream and returns without
// synchronising, so the whole iteration can be captured into a CUDA graph.
#pragma once
#include <cuda_runtime.h>

#include "device.h"

namespace ct {

// Fine-level operator as the outer PCG sees it (split layout).
struct OpView {
    Geo g;
    const float *gE, *gN, *gU, *gB, *cap;
};

// Reduction context of one kernel: its slot's partials and grid size.
struct Red {
    double* part;  // 4 * maxb doubles
    int maxb;      // row stride of part
    int blocks;    // grid size (<= maxb)
};

enum MgType { MG_NONE = 0, MG_F32 = 1, MG_F64 = 2 };

// ---- outer PCG (FP64), k_outer.cu ----------------------------------------
// r = b - (A + C/dt) x, b0 = r in the V-cycle precision; rr, bb; start test.
void launch_residual(cudaStream_t st, MgType mt, const OpView& o, const double* diag,
                     const double* b, const double* x, double* r, void* b0, Ctl* ctl,
                     const Red& red, Cond cond);
// Ap = (A + C/dt) p; p.Ap; alpha = rz / p.Ap.
void launch_apply(cudaStream_t st, const OpView& o, const double* diag, const double* p,
                  double* Ap, Ctl* ctl, const Red& red, Cond cond);
// x += alpha p, r -= alpha Ap, b0 = r; rr; convergence test.
void launch_update(cudaStream_t st, MgType mt, unsigned n, const double* p, const double* Ap,
                   double* x, double* r, void* b0, Ctl* ctl, const Red& red, Cond cond);
// rz = r.z (and z.Ap for the flexible beta); beta. z = V-cycle result
// (mt = MG_F32 / MG_F64) or r * invd (mt = MG_NONE, Jacobi).
void launch_dot(cudaStream_t st, MgType mt, bool flexible, unsigned n, const double* r,
                const void* z, const double* invd, const double* Ap, Ctl* ctl, const Red& red,
                Cond cond);
// p = z + beta p (p = z on the first iteration).
void launch_update_p(cudaStream_t st, MgType mt, unsigned n, const void* z, const double* r,
                     const double* invd, double* p, Ctl* ctl, Cond cond);

// ---- setup and auxiliary kernels, k_outer.cu ------------------------------
void launch_to_split_f(cudaStream_t st, const Geo& g, int planes, const float* nat, float* split);
void launch_to_split_d(cudaStream_t st, const Geo& g, const double* nat, double* split);
void launch_to_natural_d(cudaStream_t st, const Geo& g, const double* split, double* nat);
// diag = op_diag (FP64, no contraction); invd = 1 / diag when invd != null.
void launch_diag(cudaStream_t st, const OpView& o, double inv_dt, double* diag, double* invd);
// b = P + cap * inv_dt * x; xold = x.
void launch_rhs_transient(cudaStream_t st, unsigned n, const float* cap, double inv_dt,
                          const double* P, const double* x, double* b, double* xold);
// ctl->aux0 = ||P - A x||^2, aux1 = ||P||^2 (steady operator, FP64).
void launch_true_residual(cudaStream_t st, const OpView& o, const double* P, const double* x,
                          Ctl* ctl, const Red& red);
// ctl->aux0 = T_max, aux1 = heat out, aux2 = sum cap (x - xold).
void launch_step_record(cudaStream_t st, const OpView& o, const double* x, const double* xold,
                        Ctl* ctl, const Red& red);

// ---- multigrid, k_mg.cu ---------------------------------------------------
// Coarse level from the fine one (mg_coarse_cell arithmetic, split layouts).
void launch_coarsen(cudaStream_t st, const Geo& fg, const float* fgE, const float* fgN,
                    const float* fgU, const float* fgB, const float* fcap, const double* fdx,
                    const double* fdy, const Geo& cg, const double* cdx, const double* cdy,
                    float* cgE, float* cgN, float* cgU, float* cgB, float* ccap);
// Column factors of one level for 1/dt (mg_factor_column arithmetic).
template <class T>
void launch_factor(cudaStream_t st, const LevelView<T>& L, T inv_dt);
// One red-black sweep. zero_x: x = 0 before the sweep (the first sweep of a
// V-cycle), so lateral neighbours are not read. xc: when not null, the
// coarser level's x is added to every neighbour value read (prolongation
// fused into the sweep).
template <class T>
void launch_sweep(cudaStream_t st, const LevelView<T>& L, int color, bool zero_x,
                  const LevelView<T>* coarse_for_prolong, const Ctl* ctl, Cond cond);
// coarse b = sum over the children of (b - (A + C/dt) x).
template <class T>
void launch_restrict(cudaStream_t st, const LevelView<T>& F, const LevelView<T>& C, const Ctl* ctl,
                     Cond cond);

}  // namespace ct
