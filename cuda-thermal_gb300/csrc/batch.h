// batch.h - device-side structures and launchers of the batched solver
// (k_batch.cu): many independent stacks of uneven size solved together, one
// launch per stage for all of them.
//
// Work assignment. Every batched launch runs over a block table: block b
// works on items [begin, end) of ONE instance (columns, cells or value pairs
// of that instance's arrays). A block never straddles two instances, so each
// reduction is per instance and deterministic: a block writes its partial
// sums to its own slot, and the instance's last block (by ticket) adds its
// blocks' slots in table order and finishes that instance's scalar work.
//
// Convergence mask: every block first reads its instance's control block and
// returns at once when that instance is done; the batch's active-instance
// count reaching zero ends the graph loop.
#pragma once
#include "kernels.h"

namespace ct {

struct Task {
    int inst;
    unsigned begin, end;
};

// Device view of one stage's block table.
struct Plan {
    const Task* tasks;
    int ntasks;
    const int* inst_first;  // per instance: first block of the instance (reducing stages)
    const int* inst_count;  // per instance: number of its blocks (0 = not in this stage)
};

// One instance's fine-level arrays (split layout). The double-word mode
// (CT_MG_FP32_FLEX_DW) reads r, p, Ap as float pairs and keeps x as an FP64
// base plus xw; the FP64 mode (CT_MG_FP32_FLEX) reads the same storage as
// doubles (r64, p64, Ap64) and x is the whole iterate (xw, dgw null).
struct BInst {
    OpView o;
    const double* P;
    double* x;      // FP64 base of x
    double* b;
    const double* diag;
    const double* dface;  // the diagonal's face sum
    float2* xw;     // double-word correction of x
    float2* r;
    float2* p;
    float2* Ap;
    const float2* dgw;
    float* b0;      // V-cycle input (level 0 b)
    const float* z; // V-cycle result (level 0 x)
    double* xold;   // x at the last set_rhs_transient (step bookkeeping)
    double* r64;    // r, p, Ap as doubles (the FP64 outer mode)
    double* p64;
    double* Ap64;
    unsigned n;     // slots of all planes
};

struct BCtl {
    int active;   // instances not yet done
    int body;     // loop bodies entered
    int maxbody;  // bound on loop bodies (maxit + 2)
    int pad;
};

// Per-instance reduction bookkeeping of one stage.
struct BRed {
    double* part;       // 2 * ntasks doubles
    unsigned* tickets;  // per instance
};

// ---- outer PCG (double-word, FP64 residual), one launch for the batch ------
// First kernel of a loop body: ends the loop when no instance is active.
void launch_b_guard(cudaStream_t st, BCtl* bc, Cond cond);
void launch_b_fold(cudaStream_t st, const Plan& p, const BInst* bi, Ctl* ctl, int only_phase_end);
void launch_b_residual(cudaStream_t st, const Plan& p, const BInst* bi, Ctl* ctl, BRed red,
                       int start, BCtl* bc, Cond cond);
void launch_b_apply(cudaStream_t st, const Plan& p, const BInst* bi, Ctl* ctl, BRed red,
                    BCtl* bc, Cond cond);
void launch_b_update(cudaStream_t st, const Plan& p, const BInst* bi, Ctl* ctl, BRed red,
                     BCtl* bc, Cond cond);
void launch_b_dot(cudaStream_t st, const Plan& p, const BInst* bi, Ctl* ctl, BRed red, BCtl* bc,
                  Cond cond);
void launch_b_update_p(cudaStream_t st, const Plan& p, const BInst* bi, const Ctl* ctl);

// ---- outer PCG in FP64 (CT_MG_FP32_FLEX), one launch for the batch, k_batch64.cu
// Items: residual and apply, rows of one colour and plane; the others, value
// pairs.
void launch_b_residual64(cudaStream_t st, const Plan& p, const BInst* bi, Ctl* ctl, BRed red, BCtl* bc,
                         Cond cond);
void launch_b_apply64(cudaStream_t st, const Plan& p, const BInst* bi, Ctl* ctl, BRed red, BCtl* bc,
                      Cond cond);
void launch_b_update64(cudaStream_t st, const Plan& p, const BInst* bi, Ctl* ctl, BRed red, BCtl* bc,
                       Cond cond);
void launch_b_dot64(cudaStream_t st, const Plan& p, const BInst* bi, Ctl* ctl, BRed red, BCtl* bc,
                    Cond cond);
void launch_b_update_p64(cudaStream_t st, const Plan& p, const BInst* bi, const Ctl* ctl);

// ---- multigrid, one launch per stage and depth for the batch ----------------
// views / cviews: this depth's and the next coarser depth's LevelView per
// instance (indexed by instance).
void launch_b_sweep(cudaStream_t st, const Plan& p, const LevelView<float>* views,
                    const LevelView<float>* cviews, int color, bool zero_x, bool prolong, int mz,
                    const Ctl* ctl);
void launch_b_restrict(cudaStream_t st, const Plan& p, const LevelView<float>* views,
                       const LevelView<float>* cviews, const Ctl* ctl);
// The same sweep staged by bulk tensor copies (k_sweep_tma.cu): the plan's
// items are the tiles of each instance's level (sweep_tma_tiles), maps[i]
// instance i's tensor maps for this level and colour. A wait that runs out
// sets that instance's ctl->err and stops it.
void launch_b_sweep_tma(cudaStream_t st, const Plan& p, const SweepMaps* maps,
                        const LevelView<float>* views, const LevelView<float>* cviews, int color,
                        bool zero_x, bool prolong, int mz, Ctl* ctl, BCtl* bc, Cond cond);
int sweep_tma_tiles(const Geo& g);
// The bottom of every instance's V-cycle: one block per instance in `insts`.
cudaError_t launch_b_small(cudaStream_t st, const int* insts, int n,
                           const TailLevels<float>* small, size_t smem, int mz, Ctl* ctl, BCtl* bc,
                           Cond cond);
// set_dt for all instances (1/dt from ctl[i].inv_dt): the fine FP64 and
// double-word diagonal (items: natural fine columns), and the column factors
// of one level index (items: natural columns of that level; views[i] =
// instance i's level).
void launch_b_diag(cudaStream_t st, const Plan& p, const BInst* bi, const Ctl* ctl);
void launch_b_factor(cudaStream_t st, const Plan& p, const LevelView<float>* views, const Ctl* ctl);
// Per-instance T_max, heat out and sum C (x - x_old) into rec[3 i + 0..2]
// (items: fine column slots; x folded; mx: one double per task).
void launch_b_step_record(cudaStream_t st, const Plan& p, const BInst* bi, BRed red, double* mx,
                          double* rec);
// b = P + cap / dt x (per-instance 1/dt from ctl), x_old = x, for all
// instances (x folded first).
void launch_b_rhs_transient(cudaStream_t st, const Plan& p, const BInst* bi, const Ctl* ctl);

}  // namespace ct
