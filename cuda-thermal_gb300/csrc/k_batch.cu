// k_batch.cu - batched solver kernels: the double-word outer PCG and the
// FP32 V-cycle stages for many instances per launch (see batch.h for the
// block table and the per-instance reductions).
//
// Each kernel is the batched form of a single-solver kernel and uses the same
// per-column / per-cell device code (dw_dev.cuh, mg_dev.cuh), so one instance
// of a batch computes what a single solver computes for it.
#include <cstdlib>
#include <algorithm>
#include <cmath>

#include "batch.h"
#include "batch_dev.cuh"
#include "dw_dev.cuh"
#include "mg_dev.cuh"
#include "reduce.cuh"
#include "setup_dev.cuh"

namespace ct {

using namespace dwdev;
using namespace mgdev;

namespace {

// The same for double-word accumulators (float pairs in the same slots),
// summed on the FP32 pipe.
__device__ __forceinline__ bool publish_inst_acc(const DwAcc& a, const DwAcc& b, const BRed& red, int ntasks,
                                                 int inst, int count) {
    return publish_acc2(a, b, red.part, ntasks, blockIdx.x, &red.tickets[inst], (unsigned)count);
}

__device__ __forceinline__ void gather_inst_acc(const BRed& red, int ntasks, int inst, int first, int count,
                                                double& A, double& B) {
    gather_acc2(red.part, ntasks, (unsigned)first, (unsigned)count, &red.tickets[inst], A, B);
}

// Start of every loop body: ends the loop once no instance is active, and
// bounds the number of bodies.
__global__ void kb_guard(BCtl* bc, Cond cond) {
    pdl_enter();
    pdl_trigger();
    if (threadIdx.x != 0) return;
    bc->body += 1;
    if (bc->active <= 0 || bc->body > bc->maxbody) {
        if (cond.use) cudaGraphSetConditional(cond.h, 0u);
    }
}

__global__ void __launch_bounds__(NT)
    kb_fold(Plan p, const BInst* __restrict__ bi, const Ctl* ctl, int only_phase_end) {
    pdl_enter();
    const Task t = p.tasks[blockIdx.x];
    const Ctl* c = &ctl[t.inst];
    if (only_phase_end && (inst_done(c) || !c->phase_end)) return;
    double2* xb = reinterpret_cast<double2*>(bi[t.inst].x);
    float4* xw = reinterpret_cast<float4*>(bi[t.inst].xw);
    for (unsigned k = t.begin + threadIdx.x; k < t.end; k += NT) {
        const float4 w = xw[k];
        if (w.x != 0.0f || w.z != 0.0f) {
            double2 v = xb[k];
            v.x += dw_d(make_float2(w.x, w.y));
            v.y += dw_d(make_float2(w.z, w.w));
            xb[k] = v;
            xw[k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
    }
}

// r = b - A x in FP64 from the FP64 base x: the start of a solve, or (start
// = 0) the residual replacement of instances whose first phase ended.
__global__ void __launch_bounds__(NT)
    kb_residual(Plan p, const BInst* __restrict__ bi, Ctl* ctl, BRed red, int start, BCtl* bc,
                Cond cond) {
    pdl_enter();
    const Task t = p.tasks[blockIdx.x];
    Ctl* c = &ctl[t.inst];
    if (inst_done(c) || (!start && !c->phase_end)) return;
    const BInst I = bi[t.inst];
    const Geo& g = I.o.g;
    const bool zero = start && c->x_zero;
    double rr = 0.0, bb = 0.0;
    for (unsigned s = t.begin + threadIdx.x; s < t.end; s += NT) {
        const Col cl = col_of_slot(g, s);
        if (!cl.valid) {
            for (int l = 0; l < g.nz; ++l) {
                I.r[(unsigned)l * g.plane + s] = make_float2(0.0f, 0.0f);
                I.b0[(unsigned)l * g.plane + s] = 0.0f;
            }
            continue;
        }
        if (zero) {
            for (int l = 0; l < g.nz; ++l) {
                const unsigned id = (unsigned)l * g.plane + cl.s;
                const double bv = I.b[id];
                const float2 rw = dw_of(bv);
                I.r[id] = rw;
                I.b0[id] = rw.x;
                bb += bv * bv;
                rr += bv * bv;
            }
            continue;
        }
        double x_c = I.x[cl.s], x_b = 0.0;
        float gu_b = 0.0f;
        for (int l = 0; l < g.nz; ++l) {
            const unsigned base = (unsigned)l * g.plane, id = base + cl.s;
            const bool up = l < g.nz - 1;
            const double x_a = up ? I.x[id + g.plane] : 0.0;
            const float gu = I.o.gU[id];
            double off = 0.0;
            if (cl.i > 0) off += (double)I.o.gE[base + cl.sw] * I.x[base + cl.sw];
            if (cl.i < g.nx - 1) off += (double)I.o.gE[id] * I.x[base + cl.se];
            if (cl.j > 0) off += (double)I.o.gN[base + cl.ss] * I.x[base + cl.ss];
            if (cl.j < g.ny - 1) off += (double)I.o.gN[id] * I.x[base + cl.sn];
            if (l > 0) off += (double)gu_b * x_b;
            if (up) off += (double)gu * x_a;
            const double bv = I.b[id];
            const double rv = bv - (I.diag[id] * x_c - off);
            const float2 rw = dw_of(rv);
            I.r[id] = rw;
            I.b0[id] = rw.x;
            rr += rv * rv;
            bb += bv * bv;
            x_b = x_c;
            x_c = x_a;
            gu_b = gu;
        }
    }
    block_sum2(rr, bb);
    if (publish_inst(rr, bb, red, p.ntasks, t.inst, p.inst_count[t.inst])) {
        double RR, BB;
        gather_inst(red, p.ntasks, t.inst, p.inst_first[t.inst], p.inst_count[t.inst], RR, BB);
        if (threadIdx.x == 0) {
            c->rr = RR;
            if (start) {
                c->bb = BB;
                if (BB == 0.0) {
                    c->bb_zero = 1;
                    c->converged = 1;
                    c->relres = 0.0;
                    inst_stop(c, bc, cond);
                    return;
                }
            }
            const double rel = sqrt(RR / c->bb);
            c->relres = rel;
            c->phase_end = 0;
            if (!start) c->stop = c->tol;
            if (rel < c->tol) {
                c->converged = 1;
                inst_stop(c, bc, cond);
            } else if (!isfinite(rel)) {
                c->breakdown = 1;
                inst_stop(c, bc, cond);
            } else if (c->iter >= c->maxit) {
                inst_stop(c, bc, cond);
            }
        }
    }
}

// Ap = d p - sum G p_nbr over rows [begin, end) of the instance (one warp
// per row of one colour of one plane, apply_row with one cell per lane, every
// operand of it gathered at once), p.Ap, alpha. Measured on the 256-instance
// floorplan batch: 40.7 ms per solve against 50.0 ms with the operands loaded
// term by term and 59.0 ms with two cells per lane; compiled for 4 blocks per
// SM (64 registers: 600 us per launch against 722 us with the compiler's 78).
__global__ void __launch_bounds__(NT, 4)
    kb_apply(Plan p, const BInst* __restrict__ bi, Ctl* ctl, BRed red, BCtl* bc, Cond cond) {
    pdl_enter();
    const Task t = p.tasks[blockIdx.x];
    Ctl* c = &ctl[t.inst];
    if (inst_done(c)) return;
    const OpView o = bi[t.inst].o;
    const float2* __restrict__ pv = bi[t.inst].p;
    const float2* __restrict__ dgw = bi[t.inst].dgw;
    float2* __restrict__ Ap = bi[t.inst].Ap;
    const int lane = (int)(threadIdx.x & 31u);
    DwAcc pacc = {0.0f, 0.0f};
    for (unsigned R = t.begin + (threadIdx.x >> 5); R < t.end; R += NT / 32)
        apply_row<1>(o, dgw, pv, Ap, R, lane, pacc);
    pdl_trigger();
    DwAcc unused = {0.0f, 0.0f};
    block_sum_acc2(pacc, unused);
    if (publish_inst_acc(pacc, unused, red, p.ntasks, t.inst, p.inst_count[t.inst])) {
        double PAP, unused2;
        gather_inst_acc(red, p.ntasks, t.inst, p.inst_first[t.inst], p.inst_count[t.inst], PAP, unused2);
        if (threadIdx.x == 0) {
            c->pAp = PAP;
            if (!(PAP > 0.0) || !isfinite(PAP)) {
                c->breakdown = 1;
                c->alpha = 0.0;
                inst_stop(c, bc, cond);
            } else {
                c->alpha = c->rz / PAP;
                c->alpha_w = dw_of(c->alpha);
            }
        }
    }
}

// x += alpha p, r -= alpha Ap, b0 = r, ||r||^2, the instance's convergence
// test. Items are value pairs.
__global__ void __launch_bounds__(NT)
    kb_update(Plan p, const BInst* __restrict__ bi, Ctl* ctl, BRed red, BCtl* bc, Cond cond) {
    pdl_enter();
    const Task t = p.tasks[blockIdx.x];
    Ctl* c = &ctl[t.inst];
    if (inst_done(c)) return;
    DwAcc acc = {0.0f, 0.0f};
    update_range(t.begin + threadIdx.x, t.end, NT, c->alpha_w,
                 reinterpret_cast<const float4*>(bi[t.inst].p),
                 reinterpret_cast<const float4*>(bi[t.inst].Ap),
                 reinterpret_cast<float4*>(bi[t.inst].xw), reinterpret_cast<float4*>(bi[t.inst].r),
                 reinterpret_cast<float2*>(bi[t.inst].b0), acc);
    pdl_trigger();
    DwAcc unused = {0.0f, 0.0f};
    block_sum_acc2(acc, unused);
    if (publish_inst_acc(acc, unused, red, p.ntasks, t.inst, p.inst_count[t.inst])) {
        double RR, U;
        gather_inst_acc(red, p.ntasks, t.inst, p.inst_first[t.inst], p.inst_count[t.inst], RR, U);
        if (threadIdx.x == 0) {
            c->rr = RR;
            c->iter += 1;
            const double rel = sqrt(RR / c->bb);
            c->relres = rel;
            if (rel < c->tol) {
                c->converged = 1;
                inst_stop(c, bc, cond);
            } else if (!isfinite(rel)) {
                c->breakdown = 1;
                inst_stop(c, bc, cond);
            } else if (c->iter >= c->maxit) {
                inst_stop(c, bc, cond);
            } else if (rel < c->stop) {
                c->phase_end = 1;  // the replacement at the end of this body
            }
        }
    }
}

// rz = r.z, z.Ap, flexible beta.
__global__ void __launch_bounds__(NT)
    kb_dot(Plan p, const BInst* __restrict__ bi, Ctl* ctl, BRed red, BCtl* bc, Cond cond) {
    pdl_enter();
    const Task t = p.tasks[blockIdx.x];
    Ctl* c = &ctl[t.inst];
    if (inst_done(c)) return;
    DwAcc rz = {0.0f, 0.0f}, zap = {0.0f, 0.0f};
    dot_range(t.begin + threadIdx.x, t.end, NT, reinterpret_cast<const float4*>(bi[t.inst].r),
              reinterpret_cast<const float2*>(bi[t.inst].z),
              reinterpret_cast<const float4*>(bi[t.inst].Ap), rz, zap);
    pdl_trigger();
    block_sum_acc2(rz, zap);
    if (publish_inst_acc(rz, zap, red, p.ntasks, t.inst, p.inst_count[t.inst])) {
        double RZ, ZAP;
        gather_inst_acc(red, p.ntasks, t.inst, p.inst_first[t.inst], p.inst_count[t.inst], RZ, ZAP);
        if (threadIdx.x == 0) {
            c->beta = c->iter > 0 ? -ZAP / c->pAp : 0.0;
            c->beta_w = dw_of(c->beta);
            c->rz = RZ;
            c->zAp = ZAP;
            if (!isfinite(RZ) || !isfinite(c->beta)) {
                c->breakdown = 1;
                inst_stop(c, bc, cond);
            }
        }
    }
}

__global__ void __launch_bounds__(NT)
    kb_update_p(Plan p, const BInst* __restrict__ bi, const Ctl* ctl) {
    pdl_enter();
    const Task t = p.tasks[blockIdx.x];
    const Ctl* c = &ctl[t.inst];
    if (inst_done(c)) return;
    update_p_range(t.begin + threadIdx.x, t.end, NT, c->beta_w, c->iter == 0,
                   reinterpret_cast<const float2*>(bi[t.inst].z), reinterpret_cast<float4*>(bi[t.inst].p));
}

// Pairs of values: b = P + C/dt x (x = FP64 base, folded), x_old = x.
__global__ void __launch_bounds__(NT)
    kb_rhs_transient(Plan p, const BInst* __restrict__ bi, const Ctl* ctl) {
    const Task t = p.tasks[blockIdx.x];
    const double inv_dt = ctl[t.inst].inv_dt;
    const BInst I = bi[t.inst];
    const double2* __restrict__ P = reinterpret_cast<const double2*>(I.P);
    const double2* __restrict__ x = reinterpret_cast<const double2*>(I.x);
    const float2* __restrict__ cap = reinterpret_cast<const float2*>(I.o.cap);
    double2* __restrict__ b = reinterpret_cast<double2*>(I.b);
    double2* __restrict__ xold = reinterpret_cast<double2*>(I.xold);
    for (unsigned k = t.begin + threadIdx.x; k < t.end; k += NT) {
        const double2 xv = x[k], pv = P[k];
        const float2 cv = cap[k];
        b[k] = make_double2(__dadd_rn(pv.x, __dmul_rn(__dmul_rn((double)cv.x, inv_dt), xv.x)),
                            __dadd_rn(pv.y, __dmul_rn(__dmul_rn((double)cv.y, inv_dt), xv.y)));
        xold[k] = xv;
    }
}

// Step records of every instance (items: fine column slots): T_max,
// heat_out = sum over the top and bottom faces of g x, and sum C (x - x_old)
// (src/stack3d.h:252-273), x the folded FP64 base; rec[3 i + 0..2].
__global__ void __launch_bounds__(NT)
    kb_step_record(Plan p, const BInst* __restrict__ bi, BRed red, double* __restrict__ mx,
                   double* __restrict__ rec) {
    const Task t = p.tasks[blockIdx.x];
    const BInst I = bi[t.inst];
    const Geo& g = I.o.g;
    double tmax = -INFINITY, qout = 0.0, qst = 0.0;
    for (unsigned s = t.begin + threadIdx.x; s < t.end; s += NT) {
        const Col c = col_of_slot(g, s);
        if (!c.valid) continue;
        for (int l = 0; l < g.nz; ++l) {
            const unsigned id = (unsigned)l * g.plane + s;
            const double xv = I.x[id];
            tmax = fmax(tmax, xv);
            qst += (double)I.o.cap[id] * (xv - I.xold[id]);
        }
        const unsigned top = (unsigned)(g.nz - 1) * g.plane + s;
        qout += (double)I.o.gU[top] * I.x[top];
        qout += (double)I.o.gB[s] * I.x[s];
    }
    __shared__ double sm[NT / 32];
    double m = tmax;
    for (int off = 16; off > 0; off >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, off));
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        m = threadIdx.x < NT / 32 ? sm[threadIdx.x] : -INFINITY;
        for (int off = 16; off > 0; off >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, off));
    }
    block_sum2(qout, qst);
    if (threadIdx.x == 0) mx[blockIdx.x] = m;
    const int first = p.inst_first[t.inst], count = p.inst_count[t.inst];
    if (publish_inst(qout, qst, red, p.ntasks, t.inst, count)) {
        __threadfence();
        double mm = -INFINITY;
        for (int k = threadIdx.x; k < count; k += NT) mm = fmax(mm, __ldcg(mx + first + k));
        for (int off = 16; off > 0; off >>= 1) mm = fmax(mm, __shfl_down_sync(0xffffffffu, mm, off));
        __syncthreads();
        if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = mm;
        __syncthreads();
        if (threadIdx.x < 32) {
            mm = threadIdx.x < NT / 32 ? sm[threadIdx.x] : -INFINITY;
            for (int off = 16; off > 0; off >>= 1) mm = fmax(mm, __shfl_down_sync(0xffffffffu, mm, off));
        }
        double QO, QS;
        gather_inst(red, p.ntasks, t.inst, first, count, QO, QS);
        if (threadIdx.x == 0) {
            rec[3 * t.inst] = mm;
            rec[3 * t.inst + 1] = QO;
            rec[3 * t.inst + 2] = QS;
        }
    }
}

// set_dt of every instance: its FP64 (and double-word) diagonal, items =
// natural fine columns; 1/dt per instance from its control block.
__global__ void __launch_bounds__(NT) kb_diag(Plan p, const BInst* __restrict__ bi, const Ctl* ctl) {
    const Task t = p.tasks[blockIdx.x];
    const BInst& I = bi[t.inst];
    const double inv_dt = ctl[t.inst].inv_dt;
    for (unsigned q = t.begin + threadIdx.x; q < t.end; q += NT)
        setupdev::diag_column(I.o, I.dface, inv_dt, q, const_cast<double*>(I.diag), nullptr,
                              const_cast<float2*>(I.dgw));
}

// ... and the column factors of one level index of every instance that has it
// (items = natural columns of that level).
__global__ void __launch_bounds__(NT)
    kb_factor(Plan p, const LevelView<float>* __restrict__ views, const Ctl* ctl) {
    const Task t = p.tasks[blockIdx.x];
    const LevelView<float> L = views[t.inst];
    const float inv_dt = (float)ctl[t.inst].inv_dt;
    for (unsigned q = t.begin + threadIdx.x; q < t.end; q += NT) setupdev::factor_column<float>(L, inv_dt, q);
}

template <int MZ, bool ZERO, bool PRO>
__global__ void __launch_bounds__(NT)
    kb_sweep(Plan p, const LevelView<float>* __restrict__ views,
             const LevelView<float>* __restrict__ cviews, int color, const Ctl* ctl) {
    pdl_enter();
    const Task t = p.tasks[blockIdx.x];
    if (inst_done(&ctl[t.inst])) return;
    const LevelView<float> L = views[t.inst];
    const LevelView<float> C = PRO ? cviews[t.inst] : L;
    for (unsigned q = t.begin + threadIdx.x; q < t.end; q += NT)
        sweep_column<float, MZ, ZERO, PRO, false>(L, C, color, q);
}

// Compiled for 4 blocks per SM (64 registers): level 0 of the 256-instance
// batch 296 us per launch against 429 us with the compiler's own choice (also
// 64 registers), as for the single solver's k_restrict2.
__global__ void __launch_bounds__(NT, 4)
    kb_restrict(Plan p, const LevelView<float>* __restrict__ views,
                const LevelView<float>* __restrict__ cviews, const Ctl* ctl) {
    pdl_enter();
    const Task t = p.tasks[blockIdx.x];
    const Ctl* c = &ctl[t.inst];
    if (inst_done(c)) return;
    const LevelView<float> L = views[t.inst];
    const LevelView<float> C = cviews[t.inst];
    const float inv_dt = (float)c->inv_dt;
    const unsigned ccols = (unsigned)C.g.nx * (unsigned)C.g.ny;
    for (unsigned w = t.begin + threadIdx.x; w < t.end; w += NT) {
        const int l = (int)(w / ccols);
        restrict_cell<float, false>(L, C, inv_dt, w - (unsigned)l * ccols, l);
    }
}

template <int MZ>
__global__ void __launch_bounds__(kSmallThreads, 1)
    kb_small(const int* __restrict__ insts, const TailLevels<float>* __restrict__ small,
             Ctl* ctl, BCtl* bc, Cond cond) {
    const int i = insts[blockIdx.x];
    Ctl* c = &ctl[i];
    extern __shared__ __align__(16) unsigned char smem[];
    // the levels' operators and factors (not written inside the loop) are
    // copied before the dependent-launch wait, b and the done flag after it
    const auto wait = [] { pdl_enter(); };
    const auto go = [&] { return !inst_done(c); };
    if (vsmall_body<float, MZ>(small[i], &c->inv_dt, smem, wait, go) == kSmallTimeout &&
        threadIdx.x == 0) {
        // a bounded wait ran out: record it and stop this instance
        atomicExch(&c->err, 1);
        c->breakdown = 1;
        inst_stop(c, bc, cond);
    }
}

}  // namespace

void launch_b_guard(cudaStream_t st, BCtl* bc, Cond cond) { launch_pdl(kb_guard, 1, 32, 0, st, bc, cond); }

void launch_b_fold(cudaStream_t st, const Plan& p, const BInst* bi, Ctl* ctl, int only_phase_end) {
    launch_pdl(kb_fold, p.ntasks, NT, 0, st, p, bi, ctl, only_phase_end);
}

void launch_b_residual(cudaStream_t st, const Plan& p, const BInst* bi, Ctl* ctl, BRed red,
                       int start, BCtl* bc, Cond cond) {
    launch_pdl(kb_residual, p.ntasks, NT, 0, st, p, bi, ctl, red, start, bc, cond);
}

void launch_b_apply(cudaStream_t st, const Plan& p, const BInst* bi, Ctl* ctl, BRed red,
                    BCtl* bc, Cond cond) {
    launch_pdl(kb_apply, p.ntasks, NT, 0, st, p, bi, ctl, red, bc, cond);
}

void launch_b_update(cudaStream_t st, const Plan& p, const BInst* bi, Ctl* ctl, BRed red,
                     BCtl* bc, Cond cond) {
    launch_pdl(kb_update, p.ntasks, NT, 0, st, p, bi, ctl, red, bc, cond);
}

void launch_b_dot(cudaStream_t st, const Plan& p, const BInst* bi, Ctl* ctl, BRed red, BCtl* bc,
                  Cond cond) {
    launch_pdl(kb_dot, p.ntasks, NT, 0, st, p, bi, ctl, red, bc, cond);
}

void launch_b_update_p(cudaStream_t st, const Plan& p, const BInst* bi, const Ctl* ctl) {
    launch_pdl(kb_update_p, p.ntasks, NT, 0, st, p, bi, ctl);
}

void launch_b_step_record(cudaStream_t st, const Plan& p, const BInst* bi, BRed red, double* mx,
                          double* rec) {
    if (p.ntasks > 0) kb_step_record<<<p.ntasks, NT, 0, st>>>(p, bi, red, mx, rec);
}

void launch_b_diag(cudaStream_t st, const Plan& p, const BInst* bi, const Ctl* ctl) {
    if (p.ntasks > 0) kb_diag<<<p.ntasks, NT, 0, st>>>(p, bi, ctl);
}

void launch_b_factor(cudaStream_t st, const Plan& p, const LevelView<float>* views, const Ctl* ctl) {
    if (p.ntasks > 0) kb_factor<<<p.ntasks, NT, 0, st>>>(p, views, ctl);
}

void launch_b_rhs_transient(cudaStream_t st, const Plan& p, const BInst* bi, const Ctl* ctl) {
    kb_rhs_transient<<<p.ntasks, NT, 0, st>>>(p, bi, ctl);
}

void launch_b_sweep(cudaStream_t st, const Plan& p, const LevelView<float>* views,
                    const LevelView<float>* cviews, int color, bool zero_x, bool prolong, int mz,
                    const Ctl* ctl) {
#define CT_BSWEEP(MZ)                                                                          \
    do {                                                                                       \
        if (zero_x)                                                                            \
            launch_pdl(kb_sweep<MZ, true, false>, p.ntasks, NT, 0, st, p, views, cviews, color, ctl);  \
        else if (prolong)                                                                      \
            launch_pdl(kb_sweep<MZ, false, true>, p.ntasks, NT, 0, st, p, views, cviews, color, ctl);  \
        else                                                                                   \
            launch_pdl(kb_sweep<MZ, false, false>, p.ntasks, NT, 0, st, p, views, cviews, color, ctl); \
    } while (0)
    if (mz <= 8)
        CT_BSWEEP(8);
    else if (mz <= 12)
        CT_BSWEEP(12);
    else if (mz <= 16)
        CT_BSWEEP(16);
    else if (mz <= 32)
        CT_BSWEEP(32);
    else
        CT_BSWEEP(0);
#undef CT_BSWEEP
}

void launch_b_restrict(cudaStream_t st, const Plan& p, const LevelView<float>* views,
                       const LevelView<float>* cviews, const Ctl* ctl) {
    launch_pdl(kb_restrict, p.ntasks, NT, 0, st, p, views, cviews, ctl);
}

cudaError_t launch_b_small(cudaStream_t st, const int* insts, int n,
                           const TailLevels<float>* small, size_t smem, int mz, Ctl* ctl, BCtl* bc,
                           Cond cond) {
    auto go = [&](auto kern) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             kSmallSmemMax);
        if (e != cudaSuccess) return e;
        launch_pdl(kern, n, kSmallThreads, smem, st, insts, small, ctl, bc, cond);
        return cudaGetLastError();
    };
    if (mz <= 8) return go(kb_small<8>);
    if (mz <= 12) return go(kb_small<12>);
    if (mz <= 16) return go(kb_small<16>);
    if (mz <= 32) return go(kb_small<32>);
    return go(kb_small<0>);
}

}  // namespace ct
