// k_batch64.cu - the batched solver's FP64 outer PCG (CT_MG_FP32_FLEX): the
// start residual, operator apply, x/r update, dot products and p update of
// every instance of a bucket, one launch each, in IEEE double arithmetic as
// the single solver's k_fp64.cu (same per-cell code, f64_dev.cuh: the fewest
// FP64 instructions, float <-> double conversions by integer operations).
// Block tables and per-instance reductions as in k_batch.cu (batch.h).
#include <cmath>

#include "batch.h"
#include "batch_dev.cuh"
#include "f64_dev.cuh"
#include "reduce.cuh"

namespace ct {

using namespace f64dev;

namespace {

// Cells per lane of a row pass: one. The batch's half-rows are 32 to 256
// slots, so a pass of 64 slots leaves lanes idle on most of them (the
// 256-instance batch: 48.5 ms of apply per solve against 59.7 ms with two).
constexpr int kRowU = 1;

// r = b - (A + C/dt) x, b0 = r (float), ||r||^2, ||b||^2 and the start test
// of every instance; items = rows of one colour and plane (a start from
// x = 0 copies b).
__global__ void __launch_bounds__(NT)
    kb_residual64(Plan p, const BInst* __restrict__ bi, Ctl* ctl, BRed red, BCtl* bc, Cond cond) {
    pdl_enter();
    const Task t = p.tasks[blockIdx.x];
    Ctl* c = &ctl[t.inst];
    if (inst_done(c)) return;
    const BInst I = bi[t.inst];
    const Geo& g = I.o.g;
    const bool zero = c->x_zero;
    const int lane = (int)(threadIdx.x & 31u);
    double rr = 0.0, bb = 0.0;
    for (unsigned R = t.begin + (threadIdx.x >> 5); R < t.end; R += NT / 32) {
        if (zero) {
            const unsigned rows = 2u * (unsigned)g.ny;
            const unsigned l = R / rows, row = l * g.plane + (R - l * rows) * (unsigned)g.hx;
            for (unsigned s = (unsigned)lane; s < (unsigned)g.hx; s += 32u) {
                const double bv = I.b[row + s];
                I.r64[row + s] = bv;
                I.b0[row + s] = narrow(bv);
                bb = __fma_rn(bv, bv, bb);
            }
        } else {
            row64<kRowU>(I.o, I.diag, I.x, R, lane, [&](unsigned k, bool valid, double ax, double) {
                if (!valid) {
                    I.r64[k] = 0.0;
                    I.b0[k] = 0.0f;
                    return;
                }
                const double bv = I.b[k];
                const double rv = bv - ax;
                I.r64[k] = rv;
                I.b0[k] = narrow(rv);
                rr = __fma_rn(rv, rv, rr);
                bb = __fma_rn(bv, bv, bb);
            });
        }
    }
    if (zero) rr = bb;
    block_sum2(rr, bb);
    if (publish_inst(rr, bb, red, p.ntasks, t.inst, p.inst_count[t.inst])) {
        double RR, BB;
        gather_inst(red, p.ntasks, t.inst, p.inst_first[t.inst], p.inst_count[t.inst], RR, BB);
        if (threadIdx.x == 0) {
            c->rr = RR;
            c->bb = BB;
            if (BB == 0.0) {  // no heat in: x = 0 (src/pcg3d_cpu.cpp:146)
                c->bb_zero = 1;
                c->converged = 1;
                c->relres = 0.0;
                inst_stop(c, bc, cond);
                return;
            }
            const double rel = sqrt(RR / BB);
            c->relres = rel;
            if (rel < c->tol) {
                c->converged = 1;
                inst_stop(c, bc, cond);
            } else if (!isfinite(rel)) {
                c->breakdown = 1;
                inst_stop(c, bc, cond);
            } else if (c->maxit <= 0) {
                inst_stop(c, bc, cond);
            }
        }
    }
}

// Ap = (A + C/dt) p, p.Ap, alpha; items = rows of one colour and plane.
__global__ void __launch_bounds__(NT)
    kb_apply64(Plan p, const BInst* __restrict__ bi, Ctl* ctl, BRed red, BCtl* bc, Cond cond) {
    pdl_enter();
    const Task t = p.tasks[blockIdx.x];
    Ctl* c = &ctl[t.inst];
    if (inst_done(c)) return;
    const BInst I = bi[t.inst];
    const int lane = (int)(threadIdx.x & 31u);
    double pap = 0.0, unused = 0.0;
    for (unsigned R = t.begin + (threadIdx.x >> 5); R < t.end; R += NT / 32)
        row64<kRowU>(I.o, I.diag, I.p64, R, lane, [&](unsigned k, bool valid, double av, double pc) {
            I.Ap64[k] = av;
            if (valid) pap = __fma_rn(pc, av, pap);
        });
    pdl_trigger();
    block_sum2(pap, unused);
    if (publish_inst(pap, unused, red, p.ntasks, t.inst, p.inst_count[t.inst])) {
        double PAP, U;
        gather_inst(red, p.ntasks, t.inst, p.inst_first[t.inst], p.inst_count[t.inst], PAP, U);
        if (threadIdx.x == 0) {
            c->pAp = PAP;
            if (!(PAP > 0.0) || !isfinite(PAP)) {
                c->breakdown = 1;
                c->alpha = 0.0;
                inst_stop(c, bc, cond);
            } else {
                c->alpha = c->rz / PAP;
            }
        }
    }
}

// x += alpha p, r -= alpha Ap, b0 = r (float), ||r||^2, the instance's
// convergence test; items = value pairs.
__global__ void __launch_bounds__(NT)
    kb_update64(Plan p, const BInst* __restrict__ bi, Ctl* ctl, BRed red, BCtl* bc, Cond cond) {
    pdl_enter();
    const Task t = p.tasks[blockIdx.x];
    Ctl* c = &ctl[t.inst];
    if (inst_done(c)) return;
    const BInst I = bi[t.inst];
    const double alpha = c->alpha, malpha = -alpha;
    const double2* __restrict__ p2 = reinterpret_cast<const double2*>(I.p64);
    const double2* __restrict__ a2 = reinterpret_cast<const double2*>(I.Ap64);
    double2* __restrict__ x2 = reinterpret_cast<double2*>(I.x);
    double2* __restrict__ r2 = reinterpret_cast<double2*>(I.r64);
    float2* __restrict__ b02 = reinterpret_cast<float2*>(I.b0);
    double rr = 0.0, unused = 0.0;
    struct Item {
        double2 p, a, x, r;
    };
    stream_pipelined<1, Item>(
        t.begin + threadIdx.x, t.end, NT, [&](unsigned k) { return Item{p2[k], a2[k], x2[k], r2[k]}; },
        [&](unsigned k, Item it) {
            it.x.x = __fma_rn(alpha, it.p.x, it.x.x);
            it.x.y = __fma_rn(alpha, it.p.y, it.x.y);
            it.r.x = __fma_rn(malpha, it.a.x, it.r.x);
            it.r.y = __fma_rn(malpha, it.a.y, it.r.y);
            x2[k] = it.x;
            r2[k] = it.r;
            b02[k] = make_float2(narrow(it.r.x), narrow(it.r.y));
            rr = __fma_rn(it.r.x, it.r.x, rr);
            rr = __fma_rn(it.r.y, it.r.y, rr);
        });
    pdl_trigger();
    block_sum2(rr, unused);
    if (publish_inst(rr, unused, red, p.ntasks, t.inst, p.inst_count[t.inst])) {
        double RR, U;
        gather_inst(red, p.ntasks, t.inst, p.inst_first[t.inst], p.inst_count[t.inst], RR, U);
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
            }
        }
    }
}

// rz = r.z, z.Ap, flexible beta; items = value pairs.
__global__ void __launch_bounds__(NT)
    kb_dot64(Plan p, const BInst* __restrict__ bi, Ctl* ctl, BRed red, BCtl* bc, Cond cond) {
    pdl_enter();
    const Task t = p.tasks[blockIdx.x];
    Ctl* c = &ctl[t.inst];
    if (inst_done(c)) return;
    const BInst I = bi[t.inst];
    const double2* __restrict__ r2 = reinterpret_cast<const double2*>(I.r64);
    const double2* __restrict__ a2 = reinterpret_cast<const double2*>(I.Ap64);
    const float2* __restrict__ z2 = reinterpret_cast<const float2*>(I.z);
    double rz = 0.0, zap = 0.0;
    struct Item {
        double2 r, a;
        float2 z;
    };
    stream_pipelined<2, Item>(
        t.begin + threadIdx.x, t.end, NT, [&](unsigned k) { return Item{r2[k], a2[k], z2[k]}; },
        [&](unsigned, const Item& it) {
            const double za = widen(it.z.x), zb = widen(it.z.y);
            rz = __fma_rn(it.r.x, za, rz);
            rz = __fma_rn(it.r.y, zb, rz);
            zap = __fma_rn(za, it.a.x, zap);
            zap = __fma_rn(zb, it.a.y, zap);
        });
    pdl_trigger();
    block_sum2(rz, zap);
    if (publish_inst(rz, zap, red, p.ntasks, t.inst, p.inst_count[t.inst])) {
        double RZ, ZAP;
        gather_inst(red, p.ntasks, t.inst, p.inst_first[t.inst], p.inst_count[t.inst], RZ, ZAP);
        if (threadIdx.x == 0) {
            c->beta = c->iter > 0 ? -ZAP / c->pAp : 0.0;
            c->rz = RZ;
            c->zAp = ZAP;
            if (!isfinite(RZ) || !isfinite(c->beta)) {
                c->breakdown = 1;
                inst_stop(c, bc, cond);
            }
        }
    }
}

// p = z + beta p (p = z on the first iteration); items = value pairs.
__global__ void __launch_bounds__(NT)
    kb_update_p64(Plan p, const BInst* __restrict__ bi, const Ctl* ctl) {
    pdl_enter();
    const Task t = p.tasks[blockIdx.x];
    const Ctl* c = &ctl[t.inst];
    if (inst_done(c)) return;
    const BInst I = bi[t.inst];
    const double beta = c->beta;
    const bool first = c->iter == 0;
    const float2* __restrict__ z2 = reinterpret_cast<const float2*>(I.z);
    double2* __restrict__ p2 = reinterpret_cast<double2*>(I.p64);
    if (first) {
        for (unsigned k = t.begin + threadIdx.x; k < t.end; k += NT) {
            const float2 zf = z2[k];
            p2[k] = make_double2(widen(zf.x), widen(zf.y));
        }
        return;
    }
    struct Item {
        double2 p;
        float2 z;
    };
    stream_pipelined<2, Item>(
        t.begin + threadIdx.x, t.end, NT, [&](unsigned k) { return Item{p2[k], z2[k]}; },
        [&](unsigned k, const Item& it) {
            p2[k] = make_double2(__fma_rn(beta, it.p.x, widen(it.z.x)), __fma_rn(beta, it.p.y, widen(it.z.y)));
        });
}

}  // namespace

void launch_b_residual64(cudaStream_t st, const Plan& p, const BInst* bi, Ctl* ctl, BRed red, BCtl* bc,
                         Cond cond) {
    launch_pdl(kb_residual64, p.ntasks, NT, 0, st, p, bi, ctl, red, bc, cond);
}

void launch_b_apply64(cudaStream_t st, const Plan& p, const BInst* bi, Ctl* ctl, BRed red, BCtl* bc,
                      Cond cond) {
    launch_pdl(kb_apply64, p.ntasks, NT, 0, st, p, bi, ctl, red, bc, cond);
}

void launch_b_update64(cudaStream_t st, const Plan& p, const BInst* bi, Ctl* ctl, BRed red, BCtl* bc,
                       Cond cond) {
    launch_pdl(kb_update64, p.ntasks, NT, 0, st, p, bi, ctl, red, bc, cond);
}

void launch_b_dot64(cudaStream_t st, const Plan& p, const BInst* bi, Ctl* ctl, BRed red, BCtl* bc,
                    Cond cond) {
    launch_pdl(kb_dot64, p.ntasks, NT, 0, st, p, bi, ctl, red, bc, cond);
}

void launch_b_update_p64(cudaStream_t st, const Plan& p, const BInst* bi, const Ctl* ctl) {
    launch_pdl(kb_update_p64, p.ntasks, NT, 0, st, p, bi, ctl);
}

}  // namespace ct
