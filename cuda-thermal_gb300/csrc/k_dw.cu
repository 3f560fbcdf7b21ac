// k_dw.cu - the outer PCG on the FP32 pipes: double-word (float-pair)
// arithmetic for CT_MG_FP32_FLEX_DW.
//
// On GB300 an FP64 instruction issues at ~1/70 of the FP32 rate (and float <->
// double conversions at the FP64 rate), so the FP64 outer kernels of the
// reference's algorithm are bound by the FP64 pipe, not by HBM. Here x, r, p,
// Ap and the diagonal are stored as float pairs (hi, lo) - the same 8 bytes
// per value as a double - and combined with error-free transformations
// (TwoSum, Fast2Sum, FMA-based TwoProd; Joldes, Muller and Popescu, "Tight
// and rigorous error bounds for basic building blocks of double-word
// arithmetic", 2017), which carry ~48 significant bits. Dot products are
// accumulated in double words per thread, per block and over the grid (on the
// FP32 pipe; only the grid's total is converted); alpha and beta stay FP64
// scalars on the device.
//
// Two limits of 48 bits, and how they are lifted:
//  - the recurrence residual drifts from the true residual by ~2^-48 times the
//    operator's cancellation (up to ~1e4 here). So the solve recomputes
//    r = b - A x once in FP64 (k_residual_x, "residual replacement") when the
//    recurrence first passes a threshold (1e-5 by default);
//  - a 48-bit x cannot hold T (~50 K) finely enough for ||P - A T|| / ||P|| to
//    reach 1e-10 where lateral conductances are large (the copper spreader).
//    So x is an FP64 base xb plus a double-word correction xw: the iteration
//    updates xw, and k_fold adds xw into xb (in FP64) before every FP64
//    residual - at the start and at the replacement - after which xw only
//    carries the small remaining correction.
#include <algorithm>
#include <cmath>
#include <cstdlib>

#include "dw_dev.cuh"
#include "kernels.h"
#include "reduce.cuh"

namespace ct {

using namespace dwdev;

namespace {

// Block b of the grid streams the contiguous items [begin, end) with stride
// NT (as a batched task does) rather than striding over the whole vector.
struct BlockRange {
    unsigned begin, end;
};
__device__ __forceinline__ BlockRange block_range(unsigned n) {
    const unsigned per = ((n + gridDim.x - 1) / gridDim.x + NT * kU - 1) / (NT * kU) * (NT * kU);
    const unsigned b = blockIdx.x * per;
    return BlockRange{b + threadIdx.x, b + per < n ? b + per : n};
}

// ---- FP64 residual from a double-word x: start and replacement -------------

// r = b - (A + C/dt) x in FP64 with x = hi + lo, the stored FP64 diagonal;
// stores r as a double word and b0 = r (float, the V-cycle's input). `start`:
// the first residual of a solve (sets ||b||^2 and the start test); otherwise
// the residual replacement (phase 2 begins, or the solve ends if already
// converged).
__global__ void __launch_bounds__(NT)
    k_residual_x(OpView o, const double* __restrict__ diag, const double* __restrict__ b,
                 const double* __restrict__ x, float2* __restrict__ r, float* __restrict__ b0,
                 int start, Ctl* ctl, double* part, int maxb, Cond cond) {
    pdl_enter();
    if (!start && *(volatile const int*)&ctl->done) {  // converged or stopped in phase 1
        if (cond.use && blockIdx.x == 0 && threadIdx.x == 0) cudaGraphSetConditional(cond.h, 0u);
        return;
    }
    const Geo& g = o.g;
    double rr = 0.0, bb = 0.0;
    // A solve that starts from x = 0 (every steady solve) has r = b exactly.
    const bool zero = start && ctl->x_zero;
    for (unsigned s = blockIdx.x * NT + threadIdx.x; s < g.plane; s += gridDim.x * NT) {
        const Col c = col_of_slot(g, s);
        if (!c.valid) {
            for (int l = 0; l < g.nz; ++l) {
                r[(unsigned)l * g.plane + s] = make_float2(0.0f, 0.0f);
                b0[(unsigned)l * g.plane + s] = 0.0f;
            }
            continue;
        }
        if (zero) {
            for (int l = 0; l < g.nz; ++l) {
                const unsigned id = (unsigned)l * g.plane + c.s;
                const double bi = b[id];
                const float2 rw = dw_of(bi);
                r[id] = rw;
                b0[id] = rw.x;
                bb += bi * bi;
            }
            continue;
        }
        double x_c = x[c.s], x_b = 0.0;
        float gu_b = 0.0f;
        for (int l = 0; l < g.nz; ++l) {
            const unsigned base = (unsigned)l * g.plane, id = base + c.s;
            const bool up = l < g.nz - 1;
            const double x_a = up ? x[id + g.plane] : 0.0;
            const float gu = o.gU[id];
            double off = 0.0;
            if (c.i > 0) off += (double)o.gE[base + c.sw] * x[base + c.sw];
            if (c.i < g.nx - 1) off += (double)o.gE[id] * x[base + c.se];
            if (c.j > 0) off += (double)o.gN[base + c.ss] * x[base + c.ss];
            if (c.j < g.ny - 1) off += (double)o.gN[id] * x[base + c.sn];
            if (l > 0) off += (double)gu_b * x_b;
            if (up) off += (double)gu * x_a;
            const double bi = b[id];
            const double ri = bi - (diag[id] * x_c - off);
            const float2 rw = dw_of(ri);
            r[id] = rw;
            b0[id] = rw.x;
            rr += ri * ri;
            bb += bi * bi;
            x_b = x_c;
            x_c = x_a;
            gu_b = gu;
        }
    }
    if (zero) rr = bb;
    block_sum2(rr, bb);
    if (publish2(rr, bb, part, maxb, &ctl->ticket[SL_INIT])) {
        double RR, BB;
        gather2(part, maxb, &ctl->ticket[SL_INIT], RR, BB);
        if (threadIdx.x == 0) {
            ctl->rr = RR;
            if (start) {
                ctl->bb = BB;
                if (BB == 0.0) {
                    ctl->bb_zero = 1;
                    ctl->converged = 1;
                    ctl->relres = 0.0;
                    stop_loop(ctl, cond);
                    return;
                }
            }
            const double rel = sqrt(RR / ctl->bb);
            ctl->relres = rel;
            ctl->phase_end = 0;
            if (!start) ctl->stop = ctl->tol;  // phase 2 runs to tol
            if (rel < ctl->tol) {
                ctl->converged = 1;
                stop_loop(ctl, cond);
            } else if (!isfinite(rel)) {
                ctl->breakdown = 1;
                stop_loop(ctl, cond);
            } else if (ctl->iter >= ctl->maxit) {
                stop_loop(ctl, cond);
            }
        }
    }
}

// ---- the iteration ------------------------------------------------------------

// Ap = d p - sum G p_nbr (op_apply, src/operator3d.h:108-112), p.Ap and
// alpha: one warp per row of one colour of one plane (no integer division per
// cell), two cells per lane, products summed with DwAcc.
__global__ void __launch_bounds__(NT)
    k_apply_dw_rows(OpView o, const float2* __restrict__ dgw, const float2* __restrict__ p,
                    float2* __restrict__ Ap, Ctl* ctl, double* part, int maxb, Cond cond) {
    pdl_enter();
    if (loop_done(ctl, cond)) return;
    const Geo& g = o.g;
    const unsigned rows = 2u * (unsigned)g.ny * (unsigned)g.nz;
    const int lane = (int)(threadIdx.x & 31u);
    DwAcc acc = {0.0f, 0.0f};
    for (unsigned R = blockIdx.x * (NT / 32) + (threadIdx.x >> 5); R < rows; R += gridDim.x * (NT / 32))
        apply_row<2>(o, dgw, p, Ap, R, lane, acc);
    DwAcc unused = {0.0f, 0.0f};
    pdl_trigger();
    block_sum_acc2(acc, unused);
    if (publish_acc2(acc, unused, part, maxb, blockIdx.x, &ctl->ticket[SL_APPLY], gridDim.x)) {
        double PAP, U;
        gather_acc2(part, maxb, 0u, gridDim.x, &ctl->ticket[SL_APPLY], PAP, U);
        if (threadIdx.x == 0) {
            ctl->pAp = PAP;
            if (!(PAP > 0.0) || !isfinite(PAP)) {
                ctl->breakdown = 1;
                ctl->alpha = 0.0;
                stop_loop(ctl, cond);
            } else {
                ctl->alpha = ctl->rz / PAP;
                ctl->alpha_w = dw_of(ctl->alpha);
            }
        }
    }
}


// x += alpha p, r -= alpha Ap, b0 = r (hi word), ||r||^2, convergence test.
// Two values per thread and step (float4 = two double words).
__global__ void __launch_bounds__(NT)
    k_update_dw(unsigned n2, const float4* __restrict__ p, const float4* __restrict__ Ap,
                float4* __restrict__ x, float4* __restrict__ r, float2* __restrict__ b0, Ctl* ctl,
                double* part, int maxb, Cond cond) {
    pdl_enter();
    if (loop_done(ctl, cond)) return;
    DwAcc acc = {0.0f, 0.0f};
    const BlockRange br = block_range(n2);
    update_range(br.begin, br.end, NT, ctl->alpha_w, p, Ap, x, r, b0, acc);
    DwAcc unused = {0.0f, 0.0f};
    pdl_trigger();
    block_sum_acc2(acc, unused);
    if (publish_acc2(acc, unused, part, maxb, blockIdx.x, &ctl->ticket[SL_UPDATE], gridDim.x)) {
        double RR, U;
        gather_acc2(part, maxb, 0u, gridDim.x, &ctl->ticket[SL_UPDATE], RR, U);
        if (threadIdx.x == 0) {
            ctl->rr = RR;
            ctl->iter += 1;
            const double rel = sqrt(RR / ctl->bb);
            ctl->relres = rel;
            if (rel < ctl->tol) {
                ctl->converged = 1;
                stop_loop(ctl, cond);
            } else if (!isfinite(rel)) {
                ctl->breakdown = 1;
                stop_loop(ctl, cond);
            } else if (ctl->iter >= ctl->maxit) {
                stop_loop(ctl, cond);
            } else if (rel < ctl->stop) {
                // end of phase 1: the next step is the FP64 residual replacement
                ctl->phase_end = 1;
                if (cond.use) cudaGraphSetConditional(cond.h, 0u);
            }
        }
    }
}

// rz = r.z and z.Ap (flexible beta); beta. Items strided over the whole grid
// on 4 blocks per SM, compiled for 4 blocks per SM: 31.7 us at 800 x 800 x 10
// against 32.9 us with the compiler's own register choice and 34.5 us with
// one contiguous range per block on 6 blocks per SM.
__global__ void __launch_bounds__(NT, 4)
    k_dot_dw(unsigned n2, const float4* __restrict__ r, const float2* __restrict__ z,
             const float4* __restrict__ Ap, Ctl* ctl, double* part, int maxb, Cond cond) {
    pdl_enter();
    if (loop_done(ctl, cond)) return;
    DwAcc rz = {0.0f, 0.0f}, zap = {0.0f, 0.0f};
    dot_range(blockIdx.x * NT + threadIdx.x, n2, gridDim.x * NT, r, z, Ap, rz, zap);
    pdl_trigger();
    block_sum_acc2(rz, zap);
    if (publish_acc2(rz, zap, part, maxb, blockIdx.x, &ctl->ticket[SL_DOT], gridDim.x)) {
        double RZ, ZAP;
        gather_acc2(part, maxb, 0u, gridDim.x, &ctl->ticket[SL_DOT], RZ, ZAP);
        if (threadIdx.x == 0) {
            ctl->beta = ctl->iter > 0 ? -ZAP / ctl->pAp : 0.0;
            ctl->beta_w = dw_of(ctl->beta);
            ctl->rz = RZ;
            ctl->zAp = ZAP;
            if (!isfinite(RZ) || !isfinite(ctl->beta)) {
                ctl->breakdown = 1;
                stop_loop(ctl, cond);
            }
        }
    }
}

// p = z + beta p (p = z on the first iteration).
__global__ void __launch_bounds__(NT)
    k_update_p_dw(unsigned n2, const float2* __restrict__ z, float4* __restrict__ p, const Ctl* ctl,
                  Cond cond) {
    pdl_enter();
    if (loop_done(ctl, cond)) return;
    const BlockRange br = block_range(n2);
    update_p_range(br.begin, br.end, NT, ctl->beta_w, ctl->iter == 0, z, p);
}

// xb += xw (in FP64), xw = 0: the double-word correction goes into the base.
// Skipped (all blocks) once the solve is done; runs before the residual
// replacement, which is what it serves.
__global__ void k_fold(unsigned n2, double2* __restrict__ xb, float4* __restrict__ xw,
                       const Ctl* ctl, int check_done) {
    pdl_enter();
    if (check_done && *(volatile const int*)&ctl->done) return;
    for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < n2; k += gridDim.x * blockDim.x) {
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

// ---- conversions at the boundary -------------------------------------------

// FP64 diagonal -> double word.
__global__ void k_to_dw(unsigned n, const double* __restrict__ in, float2* __restrict__ out) {
    for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
        out[k] = dw_of(in[k]);
}

// split double word -> natural double.
__global__ void k_dw_to_natural(Geo g, const float2* __restrict__ in, double* __restrict__ out) {
    const size_t nxy = (size_t)g.nx * g.ny;
    const size_t n = nxy * (size_t)g.nz;
    for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n;
         c += (size_t)gridDim.x * blockDim.x) {
        const int l = (int)(c / nxy);
        const size_t rem = c - (size_t)l * nxy;
        const int j = (int)(rem / g.nx), i = (int)(rem - (size_t)j * g.nx);
        out[c] = dw_d(in[(size_t)l * g.plane + scol(g, i, j)]);
    }
}

// natural double -> split double word.
__global__ void k_natural_to_dw(Geo g, const double* __restrict__ in, float2* __restrict__ out) {
    const size_t nxy = (size_t)g.nx * g.ny;
    const size_t n = nxy * (size_t)g.nz;
    for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n;
         c += (size_t)gridDim.x * blockDim.x) {
        const int l = (int)(c / nxy);
        const size_t rem = c - (size_t)l * nxy;
        const int j = (int)(rem / g.nx), i = (int)(rem - (size_t)j * g.nx);
        out[(size_t)l * g.plane + scol(g, i, j)] = dw_of(in[c]);
    }
}

// split double word -> split double (for the FP64 bookkeeping kernels).
__global__ void k_dw_to_d(unsigned n, const float2* __restrict__ in, double* __restrict__ out) {
    for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
        out[k] = dw_d(in[k]);
}

unsigned blocks_of(size_t n) {
    size_t b = (n + NT - 1) / NT;
    if (b < 1) b = 1;
    if (b > 65535u * 16u) b = 65535u * 16u;
    return (unsigned)b;
}

}  // namespace

void launch_fold(cudaStream_t st, unsigned n, double* xb, float2* xw, const Ctl* ctl,
                 bool check_done) {
    static const int wb = wave_blocks(k_fold, 1 << 30);
    launch_pdl(k_fold, std::min((int)blocks_of(n / 2), wb), NT, 0, st, n / 2, (double2*)xb, (float4*)xw, ctl,
                                                               check_done ? 1 : 0);
}

void launch_residual_x(cudaStream_t st, const OpView& o, const double* diag, const double* b,
                       const double* x, float2* r, float* b0, bool start, Ctl* ctl,
                       const Red& red, Cond cond) {
    static const int wb = wave_blocks(k_residual_x, 1 << 30);
    launch_pdl(k_residual_x, std::min(red.blocks, wb), NT, 0, st, o, diag, b, x, r, b0, start ? 1 : 0, ctl, red.part,
                                            red.maxb, cond);
}

void launch_apply_dw(cudaStream_t st, const OpView& o, const float2* dgw, const float2* p,
                     float2* Ap, Ctl* ctl, const Red& red, Cond cond) {
    static const int wb = wave_blocks(k_apply_dw_rows, 1 << 30);
    launch_pdl(k_apply_dw_rows, std::min(red.maxb, wb), NT, 0, st, o, dgw, p, Ap, ctl, red.part, red.maxb, cond);
}

void launch_update_dw(cudaStream_t st, unsigned n, const float2* p, const float2* Ap, float2* x,
                      float2* r, float* b0, Ctl* ctl, const Red& red, Cond cond) {
    static const int wb = wave_blocks(k_update_dw, 1 << 30);
    launch_pdl(k_update_dw, std::min(red.blocks, wb), NT, 0, st, n / 2, (const float4*)p, (const float4*)Ap, (float4*)x,
                                           (float4*)r, (float2*)b0, ctl, red.part, red.maxb, cond);
}

void launch_dot_dw(cudaStream_t st, unsigned n, const float2* r, const float* z, const float2* Ap,
                   Ctl* ctl, const Red& red, Cond cond) {
    static const int wb = wave_blocks(k_dot_dw, 1 << 30);
    launch_pdl(k_dot_dw, std::min(std::max(1, red.maxb / 2), wb), NT, 0, st, n / 2, (const float4*)r,
               (const float2*)z, (const float4*)Ap, ctl, red.part, red.maxb, cond);
}

void launch_update_p_dw(cudaStream_t st, unsigned n, const float* z, float2* p, Ctl* ctl,
                        Cond cond) {
    static const int wb = wave_blocks(k_update_p_dw, 1 << 30);
    launch_pdl(k_update_p_dw, std::min((int)blocks_of(n / 2), wb), NT, 0, st, n / 2, (const float2*)z, (float4*)p, ctl,
               cond);
}

void launch_to_dw(cudaStream_t st, unsigned n, const double* in, float2* out) {
    k_to_dw<<<blocks_of(n), NT, 0, st>>>(n, in, out);
}

void launch_dw_to_natural(cudaStream_t st, const Geo& g, const float2* split, double* nat) {
    k_dw_to_natural<<<blocks_of((size_t)g.nx * g.ny * g.nz), NT, 0, st>>>(g, split, nat);
}

void launch_natural_to_dw(cudaStream_t st, const Geo& g, const double* nat, float2* split) {
    k_natural_to_dw<<<blocks_of((size_t)g.nx * g.ny * g.nz), NT, 0, st>>>(g, nat, split);
}

void launch_dw_to_d(cudaStream_t st, unsigned n, const float2* in, double* out) {
    k_dw_to_d<<<blocks_of(n), NT, 0, st>>>(n, in, out);
}

}  // namespace ct
