// k_fp64.cu - the FP64 outer PCG of the multigrid modes (CT_MG_FP32_FLEX,
// CT_MG_FP32, CT_MG_FP64): residual, operator apply, x/r update, dot
// products and p update, all in IEEE double arithmetic as the reference's
// outer iteration is (Real = double, src/pcg3d.h:18-22; k_residual,
// k_apply, k_update_xr, k_mg_dot, k_update_p_mg, src/pcg3d_gpu.cu:159-256).
//
// On GB300 these kernels are bound by the FP64 pipe, not by HBM: a DFMA
// issues at ~1/70 of the FFMA rate (0.53 T/s on 152 SMs), so at 800 x 800 x
// 10 every FP64 instruction per cell costs ~12 us while an 8-byte stream
// costs ~7.5 us at the measured copy bandwidth. So each kernel does the
// fewest FP64 instructions the algorithm needs: the float face conductances
// and V-cycle values are widened to double, and the residual narrowed to the
// V-cycle's float, with exact integer conversions (f64_dev.cuh) instead of
// the FP64-rate hardware conversions, and every multiply-add is one DFMA.
// Per cell: apply 8 (7 for Ap, 1 for p.Ap), update 3, dot 2, p update 1.
// The memory side follows the double-word kernels (k_dw.cu): the apply runs
// one warp per row of one colour and plane (no index division per cell),
// the streaming kernels keep several items in flight per thread, and every
// kernel is launched with programmatic dependent launch.
#include <algorithm>
#include <cmath>

#include "f64_dev.cuh"
#include "kernels.h"
#include "reduce.cuh"

namespace ct {

using namespace f64dev;

namespace {

constexpr int kRowU = 2;

// Ap = (A + C/dt) p, p.Ap and alpha = rz / p.Ap.
__global__ void __launch_bounds__(NT)
    k_apply64(OpView o, const double* __restrict__ diag, const double* __restrict__ p,
              double* __restrict__ Ap, Ctl* ctl, double* part, int maxb, Cond cond) {
    pdl_enter();
    if (loop_done(ctl, cond)) return;
    const Geo& g = o.g;
    const unsigned rows = 2u * (unsigned)g.ny * (unsigned)g.nz;
    const int lane = (int)(threadIdx.x & 31u);
    double pap = 0.0, unused = 0.0;
    for (unsigned R = blockIdx.x * (NT / 32) + (threadIdx.x >> 5); R < rows; R += gridDim.x * (NT / 32))
        row64<kRowU>(o, diag, p, R, lane, [&](unsigned k, bool valid, double av, double pc) {
            Ap[k] = av;
            if (valid) pap = __fma_rn(pc, av, pap);
        });
    pdl_trigger();
    block_sum2(pap, unused);
    if (publish2(pap, unused, part, maxb, &ctl->ticket[SL_APPLY])) {
        double PAP, U;
        gather2(part, maxb, &ctl->ticket[SL_APPLY], PAP, U);
        if (threadIdx.x == 0) {
            ctl->pAp = PAP;
            if (!(PAP > 0.0) || !isfinite(PAP)) {  // A is SPD: p.Ap > 0 unless p = 0
                ctl->breakdown = 1;
                ctl->alpha = 0.0;
                stop_loop(ctl, cond);
            } else {
                ctl->alpha = ctl->rz / PAP;
            }
        }
    }
}

// The start test of a solve from its residual sums (src/pcg3d_cpu.cpp:142-150).
__device__ __forceinline__ void start_test(Ctl* ctl, Cond cond, double RR, double BB) {
    ctl->rr = RR;
    ctl->bb = BB;
    if (BB == 0.0) {  // no heat in: x = 0 (src/pcg3d_cpu.cpp:146)
        ctl->bb_zero = 1;
        ctl->converged = 1;
        ctl->relres = 0.0;
        stop_loop(ctl, cond);
        return;
    }
    const double rel = sqrt(RR / BB);
    ctl->relres = rel;
    if (rel < ctl->tol) {
        ctl->converged = 1;
        stop_loop(ctl, cond);
    } else if (!isfinite(rel)) {
        ctl->breakdown = 1;
        stop_loop(ctl, cond);
    } else if (ctl->maxit <= 0) {
        stop_loop(ctl, cond);
    }
}

// ---- streaming kernels ---------------------------------------------------------

// Block b streams the contiguous items [begin, end), NT apart, in chunks of
// NT * U items.
struct Range {
    unsigned begin, end;
};
template <int U>
__device__ __forceinline__ Range block_range(unsigned n) {
    const unsigned per = ((n + gridDim.x - 1) / gridDim.x + NT * U - 1) / (NT * U) * (NT * U);
    const unsigned b = blockIdx.x * per;
    return Range{b + threadIdx.x, b + per < n ? b + per : n};
}

// Two values of the V-cycle's precision at pair index k, as doubles.
__device__ __forceinline__ double2 load_pair(const float* z, unsigned k) {
    const float2 v = reinterpret_cast<const float2*>(z)[k];
    return make_double2(widen(v.x), widen(v.y));
}
__device__ __forceinline__ double2 load_pair(const double* z, unsigned k) {
    return reinterpret_cast<const double2*>(z)[k];
}
__device__ __forceinline__ void store_pair(float* b0, unsigned k, double a, double b) {
    reinterpret_cast<float2*>(b0)[k] = make_float2(narrow(a), narrow(b));
}
__device__ __forceinline__ void store_pair(double* b0, unsigned k, double a, double b) {
    reinterpret_cast<double2*>(b0)[k] = make_double2(a, b);
}

// r = b - (A + C/dt) x, b0 = r in the V-cycle precision, ||r||^2, ||b||^2 and
// the start test. A solve that starts from x = 0 (every steady solve) has
// r = b exactly and streams b once.
template <class T>
__global__ void __launch_bounds__(NT)
    k_residual64(OpView o, unsigned n, const double* __restrict__ diag, const double* __restrict__ b,
                 const double* __restrict__ x, double* __restrict__ r, T* __restrict__ b0, Ctl* ctl,
                 double* part, int maxb, Cond cond) {
    pdl_enter();
    const Geo& g = o.g;
    double rr = 0.0, bb = 0.0;
    if (ctl->x_zero) {
        // r = b, streamed in pairs with the next items' loads issued before
        // the current ones are stored (n is even: whole rows of both colours)
        const double2* b2 = reinterpret_cast<const double2*>(b);
        double2* r2 = reinterpret_cast<double2*>(r);
        stream_pipelined<2, double2>(
            blockIdx.x * NT + threadIdx.x, n / 2, gridDim.x * NT, [&](unsigned k) { return b2[k]; },
            [&](unsigned k, const double2& v) {
                r2[k] = v;
                store_pair(b0, k, v.x, v.y);
                bb = __fma_rn(v.x, v.x, bb);
                bb = __fma_rn(v.y, v.y, bb);
            });
        rr = bb;
    } else {
        const unsigned rows = 2u * (unsigned)g.ny * (unsigned)g.nz;
        const int lane = (int)(threadIdx.x & 31u);
        for (unsigned R = blockIdx.x * (NT / 32) + (threadIdx.x >> 5); R < rows;
             R += gridDim.x * (NT / 32))
            row64<kRowU>(o, diag, x, R, lane, [&](unsigned k, bool valid, double ax, double) {
                if (!valid) {
                    r[k] = 0.0;
                    b0[k] = T(0);
                    return;
                }
                const double bi = b[k];
                const double ri = bi - ax;
                r[k] = ri;
                b0[k] = from_d<T>(ri);
                rr = __fma_rn(ri, ri, rr);
                bb = __fma_rn(bi, bi, bb);
            });
    }
    block_sum2(rr, bb);
    if (publish2(rr, bb, part, maxb, &ctl->ticket[SL_INIT])) {
        double RR, BB;
        gather2(part, maxb, &ctl->ticket[SL_INIT], RR, BB);
        if (threadIdx.x == 0) start_test(ctl, cond, RR, BB);
    }
}

// x += alpha p, r -= alpha Ap, b0 = r in the V-cycle precision, ||r||^2 and
// the convergence test (src/pcg3d_gpu.cu:218-233). Pairs of values (double2),
// each block a contiguous range.
constexpr int kUpdU = 1;
struct UpdItem {
    double2 p, a, x, r;
};
struct UpdItemR {
    double2 a, r;
};
// WX = false: x is left to k_update_x64 (x += alpha p off the critical path,
// beside the next V-cycle); alpha is kept in ctl->alpha_x for it.
// The r-only form keeps 4 pairs in flight a thread (98 registers): 36.8 us
// against 40.9 us with 2 and 43.0 us with 1 at 800 x 800.
template <class T, bool WX, int UR = 4>
__global__ void __launch_bounds__(NT)
    k_update64(unsigned n2, const double2* __restrict__ p, const double2* __restrict__ Ap,
               double2* __restrict__ x, double2* __restrict__ r, T* __restrict__ b0, Ctl* ctl,
               double* part, int maxb, Cond cond) {
    pdl_enter();
    if (loop_done(ctl, cond)) return;
    const double alpha = ctl->alpha, malpha = -alpha;
    double rr = 0.0, unused = 0.0;
    const Range br = block_range<2>(n2);
    if constexpr (WX) {
        stream_pipelined<kUpdU, UpdItem>(
            br.begin, br.end, NT,
            [&](unsigned k) { return UpdItem{p[k], Ap[k], x[k], r[k]}; },
            [&](unsigned k, UpdItem it) {
                it.x.x = __fma_rn(alpha, it.p.x, it.x.x);
                it.x.y = __fma_rn(alpha, it.p.y, it.x.y);
                it.r.x = __fma_rn(malpha, it.a.x, it.r.x);
                it.r.y = __fma_rn(malpha, it.a.y, it.r.y);
                x[k] = it.x;
                r[k] = it.r;
                store_pair(b0, k, it.r.x, it.r.y);
                rr = __fma_rn(it.r.x, it.r.x, rr);
                rr = __fma_rn(it.r.y, it.r.y, rr);
            });
    } else {
        if (blockIdx.x == 0 && threadIdx.x == 0) ctl->alpha_x = alpha;
        stream_pipelined<UR, UpdItemR>(
            br.begin, br.end, NT,
            [&](unsigned k) { return UpdItemR{Ap[k], r[k]}; },
            [&](unsigned k, UpdItemR it) {
                it.r.x = __fma_rn(malpha, it.a.x, it.r.x);
                it.r.y = __fma_rn(malpha, it.a.y, it.r.y);
                r[k] = it.r;
                store_pair(b0, k, it.r.x, it.r.y);
                rr = __fma_rn(it.r.x, it.r.x, rr);
                rr = __fma_rn(it.r.y, it.r.y, rr);
            });
    }
    pdl_trigger();
    block_sum2(rr, unused);
    if (publish2(rr, unused, part, maxb, &ctl->ticket[SL_UPDATE])) {
        double RR, U;
        gather2(part, maxb, &ctl->ticket[SL_UPDATE], RR, U);
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
            }
        }
    }
}

// x += alpha p with the alpha k_update64<T, false> left in ctl->alpha_x (0:
// nothing pending), the same rounding as the fused update. It runs beside the
// V-cycle of the next iteration (or after the loop for the last one) and
// before the p update of that iteration, which clears alpha_x.
struct XItem {
    double2 p, x;
};
__global__ void __launch_bounds__(NT)
    k_update_x64(unsigned n2, const double2* __restrict__ p, double2* __restrict__ x, const Ctl* ctl) {
    const double alpha = *(volatile const double*)&ctl->alpha_x;
    if (alpha == 0.0) return;
    stream_pipelined<4, XItem>(
        blockIdx.x * NT + threadIdx.x, n2, gridDim.x * NT, [&](unsigned k) { return XItem{p[k], x[k]}; },
        [&](unsigned k, const XItem& it) {
            x[k] = make_double2(__fma_rn(alpha, it.p.x, it.x.x), __fma_rn(alpha, it.p.y, it.x.y));
        });
}

// rz = r.z (and z.Ap for the flexible beta); beta (src/pcg3d_gpu.cu:239-247,
// 121-126). Pairs strided over the whole grid.
constexpr int kDotU = 2;
struct DotItem {
    double2 r, z, a;
};
template <class T>
struct DotItemN {
    double2 r;
    float2 z;
    double2 a;
};
template <class T, bool FLEX, int DU = kDotU>
__global__ void __launch_bounds__(NT)
    k_dot64(unsigned n2, const double2* __restrict__ r, const T* __restrict__ z,
            const double2* __restrict__ Ap, Ctl* ctl, double* part, int maxb, Cond cond) {
    pdl_enter();
    if (loop_done(ctl, cond)) return;
    double rz = 0.0, zap = 0.0;
    if constexpr (sizeof(T) == 4) {
        // z kept as loaded (a float pair) until it is used: 2 registers an item
        // fewer than widening it at the load (42.7 -> 38.7 us at 800 x 800)
        const float2* z2 = reinterpret_cast<const float2*>(z);
        stream_pipelined<DU, DotItemN<T>>(
            blockIdx.x * NT + threadIdx.x, n2, gridDim.x * NT,
            [&](unsigned k) {
                return DotItemN<T>{r[k], z2[k], FLEX ? Ap[k] : make_double2(0.0, 0.0)};
            },
            [&](unsigned, const DotItemN<T>& it) {
                const double zx = widen(it.z.x), zy = widen(it.z.y);
                rz = __fma_rn(it.r.x, zx, rz);
                rz = __fma_rn(it.r.y, zy, rz);
                if (FLEX) {
                    zap = __fma_rn(zx, it.a.x, zap);
                    zap = __fma_rn(zy, it.a.y, zap);
                }
            });
    } else {
        stream_pipelined<kDotU, DotItem>(
            blockIdx.x * NT + threadIdx.x, n2, gridDim.x * NT,
            [&](unsigned k) {
                return DotItem{r[k], load_pair(z, k), FLEX ? Ap[k] : make_double2(0.0, 0.0)};
            },
            [&](unsigned, const DotItem& it) {
                rz = __fma_rn(it.r.x, it.z.x, rz);
                rz = __fma_rn(it.r.y, it.z.y, rz);
                if (FLEX) {
                    zap = __fma_rn(it.z.x, it.a.x, zap);
                    zap = __fma_rn(it.z.y, it.a.y, zap);
                }
            });
    }
    pdl_trigger();
    block_sum2(rz, zap);
    if (publish2(rz, zap, part, maxb, &ctl->ticket[SL_DOT])) {
        double RZ, ZAP;
        gather2(part, maxb, &ctl->ticket[SL_DOT], RZ, ZAP);
        if (threadIdx.x == 0) {
            if (ctl->iter > 0) {
                // Fletcher-Reeves (src/pcg3d_cpu.cpp:179) or flexible
                // Polak-Ribiere: z_new.(r_new - r_old) / (z_old . r_old)
                // = -(z_new . Ap) / (p . Ap).
                ctl->beta = FLEX ? -ZAP / ctl->pAp : RZ / ctl->rz;
            } else {
                ctl->beta = 0.0;
            }
            ctl->rz = RZ;
            ctl->zAp = ZAP;
            if (!isfinite(RZ) || !isfinite(ctl->beta)) {
                ctl->breakdown = 1;
                stop_loop(ctl, cond);
            }
        }
    }
}

// p = z + beta p (p = z on the first iteration; src/pcg3d_gpu.cu:249-256).
constexpr int kPU = 2;
struct PItem {
    double2 z, p;
};
template <class T>
__global__ void __launch_bounds__(NT)
    k_update_p64(unsigned n2, const T* __restrict__ z, double2* __restrict__ p, Ctl* ctl,
                 Cond cond) {
    pdl_enter();
    // the pending x update (k_update_x64) has run by now: none pending after
    // this point, also when the loop has ended
    if (blockIdx.x == 0 && threadIdx.x == 0) ctl->alpha_x = 0.0;
    if (loop_done(ctl, cond)) return;
    const double beta = ctl->beta;
    const Range br = block_range<2 * kPU>(n2);
    if (ctl->iter == 0) {
        for (unsigned k = br.begin; k < br.end; k += NT) p[k] = load_pair(z, k);
        return;
    }
    if constexpr (sizeof(T) == 4) {
        // z kept as loaded (a float pair) until it is used, as in k_dot64
        struct Item {
            float2 z;
            double2 p;
        };
        const float2* z2 = reinterpret_cast<const float2*>(z);
        stream_pipelined<kPU, Item>(
            br.begin, br.end, NT, [&](unsigned k) { return Item{z2[k], p[k]}; },
            [&](unsigned k, const Item& it) {
                p[k] = make_double2(__fma_rn(beta, it.p.x, widen(it.z.x)), __fma_rn(beta, it.p.y, widen(it.z.y)));
            });
    } else {
        stream_pipelined<kPU, PItem>(
            br.begin, br.end, NT, [&](unsigned k) { return PItem{load_pair(z, k), p[k]}; },
            [&](unsigned k, const PItem& it) {
                p[k] = make_double2(__fma_rn(beta, it.p.x, it.z.x), __fma_rn(beta, it.p.y, it.z.y));
            });
    }
}

// ---- self-test of the integer conversions -----------------------------------

__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
    x += 0x9e3779b97f4a7c15ull;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}

// Item q tests widen() on a float bit pattern and narrow() on a double bit
// pattern against the hardware conversions; the first 2^18 items sweep every
// float exponent and every double exponent near the float range (with
// mantissas at, just below and just above the rounding tie), the rest are
// hashed. NaN results compare by NaN-ness.
__global__ void k_conv_selftest(unsigned long long n, unsigned long long seed,
                                unsigned long long* mismatches) {
    unsigned long long bad = 0;
    for (unsigned long long q = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; q < n;
         q += (unsigned long long)gridDim.x * blockDim.x) {
        const unsigned long long h = mix64(q ^ seed);
        unsigned fb;
        unsigned long long db;
        if (q < (1ull << 18)) {
            const unsigned sel = (unsigned)(q & 15u), ex = (unsigned)(q >> 4) & 0x7ffu;
            fb = ((unsigned)(h >> 32) & 0x807fffffu) | ((ex & 0xffu) << 23);
            const unsigned long long tie = 1ull << 28, low = (h & 0xffffffe0000000ull);
            const unsigned long long tail = sel < 4 ? tie : sel < 8 ? tie - 1 : sel < 12 ? tie + 1 : (h & 0x1fffffffull);
            db = (h & 0x8000000000000000ull) | ((unsigned long long)ex << 52) | (low & 0xfffffe0000000ull) | tail;
        } else {
            fb = (unsigned)h;
            db = mix64(h);
        }
        const float f = __uint_as_float(fb);
        const double wd = widen(f), hd = (double)f;
        const bool wok = (isnan(hd) && isnan(wd)) || __double_as_longlong(wd) == __double_as_longlong(hd);
        const double d = __longlong_as_double((long long)db);
        const float nf = narrow(d), hf = (float)d;
        const bool nok = (isnan(hf) && isnan(nf)) || __float_as_uint(nf) == __float_as_uint(hf);
        bad += (wok ? 0u : 1u) + (nok ? 0u : 1u);
    }
    if (bad) atomicAdd(mismatches, bad);
}

// FP64-pipe peak probe: kDfmaChains independent DFMA chains per thread, kDfmaSteps
// steps each (no memory traffic but one store per thread).
constexpr int kDfmaChains = 8, kDfmaSteps = 2048;
__global__ void k_dfma_probe(double a, double* out) {
    double v[kDfmaChains];
#pragma unroll
    for (int c = 0; c < kDfmaChains; ++c) v[c] = threadIdx.x * 1e-3 + c;
    for (int k = 0; k < kDfmaSteps; ++k)
#pragma unroll
        for (int c = 0; c < kDfmaChains; ++c) v[c] = __fma_rn(v[c], a, 1e-9);
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < kDfmaChains; ++c) s += v[c];
    out[blockIdx.x * (size_t)blockDim.x + threadIdx.x] = s;
}

}  // namespace

// ---- launchers ------------------------------------------------------------------

void launch_apply64(cudaStream_t st, const OpView& o, const double* diag, const double* p,
                    double* Ap, Ctl* ctl, const Red& red, Cond cond) {
    static const int wb = wave_blocks(k_apply64, 1 << 30);
    launch_pdl(k_apply64, std::min(red.maxb, wb), NT, 0, st, o, diag, p, Ap, ctl, red.part, red.maxb, cond);
}

void launch_residual64(cudaStream_t st, MgType mt, const OpView& o, unsigned n, const double* diag,
                       const double* b, const double* x, double* r, void* b0, Ctl* ctl, const Red& red,
                       Cond cond) {
    if (mt == MG_F64) {
        static const int wb = wave_blocks(k_residual64<double>, 1 << 30);
        launch_pdl(k_residual64<double>, std::min(red.maxb, wb), NT, 0, st, o, n, diag, b, x, r, (double*)b0,
                   ctl, red.part, red.maxb, cond);
    } else {
        static const int wb = wave_blocks(k_residual64<float>, 1 << 30);
        launch_pdl(k_residual64<float>, std::min(red.maxb, wb), NT, 0, st, o, n, diag, b, x, r, (float*)b0,
                   ctl, red.part, red.maxb, cond);
    }
}

void launch_update64(cudaStream_t st, MgType mt, unsigned n, const double* p, const double* Ap, double* x,
                     double* r, void* b0, Ctl* ctl, const Red& red, Cond cond, bool write_x) {
    const unsigned n2 = n / 2;
    const auto* p2 = reinterpret_cast<const double2*>(p);
    const auto* a2 = reinterpret_cast<const double2*>(Ap);
    auto* x2 = reinterpret_cast<double2*>(x);
    auto* r2 = reinterpret_cast<double2*>(r);
    // (wave_blocks once per kernel: the four have their own occupancies)
    auto go = [&](auto kern, int wb, auto* b) {
        launch_pdl(kern, std::min(red.blocks, wb), NT, 0, st, n2, p2, a2, x2, r2, b, ctl, red.part, red.maxb,
                   cond);
    };
    if (mt == MG_F64) {
        static const int wb1 = wave_blocks(k_update64<double, true>, 1 << 30);
        static const int wb0 = wave_blocks(k_update64<double, false>, 1 << 30);
        if (write_x) go(k_update64<double, true>, wb1, (double*)b0);
        else go(k_update64<double, false>, wb0, (double*)b0);
    } else {
        static const int wb1 = wave_blocks(k_update64<float, true>, 1 << 30);
        static const int wb0 = wave_blocks(k_update64<float, false>, 1 << 30);
        if (write_x) go(k_update64<float, true>, wb1, (float*)b0);
        else go(k_update64<float, false>, wb0, (float*)b0);
    }
}

void launch_update_x(cudaStream_t st, unsigned n, const double* p, double* x, const Ctl* ctl, int blocks) {
    static const int wb = wave_blocks(k_update_x64, 1 << 30);
    const unsigned n2 = n / 2;
    unsigned want = std::max(1u, (n2 + NT * 4 - 1) / (NT * 4));
    if (blocks > 0) want = std::min(want, (unsigned)blocks);
    k_update_x64<<<(int)std::min(want, (unsigned)wb), NT, 0, st>>>(n2, reinterpret_cast<const double2*>(p),
                                                                    reinterpret_cast<double2*>(x), ctl);
}

void launch_dot64(cudaStream_t st, MgType mt, bool flexible, unsigned n, const double* r, const void* z,
                  const double* Ap, Ctl* ctl, const Red& red, Cond cond) {
    const unsigned n2 = n / 2;
    const auto* r2 = reinterpret_cast<const double2*>(r);
    const auto* a2 = reinterpret_cast<const double2*>(Ap);
    const int nb = std::min(red.maxb, std::max(1, red.maxb / 2));
    if (mt == MG_F64) {
        if (flexible)
            launch_pdl(k_dot64<double, true>, nb, NT, 0, st, n2, r2, (const double*)z, a2, ctl, red.part,
                       red.maxb, cond);
        else
            launch_pdl(k_dot64<double, false>, nb, NT, 0, st, n2, r2, (const double*)z, a2, ctl, red.part,
                       red.maxb, cond);
    } else {
        // the flexible FP32-V-cycle dot keeps four pairs in flight a thread
        // on one wave of blocks (100 registers): 36.7 us against 38.7 us
        // with two on 608 blocks and 37.0 us with three, at 800 x 800
        static const int wb4 = wave_blocks(k_dot64<float, true, 4>, 1 << 30);
        if (flexible)
            launch_pdl(k_dot64<float, true, 4>, std::min(nb, wb4), NT, 0, st, n2, r2, (const float*)z, a2, ctl,
                       red.part, red.maxb, cond);
        else
            launch_pdl(k_dot64<float, false>, nb, NT, 0, st, n2, r2, (const float*)z, a2, ctl, red.part,
                       red.maxb, cond);
    }
}

void launch_update_p64(cudaStream_t st, MgType mt, unsigned n, const void* z, double* p, Ctl* ctl,
                       Cond cond) {
    const unsigned n2 = n / 2;
    auto* p2 = reinterpret_cast<double2*>(p);
    const unsigned want = std::max(1u, (n2 + NT * 2 * kPU - 1) / (NT * 2 * kPU));
    if (mt == MG_F64) {
        static const int wb = wave_blocks(k_update_p64<double>, 1 << 30);
        launch_pdl(k_update_p64<double>, (int)std::min(want, (unsigned)wb), NT, 0, st, n2, (const double*)z, p2,
                   ctl, cond);
    } else {
        static const int wb = wave_blocks(k_update_p64<float>, 1 << 30);
        launch_pdl(k_update_p64<float>, (int)std::min(want, (unsigned)wb), NT, 0, st, n2, (const float*)z, p2,
                   ctl, cond);
    }
}

cudaError_t measure_dfma_rate(double* per_s) {
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    const int blocks = std::max(1, sms) * 8;
    double* out = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    e = cudaMalloc(&out, (size_t)blocks * NT * sizeof(double));
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    float ms = 0.0f;
    constexpr int kReps = 5;
    if (e == cudaSuccess) {
        for (int w = 0; w < 2; ++w) k_dfma_probe<<<blocks, NT>>>(0.999999, out);
        cudaEventRecord(e0);
        for (int r = 0; r < kReps; ++r) k_dfma_probe<<<blocks, NT>>>(0.999999, out);
        cudaEventRecord(e1);
        e = cudaEventSynchronize(e1);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (out) cudaFree(out);
    if (e == cudaSuccess)
        *per_s = (double)blocks * NT * kDfmaChains * kDfmaSteps * kReps / (ms * 1e-3);
    return e;
}

cudaError_t launch_conv_selftest(cudaStream_t st, unsigned long long n, unsigned long long seed,
                                 unsigned long long* mismatches) {
    k_conv_selftest<<<1024, NT, 0, st>>>(n, seed, mismatches);
    return cudaGetLastError();
}

}  // namespace ct
