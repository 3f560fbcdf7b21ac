// dw_dev.cuh - double-word (float-pair) arithmetic and the split-layout
// column map, shared by the single solver (k_dw.cu) and the batched solver
// (k_batch.cu). Error-free transformations after Joldes, Muller and Popescu,
// "Tight and rigorous error bounds for basic building blocks of double-word
// arithmetic" (2017).
#pragma once
#include "kernels.h"

namespace ct {
namespace dwdev {

// ---- double-word arithmetic ------------------------------------------------
// A value is float2 v = (hi, lo) with v = hi + lo and |lo| <= ulp(hi) / 2.

__device__ __forceinline__ float2 two_sum(float a, float b) {
    const float s = a + b;
    const float bp = s - a;
    const float ap = s - bp;
    return make_float2(s, (a - ap) + (b - bp));
}

// |a| >= |b| (or a = 0).
__device__ __forceinline__ float2 fast_two_sum(float a, float b) {
    const float s = a + b;
    return make_float2(s, b - (s - a));
}

__device__ __forceinline__ float2 dw_add(float2 a, float2 b) {
    const float2 s = two_sum(a.x, b.x);
    return fast_two_sum(s.x, s.y + (a.y + b.y));
}

__device__ __forceinline__ float2 dw_neg(float2 a) { return make_float2(-a.x, -a.y); }

__device__ __forceinline__ float2 dw_mul(float2 a, float2 b) {
    const float p = a.x * b.x;
    float e = fmaf(a.x, b.x, -p);
    e = fmaf(a.x, b.y, e);
    e = fmaf(a.y, b.x, e);
    return fast_two_sum(p, e);
}

__device__ __forceinline__ float2 dw_of(double d) {
    const float h = __double2float_rn(d);
    return make_float2(h, __double2float_rn(d - (double)h));
}

__device__ __forceinline__ double dw_d(float2 a) { return (double)a.x + (double)a.y; }

// ---- sums of float x double-word products ------------------------------------
// (s, c): s collects the products' high parts through TwoSum, c the exact
// rounding errors of the products and the sums plus the products of the low
// parts; renormalised once at the end (fast_two_sum(s, c)). Each term costs
// eleven FP32 operations instead of the seventeen of a double-word product
// and a double-word sum, with
// an error of the same order (a few units of 2^-48 of the largest term).
struct DwAcc {
    float s, c;
};

// a += h + lo with |lo| << |h|.
__device__ __forceinline__ void acc_add(DwAcc& a, float h, float lo) {
    const float s = a.s + h;
    const float bp = s - a.s;
    const float err = (a.s - (s - bp)) + (h - bp);
    a.s = s;
    a.c += err + lo;
}

// a += g * p.
__device__ __forceinline__ void acc_mul_f(DwAcc& a, float2 p, float g) {
    const float h = g * p.x;
    acc_add(a, h, fmaf(g, p.y, fmaf(g, p.x, -h)));
}

// a += u * v (both double words; the lo * lo term is below the error).
__device__ __forceinline__ void acc_mul(DwAcc& a, float2 u, float2 v) {
    const float h = u.x * v.x;
    acc_add(a, h, fmaf(u.x, v.y, fmaf(u.y, v.x, fmaf(u.x, v.x, -h))));
}

// ---- block and grid sums of accumulators ----------------------------------------
// The fixed trees of block_sum2 / gather2 (reduce.cuh) on the FP32 pipe: each
// step adds another thread's (s, c) with acc_add (TwoSum on s, c collecting
// the errors), and only thread 0 converts the block's or the grid's total to
// FP64. Summing every thread's value in FP64 instead cost each block about a
// microsecond of FP64 adds and conversions at its end, with the memory
// system idle.
__device__ __forceinline__ void warp_sum_acc(DwAcc& a) {
    for (int o = 16; o > 0; o >>= 1) {
        const float s = __shfl_down_sync(0xffffffffu, a.s, o);
        const float c = __shfl_down_sync(0xffffffffu, a.c, o);
        acc_add(a, s, c);
    }
}

// Block sum of (a, b) over NTH threads (at most 32 warps); valid in thread 0.
template <int NTH = NT>
__device__ __forceinline__ void block_sum_acc2(DwAcc& a, DwAcc& b) {
    constexpr int NW = NTH / 32;
    static_assert(NTH % 32 == 0 && NW <= 32, "whole warps, at most 32");
    __shared__ float2 sa[NW], sb[NW];
    warp_sum_acc(a);
    warp_sum_acc(b);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        sa[w] = make_float2(a.s, a.c);
        sb[w] = make_float2(b.s, b.c);
    }
    __syncthreads();
    if (w == 0) {
        const float2 u = lane < NW ? sa[lane] : make_float2(0.0f, 0.0f);
        const float2 v = lane < NW ? sb[lane] : make_float2(0.0f, 0.0f);
        a = DwAcc{u.x, u.y};
        b = DwAcc{v.x, v.y};
        warp_sum_acc(a);
        warp_sum_acc(b);
    }
}

__device__ __forceinline__ double acc_value(const DwAcc& a) { return (double)a.s + (double)a.c; }

// Publishes the block's (a, b) (valid in thread 0) as float pairs in slots
// blockIdx.x and maxb + blockIdx.x of part, takes a ticket, and returns in
// every thread whether this block arrived last of `count`.
__device__ __forceinline__ bool publish_acc2(const DwAcc& a, const DwAcc& b, double* part, int maxb,
                                             unsigned slot, unsigned* ticket, unsigned count) {
    __shared__ int last;
    if (threadIdx.x == 0) {
        float2* pp = reinterpret_cast<float2*>(part);
        pp[slot] = make_float2(a.s, a.c);
        pp[maxb + slot] = make_float2(b.s, b.c);
        __threadfence();
        const unsigned t = atomicAdd(ticket, 1u);
        last = (t == count - 1u) ? 1 : 0;
    }
    __syncthreads();
    return last != 0;
}

// In the last block: the totals of slots [first, first + count), in slot
// order through the same tree, as FP64 in thread 0. Resets the ticket.
template <int NTH = NT>
__device__ __forceinline__ void gather_acc2(const double* part, int maxb, unsigned first, unsigned count,
                                            unsigned* ticket, double& A, double& B) {
    __threadfence();
    const float2* pp = reinterpret_cast<const float2*>(part);
    DwAcc a = {0.0f, 0.0f}, b = {0.0f, 0.0f};
    for (unsigned k = threadIdx.x; k < count; k += NTH) {
        const float2 u = __ldcg(pp + first + k), v = __ldcg(pp + maxb + first + k);
        acc_add(a, u.x, u.y);
        acc_add(b, v.x, v.y);
    }
    block_sum_acc2<NTH>(a, b);
    if (threadIdx.x == 0) {
        A = acc_value(a);
        B = acc_value(b);
        *ticket = 0u;
    }
}

// ---- streaming ranges of value pairs ------------------------------------------
// Items k = k0, k0 + stride, ... < end; each item is a pair of values (float4
// = two double words). kU items are loaded before any is used, so a thread
// keeps kU times the bytes of one item in flight. The single solver's kernels
// (grid-stride) and the batched kernels (one block per task) share these.
constexpr int kU = 4;

// rz += r.z, zap += Ap.z.
__device__ __forceinline__ void dot_range(unsigned k, unsigned end, unsigned stride,
                                          const float4* __restrict__ r, const float2* __restrict__ z,
                                          const float4* __restrict__ Ap, DwAcc& rz, DwAcc& zap) {
    for (; k + (kU - 1) * stride < end; k += kU * stride) {
        float4 rv[kU], av[kU];
        float2 zv[kU];
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            rv[u] = r[k + u * stride];
            av[u] = Ap[k + u * stride];
            zv[u] = z[k + u * stride];
        }
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            acc_mul_f(rz, make_float2(rv[u].x, rv[u].y), zv[u].x);
            acc_mul_f(rz, make_float2(rv[u].z, rv[u].w), zv[u].y);
            acc_mul_f(zap, make_float2(av[u].x, av[u].y), zv[u].x);
            acc_mul_f(zap, make_float2(av[u].z, av[u].w), zv[u].y);
        }
    }
    for (; k < end; k += stride) {
        const float4 rv = r[k], av = Ap[k];
        const float2 zv = z[k];
        acc_mul_f(rz, make_float2(rv.x, rv.y), zv.x);
        acc_mul_f(rz, make_float2(rv.z, rv.w), zv.y);
        acc_mul_f(zap, make_float2(av.x, av.y), zv.x);
        acc_mul_f(zap, make_float2(av.z, av.w), zv.y);
    }
}

// x += a p, r -= a Ap, b0 = r (hi words), rr += r.r.
__device__ __forceinline__ void update_one(float2 a, const float4& pv, const float4& av, float4* x,
                                           float4* r, float2* b0, unsigned k, const float4& xv,
                                           const float4& rv, DwAcc& rr) {
    const float2 x0 = dw_add(make_float2(xv.x, xv.y), dw_mul(a, make_float2(pv.x, pv.y)));
    const float2 x1 = dw_add(make_float2(xv.z, xv.w), dw_mul(a, make_float2(pv.z, pv.w)));
    const float2 r0 = dw_add(make_float2(rv.x, rv.y), dw_neg(dw_mul(a, make_float2(av.x, av.y))));
    const float2 r1 = dw_add(make_float2(rv.z, rv.w), dw_neg(dw_mul(a, make_float2(av.z, av.w))));
    x[k] = make_float4(x0.x, x0.y, x1.x, x1.y);
    r[k] = make_float4(r0.x, r0.y, r1.x, r1.y);
    b0[k] = make_float2(r0.x, r1.x);
    acc_mul(rr, r0, r0);
    acc_mul(rr, r1, r1);
}

__device__ __forceinline__ void update_range(unsigned k, unsigned end, unsigned stride, float2 a,
                                             const float4* __restrict__ p,
                                             const float4* __restrict__ Ap, float4* __restrict__ x,
                                             float4* __restrict__ r, float2* __restrict__ b0,
                                             DwAcc& rr) {
    constexpr int U = kU / 2;  // four arrays per item: half the items of dot_range
    for (; k + (U - 1) * stride < end; k += U * stride) {
        float4 pv[U], av[U], xv[U], rv[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            pv[u] = p[k + u * stride];
            av[u] = Ap[k + u * stride];
            xv[u] = x[k + u * stride];
            rv[u] = r[k + u * stride];
        }
#pragma unroll
        for (int u = 0; u < U; ++u) update_one(a, pv[u], av[u], x, r, b0, k + u * stride, xv[u], rv[u], rr);
    }
    for (; k < end; k += stride) update_one(a, p[k], Ap[k], x, r, b0, k, x[k], r[k], rr);
}

// p = z + beta p (p = z when first).
__device__ __forceinline__ void update_p_range(unsigned k, unsigned end, unsigned stride,
                                               float2 beta, bool first,
                                               const float2* __restrict__ z,
                                               float4* __restrict__ p) {
    if (first) {
        for (; k < end; k += stride) {
            const float2 zv = z[k];
            p[k] = make_float4(zv.x, 0.0f, zv.y, 0.0f);
        }
        return;
    }
    auto one = [&](unsigned q, const float2& zv, const float4& pv) {
        const float2 p0 = dw_add(dw_mul(beta, make_float2(pv.x, pv.y)), make_float2(zv.x, 0.0f));
        const float2 p1 = dw_add(dw_mul(beta, make_float2(pv.z, pv.w)), make_float2(zv.y, 0.0f));
        p[q] = make_float4(p0.x, p0.y, p1.x, p1.y);
    };
    for (; k + (kU - 1) * stride < end; k += kU * stride) {
        float2 zv[kU];
        float4 pv[kU];
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            zv[u] = z[k + u * stride];
            pv[u] = p[k + u * stride];
        }
#pragma unroll
        for (int u = 0; u < kU; ++u) one(k + u * stride, zv[u], pv[u]);
    }
    for (; k < end; k += stride) one(k, z[k], p[k]);
}

// Operands of one cell of the operator apply, loaded before any is used
// (absent neighbours stay zero and are skipped by the same guards).
struct ApplyCell {
    float2 pc, dg, pw, pe, ps, pn, pd, pu;
    float gw, ge, gs, gn, gd, gu;
};

__device__ __forceinline__ void apply_load(const OpView& o, const float2* __restrict__ dgw,
                                           const float2* __restrict__ p, unsigned k, unsigned t,
                                           unsigned orow, int i, int e, bool hs, bool hn, bool hd,
                                           bool hu, ApplyCell& a) {
    const Geo& g = o.g;
    const unsigned hx = (unsigned)g.hx;
    const float2 z = make_float2(0.0f, 0.0f);
    a.pc = p[k];
    a.dg = dgw[k];
    a.pw = z, a.pe = z, a.ps = z, a.pn = z, a.pd = z, a.pu = z;
    a.gw = 0.0f, a.ge = 0.0f, a.gs = 0.0f, a.gn = 0.0f, a.gd = 0.0f, a.gu = 0.0f;
    if (i > 0) {
        const unsigned w = orow + t - 1u + (unsigned)e;
        a.pw = p[w];
        a.gw = o.gE[w];
    }
    if (i < g.nx - 1) {
        a.pe = p[orow + t + (unsigned)e];
        a.ge = o.gE[k];
    }
    if (hs) {
        const unsigned sl = orow - 2u * hx + t;
        a.ps = p[sl];
        a.gs = o.gN[sl];
    }
    if (hn) {
        a.pn = p[orow + 2u * hx + t];
        a.gn = o.gN[k];
    }
    if (hd) {
        a.pd = p[k - g.plane];
        a.gd = o.gU[k - g.plane];
    }
    if (hu) {
        a.pu = p[k + g.plane];
        a.gu = o.gU[k];
    }
}

// Ap of the cell from its operands: the stored diagonal times p minus the
// west, east, south, north, down and up neighbour terms (op_apply's order,
// src/operator3d.h:108-112); p.Ap added to pap.
__device__ __forceinline__ float2 apply_compute(const ApplyCell& a, bool w, bool e, bool s, bool n,
                                                bool d, bool u, DwAcc& pap) {
    DwAcc off = {0.0f, 0.0f};
    if (w) acc_mul_f(off, a.pw, a.gw);
    if (e) acc_mul_f(off, a.pe, a.ge);
    if (s) acc_mul_f(off, a.ps, a.gs);
    if (n) acc_mul_f(off, a.pn, a.gn);
    if (d) acc_mul_f(off, a.pd, a.gd);
    if (u) acc_mul_f(off, a.pu, a.gu);
    const float h = a.dg.x * a.pc.x;
    DwAcc r = {h, fmaf(a.dg.x, a.pc.y, fmaf(a.dg.y, a.pc.x, fmaf(a.dg.x, a.pc.x, -h)))};
    acc_add(r, -off.s, -off.c);
    const float2 av = fast_two_sum(r.s, r.c);
    acc_mul(pap, a.pc, av);
    return av;
}

// Ap = (A + C/dt) p on one row of one plane (hx slots of one colour of row j).
// The calling warp strides over the row, U cells per lane and step (32 slots
// apart) with every operand of all U loaded first; p.Ap of its cells is added
// to pap in slot order. R = l * 2 ny + 2 j + colour.
template <int U>
__device__ __forceinline__ void apply_row(const OpView& o, const float2* __restrict__ dgw,
                                          const float2* __restrict__ p, float2* __restrict__ Ap,
                                          unsigned R, int lane, DwAcc& pap) {
    const Geo& g = o.g;
    const unsigned rows = 2u * (unsigned)g.ny;
    const unsigned l = R / rows;
    const unsigned r = R - l * rows;
    const int j = (int)(r >> 1), c = (int)(r & 1u), e = (j + c) & 1;
    const unsigned hx = (unsigned)g.hx;
    const unsigned base = l * g.plane;
    const unsigned row = base + r * hx;
    const unsigned orow = base + (unsigned)(2 * j + (c ^ 1)) * hx;  // other colour, same j
    const bool hs = j > 0, hn = j < g.ny - 1, hd = l > 0, hu = (int)l < g.nz - 1;
    for (unsigned t0 = (unsigned)lane; t0 < hx; t0 += 32u * U) {
        ApplyCell a[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const unsigned t = t0 + 32u * u;
            const int i = 2 * (int)t + e;
            if (t < hx && i < g.nx) apply_load(o, dgw, p, row + t, t, orow, i, e, hs, hn, hd, hu, a[u]);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const unsigned t = t0 + 32u * u;
            const int i = 2 * (int)t + e;
            if (t < hx)
                Ap[row + t] = i < g.nx ? apply_compute(a[u], i > 0, i < g.nx - 1, hs, hn, hd, hu, pap)
                                       : make_float2(0.0f, 0.0f);
        }
    }
}

// ---- column walk (split layout), as in k_outer.cu ----------------------------
struct Col {
    int i, j;
    unsigned s, sw, se, ss, sn;
    bool valid;
};

__device__ __forceinline__ Col col_of_slot(const Geo& g, unsigned s) {
    Col c;
    const unsigned row2 = 2u * (unsigned)g.hx;
    const int j = (int)(s / row2);
    const unsigned rem = s - (unsigned)j * row2;
    const int colour = rem >= (unsigned)g.hx ? 1 : 0;
    const int t = (int)rem - colour * g.hx;
    const int i = 2 * t + ((j + colour) & 1);
    const int oc = colour ^ 1;
    const unsigned row_o = (unsigned)(2 * j + oc) * (unsigned)g.hx;
    c.i = i;
    c.j = j;
    c.s = s;
    c.sw = row_o + (unsigned)((i - 1) >> 1);
    c.se = row_o + (unsigned)((i + 1) >> 1);
    c.ss = (unsigned)(2 * j - 2 + oc) * (unsigned)g.hx + (unsigned)t;
    c.sn = (unsigned)(2 * j + 2 + oc) * (unsigned)g.hx + (unsigned)t;
    c.valid = i < g.nx;
    return c;
}


}  // namespace dwdev
}  // namespace ct
