// f64_dev.cuh - float <-> double conversions without the FP64 pipe.
//
// On GB300 the hardware conversions F2F.F64.F32 and F2F.F32.F64 issue at the
// FP64 rate (measured with independent chains on 152 SMs: 0.63 T conversions
// per second, against 0.53 T DFMA/s and 38.6 T FFMA/s). The FP64 outer kernels
// convert every float face conductance and every float V-cycle value they
// touch, so those conversions cost as much as their FP64 arithmetic. These
// helpers rebuild the IEEE-754 results with integer operations (which issue on
// the FP32/INT32 pipes) and bit for bit equal the hardware conversion:
//  - widen: a float is exactly representable as a double; for normal floats
//    the exponent is rebiased (+896 = 1023 - 127) and the 23-bit mantissa
//    shifted into the top of the 52-bit one; zeros keep their sign;
//  - narrow: round to nearest, ties to even, of the 52-bit mantissa to 23
//    bits when the result is a normal float (a carry out of the mantissa
//    correctly bumps the exponent, up to infinity); zeros keep their sign.
// Every other input (subnormal, infinite or NaN floats; doubles whose float
// is subnormal or zero-by-underflow, or out of range) takes the hardware
// conversion, so the helpers are exact for every input.
// ct_selftest_conversions checks both against the hardware on the GPU.
#pragma once
#include <cuda_runtime.h>

#include "kernels.h"

namespace ct {
namespace f64dev {

__device__ __forceinline__ double widen(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xffu;
    if (e - 1u < 254u) {  // normal
        const unsigned hi = (u & 0x80000000u) | (((u & 0x7fffffffu) >> 3) + (896u << 20));
        return __hiloint2double((int)hi, (int)(u << 29));
    }
    if ((u & 0x7fffffffu) == 0u) return __hiloint2double((int)(u & 0x80000000u), 0);
    return (double)f;
}

__device__ __forceinline__ float narrow(double d) {
    const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
    const unsigned E = (hi >> 20) & 0x7ffu;
    if (E - 897u < 254u) {  // the float is normal: 1 <= E - 896 <= 254
        const unsigned m = ((hi & 0xfffffu) << 3) | (lo >> 29);
        const unsigned rest = lo & 0x1fffffffu;
        unsigned f = (hi & 0x80000000u) | ((E - 896u) << 23) | m;
        f += (rest > 0x10000000u || (rest == 0x10000000u && (m & 1u))) ? 1u : 0u;
        return __uint_as_float(f);
    }
    if (((hi & 0x7fffffffu) | lo) == 0u) return __uint_as_float(hi & 0x80000000u);
    return (float)d;
}

// The V-cycle's values as doubles: T = float (widened) or double (as is).
__device__ __forceinline__ double to_d(float v) { return widen(v); }
__device__ __forceinline__ double to_d(double v) { return v; }
// A double stored in the V-cycle's precision.
template <class T>
__device__ __forceinline__ T from_d(double v);
template <>
__device__ __forceinline__ float from_d<float>(double v) {
    return narrow(v);
}
template <>
__device__ __forceinline__ double from_d<double>(double v) {
    return v;
}

// Streams the items k = first, first + stride, ... below end, U per step,
// with the next step's loads issued before the current step's arithmetic (two
// register sets): the FP64 pipe, at ~1/70 of the FP32 rate, would otherwise
// hold each warp between its loads, and the memory traffic and the FP64
// instructions of these kernels would not overlap (measured: the dot took the
// sum of its DRAM time and its DFMA time, 42 us at 800 x 800 x 10).
// Single solver (k_fp64.cu) and batch (k_batch64.cu).
template <int U, class Item, class Load, class Use>
__device__ __forceinline__ void stream_pipelined(unsigned first, unsigned end, unsigned stride, Load load,
                                                 Use use) {
    Item a[U], b[U];
    bool va[U], vb[U];
    auto fetch = [&](unsigned k0, Item* it, bool* v) {
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const unsigned k = k0 + (unsigned)u * stride;
            v[u] = k < end;
            if (v[u]) it[u] = load(k);
        }
    };
    unsigned k0 = first;
    fetch(k0, a, va);
    while (k0 < end) {
        const unsigned k1 = k0 + (unsigned)U * stride;
        fetch(k1, b, vb);
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (va[u]) use(k0 + (unsigned)u * stride, a[u]);
#pragma unroll
        for (int u = 0; u < U; ++u) {
            a[u] = b[u];
            va[u] = vb[u];
        }
        k0 = k1;
    }
}

// ---- the FP64 operator apply, one warp per row (single solver and batch) ----

// Operands of one cell, loaded before any is used (absent neighbours stay
// zero and are skipped by the same guards).
struct Cell64 {
    double pc, dg, pw, pe, ps, pn, pd, pu;
    float gw, ge, gs, gn, gd, gu;
};

__device__ __forceinline__ void load64(const OpView& o, const double* __restrict__ diag,
                                       const double* __restrict__ v, unsigned k, unsigned t,
                                       unsigned orow, int i, int e, bool hs, bool hn, bool hd, bool hu,
                                       Cell64& a) {
    const Geo& g = o.g;
    const unsigned hx = (unsigned)g.hx;
    a.pc = v[k];
    a.dg = diag[k];
    a.pw = a.pe = a.ps = a.pn = a.pd = a.pu = 0.0;
    a.gw = a.ge = a.gs = a.gn = a.gd = a.gu = 0.0f;
    if (i > 0) {
        const unsigned w = orow + t - 1u + (unsigned)e;
        a.pw = v[w];
        a.gw = o.gE[w];
    }
    if (i < g.nx - 1) {
        a.pe = v[orow + t + (unsigned)e];
        a.ge = o.gE[k];
    }
    if (hs) {
        const unsigned sl = orow - 2u * hx + t;
        a.ps = v[sl];
        a.gs = o.gN[sl];
    }
    if (hn) {
        a.pn = v[orow + 2u * hx + t];
        a.gn = o.gN[k];
    }
    if (hd) {
        a.pd = v[k - g.plane];
        a.gd = o.gU[k - g.plane];
    }
    if (hu) {
        a.pu = v[k + g.plane];
        a.gu = o.gU[k];
    }
}

// (A + C/dt) v at the cell: the stored diagonal times v minus the west, east,
// south, north, down and up terms, in op_apply's order (src/operator3d.h:
// 100-112), each a DFMA: 7 FP64 instructions.
__device__ __forceinline__ double compute64(const Cell64& a, bool w, bool e, bool s, bool n, bool d,
                                            bool u) {
    double off = 0.0;
    if (w) off = __fma_rn(widen(a.gw), a.pw, off);
    if (e) off = __fma_rn(widen(a.ge), a.pe, off);
    if (s) off = __fma_rn(widen(a.gs), a.ps, off);
    if (n) off = __fma_rn(widen(a.gn), a.pn, off);
    if (d) off = __fma_rn(widen(a.gd), a.pd, off);
    if (u) off = __fma_rn(widen(a.gu), a.pu, off);
    return __fma_rn(a.dg, a.pc, -off);
}

// Row R = l * 2 ny + 2 j + colour: the calling warp strides over the row's hx
// slots, U cells per lane and step (32 slots apart) with every operand of all
// U loaded first, and hands f(slot, valid, (A + C/dt) v, v) for each slot in
// order (padding slots: valid = false, zeros).
template <int U, class F>
__device__ __forceinline__ void row64(const OpView& o, const double* __restrict__ diag,
                                      const double* __restrict__ v, unsigned R, int lane, F&& f) {
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
        Cell64 a[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const unsigned t = t0 + 32u * u;
            const int i = 2 * (int)t + e;
            if (t < hx && i < g.nx) load64(o, diag, v, row + t, t, orow, i, e, hs, hn, hd, hu, a[u]);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const unsigned t = t0 + 32u * u;
            const int i = 2 * (int)t + e;
            if (t < hx) {
                if (i < g.nx)
                    f(row + t, true, compute64(a[u], i > 0, i < g.nx - 1, hs, hn, hd, hu), a[u].pc);
                else
                    f(row + t, false, 0.0, 0.0);
            }
        }
    }
}

}  // namespace f64dev
}  // namespace ct
