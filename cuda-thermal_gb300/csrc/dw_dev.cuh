// dw_dev.cuh - double-word (float-pair) arithmetic and the split-layout
// column map, shared by the single solver (k_dw.cu) and the batched solver
// (k_batch.cu). Error-free transformations after Joldes, Muller and Popescu,
// "Tight and rigorous error bounds for basic building blocks of double-word
// arithmetic" (2017).
#pragma once
#include "device.h"

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

__device__ __forceinline__ float2 dw_mul_f(float2 a, float b) {
    const float p = a.x * b;
    float e = fmaf(a.x, b, -p);
    e = fmaf(a.y, b, e);
    return fast_two_sum(p, e);
}

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
