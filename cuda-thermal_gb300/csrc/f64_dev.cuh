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

}  // namespace f64dev
}  // namespace ct
