// setup_dev.cuh - the per-column set-up arithmetic that depends on dt: the
// FP64 diagonal of the fine operator (op_diag, src/operator3d.h:80-88) and the
// Thomas factors of a multigrid level (mg_factor_column, src/mg3d.h:46-61),
// every rounding explicit (no contraction) so both equal the CPU's bit for
// bit. Shared by the single solver (k_outer.cu, k_mg.cu) and the batched
// set_dt (k_batch.cu).
#pragma once
#include "kernels.h"

namespace ct {
namespace setupdev {

template <class T>
struct RN;
template <>
struct RN<float> {
    static __device__ float add(float a, float b) { return __fadd_rn(a, b); }
    static __device__ float sub(float a, float b) { return __fsub_rn(a, b); }
    static __device__ float mul(float a, float b) { return __fmul_rn(a, b); }
    static __device__ float div(float a, float b) { return __fdiv_rn(a, b); }
};
template <>
struct RN<double> {
    static __device__ double add(double a, double b) { return __dadd_rn(a, b); }
    static __device__ double sub(double a, double b) { return __dsub_rn(a, b); }
    static __device__ double mul(double a, double b) { return __dmul_rn(a, b); }
    static __device__ double div(double a, double b) { return __ddiv_rn(a, b); }
};

// op_diag of cell (i, j, l) of a level, in T.
template <class T>
__device__ __forceinline__ T diag_rn(const LevelView<T>& L, int i, int j, int l, T inv_dt) {
    const Geo& g = L.g;
    const unsigned base = (unsigned)l * g.plane;
    const unsigned s = scol(g, i, j), id = base + s;
    T d = 0;
    if (i > 0) d = RN<T>::add(d, (T)L.gE[base + scol(g, i - 1, j)]);
    if (i < g.nx - 1) d = RN<T>::add(d, (T)L.gE[id]);
    if (j > 0) d = RN<T>::add(d, (T)L.gN[base + scol(g, i, j - 1)]);
    if (j < g.ny - 1) d = RN<T>::add(d, (T)L.gN[id]);
    d = RN<T>::add(d, (T)L.gU[id]);
    d = RN<T>::add(d, l > 0 ? (T)L.gU[id - g.plane] : (T)L.gB[s]);
    return RN<T>::add(d, RN<T>::mul((T)L.cap[id], inv_dt));
}

// Thomas factors of natural column q = j nx + i of a level. The factors are
// written through restrict pointers, so the operand loads of the next planes
// may be issued before this plane's stores.
template <class T>
__device__ __forceinline__ void factor_column(const LevelView<T>& L, T inv_dt, unsigned q) {
    const Geo& g = L.g;
    const int j = (int)(q / (unsigned)g.nx), i = (int)(q - (unsigned)j * g.nx);
    const unsigned s = scol(g, i, j);
    T* __restrict__ finv = L.finv;
    T* __restrict__ fcp = L.fcp;
    const float* __restrict__ gU = L.gU;
    T cp_prev = 0;
#pragma unroll 4
    for (int l = 0; l < g.nz; ++l) {
        const unsigned id = (unsigned)l * g.plane + s;
        const T d = diag_rn(L, i, j, l, inv_dt);
        const T lower = l > 0 ? -(T)gU[id - g.plane] : T(0);
        const T upper = l < g.nz - 1 ? -(T)gU[id] : T(0);
        const T inv = RN<T>::div(T(1), RN<T>::sub(d, RN<T>::mul(lower, cp_prev)));
        finv[id] = inv;
        cp_prev = RN<T>::mul(upper, inv);
        fcp[id] = cp_prev;
    }
}

// The face part of op_diag (src/operator3d.h:80-88) of natural column q of
// the fine operator in FP64 — west, east, south, north, up, down or bottom
// sink, summed in that order — which does not change with dt.
__device__ __forceinline__ void faces_column(const OpView& o, unsigned q, double* __restrict__ dface) {
    const Geo& g = o.g;
    const int j = (int)(q / (unsigned)g.nx), i = (int)(q - (unsigned)j * g.nx);
    const unsigned s = scol(g, i, j);
#pragma unroll 4
    for (int l = 0; l < g.nz; ++l) {
        const unsigned base = (unsigned)l * g.plane, id = base + s;
        double d = 0.0;
        if (i > 0) d = __dadd_rn(d, (double)o.gE[base + scol(g, i - 1, j)]);
        if (i < g.nx - 1) d = __dadd_rn(d, (double)o.gE[id]);
        if (j > 0) d = __dadd_rn(d, (double)o.gN[base + scol(g, i, j - 1)]);
        if (j < g.ny - 1) d = __dadd_rn(d, (double)o.gN[id]);
        d = __dadd_rn(d, (double)o.gU[id]);
        d = __dadd_rn(d, l > 0 ? (double)o.gU[id - g.plane] : (double)o.gB[s]);
        dface[id] = d;
    }
}

// FP64 diagonal of natural column q of the fine operator: the stored face
// sum plus C/dt, the last term of op_diag's sum, so the same bits as summing
// it all here (and 1/d for Jacobi, the double-word copy for the double-word
// mode, where requested).
__device__ __forceinline__ void diag_column(const OpView& o, const double* __restrict__ dface, double inv_dt,
                                            unsigned q, double* __restrict__ diag, double* __restrict__ invd,
                                            float2* __restrict__ dgw) {
    const Geo& g = o.g;
    const int j = (int)(q / (unsigned)g.nx), i = (int)(q - (unsigned)j * g.nx);
    const unsigned s = scol(g, i, j);
    const float* __restrict__ cap = o.cap;
#pragma unroll 4
    for (int l = 0; l < g.nz; ++l) {
        const unsigned id = (unsigned)l * g.plane + s;
        const double d = __dadd_rn(dface[id], __dmul_rn((double)cap[id], inv_dt));
        diag[id] = d;
        if (invd) invd[id] = __drcp_rn(d);
        if (dgw) {
            const float h = __double2float_rn(d);
            dgw[id] = make_float2(h, __double2float_rn(d - (double)h));
        }
    }
}

}  // namespace setupdev
}  // namespace ct
