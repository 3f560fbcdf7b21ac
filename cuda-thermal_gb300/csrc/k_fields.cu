// k_fields.cu - field products computed on the device from a solver's
// temperature (split layout, FP64 after the double-word fold), so a caller
// never copies the 3-D field to the host for them:
//  * the die map of the live view without a window (k_colorize,
//    src/viewer.cu:52-87): the hottest of planes l0..l1 at each column, mapped
//    to RGBA on the scale [0, rise_hi], and the die's hottest cell as one
//    64-bit key (float bits of the value, then the cell index);
//  * the per-column maximum over planes l0..l1 (the tmap_layer*.csv maps,
//    src/main3d.cu:303-323, before the ambient offset);
//  * a block's maximum and area-weighted mean over its footprint in planes
//    l0..l1 (block_temps, src/main3d.cu:286-300), with the covered fractions
//    of for_each_overlap (src/stack3d.h:175-191).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "cthermal.h"
#include "kernels.h"
#include "reduce.cuh"
#include "solver.h"
#include "status.h"

namespace ct {
namespace {

// Black -> purple -> red -> orange -> pale yellow colour scale (the live
// view's stops), s clamped to [0, 1], linear between stops, truncated to bytes.
__device__ __forceinline__ uchar4 colour(float s) {
    const float stops[5][3] = {{0, 0, 4}, {87, 16, 110}, {188, 55, 84}, {249, 142, 9}, {252, 255, 164}};
    s = s < 0.0f ? 0.0f : (s > 1.0f ? 1.0f : s);
    float f = s * 4.0f;
    int k = (int)f;
    if (k > 3) k = 3;
    f -= (float)k;
    uchar4 c;
    c.x = (unsigned char)__fmaf_rn(f, stops[k + 1][0] - stops[k][0], stops[k][0]);
    c.y = (unsigned char)__fmaf_rn(f, stops[k + 1][1] - stops[k][1], stops[k][1]);
    c.z = (unsigned char)__fmaf_rn(f, stops[k + 1][2] - stops[k][2], stops[k][2]);
    c.w = 255;
    return c;
}

// Per column q = j nx + i: v = max over planes l0..l1 of (float) x (0 when the
// range is empty, as the view starts from 0); optional map (float), RGBA and
// the packed argmax.
__global__ void __launch_bounds__(NT)
    k_column_max(Geo g, const double* __restrict__ x, int l0, int l1, float rise_hi,
                 float* __restrict__ map, uchar4* __restrict__ rgba,
                 unsigned long long* __restrict__ key_out) {
    const unsigned ncol = (unsigned)g.nx * (unsigned)g.ny;
    unsigned long long key = 0;
    for (unsigned q = blockIdx.x * NT + threadIdx.x; q < ncol; q += gridDim.x * NT) {
        const int j = (int)(q / (unsigned)g.nx), i = (int)(q - (unsigned)j * g.nx);
        const unsigned s = scol(g, i, j);
        float v = 0.0f;
        for (int l = l0; l <= l1; ++l) v = fmaxf(v, (float)x[(unsigned)l * g.plane + s]);
        if (map) map[q] = v;
        if (rgba) rgba[q] = colour(v / rise_hi);
        const unsigned long long k = ((unsigned long long)__float_as_uint(v) << 32) | q;
        key = k > key ? k : key;
    }
    if (key_out) {
        for (int off = 16; off > 0; off >>= 1) {
            const unsigned long long o = __shfl_down_sync(0xffffffffu, key, off);
            key = o > key ? o : key;
        }
        if ((threadIdx.x & 31u) == 0) atomicMax(key_out, key);
    }
}

// A block's max and sum of frac * T and of frac over its footprint in planes
// l0..l1; one thread per covered column (i0..i1 x j0..j1).
__global__ void __launch_bounds__(NT)
    k_block_stats(Geo g, const double* __restrict__ x, int l0, int l1, double dx, double dy,
                  double x0, double y0, double w, double h, int i0, int i1, int j0, int j1,
                  double* __restrict__ out) {
    const int ni = i1 - i0 + 1;
    const unsigned n = (unsigned)ni * (unsigned)(j1 - j0 + 1);
    double tmax = -INFINITY, sum = 0.0, wsum = 0.0;
    for (unsigned q = blockIdx.x * NT + threadIdx.x; q < n; q += gridDim.x * NT) {
        const int j = j0 + (int)(q / (unsigned)ni), i = i0 + (int)(q % (unsigned)ni);
        // overlap of [i dx, (i+1) dx] x [j dy, (j+1) dy] with the block
        const double ox = fmax(0.0, fmin((i + 1) * dx, x0 + w) - fmax(i * dx, x0));
        const double oy = fmax(0.0, fmin((j + 1) * dy, y0 + h) - fmax(j * dy, y0));
        const double a = __dmul_rn(ox, oy);
        if (!(a > 1e-9 * dx * dy)) continue;
        const double frac = a / (dx * dy);
        const unsigned s = scol(g, i, j);
        for (int l = l0; l <= l1; ++l) {
            const double t = x[(unsigned)l * g.plane + s];
            tmax = fmax(tmax, t);
            sum += frac * t;
            wsum += frac;
        }
    }
    // block reductions: max, then the two sums; one triple per block, combined
    // on the host in block order
    __shared__ double smax[NT / 32];
    for (int off = 16; off > 0; off >>= 1) tmax = fmax(tmax, __shfl_down_sync(0xffffffffu, tmax, off));
    if ((threadIdx.x & 31u) == 0) smax[threadIdx.x >> 5] = tmax;
    block_sum2(sum, wsum);
    if (threadIdx.x == 0) {
        double m = -INFINITY;
        for (int k = 0; k < NT / 32; ++k) m = fmax(m, smax[k]);
        out[3 * blockIdx.x] = m;
        out[3 * blockIdx.x + 1] = sum;
        out[3 * blockIdx.x + 2] = wsum;
    }
}

}  // namespace
}  // namespace ct

using ct::fail;

namespace {
// x of the solver as FP64 split layout (double-word correction folded).
const double* solver_x(ct::Solver& v) { return v.x_as_double(nullptr); }

ct_status check_planes(const ct::Solver& v, int l0, int l1, const char* who) {
    if (l0 < 0 || l1 >= v.g0.nz || l0 > l1) return fail(CT_BAD_ARG, "%s: bad plane range %d..%d", who, l0, l1);
    return CT_OK;
}
}  // namespace

extern "C" {

ct_status ct_colorize(ct_solver* s, int l0, int l1, float rise_hi, void* rgba_dev, void* map_dev,
                      double* max_rise, int* max_i, int* max_j) {
    if (!s) return fail(CT_BAD_ARG, "ct_colorize: null solver");
    ct::Solver& v = s->impl;
    ct_status st = check_planes(v, l0, l1, "ct_colorize");
    if (st != CT_OK) return st;
    if (!(rise_hi > 0)) return fail(CT_BAD_ARG, "ct_colorize: rise_hi must be > 0");
    const double* x = solver_x(v);
    unsigned long long* key = reinterpret_cast<unsigned long long*>(v.part);  // reduction scratch
    cudaError_t e = cudaMemsetAsync(key, 0, sizeof(unsigned long long), v.st);
    const unsigned ncol = (unsigned)v.g0.nx * (unsigned)v.g0.ny;
    const unsigned grid = std::min(4096u, (ncol + ct::NT - 1) / ct::NT);
    if (e == cudaSuccess) {
        ct::k_column_max<<<grid, ct::NT, 0, v.st>>>(v.g0, x, l0, l1, rise_hi, (float*)map_dev,
                                                    (uchar4*)rgba_dev, key);
        e = cudaGetLastError();
    }
    unsigned long long hk = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hk, key, sizeof hk, cudaMemcpyDeviceToHost, v.st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(v.st);
    if (e != cudaSuccess) return fail(CT_CUDA_ERROR, "ct_colorize: %s", cudaGetErrorString(e));
    const unsigned q = (unsigned)(hk & 0xffffffffull);
    const unsigned bits = (unsigned)(hk >> 32);
    float f;
    std::memcpy(&f, &bits, sizeof f);
    if (max_rise) *max_rise = f;
    if (max_i) *max_i = (int)(q % (unsigned)v.g0.nx);
    if (max_j) *max_j = (int)(q / (unsigned)v.g0.nx);
    return CT_OK;
}

ct_status ct_block_temps(ct_solver* s, int l0, int l1, double x0, double y0, double w, double h,
                         double* tmax, double* tavg) {
    if (!s) return fail(CT_BAD_ARG, "ct_block_temps: null solver");
    ct::Solver& v = s->impl;
    ct_status st = check_planes(v, l0, l1, "ct_block_temps");
    if (st != CT_OK) return st;
    const double dx = v.dx, dy = v.dy;
    const int i0 = std::max(0, (int)std::floor(x0 / dx));
    const int i1 = std::min(v.g0.nx - 1, (int)std::ceil((x0 + w) / dx));
    const int j0 = std::max(0, (int)std::floor(y0 / dy));
    const int j1 = std::min(v.g0.ny - 1, (int)std::ceil((y0 + h) / dy));
    if (i0 > i1 || j0 > j1) return fail(CT_BAD_ARG, "ct_block_temps: the block covers no cell");
    const unsigned n = (unsigned)(i1 - i0 + 1) * (unsigned)(j1 - j0 + 1);
    const unsigned grid = std::min(1024u, (n + ct::NT - 1) / ct::NT);
    const double* x = solver_x(v);
    double* out = v.part;  // reduction scratch: 3 doubles per block
    ct::k_block_stats<<<grid, ct::NT, 0, v.st>>>(v.g0, x, l0, l1, dx, dy, x0, y0, w, h, i0, i1, j0, j1, out);
    std::vector<double> hb((size_t)3 * grid);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(hb.data(), out, hb.size() * 8, cudaMemcpyDeviceToHost, v.st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(v.st);
    if (e != cudaSuccess) return fail(CT_CUDA_ERROR, "ct_block_temps: %s", cudaGetErrorString(e));
    double m = -INFINITY, sum = 0.0, wsum = 0.0;
    for (unsigned b = 0; b < grid; ++b) {
        m = std::max(m, hb[3 * b]);
        sum += hb[3 * b + 1];
        wsum += hb[3 * b + 2];
    }
    if (!(wsum > 0)) return fail(CT_BAD_ARG, "ct_block_temps: the block covers no cell");
    if (tmax) *tmax = m;
    if (tavg) *tavg = sum / wsum;
    return CT_OK;
}

}  // extern "C"
