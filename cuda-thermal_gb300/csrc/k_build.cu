// k_build.cu - the stack model built on the device from its description
// (layers, power blocks, TSV regions), straight into a solver's split-layout
// arrays: no host arrays and no upload. The arithmetic is the host builder's
// (model.cpp: add_tsv_region, add_power_block, finalize of
// src/stack3d.h:110-220) with every rounding explicit, so the arrays are the
// same bits.
#include <algorithm>
#include <cmath>

#include "build.h"
#include "kernels.h"

namespace ct {
namespace {

__device__ __forceinline__ double ovl(double a0, double a1, double b0, double b1) {
    return fmax(0.0, __dsub_rn(fmin(a1, b1), fmax(a0, b0)));
}

// Covered fraction of column (i, j) by the rectangle (0 when only a rounding
// sliver touches it), for_each_overlap (src/stack3d.h:175-191).
__device__ __forceinline__ double covered(int i, int j, double dx, double dy, double x0, double y0,
                                          double w, double h) {
    const double a = __dmul_rn(ovl(__dmul_rn((double)i, dx), __dmul_rn((double)(i + 1), dx), x0, __dadd_rn(x0, w)),
                               ovl(__dmul_rn((double)j, dy), __dmul_rn((double)(j + 1), dy), y0, __dadd_rn(y0, h)));
    if (!(a > __dmul_rn(__dmul_rn(1e-9, dx), dy))) return 0.0;
    return __ddiv_rn(a, __dmul_rn(dx, dy));
}

// add_tsv_region on plane l: t = min(1, t + f frac) over the covered columns.
__global__ void k_rect_tsv(int nx, int ny, int l, double dx, double dy, BuildRect r, int i0, int i1,
                           int j0, int j1, double* __restrict__ frac) {
    const int ni = i1 - i0 + 1;
    const int n = ni * (j1 - j0 + 1);
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        const int j = j0 + q / ni, i = i0 + q % ni;
        const double c = covered(i, j, dx, dy, r.x0, r.y0, r.w, r.h);
        if (c == 0.0) continue;
        double& t = frac[((size_t)l * ny + j) * nx + i];
        const double v = __dadd_rn(t, __dmul_rn(r.v, c));
        t = v < 1.0 ? v : 1.0;
    }
}

// add_power_block on plane l: P += density frac dx dy / planes.
__global__ void k_rect_power(int nx, int ny, int l, double dx, double dy, BuildRect r, double density,
                             int planes, int i0, int i1, int j0, int j1, double* __restrict__ P) {
    const int ni = i1 - i0 + 1;
    const int n = ni * (j1 - j0 + 1);
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        const int j = j0 + q / ni, i = i0 + q % ni;
        const double c = covered(i, j, dx, dy, r.x0, r.y0, r.w, r.h);
        if (c == 0.0) continue;
        double& p = P[((size_t)l * ny + j) * nx + i];
        p = __dadd_rn(p, __ddiv_rn(__dmul_rn(__dmul_rn(__dmul_rn(density, c), dx), dy), (double)planes));
    }
}

__device__ __forceinline__ double eff_kz(double k, double kc, double f) {
    return __dadd_rn(__dmul_rn(f, kc), __dmul_rn(__dsub_rn(1.0, f), k));
}
__device__ __forceinline__ double eff_kxy(double k, double kc, double f) {
    const double num = __dadd_rn(__dmul_rn(__dadd_rn(1.0, f), kc), __dmul_rn(__dsub_rn(1.0, f), k));
    const double den = __dadd_rn(__dmul_rn(__dsub_rn(1.0, f), kc), __dmul_rn(__dadd_rn(1.0, f), k));
    return __ddiv_rn(__dmul_rn(k, num), den);
}

// finalize (src/stack3d.h:110-148) for natural cell (i, j, l): capacity and
// the east, north and up face conductances (two half cells in series), the
// bottom one at l = 0, written to the split layout.
__global__ void k_finalize(Geo g, PlaneTable pt, double dx, double dy, double h_top, double h_bot,
                           double tsv_k, double tsv_rho_c, const double* __restrict__ frac,
                           float* __restrict__ gE, float* __restrict__ gN, float* __restrict__ gU,
                           float* __restrict__ gB, float* __restrict__ cap) {
    const size_t nxy = (size_t)g.nx * g.ny, n = nxy * g.nz;
    const double A = __dmul_rn(dx, dy);
    for (size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x; id < n; id += (size_t)gridDim.x * blockDim.x) {
        const int l = (int)(id / nxy);
        const size_t c = id - (size_t)l * nxy;
        const int j = (int)(c / (size_t)g.nx), i = (int)(c - (size_t)j * g.nx);
        const unsigned s = (unsigned)l * g.plane + scol(g, i, j);
        const double k = pt.k[l], d = pt.dz[l];
        const double f = frac[id];
        const double kxy = eff_kxy(k, tsv_k, f), kz = eff_kz(k, tsv_k, f);
        cap[s] = __double2float_rn(__dmul_rn(
            __dmul_rn(__dadd_rn(__dmul_rn(f, tsv_rho_c), __dmul_rn(__dsub_rn(1.0, f), pt.rho_c[l])), A), d));
        float e = 0.0f, nn = 0.0f;
        if (i < g.nx - 1) {
            const double k2 = eff_kxy(k, tsv_k, frac[id + 1]);
            e = __double2float_rn(__ddiv_rn(__dmul_rn(dy, d), __dadd_rn(__ddiv_rn(dx, __dmul_rn(2.0, kxy)),
                                                                         __ddiv_rn(dx, __dmul_rn(2.0, k2)))));
        }
        if (j < g.ny - 1) {
            const double k2 = eff_kxy(k, tsv_k, frac[id + g.nx]);
            nn = __double2float_rn(__ddiv_rn(__dmul_rn(dx, d), __dadd_rn(__ddiv_rn(dy, __dmul_rn(2.0, kxy)),
                                                                          __ddiv_rn(dy, __dmul_rn(2.0, k2)))));
        }
        gE[s] = e;
        gN[s] = nn;
        double r_up;
        if (l < g.nz - 1) {
            const double kz2 = eff_kz(pt.k[l + 1], tsv_k, frac[id + nxy]);
            r_up = __dadd_rn(__ddiv_rn(d, __dmul_rn(2.0, kz)), __ddiv_rn(pt.dz[l + 1], __dmul_rn(2.0, kz2)));
        } else {
            r_up = __dadd_rn(__ddiv_rn(d, __dmul_rn(2.0, kz)), __ddiv_rn(1.0, h_top));
        }
        gU[s] = __double2float_rn(__ddiv_rn(A, r_up));
        if (l == 0)
            gB[scol(g, i, j)] = h_bot > 0 ? __double2float_rn(__ddiv_rn(
                                                A, __dadd_rn(__ddiv_rn(d, __dmul_rn(2.0, kz)), __ddiv_rn(1.0, h_bot))))
                                          : 0.0f;
    }
}

// Columns the rectangle may cover (for_each_overlap's index range).
bool rect_range(const DeviceBuild& b, const BuildRect& r, int* i0, int* i1, int* j0, int* j1) {
    *i0 = std::max(0, (int)std::floor(r.x0 / b.dx));
    *i1 = std::min(b.nx - 1, (int)std::ceil((r.x0 + r.w) / b.dx));
    *j0 = std::max(0, (int)std::floor(r.y0 / b.dy));
    *j1 = std::min(b.ny - 1, (int)std::ceil((r.y0 + r.h) / b.dy));
    return *i0 <= *i1 && *j0 <= *j1;
}

unsigned grid_of(size_t n) { return (unsigned)std::max<size_t>(1, std::min<size_t>((n + 255) / 256, 65535u * 16u)); }

}  // namespace

cudaError_t launch_build(cudaStream_t st, const DeviceBuild& b, const Geo& g, double* frac_nat,
                         double* P_nat, float* gE, float* gN, float* gU, float* gB, float* cap) {
    const size_t n = (size_t)b.nx * b.ny * b.nz;
    cudaError_t e = cudaMemsetAsync(frac_nat, 0, n * sizeof(double), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(P_nat, 0, n * sizeof(double), st);
    if (e != cudaSuccess) return e;
    // TSV regions, then power blocks, each in the caller's order, plane by plane
    for (const BuildRect& r : b.tsvs) {
        int i0, i1, j0, j1;
        if (!rect_range(b, r, &i0, &i1, &j0, &j1)) continue;
        const size_t cols = (size_t)(i1 - i0 + 1) * (j1 - j0 + 1);
        for (int l = 0; l < b.nz; ++l)
            if (b.plane_layer[l] == r.layer)
                k_rect_tsv<<<grid_of(cols), 256, 0, st>>>(b.nx, b.ny, l, b.dx, b.dy, r, i0, i1, j0, j1, frac_nat);
    }
    for (const BuildRect& r : b.blocks) {
        int i0, i1, j0, j1;
        if (!rect_range(b, r, &i0, &i1, &j0, &j1)) continue;
        const double density = r.v / (r.w * r.h);
        const size_t cols = (size_t)(i1 - i0 + 1) * (j1 - j0 + 1);
        for (int l = 0; l < b.nz; ++l)
            if (b.plane_layer[l] == r.layer)
                k_rect_power<<<grid_of(cols), 256, 0, st>>>(b.nx, b.ny, l, b.dx, b.dy, r, density,
                                                            b.layer_planes[r.layer], i0, i1, j0, j1, P_nat);
    }
    k_finalize<<<grid_of(n), 256, 0, st>>>(g, b.planes, b.dx, b.dy, b.h_top, b.h_bot, b.tsv_k, b.tsv_rho_c,
                                           frac_nat, gE, gN, gU, gB, cap);
    return cudaGetLastError();
}

}  // namespace ct
