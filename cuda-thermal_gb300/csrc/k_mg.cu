// k_mg.cu - multigrid V-cycle kernels (x-y semi-coarsening, red-black column
// line smoother) and the multigrid setup kernels, for T = float or double.
//
// Sweeps (mg_line_solve, src/mg3d.h:175-196): one thread per column of the
// active colour, so a warp reads one contiguous half-row of the split layout
// per z-plane. The column is eliminated forward through the planes with the
// precomputed Thomas factors and substituted back in registers, so x is
// written once per cell. Two fusions remove whole passes over the level:
//  - the first sweep of a V-cycle starts from x = 0, so it reads no lateral
//    neighbours and needs no memset of x (src/pcg3d_cpu.cpp:71);
//  - prolongation (fine x += coarse parent x, src/pcg3d_cpu.cpp:105-109) is
//    folded into the following black sweep: a black column's line solve reads
//    only its red neighbours, to which it adds their parents' correction on
//    the fly, and the red sweep after it overwrites the red cells.
// The arithmetic of each line solve, restriction and factorisation follows the
// reference functions named beside them.
#include "kernels.h"
#include "reduce.cuh"

namespace ct {

namespace {

// Rounding-explicit arithmetic for the setup kernels: no contraction into
// FMAs, so factors and coarse operators equal the CPU's bit for bit.
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

// op_diag (src/operator3d.h:80-88) of cell (i, j, l), in T, rounding-explicit.
template <class T>
__device__ T diag_rn(const LevelView<T>& L, int i, int j, int l, T inv_dt) {
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

// mg_factor_column (src/mg3d.h:157-173): Thomas factors of every column.
template <class T>
__global__ void k_factor(LevelView<T> L, T inv_dt) {
    const Geo& g = L.g;
    const unsigned ncol = (unsigned)g.nx * g.ny;
    for (unsigned q = blockIdx.x * blockDim.x + threadIdx.x; q < ncol; q += gridDim.x * blockDim.x) {
        const int j = (int)(q / g.nx), i = (int)(q - (unsigned)j * g.nx);
        const unsigned s = scol(g, i, j);
        T cp_prev = 0;
        for (int l = 0; l < g.nz; ++l) {
            const unsigned id = (unsigned)l * g.plane + s;
            const T d = diag_rn(L, i, j, l, inv_dt);
            const T lower = l > 0 ? -(T)L.gU[id - g.plane] : T(0);
            const T upper = l < g.nz - 1 ? -(T)L.gU[id] : T(0);
            const T inv = RN<T>::div(T(1), RN<T>::sub(d, RN<T>::mul(lower, cp_prev)));
            L.finv[id] = inv;
            cp_prev = RN<T>::mul(upper, inv);
            L.fcp[id] = cp_prev;
        }
    }
}

// mg_coarse_cell (src/mg3d.h:206-248) on split layouts: one thread per coarse
// cell, sums in double in the reference's child order, one cast to float.
__global__ void k_coarsen(Geo fg, const float* __restrict__ fgE, const float* __restrict__ fgN,
                          const float* __restrict__ fgU, const float* __restrict__ fgB,
                          const float* __restrict__ fcap, const double* __restrict__ fdx,
                          const double* __restrict__ fdy, Geo cg, const double* __restrict__ cdx,
                          const double* __restrict__ cdy, float* cgE, float* cgN, float* cgU,
                          float* cgB, float* ccap) {
    const unsigned cxy = (unsigned)cg.nx * cg.ny, n = cxy * (unsigned)cg.nz;
    for (unsigned q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        const int l = (int)(q / cxy);
        const unsigned rem = q - (unsigned)l * cxy;
        const int J = (int)(rem / cg.nx), I = (int)(rem - (unsigned)J * cg.nx);
        const unsigned fb = (unsigned)l * fg.plane, cb = (unsigned)l * cg.plane;
        const int i0 = 2 * I, i1 = (2 * I + 1 < fg.nx - 1) ? 2 * I + 1 : fg.nx - 1;
        const int j0 = 2 * J, j1 = (2 * J + 1 < fg.ny - 1) ? 2 * J + 1 : fg.ny - 1;
        double gu = 0, cp = 0, gb = 0;
        for (int j = j0; j <= j1; ++j)
            for (int i = i0; i <= i1; ++i) {
                const unsigned fs = scol(fg, i, j);
                gu = __dadd_rn(gu, (double)fgU[fb + fs]);
                cp = __dadd_rn(cp, (double)fcap[fb + fs]);
                if (l == 0) gb = __dadd_rn(gb, (double)fgB[fs]);
            }
        const unsigned cs = scol(cg, I, J);
        cgU[cb + cs] = __double2float_rn(gu);
        ccap[cb + cs] = __double2float_rn(cp);
        if (l == 0) cgB[cs] = __double2float_rn(gb);
        float e = 0.0f, nn = 0.0f;
        if (I < cg.nx - 1) {  // fine faces between columns 2I+1 and 2I+2
            double sum = 0;
            for (int j = j0; j <= j1; ++j) sum = __dadd_rn(sum, (double)fgE[fb + scol(fg, 2 * I + 1, j)]);
            const double df = __dmul_rn(0.5, __dadd_rn(fdx[2 * I + 1], fdx[2 * I + 2]));
            const double dc = __dmul_rn(0.5, __dadd_rn(cdx[I], cdx[I + 1]));
            e = __double2float_rn(__ddiv_rn(__dmul_rn(sum, df), dc));
        }
        if (J < cg.ny - 1) {  // fine faces between rows 2J+1 and 2J+2
            double sum = 0;
            for (int i = i0; i <= i1; ++i) sum = __dadd_rn(sum, (double)fgN[fb + scol(fg, i, 2 * J + 1)]);
            const double df = __dmul_rn(0.5, __dadd_rn(fdy[2 * J + 1], fdy[2 * J + 2]));
            const double dc = __dmul_rn(0.5, __dadd_rn(cdy[J], cdy[J + 1]));
            nn = __double2float_rn(__ddiv_rn(__dmul_rn(sum, df), dc));
        }
        cgE[cb + cs] = e;
        cgN[cb + cs] = nn;
    }
}

// Neighbour slots of an active column, and (for fused prolongation) the
// coarse slots of those neighbours' parents.
struct Nbr {
    unsigned s, sw, se, ss, sn;
    unsigned pw, pe, ps, pn;
    bool w, e, so, no;
};

template <bool PRO>
__device__ __forceinline__ Nbr neighbours(const Geo& g, const Geo& cg, int i, int j, int t,
                                          int color) {
    Nbr n;
    const int oc = color ^ 1;
    const unsigned row_o = (unsigned)(2 * j + oc) * (unsigned)g.hx;
    n.s = (unsigned)(2 * j + color) * (unsigned)g.hx + (unsigned)t;
    n.w = i > 0;
    n.e = i < g.nx - 1;
    n.so = j > 0;
    n.no = j < g.ny - 1;
    n.sw = row_o + (unsigned)((i - 1) >> 1);
    n.se = row_o + (unsigned)((i + 1) >> 1);
    n.ss = (unsigned)(2 * j - 2 + oc) * (unsigned)g.hx + (unsigned)t;
    n.sn = (unsigned)(2 * j + 2 + oc) * (unsigned)g.hx + (unsigned)t;
    if (PRO) {
        n.pw = n.w ? scol(cg, (i - 1) >> 1, j >> 1) : 0u;
        n.pe = n.e ? scol(cg, (i + 1) >> 1, j >> 1) : 0u;
        n.ps = n.so ? scol(cg, i >> 1, (j - 1) >> 1) : 0u;
        n.pn = n.no ? scol(cg, i >> 1, (j + 1) >> 1) : 0u;
    }
    return n;
}

// Lateral neighbour sum of op_lat_sum (src/operator3d.h:62-78) at plane l:
// west, east, south, north; with PRO each neighbour value carries its
// parent's coarse correction.
template <class T, bool PRO>
__device__ __forceinline__ T lat_sum(const LevelView<T>& L, const LevelView<T>& C, const Nbr& n,
                                     int l) {
    const unsigned base = (unsigned)l * L.g.plane;
    const unsigned cbase = PRO ? (unsigned)l * C.g.plane : 0u;
    T s = 0;
    if (n.w) {
        T xv = L.x[base + n.sw];
        if (PRO) xv = xv + C.x[cbase + n.pw];
        s += (T)L.gE[base + n.sw] * xv;
    }
    if (n.e) {
        T xv = L.x[base + n.se];
        if (PRO) xv = xv + C.x[cbase + n.pe];
        s += (T)L.gE[base + n.s] * xv;
    }
    if (n.so) {
        T xv = L.x[base + n.ss];
        if (PRO) xv = xv + C.x[cbase + n.ps];
        s += (T)L.gN[base + n.ss] * xv;
    }
    if (n.no) {
        T xv = L.x[base + n.sn];
        if (PRO) xv = xv + C.x[cbase + n.pn];
        s += (T)L.gN[base + n.s] * xv;
    }
    return s;
}

// Red-black sweep with the column held in registers (nz <= MZ).
template <class T, int MZ, bool ZERO, bool PRO>
__global__ void __launch_bounds__(NT)
    k_sweep_reg(LevelView<T> L, int color, LevelView<T> C, const Ctl* ctl, Cond cond) {
    if (loop_done(ctl, cond)) return;
    const Geo& g = L.g;
    const unsigned q = blockIdx.x * NT + threadIdx.x;
    if (q >= (unsigned)g.ny * (unsigned)g.hx) return;
    const int j = (int)(q / (unsigned)g.hx), t = (int)(q - (unsigned)j * g.hx);
    const int i = 2 * t + ((j + color) & 1);
    if (i >= g.nx) return;
    const Nbr n = neighbours<PRO>(g, C.g, i, j, t, color);
    T v[MZ];
    T prev = 0;
    float gu_b = 0.0f;
#pragma unroll
    for (int l = 0; l < MZ; ++l) {
        if (l < g.nz) {
            const unsigned id = (unsigned)l * g.plane + n.s;
            T rhs = L.b[id];
            if (!ZERO) rhs = rhs + lat_sum<T, PRO>(L, C, n, l);
            const T lower = l > 0 ? -(T)gu_b : T(0);
            prev = (rhs - lower * prev) * L.finv[id];
            v[l] = prev;
            gu_b = L.gU[id];
        }
    }
#pragma unroll
    for (int l = MZ - 2; l >= 0; --l)
        if (l < g.nz - 1) v[l] -= L.fcp[(unsigned)l * g.plane + n.s] * v[l + 1];
#pragma unroll
    for (int l = 0; l < MZ; ++l)
        if (l < g.nz) L.x[(unsigned)l * g.plane + n.s] = v[l];
}

// Same for deep columns: forward values go through x, as in the reference.
template <class T, bool ZERO, bool PRO>
__global__ void __launch_bounds__(NT)
    k_sweep_mem(LevelView<T> L, int color, LevelView<T> C, const Ctl* ctl, Cond cond) {
    if (loop_done(ctl, cond)) return;
    const Geo& g = L.g;
    const unsigned q = blockIdx.x * NT + threadIdx.x;
    if (q >= (unsigned)g.ny * (unsigned)g.hx) return;
    const int j = (int)(q / (unsigned)g.hx), t = (int)(q - (unsigned)j * g.hx);
    const int i = 2 * t + ((j + color) & 1);
    if (i >= g.nx) return;
    const Nbr n = neighbours<PRO>(g, C.g, i, j, t, color);
    T prev = 0;
    float gu_b = 0.0f;
    for (int l = 0; l < g.nz; ++l) {
        const unsigned id = (unsigned)l * g.plane + n.s;
        T rhs = L.b[id];
        if (!ZERO) rhs = rhs + lat_sum<T, PRO>(L, C, n, l);
        const T lower = l > 0 ? -(T)gu_b : T(0);
        prev = (rhs - lower * prev) * L.finv[id];
        L.x[id] = prev;
        gu_b = L.gU[id];
    }
    for (int l = g.nz - 2; l >= 0; --l) {
        const unsigned id = (unsigned)l * g.plane + n.s;
        prev = L.x[id] - L.fcp[id] * prev;
        L.x[id] = prev;
    }
}

// Restriction (src/pcg3d_cpu.cpp:87-100): coarse b(I, J, l) = sum over the
// (up to 4) children, j then i, of b - (A + C/dt) x, the operator applied
// with op_apply's order (src/operator3d.h:108-112). One thread per coarse
// column; each child keeps its x at l-1, l and the face below in registers.
template <class T>
__global__ void __launch_bounds__(NT)
    k_restrict(LevelView<T> F, LevelView<T> C, const Ctl* ctl, Cond cond) {
    if (loop_done(ctl, cond)) return;
    const Geo& fg = F.g;
    const Geo& cg = C.g;
    const unsigned q = blockIdx.x * NT + threadIdx.x;
    if (q >= (unsigned)cg.nx * (unsigned)cg.ny) return;
    const int J = (int)(q / (unsigned)cg.nx), I = (int)(q - (unsigned)J * cg.nx);
    const T inv_dt = (T)ctl->inv_dt;
    int ci[4], cj[4];
    int nc = 0;
    for (int j = 2 * J; j < min(2 * J + 2, fg.ny); ++j)
        for (int i = 2 * I; i < min(2 * I + 2, fg.nx); ++i) {
            ci[nc] = i;
            cj[nc] = j;
            ++nc;
        }
    Nbr nb[4];
    T xc[4], xb[4];
    float gub[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (k < nc) {
            const int colour = (ci[k] + cj[k]) & 1;
            nb[k] = neighbours<false>(fg, cg, ci[k], cj[k], ci[k] >> 1, colour);
            xc[k] = F.x[nb[k].s];
            xb[k] = 0;
            gub[k] = 0.0f;
        }
    }
    const unsigned cs = scol(cg, I, J);
    for (int l = 0; l < fg.nz; ++l) {
        const unsigned base = (unsigned)l * fg.plane;
        const bool up = l < fg.nz - 1;
        T sum = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (k < nc) {
                const Nbr& n = nb[k];
                const unsigned id = base + n.s;
                const T xa = up ? F.x[id + fg.plane] : T(0);
                const float gu = F.gU[id];
                T d = 0, off = 0;
                if (n.w) {
                    const T ge = (T)F.gE[base + n.sw];
                    d += ge;
                    off += ge * F.x[base + n.sw];
                }
                if (n.e) {
                    const T ge = (T)F.gE[id];
                    d += ge;
                    off += ge * F.x[base + n.se];
                }
                if (n.so) {
                    const T gn = (T)F.gN[base + n.ss];
                    d += gn;
                    off += gn * F.x[base + n.ss];
                }
                if (n.no) {
                    const T gn = (T)F.gN[id];
                    d += gn;
                    off += gn * F.x[base + n.sn];
                }
                d += (T)gu;
                d += l > 0 ? (T)gub[k] : (T)F.gB[n.s];
                d += (T)F.cap[id] * inv_dt;
                if (l > 0) off += (T)gub[k] * xb[k];
                if (up) off += (T)gu * xa;
                sum += F.b[id] - (d * xc[k] - off);
                xb[k] = xc[k];
                xc[k] = xa;
                gub[k] = gu;
            }
        }
        C.b[(unsigned)l * cg.plane + cs] = sum;
    }
}

unsigned blocks_for(unsigned n) { return n == 0 ? 1u : (n + NT - 1) / NT; }

}  // namespace

void launch_coarsen(cudaStream_t st, const Geo& fg, const float* fgE, const float* fgN,
                    const float* fgU, const float* fgB, const float* fcap, const double* fdx,
                    const double* fdy, const Geo& cg, const double* cdx, const double* cdy,
                    float* cgE, float* cgN, float* cgU, float* cgB, float* ccap) {
    const unsigned n = (unsigned)cg.nx * cg.ny * cg.nz;
    k_coarsen<<<blocks_for(n), NT, 0, st>>>(fg, fgE, fgN, fgU, fgB, fcap, fdx, fdy, cg, cdx, cdy,
                                            cgE, cgN, cgU, cgB, ccap);
}

template <class T>
void launch_factor(cudaStream_t st, const LevelView<T>& L, T inv_dt) {
    k_factor<T><<<blocks_for((unsigned)L.g.nx * L.g.ny), NT, 0, st>>>(L, inv_dt);
}

template <class T>
void launch_sweep(cudaStream_t st, const LevelView<T>& L, int color, bool zero_x,
                  const LevelView<T>* coarse, const Ctl* ctl, Cond cond) {
    const unsigned grid = blocks_for((unsigned)L.g.ny * (unsigned)L.g.hx);
    const LevelView<T> C = coarse ? *coarse : L;
    const int nz = L.g.nz;
#define CT_SWEEP(MZ)                                                                        \
    do {                                                                                    \
        if (zero_x)                                                                         \
            k_sweep_reg<T, MZ, true, false><<<grid, NT, 0, st>>>(L, color, C, ctl, cond);   \
        else if (coarse)                                                                    \
            k_sweep_reg<T, MZ, false, true><<<grid, NT, 0, st>>>(L, color, C, ctl, cond);   \
        else                                                                                \
            k_sweep_reg<T, MZ, false, false><<<grid, NT, 0, st>>>(L, color, C, ctl, cond);  \
    } while (0)
    if (nz <= 16) {
        CT_SWEEP(16);
    } else if (nz <= 32) {
        CT_SWEEP(32);
    } else if (zero_x) {
        k_sweep_mem<T, true, false><<<grid, NT, 0, st>>>(L, color, C, ctl, cond);
    } else if (coarse) {
        k_sweep_mem<T, false, true><<<grid, NT, 0, st>>>(L, color, C, ctl, cond);
    } else {
        k_sweep_mem<T, false, false><<<grid, NT, 0, st>>>(L, color, C, ctl, cond);
    }
#undef CT_SWEEP
}

template <class T>
void launch_restrict(cudaStream_t st, const LevelView<T>& F, const LevelView<T>& C, const Ctl* ctl,
                     Cond cond) {
    k_restrict<T><<<blocks_for((unsigned)C.g.nx * C.g.ny), NT, 0, st>>>(F, C, ctl, cond);
}

template void launch_factor<float>(cudaStream_t, const LevelView<float>&, float);
template void launch_factor<double>(cudaStream_t, const LevelView<double>&, double);
template void launch_sweep<float>(cudaStream_t, const LevelView<float>&, int, bool,
                                  const LevelView<float>*, const Ctl*, Cond);
template void launch_sweep<double>(cudaStream_t, const LevelView<double>&, int, bool,
                                   const LevelView<double>*, const Ctl*, Cond);
template void launch_restrict<float>(cudaStream_t, const LevelView<float>&,
                                     const LevelView<float>&, const Ctl*, Cond);
template void launch_restrict<double>(cudaStream_t, const LevelView<double>&,
                                      const LevelView<double>&, const Ctl*, Cond);

}  // namespace ct
