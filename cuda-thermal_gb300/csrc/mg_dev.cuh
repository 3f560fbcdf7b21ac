// mg_dev.cuh - device code of the multigrid V-cycle shared by the single
// solver (k_mg.cu) and the batched solver (k_batch.cu): neighbour maps of the
// colour-split layout, the column line solve (mg_line_solve,
// src/mg3d.h:67-84), the fine residual and restriction
// (src/pcg3d_cpu.cpp:87-100), and the shared-memory bottom of the V-cycle.
#pragma once
#include "kernels.h"
#include "tma.cuh"

namespace ct {
namespace mgdev {

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

// The Thomas factor fcp of a cell from its up face and 1/pivot, rounded as
// factor_column rounds it: -gU * finv, one rounding.
__device__ __forceinline__ float fcp_of(float gu, float fi) { return __fmul_rn(-gu, fi); }
__device__ __forceinline__ double fcp_of(float gu, double fi) { return __dmul_rn(-(double)gu, fi); }

// Loads of values that other blocks of the same kernel may have written
// (x and b inside the cluster tail kernel) go to L2 (CG = true); everything
// else may use the L1 path.
template <bool CG, class T>
__device__ __forceinline__ T ldm(const T* p) {
    if (CG) return __ldcg(p);
    return *p;
}

// Lateral neighbour sum of op_lat_sum (src/operator3d.h:62-78) at plane l:
// west, east, south, north; with PRO each neighbour value carries its
// parent's coarse correction.
template <class T, bool PRO, bool CG>
__device__ __forceinline__ T lat_sum(const LevelView<T>& L, const LevelView<T>& C, const Nbr& n,
                                     int l) {
    const unsigned base = (unsigned)l * L.g.plane;
    const unsigned cbase = PRO ? (unsigned)l * C.g.plane : 0u;
    T s = 0;
    if (n.w) {
        T xv = ldm<CG>(L.x + base + n.sw);
        if (PRO) xv = xv + ldm<CG>(C.x + cbase + n.pw);
        s += (T)L.gE[base + n.sw] * xv;
    }
    if (n.e) {
        T xv = ldm<CG>(L.x + base + n.se);
        if (PRO) xv = xv + ldm<CG>(C.x + cbase + n.pe);
        s += (T)L.gE[base + n.s] * xv;
    }
    if (n.so) {
        T xv = ldm<CG>(L.x + base + n.ss);
        if (PRO) xv = xv + ldm<CG>(C.x + cbase + n.ps);
        s += (T)L.gN[base + n.ss] * xv;
    }
    if (n.no) {
        T xv = ldm<CG>(L.x + base + n.sn);
        if (PRO) xv = xv + ldm<CG>(C.x + cbase + n.pn);
        s += (T)L.gN[base + n.s] * xv;
    }
    return s;
}

// Right-hand side of plane l of a column in the branch-free form (BF below):
// b plus the lateral sum in op_lat_sum's order (west, east, south, north),
// each neighbour value with its parent's coarse correction under PRO; an
// absent neighbour reads the column itself with weight 0.
template <class T, bool ZERO, bool PRO, bool CG>
__device__ __forceinline__ T bf_rhs(const LevelView<T>& L, const LevelView<T>& C, const Nbr& n, unsigned l) {
    const Geo& g = L.g;
    const unsigned base = l * g.plane, id = base + n.s;
    T rhs = ldm<CG>(L.b + id);
    if (!ZERO) {
        const unsigned sw = n.w ? n.sw : n.s, se = n.e ? n.se : n.s;
        const unsigned ss = n.so ? n.ss : n.s, sn = n.no ? n.sn : n.s;
        T xw = ldm<CG>(L.x + base + sw), xe = ldm<CG>(L.x + base + se);
        T xs = ldm<CG>(L.x + base + ss), xn = ldm<CG>(L.x + base + sn);
        if (PRO) {
            const T* cx = C.x + l * C.g.plane;
            xw = xw + ldm<CG>(cx + n.pw);
            xe = xe + ldm<CG>(cx + n.pe);
            xs = xs + ldm<CG>(cx + n.ps);
            xn = xn + ldm<CG>(cx + n.pn);
        }
        const float ew = L.gE[base + sw], ee = L.gE[id], ns = L.gN[base + ss], nn = L.gN[id];
        T sum = 0;
        sum += (n.w ? (T)ew : T(0)) * xw;
        sum += (n.e ? (T)ee : T(0)) * xe;
        sum += (n.so ? (T)ns : T(0)) * xs;
        sum += (n.no ? (T)nn : T(0)) * xn;
        rhs = rhs + sum;
    }
    return rhs;
}

// The Thomas recurrence of sweep_column on the column at slot s whose
// right-hand sides are src[l * plane + s] (nz <= MZ): every operand loaded
// first, the recurrence on registers, x written once.
template <class T, int MZ>
__device__ __forceinline__ void column_solve(const LevelView<T>& L, const T* src, unsigned s) {
    const Geo& g = L.g;
    T v[MZ], fi[MZ], fc[MZ];
    float gu[MZ];
#pragma unroll
    for (int l = 0; l < MZ; ++l) {
        if (l < g.nz) {
            const unsigned id = (unsigned)l * g.plane + s;
            v[l] = src[id];
            fi[l] = L.finv[id];
            fc[l] = L.fcp[id];
            gu[l] = L.gU[id];
        }
    }
    T prev = 0;
#pragma unroll
    for (int l = 0; l < MZ; ++l) {
        if (l < g.nz) {
            const T lower = l > 0 ? -(T)gu[l - 1] : T(0);
            prev = (v[l] - lower * prev) * fi[l];
            v[l] = prev;
        }
    }
#pragma unroll
    for (int l = MZ - 2; l >= 0; --l)
        if (l < g.nz - 1) v[l] -= fc[l] * v[l + 1];
#pragma unroll
    for (int l = 0; l < MZ; ++l)
        if (l < g.nz) L.x[(unsigned)l * g.plane + s] = v[l];
}

// Line solve of the q-th column of colour `color` (mg_line_solve,
// src/mg3d.h:67-84). With MZ > 0 (nz <= MZ) the column stays in registers:
// every plane's right-hand side (b plus the lateral sum) is gathered first,
// all loads independent of one another, then the Thomas recurrence runs on
// registers and x is written once. MZ = 0 is the general path for deep
// columns, with forward values going through x as in the reference.
//
// BF (branch-free gather, for levels held in shared memory or L2, where load
// latency rather than bandwidth bounds a sweep): planes past nz read the last
// plane (values unused) and an absent neighbour reads the column itself with
// weight 0 — an exact zero added where lat_sum skips the term — so every
// load of every plane can be in flight at once.
template <class T, int MZ, bool ZERO, bool PRO, bool CG, bool BF = false>
__device__ __forceinline__ void sweep_column(const LevelView<T>& L, const LevelView<T>& C,
                                             int color, unsigned q) {
    const Geo& g = L.g;
    const int j = (int)(q / (unsigned)g.hx), t = (int)(q - (unsigned)j * g.hx);
    const int i = 2 * t + ((j + color) & 1);
    if (i >= g.nx) return;
    const Nbr n = neighbours<PRO>(g, C.g, i, j, t, color);
    if constexpr (MZ > 0 && BF) {
        T v[MZ], fi[MZ], fc[MZ];
        float gu[MZ];
#pragma unroll
        for (int l = 0; l < MZ; ++l) {
            const unsigned lc = (unsigned)(l < g.nz ? l : g.nz - 1);
            const unsigned id = lc * g.plane + n.s;
            v[l] = bf_rhs<T, ZERO, PRO, CG>(L, C, n, lc);
            fi[l] = L.finv[id];
            fc[l] = L.fcp[id];
            gu[l] = L.gU[id];
        }
        T prev = 0;
#pragma unroll
        for (int l = 0; l < MZ; ++l) {
            if (l < g.nz) {
                const T lower = l > 0 ? -(T)gu[l - 1] : T(0);
                prev = (v[l] - lower * prev) * fi[l];
                v[l] = prev;
            }
        }
#pragma unroll
        for (int l = MZ - 2; l >= 0; --l)
            if (l < g.nz - 1) v[l] -= fc[l] * v[l + 1];
#pragma unroll
        for (int l = 0; l < MZ; ++l)
            if (l < g.nz) L.x[(unsigned)l * g.plane + n.s] = v[l];
    } else if constexpr (MZ > 0) {
        // Gather: every operand of every plane, all loads independent, so the
        // whole column costs about one memory latency.
        T v[MZ], fi[MZ], fc[MZ];
        float gu[MZ];
#pragma unroll
        for (int l = 0; l < MZ; ++l) {
            if (l < g.nz) {
                const unsigned id = (unsigned)l * g.plane + n.s;
                T rhs = ldm<CG>(L.b + id);
                if (!ZERO) rhs = rhs + lat_sum<T, PRO, CG>(L, C, n, l);
                v[l] = rhs;
                fi[l] = L.finv[id];
                gu[l] = L.gU[id];
                // the x = 0 sweep recomputes fcp as factor_column rounded it
                // (one operand stream less)
                if (ZERO)
                    fc[l] = fcp_of(gu[l], fi[l]);
                else
                    fc[l] = L.fcp[id];
            }
        }
        // Thomas recurrence on registers.
        T prev = 0;
#pragma unroll
        for (int l = 0; l < MZ; ++l) {
            if (l < g.nz) {
                const T lower = l > 0 ? -(T)gu[l - 1] : T(0);
                prev = (v[l] - lower * prev) * fi[l];
                v[l] = prev;
            }
        }
#pragma unroll
        for (int l = MZ - 2; l >= 0; --l)
            if (l < g.nz - 1) v[l] -= fc[l] * v[l + 1];
#pragma unroll
        for (int l = 0; l < MZ; ++l)
            if (l < g.nz) L.x[(unsigned)l * g.plane + n.s] = v[l];
    } else {
        T prev = 0;
        float gu_b = 0.0f;
        for (int l = 0; l < g.nz; ++l) {
            const unsigned id = (unsigned)l * g.plane + n.s;
            T rhs = ldm<CG>(L.b + id);
            if (!ZERO) rhs = rhs + lat_sum<T, PRO, CG>(L, C, n, l);
            const T lower = l > 0 ? -(T)gu_b : T(0);
            prev = (rhs - lower * prev) * L.finv[id];
            L.x[id] = prev;
            gu_b = L.gU[id];
        }
        for (int l = g.nz - 2; l >= 0; --l) {
            const unsigned id = (unsigned)l * g.plane + n.s;
            prev = ldm<CG>(L.x + id) - L.fcp[id] * prev;
            L.x[id] = prev;
        }
    }
}

// (b - (A + C/dt) x) at fine cell (i, j, l), in op_apply's order
// (src/operator3d.h:108-112): diagonal (lateral faces, up, down or ambient,
// C/dt) times x, minus the six neighbour terms.
template <class T, bool CG>
__device__ __forceinline__ T residual_at(const LevelView<T>& F, T inv_dt, int i, int j, int l) {
    const Geo& fg = F.g;
    const Nbr n = neighbours<false>(fg, fg, i, j, i >> 1, (i + j) & 1);
    const unsigned base = (unsigned)l * fg.plane, id = base + n.s;
    const bool up = l < fg.nz - 1;
    const T xc = ldm<CG>(F.x + id);
    T d = 0, off = 0;
    if (n.w) {
        const T ge = (T)F.gE[base + n.sw];
        d += ge;
        off += ge * ldm<CG>(F.x + base + n.sw);
    }
    if (n.e) {
        const T ge = (T)F.gE[id];
        d += ge;
        off += ge * ldm<CG>(F.x + base + n.se);
    }
    if (n.so) {
        const T gn = (T)F.gN[base + n.ss];
        d += gn;
        off += gn * ldm<CG>(F.x + base + n.ss);
    }
    if (n.no) {
        const T gn = (T)F.gN[id];
        d += gn;
        off += gn * ldm<CG>(F.x + base + n.sn);
    }
    const float gu = F.gU[id];
    d += (T)gu;
    d += l > 0 ? (T)F.gU[id - fg.plane] : (T)F.gB[n.s];
    d += (T)F.cap[id] * inv_dt;
    if (l > 0) off += (T)F.gU[id - fg.plane] * ldm<CG>(F.x + id - fg.plane);
    if (up) off += (T)gu * ldm<CG>(F.x + id + fg.plane);
    return ldm<CG>(F.b + id) - (d * xc - off);
}

// residual_at's arithmetic on operands already loaded, in its order: the
// diagonal (west, east, south, north faces, up face, down face or gB, C/dt)
// times x minus the neighbour terms (west, east, south, north, down, up).
template <class T>
__device__ __forceinline__ T residual_of(T b, T xc, T xw, T xe, T xs, T xn, T xd, T xu, float gew, float gee,
                                         float gns, float gnn, float gu, float gd, float cap, T inv_dt, bool w,
                                         bool e, bool so, bool no, bool down, bool up) {
    T d = 0, off = 0;
    if (w) {
        const T ge = (T)gew;
        d += ge;
        off += ge * xw;
    }
    if (e) {
        const T ge = (T)gee;
        d += ge;
        off += ge * xe;
    }
    if (so) {
        const T gn = (T)gns;
        d += gn;
        off += gn * xs;
    }
    if (no) {
        const T gn = (T)gnn;
        d += gn;
        off += gn * xn;
    }
    d += (T)gu;
    d += (T)gd;
    d += (T)cap * inv_dt;
    if (down) off += (T)gd * xd;
    if (up) off += (T)gu * xu;
    return b - (d * xc - off);
}

// The four children of an interior coarse cell at once: their x, faces and
// the eight outside neighbours are loaded once each (48 values instead of
// four residual_at's 60, with the index arithmetic shared), and each child's
// residual is residual_at's, operation for operation.
template <class T, bool CG>
__device__ __forceinline__ T restrict_sum4(const LevelView<T>& F, T inv_dt, int I, int J, int l) {
    const Geo& g = F.g;
    const int i0 = 2 * I, j0 = 2 * J;
    const bool w = i0 > 0, e = i0 + 2 < g.nx, so = j0 > 0, no = j0 + 2 < g.ny;
    const bool down = l > 0, up = l < g.nz - 1;
    const unsigned base = (unsigned)l * g.plane;
    const unsigned c00 = base + scol(g, i0, j0), c10 = base + scol(g, i0 + 1, j0);
    const unsigned c01 = base + scol(g, i0, j0 + 1), c11 = base + scol(g, i0 + 1, j0 + 1);
    // outside neighbours (an absent one reads the child beside it; unused)
    const unsigned w0 = w ? base + scol(g, i0 - 1, j0) : c00, w1 = w ? base + scol(g, i0 - 1, j0 + 1) : c01;
    const unsigned e0 = e ? base + scol(g, i0 + 2, j0) : c10, e1 = e ? base + scol(g, i0 + 2, j0 + 1) : c11;
    const unsigned s0 = so ? base + scol(g, i0, j0 - 1) : c00, s1 = so ? base + scol(g, i0 + 1, j0 - 1) : c10;
    const unsigned n0 = no ? base + scol(g, i0, j0 + 2) : c01, n1 = no ? base + scol(g, i0 + 1, j0 + 2) : c11;
    const unsigned dn = down ? g.plane : 0u, upo = up ? g.plane : 0u;
    const T x00 = ldm<CG>(F.x + c00), x10 = ldm<CG>(F.x + c10), x01 = ldm<CG>(F.x + c01), x11 = ldm<CG>(F.x + c11);
    const T xw0 = ldm<CG>(F.x + w0), xw1 = ldm<CG>(F.x + w1), xe0 = ldm<CG>(F.x + e0), xe1 = ldm<CG>(F.x + e1);
    const T xs0 = ldm<CG>(F.x + s0), xs1 = ldm<CG>(F.x + s1), xn0 = ldm<CG>(F.x + n0), xn1 = ldm<CG>(F.x + n1);
    const T d00 = ldm<CG>(F.x + c00 - dn), d10 = ldm<CG>(F.x + c10 - dn);
    const T d01 = ldm<CG>(F.x + c01 - dn), d11 = ldm<CG>(F.x + c11 - dn);
    const T u00 = ldm<CG>(F.x + c00 + upo), u10 = ldm<CG>(F.x + c10 + upo);
    const T u01 = ldm<CG>(F.x + c01 + upo), u11 = ldm<CG>(F.x + c11 + upo);
    const float gEw0 = F.gE[w0], gE00 = F.gE[c00], gE10 = F.gE[c10];
    const float gEw1 = F.gE[w1], gE01 = F.gE[c01], gE11 = F.gE[c11];
    const float gNs0 = F.gN[s0], gN00 = F.gN[c00], gNs1 = F.gN[s1], gN10 = F.gN[c10];
    const float gN01 = F.gN[c01], gN11 = F.gN[c11];
    const float gu00 = F.gU[c00], gu10 = F.gU[c10], gu01 = F.gU[c01], gu11 = F.gU[c11];
    // down face: gU of the plane below, or gB at the bottom plane
    const unsigned cb = (unsigned)l * g.plane;
    const float gd00 = down ? F.gU[c00 - dn] : F.gB[c00 - cb], gd10 = down ? F.gU[c10 - dn] : F.gB[c10 - cb];
    const float gd01 = down ? F.gU[c01 - dn] : F.gB[c01 - cb], gd11 = down ? F.gU[c11 - dn] : F.gB[c11 - cb];
    T sum = 0;
    sum += residual_of<T>(ldm<CG>(F.b + c00), x00, xw0, x10, xs0, x01, d00, u00, gEw0, gE00, gNs0, gN00, gu00, gd00,
                          F.cap[c00], inv_dt, w, true, so, true, down, up);
    sum += residual_of<T>(ldm<CG>(F.b + c10), x10, x00, xe0, xs1, x11, d10, u10, gE00, gE10, gNs1, gN10, gu10, gd10,
                          F.cap[c10], inv_dt, true, e, so, true, down, up);
    sum += residual_of<T>(ldm<CG>(F.b + c01), x01, xw1, x11, x00, xn0, d01, u01, gEw1, gE01, gN00, gN01, gu01, gd01,
                          F.cap[c01], inv_dt, w, true, true, no, down, up);
    sum += residual_of<T>(ldm<CG>(F.b + c11), x11, x01, xe1, x10, xn1, d11, u11, gE01, gE11, gN10, gN11, gu11, gd11,
                          F.cap[c11], inv_dt, true, e, true, no, down, up);
    return sum;
}

// Restriction (src/pcg3d_cpu.cpp:87-100) of coarse cell (I, J, l): the sum
// over the (up to 4) children, j then i, of the fine residual.
template <class T, bool CG>
__device__ __forceinline__ T restrict_sum(const LevelView<T>& F, T inv_dt, int I, int J, int l) {
    const Geo& fg = F.g;
    if (2 * I + 1 < fg.nx && 2 * J + 1 < fg.ny) return restrict_sum4<T, CG>(F, inv_dt, I, J, l);
    const int i1 = min(2 * I + 2, fg.nx), j1 = min(2 * J + 2, fg.ny);
    T sum = 0;
    for (int j = 2 * J; j < j1; ++j)
        for (int i = 2 * I; i < i1; ++i) sum += residual_at<T, CG>(F, inv_dt, i, j, l);
    return sum;
}

// Coarse cell q = J cnx + I of the planes l and l + 1 (when it exists):
// both sums before either store, so the shared vertical operands are loaded
// once.
template <class T, bool CG>
__device__ __forceinline__ void restrict_pair(const LevelView<T>& F, const LevelView<T>& C, T inv_dt,
                                              unsigned q, int l) {
    const Geo& cg = C.g;
    const int J = (int)(q / (unsigned)cg.nx), I = (int)(q - (unsigned)J * cg.nx);
    const unsigned cs = scol(cg, I, J);
    const T s0 = restrict_sum<T, CG>(F, inv_dt, I, J, l);
    if (l + 1 < cg.nz) {
        const T s1 = restrict_sum<T, CG>(F, inv_dt, I, J, l + 1);
        C.b[(unsigned)l * cg.plane + cs] = s0;
        C.b[(unsigned)(l + 1) * cg.plane + cs] = s1;
    } else {
        C.b[(unsigned)l * cg.plane + cs] = s0;
    }
}

// The same stored as coarse b; q = J cnx + I.
template <class T, bool CG>
__device__ __forceinline__ void restrict_cell(const LevelView<T>& F, const LevelView<T>& C,
                                              T inv_dt, unsigned q, int l) {
    const Geo& cg = C.g;
    const int J = (int)(q / (unsigned)cg.nx), I = (int)(q - (unsigned)J * cg.nx);
    C.b[(unsigned)l * cg.plane + scol(cg, I, J)] = restrict_sum<T, CG>(F, inv_dt, I, J, l);
}


// Writes the right-hand side (bf_rhs) of every plane of every column of
// colour `color` into that column's x slots; tasks are (plane, column) pairs
// strided over the nth threads of the block.
template <class T, bool PRO>
__device__ __forceinline__ void gather_rhs(const LevelView<T>& L, const LevelView<T>& C, int color, unsigned tid,
                                           unsigned nth) {
    const Geo& g = L.g;
    const unsigned ncol = (unsigned)g.ny * (unsigned)g.hx;
    const unsigned work = ncol * (unsigned)g.nz;
    for (unsigned w = tid; w < work; w += nth) {
        const unsigned l = w / ncol, q = w - l * ncol;
        const int j = (int)(q / (unsigned)g.hx), t = (int)(q - (unsigned)j * g.hx);
        const int i = 2 * t + ((j + color) & 1);
        if (i >= g.nx) continue;
        const Nbr n = neighbours<PRO>(g, C.g, i, j, t, color);
        L.x[l * g.plane + n.s] = bf_rhs<T, false, PRO, false>(L, C, n, l);
    }
}

// Level views of the shared-memory bottom: a level's arrays lie at base in
// the order gE, gN, gU, cap, gB, fcp, finv, x, b, each rounded up to 16 bytes
// (small_level_bytes adds the same sizes). The views are rebuilt from the
// block's base and a byte offset wherever they are used, never stored as
// pointers, so every pointer visibly points into shared memory and the
// compiler issues shared-memory loads through them rather than generic ones.
template <class T>
__device__ __forceinline__ LevelView<T> small_view(unsigned char* base, const Geo& g) {
    const unsigned ln = g.plane * (unsigned)g.nz;
    unsigned char* p = base;
    auto take = [&](unsigned bytes) {
        unsigned char* r = p;
        p += small_round16(bytes);
        return r;
    };
    LevelView<T> S;
    S.g = g;
    S.gE = (const float*)take(ln * 4u);
    S.gN = (const float*)take(ln * 4u);
    S.gU = (const float*)take(ln * 4u);
    S.cap = (const float*)take(ln * 4u);
    S.gB = (const float*)take(g.plane * 4u);
    S.fcp = (T*)take(ln * (unsigned)sizeof(T));
    S.finv = (T*)take(ln * (unsigned)sizeof(T));
    S.x = (T*)take(ln * (unsigned)sizeof(T));
    S.b = (T*)take(ln * (unsigned)sizeof(T));
    return S;
}

// The bottom of the V-cycle (levels k0 .. single column) in ONE block, with
// every one of those levels held in shared memory: operator and factors of
// every level and level k0's b come in by bulk copies (all in flight at once),
// x and the coarser b start at zero, the phases run with block barriers, and
// level k0's x goes back out for the prolongation above it. Same line-solve
// and restriction code as the grid-wide kernels, pointed at shared memory.
//
// The operator and factors do not change during a solve, so their copies are
// issued (one per lane of the first warp) before wait() (every thread calls
// it: it waits for the preceding kernel); level k0's b, the preceding
// kernel's output, is copied after it, and go() (called after that copy is
// issued, so the two latencies overlap) says whether to run the phases at
// all. Returns kSmallDone, kSmallClosed (go() said no: nothing written once
// the copies have landed) or kSmallTimeout (a bounded wait for the copies ran
// out: nothing written). col_sweeps (FP32): each sweep one thread per column
// over every plane; otherwise one task per column and plane gathers the
// right-hand sides first. Same bits either way; any block size.
constexpr int kSmallDone = 0, kSmallTimeout = 1, kSmallClosed = 2;

template <class T, int MZ, class Wait, class Go>
__device__ __forceinline__ int vsmall_body(const TailLevels<T>& tl, const double* inv_dt_src,
                                           unsigned char* smem, Wait wait, Go go, bool col_sweeps = false) {
    __shared__ Geo sg[kMaxTail];      // level geometry
    __shared__ unsigned soff[kMaxTail];  // byte offset of each level in smem
    __shared__ uint64_t bar, barb;    // operator and factors; level k0's b
    const int nl = tl.n;
    if (threadIdx.x == 0) {
        unsigned off = 0, total = 0;
        for (int k = 0; k < nl; ++k) {
            const Geo g = tl.L[k].g;
            sg[k] = g;
            soff[k] = off;
            off += (unsigned)small_level_bytes(g, sizeof(T));
            const unsigned ln = g.plane * (unsigned)g.nz;
            total += 4u * ln * 4u + g.plane * 4u + 2u * ln * (unsigned)sizeof(T);
        }
        tma::mbar_init(&bar, 1);
        tma::mbar_init(&barb, 1);
        tma::fence_barrier_init();
        tma::mbar_arrive_expect_tx(&bar, total);
    }
    __syncthreads();
    if (threadIdx.x < 32u) {
        // copy c of level k = c / 7: gE, gN, gU, cap, gB, fcp, finv
        for (int c = (int)threadIdx.x; c < 7 * nl; c += 32) {
            const int k = c / 7, a = c - 7 * k;
            const LevelView<T>& G = tl.L[k];
            const LevelView<T> S = small_view<T>(smem + soff[k], sg[k]);
            const unsigned ln = sg[k].plane * (unsigned)sg[k].nz;
            const unsigned fb = ln * 4u, tb = ln * (unsigned)sizeof(T);
            if (a == 0) tma::bulk_load((void*)S.gE, G.gE, fb, &bar);
            else if (a == 1) tma::bulk_load((void*)S.gN, G.gN, fb, &bar);
            else if (a == 2) tma::bulk_load((void*)S.gU, G.gU, fb, &bar);
            else if (a == 3) tma::bulk_load((void*)S.cap, G.cap, fb, &bar);
            else if (a == 4) tma::bulk_load((void*)S.gB, G.gB, sg[k].plane * 4u, &bar);
            else if (a == 5) tma::bulk_load(S.fcp, G.fcp, tb, &bar);
            else tma::bulk_load(S.finv, G.finv, tb, &bar);
        }
    }
    // Padding slots are never written by the phases below but go back out
    // with level k0's x: start every slot at zero, as the global arrays'
    // padding is, so no stale shared-memory value (possibly a NaN) reaches
    // the outer iteration.
    for (int k = 0; k < nl; ++k) {
        const LevelView<T> S = small_view<T>(smem + soff[k], sg[k]);
        const unsigned ln = sg[k].plane * (unsigned)sg[k].nz;
        for (unsigned i = threadIdx.x; i < ln; i += blockDim.x) {
            S.x[i] = T(0);
            if (k > 0) S.b[i] = T(0);
        }
    }
    wait();
    if (threadIdx.x == 0) {
        const unsigned bytes = sg[0].plane * (unsigned)sg[0].nz * (unsigned)sizeof(T);
        tma::mbar_arrive_expect_tx(&barb, bytes);
        tma::bulk_load(small_view<T>(smem, sg[0]).b, tl.L[0].b, bytes, &barb);
    }
    if (!__syncthreads_and(go() ? 1 : 0)) {
        if (threadIdx.x == 0) {  // let the copies land before leaving
            tma::mbar_wait(&bar, 0u);
            tma::mbar_wait(&barb, 0u);
        }
        return kSmallClosed;
    }
    const T inv_dt = (T)*inv_dt_src;
    const bool got = tma::mbar_wait(&bar, 0u) && tma::mbar_wait(&barb, 0u);
    if (!__syncthreads_and(got)) {
        if (threadIdx.x == 0) {  // let the copies land before leaving
            tma::mbar_wait(&bar, 0u);
            tma::mbar_wait(&barb, 0u);
        }
        return kSmallTimeout;
    }
    const unsigned tid = threadIdx.x, nth = blockDim.x;
    const int last = nl - 1;
    // The phases in V-cycle order, driven by one loop so that each kind of
    // phase (x = 0 sweep, sweep, restriction, prolongating sweep) is one
    // code region, warm in the instruction cache after its first use: down
    // the levels k < last (red x = 0 sweep, black sweep, restriction), the
    // single column (x = 0 sweep), back up (black sweep with the coarse
    // correction, red sweep).
    const int nph = 3 * last + 1 + 2 * last;
    for (int ph = 0; ph < nph; ++ph) {
        int k, kind;  // kind: 0 x = 0 sweep, 1 sweep, 2 restriction, 3 prolongating sweep
        int color = 0;
        if (ph < 3 * last) {
            k = ph / 3;
            kind = ph - 3 * k;
            color = kind == 1 ? 1 : 0;
        } else if (ph == 3 * last) {
            k = last;
            kind = 0;
        } else {
            const int u = ph - 3 * last - 1;
            k = last - 1 - u / 2;
            kind = (u & 1) ? 1 : 3;
            color = (u & 1) ? 0 : 1;
        }
        const LevelView<T> L = small_view<T>(smem + soff[k], sg[k]);
        const unsigned ncol = (unsigned)L.g.ny * (unsigned)L.g.hx;
        if (kind == 2) {
            const LevelView<T> C = small_view<T>(smem + soff[k + 1], sg[k + 1]);
            const unsigned ccols = (unsigned)C.g.nx * (unsigned)C.g.ny;
            const unsigned work = ccols * (unsigned)C.g.nz;
            for (unsigned w = tid; w < work; w += nth) {
                const int l = (int)(w / ccols);
                restrict_cell<T, false>(L, C, inv_dt, w - (unsigned)l * ccols, l);
            }
        } else if (sizeof(T) == 4 && MZ > 0 && kind != 0 && col_sweeps) {
            // One thread per column gathers every plane's right-hand side
            // (branch-free, all loads in flight at once) and runs the
            // recurrence: one block barrier a sweep instead of two (FP32
            // only: the FP64 columns' registers would spill).
            if constexpr (sizeof(T) == 4 && MZ > 0) {
                for (unsigned q = tid; q < ncol; q += nth) {
                    if (kind == 1)
                        sweep_column<T, MZ, false, false, false, true>(L, L, color, q);
                    else
                        sweep_column<T, MZ, false, true, false, true>(
                            L, small_view<T>(smem + soff[k + 1], sg[k + 1]), 1, q);
                }
            }
        } else if constexpr (MZ > 0) {
            // A sweep in two steps: one task per column and plane gathers
            // that plane's right-hand side into the column's own x slot (the
            // sweep reads only the other colour's x, so no task reads a slot
            // another one writes), then one thread per column runs the
            // recurrence. Same operations as sweep_column, with the gathers
            // spread over the block instead of one thread walking the planes.
            if (kind == 1)
                gather_rhs<T, false>(L, L, color, tid, nth);
            else if (kind == 3)
                gather_rhs<T, true>(L, small_view<T>(smem + soff[k + 1], sg[k + 1]), color, tid, nth);
            if (kind != 0) __syncthreads();
            const T* src = kind == 0 ? L.b : L.x;
            for (unsigned q = tid; q < ncol; q += nth) {
                const int j = (int)(q / (unsigned)L.g.hx), t = (int)(q - (unsigned)j * L.g.hx);
                if (2 * t + ((j + color) & 1) < L.g.nx)
                    column_solve<T, MZ>(L, src, (unsigned)(2 * j + color) * (unsigned)L.g.hx + (unsigned)t);
            }
        } else if (kind == 0) {  // deep columns (MZ = 0): x goes through memory
            for (unsigned q = tid; q < ncol; q += nth) sweep_column<T, MZ, true, false, false, true>(L, L, 0, q);
        } else if (kind == 1) {
            for (unsigned q = tid; q < ncol; q += nth) sweep_column<T, MZ, false, false, false, true>(L, L, color, q);
        } else {
            const LevelView<T> C = small_view<T>(smem + soff[k + 1], sg[k + 1]);
            for (unsigned q = tid; q < ncol; q += nth) sweep_column<T, MZ, false, true, false, true>(L, C, 1, q);
        }
        __syncthreads();
    }
    pdl_trigger();
    const LevelView<T> S0 = small_view<T>(smem, sg[0]);
    const unsigned ln0 = S0.g.plane * (unsigned)S0.g.nz;
    T* out = tl.L[0].x;
    for (unsigned i = tid; i < ln0; i += nth) out[i] = S0.x[i];
    return kSmallDone;
}


}  // namespace mgdev
}  // namespace ct
