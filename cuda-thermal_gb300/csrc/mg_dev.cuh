// mg_dev.cuh - device code of the multigrid V-cycle shared by the single
// solver (k_mg.cu) and the batched solver (k_batch.cu): neighbour maps of the
// colour-split layout, the column line solve (mg_line_solve,
// src/mg3d.h:179-196), the fine residual and restriction
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

// Line solve of the q-th column of colour `color` (mg_line_solve,
// src/mg3d.h:179-196). With MZ > 0 (nz <= MZ) the column stays in registers:
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
        const unsigned sw = n.w ? n.sw : n.s, se = n.e ? n.se : n.s;
        const unsigned ss = n.so ? n.ss : n.s, sn = n.no ? n.sn : n.s;
        T v[MZ], fi[MZ], fc[MZ];
        float gu[MZ];
#pragma unroll
        for (int l = 0; l < MZ; ++l) {
            const unsigned lc = (unsigned)(l < g.nz ? l : g.nz - 1);
            const unsigned base = lc * g.plane, id = base + n.s;
            T rhs = ldm<CG>(L.b + id);
            if (!ZERO) {
                T xw = ldm<CG>(L.x + base + sw), xe = ldm<CG>(L.x + base + se);
                T xs = ldm<CG>(L.x + base + ss), xn = ldm<CG>(L.x + base + sn);
                if (PRO) {
                    const T* cx = C.x + lc * C.g.plane;
                    xw = xw + ldm<CG>(cx + n.pw);
                    xe = xe + ldm<CG>(cx + n.pe);
                    xs = xs + ldm<CG>(cx + n.ps);
                    xn = xn + ldm<CG>(cx + n.pn);
                }
                const float ew = L.gE[base + sw], ee = L.gE[id], ns = L.gN[base + ss], nn = L.gN[id];
                T sum = 0;  // op_lat_sum order: west, east, south, north
                sum += (n.w ? (T)ew : T(0)) * xw;
                sum += (n.e ? (T)ee : T(0)) * xe;
                sum += (n.so ? (T)ns : T(0)) * xs;
                sum += (n.no ? (T)nn : T(0)) * xn;
                rhs = rhs + sum;
            }
            v[l] = rhs;
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
                fc[l] = L.fcp[id];
                gu[l] = L.gU[id];
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

// Restriction (src/pcg3d_cpu.cpp:87-100) of coarse cell (I, J, l): the sum
// over the (up to 4) children, j then i, of the fine residual.
template <class T, bool CG>
__device__ __forceinline__ T restrict_sum(const LevelView<T>& F, T inv_dt, int I, int J, int l) {
    const Geo& fg = F.g;
    const int i1 = min(2 * I + 2, fg.nx), j1 = min(2 * J + 2, fg.ny);
    T sum = 0;
    for (int j = 2 * J; j < j1; ++j)
        for (int i = 2 * I; i < i1; ++i) sum += residual_at<T, CG>(F, inv_dt, i, j, l);
    return sum;
}

// The same stored as coarse b; q = J cnx + I.
template <class T, bool CG>
__device__ __forceinline__ void restrict_cell(const LevelView<T>& F, const LevelView<T>& C,
                                              T inv_dt, unsigned q, int l) {
    const Geo& cg = C.g;
    const int J = (int)(q / (unsigned)cg.nx), I = (int)(q - (unsigned)J * cg.nx);
    C.b[(unsigned)l * cg.plane + scol(cg, I, J)] = restrict_sum<T, CG>(F, inv_dt, I, J, l);
}


// The bottom of the V-cycle (levels k0 .. single column) in ONE block, with
// every one of those levels held in shared memory: operator and factors of
// every level and level k0's b come in by bulk copies (all in flight at once,
// one mbarrier), x and the coarser b start at zero, the phases run with block
// barriers, and level k0's x goes back out for the prolongation above it.
// Same line-solve and restriction code as the grid-wide kernels, pointed at
// shared memory. Returns false (nothing written) if the bounded wait for the
// copies ran out.
template <class T, int MZ>
__device__ __forceinline__ bool vsmall_body(const TailLevels<T>& tl, T inv_dt,
                                            unsigned char* smem) {
    __shared__ TailLevels<T> sl;  // views of the same levels, in shared memory
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        sl.n = tl.n;
        tma::mbar_init(&bar, 1);
        tma::fence_barrier_init();
    }
    __syncthreads();
    {
        unsigned char* q = smem;
        auto take = [&](size_t bytes) {
            unsigned char* r = q;
            q += (bytes + 15) & ~size_t(15);
            return r;
        };
        if (threadIdx.x == 0) {
            unsigned total = 0;
            for (int k = 0; k < tl.n; ++k) {
                const unsigned ln = tl.L[k].g.plane * (unsigned)tl.L[k].g.nz;
                total += 4u * ln * 4u + tl.L[k].g.plane * 4u + 2u * ln * (unsigned)sizeof(T);
                if (k == 0) total += ln * (unsigned)sizeof(T);
            }
            tma::mbar_arrive_expect_tx(&bar, total);
        }
        for (int k = 0; k < tl.n; ++k) {
            const LevelView<T>& G = tl.L[k];
            LevelView<T> S;
            const unsigned ln = G.g.plane * (unsigned)G.g.nz;
            S.g = G.g;
            float* gE = (float*)take(ln * 4);
            float* gN = (float*)take(ln * 4);
            float* gU = (float*)take(ln * 4);
            float* cap = (float*)take(ln * 4);
            float* gB = (float*)take(G.g.plane * 4);
            T* fcp = (T*)take(ln * sizeof(T));
            T* finv = (T*)take(ln * sizeof(T));
            T* x = (T*)take(ln * sizeof(T));
            T* b = (T*)take(ln * sizeof(T));
            if (threadIdx.x == 0) {
                tma::bulk_load(gE, G.gE, ln * 4u, &bar);
                tma::bulk_load(gN, G.gN, ln * 4u, &bar);
                tma::bulk_load(gU, G.gU, ln * 4u, &bar);
                tma::bulk_load(cap, G.cap, ln * 4u, &bar);
                tma::bulk_load(gB, G.gB, G.g.plane * 4u, &bar);
                tma::bulk_load(fcp, G.fcp, ln * (unsigned)sizeof(T), &bar);
                tma::bulk_load(finv, G.finv, ln * (unsigned)sizeof(T), &bar);
                if (k == 0) tma::bulk_load(b, G.b, ln * (unsigned)sizeof(T), &bar);
            }
            // Padding slots are never written by the phases below but go back
            // out with level k0's x: start every slot at zero, as the global
            // arrays' padding is, so no stale shared-memory value (possibly a
            // NaN) reaches the outer iteration.
            for (unsigned i = threadIdx.x; i < ln; i += kSmallThreads) {
                x[i] = T(0);
                if (k > 0) b[i] = T(0);
            }
            S.gE = gE;
            S.gN = gN;
            S.gU = gU;
            S.cap = cap;
            S.gB = gB;
            S.fcp = fcp;
            S.finv = finv;
            S.x = x;
            S.b = b;
            if (threadIdx.x == 0) sl.L[k] = S;
        }
    }
    const bool got = tma::mbar_wait(&bar, 0u);
    if (!__syncthreads_and(got)) {
        if (threadIdx.x == 0) tma::mbar_wait(&bar, 0u);  // let the copies land before leaving
        return false;
    }
    const unsigned tid = threadIdx.x, nth = kSmallThreads;
    const int last = sl.n - 1;
    // Each phase works on register copies of the level views: the views live
    // in shared memory, where the sweeps also store x through generic
    // pointers, so reading them in place would reload every field after
    // every store.
    for (int k = 0; k < last; ++k) {
        const LevelView<T> L = sl.L[k];
        const unsigned ncol = (unsigned)L.g.ny * (unsigned)L.g.hx;
        for (unsigned q = tid; q < ncol; q += nth) sweep_column<T, MZ, true, false, false, true>(L, L, 0, q);
        __syncthreads();
        for (unsigned q = tid; q < ncol; q += nth) sweep_column<T, MZ, false, false, false, true>(L, L, 1, q);
        __syncthreads();
        const LevelView<T> C = sl.L[k + 1];
        const unsigned ccols = (unsigned)C.g.nx * (unsigned)C.g.ny;
        const unsigned work = ccols * (unsigned)C.g.nz;
        for (unsigned w = tid; w < work; w += nth) {
            const int l = (int)(w / ccols);
            restrict_cell<T, false>(L, C, inv_dt, w - (unsigned)l * ccols, l);
        }
        __syncthreads();
    }
    {
        const LevelView<T> L = sl.L[last];
        const unsigned ncol = (unsigned)L.g.ny * (unsigned)L.g.hx;
        for (unsigned q = tid; q < ncol; q += nth) sweep_column<T, MZ, true, false, false, true>(L, L, 0, q);
        __syncthreads();
    }
    for (int k = last - 1; k >= 0; --k) {
        const LevelView<T> L = sl.L[k];
        const LevelView<T> C = sl.L[k + 1];
        const unsigned ncol = (unsigned)L.g.ny * (unsigned)L.g.hx;
        for (unsigned q = tid; q < ncol; q += nth) sweep_column<T, MZ, false, true, false, true>(L, C, 1, q);
        __syncthreads();
        for (unsigned q = tid; q < ncol; q += nth) sweep_column<T, MZ, false, false, false, true>(L, L, 0, q);
        __syncthreads();
    }
    const LevelView<T> S0 = sl.L[0];
    const unsigned ln0 = S0.g.plane * (unsigned)S0.g.nz;
    T* out = tl.L[0].x;
    for (unsigned i = tid; i < ln0; i += nth) out[i] = S0.x[i];
    return true;
}


}  // namespace mgdev
}  // namespace ct
