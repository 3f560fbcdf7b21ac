// k_tail.cu - the coarse end of the V-cycle (vcycle, src/pcg3d_gpu.cu:561-590;
// src/pcg3d_cpu.cpp:69-113) in ONE launch of one thread-block cluster.
//
// Below a few thousand columns a level's sweep or restriction is a few
// microseconds of dependent memory round trips, and launching it as a grid
// kernel costs as much again: at 800 x 800 the levels from 50 x 50 down took
// a dozen launches per V-cycle, each 7-11 us whatever its size. Here one
// cluster of CTAs (one per SM, all co-scheduled on one GPC) runs every phase
// of those levels - the restriction into the first of them, then per level
// the red x = 0 sweep, the black sweep and the restriction, the single
// column's solve, and back up the prolongating black sweep and the red sweep
// - separated by the cluster's hardware barrier (barrier.cluster with
// release / acquire semantics) instead of kernel boundaries. The level
// arrays stay where they are (global memory, resident in L2); values that
// other CTAs of the cluster wrote in an earlier phase (x, b) are loaded from
// L2 (ld.global.cg), the read-only operator and factors through L1.
//
// Each phase runs the same per-column and per-cell device code as the grid
// kernels (mgdev::sweep_column, mgdev::restrict_cell), so results are bit
// for bit those of the separate launches. Every CTA runs every phase and
// every barrier (the loop over phases has no early exit); the only early
// return is at entry, when the solve is already done, and every CTA takes it
// alike (they all read the same control flag after the predecessor
// completed).
#include <algorithm>
#include <cooperative_groups.h>

#include "kernels.h"
#include "mg_dev.cuh"
#include "reduce.cuh"

namespace cg = cooperative_groups;

namespace ct {

namespace {

constexpr int kTailThreads = 512;

template <class T, int MZ>
__global__ void __launch_bounds__(kTailThreads, 1)
    k_vtail(LevelView<T> F, TailLevels<T> tl, Ctl* ctl, Cond cond) {
    pdl_enter();
    if (loop_done(ctl, cond)) return;
    cg::cluster_group cl = cg::this_cluster();
    const unsigned tid = cl.block_rank() * kTailThreads + threadIdx.x;
    const unsigned nth = cl.num_blocks() * kTailThreads;
    const T inv_dt = (T)ctl->inv_dt;
    const int last = tl.n - 1;
    // phase -1: restriction of level F (above the tail) into tail level 0;
    // then down the levels k < last (red x = 0 sweep, black sweep,
    // restriction), the single column (x = 0 sweep), back up (black sweep
    // with the coarse correction, red sweep)
    const int nph = 1 + 3 * last + 1 + 2 * last;
    for (int ph = 0; ph < nph; ++ph) {
        if (ph == 0) {
            const LevelView<T>& C = tl.L[0];
            const unsigned ccols = (unsigned)C.g.nx * (unsigned)C.g.ny;
            const unsigned work = ccols * (unsigned)C.g.nz;
            for (unsigned w = tid; w < work; w += nth) {
                const int l = (int)(w / ccols);
                mgdev::restrict_cell<T, true>(F, C, inv_dt, w - (unsigned)l * ccols, l);
            }
        } else {
            const int p = ph - 1;
            int k, kind;  // kind: 0 x = 0 sweep, 1 sweep, 2 restriction, 3 prolongating sweep
            int color = 0;
            if (p < 3 * last) {
                k = p / 3;
                kind = p - 3 * k;
                color = kind == 1 ? 1 : 0;
            } else if (p == 3 * last) {
                k = last;
                kind = 0;
            } else {
                const int u = p - 3 * last - 1;
                k = last - 1 - u / 2;
                kind = (u & 1) ? 1 : 3;
                color = (u & 1) ? 0 : 1;
            }
            const LevelView<T>& L = tl.L[k];
            if (kind == 2) {
                const LevelView<T>& C = tl.L[k + 1];
                const unsigned ccols = (unsigned)C.g.nx * (unsigned)C.g.ny;
                const unsigned work = ccols * (unsigned)C.g.nz;
                for (unsigned w = tid; w < work; w += nth) {
                    const int l = (int)(w / ccols);
                    mgdev::restrict_cell<T, true>(L, C, inv_dt, w - (unsigned)l * ccols, l);
                }
            } else {
                const unsigned ncol = (unsigned)L.g.ny * (unsigned)L.g.hx;
                for (unsigned q = tid; q < ncol; q += nth) {
                    if (kind == 0)
                        mgdev::sweep_column<T, MZ, true, false, true, true>(L, L, 0, q);
                    else if (kind == 1)
                        mgdev::sweep_column<T, MZ, false, false, true, true>(L, L, color, q);
                    else
                        mgdev::sweep_column<T, MZ, false, true, true, true>(L, tl.L[k + 1], 1, q);
                }
            }
        }
        cl.sync();
    }
}

template <class T, int MZ>
cudaError_t go_tail(cudaStream_t st, int csize, const LevelView<T>& F, const TailLevels<T>& tl, Ctl* ctl,
                    Cond cond) {
    auto kern = k_vtail<T, MZ>;
    if (csize > 8) {
        const cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        if (e != cudaSuccess) return e;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)csize);
    cfg.blockDim = dim3(kTailThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute at[2];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)csize;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    at[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[1].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl_enabled() ? 2 : 1;
    cudaLaunchKernelEx(&cfg, kern, F, tl, ctl, cond);
    return cudaGetLastError();
}

template <class T, int MZ>
int probe_one(int csize) {
    auto kern = k_vtail<T, MZ>;
    if (csize > 8 &&
        cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)csize);
    cfg.blockDim = dim3(kTailThreads);
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)csize;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, kern, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

}  // namespace

template <class T>
int tail_cluster_size(int mz) {
    // the largest of 16 (non-portable) and 8 CTAs that the device can place
    for (int cs : {16, 8}) {
        int n = 0;
        if (mz <= 8)
            n = probe_one<T, 8>(cs);
        else if (mz <= 12)
            n = probe_one<T, 12>(cs);
        else if (mz <= 16)
            n = probe_one<T, 16>(cs);
        else if (mz <= 32)
            n = probe_one<T, 32>(cs);
        else
            n = probe_one<T, 0>(cs);
        if (n > 0) return cs;
    }
    return 0;
}

template <class T>
cudaError_t launch_vtail(cudaStream_t st, int csize, const LevelView<T>& F, const TailLevels<T>& tl, Ctl* ctl,
                         Cond cond) {
    const int mz = tl.L[0].g.nz;
    if (mz <= 8) return go_tail<T, 8>(st, csize, F, tl, ctl, cond);
    if (mz <= 12) return go_tail<T, 12>(st, csize, F, tl, ctl, cond);
    if (mz <= 16) return go_tail<T, 16>(st, csize, F, tl, ctl, cond);
    if (mz <= 32) return go_tail<T, 32>(st, csize, F, tl, ctl, cond);
    return go_tail<T, 0>(st, csize, F, tl, ctl, cond);
}

template int tail_cluster_size<float>(int);
template int tail_cluster_size<double>(int);
template cudaError_t launch_vtail<float>(cudaStream_t, int, const LevelView<float>&, const TailLevels<float>&,
                                         Ctl*, Cond);
template cudaError_t launch_vtail<double>(cudaStream_t, int, const LevelView<double>&, const TailLevels<double>&,
                                          Ctl*, Cond);

}  // namespace ct
