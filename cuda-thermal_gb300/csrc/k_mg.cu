// k_mg.cu - multigrid V-cycle kernels (x-y semi-coarsening, red-black column
// line smoother) and the multigrid setup kernels, for T = float or double.
//
// Sweeps (mg_line_solve, src/mg3d.h:67-84) of the levels that are not staged
// by bulk tensor copies (k_sweep_tma.cu): one thread per column and plane
// gathers that plane's right-hand side, then one thread per column of the
// active colour runs the Thomas recurrence (k_sweep_split), or one thread per
// column does both for columns deeper than 32 planes (k_sweep). A warp reads
// one contiguous half-row of the split layout per z-plane, and x is written
// once per cell. Two fusions remove whole passes over the level:
//  - the first sweep of a V-cycle starts from x = 0, so it reads no lateral
//    neighbours and needs no memset of x (src/pcg3d_cpu.cpp:71);
//  - prolongation (fine x += coarse parent x, src/pcg3d_cpu.cpp:105-109) is
//    folded into the following black sweep: a black column's line solve reads
//    only its red neighbours, to which it adds their parents' correction on
//    the fly, and the red sweep after it overwrites the red cells.
// The arithmetic of each line solve, restriction and factorisation follows the
// reference functions named beside them.

#include <cstdlib>

#include "kernels.h"
#include "mg_dev.cuh"
#include "reduce.cuh"
#include "setup_dev.cuh"


namespace ct {

using namespace mgdev;
using namespace setupdev;

namespace {

// mg_factor_column (src/mg3d.h:46-61): Thomas factors of every column.
template <class T>
__global__ void k_factor(LevelView<T> L, T inv_dt) {
    const unsigned ncol = (unsigned)L.g.nx * L.g.ny;
    for (unsigned q = blockIdx.x * blockDim.x + threadIdx.x; q < ncol; q += gridDim.x * blockDim.x)
        factor_column<T>(L, inv_dt, q);
}

// set_dt in one launch: the Thomas factors of every column of every level
// (factor_column, mg_factor_column's arithmetic) and, on the finest level's
// columns, the FP64 diagonal (diag_column: d, 1/d for Jacobi, the
// double-word copy). One thread per column of the levels' columns laid end
// to end; each column's operations are those of k_factor and k_diag, so the
// same bits, without a launch per level (ten of the eleven levels of an
// 800 x 800 stack are a few blocks of latency each).
template <class T>
__global__ void __launch_bounds__(NT)
    k_factor_levels(FactorLevels<T> fl, T inv_dt, OpView o, const double* __restrict__ dface, double inv_dt64,
                    double* __restrict__ diag, double* __restrict__ invd, float2* __restrict__ dgw) {
    const unsigned total = fl.first[fl.n];
    for (unsigned q = blockIdx.x * NT + threadIdx.x; q < total; q += gridDim.x * NT) {
        int k = 0;
        while (k + 1 < fl.n && q >= fl.first[k + 1]) ++k;
        const unsigned c = q - fl.first[k];
        factor_column<T>(fl.L[k], inv_dt, c);
        if (k == 0 && diag) diag_column(o, dface, inv_dt64, c, diag, invd, dgw);
    }
}

// mg_coarse_cell (src/mg3d.h:100-136) on split layouts: one thread per coarse
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

// The x = 0 form (the staged levels' first sweep: several waves of short
// blocks) is compiled for 4 blocks per SM in FP32 up to 12 planes (64
// registers; 16 planes or 5 blocks would spill) and lets its dependent launch
// as soon as it starts (800 x 800 FLEX solve 154.9 -> 155.4 solves/s).
template <class T, int MZ, bool ZERO, bool PRO>
__global__ void __launch_bounds__(NT, (ZERO && sizeof(T) == 4 && MZ > 0 && MZ <= 12) ? 4 : 1)
    k_sweep(LevelView<T> L, int color, LevelView<T> C, const Ctl* ctl, Cond cond) {
    pdl_enter();
    if (loop_done(ctl, cond)) return;
    if (ZERO) pdl_trigger();
    const unsigned q = blockIdx.x * NT + threadIdx.x;
    if (q >= (unsigned)L.g.ny * (unsigned)L.g.hx) return;
    sweep_column<T, MZ, ZERO, PRO, false>(L, C, color, q);
}

// Sweep of a small level (L2-resident, latency-bound) with one thread per
// column and plane: a block is 32 columns of the active colour x nz planes.
// Each thread gathers its plane's right-hand side (b plus lat_sum, the same
// operations as sweep_column) and the column's factors into shared memory;
// after one block barrier, one thread per column runs sweep_column's
// recurrence there, and after a second the block writes x plane by plane.
// Same operations in the same order as k_sweep, so the same bits, but a
// thread issues one plane's loads instead of nz planes' (k_sweep: 6.5-7.8 us
// per launch on the 100 x 100 to 25 x 25 levels of an 800 x 800 stack).
template <class T, int MZ, bool ZERO, bool PRO>
__global__ void __launch_bounds__(32 * MZ)
    k_sweep_split(LevelView<T> L, int color, LevelView<T> C, const Ctl* ctl, Cond cond) {
    pdl_enter();
    const int2 flags = loop_flags(ctl);  // tested after the gathers are issued
    __shared__ T sv[MZ][32], sfi[MZ][32], sfc[MZ][32];
    __shared__ float sgu[MZ][32];
    const Geo& g = L.g;
    const unsigned tx = threadIdx.x;
    const int l = (int)threadIdx.y;
    const unsigned q = blockIdx.x * 32u + tx;
    const int j = (int)(q / (unsigned)g.hx), t = (int)(q - (unsigned)j * g.hx);
    const int i = 2 * t + ((j + color) & 1);
    const bool on = q < (unsigned)g.ny * (unsigned)g.hx && i < g.nx;
    unsigned s = 0;
    T rhs = 0, fi = 0, fc = 0;
    float gu = 0.0f;
    if (on) {
        const Nbr n = neighbours<PRO>(g, C.g, i, j, t, color);
        s = n.s;
        const unsigned id = (unsigned)l * g.plane + n.s;
        rhs = L.b[id];
        if (!ZERO) rhs = rhs + lat_sum<T, PRO, false>(L, C, n, l);
        fi = L.finv[id];
        gu = L.gU[id];
        // the x = 0 sweep recomputes fcp as factor_column rounded it (one
        // operand stream less); the others load it
        fc = ZERO ? RN<T>::mul(-(T)gu, fi) : L.fcp[id];
    }
    if (loop_done(flags, cond)) return;  // the same for every thread of the grid
    pdl_trigger();
    if (on) {
        sv[l][tx] = rhs;
        sfi[l][tx] = fi;
        sfc[l][tx] = fc;
        sgu[l][tx] = gu;
    }
    __syncthreads();
    const int nz = g.nz;
    if (on && l == 0) {
        // the recurrence of sweep_column, on shared memory
        T prev = 0;
#pragma unroll 4
        for (int k = 0; k < nz; ++k) {
            const T lower = k > 0 ? -(T)sgu[k - 1][tx] : T(0);
            prev = (sv[k][tx] - lower * prev) * sfi[k][tx];
            sv[k][tx] = prev;
        }
#pragma unroll 4
        for (int k = nz - 2; k >= 0; --k) {
            prev = sv[k][tx] - sfc[k][tx] * prev;
            sv[k][tx] = prev;
        }
    }
    __syncthreads();
    if (on) L.x[(unsigned)l * g.plane + s] = sv[l][tx];
}

// Restriction F -> C, one thread per coarse cell and plane (blockIdx.y is
// the plane; k_restrict), or per coarse cell and pair of consecutive planes
// (k_restrict2: both sums before either store, so the planes' shared
// operands, a child's x one plane up being the next plane's own, are loaded
// once). Pairs pay on large fine levels (800 x 800: 46 us against 49 us),
// single planes on small ones (25 x 25: 8.8 us against 10.5 us, twice the
// threads for a latency-bound launch). k_restrict2 is compiled for 4 blocks
// per SM (64 registers): 38.8 us at 800 x 800, against 39.5 us with 80
// registers and 46.8 / 53.7 us with 48 / 40; the load round trips of a
// thread, not the number of resident warps, bound it.
template <class T>
__global__ void __launch_bounds__(NT)
    k_restrict(LevelView<T> F, LevelView<T> C, const Ctl* ctl, Cond cond) {
    pdl_enter();
    const int2 flags = loop_flags(ctl);  // tested after the sums' loads are issued
    const unsigned q = blockIdx.x * NT + threadIdx.x;
    const Geo& cg = C.g;
    const bool on = q < (unsigned)cg.nx * (unsigned)cg.ny;
    const int J = on ? (int)(q / (unsigned)cg.nx) : 0, I = on ? (int)(q - (unsigned)J * cg.nx) : 0;
    const int l = (int)blockIdx.y;
    const T sum = on ? restrict_sum<T, false>(F, (T)ctl->inv_dt, I, J, l) : T(0);
    if (loop_done(flags, cond) || !on) return;
    pdl_trigger();
    C.b[(unsigned)l * cg.plane + scol(cg, I, J)] = sum;
}

template <class T>
__global__ void __launch_bounds__(NT, 4)
    k_restrict2(LevelView<T> F, LevelView<T> C, const Ctl* ctl, Cond cond) {
    pdl_enter();
    if (loop_done(ctl, cond)) return;
    pdl_trigger();  // several waves: the dependent launches as the last one starts
    const unsigned q = blockIdx.x * NT + threadIdx.x;
    if (q >= (unsigned)C.g.nx * (unsigned)C.g.ny) return;
    restrict_pair<T, false>(F, C, (T)ctl->inv_dt, q, 2 * (int)blockIdx.y);
}

// Restriction F -> C fused with C's first sweep (x = 0, red columns). A
// block is 32 coarse columns x nz planes, one thread per coarse cell and
// plane; each thread also stages its cell's b and, for a red column,
// the cell's 1/pivot and up face in shared memory (the other Thomas factor
// is their rounded product). After one block
// barrier, one thread per red column runs sweep_column<ZERO>'s recurrence on
// them (same operations, same order) and writes the column's x.
template <class T, int MZ>
__global__ void __launch_bounds__(32 * MZ)
    k_restrict_sweep0(LevelView<T> F, LevelView<T> C, const Ctl* ctl, Cond cond) {
    pdl_enter();
    const int2 flags = loop_flags(ctl);  // tested after the sums' loads are issued
    __shared__ T sb[MZ][32], sfi[MZ][32];
    __shared__ float sgu[MZ][32];
    const Geo& cg = C.g;
    const unsigned q = blockIdx.x * 32u + threadIdx.x;
    const int l = (int)threadIdx.y;
    const bool on = q < (unsigned)cg.nx * (unsigned)cg.ny;
    const int J = on ? (int)(q / (unsigned)cg.nx) : 0, I = on ? (int)(q - (unsigned)J * cg.nx) : 0;
    const bool red = on && ((I + J) & 1) == 0;
    const unsigned cs = scol(cg, I, J);
    const unsigned id = (unsigned)l * cg.plane + cs;
    T sum = 0, fi = 0;
    float gu = 0.0f;
    if (on) {
        sum = restrict_sum<T, false>(F, (T)ctl->inv_dt, I, J, l);
        if (red) {
            fi = C.finv[id];
            gu = C.gU[id];
        }
    }
    if (loop_done(flags, cond)) return;  // the same for every thread of the grid
    pdl_trigger();
    if (on) {
        C.b[id] = sum;
        if (red) {
            sb[l][threadIdx.x] = sum;
            sfi[l][threadIdx.x] = fi;
            sgu[l][threadIdx.x] = gu;
        }
    }
    __syncthreads();
    if (threadIdx.y != 0 || !red) return;
    const int nz = cg.nz;
    T v[MZ], fcr[MZ];
    T prev = 0;
#pragma unroll
    for (int k = 0; k < MZ; ++k) {
        if (k < nz) {
            const T lower = k > 0 ? -(T)sgu[k - 1][threadIdx.x] : T(0);
            prev = (sb[k][threadIdx.x] - lower * prev) * sfi[k][threadIdx.x];
            v[k] = prev;
            fcr[k] = RN<T>::mul(-(T)sgu[k][threadIdx.x], sfi[k][threadIdx.x]);  // fcp, as factor_column rounds it
        }
    }
#pragma unroll
    for (int k = MZ - 2; k >= 0; --k)
        if (k < nz - 1) v[k] -= fcr[k] * v[k + 1];
#pragma unroll
    for (int k = 0; k < MZ; ++k)
        if (k < nz) C.x[(unsigned)k * cg.plane + cs] = v[k];
}

// The bottom of the V-cycle in one block from shared memory (mgdev::vsmall_body),
// bounded at the 256 threads it is launched with, so a thread may hold up to
// 255 registers (12 planes: 167, 16 planes: 219, no spills).
template <class T, int MZ>
__global__ void __launch_bounds__(kSmallThreadsSolver, 1)
    k_vsmall(TailLevels<T> tl, Ctl* ctl, Cond cond, bool col_sweeps) {
    extern __shared__ __align__(16) unsigned char smem[];
    const auto wait = [] { pdl_enter(); };
    const auto go = [&] { return !loop_done(ctl, cond); };
    if (mgdev::vsmall_body<T, MZ>(tl, &ctl->inv_dt, smem, wait, go, col_sweeps) == mgdev::kSmallTimeout &&
        threadIdx.x == 0) {
        // a bounded wait ran out: record it and stop the solve
        atomicExch(&ctl->err, 1);
        ctl->breakdown = 1;
        stop_loop(ctl, cond);
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
void launch_factor_levels(cudaStream_t st, const FactorLevels<T>& fl, T inv_dt, const OpView& o,
                          const double* dface, double inv_dt64, double* diag, double* invd, float2* dgw) {
    const unsigned total = fl.first[fl.n];
    k_factor_levels<T><<<blocks_for(total), NT, 0, st>>>(fl, inv_dt, o, dface, inv_dt64, diag, invd, dgw);
}

template <class T>
void launch_sweep(cudaStream_t st, const LevelView<T>& L, int color, bool zero_x,
                  const LevelView<T>* coarse, const Ctl* ctl, Cond cond) {
    const unsigned grid = blocks_for((unsigned)L.g.ny * (unsigned)L.g.hx);
    const LevelView<T> C = coarse ? *coarse : L;
    const int nz = L.g.nz;
    // One thread per column and plane on levels of at most split_cols columns
    // (FP64 levels: all) with at most 32 planes; otherwise one thread per
    // column (CT_SWEEP_SPLIT=0 forces it; CT_SWEEP_SPLIT_COLS moves the
    // threshold). Both give the same bits.
    const char* split_env = std::getenv("CT_SWEEP_SPLIT");
    long long split_cols = sizeof(T) == 8 ? kSweepSplitColumns64 : kSweepSplitColumns;
    if (const char* c = std::getenv("CT_SWEEP_SPLIT_COLS")) split_cols = std::atoll(c);
    if ((long long)L.g.nx * L.g.ny <= split_cols && nz <= 32 && !(split_env && split_env[0] == '0')) {
        const unsigned sgrid = ((unsigned)L.g.ny * (unsigned)L.g.hx + 31u) / 32u;
        const dim3 block(32, (unsigned)nz);
#define CT_SPLIT(MZ)                                                                                     \
    do {                                                                                                 \
        if (zero_x)                                                                                      \
            launch_pdl(k_sweep_split<T, MZ, true, false>, sgrid, block, 0, st, L, color, C, ctl, cond);  \
        else if (coarse)                                                                                 \
            launch_pdl(k_sweep_split<T, MZ, false, true>, sgrid, block, 0, st, L, color, C, ctl, cond);  \
        else                                                                                             \
            launch_pdl(k_sweep_split<T, MZ, false, false>, sgrid, block, 0, st, L, color, C, ctl, cond); \
    } while (0)
        if (nz <= 8)
            CT_SPLIT(8);
        else if (nz <= 16)
            CT_SPLIT(16);
        else
            CT_SPLIT(32);
#undef CT_SPLIT
        return;
    }
#define CT_SWEEP(MZ)                                                                               \
    do {                                                                                           \
        if (zero_x)                                                                                \
            launch_pdl(k_sweep<T, MZ, true, false>, grid, NT, 0, st, L, color, C, ctl, cond);      \
        else if (coarse)                                                                           \
            launch_pdl(k_sweep<T, MZ, false, true>, grid, NT, 0, st, L, color, C, ctl, cond);      \
        else                                                                                       \
            launch_pdl(k_sweep<T, MZ, false, false>, grid, NT, 0, st, L, color, C, ctl, cond);     \
    } while (0)
    if (nz <= 8)
        CT_SWEEP(8);
    else if (nz <= 12)
        CT_SWEEP(12);
    else if (nz <= 16)
        CT_SWEEP(16);
    else if (nz <= 32)
        CT_SWEEP(32);
    else
        CT_SWEEP(0);
#undef CT_SWEEP
}

template <class T>
void launch_restrict(cudaStream_t st, const LevelView<T>& F, const LevelView<T>& C, const Ctl* ctl,
                     Cond cond) {
    if ((unsigned)F.g.nx * (unsigned)F.g.ny > kSweepBfColumns) {
        const dim3 grid(blocks_for((unsigned)C.g.nx * C.g.ny), (unsigned)(C.g.nz + 1) / 2);
        launch_pdl(k_restrict2<T>, grid, NT, 0, st, F, C, ctl, cond);
    } else {
        const dim3 grid(blocks_for((unsigned)C.g.nx * C.g.ny), (unsigned)C.g.nz);
        launch_pdl(k_restrict<T>, grid, NT, 0, st, F, C, ctl, cond);
    }
}

template <class T>
bool launch_restrict_sweep0(cudaStream_t st, const LevelView<T>& F, const LevelView<T>& C, const Ctl* ctl,
                            Cond cond) {
    const int nz = F.g.nz;
    const unsigned grid = ((unsigned)C.g.nx * C.g.ny + 31u) / 32u;
    const dim3 block(32, (unsigned)nz);
    if (nz <= 8)
        launch_pdl(k_restrict_sweep0<T, 8>, grid, block, 0, st, F, C, ctl, cond);
    else if (nz <= 16)
        launch_pdl(k_restrict_sweep0<T, 16>, grid, block, 0, st, F, C, ctl, cond);
    else if (nz <= 32)
        launch_pdl(k_restrict_sweep0<T, 32>, grid, block, 0, st, F, C, ctl, cond);
    else
        return false;
    return true;
}

template void launch_factor_levels<float>(cudaStream_t, const FactorLevels<float>&, float, const OpView&,
                                          const double*, double, double*, double*, float2*);
template void launch_factor_levels<double>(cudaStream_t, const FactorLevels<double>&, double, const OpView&,
                                           const double*, double, double*, double*, float2*);
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
template bool launch_restrict_sweep0<float>(cudaStream_t, const LevelView<float>&, const LevelView<float>&,
                                            const Ctl*, Cond);
template bool launch_restrict_sweep0<double>(cudaStream_t, const LevelView<double>&, const LevelView<double>&,
                                             const Ctl*, Cond);

template <class T>
size_t small_smem_bytes(const TailLevels<T>& tl) {
    size_t b = 0;
    for (int k = 0; k < tl.n; ++k) b += small_level_bytes(tl.L[k].g, sizeof(T));
    return b;
}

template <class T>
cudaError_t launch_vsmall(cudaStream_t st, const TailLevels<T>& tl, Ctl* ctl, Cond cond) {
    const size_t smem = small_smem_bytes(tl);
    int mz = 0;
    for (int k = 0; k < tl.n; ++k) mz = tl.L[k].g.nz;
    auto go = [&](auto kern) {
        // Every k_vsmall instantiation needs its own opt-in to more than 48 KB
        // of dynamic shared memory; set it on every launch (host-side only).
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             kSmallSmemMax);
        if (e != cudaSuccess) return e;
        // FP32 sweeps one thread per column (CT_SMALL_COL_SWEEPS=0: gather
        // and recurrence as two steps, as in FP64 and the batch)
        const char* cs_env = std::getenv("CT_SMALL_COL_SWEEPS");
        const bool col_sweeps = !(cs_env && cs_env[0] == '0');
        // 256 threads (8 warps to a block barrier): 158.5 vs 158.2 solves/s
        // with 512 at 800 x 800 (the batch's instance blocks keep 512)
        launch_pdl(kern, 1, kSmallThreadsSolver, smem, st, tl, ctl, cond, col_sweeps);
        return cudaGetLastError();
    };
    if (mz <= 8) return go(k_vsmall<T, 8>);
    if (mz <= 12) return go(k_vsmall<T, 12>);
    if (mz <= 16) return go(k_vsmall<T, 16>);
    if (mz <= 32) return go(k_vsmall<T, 32>);
    return go(k_vsmall<T, 0>);
}

template size_t small_smem_bytes<float>(const TailLevels<float>&);
template size_t small_smem_bytes<double>(const TailLevels<double>&);
template cudaError_t launch_vsmall<float>(cudaStream_t, const TailLevels<float>&, Ctl*, Cond);
template cudaError_t launch_vsmall<double>(cudaStream_t, const TailLevels<double>&, Ctl*,
                                           Cond);

}  // namespace ct
