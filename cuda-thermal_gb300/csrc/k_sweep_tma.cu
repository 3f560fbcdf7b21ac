// k_sweep_tma.cu - the red-black column line solve of the large multigrid
// levels (mg_line_solve, src/mg3d.h:67-84), with its operands staged in
// shared memory by bulk tensor copies (TMA).
//
// Work unit: a tile of 32 x 8 columns of the sweep's colour (32 consecutive
// slots of 8 rows j), one thread per column, all nz planes. A block is 8
// consumer warps (one tile row each) and one producer warp, whose lane 0
// issues, for each plane of the tile, a handful of TMA box loads (the tile's
// own b, column factors, gU, gE, gN and, with halos, the other colour's x, gE
// and gN around it) into one stage of a ring of kSweepStagesWs stages. The
// block is persistent over its tiles and the ring runs across tile
// boundaries, so the copies for the next planes (and the next tile) are in
// flight while the consumers run the Thomas recurrence on the current one.
// Each consumer thread keeps its column's forward values in registers and
// writes x once after the last plane. The arithmetic is the grid kernel's
// (k_mg.cu), operation for operation.
//
// Every mbarrier wait is bounded; a wait that runs out sets ctl->err and ends
// the solve, and the block leaves after waiting (bounded) for its own copies.
#include <algorithm>
#include <cstdlib>
#include <cudaTypedefs.h>

#include "batch.h"
#include "kernels.h"
#include "reduce.cuh"
#include "tma.cuh"

namespace ct {

namespace {

using namespace tma;

// Stage layout of one plane of a TT x TJ tile, in floats: six own-colour
// boxes (b, finv, fcp, gU, gE, gN), then the other colour's x (TJ + 2 rows,
// 4 halo slots each side), gE (TJ rows, same halo) and gN (TJ + 1 rows). Each
// box starts on a 128-byte boundary.
template <int TT, int TJ>
struct Stage {
    static constexpr int round(int f) { return (f + 31) & ~31; }
    static constexpr int own = TT * TJ;
    static constexpr int oxw = TT + 8;
    static constexpr int ox = round((TJ + 2) * oxw);
    static constexpr int oge = round(TJ * oxw);
    static constexpr int ogn = round((TJ + 1) * TT);
    // own boxes: b, finv, gU (and gE, gN unless x = 0); the Thomas factor
    // fcp is not loaded: it is -gU finv rounded once, recomputed in place
    static constexpr int full = 5 * own + ox + oge + ogn;
    static constexpr int zero = 3 * own;
    static constexpr unsigned tx_full = 4u * (5 * own + (TJ + 2) * oxw + TJ * oxw + (TJ + 1) * TT);
    static constexpr unsigned tx_zero = 4u * (3 * own);
    static_assert((own * 4) % 128 == 0, "own box must be a multiple of 128 bytes");
};

// Records a timed-out wait and stops the solve.
__device__ void fail_wait(Ctl* ctl, Cond cond) {
    atomicExch(&ctl->err, 1);
    *(volatile int*)&ctl->breakdown = 1;
    *(volatile int*)&ctl->done = 1;
    if (cond.use) cudaGraphSetConditional(cond.h, 0u);
}

// The tiles a block works on: first, first + step, ... (my_tiles of them).
struct TileList {
    int first, step, count;
    __device__ int tile(int mt) const { return first + mt * step; }
};

// Item w of a block = plane w % nz of its (w / nz)-th tile, into stage
// w % NS: one arrival with the stage's byte count, then the boxes.
template <int TT, int TJ, int NS, bool ZERO>
__device__ __forceinline__ void issue_plane(const SweepMaps* m, float* sm, uint64_t* full, int w,
                                            int nz, int tilesx, const TileList& tl) {
    using S = Stage<TT, TJ>;
    constexpr int stage_f = ZERO ? S::zero : S::full;
    const int s = w % NS;
    const int mt = w / nz, l = w - mt * nz;
    const int tile = tl.tile(mt);
    const int tyi = tile / tilesx;
    const int t0 = (tile - tyi * tilesx) * TT, j0 = tyi * TJ;
    float* st = sm + s * stage_f;
    uint64_t* bar = &full[s];
    mbar_arrive_expect_tx(bar, ZERO ? S::tx_zero : S::tx_full);
    load_3d(st, &m->b, t0, j0, l, bar);
    load_3d(st + S::own, &m->fi, t0, j0, l, bar);
    load_3d(st + 2 * S::own, &m->gu, t0, j0, l, bar);
    if (!ZERO) {
        load_3d(st + 3 * S::own, &m->ge, t0, j0, l, bar);
        load_3d(st + 4 * S::own, &m->gn, t0, j0, l, bar);
        load_3d(st + 5 * S::own, &m->ox, t0 - 4, j0 - 1, l, bar);
        load_3d(st + 5 * S::own + S::ox, &m->oge, t0 - 4, j0, l, bar);
        load_3d(st + 5 * S::own + S::ox + S::oge, &m->ogn, t0, j0 - 1, l, bar);
    }
}

// The same line solves with a producer warp: TJ consumer warps (one tile row
// each) and one more warp whose lane 0 issues the boxes. Consumers wait on a
// stage's `full` barrier and, when their warp is done with it, arrive on its
// `empty` barrier; the producer refills a stage once all TJ consumer warps
// have arrived. No block-wide barrier inside the loop, so warps drift apart
// and cover one another's waits. A wait that runs out raises `abort`, which
// ends every other wait.
template <int TT, int TJ, int NS, int MZ, bool ZERO, bool PRO>
__device__ __forceinline__ bool sweep_tiles_ws(const SweepMaps* m, const LevelView<float>& L,
                                               const LevelView<float>& C, int color,
                                               const TileList& tl, float* sm, uint64_t* full,
                                               uint64_t* empty, volatile int* abort, volatile int* issued) {
    static_assert(TT == 32, "one consumer warp per tile row");
    using S = Stage<TT, TJ>;
    constexpr int stage_f = ZERO ? S::zero : S::full;
    const Geo& g = L.g;
    const int nz = g.nz;
    const int tilesx = (g.hx + TT - 1) / TT;
    const int nitems = tl.count * nz;
    const int warp = (int)threadIdx.x / 32, lane = (int)threadIdx.x % 32;
    if (threadIdx.x == 0) {
        for (int s = 0; s < NS; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], TJ);
        }
        *abort = 0;
        *issued = 0;
        fence_barrier_init();
    }
    __syncthreads();
    if (warp == TJ) {  // producer
        if (lane == 0) {
            for (int w = 0; w < nitems; ++w) {
                const int s = w % NS;
                if (w >= NS && !mbar_wait_or_abort(&empty[s], (unsigned)(w / NS - 1) & 1u, abort)) break;
                issue_plane<TT, TJ, NS, ZERO>(m, sm, full, w, nz, tilesx, tl);
                *issued = w + 1;
            }
            pdl_trigger();  // every copy of this block issued
        }
    } else {  // consumers: warp = tile row
        const int tx = lane, ty = warp;
        const int o = ty * TT + tx;
        int w = 0;
        for (int mt = 0; mt < tl.count && !*abort; ++mt) {
            const int tile = tl.tile(mt);
            const int tyi = tile / tilesx;
            const int t = (tile - tyi * tilesx) * TT + tx, j = tyi * TJ + ty;
            const int e = (j + color) & 1;
            const int i = 2 * t + e;
            const bool act = j < g.ny && i < g.nx;
            const bool hw = i > 0, he = i < g.nx - 1, hs = j > 0, hn = j < g.ny - 1;
            unsigned pw = 0, pe = 0, ps = 0, pn = 0;
            if (PRO && act) {
                if (hw) pw = scol(C.g, (i - 1) >> 1, j >> 1);
                if (he) pe = scol(C.g, (i + 1) >> 1, j >> 1);
                if (hs) ps = scol(C.g, i >> 1, (j - 1) >> 1);
                if (hn) pn = scol(C.g, i >> 1, (j + 1) >> 1);
            }
            float v[MZ], fcr[MZ];
            float prev = 0.0f, gu_prev = 0.0f;
            bool ok = true;
            // the neighbours' coarse corrections (PRO) one plane ahead: plane
            // l + 1's loads are in flight while plane l waits and computes
            float nw = 0.0f, ne = 0.0f, nso = 0.0f, nno = 0.0f;
            auto load_corr = [&](int l) {
                const float* cx = C.x + (unsigned)l * C.g.plane;
                nw = hw ? cx[pw] : 0.0f;
                ne = he ? cx[pe] : 0.0f;
                nso = hs ? cx[ps] : 0.0f;
                nno = hn ? cx[pn] : 0.0f;
            };
            if (PRO && act) load_corr(0);
#pragma unroll
            for (int l = 0; l < MZ; ++l) {
                if (l < nz && ok) {
                    const float cw = nw, ce = ne, cs = nso, cn = nno;
                    if (PRO && act && l + 1 < nz) load_corr(l + 1);
                    const int s = w % NS;
                    ok = mbar_wait_or_abort(&full[s], (unsigned)(w / NS) & 1u, abort);
                    ok = __all_sync(0xffffffffu, ok);
                    if (ok) {
                        const float* st = sm + s * stage_f;
                        if (act) {
                            float rhs = st[o];
                            const float fi = st[S::own + o], gu = st[2 * S::own + o];
                            const float fc = __fmul_rn(-gu, fi);  // fcp as factor_column rounds it
                            if (!ZERO) {
                                const float* ox = st + 5 * S::own;
                                const float* oge = ox + S::ox;
                                const float* ogn = oge + S::oge;
                                constexpr int W = S::oxw;
                                float sl = 0.0f;  // op_lat_sum order: west, east, south, north
                                if (hw) {
                                    float xv = ox[(ty + 1) * W + tx + 3 + e];
                                    if (PRO) xv = xv + cw;
                                    sl += oge[ty * W + tx + 3 + e] * xv;
                                }
                                if (he) {
                                    float xv = ox[(ty + 1) * W + tx + 4 + e];
                                    if (PRO) xv = xv + ce;
                                    sl += st[3 * S::own + o] * xv;
                                }
                                if (hs) {
                                    float xv = ox[ty * W + tx + 4];
                                    if (PRO) xv = xv + cs;
                                    sl += ogn[ty * TT + tx] * xv;
                                }
                                if (hn) {
                                    float xv = ox[(ty + 2) * W + tx + 4];
                                    if (PRO) xv = xv + cn;
                                    sl += st[4 * S::own + o] * xv;
                                }
                                rhs = rhs + sl;
                            }
                            const float lower = l > 0 ? -gu_prev : 0.0f;
                            prev = (rhs - lower * prev) * fi;
                            v[l] = prev;
                            fcr[l] = fc;
                            gu_prev = gu;
                        }
                        __syncwarp();
                        if (lane == 0) mbar_arrive(&empty[s]);
                        ++w;
                    }
                }
            }
            if (!ok) break;
            if (act) {
#pragma unroll
                for (int l = MZ - 2; l >= 0; --l)
                    if (l < nz - 1) v[l] -= fcr[l] * v[l + 1];
                const unsigned s0 = (unsigned)(2 * j + color) * (unsigned)g.hx + (unsigned)t;
#pragma unroll
                for (int l = 0; l < MZ; ++l)
                    if (l < nz) L.x[(unsigned)l * g.plane + s0] = v[l];
            }
        }
    }
    __syncthreads();
    const bool failed = *abort != 0;
    if (failed && threadIdx.x == 0) {
        // let this block's copies still in flight land before it leaves: the
        // last NS items issued (bounded)
        volatile int never = 0;
        const int n = *issued;
        for (int q = n - 1; q >= 0 && q >= n - NS; --q)
            mbar_wait_or_abort(&full[q % NS], (unsigned)(q / NS) & 1u, &never);
    }
    return !failed;
}

// Single solver: the level's tiles spread over a persistent grid.
template <int TT, int TJ, int NS, int MZ, bool ZERO, bool PRO>
__global__ void __launch_bounds__(TT * TJ + 32, MZ <= 16 ? kSweepWsBlocks : 2)
    k_sweep_tma_ws(const __grid_constant__ SweepMaps m, LevelView<float> L, LevelView<float> C,
                   int color, Ctl* ctl, Cond cond) {
    pdl_enter();
    if (loop_done(ctl, cond)) return;
    extern __shared__ __align__(128) float sm[];
    __shared__ uint64_t full[NS], empty[NS];
    __shared__ int flags[2];  // abort, items issued
    const Geo& g = L.g;
    const int ntiles = ((g.hx + TT - 1) / TT) * ((g.ny + TJ - 1) / TJ);
    const int count = (int)blockIdx.x < ntiles ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    const TileList tl{(int)blockIdx.x, (int)gridDim.x, count};
    if (!sweep_tiles_ws<TT, TJ, NS, MZ, ZERO, PRO>(&m, L, C, color, tl, sm, full, empty, &flags[0],
                                                     &flags[1]) &&
        threadIdx.x == 0)
        fail_wait(ctl, cond);
}

// Batch: block b runs task b of the plan (consecutive tiles of one
// instance's level); maps[i] are instance i's maps for this level and colour.
template <int TT, int TJ, int NS, int MZ, bool ZERO, bool PRO>
__global__ void __launch_bounds__(TT * TJ + 32, MZ <= 16 ? kSweepWsBlocks : 2)
    kb_sweep_tma_ws(Plan p, const SweepMaps* __restrict__ maps, const LevelView<float>* __restrict__ views,
                    const LevelView<float>* __restrict__ cviews, int color, Ctl* ctl, BCtl* bc, Cond cond) {
    pdl_enter();
    const Task t = p.tasks[blockIdx.x];
    Ctl* c = &ctl[t.inst];
    if (*(volatile const int*)&c->done) return;
    extern __shared__ __align__(128) float sm[];
    __shared__ uint64_t full[NS], empty[NS];
    __shared__ int flags[2];  // abort, items issued
    const LevelView<float> L = views[t.inst];
    const LevelView<float> C = PRO ? cviews[t.inst] : L;
    const TileList tl{(int)t.begin, 1, (int)(t.end - t.begin)};
    if (!sweep_tiles_ws<TT, TJ, NS, MZ, ZERO, PRO>(&maps[t.inst], L, C, color, tl, sm, full, empty, &flags[0],
                                                   &flags[1]) &&
        threadIdx.x == 0) {
        atomicExch(&c->err, 1);
        *(volatile int*)&c->breakdown = 1;
        if (atomicExch(&c->done, 1) == 0 && atomicSub(&bc->active, 1) == 1 && cond.use)
            cudaGraphSetConditional(cond.h, 0u);
    }
}

template <int TT, int TJ, int NS>
constexpr size_t stage_bytes(bool zero_x) {
    return (size_t)NS * (zero_x ? Stage<TT, TJ>::zero : Stage<TT, TJ>::full) * sizeof(float);
}

template <int NS, int MZ, bool ZERO, bool PRO>
void go_ws_ns(cudaStream_t st, const SweepMaps& m, const LevelView<float>& L, const LevelView<float>& C,
              int color, Ctl* ctl, Cond cond) {
    constexpr int TT = kTileT, TJ = kTileJ;
    auto kern = k_sweep_tma_ws<TT, TJ, NS, MZ, ZERO, PRO>;
    static int full_wave = 0;
    if (!full_wave) {
        int dev = 0, sms = 0, per = 0;
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)stage_bytes<TT, TJ, NS>(ZERO));
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, TT * TJ + 32,
                                                          stage_bytes<TT, TJ, NS>(ZERO)) != cudaSuccess ||
            per < 1) {
            cudaGetLastError();
            per = 1;
        }
        full_wave = std::max(1, sms) * per;
    }
    const Geo& g = L.g;
    const int ntiles = ((g.hx + TT - 1) / TT) * ((g.ny + TJ - 1) / TJ);
    const int grid = std::max(1, std::min(ntiles, full_wave));
    launch_pdl(kern, grid, TT * TJ + 32, stage_bytes<TT, TJ, NS>(ZERO), st, m, L, C, color, ctl, cond);
}

template <int MZ, bool ZERO, bool PRO>
void go(cudaStream_t st, const SweepMaps& m, const LevelView<float>& L, const LevelView<float>& C,
        int color, Ctl* ctl, Cond cond) {
    go_ws_ns<kSweepStagesWs, MZ, ZERO, PRO>(st, m, L, C, color, ctl, cond);
}

template <int MZ>
void go_sweep(cudaStream_t st, const SweepMaps& m, const LevelView<float>& L,
              const LevelView<float>* C, int color, bool zero_x, Ctl* ctl, Cond cond) {
    if (zero_x)
        go<MZ, true, false>(st, m, L, L, color, ctl, cond);
    else if (C)
        go<MZ, false, true>(st, m, L, *C, color, ctl, cond);
    else
        go<MZ, false, false>(st, m, L, L, color, ctl, cond);
}

}  // namespace

size_t sweep_tma_smem(bool zero_x) { return stage_bytes<kTileT, kTileJ, kSweepStagesWs>(zero_x); }

bool sweep_tma_fits(const Geo& g) { return g.nz <= 32 && g.hx >= kTileT; }

void launch_sweep_tma(cudaStream_t st, const SweepMaps& m, const LevelView<float>& L,
                      const LevelView<float>* coarse_for_prolong, int color, bool zero_x, Ctl* ctl,
                      Cond cond) {
    const int nz = L.g.nz;
    if (nz <= 8)
        go_sweep<8>(st, m, L, coarse_for_prolong, color, zero_x, ctl, cond);
    else if (nz <= 12)
        go_sweep<12>(st, m, L, coarse_for_prolong, color, zero_x, ctl, cond);
    else if (nz <= 16)
        go_sweep<16>(st, m, L, coarse_for_prolong, color, zero_x, ctl, cond);
    else
        go_sweep<32>(st, m, L, coarse_for_prolong, color, zero_x, ctl, cond);
}

namespace {
template <int MZ, bool ZERO, bool PRO>
void go_b(cudaStream_t st, const Plan& p, const SweepMaps* maps, const LevelView<float>* views,
          const LevelView<float>* cviews, int color, Ctl* ctl, BCtl* bc, Cond cond) {
    constexpr int TT = kTileT, TJ = kTileJ, NW = kSweepStagesWs;
    auto kern = kb_sweep_tma_ws<TT, TJ, NW, MZ, ZERO, PRO>;
    static const bool attr = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                  (int)stage_bytes<TT, TJ, NW>(ZERO)) == cudaSuccess;
    (void)attr;
    launch_pdl(kern, p.ntasks, TT * TJ + 32, stage_bytes<TT, TJ, NW>(ZERO), st, p, maps, views, cviews, color,
               ctl, bc, cond);
}
template <int MZ>
void go_b_sweep(cudaStream_t st, const Plan& p, const SweepMaps* maps, const LevelView<float>* views,
                const LevelView<float>* cviews, int color, bool zero_x, bool prolong, Ctl* ctl,
                BCtl* bc, Cond cond) {
    if (zero_x)
        go_b<MZ, true, false>(st, p, maps, views, cviews, color, ctl, bc, cond);
    else if (prolong)
        go_b<MZ, false, true>(st, p, maps, views, cviews, color, ctl, bc, cond);
    else
        go_b<MZ, false, false>(st, p, maps, views, cviews, color, ctl, bc, cond);
}
}  // namespace

void launch_b_sweep_tma(cudaStream_t st, const Plan& p, const SweepMaps* maps,
                        const LevelView<float>* views, const LevelView<float>* cviews, int color,
                        bool zero_x, bool prolong, int mz, Ctl* ctl, BCtl* bc, Cond cond) {
    if (p.ntasks <= 0) return;
    if (mz <= 8)
        go_b_sweep<8>(st, p, maps, views, cviews, color, zero_x, prolong, ctl, bc, cond);
    else if (mz <= 12)
        go_b_sweep<12>(st, p, maps, views, cviews, color, zero_x, prolong, ctl, bc, cond);
    else if (mz <= 16)
        go_b_sweep<16>(st, p, maps, views, cviews, color, zero_x, prolong, ctl, bc, cond);
    else
        go_b_sweep<32>(st, p, maps, views, cviews, color, zero_x, prolong, ctl, bc, cond);
}

int sweep_tma_tiles(const Geo& g) { return ((g.hx + kTileT - 1) / kTileT) * ((g.ny + kTileJ - 1) / kTileJ); }

// ---- tensor maps -------------------------------------------------------------

namespace {
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                             &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            p = nullptr;
        }
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }();
    return fn;
}
}  // namespace

bool encode_rows_map(CUtensorMap* out, const float* base, int hx, int ny, int nz, unsigned plane,
                     unsigned bx, unsigned by) {
    PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
    if (!fn) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)hx, (cuuint64_t)ny, (cuuint64_t)nz};
    const cuuint64_t strides[2] = {(cuuint64_t)hx * 2u * 4u, (cuuint64_t)plane * 4u};
    const cuuint32_t box[3] = {bx, by, 1u};
    const cuuint32_t estr[3] = {1u, 1u, 1u};
    return fn(out, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), dims, strides, box,
              estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
              CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

bool make_sweep_maps(const LevelView<float>& L, int color, SweepMaps* m, int tile_t, int tile_j) {
    const Geo& g = L.g;
    const int oc = color ^ 1;
    const size_t own = (size_t)color * g.hx, oth = (size_t)oc * g.hx;
    const unsigned T = (unsigned)tile_t, J = (unsigned)tile_j;
    bool ok = true;
    ok = ok && encode_rows_map(&m->b, L.b + own, g.hx, g.ny, g.nz, g.plane, T, J);
    ok = ok && encode_rows_map(&m->fi, L.finv + own, g.hx, g.ny, g.nz, g.plane, T, J);
    ok = ok && encode_rows_map(&m->gu, L.gU + own, g.hx, g.ny, g.nz, g.plane, T, J);
    ok = ok && encode_rows_map(&m->ge, L.gE + own, g.hx, g.ny, g.nz, g.plane, T, J);
    ok = ok && encode_rows_map(&m->gn, L.gN + own, g.hx, g.ny, g.nz, g.plane, T, J);
    ok = ok && encode_rows_map(&m->ox, L.x + oth, g.hx, g.ny, g.nz, g.plane, T + 8, J + 2);
    ok = ok && encode_rows_map(&m->oge, L.gE + oth, g.hx, g.ny, g.nz, g.plane, T + 8, J);
    ok = ok && encode_rows_map(&m->ogn, L.gN + oth, g.hx, g.ny, g.nz, g.plane, T, J + 1);
    return ok;
}

}  // namespace ct
