// k_apply_tma.cu - the double-word operator apply Ap = (A + C/dt) p and p.Ap
// (op_apply, src/operator3d.h:108-112) with its operands staged in shared
// memory by bulk tensor copies (TMA).
//
// Work unit: a tile of 32 slots x 4 rows j, both colours (8 physical rows of
// the split layout), one thread per cell, walking the planes. For each plane
// one thread issues five TMA boxes into one stage of a ring: p with a halo
// of one row j and 4 slots on each side, gE with the slot halo, gN with the
// row below, gU, and the double-word diagonal. A cell's vertical neighbours
// are the same cell in the previous and next planes' stages, so the ring
// keeps three planes of a tile resident and a stage is refilled only after
// the step that reads it as the plane below. The arithmetic and its order
// are apply_compute's (dw_dev.cuh), so Ap equals the row kernel's bit for
// bit; p.Ap is summed in a different order.
//
// Every mbarrier wait is bounded; a wait that runs out sets ctl->err, stops
// the solve, and the block leaves after waiting (bounded) for its copies.
#include <algorithm>
#include <cudaTypedefs.h>

#include "dw_dev.cuh"
#include "kernels.h"
#include "reduce.cuh"
#include "tma.cuh"

namespace ct {

namespace {

using namespace tma;
using namespace dwdev;

constexpr int AT = 32;      // slots per tile
constexpr int AJ = 4;       // rows j per tile (8 physical rows)
constexpr int AR = 2 * AJ;  // physical rows per tile
constexpr int ANS = 6;      // stages
constexpr int AW = AT + 8;  // halo width

// Stage layout (bytes), every box 128-byte aligned.
constexpr int kP = AW * (AR + 4) * 8;  // p: rows 2 j0 - 2 .. 2 (j0 + AJ) + 1
constexpr int kE = AW * AR * 4;        // gE: rows 2 j0 .. 2 (j0 + AJ) - 1
constexpr int kN = AT * (AR + 2) * 4;  // gN: rows 2 j0 - 2 .. 2 (j0 + AJ) - 1
constexpr int kU = AT * AR * 4;        // gU
constexpr int kD = AT * AR * 8;        // dgw
constexpr int kStage = kP + kE + kN + kU + kD;
static_assert(kP % 128 == 0 && kE % 128 == 0 && kN % 128 == 0 && kU % 128 == 0 && kD % 128 == 0,
              "boxes must start on 128-byte boundaries");

__device__ void fail_wait(Ctl* ctl, Cond cond) {
    atomicExch(&ctl->err, 1);
    *(volatile int*)&ctl->breakdown = 1;
    *(volatile int*)&ctl->done = 1;
    if (cond.use) cudaGraphSetConditional(cond.h, 0u);
}

__device__ __forceinline__ void issue(const ApplyMaps& m, unsigned char* sm, uint64_t* full, int w,
                                      int nz, int tilesx) {
    const int s = w % ANS;
    const int mt = w / nz, l = w - mt * nz;
    const int tile = (int)blockIdx.x + mt * (int)gridDim.x;
    const int tyi = tile / tilesx;
    const int t0 = (tile - tyi * tilesx) * AT, r0 = 2 * tyi * AJ;
    unsigned char* st = sm + (size_t)s * kStage;
    uint64_t* bar = &full[s];
    mbar_arrive_expect_tx(bar, (unsigned)kStage);
    load_3d(st, &m.p, t0 - 4, r0 - 2, l, bar);
    load_3d(st + kP, &m.ge, t0 - 4, r0, l, bar);
    load_3d(st + kP + kE, &m.gn, t0, r0 - 2, l, bar);
    load_3d(st + kP + kE + kN, &m.gu, t0, r0, l, bar);
    load_3d(st + kP + kE + kN + kU, &m.dg, t0, r0, l, bar);
}

__global__ void __launch_bounds__(AT * AR)
    k_apply_tma(const __grid_constant__ ApplyMaps m, OpView o, float2* __restrict__ Ap, Ctl* ctl,
                double* part, int maxb, Cond cond) {
    pdl_enter();
    if (loop_done(ctl, cond)) return;
    extern __shared__ __align__(128) unsigned char sm[];
    __shared__ uint64_t full[ANS];
    const Geo& g = o.g;
    const int nz = g.nz;
    const int tilesx = (g.hx + AT - 1) / AT;
    const int ntiles = tilesx * ((g.ny + AJ - 1) / AJ);
    const int my_tiles = (int)blockIdx.x < ntiles ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    const int nitems = my_tiles * nz;
    if (threadIdx.x == 0) {
        for (int s = 0; s < ANS; ++s) mbar_init(&full[s], 1);
        fence_barrier_init();
    }
    __syncthreads();
    if (threadIdx.x == 0)
        for (int w = 0; w < ANS && w < nitems; ++w) issue(m, sm, full, w, nz, tilesx);

    const int tx = (int)threadIdx.x % AT, pr = (int)threadIdx.x / AT;  // slot, physical row in the tile
    const int po = pr ^ 1;                                               // the other colour's row, same j
    DwAcc pap = {0.0f, 0.0f};
    int waited = -1;  // items up to this one have landed
    bool ok = true;
    int w = 0;
    for (int mt = 0; mt < my_tiles && ok; ++mt) {
        const int tile = (int)blockIdx.x + mt * (int)gridDim.x;
        const int tyi = tile / tilesx;
        const int t = (tile - tyi * tilesx) * AT + tx;
        const int r = 2 * tyi * AJ + pr;  // physical row
        const int j = r >> 1, c = r & 1, e = (j + c) & 1;
        const int i = 2 * t + e;
        const bool inrow = j < g.ny && t < g.hx;
        const bool act = inrow && i < g.nx;
        const bool hw = i > 0, he = i < g.nx - 1, hs = j > 0, hn = j < g.ny - 1;
        for (int l = 0; l < nz; ++l, ++w) {
            // this plane and the next one (the up neighbour) must have landed
            const int need = l + 1 < nz ? w + 1 : w;
            bool got = true;
            while (waited < need && got) {
                ++waited;
                got = mbar_wait(&full[waited % ANS], (unsigned)(waited / ANS) & 1u);
            }
            if (act && got) {
                const unsigned char* st = sm + (size_t)(w % ANS) * kStage;
                const float2* P = reinterpret_cast<const float2*>(st);
                const float* GE = reinterpret_cast<const float*>(st + kP);
                const float* GN = reinterpret_cast<const float*>(st + kP + kE);
                const float* GU = reinterpret_cast<const float*>(st + kP + kE + kN);
                const float2* DG = reinterpret_cast<const float2*>(st + kP + kE + kN + kU);
                ApplyCell a;
                const float2 z = make_float2(0.0f, 0.0f);
                a.pc = P[(pr + 2) * AW + tx + 4];
                a.dg = DG[pr * AT + tx];
                a.pw = hw ? P[(po + 2) * AW + tx + 3 + e] : z;
                a.gw = hw ? GE[po * AW + tx + 3 + e] : 0.0f;
                a.pe = he ? P[(po + 2) * AW + tx + 4 + e] : z;
                a.ge = he ? GE[pr * AW + tx + 4] : 0.0f;
                a.ps = hs ? P[po * AW + tx + 4] : z;
                a.gs = hs ? GN[po * AT + tx] : 0.0f;
                a.pn = hn ? P[(po + 4) * AW + tx + 4] : z;
                a.gn = hn ? GN[(pr + 2) * AT + tx] : 0.0f;
                a.gu = GU[pr * AT + tx];
                a.pu = z;
                a.pd = z;
                a.gd = 0.0f;
                if (l > 0) {
                    const unsigned char* sd = sm + (size_t)((w - 1) % ANS) * kStage;
                    a.pd = reinterpret_cast<const float2*>(sd)[(pr + 2) * AW + tx + 4];
                    a.gd = reinterpret_cast<const float*>(sd + kP + kE + kN)[pr * AT + tx];
                }
                if (l + 1 < nz) {
                    const unsigned char* su = sm + (size_t)((w + 1) % ANS) * kStage;
                    a.pu = reinterpret_cast<const float2*>(su)[(pr + 2) * AW + tx + 4];
                }
                Ap[(unsigned)l * g.plane + (unsigned)r * (unsigned)g.hx + (unsigned)t] =
                    apply_compute(a, hw, he, hs, hn, l > 0, l + 1 < nz, pap);
            } else if (inrow && got) {
                Ap[(unsigned)l * g.plane + (unsigned)r * (unsigned)g.hx + (unsigned)t] = make_float2(0.0f, 0.0f);
            }
            // every thread is done with step w: the plane below it (item w - 1)
            // is no longer needed, so its stage takes item w - 1 + ANS
            ok = __syncthreads_and(got) != 0;
            if (!ok) break;
            if (threadIdx.x == 0 && w >= 1 && w - 1 + ANS < nitems) issue(m, sm, full, w - 1 + ANS, nz, tilesx);
        }
    }
    if (!ok) {
        if (threadIdx.x == 0) {
            fail_wait(ctl, cond);
            // let this block's copies still in flight land before it leaves
            const int last = w - 1 + ANS > ANS ? w - 1 + ANS : ANS;  // items issued so far
            const int issued = last < nitems ? last : nitems;
            for (int q = waited; q < issued; ++q) mbar_wait(&full[q % ANS], (unsigned)(q / ANS) & 1u);
        }
        return;
    }
    DwAcc unused = {0.0f, 0.0f};
    block_sum_acc2(pap, unused);
    if (publish_acc2(pap, unused, part, maxb, blockIdx.x, &ctl->ticket[SL_APPLY], gridDim.x)) {
        double PAP, U;
        gather_acc2(part, maxb, 0u, gridDim.x, &ctl->ticket[SL_APPLY], PAP, U);
        if (threadIdx.x == 0) {
            ctl->pAp = PAP;
            if (!(PAP > 0.0) || !isfinite(PAP)) {
                ctl->breakdown = 1;
                ctl->alpha = 0.0;
                stop_loop(ctl, cond);
            } else {
                ctl->alpha = ctl->rz / PAP;
                ctl->alpha_w = dw_of(ctl->alpha);
            }
        }
    }
}

}  // namespace

bool apply_tma_fits(const Geo& g) { return g.hx >= AT; }

int apply_tma_grid(const Geo& g) {
    static int full_wave = 0;
    if (!full_wave) {
        int dev = 0, sms = 0, per = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaFuncSetAttribute(k_apply_tma, cudaFuncAttributeMaxDynamicSharedMemorySize, ANS * kStage);
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_apply_tma, AT * AR, ANS * kStage) !=
                cudaSuccess ||
            per < 1) {
            cudaGetLastError();
            per = 1;
        }
        full_wave = std::max(1, sms) * per;
    }
    const int ntiles = ((g.hx + AT - 1) / AT) * ((g.ny + AJ - 1) / AJ);
    return std::max(1, std::min(ntiles, full_wave));
}

cudaError_t launch_apply_tma(cudaStream_t st, const ApplyMaps& m, const OpView& o, float2* Ap,
                             Ctl* ctl, const Red& red, Cond cond) {
    const int grid = std::min(apply_tma_grid(o.g), red.maxb);
    cudaError_t e = cudaFuncSetAttribute(k_apply_tma, cudaFuncAttributeMaxDynamicSharedMemorySize, ANS * kStage);
    if (e != cudaSuccess) return e;
    launch_pdl(k_apply_tma, grid, AT * AR, (size_t)ANS * kStage, st, m, o, Ap, ctl, red.part, red.maxb, cond);
    return cudaGetLastError();
}

// 3-D maps over both colours' rows (x = slot, y = physical row 2 j + colour,
// z = plane) of the fine arrays.
namespace {
PFN_cuTensorMapEncodeTiled_v12000 encode_fn_apply() {
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

bool encode_all_rows(CUtensorMap* out, const void* base, CUtensorMapDataType dt, unsigned esize,
                     const Geo& g, unsigned bx, unsigned by) {
    PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn_apply();
    if (!fn) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)g.hx, (cuuint64_t)(2 * g.ny), (cuuint64_t)g.nz};
    const cuuint64_t strides[2] = {(cuuint64_t)g.hx * esize, (cuuint64_t)g.plane * esize};
    const cuuint32_t box[3] = {bx, by, 1u};
    const cuuint32_t estr[3] = {1u, 1u, 1u};
    return fn(out, dt, 3, const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
              CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}
}  // namespace

bool make_apply_maps(const OpView& o, const float2* p, const float2* dgw, ApplyMaps* m) {
    const Geo& g = o.g;
    // float2 values are encoded as 64-bit elements (8-byte moves; no arithmetic)
    bool ok = encode_all_rows(&m->p, p, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 8, g, AW, AR + 4);
    ok = ok && encode_all_rows(&m->ge, o.gE, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, g, AW, AR);
    ok = ok && encode_all_rows(&m->gn, o.gN, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, g, AT, AR + 2);
    ok = ok && encode_all_rows(&m->gu, o.gU, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, g, AT, AR);
    ok = ok && encode_all_rows(&m->dg, dgw, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 8, g, AT, AR);
    return ok;
}

}  // namespace ct
