// kernels.h - host-side launchers of the solver kernels (k_outer.cu, k_mg.cu).
// Every launcher enqueues on the given stream and returns without
// synchronising, so the whole iteration can be captured into a CUDA graph.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include "device.h"

namespace ct {

// Fine-level operator as the outer PCG sees it (split layout).
struct OpView {
    Geo g;
    const float *gE, *gN, *gU, *gB, *cap;
};

// Reduction context of one kernel: its slot's partials and grid size.
struct Red {
    double* part;  // 4 * maxb doubles
    int maxb;      // row stride of part
    int blocks;    // grid size (<= maxb)
};

enum MgType { MG_NONE = 0, MG_F32 = 1, MG_F64 = 2 };

// Grid for a grid-stride kernel: one full wave, SMs x resident blocks of
// this kernel (from the occupancy calculator), capped at `cap` blocks.
template <class K>
inline int wave_blocks(K kernel, int cap) {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, NT, 0) != cudaSuccess ||
        per_sm <= 0) {
        cudaGetLastError();
        per_sm = 1;
    }
    const int b = sms * per_sm;
    return b < cap ? b : cap;
}

// Programmatic dependent launch: the solve-loop kernels are launched with
// programmatic stream serialization, so a kernel's launch overlaps the end of
// its predecessor (each block of the predecessor releases it as it exits);
// every such kernel starts with pdl_enter() (wait until the predecessor grid
// has completed and its memory is visible) before it touches memory. Without
// the launch attribute both instructions are no-ops. CT_PDL=0 turns the
// attribute off.
bool pdl_enabled();
__device__ __forceinline__ void pdl_enter() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
}
// Called by a block once its main work is issued (before a reduction's tail,
// a sweep's last stores): the dependent kernel may be scheduled once every
// block has called it or exited, so its launch overlaps this kernel's tail.
// It still waits (pdl_enter) for this whole grid to complete and its memory
// to be visible, so where the call sits changes timing, never results.
#ifndef CT_PDL_TRIGGER
#define CT_PDL_TRIGGER 1
#endif
__device__ __forceinline__ void pdl_trigger() {
#if CT_PDL_TRIGGER
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
#endif
}
template <class... KArgs, class... Args>
inline void launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                       Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl_enabled() ? 1 : 0;
    cudaLaunchKernelEx(&cfg, kern, static_cast<KArgs>(args)...);
}

// ---- outer PCG (FP64), k_outer.cu ----------------------------------------
// r = b - (A + C/dt) x, b0 = r in the V-cycle precision; rr, bb; start test.
void launch_residual(cudaStream_t st, MgType mt, const OpView& o, const double* diag,
                     const double* b, const double* x, double* r, void* b0, Ctl* ctl,
                     const Red& red, Cond cond);
// Ap = (A + C/dt) p; p.Ap; alpha = rz / p.Ap.
void launch_apply(cudaStream_t st, const OpView& o, const double* diag, const double* p,
                  double* Ap, Ctl* ctl, const Red& red, Cond cond);
// x += alpha p, r -= alpha Ap, b0 = r; rr; convergence test (write_x =
// false, FP64 outer loop only: x left to launch_update_x).
void launch_update(cudaStream_t st, MgType mt, unsigned n, const double* p, const double* Ap,
                   double* x, double* r, void* b0, Ctl* ctl, const Red& red, Cond cond, bool write_x = true);
// rz = r.z (and z.Ap for the flexible beta); beta. z = V-cycle result
// (mt = MG_F32 / MG_F64) or r * invd (mt = MG_NONE, Jacobi).
void launch_dot(cudaStream_t st, MgType mt, bool flexible, unsigned n, const double* r,
                const void* z, const double* invd, const double* Ap, Ctl* ctl, const Red& red,
                Cond cond);
// p = z + beta p (p = z on the first iteration).
void launch_update_p(cudaStream_t st, MgType mt, unsigned n, const void* z, const double* r,
                     const double* invd, double* p, Ctl* ctl, Cond cond);

// ---- FP64 outer PCG of the multigrid modes, k_fp64.cu --------------------------
// The same operations for mt = MG_F32 / MG_F64 with the fewest FP64
// instructions (integer float <-> double conversions); the launchers above
// hand the multigrid modes to these.
void launch_residual64(cudaStream_t st, MgType mt, const OpView& o, unsigned n, const double* diag,
                       const double* b, const double* x, double* r, void* b0, Ctl* ctl, const Red& red,
                       Cond cond);
void launch_apply64(cudaStream_t st, const OpView& o, const double* diag, const double* p,
                    double* Ap, Ctl* ctl, const Red& red, Cond cond);
// write_x = false: r only; alpha left in ctl->alpha_x for launch_update_x.
void launch_update64(cudaStream_t st, MgType mt, unsigned n, const double* p, const double* Ap, double* x,
                     double* r, void* b0, Ctl* ctl, const Red& red, Cond cond, bool write_x = true);
// x += ctl->alpha_x p where an update is pending (a plain launch: it runs
// beside other work and is ordered by events, not by programmatic launch), on
// at most `blocks` blocks (0: as many as the vector wants, up to one wave).
void launch_update_x(cudaStream_t st, unsigned n, const double* p, double* x, const Ctl* ctl, int blocks);
void launch_dot64(cudaStream_t st, MgType mt, bool flexible, unsigned n, const double* r, const void* z,
                  const double* Ap, Ctl* ctl, const Red& red, Cond cond);
void launch_update_p64(cudaStream_t st, MgType mt, unsigned n, const void* z, double* p, Ctl* ctl,
                       Cond cond);
// The GPU's DFMA issue rate (instructions per second, independent chains on
// every SM; synchronises the device): the FP64-pipe roofline's denominator.
cudaError_t measure_dfma_rate(double* per_s);
// k_probe.cu: microseconds per phase of `phases` dependent phases on
// SMs x blocks_per_sm blocks (capped at the resident limit), separated by a
// grid barrier inside one cooperative kernel and by dependent launches in a
// graph; gave_up: a barrier wait ran out of polls.
cudaError_t measure_sync_costs(int phases, int blocks_per_sm, double* us_barrier, double* us_launch,
                               int* blocks, int* gave_up);
// Integer conversions against the hardware on n bit patterns (adds the
// mismatch count to *mismatches).
cudaError_t launch_conv_selftest(cudaStream_t st, unsigned long long n, unsigned long long seed,
                                 unsigned long long* mismatches);

// ---- setup and auxiliary kernels, k_outer.cu ------------------------------
void launch_to_split_f(cudaStream_t st, const Geo& g, int planes, const float* nat, float* split);
void launch_to_split_d(cudaStream_t st, const Geo& g, const double* nat, double* split);
void launch_to_natural_d(cudaStream_t st, const Geo& g, const double* split, double* nat);
// diag = op_diag (FP64, no contraction); invd = 1 / diag when invd != null.
// One warp waiting, `limit` polls, on an mbarrier that nothing completes
// (*status: 1 the wait ran out as it must, 2 it completed, 3 no abort flag).
cudaError_t launch_wait_selftest(cudaStream_t st, unsigned limit, int* status);
// The FP64 face sum of the diagonal (once per operator), and the diagonal
// face sum + C/dt (per dt).
void launch_faces(cudaStream_t st, const OpView& o, double* dface);
void launch_diag(cudaStream_t st, const OpView& o, const double* dface, double inv_dt, double* diag,
                 double* invd);
// b = P + cap * inv_dt * x; xold = x.
// *ctl = c on the stream (a queued solve's control block).
void launch_ctl_set(cudaStream_t st, Ctl* ctl, const Ctl& c);
// x (and the double-word correction xw, when not null) = 0 if the solve just
// run found no heat in (ctl->bb_zero); otherwise it does nothing.
void launch_zero_if_no_heat(cudaStream_t st, const Ctl* ctl, unsigned n, double* x, float2* xw);
void launch_rhs_transient(cudaStream_t st, unsigned n, const float* cap, double inv_dt,
                          const double* P, const double* x, double* b, double* xold);
// ctl->aux0 = ||P - A x||^2, aux1 = ||P||^2 (steady operator, FP64).
void launch_true_residual(cudaStream_t st, const OpView& o, const double* P, const double* x,
                          Ctl* ctl, const Red& red);
// ctl->aux0 = T_max, aux1 = heat out, aux2 = sum cap (x - xold).
void launch_step_record(cudaStream_t st, const OpView& o, const double* x, const double* xold,
                        Ctl* ctl, const Red& red);
// One entry of the device table of queued step records.
struct StepEntry {
    double T_max, q_out, q_stored, relres;
    int iters, converged, breakdown, err;
};
void launch_record_keep(cudaStream_t st, const Ctl* ctl, double dt, StepEntry* table, int slot);

// ---- double-word outer PCG (FP32 pipes), k_dw.cu -----------------------------
// r = b - A x in FP64 from the double-word x; start of a solve, or the residual
// replacement that begins phase 2.
void launch_residual_x(cudaStream_t st, const OpView& o, const double* diag, const double* b,
                       const double* x, float2* r, float* b0, bool start, Ctl* ctl,
                       const Red& red, Cond cond);
// xb += xw in FP64, xw = 0 (skipped once the solve is done when check_done).
void launch_fold(cudaStream_t st, unsigned n, double* xb, float2* xw, const Ctl* ctl,
                 bool check_done);
void launch_apply_dw(cudaStream_t st, const OpView& o, const float2* dgw, const float2* p,
                     float2* Ap, Ctl* ctl, const Red& red, Cond cond);
void launch_update_dw(cudaStream_t st, unsigned n, const float2* p, const float2* Ap, float2* x,
                      float2* r, float* b0, Ctl* ctl, const Red& red, Cond cond);
void launch_dot_dw(cudaStream_t st, unsigned n, const float2* r, const float* z, const float2* Ap,
                   Ctl* ctl, const Red& red, Cond cond);
void launch_update_p_dw(cudaStream_t st, unsigned n, const float* z, float2* p, Ctl* ctl,
                        Cond cond);
void launch_to_dw(cudaStream_t st, unsigned n, const double* in, float2* out);
void launch_dw_to_natural(cudaStream_t st, const Geo& g, const float2* split, double* nat);
void launch_natural_to_dw(cudaStream_t st, const Geo& g, const double* nat, float2* split);
void launch_dw_to_d(cudaStream_t st, unsigned n, const float2* in, double* out);

// ---- multigrid, k_mg.cu ---------------------------------------------------
// Coarse level from the fine one (mg_coarse_cell arithmetic, split layouts).
void launch_coarsen(cudaStream_t st, const Geo& fg, const float* fgE, const float* fgN,
                    const float* fgU, const float* fgB, const float* fcap, const double* fdx,
                    const double* fdy, const Geo& cg, const double* cdx, const double* cdy,
                    float* cgE, float* cgN, float* cgU, float* cgB, float* ccap);
// Column factors of one level for 1/dt (mg_factor_column arithmetic).
template <class T>
void launch_factor(cudaStream_t st, const LevelView<T>& L, T inv_dt);
// One red-black sweep. zero_x: x = 0 before the sweep (the first sweep of a
// V-cycle), so lateral neighbours are not read. xc: when not null, the
// coarser level's x is added to every neighbour value read (prolongation
// fused into the sweep).
// Fine levels of more than this many columns restrict by pairs of planes
// (k_restrict2), smaller ones by single planes (k_restrict).
constexpr unsigned kSweepBfColumns = 128u * 128u;
// Levels of at most this many columns sweep with one thread per column and
// plane (k_sweep_split); larger FP32 levels are staged by bulk tensor copies
// (at 800 x 800: the 200 x 200 level split 6.96 ms per solve against 7.07 ms
// staged, the 400 x 400 level split 7.11 ms).
constexpr unsigned kSweepSplitColumns = 256u * 256u;
// FP64 levels (the plain FP64 MG-PCG) are never staged and sweep this way at
// every size (800 x 800: 56.6 solves/s, against 52.4 with the one-thread-per-
// column sweep above 512 x 512 columns and 50.7 above 256 x 256).
constexpr unsigned kSweepSplitColumns64 = 0xffffffffu;
template <class T>
void launch_sweep(cudaStream_t st, const LevelView<T>& L, int color, bool zero_x,
                  const LevelView<T>* coarse_for_prolong, const Ctl* ctl, Cond cond);
// The same sweep for the large FP32 levels, operands staged in shared memory
// by bulk tensor copies (k_sweep_tma.cu). Tiles of kTileT x kTileJ columns,
// one thread per column; the tensor maps cover one colour's rows of each
// array (make_sweep_maps, built once per level and colour at set-up).
constexpr int kTileT = 32;  // slots per tile row
constexpr int kTileJ = 8;   // rows per tile
constexpr int kTileThreads = kTileT * kTileJ;
constexpr int kSweepStagesWs = 6;  // planes in flight per block (a producer warp, no block barrier per plane)
constexpr int kSweepWsBlocks = 3;  // resident blocks per SM the producer-warp sweeps are compiled for
struct SweepMaps {
    CUtensorMap b, fi, gu, ge, gn;      // the sweep colour's rows, box kTileT x kTileJ
    CUtensorMap ox;                     // other colour's x, box (kTileT + 8) x (kTileJ + 2)
    CUtensorMap oge;                    // other colour's gE, box (kTileT + 8) x kTileJ
    CUtensorMap ogn;                    // other colour's gN, box kTileT x (kTileJ + 1)
};
bool sweep_tma_fits(const Geo& g);  // nz <= 32 and at least one full tile row
size_t sweep_tma_smem(bool zero_x);
bool make_sweep_maps(const LevelView<float>& L, int color, SweepMaps* m, int tile_t = kTileT,
                     int tile_j = kTileJ);
void launch_sweep_tma(cudaStream_t st, const SweepMaps& m, const LevelView<float>& L,
                      const LevelView<float>* coarse_for_prolong, int color, bool zero_x, Ctl* ctl,
                      Cond cond);
// coarse b = sum over the children of (b - (A + C/dt) x).
template <class T>
void launch_restrict(cudaStream_t st, const LevelView<T>& F, const LevelView<T>& C, const Ctl* ctl,
                     Cond cond);

// The restriction F -> C fused with C's first sweep (x = 0, red columns).
// false (nothing launched) for columns deeper than 32 planes.
template <class T>
bool launch_restrict_sweep0(cudaStream_t st, const LevelView<T>& F, const LevelView<T>& C, const Ctl* ctl,
                            Cond cond);

// The levels from some level down to the single column, finest first.
constexpr int kMaxTail = 24;
// Every level of a hierarchy (at most kMaxTail) with the first index of each
// level's columns when they are laid end to end (first[n] = all columns).
template <class T>
struct FactorLevels {
    int n;
    unsigned first[kMaxTail + 1];
    LevelView<T> L[kMaxTail];
};
// set_dt in one launch: every level's column factors for 1/dt and, when diag
// is not null, the fine operator's FP64 diagonal (and 1/d, the double-word
// copy where invd, dgw are not null); the same bits as launch_factor per
// level and launch_diag (+ the double-word copy).
template <class T>
void launch_factor_levels(cudaStream_t st, const FactorLevels<T>& fl, T inv_dt, const OpView& o,
                          const double* dface, double inv_dt64, double* diag, double* invd, float2* dgw);
template <class T>
struct TailLevels {
    int n;  // levels in L, the finest of them first, the single column last
    LevelView<T> L[kMaxTail];
};
// The smallest levels (those whose arrays together fit kSmallSmemMax bytes),
// run by one block out of shared memory.
constexpr int kSmallThreads = 512;        // the bottom kernel's launch bound (and the batch's blocks)
constexpr int kSmallThreadsSolver = 256;  // the single solver's bottom block
constexpr int kSmallSmemMax = 200 * 1024;
// Bytes one level takes there: gE, gN, gU, cap (float), gB (one plane of
// float), fcp, finv, x, b (elem bytes each), every array rounded up to 16
// bytes. The device carving of the block's shared memory, its size at launch
// and the choice of the first level held there all use this one sum.
__host__ __device__ inline size_t small_round16(size_t b) { return (b + 15) & ~size_t(15); }
__host__ __device__ inline size_t small_level_bytes(const Geo& g, size_t elem) {
    const size_t ln = (size_t)g.plane * (size_t)g.nz;
    return 4 * small_round16(ln * 4) + small_round16((size_t)g.plane * 4) + 4 * small_round16(ln * elem);
}
template <class T>
size_t small_smem_bytes(const TailLevels<T>& tl);
template <class T>
cudaError_t launch_vsmall(cudaStream_t st, const TailLevels<T>& tl, Ctl* ctl, Cond cond);

}  // namespace ct
