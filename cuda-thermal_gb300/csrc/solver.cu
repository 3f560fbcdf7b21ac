// solver.cu - the solver object behind ct_solver_* (GpuPcg, src/pcg3d.h:115-163).
//
// Memory: one device allocation per solver (an arena), carved into the fine
// operator, the FP64 PCG vectors, every multigrid level and the reduction
// scratch, all in the split layout (device.h), zeroed once so padding slots
// stay zero. One CUDA stream per solver.
//
// Control flow of a solve: the host writes tol / maxit into the control block
// and launches ONE CUDA graph: the start residual, then a conditional WHILE
// node whose body is one PCG iteration rotated so that it ends with the
// convergence test,
//     V-cycle(r) -> z;  beta;  p = z + beta p;  Ap, alpha;  x, r update, test
// The kernel that finishes the test clears the loop condition, and once the
// solve is done every later kernel of the body returns at entry. alpha, beta
// and the dot products never leave the device; the host reads the control
// block once at the end. Where conditional nodes are unavailable the same two
// parts are replayed as plain graphs with a host check every few iterations,
// and with ct_use_graphs(0) every kernel is launched directly with a host
// check per iteration, as the reference does (src/pcg3d_gpu.cu:672-680).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <type_traits>
#include <vector>

#include "trace.h"
#include "cthermal.h"
#include "kernels.h"
#include "solver.h"
#include "status.h"

namespace ct {

namespace {

bool g_use_graphs = true;
std::mutex g_setup_mu;
ct_setup_times g_last_setup{};

using clk = std::chrono::steady_clock;
double ms_since(clk::time_point t) {
    return std::chrono::duration<double, std::milli>(clk::now() - t).count();
}

#define CT_CK(call)                                                                              \
    do {                                                                                         \
        const cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess)                                                                   \
            return ct::fail(e_ == cudaErrorMemoryAllocation ? CT_OUT_OF_MEMORY : CT_CUDA_ERROR,  \
                            "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
    } while (0)

}  // namespace

// ---- setup ---------------------------------------------------------------

ct_status Solver::create(const ct_model* m_in, ct_precond pc_, ct_precision prec_, const DeviceBuild* build) {
    const TraceRange trace("ct_solver_create");
    ct_model geo{};  // the geometry when the model is built on the device
    if (build) {
        geo.nx = build->nx;
        geo.ny = build->ny;
        geo.nz = build->nz;
        geo.dx = build->dx;
        geo.dy = build->dy;
    }
    const ct_model* m = build ? &geo : m_in;
    if (!m) return fail(CT_BAD_ARG, "ct_solver_create: null model");
    if (m->nx < 1 || m->ny < 1 || m->nz < 1 || m->nz > CT_MAXZ)
        return fail(CT_BAD_ARG, "ct_solver_create: bad size %d x %d x %d (nz must be 1..%d)", m->nx,
                    m->ny, m->nz, CT_MAXZ);
    if (!build && (!m->gE || !m->gN || !m->gU || !m->gB || !m->cap))
        return fail(CT_NOT_FINALIZED, "Model3D used before finalize()");
    if (!build && !m->P) return fail(CT_BAD_ARG, "ct_solver_create: null power map");
    if (!(m->dx > 0) || !(m->dy > 0)) return fail(CT_BAD_ARG, "ct_solver_create: dx, dy must be > 0");
    if (pc_ != CT_JACOBI && pc_ != CT_MULTIGRID) return fail(CT_BAD_ARG, "bad preconditioner");
    if (prec_ != CT_MG_FP64 && prec_ != CT_MG_FP32 && prec_ != CT_MG_FP32_FLEX &&
        prec_ != CT_MG_FP32_FLEX_DW)
        return fail(CT_BAD_ARG, "bad precision");
    pc = pc_;
    prec = prec_;
    mt = pc == CT_JACOBI ? MG_NONE : (prec == CT_MG_FP64 ? MG_F64 : MG_F32);
    flex = pc == CT_MULTIGRID && (prec == CT_MG_FP32_FLEX || prec == CT_MG_FP32_FLEX_DW);
    dw = pc == CT_MULTIGRID && prec == CT_MG_FP32_FLEX_DW;
    if (const char* e = std::getenv("CT_RR_THRESHOLD")) rr_thr = std::atof(e);
    tsize = mt == MG_F64 ? 8 : 4;
    g0 = geo_of(m->nx, m->ny, m->nz);
    const double slots = (double)g0.plane * g0.nz;
    if (slots > 2.0e9) return fail(CT_BAD_ARG, "model too large for one solver (%.0f cells)", slots);
    n = g0.plane * (unsigned)g0.nz;
    ncells = (size_t)m->nx * m->ny * m->nz;
    dx = m->dx;
    dy = m->dy;
    use_graphs = g_use_graphs;

    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(CT_NO_DEVICE, "no CUDA device");
    }
    int dev = 0;
    CT_CK(cudaGetDevice(&dev));
    CT_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    maxb = std::max(1, sms * (2048 / NT));

    auto t0 = clk::now();
    if (st)
        own_stream = false;  // a batch's stream
    else
        CT_CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    if (!skip_graphs) {
        CT_CK(cudaStreamCreateWithFlags(&st_body, cudaStreamNonBlocking));
        CT_CK(cudaStreamCreateWithFlags(&st_side, cudaStreamNonBlocking));
        CT_CK(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
        CT_CK(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming));
    }
    cs = st;
    CT_CK(cudaMallocHost(&h_ctl, sizeof(Ctl)));
    std::memset(h_ctl, 0, sizeof(Ctl));

    // Level sizes (src/mg3d.h:159-181) and the arena layout.
    Arena ar;
    const size_t o_gE = ar.take(n * 4), o_gN = ar.take(n * 4), o_gU = ar.take(n * 4);
    const size_t o_cap = ar.take(n * 4), o_gB = ar.take((size_t)g0.plane * 4);
    size_t o_vec[9];
    for (size_t& o : o_vec) o = ar.take((size_t)n * 8);
    const size_t o_invd = pc == CT_JACOBI ? ar.take((size_t)n * 8) : 0;
    const size_t o_dgw = dw ? ar.take((size_t)n * 8) : 0;
    const size_t o_xwc = dw ? ar.take((size_t)n * 8) : 0;
    const size_t o_nat = ar.take(ncells * 8);
    const size_t o_part = ar.take((size_t)NSLOT * 4 * maxb * 8);
    const size_t o_ctl = ar.take(sizeof(Ctl));
    if (pc == CT_MULTIGRID) {
        Level L;
        L.g = g0;
        L.dx.assign(m->nx, m->dx);
        L.dy.assign(m->ny, m->dy);
        while (true) {
            const size_t ln = (size_t)L.g.plane * L.g.nz;
            if (lv.empty()) {  // level 0 shares the fine operator
                L.o_gE = o_gE;
                L.o_gN = o_gN;
                L.o_gU = o_gU;
                L.o_cap = o_cap;
                L.o_gB = o_gB;
            } else {
                L.o_gE = ar.take(ln * 4);
                L.o_gN = ar.take(ln * 4);
                L.o_gU = ar.take(ln * 4);
                L.o_cap = ar.take(ln * 4);
                L.o_gB = ar.take((size_t)L.g.plane * 4);
            }
            L.o_fcp = ar.take(ln * tsize);
            L.o_finv = ar.take(ln * tsize);
            L.o_x = ar.take(ln * tsize);
            L.o_b = ar.take(ln * tsize);
            L.o_dx = ar.take(L.dx.size() * 8);
            L.o_dy = ar.take(L.dy.size() * 8);
            lv.push_back(L);
            if (L.g.nx == 1 && L.g.ny == 1) break;
            Level C;
            C.g = geo_of((L.g.nx + 1) / 2, (L.g.ny + 1) / 2, L.g.nz);
            C.dx = coarse_widths(L.dx);
            C.dy = coarse_widths(L.dy);
            L = C;
        }
    }
    {
        // The smallest levels whose arrays fit one block's shared memory.
        small_k0 = lv.size();
        // CT_SMALL_BYTES lowers the budget (a diagnostics knob); it can never
        // exceed what one block may hold on this device
        int optin = 0;
        CT_CK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
        long small_max = std::min<long>(kSmallSmemMax, optin);
        if (const char* e = std::getenv("CT_SMALL_BYTES")) {
            char* end = nullptr;
            const long v = std::strtol(e, &end, 10);
            if (end == e || *end != '\0' || v < 0)
                return fail(CT_BAD_ARG, "CT_SMALL_BYTES=%s is not a byte count", e);
            small_max = std::min(small_max, v);
        }
        size_t acc = 0;
        for (size_t k = lv.size(); k-- > 0;) {
            acc += small_level_bytes(lv[k].g, tsize);
            if ((long)acc > small_max || lv.size() - k > (size_t)kMaxTail) break;
            small_k0 = k;
        }
    }
    bytes = ar.used;
    {
        const cudaError_t e = cudaMalloc(&base, bytes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            base = nullptr;
            return fail(CT_OUT_OF_MEMORY, "cudaMalloc of %.1f MB failed: %s", bytes / 1e6,
                        cudaGetErrorString(e));
        }
    }
    CT_CK(cudaMemsetAsync(base, 0, bytes, st));
    gE = at<float>(o_gE);
    gN = at<float>(o_gN);
    gU = at<float>(o_gU);
    cap = at<float>(o_cap);
    gB = at<float>(o_gB);
    P = at<double>(o_vec[0]);
    x = at<double>(o_vec[1]);
    b = at<double>(o_vec[2]);
    r = at<double>(o_vec[3]);
    p = at<double>(o_vec[4]);
    Ap = at<double>(o_vec[5]);
    diag = at<double>(o_vec[6]);
    xold = at<double>(o_vec[7]);
    dface = at<double>(o_vec[8]);
    invd = pc == CT_JACOBI ? at<double>(o_invd) : nullptr;
    dgw = dw ? at<float2>(o_dgw) : nullptr;
    xwc = dw ? at<float2>(o_xwc) : nullptr;
    nat = at<double>(o_nat);
    part = at<double>(o_part);
    ctl = at<Ctl>(o_ctl);
    CT_CK(cudaStreamSynchronize(st));
    times.alloc_ms = ms_since(t0);

    // CT_FUSE_SWEEP0=0 keeps each level's first sweep a launch of its own
    // instead of riding along with the restriction into that level.
    if (const char* e = std::getenv("CT_FUSE_SWEEP0")) fuse_sweep0 = e[0] != '0';
    // The x = 0 sweeps of the staged levels run on the grid kernel: with no
    // neighbour values to share there is nothing to stage, and one thread per
    // column with every plane's loads in flight at once moves the level's
    // three operand streams faster than the tile ring (800 x 800 x 10 FLEX
    // solve 6.52 -> 6.46 ms). CT_SWEEP0_GRID=0 stages them too.
    if (const char* e = std::getenv("CT_SWEEP0_GRID")) sweep0_grid = e[0] != '0';
    // x += alpha p leaves the update (which then moves 24 B a cell fewer on
    // the iteration's critical path) for a launch of a few blocks beside the
    // next V-cycle, forked after the restriction out of level 1: it streams x
    // and p while the coarse levels, latency-bound, leave the memory system
    // idle (800 x 800 FLEX solve 155.3 -> 157.8 solves/s at 64 blocks; 16 /
    // 32 / 128 / 192 blocks: 145.7 / 155.4 / 157.6 / 156.8; forked after
    // level 0's restriction: 156.3; the whole grid at once: 154.3).
    // CT_XLAG = k forks after level k's restriction instead, -1 keeps x in
    // the update; CT_XLAG_BLOCKS sets the blocks.
    if (const char* e = std::getenv("CT_XLAG")) xlag = std::atoi(e);
    xlag_blocks = std::max(1, sms * 64 / 152);
    if (const char* e = std::getenv("CT_XLAG_BLOCKS")) xlag_blocks = std::max(1, std::atoi(e));
    // Tensor maps of the levels whose sweeps are staged by bulk tensor copies
    // (FP32 levels with at least one full tile row, above the shared-memory
    // levels); CT_SWEEP_TMA=0 keeps every level on the grid kernels. Levels of
    // at most kSweepSplitColumns columns stay on the grid kernel too: they sit
    // in L2, and a tile pipeline of a few tiles per block costs more latency
    // than one thread per column and plane (CT_SWEEP_TMA_COLS sets the
    // smallest staged level instead).
    {
        const char* e = std::getenv("CT_SWEEP_TMA");
        const bool want = mt == MG_F32 && !(e && e[0] == '0');
        long min_cols = (long)kSweepSplitColumns + 1;
        if (const char* c = std::getenv("CT_SWEEP_TMA_COLS")) min_cols = std::atol(c);
        for (size_t k = 0; want && k < lv.size() && k < small_k0; ++k) {
            Level& L = lv[k];
            if (!sweep_tma_fits(L.g) || (long)L.g.nx * L.g.ny < min_cols) continue;
            const LevelView<float> v = view<float>(k);
            L.tma = make_sweep_maps(v, 0, &L.maps[0]) && make_sweep_maps(v, 1, &L.maps[1]);
        }
    }

    // Upload the fine operator and P through the natural staging buffer, or
    // build them on the device (TSV fractions in r, power in the staging
    // buffer, both natural-layout scratch at this point).
    t0 = clk::now();
    if (build) {
        CT_CK(launch_build(st, *build, g0, r, nat, gE, gN, gU, gB, cap));
        launch_to_split_d(st, g0, nat, P);
    } else {
        float* natf = reinterpret_cast<float*>(nat);
        const float* src[4] = {m->gE, m->gN, m->gU, m->cap};
        float* dst[4] = {gE, gN, gU, cap};
        for (int a = 0; a < 4; ++a) {
            CT_CK(cudaMemcpyAsync(natf, src[a], ncells * 4, cudaMemcpyHostToDevice, st));
            launch_to_split_f(st, g0, g0.nz, natf, dst[a]);
        }
        CT_CK(cudaMemcpyAsync(natf, m->gB, (size_t)m->nx * m->ny * 4, cudaMemcpyHostToDevice, st));
        launch_to_split_f(st, g0, 1, natf, gB);
        CT_CK(cudaMemcpyAsync(nat, m->P, ncells * 8, cudaMemcpyHostToDevice, st));
        launch_to_split_d(st, g0, nat, P);
    }
    for (Level& L : lv) {
        CT_CK(cudaMemcpyAsync(base + L.o_dx, L.dx.data(), L.dx.size() * 8, cudaMemcpyHostToDevice, st));
        CT_CK(cudaMemcpyAsync(base + L.o_dy, L.dy.data(), L.dy.size() * 8, cudaMemcpyHostToDevice, st));
    }
    CT_CK(cudaGetLastError());
    CT_CK(cudaStreamSynchronize(st));
    times.upload_ms = ms_since(t0);

    // Coarse levels, built on the device from the next finer one.
    t0 = clk::now();
    for (size_t k = 1; k < lv.size(); ++k) {
        const Level& F = lv[k - 1];
        const Level& C = lv[k];
        launch_coarsen(st, F.g, at<float>(F.o_gE), at<float>(F.o_gN), at<float>(F.o_gU),
                       at<float>(F.o_gB), at<float>(F.o_cap), at<double>(F.o_dx),
                       at<double>(F.o_dy), C.g, at<double>(C.o_dx), at<double>(C.o_dy),
                       at<float>(C.o_gE), at<float>(C.o_gN), at<float>(C.o_gU), at<float>(C.o_gB),
                       at<float>(C.o_cap));
    }
    CT_CK(cudaGetLastError());
    CT_CK(cudaStreamSynchronize(st));
    times.levels_ms = ms_since(t0);

    t0 = clk::now();
    launch_faces(st, op(), dface);
    ct_status s = set_dt(0.0);
    if (s != CT_OK) return s;
    CT_CK(cudaStreamSynchronize(st));
    times.factor_ms = ms_since(t0);

    t0 = clk::now();
    if (use_graphs && !skip_graphs) {
        s = record_graphs();
        if (s != CT_OK) return s;
    }
    CT_CK(cudaStreamSynchronize(st));
    times.graphs_ms = ms_since(t0);
    {
        std::lock_guard<std::mutex> lk(g_setup_mu);
        g_last_setup = times;
    }
    return CT_OK;
}

ct_status Solver::set_dt(double dt) {
    const TraceRange trace("ct_set_dt");
    if (!(dt >= 0) || !std::isfinite(dt)) return fail(CT_BAD_ARG, "ct_set_dt: dt must be >= 0");
    inv_dt = dt > 0 ? 1.0 / dt : 0.0;
    // one launch for the diagonal and every level's factors (CT_FACTOR_LEVELS=0:
    // a launch for the diagonal and one per level)
    const char* fl_env = std::getenv("CT_FACTOR_LEVELS");
    const bool one_launch = !(fl_env && fl_env[0] == '0');
    if (one_launch && mt != MG_NONE && lv.size() <= (size_t)kMaxTail) {
        if (mt == MG_F32)
            launch_factor_levels<float>(st, factor_levels<float>(), (float)inv_dt, op(), dface, inv_dt, diag, invd,
                                        dw ? dgw : nullptr);
        else
            launch_factor_levels<double>(st, factor_levels<double>(), inv_dt, op(), dface, inv_dt, diag, invd,
                                         nullptr);
    } else {
        launch_diag(st, op(), dface, inv_dt, diag, invd);
        if (dw) launch_to_dw(st, n, diag, dgw);
        if (mt == MG_F32)
            for (size_t k = 0; k < lv.size(); ++k) launch_factor<float>(st, view<float>(k), (float)inv_dt);
        else if (mt == MG_F64)
            for (size_t k = 0; k < lv.size(); ++k) launch_factor<double>(st, view<double>(k), inv_dt);
    }
    CT_CK(cudaGetLastError());
    return CT_OK;
}

// ---- one PCG iteration ----------------------------------------------------

template <class T>
void Solver::sweep(size_t k, const LevelView<T>& L, int color, bool zero_x, const LevelView<T>* coarse,
                   Cond cond) {
    if constexpr (std::is_same<T, float>::value) {
        if (lv[k].tma && !(zero_x && sweep0_grid)) {
            launch_sweep_tma(cs, lv[k].maps[color], L, coarse, color, zero_x, ctl, cond);
            return;
        }
    }
    launch_sweep<T>(cs, L, color, zero_x, coarse, ctl, cond);
}

template <class T>
void Solver::vcycle(size_t k, Cond cond, bool first_sweep_done) {
    if (k == small_k0) {
        TailLevels<T> tl;
        tl.n = (int)(lv.size() - k);
        double b = 0;
        for (int q = 0; q < tl.n; ++q) {
            tl.L[q] = view<T>(k + q);
            const Geo& g = tl.L[q].g;
            b += (double)g.nx * g.ny * g.nz * (4 * sizeof(T) + 4 + 2 * sizeof(T) + 16);
        }
        enq(("mg_small_l" + std::to_string(k)).c_str(), b, [&] {
            const cudaError_t e = launch_vsmall<T>(cs, tl, ctl, cond);
            if (e != cudaSuccess && launch_error == cudaSuccess) launch_error = e;
        });
        return;
    }
    const LevelView<T> L = view<T>(k);
    const double cells = (double)L.g.nx * L.g.ny * L.g.nz;
    const double t = (double)sizeof(T);
    const std::string lvl = "_l" + std::to_string(k);
    // algorithmic bytes: each array touched once per kernel
    const double b_zero = cells / 2 * (4 * t + 4);
    const double b_sweep = cells / 2 * (4 * t + 12) + cells / 2 * (t + 8);
    if (k + 1 == lv.size()) {
        if (!first_sweep_done)
            enq(("mg_sweep0" + lvl).c_str(), b_zero, [&] { sweep<T>(k, L, 0, true, nullptr, cond); });
        return;
    }
    const LevelView<T> C = view<T>(k + 1);
    if (!first_sweep_done)
        enq(("mg_sweep0" + lvl).c_str(), b_zero, [&] { sweep<T>(k, L, 0, true, nullptr, cond); });
    enq(("mg_sweep" + lvl).c_str(), b_sweep, [&] { sweep<T>(k, L, 1, false, nullptr, cond); });
    // The coarse level's first sweep rides along with the restriction unless
    // the shared-memory bottom starts there,
    // or the restriction is from the finest level: there it is bandwidth
    // bound, and the block's serial line-solve tail costs more (measured at
    // 800 x 800: 78 us fused against 51 + 13 us) than the launch it saves.
    const bool fuse = fuse_sweep0 && k > 0 && k + 1 != small_k0 && L.g.nz <= 32;
    const double b_restrict = cells * (2 * t + 16) + cells / 4 * t;
    const double cc = (double)C.g.nx * C.g.ny * C.g.nz;
    if (fuse)
        enq(("mg_restrict_sweep0" + lvl).c_str(), b_restrict + cc / 2 * (3 * t + 4),
            [&] { launch_restrict_sweep0<T>(cs, L, C, ctl, cond); });
    else
        enq(("mg_restrict" + lvl).c_str(), b_restrict, [&] { launch_restrict<T>(cs, L, C, ctl, cond); });
    if (lag_now && (int)k == fork_level()) fork_x();
    vcycle<T>(k + 1, cond, fuse);
    enq(("mg_sweep" + lvl).c_str(), b_sweep + cells / 4 * t,
        [&] { sweep<T>(k, L, 1, false, &C, cond); });
    enq(("mg_sweep" + lvl).c_str(), b_sweep, [&] { sweep<T>(k, L, 0, false, nullptr, cond); });
}

void Solver::enqueue_init(Cond cond) {
    void* b0 = mt == MG_NONE ? nullptr : (void*)(base + lv[0].o_b);
    if (dw) {
        enq("pcg_fold_x", (double)ncells * 32, [&] { launch_fold(cs, n, x, xwc, ctl, false); });
        enq("pcg_residual_fp64", (double)ncells * (36 + 8 + 8 + 4), [&] {
            launch_residual_x(cs, op(), diag, b, x, rw(), (float*)b0, true, ctl,
                              red_cols(SL_INIT), cond);
        });
        return;
    }
    enq("pcg_residual", (double)ncells * (36 + 8 + 8 + tsize), [&] {
        launch_residual(cs, mt, op(), diag, b, x, r, b0, ctl, red_cols(SL_INIT), cond);
    });
}

void Solver::enqueue_replace(Cond cond) {
    float* b0 = at<float>(lv[0].o_b);
    enq("pcg_fold_x", (double)ncells * 32, [&] { launch_fold(cs, n, x, xwc, ctl, true); });
    enq("pcg_residual_fp64", (double)ncells * (36 + 8 + 8 + 4), [&] {
        launch_residual_x(cs, op(), diag, b, x, rw(), b0, false, ctl, red_cols(SL_INIT), cond);
    });
}

void Solver::enqueue_body(Cond cond) {
    const double N = (double)ncells;
    const void* z = nullptr;
    if (dw) {
        vcycle<float>(0, cond);
        const float* zf = at<float>(lv[0].o_x);
        float* b0 = at<float>(lv[0].o_b);
        enq("pcg_dot", N * (8 + 4 + 8),
            [&] { launch_dot_dw(cs, n, rw(), zf, Apw(), ctl, red_vec(SL_DOT), cond); });
        enq("pcg_update_p", N * (4 + 16), [&] { launch_update_p_dw(cs, n, zf, pw(), ctl, cond); });
        enq("pcg_apply", N * 36,
            [&] { launch_apply_dw(cs, op(), dgw, pw(), Apw(), ctl, red_cols(SL_APPLY), cond); });
        enq("pcg_update_xr", N * (48 + 4), [&] {
            launch_update_dw(cs, n, pw(), Apw(), xw(), rw(), b0, ctl, red_vec(SL_UPDATE), cond);
        });
        return;
    }
    // x += alpha p of the previous iteration beside this V-cycle (x_lag())
    lag_now = x_lag();
    forked = false;
    if (lag_now && fork_level() >= (int)lv.size()) fork_x();
    if (mt == MG_F32) {
        vcycle<float>(0, cond);
        z = base + lv[0].o_x;
    } else if (mt == MG_F64) {
        vcycle<double>(0, cond);
        z = base + lv[0].o_x;
    }
    if (lag_now && !forked) fork_x();
    const double zb = mt == MG_NONE ? 16.0 : (double)tsize;
    enq("pcg_dot", N * (8 + zb + (flex ? 8 : 0)),
        [&] { launch_dot(cs, mt, flex, n, r, z, invd, Ap, ctl, red_vec(SL_DOT), cond); });
    // the p update overwrites the p that the x update reads: join first
    if (lag_now && !prof) cudaStreamWaitEvent(cs, ev_join, 0);
    enq("pcg_update_p", N * (zb + 16), [&] { launch_update_p(cs, mt, n, z, r, invd, p, ctl, cond); });
    enq("pcg_apply", N * 36, [&] { launch_apply(cs, op(), diag, p, Ap, ctl, red_cols(SL_APPLY), cond); });
    void* b0 = mt == MG_NONE ? nullptr : (void*)(base + lv[0].o_b);
    enq("pcg_update_xr", N * ((lag_now ? 24 : 48) + (mt == MG_NONE ? 0 : tsize)),
        [&] { launch_update(cs, mt, n, p, Ap, x, r, b0, ctl, red_vec(SL_UPDATE), cond, !lag_now); });
    lag_now = false;
}

void Solver::fork_x() {
    forked = true;
    if (prof) {  // timed in line, on as many blocks as it wants
        enq("pcg_update_x", (double)ncells * 24, [&] { launch_update_x(cs, n, p, x, ctl, 0); });
        return;
    }
    cudaEventRecord(ev_fork, cs);
    cudaStreamWaitEvent(st_side, ev_fork, 0);
    launch_update_x(st_side, n, p, x, ctl, xlag_blocks);
    cudaEventRecord(ev_join, st_side);
}

ct_status Solver::record_graphs() {
    launch_error = cudaSuccess;
    // Preferred: one graph per solve: the start residual and a conditional
    // WHILE loop over the iteration body (in the double-word mode: a first
    // loop, the FP64 residual replacement, a second loop).
    cudaGraph_t graph = nullptr;
    CT_CK(cudaGraphCreate(&graph, 0));
    cudaGraphConditionalHandle h1{}, h2{};
    // CT_COND_GRAPHS=0 selects the plain part graphs (profilers cannot see
    // inside conditional nodes).
    const char* cg_env = std::getenv("CT_COND_GRAPHS");
    bool ok = !(cg_env && cg_env[0] == '0') &&
              cudaGraphConditionalHandleCreate(&h1, graph, 1u, cudaGraphCondAssignDefault) == cudaSuccess;
    if (ok && dw)
        ok = cudaGraphConditionalHandleCreate(&h2, graph, 1u, cudaGraphCondAssignDefault) == cudaSuccess;
    // Adds a WHILE node after the captured work so far and captures its body.
    auto add_while = [&](cudaGraphConditionalHandle h) -> bool {
        cudaStreamCaptureStatus cst;
        const cudaGraphNode_t* deps = nullptr;
        size_t ndeps = 0;
        cudaGraph_t cg = nullptr;
        if (cudaStreamGetCaptureInfo(st, &cst, nullptr, &cg, &deps, nullptr, &ndeps) != cudaSuccess)
            return false;
        cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t cnode = nullptr;
        if (cudaGraphAddNode(&cnode, cg, deps, nullptr, ndeps, &cp) != cudaSuccess) return false;
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        if (cudaStreamBeginCaptureToGraph(st_body, body, nullptr, nullptr, 0,
                                          cudaStreamCaptureModeThreadLocal) != cudaSuccess)
            return false;
        cs = st_body;
        enqueue_body(Cond{h, 1});
        cs = st;
        cudaGraph_t bg = nullptr;
        if (cudaStreamEndCapture(st_body, &bg) != cudaSuccess) return false;
        return cudaStreamUpdateCaptureDependencies(st, &cnode, nullptr, 1,
                                                   cudaStreamSetCaptureDependencies) == cudaSuccess;
    };
    if (ok) {
        ok = cudaStreamBeginCaptureToGraph(st, graph, nullptr, nullptr, 0,
                                           cudaStreamCaptureModeThreadLocal) == cudaSuccess;
        if (ok) {
            cs = st;
            enqueue_init(Cond{h1, 1});
            ok = add_while(h1);
            if (ok && x_lag()) launch_update_x(st, n, p, x, ctl, 0);  // the last iteration's x update
            if (ok && dw) {
                enqueue_replace(Cond{h2, 1});
                ok = add_while(h2);
            }
            cudaGraph_t outg = nullptr;
            const bool ended = cudaStreamEndCapture(st, &outg) == cudaSuccess;
            ok = ok && ended && launch_error == cudaSuccess;
            if (ok) ok = cudaGraphInstantiate(&gx_solve, graph, 0) == cudaSuccess;
        }
    }
    cs = st;
    cudaGraphDestroy(graph);
    if (ok) {
        have_cond = true;
        return CT_OK;
    }
    cudaGetLastError();  // clear the failed attempt
    if (launch_error != cudaSuccess)
        return fail(CT_CUDA_ERROR, "V-cycle kernel launch failed while recording: %s",
                    cudaGetErrorString(launch_error));
    if (gx_solve) {
        cudaGraphExecDestroy(gx_solve);
        gx_solve = nullptr;
    }
    // Fallback: the parts as plain graphs, polled by the host.
    const Cond none{0, 0};
    for (int part_i = 0; part_i < (dw ? 3 : 2); ++part_i) {
        cudaGraph_t g = nullptr;
        CT_CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        if (part_i == 0)
            enqueue_init(none);
        else if (part_i == 1)
            enqueue_body(none);
        else
            enqueue_replace(none);
        CT_CK(cudaStreamEndCapture(st, &g));
        cudaGraphExec_t* dst = part_i == 0 ? &gx_init : (part_i == 1 ? &gx_body : &gx_replace);
        const cudaError_t e = cudaGraphInstantiate(dst, g, 0);
        cudaGraphDestroy(g);
        CT_CK(e);
    }
    have_cond = false;
    return CT_OK;
}

ct_status Solver::solve(double tol, int maxit, ct_stats* out) {
    const TraceRange trace("ct_solve");
    if (!(tol >= 0)) return fail(CT_BAD_ARG, "ct_solve: tol must be >= 0");
    if (maxit > 100000000) return fail(CT_BAD_ARG, "ct_solve: maxit above 1e8");
    Ctl c;
    std::memset(&c, 0, sizeof c);
    c.tol = tol;
    c.maxit = maxit;
    c.inv_dt = inv_dt;
    c.stop = dw ? std::max(tol, rr_thr) : tol;
    c.x_zero = x_zero ? 1 : 0;
    x_zero = false;
    *h_ctl = c;
    CT_CK(cudaMemcpyAsync(ctl, h_ctl, sizeof(Ctl), cudaMemcpyHostToDevice, st));
    const Cond none{0, 0};
    cs = st;
    if (have_cond && !prof) {
        CT_CK(cudaGraphLaunch(gx_solve, st));
    } else {
        // Host-driven loop: direct launches (profiling, ct_use_graphs(0)) or
        // the part graphs, with a host check after every body (direct) or
        // after a few (graphs); the double-word mode's replacement step runs
        // when the first phase ends.
        const bool graphs = gx_init && !prof;
        if (graphs)
            CT_CK(cudaGraphLaunch(gx_init, st));
        else
            enqueue_init(none);
        int launched = 0, k = graphs ? 2 : 1;
        while (true) {
            CT_CK(cudaMemcpyAsync(h_ctl, ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
            CT_CK(cudaStreamSynchronize(st));
            if (h_ctl->done || launched > maxit + 2) break;
            if (h_ctl->phase_end) {
                if (graphs)
                    CT_CK(cudaGraphLaunch(gx_replace, st));
                else
                    enqueue_replace(none);
                continue;
            }
            for (int q = 0; q < k; ++q) {
                if (graphs)
                    CT_CK(cudaGraphLaunch(gx_body, st));
                else
                    enqueue_body(none);
            }
            launched += k;
            if (graphs) k = std::min(k * 2, 8);
        }
        if (x_lag()) launch_update_x(st, n, p, x, ctl, 0);  // the last iteration's x update
    }
    CT_CK(cudaGetLastError());
    return finish_solve(out);
}

ct_status Solver::solve_async(double tol, int maxit) {
    const TraceRange trace("ct_solve_async");
    if (!(tol >= 0)) return fail(CT_BAD_ARG, "ct_solve_async: tol must be >= 0");
    if (maxit > 100000000) return fail(CT_BAD_ARG, "ct_solve_async: maxit above 1e8");
    if (!(have_cond && !prof)) {
        // no single-graph solve here: run it now and keep its result
        async_status = solve(tol, maxit, &async_done);
        async_pending = 2;
        return async_status == CT_NOT_CONVERGED || async_status == CT_BREAKDOWN ? CT_OK : async_status;
    }
    Ctl c;
    std::memset(&c, 0, sizeof c);
    c.tol = tol;
    c.maxit = maxit;
    c.inv_dt = inv_dt;
    c.stop = dw ? std::max(tol, rr_thr) : tol;
    c.x_zero = x_zero ? 1 : 0;
    x_zero = false;
    cs = st;
    launch_ctl_set(st, ctl, c);
    CT_CK(cudaGraphLaunch(gx_solve, st));
    launch_zero_if_no_heat(st, ctl, n, x, xwc);
    CT_CK(cudaGetLastError());
    async_pending = 1;
    return CT_OK;
}

ct_status Solver::solve_wait(ct_stats* out) {
    const TraceRange trace("ct_solve_wait");
    const int pending = async_pending;
    async_pending = 0;
    if (pending == 0) return fail(CT_BAD_ARG, "ct_solve_wait: no solve queued");
    if (pending == 2) {
        if (out) *out = async_done;
        return async_status;
    }
    return finish_solve(out);
}

ct_status Solver::ensure_copy_queues() {
    if (st_h2d) return CT_OK;
    CT_CK(cudaStreamCreateWithFlags(&st_h2d, cudaStreamNonBlocking));
    CT_CK(cudaStreamCreateWithFlags(&st_d2h, cudaStreamNonBlocking));
    for (int i = 0; i < 2; ++i) {
        CT_CK(cudaMalloc(&nat_in[i], ncells * 8));
        CT_CK(cudaMalloc(&nat_out[i], ncells * 8));
        for (cudaEvent_t* e : {&ev_in_copied[i], &ev_in_used[i], &ev_out_ready[i], &ev_out_copied[i]})
            CT_CK(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    }
    return CT_OK;
}

ct_status Solver::set_power_async(const double* P_host) {
    const ct_status s0 = ensure_copy_queues();
    if (s0 != CT_OK) return s0;
    const int i = (int)(n_in & 1u);
    // The copy waits for the conversion of the previous copy in (in stream
    // order after the one that last used this buffer), not for the solves
    // queued since: it overlaps them. The first waits for the solver's stream
    // as it stands.
    if (n_in == 0) CT_CK(cudaEventRecord(ev_in_used[1], st));
    CT_CK(cudaStreamWaitEvent(st_h2d, ev_in_used[1 - i], 0));
    CT_CK(cudaMemcpyAsync(nat_in[i], P_host, ncells * 8, cudaMemcpyHostToDevice, st_h2d));
    CT_CK(cudaEventRecord(ev_in_copied[i], st_h2d));
    CT_CK(cudaStreamWaitEvent(st, ev_in_copied[i], 0));
    launch_to_split_d(st, g0, nat_in[i], P);
    CT_CK(cudaGetLastError());
    CT_CK(cudaEventRecord(ev_in_used[i], st));
    ++n_in;
    return CT_OK;
}

ct_status Solver::get_x_async(double* T_host) {
    const ct_status s0 = ensure_copy_queues();
    if (s0 != CT_OK) return s0;
    const int j = (int)(n_out & 1u);
    // refill this buffer only once its previous copy out is done
    if (n_out >= 2) CT_CK(cudaStreamWaitEvent(st, ev_out_copied[j], 0));
    launch_to_natural_d(st, g0, x_as_double(nullptr), nat_out[j]);
    CT_CK(cudaGetLastError());
    CT_CK(cudaEventRecord(ev_out_ready[j], st));
    CT_CK(cudaStreamWaitEvent(st_d2h, ev_out_ready[j], 0));
    CT_CK(cudaMemcpyAsync(T_host, nat_out[j], ncells * 8, cudaMemcpyDeviceToHost, st_d2h));
    CT_CK(cudaEventRecord(ev_out_copied[j], st_d2h));
    ++n_out;
    return CT_OK;
}

ct_status Solver::copies_wait() {
    if (!st_h2d) return CT_OK;
    // the solver's stream then orders after every copy queued so far
    if (n_out > 0) CT_CK(cudaStreamWaitEvent(st, ev_out_copied[(n_out - 1) & 1u], 0));
    CT_CK(cudaStreamSynchronize(st_h2d));
    CT_CK(cudaStreamSynchronize(st_d2h));
    CT_CK(cudaStreamSynchronize(st));
    return CT_OK;
}

ct_status Solver::finish_solve(ct_stats* out) {
    CT_CK(cudaMemcpyAsync(h_ctl, ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, st));
    CT_CK(cudaStreamSynchronize(st));
    if (h_ctl->bb_zero) {  // no heat in: x = 0 (src/pcg3d_cpu.cpp:146)
        CT_CK(cudaMemsetAsync(x, 0, (size_t)n * 8, st));
        if (xwc) CT_CK(cudaMemsetAsync(xwc, 0, (size_t)n * 8, st));
        CT_CK(cudaStreamSynchronize(st));
    }
    if (h_ctl->err)
        return fail(CT_TIMEOUT, "a bounded wait for staged level data ran out (solve stopped after %d iterations)",
                    h_ctl->iter);
    ct_stats s;
    s.iters = h_ctl->iter;
    s.relres = h_ctl->relres;
    s.converged = h_ctl->converged;
    s.breakdown = h_ctl->breakdown;
    if (out) *out = s;
    if (s.breakdown) return fail(CT_BREAKDOWN, "PCG breakdown after %d iterations (p.Ap = %g)", s.iters, h_ctl->pAp);
    if (!s.converged) return fail(CT_NOT_CONVERGED, "not converged after %d iterations (relres %g)", s.iters, s.relres);
    return CT_OK;
}

}  // namespace ct

// ---- C ABI ----------------------------------------------------------------

using ct::fail;

#define CT_SOLVER_OK(s) \
    if (!(s)) return fail(CT_BAD_ARG, "%s: null solver", __func__)

#define CT_CUDA(call)                                                                         \
    do {                                                                                      \
        const cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess)                                                                \
            return fail(CT_CUDA_ERROR, "%s: %s", #call, cudaGetErrorString(e_));              \
    } while (0)

namespace {
// Copies a split-layout level array to the host in the natural layout.
template <class S, class D>
ct_status level_to_host(ct::Solver& v, const ct::Geo& g, size_t off, int planes, D* out) {
    std::vector<S> tmp((size_t)g.plane * planes);
    CT_CUDA(cudaMemcpyAsync(tmp.data(), v.base + off, tmp.size() * sizeof(S), cudaMemcpyDeviceToHost, v.st));
    CT_CUDA(cudaStreamSynchronize(v.st));
    for (int l = 0; l < planes; ++l)
        for (int j = 0; j < g.ny; ++j)
            for (int i = 0; i < g.nx; ++i)
                out[((size_t)l * g.ny + j) * g.nx + i] = (D)tmp[(size_t)l * g.plane + ct::scol(g, i, j)];
    return CT_OK;
}
}  // namespace

extern "C" {

void ct_use_graphs(int on) { ct::g_use_graphs = on != 0; }

ct_status ct_selftest_bounded_wait(unsigned polls, int* timed_out) {
    if (!timed_out) return fail(CT_BAD_ARG, "ct_selftest_bounded_wait: null");
    if (polls == 0 || polls > (1u << 22)) return fail(CT_BAD_ARG, "ct_selftest_bounded_wait: polls in 1..2^22");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(CT_NO_DEVICE, "no CUDA device");
    }
    int* d = nullptr;
    int h = 0;
    cudaError_t e = cudaMalloc(&d, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(d, 0, sizeof(int));
    if (e == cudaSuccess) e = ct::launch_wait_selftest(nullptr, polls, d);
    if (e == cudaSuccess) e = cudaMemcpy(&h, d, sizeof(int), cudaMemcpyDeviceToHost);
    if (d) cudaFree(d);
    if (e != cudaSuccess) return fail(CT_CUDA_ERROR, "ct_selftest_bounded_wait: %s", cudaGetErrorString(e));
    if (h != 1 && h != 2) return fail(CT_CUDA_ERROR, "ct_selftest_bounded_wait: status %d", h);
    *timed_out = h == 1 ? 1 : 0;
    return CT_OK;
}

ct_status ct_selftest_conversions(unsigned long long n, unsigned long long seed,
                                  unsigned long long* mismatches) {
    if (!mismatches) return fail(CT_BAD_ARG, "ct_selftest_conversions: null");
    if (n == 0 || n > (1ull << 32)) return fail(CT_BAD_ARG, "ct_selftest_conversions: n in 1..2^32");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(CT_NO_DEVICE, "no CUDA device");
    }
    unsigned long long* d = nullptr;
    unsigned long long h = 0;
    cudaError_t e = cudaMalloc(&d, sizeof(*d));
    if (e == cudaSuccess) e = cudaMemset(d, 0, sizeof(*d));
    if (e == cudaSuccess) e = ct::launch_conv_selftest(nullptr, n, seed, d);
    if (e == cudaSuccess) e = cudaMemcpy(&h, d, sizeof(h), cudaMemcpyDeviceToHost);
    if (d) cudaFree(d);
    if (e != cudaSuccess) return fail(CT_CUDA_ERROR, "ct_selftest_conversions: %s", cudaGetErrorString(e));
    *mismatches = h;
    return CT_OK;
}

ct_status ct_probe_fp64_rate(double* dfma_per_s) {
    if (!dfma_per_s) return fail(CT_BAD_ARG, "ct_probe_fp64_rate: null");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(CT_NO_DEVICE, "no CUDA device");
    }
    const cudaError_t e = ct::measure_dfma_rate(dfma_per_s);
    if (e != cudaSuccess) return fail(CT_CUDA_ERROR, "ct_probe_fp64_rate: %s", cudaGetErrorString(e));
    return CT_OK;
}

ct_status ct_probe_sync_costs(int phases, int blocks_per_sm, double* us_grid_barrier,
                              double* us_dependent_launch, int* blocks) {
    if (!us_grid_barrier || !us_dependent_launch || !blocks) return fail(CT_BAD_ARG, "ct_probe_sync_costs: null");
    if (phases < 1 || phases > 100000) return fail(CT_BAD_ARG, "ct_probe_sync_costs: phases in 1..100000");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(CT_NO_DEVICE, "no CUDA device");
    }
    int gave_up = 0;
    const cudaError_t e =
        ct::measure_sync_costs(phases, blocks_per_sm, us_grid_barrier, us_dependent_launch, blocks, &gave_up);
    if (e != cudaSuccess) return fail(CT_CUDA_ERROR, "ct_probe_sync_costs: %s", cudaGetErrorString(e));
    if (gave_up) return fail(CT_TIMEOUT, "ct_probe_sync_costs: a grid barrier wait ran out");
    return CT_OK;
}

ct_status ct_last_setup(ct_setup_times* out) {
    if (!out) return fail(CT_BAD_ARG, "ct_last_setup: null");
    std::lock_guard<std::mutex> lk(ct::g_setup_mu);
    *out = ct::g_last_setup;
    return CT_OK;
}

ct_status ct_solver_create(const ct_model* m, ct_precond pc, ct_precision prec, ct_solver** out) {
    if (!out) return fail(CT_BAD_ARG, "ct_solver_create: null output");
    *out = nullptr;
    ct_solver* s = new (std::nothrow) ct_solver();
    if (!s) return fail(CT_OUT_OF_MEMORY, "host allocation failed");
    const ct_status st = s->impl.create(m, pc, prec);
    if (st != CT_OK) {
        delete s;
        return st;
    }
    *out = s;
    return CT_OK;
}

ct_status ct_solver_create_case(const ct_case* c, int nx, int ny, int with_tsv, ct_precond pc,
                                ct_precision prec, ct_solver** out) {
    if (!out) return fail(CT_BAD_ARG, "ct_solver_create_case: null output");
    *out = nullptr;
    ct::DeviceBuild b;
    ct_status st = ct::case_build(c, nx, ny, with_tsv != 0, &b);
    if (st != CT_OK) return st;
    ct_solver* s = new (std::nothrow) ct_solver();
    if (!s) return fail(CT_OUT_OF_MEMORY, "host allocation failed");
    st = s->impl.create(nullptr, pc, prec, &b);
    if (st != CT_OK) {
        delete s;
        return st;
    }
    *out = s;
    return CT_OK;
}

ct_status ct_solver_destroy(ct_solver* s) {
    delete s;
    return CT_OK;
}

ct_status ct_set_dt(ct_solver* s, double dt) {
    CT_SOLVER_OK(s);
    return s->impl.set_dt(dt);
}

ct_status ct_set_x_zero(ct_solver* s) {
    CT_SOLVER_OK(s);
    s->impl.x_zero = true;
    CT_CUDA(cudaMemsetAsync(s->impl.x, 0, (size_t)s->impl.n * 8, s->impl.st));
    if (s->impl.xwc) CT_CUDA(cudaMemsetAsync(s->impl.xwc, 0, (size_t)s->impl.n * 8, s->impl.st));
    return CT_OK;
}

ct_status ct_set_x(ct_solver* s, const double* T) {
    CT_SOLVER_OK(s);
    if (!T) return fail(CT_BAD_ARG, "ct_set_x: null");
    s->impl.x_zero = false;
    ct::Solver& v = s->impl;
    CT_CUDA(cudaMemcpyAsync(v.nat, T, v.ncells * 8, cudaMemcpyHostToDevice, v.st));
    ct::launch_to_split_d(v.st, v.g0, v.nat, v.x);
    if (v.xwc) CT_CUDA(cudaMemsetAsync(v.xwc, 0, (size_t)v.n * 8, v.st));
    CT_CUDA(cudaGetLastError());
    CT_CUDA(cudaStreamSynchronize(v.st));
    return CT_OK;
}

ct_status ct_set_rhs_steady(ct_solver* s) {
    CT_SOLVER_OK(s);
    CT_CUDA(cudaMemcpyAsync(s->impl.b, s->impl.P, (size_t)s->impl.n * 8, cudaMemcpyDeviceToDevice,
                            s->impl.st));
    return CT_OK;
}

ct_status ct_set_rhs_transient(ct_solver* s) {
    CT_SOLVER_OK(s);
    ct::Solver& v = s->impl;
    const double* xd = v.x_as_double(nullptr);
    ct::launch_rhs_transient(v.st, v.n, v.cap, v.inv_dt, v.P, xd, v.b, v.xold);
    CT_CUDA(cudaGetLastError());
    return CT_OK;
}

ct_status ct_set_power(ct_solver* s, const double* P) {
    CT_SOLVER_OK(s);
    if (!P) return fail(CT_BAD_ARG, "ct_set_power: null");
    ct::Solver& v = s->impl;
    CT_CUDA(cudaMemcpyAsync(v.nat, P, v.ncells * 8, cudaMemcpyHostToDevice, v.st));
    ct::launch_to_split_d(v.st, v.g0, v.nat, v.P);
    CT_CUDA(cudaGetLastError());
    CT_CUDA(cudaStreamSynchronize(v.st));
    return CT_OK;
}

ct_status ct_set_power_device(ct_solver* s, const double* P_dev) {
    CT_SOLVER_OK(s);
    if (!P_dev) return fail(CT_BAD_ARG, "ct_set_power_device: null");
    ct::Solver& v = s->impl;
    ct::launch_to_split_d(v.st, v.g0, P_dev, v.P);
    CT_CUDA(cudaGetLastError());
    return CT_OK;
}

ct_status ct_solve(ct_solver* s, double tol, int maxit, ct_stats* st) {
    CT_SOLVER_OK(s);
    s->impl.async_pending = 0;
    return s->impl.solve(tol, maxit, st);
}

ct_status ct_solve_async(ct_solver* s, double tol, int maxit) {
    CT_SOLVER_OK(s);
    return s->impl.solve_async(tol, maxit);
}

ct_status ct_solve_wait(ct_solver* s, ct_stats* st) {
    CT_SOLVER_OK(s);
    return s->impl.solve_wait(st);
}

ct_status ct_set_power_async(ct_solver* s, const double* P) {
    CT_SOLVER_OK(s);
    if (!P) return fail(CT_BAD_ARG, "ct_set_power_async: null");
    return s->impl.set_power_async(P);
}

ct_status ct_get_x_async(ct_solver* s, double* T) {
    CT_SOLVER_OK(s);
    if (!T) return fail(CT_BAD_ARG, "ct_get_x_async: null");
    return s->impl.get_x_async(T);
}

ct_status ct_copies_wait(ct_solver* s) {
    CT_SOLVER_OK(s);
    return s->impl.copies_wait();
}

ct_status ct_get_x(ct_solver* s, double* T) {
    CT_SOLVER_OK(s);
    if (!T) return fail(CT_BAD_ARG, "ct_get_x: null");
    ct::Solver& v = s->impl;
    ct::launch_to_natural_d(v.st, v.g0, v.x_as_double(nullptr), v.nat);
    CT_CUDA(cudaGetLastError());
    CT_CUDA(cudaMemcpyAsync(T, v.nat, v.ncells * 8, cudaMemcpyDeviceToHost, v.st));
    CT_CUDA(cudaStreamSynchronize(v.st));
    return CT_OK;
}

ct_status ct_device_x(ct_solver* s, const double** T_dev) {
    CT_SOLVER_OK(s);
    if (!T_dev) return fail(CT_BAD_ARG, "ct_device_x: null");
    ct::Solver& v = s->impl;
    ct::launch_to_natural_d(v.st, v.g0, v.x_as_double(nullptr), v.nat);
    CT_CUDA(cudaGetLastError());
    CT_CUDA(cudaStreamSynchronize(v.st));
    *T_dev = v.nat;
    return CT_OK;
}

ct_status ct_solver_setup_times(const ct_solver* s, ct_setup_times* out) {
    CT_SOLVER_OK(s);
    if (!out) return fail(CT_BAD_ARG, "ct_solver_setup_times: null");
    *out = s->impl.times;
    return CT_OK;
}

ct_status ct_solver_stream(const ct_solver* s, void** stream) {
    CT_SOLVER_OK(s);
    if (!stream) return fail(CT_BAD_ARG, "ct_solver_stream: null");
    *stream = (void*)s->impl.st;
    return CT_OK;
}

ct_status ct_true_relres(ct_solver* s, double* out) {
    CT_SOLVER_OK(s);
    if (!out) return fail(CT_BAD_ARG, "ct_true_relres: null");
    ct::Solver& v = s->impl;
    ct::launch_true_residual(v.st, v.op(), v.P, v.x_as_double(nullptr), v.ctl, v.red_cols(ct::SL_AUX));
    CT_CUDA(cudaGetLastError());
    CT_CUDA(cudaMemcpyAsync(v.h_ctl, v.ctl, sizeof(ct::Ctl), cudaMemcpyDeviceToHost, v.st));
    CT_CUDA(cudaStreamSynchronize(v.st));
    *out = std::sqrt(v.h_ctl->aux0 / v.h_ctl->aux1);
    return CT_OK;
}

ct_status ct_solver_step_record(ct_solver* s, double dt, ct_step_record* out) {
    CT_SOLVER_OK(s);
    if (!out || !(dt > 0)) return fail(CT_BAD_ARG, "ct_solver_step_record: null output or dt <= 0");
    ct::Solver& v = s->impl;
    ct::launch_step_record(v.st, v.op(), v.x_as_double(nullptr), v.xold, v.ctl, v.red_cols(ct::SL_AUX));
    CT_CUDA(cudaGetLastError());
    CT_CUDA(cudaMemcpyAsync(v.h_ctl, v.ctl, sizeof(ct::Ctl), cudaMemcpyDeviceToHost, v.st));
    CT_CUDA(cudaStreamSynchronize(v.st));
    out->T_max = v.h_ctl->aux0;
    out->q_out = v.h_ctl->aux1;
    out->q_stored = v.h_ctl->aux2 / dt;
    return CT_OK;
}

ct_status ct_solver_step_record_async(ct_solver* s, double dt, int slot) {
    CT_SOLVER_OK(s);
    if (!(dt > 0) || slot < 0) return fail(CT_BAD_ARG, "ct_solver_step_record_async: dt <= 0 or slot < 0");
    ct::Solver& v = s->impl;
    if (slot >= v.rec_cap) {  // grow the table (doubling), keeping the entries so far
        int cap = std::max(64, v.rec_cap);
        while (cap <= slot) cap *= 2;
        ct::StepEntry* t = nullptr;
        CT_CUDA(cudaMalloc(&t, (size_t)cap * sizeof(ct::StepEntry)));
        // entries never recorded read back as zeros
        CT_CUDA(cudaMemsetAsync(t, 0, (size_t)cap * sizeof(ct::StepEntry), v.st));
        if (v.rec_table) {
            CT_CUDA(cudaMemcpyAsync(t, v.rec_table, (size_t)v.rec_cap * sizeof(ct::StepEntry),
                                    cudaMemcpyDeviceToDevice, v.st));
            CT_CUDA(cudaStreamSynchronize(v.st));
            CT_CUDA(cudaFree(v.rec_table));
        }
        v.rec_table = t;
        v.rec_cap = cap;
    }
    ct::launch_step_record(v.st, v.op(), v.x_as_double(nullptr), v.xold, v.ctl, v.red_cols(ct::SL_AUX));
    ct::launch_record_keep(v.st, v.ctl, dt, v.rec_table, slot);
    CT_CUDA(cudaGetLastError());
    return CT_OK;
}

ct_status ct_solver_step_records(ct_solver* s, int first, int count, ct_step_record* out, ct_stats* stats) {
    CT_SOLVER_OK(s);
    ct::Solver& v = s->impl;
    if (first < 0 || count < 0 || first + count > v.rec_cap || (count > 0 && !out))
        return fail(CT_BAD_ARG, "ct_solver_step_records: entries %d..%d outside the table", first, first + count);
    // a queued solve's statistics are in the table; the wait is this one
    v.async_pending = 0;
    std::vector<ct::StepEntry> h((size_t)count);
    if (count > 0)
        CT_CUDA(cudaMemcpyAsync(h.data(), v.rec_table + first, (size_t)count * sizeof(ct::StepEntry),
                                cudaMemcpyDeviceToHost, v.st));
    CT_CUDA(cudaStreamSynchronize(v.st));
    bool err = false;
    for (int k = 0; k < count; ++k) {
        const ct::StepEntry& e = h[(size_t)k];
        out[k].T_max = e.T_max;
        out[k].q_out = e.q_out;
        out[k].q_stored = e.q_stored;
        if (stats) {
            stats[k].iters = e.iters;
            stats[k].relres = e.relres;
            stats[k].converged = e.converged;
            stats[k].breakdown = e.breakdown;
        }
        err = err || e.err;
    }
    if (err) return fail(CT_TIMEOUT, "a bounded wait for staged level data ran out in a queued step");
    return CT_OK;
}

ct_status ct_num_levels(const ct_solver* s, int* nlev) {
    CT_SOLVER_OK(s);
    if (!nlev) return fail(CT_BAD_ARG, "ct_num_levels: null");
    *nlev = (int)s->impl.lv.size();
    return CT_OK;
}

ct_status ct_level_dims(const ct_solver* s, int k, int* nx, int* ny, int* nz) {
    CT_SOLVER_OK(s);
    if (k < 0 || k >= (int)s->impl.lv.size() || !nx || !ny || !nz)
        return fail(CT_BAD_ARG, "ct_level_dims: bad level %d", k);
    const ct::Geo& g = s->impl.lv[(size_t)k].g;
    *nx = g.nx;
    *ny = g.ny;
    *nz = g.nz;
    return CT_OK;
}


ct_status ct_level_operator(ct_solver* s, int k, float* gE, float* gN, float* gU, float* gB,
                            float* cap) {
    CT_SOLVER_OK(s);
    ct::Solver& v = s->impl;
    if (k < 0 || k >= (int)v.lv.size() || !gE || !gN || !gU || !gB || !cap)
        return fail(CT_BAD_ARG, "ct_level_operator: bad level %d or null array", k);
    const ct::Level& L = v.lv[(size_t)k];
    ct_status r;
    if ((r = level_to_host<float>(v, L.g, L.o_gE, L.g.nz, gE)) != CT_OK) return r;
    if ((r = level_to_host<float>(v, L.g, L.o_gN, L.g.nz, gN)) != CT_OK) return r;
    if ((r = level_to_host<float>(v, L.g, L.o_gU, L.g.nz, gU)) != CT_OK) return r;
    if ((r = level_to_host<float>(v, L.g, L.o_gB, 1, gB)) != CT_OK) return r;
    return level_to_host<float>(v, L.g, L.o_cap, L.g.nz, cap);
}

ct_status ct_level_factors(ct_solver* s, int k, double* fcp, double* finv) {
    CT_SOLVER_OK(s);
    ct::Solver& v = s->impl;
    if (k < 0 || k >= (int)v.lv.size() || !fcp || !finv)
        return fail(CT_BAD_ARG, "ct_level_factors: bad level %d or null array", k);
    const ct::Level& L = v.lv[(size_t)k];
    ct_status r;
    if (v.mt == ct::MG_F64) {
        if ((r = level_to_host<double>(v, L.g, L.o_fcp, L.g.nz, fcp)) != CT_OK) return r;
        return level_to_host<double>(v, L.g, L.o_finv, L.g.nz, finv);
    }
    if ((r = level_to_host<float>(v, L.g, L.o_fcp, L.g.nz, fcp)) != CT_OK) return r;
    return level_to_host<float>(v, L.g, L.o_finv, L.g.nz, finv);
}

ct_status ct_profile_solve(ct_solver* s, double tol, int maxit, ct_stats* st, ct_kernel_time* out,
                           int max, int* nout) {
    CT_SOLVER_OK(s);
    if (!out || !nout || max <= 0) return fail(CT_BAD_ARG, "ct_profile_solve: bad output");
    ct::Solver& v = s->impl;
    v.prof = true;
    v.prof_log.clear();
    const ct_status rs = v.solve(tol, maxit, st);
    v.prof = false;
    cudaStreamSynchronize(v.st);
    std::vector<ct_kernel_time> agg;
    for (const ct::ProfEntry& e : v.prof_log) {
        float ms = 0;
        cudaEventElapsedTime(&ms, e.a, e.b);
        cudaEventDestroy(e.a);
        cudaEventDestroy(e.b);
        auto it = std::find_if(agg.begin(), agg.end(), [&](const ct_kernel_time& k) { return e.name == k.name; });
        if (it == agg.end()) {
            ct_kernel_time k;
            std::memset(&k, 0, sizeof k);
            std::snprintf(k.name, sizeof k.name, "%s", e.name.c_str());
            agg.push_back(k);
            it = agg.end() - 1;
        }
        it->launches += 1;
        it->total_ms += ms;
        it->bytes += e.bytes;
    }
    v.prof_log.clear();
    *nout = std::min((int)agg.size(), max);
    for (int k = 0; k < *nout; ++k) out[k] = agg[(size_t)k];
    return rs;
}

}  // extern "C"
