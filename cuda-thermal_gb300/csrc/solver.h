// solver.h - the single-instance solver object behind ct_solver_* (GpuPcg,
// src/pcg3d.h:115-163); solver.cu holds its member functions. The batched
// solver (batch.cu) builds one per instance for set-up and bookkeeping.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "build.h"
#include "cthermal.h"
#include "kernels.h"

namespace ct {

// Bump allocator over one device allocation, 256-byte aligned.
struct Arena {
    size_t used = 0;
    size_t take(size_t bytes) {
        const size_t off = used;
        used += (bytes + 255) & ~size_t(255);
        return off;
    }
};

// Host-side record of one multigrid level.
struct Level {
    Geo g;
    size_t o_gE, o_gN, o_gU, o_gB, o_cap, o_fcp, o_finv, o_x, o_b, o_dx, o_dy;
    std::vector<double> dx, dy;  // cell widths (m), for the coarsening
    bool tma = false;            // sweeps staged by bulk tensor copies (maps per colour)
    SweepMaps maps[2];
};

// mg_coarse_widths (src/mg3d.h:139-144).
inline std::vector<double> coarse_widths(const std::vector<double>& f) {
    std::vector<double> c;
    const int n = (int)f.size();
    for (int I = 0; I < (n + 1) / 2; ++I) c.push_back(f[2 * I] + (2 * I + 1 < n ? f[2 * I + 1] : 0.0));
    return c;
}

struct ProfEntry {
    std::string name;
    double bytes;
    cudaEvent_t a, b;
};

class Solver {
  public:
    ct_precond pc = CT_MULTIGRID;
    ct_precision prec = CT_MG_FP32_FLEX;
    MgType mt = MG_F32;
    bool flex = true;
    bool dw = false;       // double-word outer iteration (CT_MG_FP32_FLEX_DW)
    bool x_zero = true;    // x is known to be 0 (set_x_zero since the last solve)
    cudaError_t launch_error = cudaSuccess;  // first failed launch of a shaped (cluster/smem) kernel
    double rr_thr = 1e-5;  // relres of the FP64 residual replacement (dw)
    size_t tsize = 4;  // bytes per V-cycle value
    Geo g0{};
    unsigned n = 0;      // slots of all planes (split layout, with padding)
    size_t ncells = 0;   // nx * ny * nz
    double dx = 0, dy = 0;
    int sms = 0;
    cudaStream_t st = nullptr;
    cudaStream_t st_body = nullptr;  // captures the graph loops' bodies
    cudaStream_t cs = nullptr;       // stream the enqueue_* functions launch on
    char* base = nullptr;
    size_t bytes = 0;
    // fine operator and PCG vectors (split layout)
    float *gE = nullptr, *gN = nullptr, *gU = nullptr, *gB = nullptr, *cap = nullptr;
    double *P = nullptr, *x = nullptr, *b = nullptr, *r = nullptr, *p = nullptr, *Ap = nullptr;
    double *diag = nullptr, *invd = nullptr, *xold = nullptr, *nat = nullptr, *part = nullptr;
    double* dface = nullptr;  // FP64 face sum of the diagonal (the part that does not change with dt)
    float2* dgw = nullptr;  // double-word diagonal (dw)
    float2* xwc = nullptr;  // double-word correction of x (dw); x is then its FP64 base
    Ctl* ctl = nullptr;
    Ctl* h_ctl = nullptr;  // pinned mirror
    std::vector<Level> lv;
    int maxb = 0;
    double inv_dt = 0;
    bool use_graphs = true;
    bool have_cond = false;
    size_t small_k0 = 0;   // levels from small_k0 down run in one block from shared memory
    bool fuse_sweep0 = true;  // a level's first (x = 0) sweep rides with the restriction into it
    bool sweep0_grid = true;  // x = 0 sweeps of the staged levels on the grid kernel
    // x += alpha p beside the next V-cycle (FP64 outer loop, multigrid): a
    // launch of xlag_blocks blocks on st_side, forked after the restriction
    // out of level fork_level() (xlag < 0: x stays in the update)
    int xlag = 1;
    int xlag_blocks = 64;
    cudaStream_t st_side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    bool lag_now = false, forked = false;  // while a body is enqueued
    bool x_lag() const { return xlag >= 0 && !dw && mt != MG_NONE && st_side; }
    // the last level with a restriction out of it, at most xlag (a V-cycle
    // all in the shared-memory bottom: lv.size(), the start of the body)
    int fork_level() const {
        return small_k0 == 0 ? (int)lv.size() : std::min(xlag, (int)small_k0 - 1);
    }
    void fork_x();
    // queued host copies (ct_set_power_async, ct_get_x_async): two staging
    // buffers each way, a copy stream each way, events that keep a buffer
    // from being refilled before it is consumed
    cudaStream_t st_h2d = nullptr, st_d2h = nullptr;
    double* nat_in[2] = {nullptr, nullptr};
    double* nat_out[2] = {nullptr, nullptr};
    cudaEvent_t ev_in_copied[2] = {}, ev_in_used[2] = {}, ev_out_ready[2] = {}, ev_out_copied[2] = {};
    unsigned long long n_in = 0, n_out = 0;
    // device table of queued step records (ct_solver_step_record_async)
    StepEntry* rec_table = nullptr;
    int rec_cap = 0;
    ct_status ensure_copy_queues();
    ct_status set_power_async(const double* P_host);
    ct_status get_x_async(double* T_host);
    ct_status copies_wait();
    cudaGraphExec_t gx_solve = nullptr, gx_init = nullptr, gx_body = nullptr, gx_replace = nullptr;
    ct_setup_times times{};
    // per-kernel timing (ct_profile_solve)
    bool prof = false;
    std::vector<ProfEntry> prof_log;

    bool own_stream = true;   // false: st belongs to a batch that owns this solver
    bool skip_graphs = false; // batch members record no graphs of their own

    ~Solver() {
        for (cudaStream_t q : {st, st_side, st_h2d, st_d2h})
            if (q) cudaStreamSynchronize(q);
        for (cudaGraphExec_t g : {gx_solve, gx_init, gx_body, gx_replace})
            if (g) cudaGraphExecDestroy(g);
        if (base) cudaFree(base);
        if (rec_table) cudaFree(rec_table);
        if (h_ctl) cudaFreeHost(h_ctl);
        for (int i = 0; i < 2; ++i) {
            for (cudaEvent_t e : {ev_in_copied[i], ev_in_used[i], ev_out_ready[i], ev_out_copied[i]})
                if (e) cudaEventDestroy(e);
            if (nat_in[i]) cudaFree(nat_in[i]);
            if (nat_out[i]) cudaFree(nat_out[i]);
        }
        for (cudaStream_t q : {st_body, st_side, st_h2d, st_d2h})
            if (q) cudaStreamDestroy(q);
        if (ev_fork) cudaEventDestroy(ev_fork);
        if (ev_join) cudaEventDestroy(ev_join);
        if (st && own_stream) cudaStreamDestroy(st);
    }

    template <class T>
    T* at(size_t off) const { return reinterpret_cast<T*>(base + off); }

    OpView op() const { return OpView{g0, gE, gN, gU, gB, cap}; }

    template <class T>
    LevelView<T> view(size_t k) const {
        const Level& L = lv[k];
        LevelView<T> v;
        v.g = L.g;
        v.gE = at<float>(L.o_gE);
        v.gN = at<float>(L.o_gN);
        v.gU = at<float>(L.o_gU);
        v.gB = at<float>(L.o_gB);
        v.cap = at<float>(L.o_cap);
        v.fcp = at<T>(L.o_fcp);
        v.finv = at<T>(L.o_finv);
        v.x = at<T>(L.o_x);
        v.b = at<T>(L.o_b);
        return v;
    }

    // Every level with its columns' first index laid end to end (at most
    // kMaxTail levels; the caller checks).
    template <class T>
    FactorLevels<T> factor_levels() const {
        FactorLevels<T> fl;
        fl.n = (int)std::min(lv.size(), (size_t)kMaxTail);
        fl.first[0] = 0;
        for (size_t k = 0; k < (size_t)fl.n; ++k) {
            fl.L[k] = view<T>(k);
            fl.first[k + 1] = fl.first[k] + (unsigned)lv[k].g.nx * (unsigned)lv[k].g.ny;
        }
        return fl;
    }

    Red red(int blocks_wanted, Slot sl) const {
        Red rd;
        rd.part = part + (size_t)sl * 4 * maxb;
        rd.maxb = maxb;
        rd.blocks = std::max(1, std::min(blocks_wanted, maxb));
        return rd;
    }
    Red red_cols(Slot sl) const { return red((int)((g0.plane + NT - 1) / NT), sl); }
    Red red_vec(Slot sl) const { return red((int)((n / 2 + NT - 1) / NT), sl); }

    // From host arrays (m), or built on the device from a description (b, m
    // null): the same arrays either way.
    ct_status create(const ct_model* m, ct_precond pc_, ct_precision prec_,
                     const DeviceBuild* build = nullptr);
    ct_status set_dt(double dt);
    ct_status solve(double tol, int maxit, ct_stats* out);
    // A solve queued on the stream without waiting for it (the graph path;
    // otherwise solve_async runs solve() and keeps its result), and the wait
    // that returns the last queued solve's result.
    ct_status solve_async(double tol, int maxit);
    ct_status solve_wait(ct_stats* out);
    ct_status finish_solve(ct_stats* out);  // reads the control block after a solve
    int async_pending = 0;                   // 1: a queued solve; 2: a finished one kept in async_done
    ct_status async_status = CT_OK;
    ct_stats async_done{};
    ct_status record_graphs();

    // Enqueues one kernel launch; in profiling mode brackets it with events.
    template <class F>
    void enq(const char* name, double nbytes, F&& launch) {
        if (!prof) {
            launch();
            return;
        }
        ProfEntry e{name, nbytes, nullptr, nullptr};
        cudaEventCreate(&e.a);
        cudaEventCreate(&e.b);
        cudaEventRecord(e.a, cs);
        launch();
        cudaEventRecord(e.b, cs);
        prof_log.push_back(e);
    }

    void enqueue_init(Cond cond);
    void enqueue_body(Cond cond);
    void enqueue_replace(Cond cond);
    // The double-word views of x, r, p, Ap (same storage as the FP64 vectors).
    float2* xw() const { return xwc; }
    float2* rw() const { return reinterpret_cast<float2*>(r); }
    float2* pw() const { return reinterpret_cast<float2*>(p); }
    float2* Apw() const { return reinterpret_cast<float2*>(Ap); }
    // x as split-layout FP64: in the double-word mode the correction is first
    // folded into the FP64 base (which leaves x unchanged).
    const double* x_as_double(double*) const {
        if (dw) launch_fold(st, n, x, xwc, ctl, false);
        return x;
    }
    template <class T>
    void vcycle(size_t k, Cond cond, bool first_sweep_done = false);
    // One sweep of level k (the staged kernel where the level has its maps).
    template <class T>
    void sweep(size_t k, const LevelView<T>& L, int color, bool zero_x, const LevelView<T>* coarse,
               Cond cond);
};


}  // namespace ct

// The C ABI's opaque solver handle.
struct ct_solver {
    ct::Solver impl;
};
