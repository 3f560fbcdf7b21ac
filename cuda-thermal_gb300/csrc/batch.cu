// batch.cu - the batched solver behind ct_batch_*: many independent stacks of
// uneven lateral size and layer count (floorplan or power-map sweeps), each a
// full MG-PCG solve of its own, run together so that every stage of the
// iteration is ONE launch for all of them.
//
// Set-up reuses the single solver: each instance is a Solver (its arena, its
// multigrid levels, factors and boundary conversions), created on the batch's
// stream without graphs of its own. The batch adds device tables over those
// arrays (BInst per instance, LevelView per instance and depth, the small-level
// descriptors) and block tables (batch.h) per stage.
//
// Precision: the FP32 V-cycle inside flexible PCG with the outer iteration
// in FP64 (CT_MG_FP32_FLEX, k_batch64.cu) or in double words on the FP32
// pipes with an FP64 residual replacement (CT_MG_FP32_FLEX_DW, k_batch.cu).
//
// Size buckets. Instances are grouped by the number of levels their V-cycle
// runs as separate sweeps (the rest run in the one-block shared-memory kernel),
// which follows their lateral size. Each bucket has its own stream and ONE
// captured CUDA graph per solve:
//     [fold x];  r = b - A x (FP64);  WHILE (any instance active) {
//         guard;  V-cycle stages per depth;  small levels;  dot;  p;  Ap;
//         x, r update and test;  [residual replacement of instances whose
//         first phase ended] }
// (the bracketed steps in the double-word mode only)
// so instances converge one by one (their blocks return at entry) and the
// loop ends when the bucket's last one does. Buckets run concurrently.
//
// Column tiles. The sweep and restriction stages' items per block are picked
// per bucket and depth by timing candidate tiles at creation (the autotuner);
// CT_BATCH_TILE=<items> fixes them instead.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "trace.h"
#include "batch.h"
#include "cthermal.h"
#include "solver.h"
#include "status.h"

namespace ct {

namespace {

#define CT_BK(call)                                                                              \
    do {                                                                                         \
        const cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess)                                                                   \
            return ct::fail(e_ == cudaErrorMemoryAllocation ? CT_OUT_OF_MEMORY : CT_CUDA_ERROR,  \
                            "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
    } while (0)

// Items per block of the stages whose tile is not tuned.
constexpr unsigned kVecChunk = 4096;   // value pairs (fold, update, dot, p, rhs)
constexpr unsigned kColChunk = 512;    // fine columns (FP64 residual)
// fine rows of one colour and plane per block of the operator apply: the
// FP64 apply is FP64-pipe-bound, and per-block reduction overhead weighs less
// on longer tables (256 instances, two cells per lane: 16 / 32 / 64 / 128 rows
// per block, 73.6 / 63.4 / 59.4 / 58.8 ms of apply per batched solve; one cell
// per lane: 64 / 128 / 256 rows, 47.1 / 48.5 / 53.4 ms; double words 1463 /
// 1477 / 1485 / 1479 instance solves/s at 16 / 32 / 64 / 128)
constexpr unsigned kRowChunk64 = 64;
constexpr unsigned kRowChunkDw = 64;
// Candidate tiles of the autotuner (columns per block for the sweeps, coarse
// cells per block for the restriction).
constexpr unsigned kSweepTiles[] = {256, 512, 1024, 2048};
// ... and tiles per block of the staged sweeps (k_sweep_tma.cu).
constexpr unsigned kTmaTiles[] = {1, 2, 4, 8};
constexpr unsigned kRestrictTiles[] = {256, 512, 1024, 2048, 4096};

// Host form of a block table; first/count are indexed by instance.
struct HPlan {
    std::vector<Task> tasks;
    std::vector<int> first, count;
};

HPlan make_plan(int ni, const std::vector<int>& insts, const std::vector<unsigned>& items,
                unsigned chunk) {
    HPlan h;
    h.first.assign((size_t)ni, 0);
    h.count.assign((size_t)ni, 0);
    for (size_t a = 0; a < insts.size(); ++a) {
        const int i = insts[a];
        h.first[(size_t)i] = (int)h.tasks.size();
        for (unsigned b = 0; b < items[a]; b += chunk)
            h.tasks.push_back(Task{i, b, std::min(items[a], b + chunk)});
        h.count[(size_t)i] = (int)h.tasks.size() - h.first[(size_t)i];
    }
    return h;
}

}  // namespace

class Batch {
  public:
    int ni = 0;
    std::vector<std::unique_ptr<ct_solver>> sv;  // the instances (ct_solver wraps a Solver)
    cudaStream_t st = nullptr;  // set-up, copies, per-instance calls
    int sms = 0;
    ct_precision prec = CT_MG_FP32_FLEX_DW;
    bool dw = true;  // double-word outer iteration (else FP64)
    double rr_thr = 1e-5;
    bool use_cond = true;
    bool prof = false;
    std::vector<ProfEntry> prof_log;
    cudaError_t launch_error = cudaSuccess;  // first failed launch of the small-level kernel

    struct Bucket {
        std::vector<int> inst;
        int depth = 0;    // V-cycle levels run as batched sweeps
        int mz = 1;       // largest nz
        size_t smem = 0;  // shared memory of the small-level kernel
        cudaStream_t st = nullptr, st_body = nullptr;
        cudaGraphExec_t gx = nullptr;
        BCtl* bc = nullptr;
        Plan vec{}, cols{}, rows{};  // value pairs, fine columns, fine rows
        BRed r_res{}, r_apply{}, r_update{}, r_dot{};
        std::vector<Plan> sweep, restr;
        std::vector<unsigned> sweep_tile, restr_tile;
        // per depth: 0 grid sweeps, 1 sweeps staged by bulk tensor copies,
        // 2 mixed: the instances whose level fits a tile row staged (sweep),
        // the others on the grid kernel (sweep_grid)
        std::vector<char> tma;
        std::vector<Plan> sweep_grid;
        std::vector<unsigned> sweep_grid_tile;
        // per depth: the x = 0 sweep on the grid kernel over every instance
        // (sweep0) where that times faster than the staged form
        std::vector<char> sweep0_grid;
        std::vector<Plan> sweep0;
        int* small_insts = nullptr;
    };
    std::vector<Bucket> bk;

    // device tables
    BInst* bi = nullptr;
    Ctl* ctl = nullptr;
    Ctl* h_ctl = nullptr;  // pinned mirror
    std::vector<LevelView<float>*> views;  // per level index: LevelView per instance
    Plan diag_plan{};                      // set_dt: natural fine columns of every instance
    Plan rec_plan{};                       // step records: fine column slots of every instance
    BRed rec_red{};
    double* rec_mx = nullptr;              // per task of rec_plan
    double* rec_dev = nullptr;             // 3 per instance
    std::vector<double> rec_host;
    std::vector<Plan> factor_plans;        // set_dt: natural columns of level k of every instance
    std::vector<SweepMaps*> bmaps;         // per depth and colour (2 d + c): maps per instance
    std::vector<std::vector<char>> fits;   // [d][i]: instance i's level d has maps
    TailLevels<float>* small = nullptr;
    std::vector<void*> bufs;               // every device allocation of the batch
    cudaEvent_t ev_start = nullptr;
    std::vector<cudaEvent_t> ev_done;

    ~Batch() {
        if (st) cudaStreamSynchronize(st);
        for (Bucket& b : bk) {
            if (b.st) cudaStreamSynchronize(b.st);
            if (b.gx) cudaGraphExecDestroy(b.gx);
            if (b.st_body) cudaStreamDestroy(b.st_body);
            if (b.st) cudaStreamDestroy(b.st);
        }
        for (cudaEvent_t e : ev_done) cudaEventDestroy(e);
        if (ev_start) cudaEventDestroy(ev_start);
        sv.clear();  // the instances synchronise on st before it goes
        for (void* p : bufs) cudaFree(p);
        if (h_ctl) cudaFreeHost(h_ctl);
        if (st) cudaStreamDestroy(st);
    }

    template <class T>
    ct_status dalloc(T** out, size_t bytes) {
        void* p = nullptr;
        const cudaError_t e = cudaMalloc(&p, std::max<size_t>(bytes, 256));
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(CT_OUT_OF_MEMORY, "batch: cudaMalloc of %.1f MB failed: %s", bytes / 1e6,
                        cudaGetErrorString(e));
        }
        bufs.push_back(p);
        *out = static_cast<T*>(p);
        return CT_OK;
    }

    template <class T>
    ct_status upload(T** out, const std::vector<T>& v) {
        ct_status s = dalloc(out, v.size() * sizeof(T));
        if (s != CT_OK) return s;
        if (!v.empty()) CT_BK(cudaMemcpyAsync(*out, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st));
        return CT_OK;
    }

    ct_status upload_plan(const HPlan& h, Plan* p) {
        Task* t = nullptr;
        int *f = nullptr, *c = nullptr;
        ct_status s;
        if ((s = upload(&t, h.tasks)) != CT_OK) return s;
        if ((s = upload(&f, h.first)) != CT_OK) return s;
        if ((s = upload(&c, h.count)) != CT_OK) return s;
        *p = Plan{t, (int)h.tasks.size(), f, c};
        return CT_OK;
    }

    ct_status make_red(const Plan& p, BRed* r) {
        ct_status s;
        if ((s = dalloc(&r->part, (size_t)2 * std::max(1, p.ntasks) * sizeof(double))) != CT_OK) return s;
        if ((s = dalloc(&r->tickets, (size_t)ni * sizeof(unsigned))) != CT_OK) return s;
        CT_BK(cudaMemsetAsync(r->tickets, 0, (size_t)ni * sizeof(unsigned), st));
        return CT_OK;
    }

    Solver& inst(int i) const { return sv[(size_t)i]->impl; }

    // Enqueues one launch; in profiling mode brackets it with events.
    template <class F>
    void enq(cudaStream_t s, const std::string& name, double nbytes, F&& launch) {
        if (!prof) {
            launch();
            return;
        }
        ProfEntry e{name, nbytes, nullptr, nullptr};
        cudaEventCreate(&e.a);
        cudaEventCreate(&e.b);
        cudaEventRecord(e.a, s);
        launch();
        cudaEventRecord(e.b, s);
        prof_log.push_back(e);
    }
    // Algorithmic bytes of a bucket's stage: per-cell bytes times the cells
    // of level d of its instances (d < 0: fine cells).
    double cells_of(const Bucket& b, int d) const {
        double c = 0;
        for (int i : b.inst) {
            const Geo& g = inst(i).lv[(size_t)std::max(d, 0)].g;
            c += (double)g.nx * g.ny * g.nz;
        }
        return c;
    }
    int small_k0(int i) const { return (int)inst(i).small_k0; }

    ct_status create(int n, const ct_model* const* models, const DeviceBuild* builds, ct_precision pr);
    ct_status build_bucket(Bucket& b);
    ct_status tune_bucket(Bucket& b);
    ct_status record(Bucket& b);
    ct_status set_dt(const double* dt);
    ct_status solve(double tol, int maxit, ct_stats* out);

    // One bucket's launches.
    void enqueue_init(Bucket& b, cudaStream_t s, Cond cond);
    void enqueue_body(Bucket& b, cudaStream_t s, Cond cond);
    void vcycle(Bucket& b, cudaStream_t s, Cond cond);
    void sweep(Bucket& b, cudaStream_t s, int d, int color, bool zero_x, bool prolong, Cond cond);
};

ct_status Batch::create(int n, const ct_model* const* models, const DeviceBuild* builds, ct_precision pr) {
    const TraceRange trace("ct_batch_create");
    if (n < 1) return fail(CT_BAD_ARG, "ct_batch_create: n must be >= 1");
    if (pr != CT_MG_FP32_FLEX && pr != CT_MG_FP32_FLEX_DW)
        return fail(CT_BAD_ARG, "ct_batch_create: precision must be CT_MG_FP32_FLEX or CT_MG_FP32_FLEX_DW");
    prec = pr;
    dw = pr == CT_MG_FP32_FLEX_DW;
    if (!models && !builds) return fail(CT_BAD_ARG, "ct_batch_create: null model list");
    for (int i = 0; models && i < n; ++i)
        if (!models[i]) return fail(CT_BAD_ARG, "ct_batch_create: null model %d", i);
    ni = n;
    if (const char* e = std::getenv("CT_RR_THRESHOLD")) rr_thr = std::atof(e);
    if (const char* e = std::getenv("CT_COND_GRAPHS")) use_cond = e[0] != '0';
    int dev = 0;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(CT_NO_DEVICE, "no CUDA device");
    }
    CT_BK(cudaGetDevice(&dev));
    CT_BK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CT_BK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    CT_BK(cudaEventCreateWithFlags(&ev_start, cudaEventDisableTiming));

    // Instances: the single solver's set-up on the batch stream.
    sv.reserve((size_t)n);
    int maxdepth = 0;
    for (int i = 0; i < n; ++i) {
        std::unique_ptr<ct_solver> h(new (std::nothrow) ct_solver());
        if (!h) return fail(CT_OUT_OF_MEMORY, "host allocation failed");
        Solver* s = &h->impl;
        s->st = st;
        s->skip_graphs = true;
        s->rr_thr = rr_thr;
        const ct_status cs = builds ? s->create(nullptr, CT_MULTIGRID, prec, &builds[i])
                                    : s->create(models[i], CT_MULTIGRID, prec);
        if (cs != CT_OK) {
            const std::string why = ct_last_error();
            return fail(cs, "ct_batch_create: instance %d: %s", i, why.c_str());
        }
        if (s->small_k0 >= s->lv.size())
            return fail(CT_BAD_ARG, "ct_batch_create: instance %d: coarsest level too large for one block", i);
        maxdepth = std::max(maxdepth, (int)s->small_k0);
        sv.push_back(std::move(h));
    }

    // Tables over the instances' arrays.
    std::vector<BInst> hb((size_t)n);
    for (int i = 0; i < n; ++i) {
        const Solver& s = inst(i);
        BInst& I = hb[(size_t)i];
        I.o = s.op();
        I.P = s.P;
        I.x = s.x;
        I.b = s.b;
        I.diag = s.diag;
        I.dface = s.dface;
        I.xw = s.xwc;
        I.r = s.rw();
        I.p = s.pw();
        I.Ap = s.Apw();
        I.dgw = s.dgw;
        I.b0 = s.at<float>(s.lv[0].o_b);
        I.z = s.at<float>(s.lv[0].o_x);
        I.xold = s.xold;
        I.r64 = s.r;
        I.p64 = s.p;
        I.Ap64 = s.Ap;
        I.n = s.n;
    }
    ct_status s;
    if ((s = upload(&bi, hb)) != CT_OK) return s;
    int maxlev = 0;
    for (int i = 0; i < n; ++i) maxlev = std::max(maxlev, (int)inst(i).lv.size());
    views.assign((size_t)maxlev, nullptr);
    for (int d = 0; d < maxlev; ++d) {
        std::vector<LevelView<float>> hv((size_t)n);
        for (int i = 0; i < n; ++i)
            if ((size_t)d < inst(i).lv.size()) hv[(size_t)i] = inst(i).view<float>((size_t)d);
            else std::memset(&hv[(size_t)i], 0, sizeof(LevelView<float>));
        if ((s = upload(&views[(size_t)d], hv)) != CT_OK) return s;
    }
    // set_dt plans: every instance's fine columns; per level index the
    // instances that have that level.
    {
        std::vector<int> all;
        std::vector<unsigned> cols;
        for (int i = 0; i < n; ++i) {
            all.push_back(i);
            cols.push_back((unsigned)inst(i).g0.nx * (unsigned)inst(i).g0.ny);
        }
        if ((s = upload_plan(make_plan(ni, all, cols, 4 * NT), &diag_plan)) != CT_OK) return s;
        std::vector<unsigned> slots;
        for (int i = 0; i < n; ++i) slots.push_back(inst(i).g0.plane);
        if ((s = upload_plan(make_plan(ni, all, slots, 4 * NT), &rec_plan)) != CT_OK) return s;
        if ((s = make_red(rec_plan, &rec_red)) != CT_OK) return s;
        if ((s = dalloc(&rec_mx, (size_t)std::max(1, rec_plan.ntasks) * sizeof(double))) != CT_OK) return s;
        if ((s = dalloc(&rec_dev, (size_t)3 * n * sizeof(double))) != CT_OK) return s;
        rec_host.assign((size_t)3 * n, 0.0);
        factor_plans.assign((size_t)maxlev, Plan{});
        for (int k = 0; k < maxlev; ++k) {
            std::vector<int> has;
            std::vector<unsigned> kc;
            for (int i = 0; i < n; ++i)
                if ((size_t)k < inst(i).lv.size()) {
                    has.push_back(i);
                    kc.push_back((unsigned)inst(i).lv[(size_t)k].g.nx * (unsigned)inst(i).lv[(size_t)k].g.ny);
                }
            if ((s = upload_plan(make_plan(ni, has, kc, NT), &factor_plans[(size_t)k])) != CT_OK) return s;
        }
    }
    // Tensor maps of the levels whose sweeps are staged (CT_SWEEP_TMA=0: none).
    {
        const char* e = std::getenv("CT_SWEEP_TMA");
        const bool want = !(e && e[0] == '0');
        bmaps.assign((size_t)2 * (maxdepth + 1), nullptr);
        fits.assign((size_t)maxdepth + 1, std::vector<char>((size_t)n, 0));
        for (int d = 0; d <= maxdepth; ++d) {
            std::vector<SweepMaps> hm[2] = {std::vector<SweepMaps>((size_t)n),
                                            std::vector<SweepMaps>((size_t)n)};
            for (int c = 0; c < 2; ++c) std::memset(hm[c].data(), 0, sizeof(SweepMaps) * (size_t)n);
            for (int i = 0; i < n; ++i) {
                if (!want || d >= small_k0(i) || !sweep_tma_fits(inst(i).lv[(size_t)d].g)) continue;
                const LevelView<float> v = inst(i).view<float>((size_t)d);
                fits[(size_t)d][(size_t)i] = make_sweep_maps(v, 0, &hm[0][(size_t)i]) &&
                                             make_sweep_maps(v, 1, &hm[1][(size_t)i]);
            }
            for (int c = 0; c < 2; ++c)
                if ((s = upload(&bmaps[(size_t)(2 * d + c)], hm[c])) != CT_OK) return s;
        }
    }
    std::vector<TailLevels<float>> ht((size_t)n);
    for (int i = 0; i < n; ++i) {
        const Solver& v = inst(i);
        TailLevels<float>& tl = ht[(size_t)i];
        std::memset(&tl, 0, sizeof tl);
        tl.n = (int)(v.lv.size() - v.small_k0);
        for (int q = 0; q < tl.n; ++q) tl.L[q] = v.view<float>(v.small_k0 + (size_t)q);
    }
    if ((s = upload(&small, ht)) != CT_OK) return s;
    if ((s = dalloc(&ctl, (size_t)n * sizeof(Ctl))) != CT_OK) return s;
    CT_BK(cudaMemsetAsync(ctl, 0, (size_t)n * sizeof(Ctl), st));
    CT_BK(cudaMallocHost(&h_ctl, (size_t)n * sizeof(Ctl)));
    std::memset(h_ctl, 0, (size_t)n * sizeof(Ctl));

    // Buckets by V-cycle depth.
    for (int d = 0; d <= maxdepth; ++d) {
        Bucket b;
        for (int i = 0; i < n; ++i)
            if (small_k0(i) == d) b.inst.push_back(i);
        if (b.inst.empty()) continue;
        b.depth = d;
        bk.push_back(std::move(b));
    }
    for (Bucket& b : bk) {
        if ((s = build_bucket(b)) != CT_OK) return s;
    }
    CT_BK(cudaStreamSynchronize(st));
    for (Bucket& b : bk) {
        if ((s = tune_bucket(b)) != CT_OK) return s;
    }
    for (Bucket& b : bk) {
        if ((s = record(b)) != CT_OK) return s;
        cudaEvent_t e = nullptr;
        CT_BK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        ev_done.push_back(e);
    }
    CT_BK(cudaStreamSynchronize(st));
    return CT_OK;
}

ct_status Batch::build_bucket(Bucket& b) {
    CT_BK(cudaStreamCreateWithFlags(&b.st, cudaStreamNonBlocking));
    CT_BK(cudaStreamCreateWithFlags(&b.st_body, cudaStreamNonBlocking));
    ct_status s;
    if ((s = dalloc(&b.bc, sizeof(BCtl))) != CT_OK) return s;
    CT_BK(cudaMemsetAsync(b.bc, 0, sizeof(BCtl), st));
    std::vector<unsigned> pairs, cols, rows;
    for (int i : b.inst) {
        const Solver& v = inst(i);
        pairs.push_back(v.n / 2);
        cols.push_back(v.g0.plane);
        rows.push_back(2u * (unsigned)v.g0.ny * (unsigned)v.g0.nz);
        b.mz = std::max(b.mz, v.g0.nz);
        TailLevels<float> tl;
        tl.n = (int)(v.lv.size() - v.small_k0);
        for (int q = 0; q < tl.n; ++q) tl.L[q] = v.view<float>(v.small_k0 + (size_t)q);
        b.smem = std::max(b.smem, small_smem_bytes(tl));
    }
    if ((s = upload_plan(make_plan(ni, b.inst, pairs, kVecChunk), &b.vec)) != CT_OK) return s;
    if ((s = upload_plan(make_plan(ni, b.inst, cols, kColChunk), &b.cols)) != CT_OK) return s;
    if ((s = upload_plan(make_plan(ni, b.inst, rows, dw ? kRowChunkDw : kRowChunk64), &b.rows)) != CT_OK) return s;
    // the start residual walks columns (double words) or rows (FP64)
    if ((s = make_red(dw ? b.cols : b.rows, &b.r_res)) != CT_OK) return s;
    if ((s = make_red(b.rows, &b.r_apply)) != CT_OK) return s;
    if ((s = make_red(b.vec, &b.r_update)) != CT_OK) return s;
    if ((s = make_red(b.vec, &b.r_dot)) != CT_OK) return s;
    if ((s = upload(&b.small_insts, b.inst)) != CT_OK) return s;
    b.sweep.assign((size_t)b.depth, Plan{});
    b.sweep_grid.assign((size_t)b.depth, Plan{});
    b.sweep0.assign((size_t)b.depth, Plan{});
    b.sweep0_grid.assign((size_t)b.depth, 0);
    b.restr.assign((size_t)b.depth, Plan{});
    b.sweep_tile.assign((size_t)b.depth, 512);
    b.sweep_grid_tile.assign((size_t)b.depth, 0);
    b.tma.assign((size_t)b.depth, 0);
    for (int d = 0; d < b.depth; ++d) {
        size_t nf = 0;
        for (int i : b.inst) nf += fits[(size_t)d][(size_t)i] ? 1 : 0;
        b.tma[(size_t)d] = nf == b.inst.size() ? 1 : nf > 0 ? 2 : 0;
    }
    b.restr_tile.assign((size_t)b.depth, 1024);
    return CT_OK;
}

// Picks the sweep and restriction tiles of each depth by timing the
// candidates on the bucket's own levels (the level arrays are scratch between
// solves, so the timing runs leave nothing behind that a solve reads).
ct_status Batch::tune_bucket(Bucket& b) {
    unsigned fixed = 0, fixed_tma = 0;
    if (const char* e = std::getenv("CT_BATCH_TILE")) fixed = (unsigned)std::atol(e);
    if (const char* e = std::getenv("CT_BATCH_TMA_TILES")) fixed_tma = (unsigned)std::atol(e);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    CT_BK(cudaEventCreate(&e0));
    CT_BK(cudaEventCreate(&e1));
    ct_status s = CT_OK;
    for (int d = 0; d < b.depth && s == CT_OK; ++d) {
        // staged instances (all of them in mode 1, the fitting ones in mode 2)
        // and grid-swept ones (all in mode 0, the rest in mode 2)
        std::vector<int> ins_t, ins_g;
        std::vector<unsigned> items_t, items_g, restr_items;
        for (int i : b.inst) {
            const Geo& g = inst(i).lv[(size_t)d].g;
            const Geo& c = inst(i).lv[(size_t)d + 1].g;
            if (b.tma[(size_t)d] != 0 && fits[(size_t)d][(size_t)i]) {
                ins_t.push_back(i);
                items_t.push_back((unsigned)sweep_tma_tiles(g));
            } else {
                ins_g.push_back(i);
                items_g.push_back((unsigned)g.ny * (unsigned)g.hx);
            }
            restr_items.push_back((unsigned)c.nx * (unsigned)c.ny * (unsigned)c.nz);
        }
        auto time_of = [&](auto&& launch) -> float {
            launch();  // warm
            float best = 1e30f;
            for (int rep = 0; rep < 3; ++rep) {
                cudaEventRecord(e0, b.st);
                launch();
                cudaEventRecord(e1, b.st);
                cudaEventSynchronize(e1);
                float ms = 0;
                cudaEventElapsedTime(&ms, e0, e1);
                best = std::min(best, ms);
            }
            return best;
        };
        // sweeps: the staged part's tiles per block, then the grid part's;
        // then, where anything is staged, the grid kernel over every instance,
        // which replaces the staged form if it is faster (small levels)
        float part_best[2] = {0.0f, 0.0f};
        for (int part = 0; part < 2 && s == CT_OK; ++part) {
            const bool tma = part == 0;
            const std::vector<int>& ins = tma ? ins_t : ins_g;
            const std::vector<unsigned>& items = tma ? items_t : items_g;
            if (ins.empty()) continue;
            std::vector<unsigned> cands;
            if (tma && fixed_tma) cands.push_back(fixed_tma);
            else if (tma) cands.assign(std::begin(kTmaTiles), std::end(kTmaTiles));
            else if (fixed) cands.push_back(fixed);
            else cands.assign(std::begin(kSweepTiles), std::end(kSweepTiles));
            float best = 1e30f;
            for (unsigned tile : cands) {
                Plan p;
                if ((s = upload_plan(make_plan(ni, ins, items, tile), &p)) != CT_OK) break;
                CT_BK(cudaStreamSynchronize(st));
                const float t = cands.size() == 1 ? 0.0f : time_of([&] {
                    if (tma)
                        launch_b_sweep_tma(b.st, p, bmaps[(size_t)(2 * d + 1)], views[(size_t)d],
                                           views[(size_t)d], 1, false, false, b.mz, ctl, b.bc, Cond{0, 0});
                    else
                        launch_b_sweep(b.st, p, views[(size_t)d], views[(size_t)d], 1, false, false, b.mz, ctl);
                });
                if (t < best) {
                    best = t;
                    // staged part (or everything in mode 0) in sweep, the grid
                    // part of a mixed depth in sweep_grid
                    if (tma || b.tma[(size_t)d] == 0) {
                        b.sweep[(size_t)d] = p;
                        b.sweep_tile[(size_t)d] = tile;
                    } else {
                        b.sweep_grid[(size_t)d] = p;
                        b.sweep_grid_tile[(size_t)d] = tile;
                    }
                }
            }
            part_best[part] = best;
        }
        if (s == CT_OK && b.tma[(size_t)d] != 0 && !fixed_tma) {
            std::vector<unsigned> items;
            for (int i : b.inst) {
                const Geo& g = inst(i).lv[(size_t)d].g;
                items.push_back((unsigned)g.ny * (unsigned)g.hx);
            }
            const float staged = part_best[0] + (ins_g.empty() ? 0.0f : part_best[1]);
            std::vector<unsigned> cands;
            if (fixed) cands.push_back(fixed);
            else cands.assign(std::begin(kSweepTiles), std::end(kSweepTiles));
            for (unsigned tile : cands) {
                Plan p;
                if ((s = upload_plan(make_plan(ni, b.inst, items, tile), &p)) != CT_OK) break;
                CT_BK(cudaStreamSynchronize(st));
                const float t = time_of([&] {
                    launch_b_sweep(b.st, p, views[(size_t)d], views[(size_t)d], 1, false, false, b.mz, ctl);
                });
                if (t < staged && (b.tma[(size_t)d] != 0 || t < part_best[1])) {
                    b.tma[(size_t)d] = 0;
                    b.sweep[(size_t)d] = p;
                    b.sweep_tile[(size_t)d] = tile;
                    part_best[1] = t;
                }
            }
        }
        // the x = 0 sweep, where the level stays staged: it has no
        // neighbour values to stage, and the grid kernel (every plane's loads
        // of a column in flight at once) may move its three operand streams
        // faster
        // (CT_SWEEP0_GRID=0 keeps it staged, =1 takes the grid kernel)
        const char* e0 = std::getenv("CT_SWEEP0_GRID");
        const int mode0 = !e0 ? 1 : e0[0] == '0' ? 0 : 2;  // staged, timed, grid
        if (s == CT_OK && b.tma[(size_t)d] != 0 && (mode0 == 2 || (mode0 == 1 && !fixed_tma))) {
            std::vector<unsigned> items;
            for (int i : b.inst) {
                const Geo& g = inst(i).lv[(size_t)d].g;
                items.push_back((unsigned)g.ny * (unsigned)g.hx);
            }
            float best = mode0 == 2 ? 1e30f : time_of([&] {
                launch_b_sweep_tma(b.st, b.sweep[(size_t)d], bmaps[(size_t)(2 * d)], views[(size_t)d],
                                   views[(size_t)d], 0, true, false, b.mz, ctl, b.bc, Cond{0, 0});
                if (b.tma[(size_t)d] == 2)
                    launch_b_sweep(b.st, b.sweep_grid[(size_t)d], views[(size_t)d], views[(size_t)d], 0, true,
                                   false, b.mz, ctl);
            });
            std::vector<unsigned> cands;
            if (fixed) cands.push_back(fixed);
            else cands.assign(std::begin(kSweepTiles), std::end(kSweepTiles));
            for (unsigned tile : cands) {
                Plan p;
                if ((s = upload_plan(make_plan(ni, b.inst, items, tile), &p)) != CT_OK) break;
                CT_BK(cudaStreamSynchronize(st));
                const float t = time_of([&] {
                    launch_b_sweep(b.st, p, views[(size_t)d], views[(size_t)d], 0, true, false, b.mz, ctl);
                });
                if (t < best) {
                    best = t;
                    b.sweep0[(size_t)d] = p;
                    b.sweep0_grid[(size_t)d] = 1;
                }
            }
        }
        // restriction
        {
            std::vector<unsigned> cands;
            if (fixed) cands.push_back(fixed);
            else cands.assign(std::begin(kRestrictTiles), std::end(kRestrictTiles));
            float best = 1e30f;
            for (unsigned tile : cands) {
                Plan p;
                if ((s = upload_plan(make_plan(ni, b.inst, restr_items, tile), &p)) != CT_OK) break;
                CT_BK(cudaStreamSynchronize(st));
                const float t = cands.size() == 1 ? 0.0f : time_of([&] {
                    launch_b_restrict(b.st, p, views[(size_t)d], views[(size_t)d + 1], ctl);
                });
                if (t < best) {
                    best = t;
                    b.restr[(size_t)d] = p;
                    b.restr_tile[(size_t)d] = tile;
                }
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (s != CT_OK) return s;
    CT_BK(cudaGetLastError());
    CT_BK(cudaStreamSynchronize(b.st));
    return CT_OK;
}

void Batch::sweep(Bucket& b, cudaStream_t s, int d, int color, bool zero_x, bool prolong, Cond cond) {
    const LevelView<float>* L = views[(size_t)d];
    const LevelView<float>* C = views[(size_t)d + 1];
    if (zero_x && b.sweep0_grid[(size_t)d]) {
        launch_b_sweep(s, b.sweep0[(size_t)d], L, C, color, true, prolong, b.mz, ctl);
        return;
    }
    if (b.tma[(size_t)d]) {
        launch_b_sweep_tma(s, b.sweep[(size_t)d], bmaps[(size_t)(2 * d + color)], L, C, color, zero_x,
                           prolong, b.mz, ctl, b.bc, cond);
        if (b.tma[(size_t)d] == 2)  // the instances that do not fit a tile row
            launch_b_sweep(s, b.sweep_grid[(size_t)d], L, C, color, zero_x, prolong, b.mz, ctl);
    } else {
        launch_b_sweep(s, b.sweep[(size_t)d], L, C, color, zero_x, prolong, b.mz, ctl);
    }
}

void Batch::vcycle(Bucket& b, cudaStream_t s, Cond cond) {
    // algorithmic bytes per level cell, as in the single solver
    for (int d = 0; d < b.depth; ++d) {
        const LevelView<float>* L = views[(size_t)d];
        const LevelView<float>* C = views[(size_t)d + 1];
        const double N = cells_of(b, d);
        const std::string lvl = "_d" + std::to_string(d);
        enq(s, "b_sweep0" + lvl, N * 10,
            [&] { sweep(b, s, d, 0, true, false, cond); });
        enq(s, "b_sweep" + lvl, N * 20,
            [&] { sweep(b, s, d, 1, false, false, cond); });
        enq(s, "b_restrict" + lvl, N * 25, [&] { launch_b_restrict(s, b.restr[(size_t)d], L, C, ctl); });
    }
    double smb = 0;
    for (int i : b.inst) {
        const Solver& v = inst(i);
        for (size_t k = v.small_k0; k < v.lv.size(); ++k) {
            const Geo& g = v.lv[k].g;
            smb += (double)g.nx * g.ny * g.nz * (4 * 4 + 4 + 2 * 4 + 16);
        }
    }
    enq(s, "b_small", smb, [&] {
        const cudaError_t e =
            launch_b_small(s, b.small_insts, (int)b.inst.size(), small, b.smem, b.mz, ctl, b.bc, cond);
        if (e != cudaSuccess && launch_error == cudaSuccess) launch_error = e;
    });
    for (int d = b.depth; d-- > 0;) {
        const double N = cells_of(b, d);
        const std::string lvl = "_d" + std::to_string(d);
        enq(s, "b_sweep" + lvl, N * 21,
            [&] { sweep(b, s, d, 1, false, true, cond); });
        enq(s, "b_sweep" + lvl, N * 20,
            [&] { sweep(b, s, d, 0, false, false, cond); });
    }
}

void Batch::enqueue_init(Bucket& b, cudaStream_t s, Cond cond) {
    const double N = cells_of(b, -1);
    if (!dw) {
        enq(s, "b_residual", N * 56, [&] { launch_b_residual64(s, b.rows, bi, ctl, b.r_res, b.bc, cond); });
        return;
    }
    enq(s, "b_fold", N * 32, [&] { launch_b_fold(s, b.vec, bi, ctl, 0); });
    enq(s, "b_residual", N * 56,
        [&] { launch_b_residual(s, b.cols, bi, ctl, b.r_res, 1, b.bc, cond); });
}

void Batch::enqueue_body(Bucket& b, cudaStream_t s, Cond cond) {
    const double N = cells_of(b, -1);
    launch_b_guard(s, b.bc, cond);
    vcycle(b, s, cond);
    if (!dw) {
        enq(s, "b_dot", N * 20, [&] { launch_b_dot64(s, b.vec, bi, ctl, b.r_dot, b.bc, cond); });
        enq(s, "b_update_p", N * 20, [&] { launch_b_update_p64(s, b.vec, bi, ctl); });
        enq(s, "b_apply", N * 36, [&] { launch_b_apply64(s, b.rows, bi, ctl, b.r_apply, b.bc, cond); });
        enq(s, "b_update_xr", N * 52,
            [&] { launch_b_update64(s, b.vec, bi, ctl, b.r_update, b.bc, cond); });
        return;
    }
    enq(s, "b_dot", N * 20, [&] { launch_b_dot(s, b.vec, bi, ctl, b.r_dot, b.bc, cond); });
    enq(s, "b_update_p", N * 20, [&] { launch_b_update_p(s, b.vec, bi, ctl); });
    enq(s, "b_apply", N * 36, [&] { launch_b_apply(s, b.rows, bi, ctl, b.r_apply, b.bc, cond); });
    enq(s, "b_update_xr", N * 52,
        [&] { launch_b_update(s, b.vec, bi, ctl, b.r_update, b.bc, cond); });
    // residual replacement of the instances whose first phase just ended
    // (blocks of the other instances return at entry)
    enq(s, "b_fold_pe", 0, [&] { launch_b_fold(s, b.vec, bi, ctl, 1); });
    enq(s, "b_residual_pe", 0,
        [&] { launch_b_residual(s, b.cols, bi, ctl, b.r_res, 0, b.bc, cond); });
}

ct_status Batch::record(Bucket& b) {
    if (!use_cond) return CT_OK;
    cudaGraph_t graph = nullptr;
    CT_BK(cudaGraphCreate(&graph, 0));
    cudaGraphConditionalHandle h{};
    bool ok = cudaGraphConditionalHandleCreate(&h, graph, 1u, cudaGraphCondAssignDefault) == cudaSuccess;
    if (ok)
        ok = cudaStreamBeginCaptureToGraph(b.st, graph, nullptr, nullptr, 0,
                                           cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    if (ok) {
        enqueue_init(b, b.st, Cond{h, 1});
        cudaStreamCaptureStatus cst;
        const cudaGraphNode_t* deps = nullptr;
        size_t ndeps = 0;
        cudaGraph_t cg = nullptr;
        ok = cudaStreamGetCaptureInfo(b.st, &cst, nullptr, &cg, &deps, nullptr, &ndeps) == cudaSuccess;
        cudaGraphNode_t cnode = nullptr;
        cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
        if (ok) {
            cp.conditional.handle = h;
            cp.conditional.type = cudaGraphCondTypeWhile;
            cp.conditional.size = 1;
            ok = cudaGraphAddNode(&cnode, cg, deps, nullptr, ndeps, &cp) == cudaSuccess;
        }
        if (ok)
            ok = cudaStreamBeginCaptureToGraph(b.st_body, cp.conditional.phGraph_out[0], nullptr,
                                               nullptr, 0, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
        if (ok) {
            enqueue_body(b, b.st_body, Cond{h, 1});
            cudaGraph_t bg = nullptr;
            ok = cudaStreamEndCapture(b.st_body, &bg) == cudaSuccess;
        }
        if (ok)
            ok = cudaStreamUpdateCaptureDependencies(b.st, &cnode, nullptr, 1,
                                                     cudaStreamSetCaptureDependencies) == cudaSuccess;
        cudaGraph_t outg = nullptr;
        const bool ended = cudaStreamEndCapture(b.st, &outg) == cudaSuccess;
        ok = ok && ended;
        if (ok) ok = cudaGraphInstantiate(&b.gx, graph, 0) == cudaSuccess;
    }
    cudaGraphDestroy(graph);
    if (launch_error != cudaSuccess)
        return fail(CT_CUDA_ERROR, "batch: small-level kernel launch failed: %s", cudaGetErrorString(launch_error));
    if (!ok) {
        cudaGetLastError();
        if (b.gx) cudaGraphExecDestroy(b.gx);
        b.gx = nullptr;
        use_cond = false;  // every bucket falls back to host-driven launches
    }
    return CT_OK;
}

// set_dt for every instance in 1 + (levels) launches: 1/dt per instance goes
// into its control block, then the batched diagonal and factor kernels run
// the single solver's per-column arithmetic (same bits as Solver::set_dt).
ct_status Batch::set_dt(const double* dt) {
    const TraceRange trace("ct_batch_set_dt");
    for (int i = 0; i < ni; ++i) {
        const double v = dt ? dt[i] : 0.0;
        if (!(v >= 0) || !std::isfinite(v)) return fail(CT_BAD_ARG, "ct_batch_set_dt: dt[%d] must be >= 0", i);
        const double inv = v > 0 ? 1.0 / v : 0.0;
        inst(i).inv_dt = inv;
        h_ctl[i].inv_dt = inv;
    }
    CT_BK(cudaMemcpyAsync(ctl, h_ctl, (size_t)ni * sizeof(Ctl), cudaMemcpyHostToDevice, st));
    launch_b_diag(st, diag_plan, bi, ctl);
    for (size_t k = 0; k < factor_plans.size(); ++k) launch_b_factor(st, factor_plans[k], views[k], ctl);
    CT_BK(cudaGetLastError());
    CT_BK(cudaStreamSynchronize(st));  // h_ctl is written again by the next call
    return CT_OK;
}

ct_status Batch::solve(double tol, int maxit, ct_stats* out) {
    const TraceRange trace("ct_batch_solve");
    if (!(tol >= 0)) return fail(CT_BAD_ARG, "ct_batch_solve: tol must be >= 0");
    if (maxit > 100000000) return fail(CT_BAD_ARG, "ct_batch_solve: maxit above 1e8");
    for (int i = 0; i < ni; ++i) {
        Solver& v = inst(i);
        Ctl& c = h_ctl[i];
        std::memset(&c, 0, sizeof c);
        c.tol = tol;
        c.maxit = maxit;
        c.inv_dt = v.inv_dt;
        c.stop = std::max(tol, rr_thr);
        c.x_zero = v.x_zero ? 1 : 0;
        v.x_zero = false;
    }
    CT_BK(cudaMemcpyAsync(ctl, h_ctl, (size_t)ni * sizeof(Ctl), cudaMemcpyHostToDevice, st));
    for (Bucket& b : bk) {
        const BCtl c{(int)b.inst.size(), 0, maxit + 2, 0};
        CT_BK(cudaMemcpyAsync(b.bc, &c, sizeof c, cudaMemcpyHostToDevice, st));
    }
    CT_BK(cudaStreamSynchronize(st));  // the pageable BCtl copies are done
    CT_BK(cudaEventRecord(ev_start, st));
    const Cond none{0, 0};
    for (size_t q = 0; q < bk.size(); ++q) {
        Bucket& b = bk[q];
        CT_BK(cudaStreamWaitEvent(b.st, ev_start, 0));
        if (use_cond && b.gx && !prof) {
            CT_BK(cudaGraphLaunch(b.gx, b.st));
        } else {
            // Host-driven: direct launches with a check of the bucket's
            // active count after every body.
            enqueue_init(b, b.st, none);
            BCtl hc{};
            for (int it = 0; it <= maxit + 2; ++it) {
                CT_BK(cudaMemcpyAsync(&hc, b.bc, sizeof hc, cudaMemcpyDeviceToHost, b.st));
                CT_BK(cudaStreamSynchronize(b.st));
                if (hc.active <= 0) break;
                enqueue_body(b, b.st, none);
            }
        }
        CT_BK(cudaGetLastError());
        if (launch_error != cudaSuccess)
            return fail(CT_CUDA_ERROR, "batch: small-level kernel launch failed: %s",
                        cudaGetErrorString(launch_error));
        CT_BK(cudaEventRecord(ev_done[q], b.st));
        CT_BK(cudaStreamWaitEvent(st, ev_done[q], 0));
    }
    CT_BK(cudaMemcpyAsync(h_ctl, ctl, (size_t)ni * sizeof(Ctl), cudaMemcpyDeviceToHost, st));
    CT_BK(cudaStreamSynchronize(st));
    int nbreak = 0, nconv = 0, nerr = 0;
    for (int i = 0; i < ni; ++i) {
        const Ctl& c = h_ctl[i];
        Solver& v = inst(i);
        if (c.bb_zero) {  // no heat in: x = 0 (src/pcg3d_cpu.cpp:146)
            CT_BK(cudaMemsetAsync(v.x, 0, (size_t)v.n * 8, st));
            if (v.xwc) CT_BK(cudaMemsetAsync(v.xwc, 0, (size_t)v.n * 8, st));
        }
        if (out) {
            out[i].iters = c.iter;
            out[i].relres = c.relres;
            out[i].converged = c.converged;
            out[i].breakdown = c.breakdown;
        }
        nbreak += c.breakdown ? 1 : 0;
        nerr += c.err ? 1 : 0;
        nconv += c.converged ? 1 : 0;
    }
    CT_BK(cudaStreamSynchronize(st));
    if (nerr)
        return fail(CT_TIMEOUT, "a bounded wait for staged level data ran out in %d of %d instances", nerr, ni);
    if (nbreak) return fail(CT_BREAKDOWN, "PCG breakdown in %d of %d instances", nbreak, ni);
    if (nconv < ni) return fail(CT_NOT_CONVERGED, "%d of %d instances not converged", ni - nconv, ni);
    return CT_OK;
}

}  // namespace ct

// ---- C ABI ----------------------------------------------------------------

struct ct_batch {
    ct::Batch impl;
};

using ct::fail;

#define CT_BATCH_OK(b) \
    if (!(b)) return fail(CT_BAD_ARG, "%s: null batch", __func__)
#define CT_BATCH_INST(b, i)                                                     \
    do {                                                                        \
        CT_BATCH_OK(b);                                                         \
        if ((i) < 0 || (i) >= (b)->impl.ni)                                     \
            return fail(CT_BAD_ARG, "%s: instance %d out of range", __func__, i); \
    } while (0)

extern "C" {

ct_status ct_batch_create(int n, const ct_model* const* models, ct_batch** out) {
    return ct_batch_create_prec(n, models, CT_MG_FP32_FLEX_DW, out);
}

ct_status ct_batch_create_prec(int n, const ct_model* const* models, ct_precision prec, ct_batch** out) {
    if (!out) return fail(CT_BAD_ARG, "ct_batch_create: null output");
    *out = nullptr;
    ct_batch* b = new (std::nothrow) ct_batch();
    if (!b) return fail(CT_OUT_OF_MEMORY, "host allocation failed");
    const ct_status s = b->impl.create(n, models, nullptr, prec);
    if (s != CT_OK) {
        delete b;
        return s;
    }
    *out = b;
    return CT_OK;
}

ct_status ct_batch_create_cases(int n, const ct_case* const* cases, const int* nx, const int* ny,
                                const int* with_tsv, ct_batch** out) {
    return ct_batch_create_cases_prec(n, cases, nx, ny, with_tsv, CT_MG_FP32_FLEX_DW, out);
}

ct_status ct_batch_create_cases_prec(int n, const ct_case* const* cases, const int* nx, const int* ny,
                                     const int* with_tsv, ct_precision prec, ct_batch** out) {
    if (!out) return fail(CT_BAD_ARG, "ct_batch_create_cases: null output");
    *out = nullptr;
    if (n < 1 || !cases || !nx || !ny) return fail(CT_BAD_ARG, "ct_batch_create_cases: bad arguments");
    std::vector<ct::DeviceBuild> builds((size_t)n);
    for (int i = 0; i < n; ++i) {
        const ct_status s = ct::case_build(cases[i], nx[i], ny[i], with_tsv ? with_tsv[i] != 0 : true,
                                           &builds[(size_t)i]);
        if (s != CT_OK) return s;
    }
    ct_batch* b = new (std::nothrow) ct_batch();
    if (!b) return fail(CT_OUT_OF_MEMORY, "host allocation failed");
    const ct_status s = b->impl.create(n, nullptr, builds.data(), prec);
    if (s != CT_OK) {
        delete b;
        return s;
    }
    *out = b;
    return CT_OK;
}

ct_status ct_batch_destroy(ct_batch* b) {
    delete b;
    return CT_OK;
}

ct_status ct_batch_size(const ct_batch* b, int* n) {
    CT_BATCH_OK(b);
    if (!n) return fail(CT_BAD_ARG, "ct_batch_size: null");
    *n = b->impl.ni;
    return CT_OK;
}

ct_status ct_batch_set_dt(ct_batch* b, const double* dt) {
    CT_BATCH_OK(b);
    return b->impl.set_dt(dt);
}

ct_status ct_batch_set_x_zero(ct_batch* b) {
    CT_BATCH_OK(b);
    for (int i = 0; i < b->impl.ni; ++i) {
        const ct_status s = ct_set_x_zero(b->impl.sv[(size_t)i].get());
        if (s != CT_OK) return s;
    }
    return CT_OK;
}

ct_status ct_batch_set_rhs_steady(ct_batch* b) {
    CT_BATCH_OK(b);
    for (int i = 0; i < b->impl.ni; ++i) {
        const ct_status s = ct_set_rhs_steady(b->impl.sv[(size_t)i].get());
        if (s != CT_OK) return s;
    }
    return CT_OK;
}

ct_status ct_batch_set_rhs_transient(ct_batch* b) {
    CT_BATCH_OK(b);
    ct::Batch& B = b->impl;
    for (ct::Batch::Bucket& k : B.bk) {
        if (B.dw) ct::launch_b_fold(B.st, k.vec, B.bi, B.ctl, 0);
        ct::launch_b_rhs_transient(B.st, k.vec, B.bi, B.ctl);
    }
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(CT_CUDA_ERROR, "ct_batch_set_rhs_transient: %s", cudaGetErrorString(e));
    return CT_OK;
}

ct_status ct_batch_set_power(ct_batch* b, int i, const double* P) {
    CT_BATCH_INST(b, i);
    return ct_set_power(b->impl.sv[(size_t)i].get(), P);
}

ct_status ct_batch_set_power_device(ct_batch* b, int i, const double* P_dev) {
    CT_BATCH_INST(b, i);
    return ct_set_power_device(b->impl.sv[(size_t)i].get(), P_dev);
}

ct_status ct_batch_set_x(ct_batch* b, int i, const double* T) {
    CT_BATCH_INST(b, i);
    return ct_set_x(b->impl.sv[(size_t)i].get(), T);
}

ct_status ct_batch_solve(ct_batch* b, double tol, int maxit, ct_stats* stats) {
    CT_BATCH_OK(b);
    return b->impl.solve(tol, maxit, stats);
}

ct_status ct_batch_step_transient(ct_batch* b, const double* dt, double tol, int maxit,
                                  ct_stats* stats) {
    CT_BATCH_OK(b);
    if (!dt) return fail(CT_BAD_ARG, "ct_batch_step_transient: null dt");
    ct_status s = b->impl.set_dt(dt);
    if (s != CT_OK) return s;
    s = ct_batch_set_rhs_transient(b);
    if (s != CT_OK) return s;
    return b->impl.solve(tol, maxit, stats);
}

ct_status ct_batch_get_x(ct_batch* b, int i, double* T) {
    CT_BATCH_INST(b, i);
    return ct_get_x(b->impl.sv[(size_t)i].get(), T);
}

ct_status ct_batch_true_relres(ct_batch* b, int i, double* out) {
    CT_BATCH_INST(b, i);
    return ct_true_relres(b->impl.sv[(size_t)i].get(), out);
}

ct_status ct_batch_step_record(ct_batch* b, int i, double dt, ct_step_record* out) {
    CT_BATCH_INST(b, i);
    return ct_solver_step_record(b->impl.sv[(size_t)i].get(), dt, out);
}

ct_status ct_batch_profile_solve(ct_batch* b, double tol, int maxit, ct_stats* stats,
                                 ct_kernel_time* out, int max, int* n) {
    CT_BATCH_OK(b);
    ct::Batch& B = b->impl;
    B.prof = true;
    B.prof_log.clear();
    const ct_status s = B.solve(tol, maxit, stats);
    B.prof = false;
    cudaDeviceSynchronize();
    std::vector<ct_kernel_time> agg;
    for (const ct::ProfEntry& e : B.prof_log) {
        float ms = 0;
        cudaEventElapsedTime(&ms, e.a, e.b);
        cudaEventDestroy(e.a);
        cudaEventDestroy(e.b);
        ct_kernel_time* k = nullptr;
        for (ct_kernel_time& a : agg)
            if (e.name == a.name) k = &a;
        if (!k) {
            agg.push_back(ct_kernel_time{});
            k = &agg.back();
            std::snprintf(k->name, sizeof k->name, "%s", e.name.c_str());
        }
        k->launches += 1;
        k->total_ms += ms;
        k->bytes += e.bytes;
    }
    B.prof_log.clear();
    if (n) *n = (int)agg.size();
    for (int k = 0; k < (int)agg.size() && k < max && out; ++k) out[k] = agg[(size_t)k];
    return s;
}

ct_status ct_batch_stream(const ct_batch* b, void** stream) {
    CT_BATCH_OK(b);
    if (!stream) return fail(CT_BAD_ARG, "ct_batch_stream: null");
    *stream = (void*)b->impl.st;
    return CT_OK;
}

ct_status ct_batch_step_records(ct_batch* b, const double* dt, ct_step_record* out) {
    CT_BATCH_OK(b);
    if (!dt || !out) return fail(CT_BAD_ARG, "ct_batch_step_records: null");
    ct::Batch& B = b->impl;
    if (B.dw)
        for (ct::Batch::Bucket& k : B.bk) ct::launch_b_fold(B.st, k.vec, B.bi, B.ctl, 0);
    ct::launch_b_step_record(B.st, B.rec_plan, B.bi, B.rec_red, B.rec_mx, B.rec_dev);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(B.rec_host.data(), B.rec_dev, B.rec_host.size() * sizeof(double),
                            cudaMemcpyDeviceToHost, B.st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(B.st);
    if (e != cudaSuccess) return fail(CT_CUDA_ERROR, "ct_batch_step_records: %s", cudaGetErrorString(e));
    for (int i = 0; i < B.ni; ++i) {
        out[i].T_max = B.rec_host[(size_t)3 * i];
        out[i].q_out = B.rec_host[(size_t)3 * i + 1];
        out[i].q_stored = B.rec_host[(size_t)3 * i + 2] / dt[i];
    }
    return CT_OK;
}

ct_status ct_batch_num_buckets(const ct_batch* b, int* nbuckets) {
    CT_BATCH_OK(b);
    if (!nbuckets) return fail(CT_BAD_ARG, "ct_batch_num_buckets: null");
    *nbuckets = (int)b->impl.bk.size();
    return CT_OK;
}

ct_status ct_batch_bucket_info(const ct_batch* b, int k, int* ninst, int* depth, unsigned* sweep_tiles,
                               unsigned* restrict_tiles, int* staged) {
    CT_BATCH_OK(b);
    if (k < 0 || k >= (int)b->impl.bk.size()) return fail(CT_BAD_ARG, "ct_batch_bucket_info: bad bucket");
    const ct::Batch::Bucket& B = b->impl.bk[(size_t)k];
    if (ninst) *ninst = (int)B.inst.size();
    if (depth) *depth = B.depth;
    for (int d = 0; d < B.depth; ++d) {
        if (sweep_tiles) sweep_tiles[d] = B.sweep_tile[(size_t)d];
        if (restrict_tiles) restrict_tiles[d] = B.restr_tile[(size_t)d];
        if (staged) staged[d] = B.tma[(size_t)d];
    }
    return CT_OK;
}

}  // extern "C"
