// cthermal.hpp - cuda-thermal's C++ solver interface on top of libcthermal's
// C ABI: the classes and functions of src/stack3d.h (model), src/pcg3d.h
// (GpuPcg, gpu_pcg, true_relres, gpu_use_graphs, gpu_last_setup) and
// src/transient3d.h (run_transient), with the same names and meaning, so code
// written against the reference's headers compiles against this one; and the
// case files of src/case3d.h (CaseSpec, load_case, build_case_model,
// export_3dice).
//
// Differences from the reference, all deliberate:
//  - errors throw cthermal::Error (a std::runtime_error carrying the
//    ct_status) instead of calling exit(1); non-convergence is still reported
//    through PcgStats.converged, as in the reference;
//  - GpuPcg takes an optional third argument, the V-cycle precision
//    (default CT_MG_FP32_FLEX: FP32 V-cycle inside flexible FP64 PCG);
//    CT_MG_FP64 is the reference's -DMG_DOUBLE arithmetic, CT_MG_FP32 its
//    default build's;
//  - there is no CpuPcg: the CPU solver of the reference is this project's
//    test oracle, not part of the library.
// Names live in namespace cthermal and are also brought into the global
// namespace (as the reference declares them) unless CTHERMAL_NO_GLOBAL_NAMES
// is defined.
#pragma once

#include <algorithm>
#include <chrono>
#include <stdexcept>
#include <string>
#include <vector>

#include "cthermal.h"
#include "cthermal_model.h"

namespace cthermal {

using Real = double;
constexpr int MAXZ = CT_MAXZ;

struct Error : std::runtime_error {
    ct_status status;
    Error(ct_status s, const std::string& what) : std::runtime_error(what), status(s) {}
};

inline void check(ct_status s) {
    if (s != CT_OK) throw Error(s, std::string(ct_status_string(s)) + ": " + ct_last_error());
}

// ---- model (src/stack3d.h) -------------------------------------------------

struct Layer {
    std::string name;
    double thickness;  // m
    double k;          // W/(m K)
    double rho_c;      // J/(m^3 K)
    int ncells;
    bool active;
};

struct Model3D {
    int nx = 0, ny = 0, nz = 0;
    double Lx = 0, Ly = 0, dx = 0, dy = 0;
    double h_top = 0, h_bot = 0;
    double T_amb = 25.0;
    double tsv_k = 400.0, tsv_rho_c = 3.45e6;
    std::vector<Layer> layers;
    std::vector<int> plane_layer;
    std::vector<double> dz;
    std::vector<double> tsv_frac;
    std::vector<double> P;
    std::vector<float> gE, gN, gU, gB, cap;
    bool finalized = false;

    size_t nxy() const { return (size_t)nx * ny; }
    size_t ncells() const { return nxy() * nz; }
    size_t idx(int i, int j, int l) const { return ((size_t)l * ny + j) * nx + i; }
    int layer_index(const std::string& name) const {
        for (size_t L = 0; L < layers.size(); ++L)
            if (layers[L].name == name) return (int)L;
        return -1;
    }
    ct_grid grid() const { return ct_grid{nx, ny, nz, Lx, Ly, dx, dy}; }
    std::vector<ct_layer> c_layers() const {
        std::vector<ct_layer> v;
        for (const Layer& L : layers) v.push_back(ct_layer{L.thickness, L.k, L.rho_c, L.ncells, L.active ? 1 : 0});
        return v;
    }
    // The ct_model view of the finalized arrays.
    ct_model view() const {
        if (!finalized) throw Error(CT_NOT_FINALIZED, "Model3D used before finalize()");
        return ct_model{nx, ny, nz, dx, dy, gE.data(), gN.data(), gU.data(), gB.data(), cap.data(), P.data()};
    }
};

inline double eff_kz(double k, double kc, double f) { return ct_eff_kz(k, kc, f); }
inline double eff_kxy(double k, double kc, double f) { return ct_eff_kxy(k, kc, f); }

inline Model3D build_model(const std::vector<Layer>& layers, int nx, int ny, double Lx, double Ly,
                           double h_top, double h_bot) {
    Model3D m;
    m.layers = layers;
    m.nx = nx;
    m.ny = ny;
    m.Lx = Lx;
    m.Ly = Ly;
    m.dx = Lx / nx;
    m.dy = Ly / ny;
    m.h_top = h_top;
    m.h_bot = h_bot;
    std::vector<ct_layer> cl = m.c_layers();
    int pl[CT_MAXZ];
    double dz[CT_MAXZ];
    check(ct_model_planes(cl.data(), (int)cl.size(), &m.nz, pl, dz));
    m.plane_layer.assign(pl, pl + m.nz);
    m.dz.assign(dz, dz + m.nz);
    m.tsv_frac.assign(m.ncells(), 0.0);
    m.P.assign(m.ncells(), 0.0);
    return m;
}

inline void finalize(Model3D& m) {
    const size_t n = m.ncells();
    m.gE.assign(n, 0.0f);
    m.gN.assign(n, 0.0f);
    m.gU.assign(n, 0.0f);
    m.cap.assign(n, 0.0f);
    m.gB.assign(m.nxy(), 0.0f);
    const ct_grid g = m.grid();
    std::vector<ct_layer> cl = m.c_layers();
    check(ct_model_finalize(&g, cl.data(), m.plane_layer.data(), m.dz.data(), m.h_top, m.h_bot,
                            m.tsv_k, m.tsv_rho_c, m.tsv_frac.data(), m.gE.data(), m.gN.data(),
                            m.gU.data(), m.gB.data(), m.cap.data()));
    m.finalized = true;
}

inline std::vector<Layer> default_stack() {
    return {{"Si tier 2 (bottom)", 50e-6, 130.0, 1.66e6, 2, true},
            {"bond + BEOL", 10e-6, 2.0, 1.70e6, 1, false},
            {"Si tier 1 (top)", 50e-6, 130.0, 1.66e6, 2, true},
            {"TIM", 25e-6, 5.0, 2.00e6, 1, false},
            {"Cu spreader", 1e-3, 400.0, 3.45e6, 4, false}};
}

inline Model3D default_model(int nx, int ny) {
    return build_model(default_stack(), nx, ny, 10e-3, 10e-3, 2e4, 0.0);
}

inline void add_power_block(Model3D& m, int layer, double x0, double y0, double w, double h,
                            double watts) {
    const ct_grid g = m.grid();
    std::vector<ct_layer> cl = m.c_layers();
    check(ct_model_add_power_block(&g, cl.data(), m.plane_layer.data(), layer, x0, y0, w, h, watts,
                                   m.P.data()));
}

inline void add_uniform_power(Model3D& m, int layer, double watts) {
    add_power_block(m, layer, 0, 0, m.Lx, m.Ly, watts);
}

inline void add_hotspot(Model3D& m, int layer, double xc, double yc, double size, double watts) {
    const ct_grid g = m.grid();
    check(ct_model_add_hotspot(&g, m.plane_layer.data(), layer, xc, yc, size, watts, m.P.data()));
}

inline void add_tsv_region(Model3D& m, int layer, double x0, double y0, double w, double h,
                           double f) {
    const ct_grid g = m.grid();
    check(ct_model_add_tsv_region(&g, m.plane_layer.data(), layer, x0, y0, w, h, f,
                                  m.tsv_frac.data()));
    m.finalized = false;
}

inline double total_power(const Model3D& m) {
    const ct_grid g = m.grid();
    return ct_model_total_power(&g, m.P.data());
}

template <class Vec>
double heat_out(const Model3D& m, const Vec& T) {
    const ct_grid g = m.grid();
    std::vector<double> t(T.begin(), T.end());
    return ct_model_heat_out(&g, m.gU.data(), m.gB.data(), t.data());
}

template <class Vec>
double heat_stored(const Model3D& m, const Vec& T_old, const Vec& T_new, double dt) {
    const ct_grid g = m.grid();
    std::vector<double> a(T_old.begin(), T_old.end()), b(T_new.begin(), T_new.end());
    return ct_model_heat_stored(&g, m.cap.data(), a.data(), b.data(), dt);
}

inline std::vector<double> analytic_1d(const Model3D& m) {
    const ct_grid g = m.grid();
    std::vector<ct_layer> cl = m.c_layers();
    std::vector<double> T(m.nz);
    check(ct_model_analytic_1d(&g, cl.data(), m.plane_layer.data(), m.dz.data(), m.h_top,
                               m.P.data(), T.data()));
    return T;
}

// ---- solver (src/pcg3d.h) --------------------------------------------------

struct PcgStats {
    int iters = 0;
    double relres = 0;
    bool converged = false;
};

enum class Precond { Jacobi, Multigrid };

inline const char* precond_name(Precond p) { return p == Precond::Jacobi ? "Jacobi" : "multigrid"; }

using GpuSetupTimes = ct_setup_times;

inline void gpu_use_graphs(bool on) { ct_use_graphs(on ? 1 : 0); }

inline GpuSetupTimes gpu_last_setup() {
    GpuSetupTimes t{};
    check(ct_last_setup(&t));
    return t;
}

class GpuPcg {
  public:
    GpuPcg(const Model3D& m, Precond pc, ct_precision prec = CT_MG_FP32_FLEX) : n_(m.ncells()) {
        const ct_model v = m.view();
        check(ct_solver_create(&v, pc == Precond::Jacobi ? CT_JACOBI : CT_MULTIGRID, prec, &s_));
    }
    ~GpuPcg() { ct_solver_destroy(s_); }
    GpuPcg(const GpuPcg&) = delete;
    GpuPcg& operator=(const GpuPcg&) = delete;

    void set_dt(double dt) { check(ct_set_dt(s_, dt)); }
    void set_x_zero() { check(ct_set_x_zero(s_)); }
    void set_rhs_steady() { check(ct_set_rhs_steady(s_)); }
    void set_rhs_transient() { check(ct_set_rhs_transient(s_)); }
    PcgStats solve(double tol, int maxit) {
        ct_stats st{};
        const ct_status r = ct_solve(s_, tol, maxit, &st);
        if (r != CT_OK && r != CT_NOT_CONVERGED && r != CT_BREAKDOWN) check(r);
        PcgStats out;
        out.iters = st.iters;
        out.relres = st.relres;
        out.converged = st.converged != 0;
        return out;
    }
    void get_x(std::vector<Real>& T) const {
        T.resize(n_);
        check(ct_get_x(s_, T.data()));
    }
    void set_power(const std::vector<double>& P) { check(ct_set_power(s_, P.data())); }
    const Real* device_x() const {
        const double* p = nullptr;
        check(ct_device_x(s_, &p));
        return p;
    }
    // Extensions: device-side step bookkeeping and true residual.
    ct_step_record step_record(double dt) {
        ct_step_record r{};
        check(ct_solver_step_record(s_, dt, &r));
        return r;
    }
    double true_relres() {
        double v = 0;
        check(ct_true_relres(s_, &v));
        return v;
    }
    // Extensions: queued work (no host wait until the matching wait call).
    void solve_async(double tol, int maxit) { check(ct_solve_async(s_, tol, maxit)); }
    PcgStats solve_wait() {
        ct_stats st{};
        const ct_status r = ct_solve_wait(s_, &st);
        if (r != CT_OK && r != CT_NOT_CONVERGED && r != CT_BREAKDOWN) check(r);
        PcgStats out;
        out.iters = st.iters;
        out.relres = st.relres;
        out.converged = st.converged != 0;
        return out;
    }
    // P and T: host memory that stays valid (P unchanged) until copies_wait.
    void set_power_async(const double* P) { check(ct_set_power_async(s_, P)); }
    void get_x_async(double* T) { check(ct_get_x_async(s_, T)); }
    void copies_wait() { check(ct_copies_wait(s_)); }
    void step_record_async(double dt, int slot) { check(ct_solver_step_record_async(s_, dt, slot)); }
    std::vector<ct_step_record> step_records(int first, int count, std::vector<ct_stats>* stats = nullptr) {
        std::vector<ct_step_record> r((size_t)count);
        if (stats) stats->resize((size_t)count);
        check(ct_solver_step_records(s_, first, count, r.data(), stats ? stats->data() : nullptr));
        return r;
    }
    ct_solver* handle() const { return s_; }

  private:
    size_t n_;
    ct_solver* s_ = nullptr;
};

struct SolveResult {
    std::vector<Real> T;
    int iters = 0;
    double relres = 0;
    double ms = 0, setup_ms = 0, solve_ms = 0;
    bool converged = false;
};

inline SolveResult gpu_pcg(const Model3D& m, double tol, int maxit, Precond pc,
                           ct_precision prec = CT_MG_FP32_FLEX) {
    using clk = std::chrono::steady_clock;
    auto ms = [](clk::time_point a, clk::time_point b) {
        return std::chrono::duration<double, std::milli>(b - a).count();
    };
    const auto t0 = clk::now();
    SolveResult res;
    clk::time_point ta, tb;
    {
        GpuPcg s(m, pc, prec);
        s.set_x_zero();
        s.set_rhs_steady();
        ta = clk::now();
        const PcgStats st = s.solve(tol, maxit);
        tb = clk::now();
        s.get_x(res.T);
        res.iters = st.iters;
        res.relres = st.relres;
        res.converged = st.converged;
    }
    const auto t1 = clk::now();
    res.ms = ms(t0, t1);
    res.setup_ms = ms(t0, ta);
    res.solve_ms = ms(ta, tb);
    return res;
}

// ||P - A T|| / ||P|| recomputed from scratch in FP64 (on the GPU).
inline double true_relres(const Model3D& m, const std::vector<Real>& T) {
    GpuPcg s(m, Precond::Jacobi);
    check(ct_set_x(s.handle(), T.data()));
    return s.true_relres();
}

// ---- transient (src/transient3d.h) ------------------------------------------

struct TransientOptions {
    double dt0 = 1e-5;
    double growth = 1.1;
    double dt_max = 0.05;
    double t_end = 1.0;
    double tol = 1e-9;
    int maxit = 50000;
    Precond precond = Precond::Multigrid;
};

struct StepRecord {
    double t, dt;
    int iters;
    double T_max;
    double q_out;
    double q_stored;
};

struct TransientResult {
    std::vector<StepRecord> steps;
    std::vector<Real> T;
    long total_iters = 0;
    double ms = 0;
    double solve_ms = 0;
    bool converged = true;
};

// Backward Euler from T = 0 (run_transient, src/transient3d.h:46-90). Works
// with any Solver offering the GpuPcg member functions.
template <class Solver>
TransientResult run_transient(const Model3D& m, const TransientOptions& o) {
    using clk = std::chrono::steady_clock;
    const auto t0 = clk::now();
    TransientResult res;
    Solver s(m, o.precond);
    s.set_x_zero();
    std::vector<Real> T_old(m.ncells(), Real(0)), T_new;
    double t = 0, dt = o.dt0, last_dt = -1;
    while (t < o.t_end * (1 - 1e-12)) {
        dt = std::min(dt, o.t_end - t);
        const auto ts = clk::now();
        if (dt != last_dt) {
            s.set_dt(dt);
            last_dt = dt;
        }
        s.set_rhs_transient();
        const PcgStats st = s.solve(o.tol, o.maxit);
        res.solve_ms += std::chrono::duration<double, std::milli>(clk::now() - ts).count();
        s.get_x(T_new);
        t += dt;
        StepRecord rec;
        rec.t = t;
        rec.dt = dt;
        rec.iters = st.iters;
        rec.T_max = *std::max_element(T_new.begin(), T_new.end());
        rec.q_out = heat_out(m, T_new);
        rec.q_stored = heat_stored(m, T_old, T_new, dt);
        res.steps.push_back(rec);
        res.total_iters += st.iters;
        res.converged = res.converged && st.converged;
        T_old.swap(T_new);
        dt = std::min(dt * o.growth, o.dt_max);
    }
    res.T = T_old;
    res.ms = std::chrono::duration<double, std::milli>(clk::now() - t0).count();
    return res;
}

// ---- cases (src/case3d.h) ----------------------------------------------------

struct PowerBlock {
    std::string name;
    int layer;
    double x0, y0, w, h;  // m
    double watts;
};

struct TsvRegion {
    int layer;
    double x0, y0, w, h;  // m
    double fraction;
};

struct CaseSpec {
    std::vector<Layer> layers;
    std::vector<PowerBlock> blocks;
    std::vector<TsvRegion> tsvs;
    double Lx = 10e-3, Ly = 10e-3;
    double h_top = 2e4, h_bot = 0.0;
    double T_amb = 25.0;
};

namespace detail {
struct CaseHandle {
    ct_case* c = nullptr;
    ~CaseHandle() {
        if (c) ct_case_destroy(c);
    }
};
}  // namespace detail

// load_case (src/case3d.h:86-156): false with the reference's message in err
// on a bad case.
inline bool load_case(const std::string& dir, CaseSpec& cs, std::string& err) {
    detail::CaseHandle h;
    if (ct_case_load(dir.c_str(), &h.c) != CT_OK) {
        err = ct_last_error();
        return false;
    }
    int nl = 0, nb = 0, nt = 0;
    cs = CaseSpec{};
    check(ct_case_info(h.c, &nl, &nb, &nt, &cs.Lx, &cs.Ly, &cs.h_top, &cs.h_bot, &cs.T_amb));
    char name[256];
    for (int k = 0; k < nl; ++k) {
        ct_layer v;
        check(ct_case_layer(h.c, k, &v, name, (int)sizeof name));
        cs.layers.push_back(Layer{name, v.thickness, v.k, v.rho_c, v.ncells, v.active != 0});
    }
    for (int k = 0; k < nb; ++k) {
        PowerBlock b;
        double rect[4];
        check(ct_case_block(h.c, k, &b.layer, rect, &b.watts, name, (int)sizeof name));
        b.name = name;
        b.x0 = rect[0], b.y0 = rect[1], b.w = rect[2], b.h = rect[3];
        cs.blocks.push_back(b);
    }
    for (int k = 0; k < nt; ++k) {
        TsvRegion t;
        double rect[4];
        check(ct_case_tsv(h.c, k, &t.layer, rect, &t.fraction));
        t.x0 = rect[0], t.y0 = rect[1], t.w = rect[2], t.h = rect[3];
        cs.tsvs.push_back(t);
    }
    return true;
}

// build_case_model (src/case3d.h:157-166).
inline Model3D build_case_model(const CaseSpec& cs, int nx, int ny, bool with_tsv = true) {
    Model3D m = build_model(cs.layers, nx, ny, cs.Lx, cs.Ly, cs.h_top, cs.h_bot);
    m.T_amb = cs.T_amb;
    for (const PowerBlock& b : cs.blocks) add_power_block(m, b.layer, b.x0, b.y0, b.w, b.h, b.watts);
    if (with_tsv)
        for (const TsvRegion& t : cs.tsvs) add_tsv_region(m, t.layer, t.x0, t.y0, t.w, t.h, t.fraction);
    finalize(m);
    return m;
}

// export_3dice (src/case3d.h:267-383): false with the reference's message in
// err when 3D-ICE cannot express the case.
inline bool export_3dice(const CaseSpec& cs, double cell_um, const std::string& outdir, std::string& err) {
    std::vector<ct_layer> ls;
    for (const Layer& L : cs.layers) ls.push_back(ct_layer{L.thickness, L.k, L.rho_c, L.ncells, L.active ? 1 : 0});
    detail::CaseHandle h;
    ct_status s = ct_case_new(ls.data(), (int)ls.size(), cs.Lx, cs.Ly, cs.h_top, cs.h_bot, &h.c);
    for (size_t k = 0; s == CT_OK && k < cs.layers.size(); ++k)
        s = ct_case_set_name(h.c, 0, (int)k, cs.layers[k].name.c_str());
    for (size_t k = 0; s == CT_OK && k < cs.blocks.size(); ++k) {
        const PowerBlock& b = cs.blocks[k];
        s = ct_case_add_block(h.c, b.layer, b.x0, b.y0, b.w, b.h, b.watts);
        if (s == CT_OK) s = ct_case_set_name(h.c, 1, (int)k, b.name.c_str());
    }
    for (size_t k = 0; s == CT_OK && k < cs.tsvs.size(); ++k) {
        const TsvRegion& t = cs.tsvs[k];
        s = ct_case_add_tsv(h.c, t.layer, t.x0, t.y0, t.w, t.h, t.fraction);
    }
    if (s == CT_OK) s = ct_case_set_ambient(h.c, cs.T_amb);
    if (s == CT_OK) s = ct_case_export_3dice(h.c, cell_um, outdir.c_str());
    if (s != CT_OK) {
        err = ct_last_error();
        return false;
    }
    return true;
}

}  // namespace cthermal

#ifndef CTHERMAL_NO_GLOBAL_NAMES
using cthermal::build_case_model;
using cthermal::CaseSpec;
using cthermal::export_3dice;
using cthermal::load_case;
using cthermal::PowerBlock;
using cthermal::TsvRegion;
using cthermal::add_hotspot;
using cthermal::add_power_block;
using cthermal::add_tsv_region;
using cthermal::add_uniform_power;
using cthermal::analytic_1d;
using cthermal::build_model;
using cthermal::default_model;
using cthermal::default_stack;
using cthermal::eff_kxy;
using cthermal::eff_kz;
using cthermal::finalize;
using cthermal::GpuPcg;
using cthermal::gpu_last_setup;
using cthermal::gpu_pcg;
using cthermal::gpu_use_graphs;
using cthermal::GpuSetupTimes;
using cthermal::heat_out;
using cthermal::heat_stored;
using cthermal::Layer;
using cthermal::MAXZ;
using cthermal::Model3D;
using cthermal::PcgStats;
using cthermal::Precond;
using cthermal::precond_name;
using cthermal::Real;
using cthermal::run_transient;
using cthermal::SolveResult;
using cthermal::StepRecord;
using cthermal::total_power;
using cthermal::TransientOptions;
using cthermal::TransientResult;
using cthermal::true_relres;
#endif
