// ref_harness.cpp - C entry points around the UNMODIFIED reference CPU solver,
// compiled from an unmodified copy of the reference's own sources
// (oracle/Makefile, targets `stage` and `ref`). TEST AND COMPARISON
// INFRASTRUCTURE ONLY: it pins the C oracle, generates the golden fixtures
// under tests/golden/ (make_golden.py) and is the timed reference CPU solver
// of the benchmark's reference arm. Nothing in the product loads it, and it is
// not built where the reference sources are absent.
//
// Models are built with the reference's own stack3d.h / case3d.h functions, in
// the order the caller lists: power operations first, then TSV regions, then
// finalize(), as build_case_model (src/case3d.h:157-166) does.
#include <chrono>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "case3d.h"
#include "mg3d.h"
#include "pcg3d.h"
#include "stack3d.h"
#include "transient3d.h"

extern "C" {

struct ref_layer {
    double thickness, k, rho_c;
    int ncells, active;
};
// kind 0: add_power_block(layer, x0, y0, w, h, watts)
// kind 1: add_uniform_power(layer, watts)
// kind 2: add_hotspot(layer, xc = x0, yc = y0, size = w, watts)
struct ref_power {
    int kind, layer;
    double x0, y0, w, h, watts;
};
struct ref_tsv {
    int layer;
    double x0, y0, w, h, f;
};

int ref_mg_double() { return sizeof(MgReal) == 8 ? 1 : 0; }

void* ref_model_new(const ref_layer* L, int nl, int nx, int ny, double Lx, double Ly,
                    double h_top, double h_bot, const ref_power* pw, int np, const ref_tsv* tv,
                    int nt) {
    std::vector<Layer> layers;
    for (int k = 0; k < nl; ++k)
        layers.push_back({"layer" + std::to_string(k), L[k].thickness, L[k].k, L[k].rho_c,
                          L[k].ncells, L[k].active != 0});
    Model3D* m = new Model3D(build_model(layers, nx, ny, Lx, Ly, h_top, h_bot));
    for (int k = 0; k < np; ++k) {
        const ref_power& p = pw[k];
        if (p.kind == 0)
            add_power_block(*m, p.layer, p.x0, p.y0, p.w, p.h, p.watts);
        else if (p.kind == 1)
            add_uniform_power(*m, p.layer, p.watts);
        else
            add_hotspot(*m, p.layer, p.x0, p.y0, p.w, p.watts);
    }
    for (int k = 0; k < nt; ++k)
        add_tsv_region(*m, tv[k].layer, tv[k].x0, tv[k].y0, tv[k].w, tv[k].h, tv[k].f);
    finalize(*m);
    return m;
}

// default_model(nx, ny) (src/stack3d.h:165-168: the two-tier stack of
// default_stack, 10 x 10 mm, h_top 2e4) with the listed power operations,
// then finalize().
void* ref_default_model_new(int nx, int ny, const ref_power* pw, int np) {
    Model3D* m = new Model3D(default_model(nx, ny));
    for (int k = 0; k < np; ++k) {
        const ref_power& p = pw[k];
        if (p.kind == 0)
            add_power_block(*m, p.layer, p.x0, p.y0, p.w, p.h, p.watts);
        else if (p.kind == 1)
            add_uniform_power(*m, p.layer, p.watts);
        else
            add_hotspot(*m, p.layer, p.x0, p.y0, p.w, p.watts);
    }
    finalize(*m);
    return m;
}

void* ref_case_model(const char* dir, int nx, int ny, int with_tsv, char* err, int errlen) {
    CaseSpec cs;
    std::string e;
    if (!load_case(dir, cs, e)) {
        snprintf(err, (size_t)errlen, "%s", e.c_str());
        return nullptr;
    }
    return new Model3D(build_case_model(cs, nx, ny, with_tsv != 0));
}

void* ref_example_case_model(int nx, int ny, int with_tsv) {
    return new Model3D(build_case_model(example_case(), nx, ny, with_tsv != 0));
}

void ref_model_free(void* h) { delete static_cast<Model3D*>(h); }

void ref_model_dims(void* h, int* nx, int* ny, int* nz, double* dx, double* dy) {
    const Model3D& m = *static_cast<Model3D*>(h);
    *nx = m.nx;
    *ny = m.ny;
    *nz = m.nz;
    *dx = m.dx;
    *dy = m.dy;
}

void ref_model_arrays(void* h, float* gE, float* gN, float* gU, float* gB, float* cap, double* P,
                      double* dz, double* tsv_frac, int* plane_layer) {
    const Model3D& m = *static_cast<Model3D*>(h);
    std::memcpy(gE, m.gE.data(), m.gE.size() * sizeof(float));
    std::memcpy(gN, m.gN.data(), m.gN.size() * sizeof(float));
    std::memcpy(gU, m.gU.data(), m.gU.size() * sizeof(float));
    std::memcpy(gB, m.gB.data(), m.gB.size() * sizeof(float));
    std::memcpy(cap, m.cap.data(), m.cap.size() * sizeof(float));
    std::memcpy(P, m.P.data(), m.P.size() * sizeof(double));
    std::memcpy(dz, m.dz.data(), m.dz.size() * sizeof(double));
    std::memcpy(tsv_frac, m.tsv_frac.data(), m.tsv_frac.size() * sizeof(double));
    std::memcpy(plane_layer, m.plane_layer.data(), m.plane_layer.size() * sizeof(int));
}

double ref_total_power(void* h) { return total_power(*static_cast<Model3D*>(h)); }

void ref_analytic_1d(void* h, double* Tz) {
    std::vector<double> t = analytic_1d(*static_cast<Model3D*>(h));
    std::memcpy(Tz, t.data(), t.size() * sizeof(double));
}

// cpu_pcg (src/pcg3d_cpu.cpp:187-205); precond 0 = Jacobi, 1 = multigrid.
int ref_cpu_pcg(void* h, double tol, int maxit, int precond, double* T, int* iters,
                double* relres, double* setup_ms, double* solve_ms) {
    SolveResult r = cpu_pcg(*static_cast<Model3D*>(h), tol, maxit,
                            precond ? Precond::Multigrid : Precond::Jacobi);
    std::memcpy(T, r.T.data(), r.T.size() * sizeof(double));
    *iters = r.iters;
    *relres = r.relres;
    *setup_ms = r.setup_ms;
    *solve_ms = r.solve_ms;
    return r.converged ? 1 : 0;
}

// A CpuPcg (src/pcg3d.h:71-99) kept across solves, so a steady solve can be
// timed without the set-up (levels, factors) that cpu_pcg includes.
void* ref_cpu_solver_new(void* model, int precond) {
    return new CpuPcg(*static_cast<Model3D*>(model), precond ? Precond::Multigrid : Precond::Jacobi);
}

void ref_cpu_solver_free(void* s) { delete static_cast<CpuPcg*>(s); }

// set_x_zero, set_rhs_steady, solve (src/pcg3d_cpu.cpp:126-185); 1 if converged.
int ref_cpu_solver_steady(void* h, double tol, int maxit, int* iters, double* relres) {
    CpuPcg* s = static_cast<CpuPcg*>(h);
    s->set_x_zero();
    s->set_rhs_steady();
    const PcgStats st = s->solve(tol, maxit);
    *iters = st.iters;
    *relres = st.relres;
    return st.converged ? 1 : 0;
}

void ref_cpu_solver_get_x(void* h, double* T) {
    std::vector<Real> x;
    static_cast<CpuPcg*>(h)->get_x(x);
    for (size_t k = 0; k < x.size(); ++k) T[k] = (double)x[k];
}

double ref_true_relres(void* h, const double* T) {
    const Model3D& m = *static_cast<Model3D*>(h);
    std::vector<Real> t(T, T + m.ncells());
    return true_relres(m, t);
}

double ref_heat_out(void* h, const double* T) {
    const Model3D& m = *static_cast<Model3D*>(h);
    std::vector<double> t(T, T + m.ncells());
    return heat_out(m, t);
}

int ref_num_levels(void* h) {
    return (int)mg_build_levels(*static_cast<Model3D*>(h)).size();
}

// Level k of mg_build_levels (src/mg3d.h:147-183), natural layout.
void ref_level(void* h, int k, int* nx, int* ny, float* gE, float* gN, float* gU, float* gB,
               float* cap) {
    std::vector<MgLevelHost> L = mg_build_levels(*static_cast<Model3D*>(h));
    const MgLevelHost& v = L[(size_t)k];
    *nx = v.nx;
    *ny = v.ny;
    if (gE) {
        std::memcpy(gE, v.gE.data(), v.gE.size() * sizeof(float));
        std::memcpy(gN, v.gN.data(), v.gN.size() * sizeof(float));
        std::memcpy(gU, v.gU.data(), v.gU.size() * sizeof(float));
        std::memcpy(gB, v.gB.data(), v.gB.size() * sizeof(float));
        std::memcpy(cap, v.cap.data(), v.cap.size() * sizeof(float));
    }
}

// run_transient<CpuPcg> (src/transient3d.h:48-90). rec gets 6 doubles per
// step (t, dt, iters, T_max, q_out, q_stored), at most max_rec steps.
int ref_run_transient(void* h, int precond, double dt0, double growth, double dt_max, double t_end,
                      double tol, int maxit, double* rec, int max_rec, double* T_end,
                      long* total_iters, int* all_converged) {
    TransientOptions o;
    o.dt0 = dt0;
    o.growth = growth;
    o.dt_max = dt_max;
    o.t_end = t_end;
    o.tol = tol;
    o.maxit = maxit;
    o.precond = precond ? Precond::Multigrid : Precond::Jacobi;
    TransientResult r = run_transient<CpuPcg>(*static_cast<Model3D*>(h), o);
    for (size_t k = 0; k < r.steps.size() && (int)k < max_rec; ++k) {
        const StepRecord& s = r.steps[k];
        double* q = rec + 6 * k;
        q[0] = s.t;
        q[1] = s.dt;
        q[2] = s.iters;
        q[3] = s.T_max;
        q[4] = s.q_out;
        q[5] = s.q_stored;
    }
    std::memcpy(T_end, r.T.data(), r.T.size() * sizeof(double));
    *total_iters = r.total_iters;
    *all_converged = r.converged ? 1 : 0;
    return (int)r.steps.size();
}

// export_3dice (src/case3d.h:267-383) of the case folder on a grid of cell_um:
// 1 on success, else 0 with the reference's message in err.
int ref_export_3dice(const char* folder, double cell_um, const char* outdir, char* err, int errcap) {
    CaseSpec cs;
    std::string e;
    if (!load_case(folder, cs, e) || !export_3dice(cs, cell_um, outdir, e)) {
        std::snprintf(err, (size_t)errcap, "%s", e.c_str());
        return 0;
    }
    return 1;
}

}  // extern "C"
