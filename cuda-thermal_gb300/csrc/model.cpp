// model.cpp - the stack model builder behind cthermal_model.h.
//
// Host code: geometry, power maps and face conductances of the layered stack,
// computed in double and stored as the reference stores them (conductances and
// capacities in float, power in double). Each function states the reference
// function it reproduces; the formulas and their operation order are kept so
// that the arrays are bit-identical to the reference's. This file must be
// compiled with -ffp-contract=off: a fused multiply-add (the default on
// aarch64) would change the last bit of some conductances.
#include <algorithm>
#include <cmath>
#include <vector>

#include "cthermal_model.h"
#include "status.h"

namespace {

bool grid_ok(const ct_grid* g) {
    return g && g->nx > 0 && g->ny > 0 && g->nz > 0 && g->nz <= CT_MAXZ && g->dx > 0 && g->dy > 0;
}

// Length of the overlap of [a0, a1] and [b0, b1].
double overlap(double a0, double a1, double b0, double b1) {
    return std::max(0.0, std::min(a1, b1) - std::max(a0, b0));
}

// for_each_overlap (src/stack3d.h:175-191): visits every column whose cell
// overlaps the rectangle by more than a rounding sliver, with the covered
// fraction of the cell.
template <class Fn>
void visit_rect(const ct_grid* g, double x0, double y0, double w, double h, Fn fn) {
    const int i0 = std::max(0, (int)std::floor(x0 / g->dx));
    const int i1 = std::min(g->nx - 1, (int)std::ceil((x0 + w) / g->dx));
    const int j0 = std::max(0, (int)std::floor(y0 / g->dy));
    const int j1 = std::min(g->ny - 1, (int)std::ceil((y0 + h) / g->dy));
    const double cell = g->dx * g->dy;
    for (int j = j0; j <= j1; ++j)
        for (int i = i0; i <= i1; ++i) {
            const double a = overlap(i * g->dx, (i + 1) * g->dx, x0, x0 + w) *
                             overlap(j * g->dy, (j + 1) * g->dy, y0, y0 + h);
            if (a > 1e-9 * g->dx * g->dy) fn((size_t)j * g->nx + i, a / cell);
        }
}

}  // namespace

extern "C" {

double ct_eff_kz(double k, double kc, double f) { return f * kc + (1 - f) * k; }

double ct_eff_kxy(double k, double kc, double f) {
    return k * ((1 + f) * kc + (1 - f) * k) / ((1 - f) * kc + (1 + f) * k);
}

ct_status ct_model_planes(const ct_layer* layers, int nlayers, int* nz, int* plane_layer,
                          double* dz) {
    if (!layers || nlayers <= 0 || !nz || !plane_layer || !dz)
        return ct::fail(CT_BAD_ARG, "ct_model_planes: null argument or no layers");
    int n = 0;
    for (int L = 0; L < nlayers; ++L) {
        if (layers[L].ncells <= 0 || !(layers[L].thickness > 0))
            return ct::fail(CT_BAD_ARG, "ct_model_planes: layer %d has no planes or thickness", L);
        for (int c = 0; c < layers[L].ncells; ++c) {
            if (n >= CT_MAXZ)
                return ct::fail(CT_BAD_ARG, "Too many z-planes (more than %d)", CT_MAXZ);
            plane_layer[n] = L;
            dz[n] = layers[L].thickness / layers[L].ncells;
            ++n;
        }
    }
    *nz = n;
    return CT_OK;
}

ct_status ct_model_finalize(const ct_grid* g, const ct_layer* layers, const int* plane_layer,
                            const double* dz, double h_top, double h_bot, double tsv_k,
                            double tsv_rho_c, const double* tsv_frac, float* gE, float* gN,
                            float* gU, float* gB, float* cap) {
    if (!grid_ok(g) || !layers || !plane_layer || !dz || !tsv_frac || !gE || !gN || !gU || !gB ||
        !cap)
        return ct::fail(CT_BAD_ARG, "ct_model_finalize: bad grid or null array");
    const size_t sxy = (size_t)g->nx * g->ny, n = sxy * g->nz;
    const double A = g->dx * g->dy;
    std::vector<double> kxy(n), kz(n);
    for (int l = 0; l < g->nz; ++l) {
        const ct_layer& L = layers[plane_layer[l]];
        for (size_t c = 0; c < sxy; ++c) {
            const size_t id = (size_t)l * sxy + c;
            const double f = tsv_frac[id];
            kxy[id] = ct_eff_kxy(L.k, tsv_k, f);
            kz[id] = ct_eff_kz(L.k, tsv_k, f);
            cap[id] = (float)((f * tsv_rho_c + (1 - f) * L.rho_c) * A * dz[l]);
        }
    }
    std::fill(gE, gE + n, 0.0f);
    std::fill(gN, gN + n, 0.0f);
    std::fill(gU, gU + n, 0.0f);
    std::fill(gB, gB + sxy, 0.0f);
    for (int l = 0; l < g->nz; ++l) {
        const double d = dz[l];
        for (int j = 0; j < g->ny; ++j)
            for (int i = 0; i < g->nx; ++i) {
                const size_t id = ((size_t)l * g->ny + j) * g->nx + i;
                // Two half cells in series across each face.
                if (i < g->nx - 1)
                    gE[id] = (float)(g->dy * d / (g->dx / (2 * kxy[id]) + g->dx / (2 * kxy[id + 1])));
                if (j < g->ny - 1)
                    gN[id] = (float)(g->dx * d /
                                     (g->dy / (2 * kxy[id]) + g->dy / (2 * kxy[id + g->nx])));
                const double r_up = (l < g->nz - 1)
                                        ? d / (2 * kz[id]) + dz[l + 1] / (2 * kz[id + sxy])
                                        : d / (2 * kz[id]) + 1.0 / h_top;
                gU[id] = (float)(A / r_up);
                if (l == 0 && h_bot > 0) gB[id] = (float)(A / (d / (2 * kz[id]) + 1.0 / h_bot));
            }
    }
    return CT_OK;
}

ct_status ct_model_add_power_block(const ct_grid* g, const ct_layer* layers, const int* plane_layer,
                                   int layer, double x0, double y0, double w, double h,
                                   double watts, double* P) {
    if (!grid_ok(g) || !layers || !plane_layer || !P || layer < 0)
        return ct::fail(CT_BAD_ARG, "ct_model_add_power_block: bad argument");
    const double density = watts / (w * h);
    const int planes = layers[layer].ncells;
    const size_t nxy = (size_t)g->nx * g->ny;
    for (int l = 0; l < g->nz; ++l) {
        if (plane_layer[l] != layer) continue;
        visit_rect(g, x0, y0, w, h, [&](size_t c, double frac) {
            P[(size_t)l * nxy + c] += density * frac * g->dx * g->dy / planes;
        });
    }
    return CT_OK;
}

ct_status ct_model_add_uniform_power(const ct_grid* g, const ct_layer* layers,
                                     const int* plane_layer, int layer, double watts, double* P) {
    if (!g) return ct::fail(CT_BAD_ARG, "ct_model_add_uniform_power: null grid");
    return ct_model_add_power_block(g, layers, plane_layer, layer, 0, 0, g->Lx, g->Ly, watts, P);
}

ct_status ct_model_add_hotspot(const ct_grid* g, const int* plane_layer, int layer, double xc,
                               double yc, double size, double watts, double* P) {
    if (!grid_ok(g) || !plane_layer || !P)
        return ct::fail(CT_BAD_ARG, "ct_model_add_hotspot: bad argument");
    std::vector<size_t> cells;
    for (int l = 0; l < g->nz; ++l) {
        if (plane_layer[l] != layer) continue;
        for (int j = 0; j < g->ny; ++j)
            for (int i = 0; i < g->nx; ++i) {
                const double x = (i + 0.5) * g->dx, y = (j + 0.5) * g->dy;
                if (std::fabs(x - xc) <= size / 2 && std::fabs(y - yc) <= size / 2)
                    cells.push_back(((size_t)l * g->ny + j) * g->nx + i);
            }
    }
    if (cells.empty()) return ct::fail(CT_BAD_ARG, "Hotspot covers no cells");
    for (size_t c : cells) P[c] += watts / (double)cells.size();
    return CT_OK;
}

ct_status ct_model_add_tsv_region(const ct_grid* g, const int* plane_layer, int layer, double x0,
                                  double y0, double w, double h, double f, double* tsv_frac) {
    if (!grid_ok(g) || !plane_layer || !tsv_frac)
        return ct::fail(CT_BAD_ARG, "ct_model_add_tsv_region: bad argument");
    const size_t nxy = (size_t)g->nx * g->ny;
    for (int l = 0; l < g->nz; ++l) {
        if (plane_layer[l] != layer) continue;
        visit_rect(g, x0, y0, w, h, [&](size_t c, double frac) {
            double& t = tsv_frac[(size_t)l * nxy + c];
            t = std::min(1.0, t + f * frac);
        });
    }
    return CT_OK;
}

double ct_model_total_power(const ct_grid* g, const double* P) {
    if (!grid_ok(g) || !P) return NAN;
    const size_t n = (size_t)g->nx * g->ny * g->nz;
    double s = 0;
    for (size_t c = 0; c < n; ++c) s += P[c];
    return s;
}

double ct_model_heat_out(const ct_grid* g, const float* gU, const float* gB, const double* T) {
    if (!grid_ok(g) || !gU || !gB || !T) return NAN;
    const size_t nxy = (size_t)g->nx * g->ny, top = (size_t)(g->nz - 1) * nxy;
    double q = 0;
    for (size_t c = 0; c < nxy; ++c) {
        q += (double)gU[top + c] * T[top + c];
        q += (double)gB[c] * T[c];
    }
    return q;
}

double ct_model_heat_stored(const ct_grid* g, const float* cap, const double* T_old,
                            const double* T_new, double dt) {
    if (!grid_ok(g) || !cap || !T_old || !T_new) return NAN;
    const size_t n = (size_t)g->nx * g->ny * g->nz;
    double q = 0;
    for (size_t c = 0; c < n; ++c) q += (double)cap[c] * (T_new[c] - T_old[c]);
    return q / dt;
}

ct_status ct_model_analytic_1d(const ct_grid* g, const ct_layer* layers, const int* plane_layer,
                               const double* dz, double h_top, const double* P, double* T) {
    if (!grid_ok(g) || !layers || !plane_layer || !dz || !P || !T)
        return ct::fail(CT_BAD_ARG, "ct_model_analytic_1d: bad argument");
    const int nz = g->nz;
    const size_t nxy = (size_t)g->nx * g->ny;
    const double A = g->dx * g->dy;
    std::vector<double> flux(nz), gz(nz);
    for (int l = 0; l < nz; ++l) {
        const double k = layers[plane_layer[l]].k;
        const double R = (l < nz - 1)
                             ? dz[l] / (2 * k) + dz[l + 1] / (2 * layers[plane_layer[l + 1]].k)
                             : dz[l] / (2 * k) + 1.0 / h_top;
        gz[l] = A / R;
    }
    double F = 0;
    for (int l = 0; l < nz; ++l) {
        for (size_t c = 0; c < nxy; ++c) F += P[(size_t)l * nxy + c];
        flux[l] = F;  // heat crossing the top face of plane l
    }
    const double cols = (double)nxy;
    T[nz - 1] = flux[nz - 1] / (gz[nz - 1] * cols);
    for (int l = nz - 2; l >= 0; --l) T[l] = T[l + 1] + flux[l] / (gz[l] * cols);
    return CT_OK;
}

}  // extern "C"
