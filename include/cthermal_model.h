/* cthermal_model.h - C ABI of libcthermal's stack model builder: the
 * reference's stack3d.h functions (layers -> z-planes, area-weighted power
 * maps, effective-medium TSVs, harmonic-mean face conductances) as stateless
 * calls over caller-owned arrays, so that C, C++ (cthermal.hpp) and Python
 * share one implementation. Results are bit-identical to the reference's
 * (same formulas, same operation order, no FMA contraction).
 *
 * Array sizes: n = nx*ny*nz cells (natural layout), nxy = nx*ny columns,
 * per-plane arrays nz entries.
 */
#ifndef CTHERMAL_MODEL_H
#define CTHERMAL_MODEL_H

#include "cthermal.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Layer (src/stack3d.h:36-43) without its name. */
typedef struct ct_layer {
    double thickness; /* m */
    double k;         /* W/(m K) */
    double rho_c;     /* J/(m^3 K) */
    int ncells;       /* z-planes in this layer */
    int active;       /* dissipates power */
} ct_layer;

/* The lateral grid of a Model3D (src/stack3d.h:46-48). */
typedef struct ct_grid {
    int nx, ny, nz;
    double Lx, Ly, dx, dy; /* m */
} ct_grid;

/* build_model (src/stack3d.h:81-102), plane part: fills plane_layer[] and
 * dz[] (CT_MAXZ entries each) and *nz. CT_BAD_ARG above CT_MAXZ planes. */
ct_status ct_model_planes(const ct_layer* layers, int nlayers, int* nz, int* plane_layer,
                          double* dz);

/* finalize (src/stack3d.h:110-148): face conductances and capacities from
 * the layers, dz and the per-cell TSV copper fraction. */
ct_status ct_model_finalize(const ct_grid* g, const ct_layer* layers, const int* plane_layer,
                            const double* dz, double h_top, double h_bot, double tsv_k,
                            double tsv_rho_c, const double* tsv_frac, float* gE, float* gN,
                            float* gU, float* gB, float* cap);

/* add_power_block (src/stack3d.h:193-206): watts spread area-weighted over
 * the rectangle [x0, x0+w] x [y0, y0+h] (m) in every plane of layer `layer`. */
ct_status ct_model_add_power_block(const ct_grid* g, const ct_layer* layers, const int* plane_layer,
                                   int layer, double x0, double y0, double w, double h,
                                   double watts, double* P);

/* add_uniform_power (src/stack3d.h:222-225). */
ct_status ct_model_add_uniform_power(const ct_grid* g, const ct_layer* layers,
                                     const int* plane_layer, int layer, double watts, double* P);

/* add_hotspot (src/stack3d.h:227-244): watts over the cells whose centres lie
 * in the square of side `size` centred at (xc, yc). CT_BAD_ARG when it covers
 * no cell (the reference exits there). */
ct_status ct_model_add_hotspot(const ct_grid* g, const int* plane_layer, int layer, double xc,
                               double yc, double size, double watts, double* P);

/* add_tsv_region (src/stack3d.h:208-220): copper fraction f over the
 * rectangle in layer `layer`, capped at 1 per cell. */
ct_status ct_model_add_tsv_region(const ct_grid* g, const int* plane_layer, int layer, double x0,
                                  double y0, double w, double h, double f, double* tsv_frac);

/* total_power, heat_out, heat_stored (src/stack3d.h:246-273). */
double ct_model_total_power(const ct_grid* g, const double* P);
double ct_model_heat_out(const ct_grid* g, const float* gU, const float* gB, const double* T);
double ct_model_heat_stored(const ct_grid* g, const float* cap, const double* T_old,
                            const double* T_new, double dt);

/* analytic_1d (src/stack3d.h:275-297): exact plane temperatures for uniform
 * power, no TSVs, adiabatic bottom. T has nz entries. */
ct_status ct_model_analytic_1d(const ct_grid* g, const ct_layer* layers, const int* plane_layer,
                               const double* dz, double h_top, const double* P, double* T);

/* ---- cases: a stack, floorplan and TSV layout from CSV files ---------------
 * load_case (src/case3d.h:86-156): dir/stack.csv, dir/floorplan.csv and, if
 * present, dir/tsv.csv, with the reference's format and checks. CT_IO_ERROR
 * when a required file cannot be opened, CT_BAD_ARG (with the reference's
 * message) for a malformed one. The model is then built with ct_model_planes,
 * ct_model_add_power_block for every block, ct_model_add_tsv_region for every
 * TSV region (when wanted) and ct_model_finalize, in that order
 * (build_case_model, src/case3d.h:157-166). */
ct_status ct_case_load(const char* dir, ct_case** out);
ct_status ct_case_destroy(ct_case* c);
/* A case built in code (no files): layers bottom to top (named layer0,
 * layer1, ...), die size and sink coefficients; then blocks (on active
 * layers) and TSV regions, in m. Used for floorplan sweeps with
 * ct_batch_create_cases. */
ct_status ct_case_new(const ct_layer* layers, int nlayers, double Lx, double Ly, double h_top,
                      double h_bot, ct_case** out);
ct_status ct_case_add_block(ct_case* c, int layer, double x0, double y0, double w, double h,
                            double watts);
ct_status ct_case_add_tsv(ct_case* c, int layer, double x0, double y0, double w, double h,
                          double fraction);
/* Names of a case built in code (kind 0: layer k, kind 1: block k; they
 * appear in the 3D-ICE export) and its ambient temperature (C). */
ct_status ct_case_set_name(ct_case* c, int kind, int k, const char* name);
ct_status ct_case_set_ambient(ct_case* c, double T_amb);
ct_status ct_case_info(const ct_case* c, int* nlayers, int* nblocks, int* ntsvs, double* Lx,
                       double* Ly, double* h_top, double* h_bot, double* T_amb);
/* Layer k (bottom to top) and its name (at most name_cap bytes with the NUL). */
ct_status ct_case_layer(const ct_case* c, int k, ct_layer* out, char* name, int name_cap);
/* Power block k: layer index, rect = {x0, y0, w, h} in m, watts, name. */
ct_status ct_case_block(const ct_case* c, int k, int* layer, double* rect, double* watts, char* name,
                        int name_cap);
/* TSV region k: layer index, rect in m, copper fraction. */
ct_status ct_case_tsv(const ct_case* c, int k, int* layer, double* rect, double* fraction);

/* export_3dice (src/case3d.h:267-383): the case as 3D-ICE 4.0 input on a
 * uniform grid of cell_um micrometres, written into the existing folder
 * outdir: case.stk, L<k>.flp for every active layer k, LT<k>_<p>.lay for every
 * TSV-carrying plane p of a passive layer k. CT_BAD_ARG (with the reference's
 * message) when the cell size does not divide the die, TSVs sit in an active
 * layer, there is a bottom heat sink, an active layer has more than one plane
 * or two blocks of one layer overlap; CT_IO_ERROR when a file cannot be
 * written. Host only. */
ct_status ct_case_export_3dice(const ct_case* c, double cell_um, const char* outdir);

/* eff_kz, eff_kxy (src/stack3d.h:104-108). */
double ct_eff_kz(double k, double kc, double f);
double ct_eff_kxy(double k, double kc, double f);

#ifdef __cplusplus
}
#endif
#endif /* CTHERMAL_MODEL_H */
