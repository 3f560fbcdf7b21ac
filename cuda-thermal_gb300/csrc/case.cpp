// case.cpp - the case loader behind ct_case_*: a chip stack, its floorplan and
// its TSV layout read from a folder of CSV files, with the reference's file
// format and checks (load_case, src/case3d.h:86-156):
//   stack.csv      name, thickness_um, k, rho_c, planes, active  (bottom to top)
//                  settings lines: "# die_mm, X, Y", "# h_top, H", "# h_bottom, H",
//                  "# ambient_C, T"
//   floorplan.csv  name, layer, x_mm, y_mm, w_mm, h_mm, power_W  (layer active)
//   tsv.csv        layer, x_mm, y_mm, w_mm, h_mm, cu_fraction   (optional)
// In each file the first non-comment line is a header; blank lines are
// skipped; '#' lines are comments (settings in stack.csv); fields are trimmed
// of blanks and double quotes. Numbers are read as leading decimal prefixes
// (as std::stod / std::stoi read them). The model is then built with the
// library's stack builder (build_case_model, src/case3d.h:157-166).
#include <algorithm>
#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <new>
#include <string>
#include <vector>

#include "build.h"
#include "cthermal.h"
#include "cthermal_model.h"
#include "status.h"

namespace {

struct CaseLayer {
    std::string name;
    ct_layer v;
};
struct CaseBlock {
    std::string name;
    int layer;
    double x0, y0, w, h, watts;  // m, W
};
struct CaseTsv {
    int layer;
    double x0, y0, w, h, f;
};

std::string trim(const std::string& s) {
    const char* ws = " \t\r\n\"";
    const size_t a = s.find_first_not_of(ws);
    if (a == std::string::npos) return "";
    const size_t b = s.find_last_not_of(ws);
    return s.substr(a, b - a + 1);
}

std::vector<std::string> split(const std::string& line) {
    std::vector<std::string> out;
    size_t p = 0;
    while (true) {
        const size_t q = line.find(',', p);
        out.push_back(trim(line.substr(p, q == std::string::npos ? std::string::npos : q - p)));
        if (q == std::string::npos) break;
        p = q + 1;
    }
    // a trailing comma gives no empty last field (std::getline behaviour)
    if (!line.empty() && line.back() == ',') out.pop_back();
    return out;
}

// Data rows (header skipped) and '#' lines (without the '#'); false if the
// file cannot be opened.
bool read_csv(const std::string& path, std::vector<std::vector<std::string>>& rows,
              std::vector<std::vector<std::string>>* settings) {
    std::ifstream f(path);
    if (!f) return false;
    std::string line;
    bool header = false;
    while (std::getline(f, line)) {
        const std::string t = trim(line);
        if (t.empty()) continue;
        if (t[0] == '#') {
            if (settings) settings->push_back(split(trim(t.substr(1))));
            continue;
        }
        if (!header) {
            header = true;
            continue;
        }
        rows.push_back(split(t));
    }
    return true;
}

// Leading decimal prefix, as std::stod; false when there is none.
bool num(const std::string& s, double* out) {
    const char* b = s.c_str();
    char* e = nullptr;
    errno = 0;
    const double v = std::strtod(b, &e);
    if (e == b || errno == ERANGE) return false;
    *out = v;
    return true;
}
bool inum(const std::string& s, int* out) {
    const char* b = s.c_str();
    char* e = nullptr;
    errno = 0;
    const long v = std::strtol(b, &e, 10);
    if (e == b || errno == ERANGE || v < -2147483647L - 1 || v > 2147483647L) return false;
    *out = (int)v;
    return true;
}

}  // namespace

struct ct_case {
    std::vector<CaseLayer> layers;
    double Lx = 10e-3, Ly = 10e-3, h_top = 2e4, h_bot = 0.0, T_amb = 25.0;
    std::vector<CaseBlock> blocks;
    std::vector<CaseTsv> tsvs;

    int find(const std::string& name) const {
        for (size_t k = 0; k < layers.size(); ++k)
            if (layers[k].name == name) return (int)k;
        return -1;
    }

    ct_status load(const std::string& dir) {
        using ct::fail;
        std::vector<std::vector<std::string>> rows, settings;
        const auto bad_number = [] { return fail(CT_BAD_ARG, "could not parse a number"); };
        if (!read_csv(dir + "/stack.csv", rows, &settings))
            return fail(CT_IO_ERROR, "cannot open %s/stack.csv", dir.c_str());
        for (const auto& s : settings) {
            if (s.empty()) continue;
            double a = 0, b = 0;
            if (s[0] == "die_mm" && s.size() >= 3) {
                if (!num(s[1], &a) || !num(s[2], &b)) return bad_number();
                Lx = a * 1e-3;
                Ly = b * 1e-3;
            } else if (s[0] == "h_top" && s.size() >= 2) {
                if (!num(s[1], &a)) return bad_number();
                h_top = a;
            } else if (s[0] == "h_bottom" && s.size() >= 2) {
                if (!num(s[1], &a)) return bad_number();
                h_bot = a;
            } else if (s[0] == "ambient_C" && s.size() >= 2) {
                if (!num(s[1], &a)) return bad_number();
                T_amb = a;
            }
        }
        for (const auto& r : rows) {
            if (r.size() < 6) return fail(CT_BAD_ARG, "stack.csv: expected 6 columns");
            CaseLayer L;
            L.name = r[0];
            double t = 0, k = 0, rc = 0;
            int planes = 0, active = 0;
            if (!num(r[1], &t) || !num(r[2], &k) || !num(r[3], &rc) || !inum(r[4], &planes) ||
                !inum(r[5], &active))
                return bad_number();
            L.v.thickness = t * 1e-6;
            L.v.k = k;
            L.v.rho_c = rc;
            L.v.ncells = planes;
            L.v.active = active != 0 ? 1 : 0;
            layers.push_back(L);
        }
        if (layers.empty()) return fail(CT_BAD_ARG, "stack.csv has no layers");

        rows.clear();
        if (!read_csv(dir + "/floorplan.csv", rows, nullptr))
            return fail(CT_IO_ERROR, "cannot open %s/floorplan.csv", dir.c_str());
        for (const auto& r : rows) {
            if (r.size() < 7) return fail(CT_BAD_ARG, "floorplan.csv: expected 7 columns");
            const int L = find(r[1]);
            if (L < 0) return fail(CT_BAD_ARG, "floorplan.csv: unknown layer '%s'", r[1].c_str());
            if (!layers[(size_t)L].v.active)
                return fail(CT_BAD_ARG, "floorplan.csv: layer '%s' is not active", r[1].c_str());
            double x = 0, y = 0, w = 0, h = 0, p = 0;
            if (!num(r[2], &x) || !num(r[3], &y) || !num(r[4], &w) || !num(r[5], &h) || !num(r[6], &p))
                return bad_number();
            CaseBlock b{r[0], L, x * 1e-3, y * 1e-3, w * 1e-3, h * 1e-3, p};
            if (b.x0 < -1e-12 || b.y0 < -1e-12 || b.x0 + b.w > Lx * (1 + 1e-9) ||
                b.y0 + b.h > Ly * (1 + 1e-9))
                return fail(CT_BAD_ARG, "floorplan.csv: block '%s' extends outside the die",
                            b.name.c_str());
            blocks.push_back(b);
        }

        rows.clear();
        if (read_csv(dir + "/tsv.csv", rows, nullptr)) {  // optional
            for (const auto& r : rows) {
                if (r.size() < 6) return fail(CT_BAD_ARG, "tsv.csv: expected 6 columns");
                const int L = find(r[0]);
                if (L < 0) return fail(CT_BAD_ARG, "tsv.csv: unknown layer '%s'", r[0].c_str());
                double x = 0, y = 0, w = 0, h = 0, f = 0;
                if (!num(r[1], &x) || !num(r[2], &y) || !num(r[3], &w) || !num(r[4], &h) ||
                    !num(r[5], &f))
                    return bad_number();
                if (f < 0 || f > 1) return fail(CT_BAD_ARG, "tsv.csv: cu_fraction must be between 0 and 1");
                tsvs.push_back(CaseTsv{L, x * 1e-3, y * 1e-3, w * 1e-3, h * 1e-3, f});
            }
        }
        return CT_OK;
    }
};

namespace ct {

// The device build of build_case_model (src/case3d.h:157-166): planes as
// ct_model_planes lays them out, every power block, every TSV region (when
// wanted), copper TSV material.
ct_status case_build(const ct_case* c, int nx, int ny, bool with_tsv, DeviceBuild* b) {
    if (!c || !b) return fail(CT_BAD_ARG, "case build: null argument");
    if (nx < 1 || ny < 1) return fail(CT_BAD_ARG, "case build: bad grid %d x %d", nx, ny);
    std::vector<ct_layer> ls;
    for (const CaseLayer& L : c->layers) ls.push_back(L.v);
    double dz[CT_MAXZ];
    int nz = 0;
    const ct_status s = ct_model_planes(ls.data(), (int)ls.size(), &nz, b->plane_layer, dz);
    if (s != CT_OK) return s;
    b->nx = nx;
    b->ny = ny;
    b->nz = nz;
    b->Lx = c->Lx;
    b->Ly = c->Ly;
    b->dx = c->Lx / nx;
    b->dy = c->Ly / ny;
    b->h_top = c->h_top;
    b->h_bot = c->h_bot;
    for (int l = 0; l < nz; ++l) {
        b->planes.k[l] = ls[(size_t)b->plane_layer[l]].k;
        b->planes.rho_c[l] = ls[(size_t)b->plane_layer[l]].rho_c;
        b->planes.dz[l] = dz[l];
    }
    b->layer_planes.clear();
    for (const ct_layer& L : ls) b->layer_planes.push_back(L.ncells);
    b->blocks.clear();
    b->tsvs.clear();
    for (const CaseBlock& k : c->blocks) b->blocks.push_back(BuildRect{k.layer, k.x0, k.y0, k.w, k.h, k.watts});
    if (with_tsv)
        for (const CaseTsv& t : c->tsvs) b->tsvs.push_back(BuildRect{t.layer, t.x0, t.y0, t.w, t.h, t.f});
    return CT_OK;
}

}  // namespace ct

namespace {
void copy_name(const std::string& s, char* out, int cap) {
    if (!out || cap <= 0) return;
    std::snprintf(out, (size_t)cap, "%s", s.c_str());
}
}  // namespace

using ct::fail;

// ---- export to 3D-ICE -----------------------------------------------------------
// export_3dice / export_3dice_layout (src/case3d.h:192-383): the case as 3D-ICE
// 4.0 input on a uniform grid of cell_um: <outdir>/case.stk (materials, top
// heat sink, dimensions, one layer type per plane of a passive layer, one die
// per active layer with its single source layer, the stack listed top to
// bottom, steady solver, Tmap/Tflp outputs per die), L<k>.flp (the blocks of
// active layer k) and LT<k>_<p>.lay (the TSV cells of plane p of passive
// layer k, one anisotropic material per distinct copper fraction, runs of
// equal cells along each row as rectangles). Units: um, W/(um K),
// J/(um^3 K), K. The number formats are the reference's, so a 3D-ICE run sees
// the same numbers.
namespace {

double overlap_len(double a0, double a1, double b0, double b1) {
    return std::max(0.0, std::min(a1, b1) - std::max(a0, b0));
}

// Names 3D-ICE accepts: letters and digits kept, anything else '_'.
std::string ice_id(const std::string& s) {
    std::string out;
    for (char ch : s) out += std::isalnum((unsigned char)ch) ? ch : '_';
    return out;
}

struct ExportGrid {
    ct_grid g;
    int plane_layer[CT_MAXZ];
    double dz[CT_MAXZ];
    std::vector<double> frac;  // copper fraction per cell (natural layout)
    size_t nxy() const { return (size_t)g.nx * g.ny; }
    double at(int l, int i, int j) const { return frac[(size_t)l * nxy() + (size_t)j * g.nx + i]; }
    bool plane_has_tsv(int l) const {
        for (size_t c = 0; c < nxy(); ++c)
            if (frac[(size_t)l * nxy() + c] > 0) return true;
        return false;
    }
};

ct_status write_layout(const ExportGrid& m, int l, const CaseLayer& ly, double cell_um,
                       const std::string& path) {
    const auto key = [&](int i, int j) { return std::llround(m.at(l, i, j) * 1e9); };
    std::map<long long, std::vector<std::string>> rects;  // fraction key -> rectangles, key order
    char buf[192];
    for (int j = 0; j < m.g.ny; ++j)
        for (int i = 0; i < m.g.nx;) {
            const long long k = key(i, j);
            int i1 = i + 1;
            while (i1 < m.g.nx && key(i1, j) == k) ++i1;
            if (k != 0) {
                std::snprintf(buf, sizeof buf, "   rectangle (%.6f, %.6f, %.6f, %.6f) ;\n", i * cell_um,
                              j * cell_um, (i1 - i) * cell_um, cell_um);
                rects[k].push_back(buf);
            }
            i = i1;
        }
    FILE* g = std::fopen(path.c_str(), "w");
    if (!g) return fail(CT_IO_ERROR, "cannot write %s", path.c_str());
    std::fprintf(g, "// %s: TSV cells, one material per copper fraction\n\n", ly.name.c_str());
    const double tk = 400.0, trc = 3.45e6;  // copper (src/stack3d.h:60-62)
    int n = 0;
    for (const auto& kv : rects) {
        const double fr = kv.first * 1e-9;
        const double kxy = ct_eff_kxy(ly.v.k, tk, fr), kz = ct_eff_kz(ly.v.k, tk, fr);
        std::fprintf(g,
                     "material TSV%d :   // Cu fraction %.6f\n"
                     "   thermal conductivity     %.10e, %.10e, %.10e ;\n"
                     "   volumetric heat capacity %.10e ;\n\n",
                     n++, fr, kxy * 1e-6, kxy * 1e-6, kz * 1e-6, (fr * trc + (1 - fr) * ly.v.rho_c) * 1e-18);
    }
    n = 0;
    for (const auto& kv : rects) {
        std::fprintf(g, "TSV%d :\n", n++);
        for (const std::string& r : kv.second) std::fputs(r.c_str(), g);
        std::fprintf(g, "\n");
    }
    std::fclose(g);
    return CT_OK;
}

}  // namespace

extern "C" {

ct_status ct_case_export_3dice(const ct_case* c, double cell_um, const char* outdir) {
    if (!c || !outdir) return fail(CT_BAD_ARG, "ct_case_export_3dice: null argument");
    if (!(cell_um > 0)) return fail(CT_BAD_ARG, "ct_case_export_3dice: cell size must be > 0");
    const std::string dir(outdir);
    const double Lx_um = c->Lx * 1e6, Ly_um = c->Ly * 1e6;
    if (std::fabs(Lx_um / cell_um - std::round(Lx_um / cell_um)) > 1e-9 ||
        std::fabs(Ly_um / cell_um - std::round(Ly_um / cell_um)) > 1e-9)
        return fail(CT_BAD_ARG, "cell size must divide the die size");
    // the grid and its per-cell copper fractions (build_case_model with TSVs)
    ExportGrid m;
    std::vector<ct_layer> ls;
    for (const CaseLayer& L : c->layers) ls.push_back(L.v);
    int nz = 0;
    ct_status st = ct_model_planes(ls.data(), (int)ls.size(), &nz, m.plane_layer, m.dz);
    if (st != CT_OK) return st;
    m.g.nx = (int)std::lround(Lx_um / cell_um);
    m.g.ny = (int)std::lround(Ly_um / cell_um);
    m.g.nz = nz;
    m.g.Lx = c->Lx;
    m.g.Ly = c->Ly;
    m.g.dx = c->Lx / m.g.nx;
    m.g.dy = c->Ly / m.g.ny;
    if (m.g.nx < 1 || m.g.ny < 1) return fail(CT_BAD_ARG, "cell size must divide the die size");
    m.frac.assign(m.nxy() * (size_t)nz, 0.0);
    for (const CaseTsv& t : c->tsvs) {
        st = ct_model_add_tsv_region(&m.g, m.plane_layer, t.layer, t.x0, t.y0, t.w, t.h, t.f, m.frac.data());
        if (st != CT_OK) return st;
    }
    std::vector<int> first(c->layers.size(), 0);  // lowest plane of each layer
    for (int l = nz - 1; l >= 0; --l) first[(size_t)m.plane_layer[l]] = l;

    // what 3D-ICE cannot express, in the reference's order of checks
    for (size_t L = 0; L < c->layers.size(); ++L)
        if (c->layers[L].v.active && m.plane_has_tsv(first[L]))
            return fail(CT_BAD_ARG,
                        "TSVs in active layer '%s' can't be exported (3D-ICE has no material layouts in "
                        "source layers)",
                        c->layers[L].name.c_str());
    if (c->h_bot > 0) return fail(CT_BAD_ARG, "a bottom heat sink is not exported");
    for (const CaseLayer& L : c->layers)
        if (L.v.active && L.v.ncells != 1)
            return fail(CT_BAD_ARG, "active layer '%s' must have 1 plane for 3D-ICE", L.name.c_str());
    for (size_t a = 0; a < c->blocks.size(); ++a)
        for (size_t b = a + 1; b < c->blocks.size(); ++b) {
            const CaseBlock &p = c->blocks[a], &q = c->blocks[b];
            if (p.layer == q.layer && overlap_len(p.x0, p.x0 + p.w, q.x0, q.x0 + q.w) *
                                              overlap_len(p.y0, p.y0 + p.h, q.y0, q.y0 + q.h) >
                                          0)
                return fail(CT_BAD_ARG, "power blocks '%s' and '%s' overlap (3D-ICE needs disjoint blocks)",
                            p.name.c_str(), q.name.c_str());
        }

    FILE* f = std::fopen((dir + "/case.stk").c_str(), "w");
    if (!f) return fail(CT_IO_ERROR, "cannot write %s/case.stk (does the folder exist?)", dir.c_str());
    std::fprintf(f, "// 3D-ICE stack description written by ct_case_export_3dice; um, W/(um K), J/(um^3 K), K\n\n");
    for (size_t L = 0; L < c->layers.size(); ++L)
        std::fprintf(f,
                     "material M%zu :   // %s\n   thermal conductivity     %.10e ;\n"
                     "   volumetric heat capacity %.10e ;\n\n",
                     L, c->layers[L].name.c_str(), c->layers[L].v.k * 1e-6, c->layers[L].v.rho_c * 1e-18);
    std::fprintf(f, "top heat sink :\n   heat transfer coefficient %.10e ;\n   temperature %.4f ;\n\n",
                 c->h_top * 1e-12, c->T_amb + 273.15);
    std::fprintf(f,
                 "dimensions :\n   chip length %.6f, width %.6f ;\n   cell length %.6f, width %.6f ;\n"
                 "   non-uniform false ;\n\n",
                 Lx_um, Ly_um, cell_um, cell_um);
    // layer types (one per plane of each passive layer) before the dies
    struct Item {
        bool die;
        size_t layer;
        int plane;
    };
    std::vector<Item> stack;  // bottom to top
    for (size_t L = 0; L < c->layers.size(); ++L) {
        const CaseLayer& ly = c->layers[L];
        if (ly.v.active) {
            stack.push_back({true, L, 0});
            continue;
        }
        for (int p = 0; p < ly.v.ncells; ++p) {
            std::fprintf(f, "layer LT%zu_%d :   // %s, plane %d\n   height %.6f ;\n   material M%zu ;\n", L, p,
                         ly.name.c_str(), p, ly.v.thickness * 1e6 / ly.v.ncells, L);
            const int l = first[L] + p;
            if (m.plane_has_tsv(l)) {
                const std::string lay = "LT" + std::to_string(L) + "_" + std::to_string(p) + ".lay";
                st = write_layout(m, l, ly, cell_um, dir + "/" + lay);
                if (st != CT_OK) {
                    std::fclose(f);
                    return st;
                }
                std::fprintf(f, "   layout \"./%s\" ;\n", lay.c_str());
            }
            std::fprintf(f, "\n");
            stack.push_back({false, L, p});
        }
    }
    for (size_t L = 0; L < c->layers.size(); ++L)
        if (c->layers[L].v.active)
            std::fprintf(f, "die DIE%zu :   // %s\n   source %.6f M%zu ;\n\n", L, c->layers[L].name.c_str(),
                         c->layers[L].v.thickness * 1e6, L);
    std::fprintf(f, "stack:\n");
    for (size_t e = stack.size(); e-- > 0;) {  // top to bottom
        const Item& it = stack[e];
        if (it.die)
            std::fprintf(f, "   die   D%zu DIE%zu floorplan \"./L%zu.flp\" ;\n", it.layer, it.layer, it.layer);
        else
            std::fprintf(f, "   layer P%zu_%d LT%zu_%d ;\n", it.layer, it.plane, it.layer, it.plane);
    }
    std::fprintf(f, "\nsolver:\n   steady ;\n   initial temperature %.4f ;\n   numofcores 1 ;\n\noutput:\n",
                 c->T_amb + 273.15);
    for (size_t L = 0; L < c->layers.size(); ++L) {
        if (!c->layers[L].v.active) continue;
        std::fprintf(f, "   Tmap ( D%zu, \"tmap_L%zu.txt\", final ) ;\n", L, L);
        std::fprintf(f, "   Tflp ( D%zu, \"tflp_max_L%zu.txt\", maximum, final ) ;\n", L, L);
        std::fprintf(f, "   Tflp ( D%zu, \"tflp_avg_L%zu.txt\", average, final ) ;\n", L, L);
    }
    std::fclose(f);

    for (size_t L = 0; L < c->layers.size(); ++L) {
        if (!c->layers[L].v.active) continue;
        const std::string path = dir + "/L" + std::to_string(L) + ".flp";
        FILE* g = std::fopen(path.c_str(), "w");
        if (!g) return fail(CT_IO_ERROR, "cannot write %s", path.c_str());
        int count = 0;
        for (const CaseBlock& b : c->blocks) {
            if ((size_t)b.layer != L) continue;
            std::fprintf(g, "%s :\n   position %.6f, %.6f ;\n   dimension %.6f, %.6f ;\n   power values %.10e ;\n\n",
                         ice_id(b.name).c_str(), b.x0 * 1e6, b.y0 * 1e6, b.w * 1e6, b.h * 1e6, b.watts);
            ++count;
        }
        if (count == 0)  // a die needs at least one floorplan element
            std::fprintf(g, "none :\n   position 0, 0 ;\n   dimension %.6f, %.6f ;\n   power values 0 ;\n\n", Lx_um,
                         Ly_um);
        std::fclose(g);
    }
    return CT_OK;
}

ct_status ct_case_load(const char* dir, ct_case** out) {
    if (!dir || !out) return fail(CT_BAD_ARG, "ct_case_load: null argument");
    *out = nullptr;
    ct_case* c = new (std::nothrow) ct_case();
    if (!c) return fail(CT_OUT_OF_MEMORY, "host allocation failed");
    const ct_status s = c->load(dir);
    if (s != CT_OK) {
        delete c;
        return s;
    }
    *out = c;
    return CT_OK;
}

ct_status ct_case_new(const ct_layer* layers, int nlayers, double Lx, double Ly, double h_top,
                      double h_bot, ct_case** out) {
    if (!out || !layers || nlayers < 1) return fail(CT_BAD_ARG, "ct_case_new: bad arguments");
    if (!(Lx > 0) || !(Ly > 0)) return fail(CT_BAD_ARG, "ct_case_new: die size must be > 0");
    *out = nullptr;
    ct_case* c = new (std::nothrow) ct_case();
    if (!c) return fail(CT_OUT_OF_MEMORY, "host allocation failed");
    for (int k = 0; k < nlayers; ++k) c->layers.push_back(CaseLayer{"layer" + std::to_string(k), layers[k]});
    c->Lx = Lx;
    c->Ly = Ly;
    c->h_top = h_top;
    c->h_bot = h_bot;
    *out = c;
    return CT_OK;
}

ct_status ct_case_set_name(ct_case* c, int kind, int k, const char* name) {
    if (!c || !name) return fail(CT_BAD_ARG, "ct_case_set_name: null argument");
    if (kind == 0 && k >= 0 && k < (int)c->layers.size()) {
        c->layers[(size_t)k].name = name;
        return CT_OK;
    }
    if (kind == 1 && k >= 0 && k < (int)c->blocks.size()) {
        c->blocks[(size_t)k].name = name;
        return CT_OK;
    }
    return fail(CT_BAD_ARG, "ct_case_set_name: no %s %d", kind == 0 ? "layer" : "block", k);
}

ct_status ct_case_set_ambient(ct_case* c, double T_amb) {
    if (!c) return fail(CT_BAD_ARG, "ct_case_set_ambient: null case");
    c->T_amb = T_amb;
    return CT_OK;
}

ct_status ct_case_add_block(ct_case* c, int layer, double x0, double y0, double w, double h,
                            double watts) {
    if (!c || layer < 0 || layer >= (int)c->layers.size())
        return fail(CT_BAD_ARG, "ct_case_add_block: bad case or layer");
    if (!c->layers[(size_t)layer].v.active) return fail(CT_BAD_ARG, "ct_case_add_block: layer %d is not active", layer);
    if (!(w > 0) || !(h > 0)) return fail(CT_BAD_ARG, "ct_case_add_block: empty block");
    c->blocks.push_back(CaseBlock{"block" + std::to_string(c->blocks.size()), layer, x0, y0, w, h, watts});
    return CT_OK;
}

ct_status ct_case_add_tsv(ct_case* c, int layer, double x0, double y0, double w, double h,
                          double fraction) {
    if (!c || layer < 0 || layer >= (int)c->layers.size())
        return fail(CT_BAD_ARG, "ct_case_add_tsv: bad case or layer");
    if (fraction < 0 || fraction > 1) return fail(CT_BAD_ARG, "tsv.csv: cu_fraction must be between 0 and 1");
    c->tsvs.push_back(CaseTsv{layer, x0, y0, w, h, fraction});
    return CT_OK;
}

ct_status ct_case_destroy(ct_case* c) {
    delete c;
    return CT_OK;
}

ct_status ct_case_info(const ct_case* c, int* nlayers, int* nblocks, int* ntsvs, double* Lx,
                       double* Ly, double* h_top, double* h_bot, double* T_amb) {
    if (!c) return fail(CT_BAD_ARG, "ct_case_info: null case");
    if (nlayers) *nlayers = (int)c->layers.size();
    if (nblocks) *nblocks = (int)c->blocks.size();
    if (ntsvs) *ntsvs = (int)c->tsvs.size();
    if (Lx) *Lx = c->Lx;
    if (Ly) *Ly = c->Ly;
    if (h_top) *h_top = c->h_top;
    if (h_bot) *h_bot = c->h_bot;
    if (T_amb) *T_amb = c->T_amb;
    return CT_OK;
}

ct_status ct_case_layer(const ct_case* c, int k, ct_layer* out, char* name, int name_cap) {
    if (!c || k < 0 || k >= (int)c->layers.size()) return fail(CT_BAD_ARG, "ct_case_layer: bad index");
    if (out) *out = c->layers[(size_t)k].v;
    copy_name(c->layers[(size_t)k].name, name, name_cap);
    return CT_OK;
}

ct_status ct_case_block(const ct_case* c, int k, int* layer, double* rect, double* watts, char* name,
                        int name_cap) {
    if (!c || k < 0 || k >= (int)c->blocks.size()) return fail(CT_BAD_ARG, "ct_case_block: bad index");
    const CaseBlock& b = c->blocks[(size_t)k];
    if (layer) *layer = b.layer;
    if (rect) {
        rect[0] = b.x0;
        rect[1] = b.y0;
        rect[2] = b.w;
        rect[3] = b.h;
    }
    if (watts) *watts = b.watts;
    copy_name(b.name, name, name_cap);
    return CT_OK;
}

ct_status ct_case_tsv(const ct_case* c, int k, int* layer, double* rect, double* fraction) {
    if (!c || k < 0 || k >= (int)c->tsvs.size()) return fail(CT_BAD_ARG, "ct_case_tsv: bad index");
    const CaseTsv& t = c->tsvs[(size_t)k];
    if (layer) *layer = t.layer;
    if (rect) {
        rect[0] = t.x0;
        rect[1] = t.y0;
        rect[2] = t.w;
        rect[3] = t.h;
    }
    if (fraction) *fraction = t.f;
    return CT_OK;
}

}  // extern "C"
