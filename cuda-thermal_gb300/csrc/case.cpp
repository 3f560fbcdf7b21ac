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
// library's stack builder (build_case_model, src/case3d.h:158-168).
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
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

// The device build of build_case_model (src/case3d.h:158-168): planes as
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

extern "C" {

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
