// build.h - a stack model described by its layers, power blocks and TSV
// regions, to be built on the device (k_build.cu) instead of uploaded.
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "cthermal.h"
#include "cthermal_model.h"
#include "device.h"

namespace ct {

struct BuildRect {
    int layer;
    double x0, y0, w, h;  // m
    double v;             // watts (power block) or copper fraction (TSV region)
};

// Per-plane material and thickness (the layer of each plane).
struct PlaneTable {
    double k[CT_MAXZ], rho_c[CT_MAXZ], dz[CT_MAXZ];
};

struct DeviceBuild {
    int nx = 0, ny = 0, nz = 0;
    double Lx = 0, Ly = 0, dx = 0, dy = 0, h_top = 0, h_bot = 0;
    double tsv_k = 400.0, tsv_rho_c = 3.45e6;  // copper (src/stack3d.h:60-62)
    int plane_layer[CT_MAXZ] = {};
    PlaneTable planes{};
    std::vector<int> layer_planes;  // planes of each layer (power is split over them)
    std::vector<BuildRect> blocks, tsvs;
};

// TSV fractions and power (natural layout, into the two scratch arrays of
// nx*ny*nz doubles), then the split-layout operator arrays.
cudaError_t launch_build(cudaStream_t st, const DeviceBuild& b, const Geo& g, double* frac_nat,
                         double* P_nat, float* gE, float* gN, float* gU, float* gB, float* cap);

// The description of a loaded case (case.cpp) on an nx x ny grid.
ct_status case_build(const ct_case* c, int nx, int ny, bool with_tsv, DeviceBuild* b);

}  // namespace ct
