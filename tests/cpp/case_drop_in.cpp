// A caller of the reference's case3d.h functions, built against
// include/cthermal.hpp: load a case folder (argv[1]), build its model on a
// 40 x 40 grid, and export it to 3D-ICE on 100 um cells into argv[2].
#include <cstdio>
#include <string>

#include "cthermal.hpp"

int main(int argc, char** argv) {
    if (argc < 3) return 1;
    CaseSpec cs;
    std::string err;
    if (!load_case(argv[1], cs, err)) {
        std::printf("load_error %s\n", err.c_str());
        return 2;
    }
    const Model3D m = build_case_model(cs, 40, 40, true);
    std::printf("nz %d\n", m.nz);
    std::printf("total_power %.17g\n", total_power(m));
    std::printf("counts %zu %zu %zu\n", cs.layers.size(), cs.blocks.size(), cs.tsvs.size());
    if (export_3dice(cs, 100.0, argv[2], err))
        std::printf("export_ok\n");
    else
        std::printf("export_error %s\n", err.c_str());
    return 0;
}
