// A caller written against the reference's solver interface (the names of
// src/stack3d.h, src/pcg3d.h and src/transient3d.h), compiled against the
// library's C++ adapter instead. Prints one line per result, or the error.
#include <cstdio>
#include <exception>

#include "cthermal.hpp"

int main() {
    Model3D m = default_model(64, 64);
    add_uniform_power(m, 0, 25.0);
    add_hotspot(m, 0, 3e-3, 4e-3, 1e-3, 3.0);
    add_uniform_power(m, 2, 25.0);
    finalize(m);
    std::printf("total_power %.17g\n", total_power(m));
    try {
        SolveResult r = gpu_pcg(m, 1e-10, 50000, Precond::Multigrid);
        double tmax = 0;
        for (double v : r.T) tmax = v > tmax ? v : tmax;
        std::printf("steady iters %d relres %.3e converged %d tmax %.17g true_relres %.3e\n", r.iters,
                    r.relres, (int)r.converged, tmax, true_relres(m, r.T));
        TransientOptions o;
        o.t_end = 0.002;
        TransientResult tr = run_transient<GpuPcg>(m, o);
        std::printf("transient steps %zu tmax %.17g\n", tr.steps.size(), tr.steps.back().T_max);
    } catch (const std::exception& e) {
        std::printf("error %s\n", e.what());
        return 3;
    }
    return 0;
}
