// ref_gpu_harness.cu - C entry points around the UNMODIFIED reference GPU
// solver (GpuPcg, src/pcg3d.h:115-163, src/pcg3d_gpu.cu:346-682), compiled
// for sm_103a from the reference's own sources (oracle/Makefile, target
// `ref-gpu`). COMPARISON AND TEST INFRASTRUCTURE ONLY: it times the reference's
// GPU MG-PCG on the same inputs as this library's solver. Models come from
// ref_model_new (ref_harness.cpp, the reference's own stack3d.h builder),
// linked into the same library.
#include <chrono>
#include <cstring>
#include <vector>

#include <cuda_runtime.h>

#include "pcg3d.h"
#include "stack3d.h"

extern "C" {

int refg_mg_double() { return sizeof(MgReal) == 8 ? 1 : 0; }

int refg_device_count() {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

// gpu_use_graphs (src/pcg3d_gpu.cu:84-85): applies to solvers built afterwards.
void refg_use_graphs(int on) { gpu_use_graphs(on != 0); }

// GpuPcg(m, pc); precond 0 = Jacobi, 1 = multigrid. *setup_ms: wall time of
// the constructor (levels, allocation, upload, factors, graph recording).
void* refg_solver_new(void* model, int precond, double* setup_ms) {
    const auto t0 = std::chrono::steady_clock::now();
    GpuPcg* s = new GpuPcg(*static_cast<Model3D*>(model),
                           precond ? Precond::Multigrid : Precond::Jacobi);
    cudaDeviceSynchronize();
    *setup_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return s;
}

void refg_solver_free(void* s) { delete static_cast<GpuPcg*>(s); }

// One steady solve from T = 0: set_x_zero, set_rhs_steady, solve (the
// reference's solve blocks until it returns). 1 if converged.
int refg_solve_steady(void* h, double tol, int maxit, int* iters, double* relres) {
    GpuPcg* s = static_cast<GpuPcg*>(h);
    s->set_x_zero();
    s->set_rhs_steady();
    const PcgStats st = s->solve(tol, maxit);
    *iters = st.iters;
    *relres = st.relres;
    return st.converged ? 1 : 0;
}

void refg_get_x(void* h, double* T) {
    std::vector<Real> x;
    static_cast<GpuPcg*>(h)->get_x(x);
    for (size_t k = 0; k < x.size(); ++k) T[k] = (double)x[k];
}

}  // extern "C"
