// device.h - data layout and control structures shared by the kernels and the
// host orchestration.
//
// Layout in HBM. Every vector and every operator array of every multigrid
// level, the finest included, uses the colour-split layout: each row j of a
// z-plane stores its red columns ((i + j) even) first and its black columns
// after them, hx slots each (ceil(nx / 2) rounded up to a multiple of 4, so
// that every half-row starts on a 16-byte boundary, as bulk tensor copies
// require), so column (i, j) sits at
//     scol(i, j) = (2 j + ((i + j) & 1)) * hx + i / 2
// and cell (i, j, l) at l * plane + scol(i, j), plane = ny * 2 * hx. A
// red-black sweep then reads and writes one contiguous half-row per colour,
// and its lateral neighbours are the other half of the same and adjacent rows.
// The outer PCG vectors share this layout, so the fine level's operator is
// stored once and the V-cycle reads the PCG residual with no permutation.
// Padding slots (up to 4 per half-row) hold zero in every vector and are
// never read as neighbours.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace ct {

constexpr int NT = 256;  // threads per block of every solver kernel

struct Geo {
    int nx, ny, nz, hx;
    unsigned plane;  // slots per z-plane: ny * 2 * hx
};

__host__ __device__ inline Geo geo_of(int nx, int ny, int nz) {
    Geo g;
    g.nx = nx;
    g.ny = ny;
    g.nz = nz;
    g.hx = (((nx + 1) / 2) + 3) & ~3;
    g.plane = (unsigned)ny * 2u * (unsigned)g.hx;
    return g;
}

__host__ __device__ inline unsigned scol(const Geo& g, int i, int j) {
    return (unsigned)(2 * j + ((i + j) & 1)) * (unsigned)g.hx + (unsigned)(i >> 1);
}

// Reduction slots: each reducing kernel owns one, with its own ticket counter
// and two rows of per-block partial sums.
enum Slot { SL_INIT = 0, SL_APPLY, SL_UPDATE, SL_DOT, SL_AUX, NSLOT };

// Per-solver control block in device memory. The kernels keep every scalar
// of the iteration here (alpha, beta and the dot products never visit the
// host), and the last block of each reduction finishes it in a fixed order,
// so results are reproducible run to run.
struct Ctl {
    // set by the host before a solve
    double tol;
    int maxit;
    int err;  // set by a kernel whose bounded wait ran out (the solve then stops)
    // scalars of the iteration
    double inv_dt;
    double bb, rr, rz, pAp, zAp, alpha, beta, relres;
    double alpha_x;           // alpha of an x update still to apply (0: none; FP64 outer loop)
    double aux0, aux1, aux2;  // results of the auxiliary reductions
    double stop;              // relres at which the current loop ends (double-word mode: phase 1)
    float2 alpha_w, beta_w;   // alpha, beta as float pairs (double-word mode)
    int iter;                 // completed iterations
    int body;                 // loop bodies entered (bounds the graph loop)
    // done and phase_end sit side by side on an 8-byte boundary: every kernel
    // of the loop body reads both with one load at entry (loop_done)
    int done;       // stop flag: every kernel of the loop body exits early
    int phase_end;  // double-word mode: phase 1 done, residual replacement next
    int converged;
    int breakdown;
    int bb_zero;
    int x_zero;     // set by the host: x = 0 at the start of this solve (r = b)
    unsigned ticket[NSLOT];
};
static_assert(offsetof(Ctl, phase_end) == offsetof(Ctl, done) + sizeof(int) && offsetof(Ctl, done) % 8 == 0,
              "loop_done reads done and phase_end with one 8-byte load");

// Graph while-loop handle: kernels that decide the loop's fate set it.
struct Cond {
    cudaGraphConditionalHandle h;
    int use;
};

// One multigrid level as the kernels see it (split layout). T = float or
// double: the V-cycle precision. Faces and capacities are always float.
template <class T>
struct LevelView {
    Geo g;
    const float *gE, *gN, *gU, *gB, *cap;
    T *fcp, *finv;
    T *x, *b;
};

}  // namespace ct
