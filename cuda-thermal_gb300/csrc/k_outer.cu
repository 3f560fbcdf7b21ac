// k_outer.cu - FP64 outer-PCG kernels, setup and bookkeeping kernels.
//
// The Jacobi-preconditioned outer iteration (FP64, as in the reference,
// src/pcg3d_gpu.cu:134-264; the multigrid modes run k_fp64.cu), the set-up
// kernels (diagonal, layout changes) and the bookkeeping reductions (true
// residual, step records). Their stencil kernels walk one column per thread
// through the z-planes, so the vertical neighbours and the face below come
// from registers and every z-plane access of a warp is one contiguous run of
// the split layout.
#include <algorithm>
#include <cmath>
#include <cstdlib>

#include "kernels.h"
#include "tma.cuh"
#include "reduce.cuh"
#include "setup_dev.cuh"

namespace ct {

namespace {

// Column of the split-layout slot s: (i, j), colour c and half-row index t.
struct Col {
    int i, j;
    unsigned s, sw, se, ss, sn;
    bool valid;
};

__device__ __forceinline__ Col col_of_slot(const Geo& g, unsigned s) {
    Col c;
    const unsigned row2 = 2u * (unsigned)g.hx;
    const int j = (int)(s / row2);
    const unsigned rem = s - (unsigned)j * row2;
    const int colour = rem >= (unsigned)g.hx ? 1 : 0;
    const int t = (int)rem - colour * g.hx;
    const int i = 2 * t + ((j + colour) & 1);
    const int oc = colour ^ 1;
    const unsigned row_o = (unsigned)(2 * j + oc) * (unsigned)g.hx;
    c.i = i;
    c.j = j;
    c.s = s;
    c.sw = row_o + (unsigned)((i - 1) >> 1);
    c.se = row_o + (unsigned)((i + 1) >> 1);
    c.ss = (unsigned)(2 * j - 2 + oc) * (unsigned)g.hx + (unsigned)t;
    c.sn = (unsigned)(2 * j + 2 + oc) * (unsigned)g.hx + (unsigned)t;
    c.valid = i < g.nx;
    return c;
}

// Walks one column through the planes computing a = (A + C/dt) v with the
// stored diagonal (op_apply_diag, src/operator3d.h:100-106), and hands each
// plane's (l, index, v, a) to f.
template <class F>
__device__ __forceinline__ void apply_column(const OpView& o, const double* __restrict__ diag,
                                             const double* __restrict__ v, const Col& c, F&& f) {
    const Geo& g = o.g;
    double v_c = v[c.s], v_b = 0.0;
    float gu_b = 0.0f;
    for (int l = 0; l < g.nz; ++l) {
        const unsigned base = (unsigned)l * g.plane;
        const unsigned id = base + c.s;
        const bool up = l < g.nz - 1;
        const double v_a = up ? v[id + g.plane] : 0.0;
        const float gu = o.gU[id];
        double off = 0.0;
        if (c.i > 0) off += (double)o.gE[base + c.sw] * v[base + c.sw];
        if (c.i < g.nx - 1) off += (double)o.gE[id] * v[base + c.se];
        if (c.j > 0) off += (double)o.gN[base + c.ss] * v[base + c.ss];
        if (c.j < g.ny - 1) off += (double)o.gN[id] * v[base + c.sn];
        if (l > 0) off += (double)gu_b * v_b;
        if (up) off += (double)gu * v_a;
        f(l, id, v_c, diag[id] * v_c - off);
        v_b = v_c;
        v_c = v_a;
        gu_b = gu;
    }
}

// ---- the Jacobi-preconditioned iteration (src/pcg3d_gpu.cu:134-264) ---------
// The multigrid modes run the FP64 kernels of k_fp64.cu; these serve the
// Jacobi preconditioner, kept for drop-in completeness.

// r = b - (A + C/dt) x, ||r||^2, ||b||^2 and the start test.
__global__ void __launch_bounds__(NT)
    k_residual(OpView o, const double* __restrict__ diag, const double* __restrict__ b,
               const double* __restrict__ x, double* __restrict__ r, Ctl* ctl, double* part,
               int maxb, Cond cond) {
    const Geo& g = o.g;
    double rr = 0.0, bb = 0.0;
    for (unsigned s = blockIdx.x * NT + threadIdx.x; s < g.plane; s += gridDim.x * NT) {
        const Col c = col_of_slot(g, s);
        if (!c.valid) {
            for (int l = 0; l < g.nz; ++l) r[(unsigned)l * g.plane + s] = 0.0;
            continue;
        }
        apply_column(o, diag, x, c, [&](int, unsigned id, double, double ax) {
            const double bi = b[id];
            const double ri = bi - ax;
            r[id] = ri;
            rr += ri * ri;
            bb += bi * bi;
        });
    }
    block_sum2(rr, bb);
    if (publish2(rr, bb, part, maxb, &ctl->ticket[SL_INIT])) {
        double RR, BB;
        gather2(part, maxb, &ctl->ticket[SL_INIT], RR, BB);
        if (threadIdx.x == 0) {
            ctl->rr = RR;
            ctl->bb = BB;
            if (BB == 0.0) {  // no heat in: x = 0 (src/pcg3d_cpu.cpp:146)
                ctl->bb_zero = 1;
                ctl->converged = 1;
                ctl->relres = 0.0;
                stop_loop(ctl, cond);
            } else {
                const double rel = sqrt(RR / BB);
                ctl->relres = rel;
                if (rel < ctl->tol) {
                    ctl->converged = 1;
                    stop_loop(ctl, cond);
                } else if (!isfinite(rel)) {
                    ctl->breakdown = 1;
                    stop_loop(ctl, cond);
                } else if (ctl->maxit <= 0) {
                    stop_loop(ctl, cond);
                }
            }
        }
    }
}

// x += alpha p, r -= alpha Ap; ||r||^2; convergence test. n2 = n / 2 pairs.
__global__ void __launch_bounds__(NT)
    k_update(unsigned n2, const double* __restrict__ p, const double* __restrict__ Ap,
             double* __restrict__ x, double* __restrict__ r, Ctl* ctl, double* part, int maxb,
             Cond cond) {
    if (loop_done(ctl, cond)) return;
    const double alpha = ctl->alpha;
    const double2* p2 = reinterpret_cast<const double2*>(p);
    const double2* a2 = reinterpret_cast<const double2*>(Ap);
    double2* x2 = reinterpret_cast<double2*>(x);
    double2* r2 = reinterpret_cast<double2*>(r);
    double rr = 0.0, unused = 0.0;
    for (unsigned k = blockIdx.x * NT + threadIdx.x; k < n2; k += gridDim.x * NT) {
        const double2 pv = p2[k], av = a2[k];
        double2 xv = x2[k], rv = r2[k];
        xv.x += alpha * pv.x;
        xv.y += alpha * pv.y;
        rv.x -= alpha * av.x;
        rv.y -= alpha * av.y;
        x2[k] = xv;
        r2[k] = rv;
        rr += rv.x * rv.x;
        rr += rv.y * rv.y;
    }
    block_sum2(rr, unused);
    if (publish2(rr, unused, part, maxb, &ctl->ticket[SL_UPDATE])) {
        double RR, U;
        gather2(part, maxb, &ctl->ticket[SL_UPDATE], RR, U);
        if (threadIdx.x == 0) {
            ctl->rr = RR;
            ctl->iter += 1;
            const double rel = sqrt(RR / ctl->bb);
            ctl->relres = rel;
            if (rel < ctl->tol) {
                ctl->converged = 1;
                stop_loop(ctl, cond);
            } else if (!isfinite(rel)) {
                ctl->breakdown = 1;
                stop_loop(ctl, cond);
            } else if (ctl->iter >= ctl->maxit) {
                stop_loop(ctl, cond);
            }
        }
    }
}

// rz = r.z with z = r * invd; beta = rz_new / rz (src/pcg3d_gpu.cu:121-126).
__global__ void __launch_bounds__(NT)
    k_dot(unsigned n2, const double* __restrict__ r, const double* __restrict__ invd, Ctl* ctl,
          double* part, int maxb, Cond cond) {
    if (loop_done(ctl, cond)) return;
    const double2* r2 = reinterpret_cast<const double2*>(r);
    const double2* d2 = reinterpret_cast<const double2*>(invd);
    double rz = 0.0, unused = 0.0;
    for (unsigned k = blockIdx.x * NT + threadIdx.x; k < n2; k += gridDim.x * NT) {
        const double2 rv = r2[k], dv = d2[k];
        rz += rv.x * (rv.x * dv.x);
        rz += rv.y * (rv.y * dv.y);
    }
    block_sum2(rz, unused);
    if (publish2(rz, unused, part, maxb, &ctl->ticket[SL_DOT])) {
        double RZ, U;
        gather2(part, maxb, &ctl->ticket[SL_DOT], RZ, U);
        if (threadIdx.x == 0) {
            ctl->beta = ctl->iter > 0 ? RZ / ctl->rz : 0.0;
            ctl->rz = RZ;
            if (!isfinite(RZ) || !isfinite(ctl->beta)) {
                ctl->breakdown = 1;
                stop_loop(ctl, cond);
            }
        }
    }
}

// p = z + beta p with z = r * invd (p = z on the first iteration).
__global__ void __launch_bounds__(NT)
    k_update_p(unsigned n2, const double* __restrict__ r, const double* __restrict__ invd,
               double* __restrict__ p, const Ctl* ctl, Cond cond) {
    if (loop_done(ctl, cond)) return;
    const double beta = ctl->beta;
    const bool first = ctl->iter == 0;
    const double2* r2 = reinterpret_cast<const double2*>(r);
    const double2* d2 = reinterpret_cast<const double2*>(invd);
    double2* p2 = reinterpret_cast<double2*>(p);
    for (unsigned k = blockIdx.x * NT + threadIdx.x; k < n2; k += gridDim.x * NT) {
        const double2 rv = r2[k], dv = d2[k];
        const double za = rv.x * dv.x, zb = rv.y * dv.y;
        if (first) {
            p2[k] = make_double2(za, zb);
        } else {
            const double2 pv = p2[k];
            p2[k] = make_double2(za + beta * pv.x, zb + beta * pv.y);
        }
    }
}

// ---- setup and bookkeeping ------------------------------------------------

__global__ void k_to_split_f(Geo g, int planes, const float* __restrict__ in,
                             float* __restrict__ out) {
    const size_t nxy = (size_t)g.nx * g.ny;
    const size_t n = nxy * (size_t)planes;
    for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n;
         c += (size_t)gridDim.x * blockDim.x) {
        const int l = (int)(c / nxy);
        const size_t rem = c - (size_t)l * nxy;
        const int j = (int)(rem / g.nx), i = (int)(rem - (size_t)j * g.nx);
        out[(size_t)l * g.plane + scol(g, i, j)] = in[c];
    }
}

__global__ void k_to_split_d(Geo g, const double* __restrict__ in, double* __restrict__ out) {
    const size_t nxy = (size_t)g.nx * g.ny;
    const size_t n = nxy * (size_t)g.nz;
    for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n;
         c += (size_t)gridDim.x * blockDim.x) {
        const int l = (int)(c / nxy);
        const size_t rem = c - (size_t)l * nxy;
        const int j = (int)(rem / g.nx), i = (int)(rem - (size_t)j * g.nx);
        out[(size_t)l * g.plane + scol(g, i, j)] = in[c];
    }
}

__global__ void k_to_natural_d(Geo g, const double* __restrict__ in, double* __restrict__ out) {
    const size_t nxy = (size_t)g.nx * g.ny;
    const size_t n = nxy * (size_t)g.nz;
    for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n;
         c += (size_t)gridDim.x * blockDim.x) {
        const int l = (int)(c / nxy);
        const size_t rem = c - (size_t)l * nxy;
        const int j = (int)(rem / g.nx), i = (int)(rem - (size_t)j * g.nx);
        out[c] = in[(size_t)l * g.plane + scol(g, i, j)];
    }
}

// op_diag (src/operator3d.h:80-88) in double with every rounding explicit
// (no contraction), so the diagonal equals the CPU's bit for bit.
__global__ void k_diag(OpView o, const double* __restrict__ dface, double inv_dt, double* __restrict__ diag,
                       double* __restrict__ invd) {
    const size_t ncol = (size_t)o.g.nx * o.g.ny;
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < ncol;
         q += (size_t)gridDim.x * blockDim.x)
        setupdev::diag_column(o, dface, inv_dt, (unsigned)q, diag, invd, nullptr);
}

// Its face part, once per operator.
__global__ void k_faces(OpView o, double* __restrict__ dface) {
    const size_t ncol = (size_t)o.g.nx * o.g.ny;
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < ncol;
         q += (size_t)gridDim.x * blockDim.x)
        setupdev::faces_column(o, (unsigned)q, dface);
}

// The control block of a solve, set from the launch's own arguments (so
// that solves queued one after another never share a host buffer), and the
// zeroing of x that a solve with no heat in asks for (bb_zero), done on the
// device after the solve so that queued solves need no host step between
// them.
__global__ void k_ctl_set(Ctl* ctl, Ctl c) { *ctl = c; }
__global__ void k_zero_if_no_heat(const Ctl* ctl, unsigned n, double* x, float2* xw) {
    if (!*(volatile const int*)&ctl->bb_zero) return;
    for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        x[k] = 0.0;
        if (xw) xw[k] = make_float2(0.0f, 0.0f);
    }
}

__global__ void k_rhs_transient(unsigned n, const float* __restrict__ cap, double inv_dt,
                                const double* __restrict__ P, const double* __restrict__ x,
                                double* __restrict__ b, double* __restrict__ xold) {
    for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const double xv = x[k];
        // b = P + C/dt x, rounded as the reference rounds it (src/pcg3d_cpu.cpp:64)
        b[k] = __dadd_rn(P[k], __dmul_rn(__dmul_rn((double)cap[k], inv_dt), xv));
        xold[k] = xv;
    }
}

// true_relres (src/pcg3d_cpu.cpp:207-220): the steady residual P - A x with
// the diagonal rebuilt from the faces, in FP64.
__global__ void __launch_bounds__(NT)
    k_true_residual(OpView o, const double* __restrict__ P, const double* __restrict__ x, Ctl* ctl,
                    double* part, int maxb) {
    const Geo& g = o.g;
    double rr = 0.0, bb = 0.0;
    for (unsigned s = blockIdx.x * NT + threadIdx.x; s < g.plane; s += gridDim.x * NT) {
        const Col c = col_of_slot(g, s);
        if (!c.valid) continue;
        double x_c = x[c.s], x_b = 0.0;
        float gu_b = 0.0f;
        for (int l = 0; l < g.nz; ++l) {
            const unsigned base = (unsigned)l * g.plane, id = base + c.s;
            const bool up = l < g.nz - 1;
            const double x_a = up ? x[id + g.plane] : 0.0;
            const float gu = o.gU[id];
            double d = 0.0, off = 0.0;
            if (c.i > 0) {
                d += (double)o.gE[base + c.sw];
                off += (double)o.gE[base + c.sw] * x[base + c.sw];
            }
            if (c.i < g.nx - 1) {
                d += (double)o.gE[id];
                off += (double)o.gE[id] * x[base + c.se];
            }
            if (c.j > 0) {
                d += (double)o.gN[base + c.ss];
                off += (double)o.gN[base + c.ss] * x[base + c.ss];
            }
            if (c.j < g.ny - 1) {
                d += (double)o.gN[id];
                off += (double)o.gN[id] * x[base + c.sn];
            }
            d += (double)gu;
            d += l > 0 ? (double)gu_b : (double)o.gB[c.s];
            if (l > 0) off += (double)gu_b * x_b;
            if (up) off += (double)gu * x_a;
            const double res = P[id] - (d * x_c - off);
            rr += res * res;
            bb += P[id] * P[id];
            x_b = x_c;
            x_c = x_a;
            gu_b = gu;
        }
    }
    block_sum2(rr, bb);
    if (publish2(rr, bb, part, maxb, &ctl->ticket[SL_AUX])) {
        double RR, BB;
        gather2(part, maxb, &ctl->ticket[SL_AUX], RR, BB);
        if (threadIdx.x == 0) {
            ctl->aux0 = RR;
            ctl->aux1 = BB;
        }
    }
}

// T_max, heat_out and sum C (x - xold) (src/stack3d.h:252-273).
__global__ void __launch_bounds__(NT)
    k_step_record(OpView o, const double* __restrict__ x, const double* __restrict__ xold,
                  Ctl* ctl, double* part, int maxb) {
    const Geo& g = o.g;
    double tmax = -INFINITY, qout = 0.0, qst = 0.0;
    for (unsigned s = blockIdx.x * NT + threadIdx.x; s < g.plane; s += gridDim.x * NT) {
        const Col c = col_of_slot(g, s);
        if (!c.valid) continue;
        for (int l = 0; l < g.nz; ++l) {
            const unsigned id = (unsigned)l * g.plane + s;
            const double xv = x[id];
            tmax = fmax(tmax, xv);
            qst += (double)o.cap[id] * (xv - xold[id]);
        }
        const unsigned top = (unsigned)(g.nz - 1) * g.plane + s;
        qout += (double)o.gU[top] * x[top];
        qout += (double)o.gB[s] * x[s];
    }
    // block max of tmax (fixed tree), then the two sums
    __shared__ double sm[NT / 32];
    double m = tmax;
    for (int off = 16; off > 0; off >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, off));
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        m = threadIdx.x < NT / 32 ? sm[threadIdx.x] : -INFINITY;
        for (int off = 16; off > 0; off >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, off));
    }
    block_sum2(qout, qst);
    if (threadIdx.x == 0) part[2 * maxb + blockIdx.x] = m;
    if (publish2(qout, qst, part, maxb, &ctl->ticket[SL_AUX])) {
        double QO, QS;
        __threadfence();
        double mm = -INFINITY;
        for (int k = threadIdx.x; k < (int)gridDim.x; k += NT) mm = fmax(mm, __ldcg(part + 2 * maxb + k));
        for (int off = 16; off > 0; off >>= 1) mm = fmax(mm, __shfl_down_sync(0xffffffffu, mm, off));
        __syncthreads();
        if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = mm;
        __syncthreads();
        if (threadIdx.x < 32) {
            mm = threadIdx.x < NT / 32 ? sm[threadIdx.x] : -INFINITY;
            for (int off = 16; off > 0; off >>= 1) mm = fmax(mm, __shfl_down_sync(0xffffffffu, mm, off));
        }
        gather2(part, maxb, &ctl->ticket[SL_AUX], QO, QS);
        if (threadIdx.x == 0) {
            ctl->aux0 = mm;
            ctl->aux1 = QO;
            ctl->aux2 = QS;
        }
    }
}

unsigned grid_for(size_t n, int threads = NT) {
    size_t b = (n + threads - 1) / threads;
    if (b < 1) b = 1;
    if (b > 65535u * 16u) b = 65535u * 16u;
    return (unsigned)b;
}

}  // namespace

bool pdl_enabled() {
    static const bool on = [] {
        const char* e = std::getenv("CT_PDL");
        return !(e && e[0] == '0');
    }();
    return on;
}

void launch_residual(cudaStream_t st, MgType mt, const OpView& o, const double* diag,
                     const double* b, const double* x, double* r, void* b0, Ctl* ctl,
                     const Red& red, Cond cond) {
    if (mt != MG_NONE) {
        launch_residual64(st, mt, o, o.g.plane * (unsigned)o.g.nz, diag, b, x, r, b0, ctl, red, cond);
        return;
    }
    static const int wb = wave_blocks(k_residual, 1 << 30);
    k_residual<<<std::min(red.blocks, wb), NT, 0, st>>>(o, diag, b, x, r, ctl, red.part, red.maxb, cond);
}

void launch_apply(cudaStream_t st, const OpView& o, const double* diag, const double* p,
                  double* Ap, Ctl* ctl, const Red& red, Cond cond) {
    launch_apply64(st, o, diag, p, Ap, ctl, red, cond);
}

void launch_update(cudaStream_t st, MgType mt, unsigned n, const double* p, const double* Ap,
                   double* x, double* r, void* b0, Ctl* ctl, const Red& red, Cond cond, bool write_x) {
    if (mt != MG_NONE) {
        launch_update64(st, mt, n, p, Ap, x, r, b0, ctl, red, cond, write_x);
        return;
    }
    static const int wb = wave_blocks(k_update, 1 << 30);
    k_update<<<std::min(red.blocks, wb), NT, 0, st>>>(n / 2, p, Ap, x, r, ctl, red.part, red.maxb, cond);
}

void launch_dot(cudaStream_t st, MgType mt, bool flexible, unsigned n, const double* r,
                const void* z, const double* invd, const double* Ap, Ctl* ctl, const Red& red,
                Cond cond) {
    if (mt != MG_NONE) {
        launch_dot64(st, mt, flexible, n, r, z, Ap, ctl, red, cond);
        return;
    }
    static const int wb = wave_blocks(k_dot, 1 << 30);
    k_dot<<<std::min(red.blocks, wb), NT, 0, st>>>(n / 2, r, invd, ctl, red.part, red.maxb, cond);
}

void launch_update_p(cudaStream_t st, MgType mt, unsigned n, const void* z, const double* r,
                     const double* invd, double* p, Ctl* ctl, Cond cond) {
    if (mt != MG_NONE) {
        launch_update_p64(st, mt, n, z, p, ctl, cond);
        return;
    }
    static const int wb = wave_blocks(k_update_p, 1 << 30);
    k_update_p<<<std::min(grid_for(n / 2), (unsigned)wb), NT, 0, st>>>(n / 2, r, invd, p, ctl, cond);
}

void launch_to_split_f(cudaStream_t st, const Geo& g, int planes, const float* nat, float* split) {
    k_to_split_f<<<grid_for((size_t)g.nx * g.ny * planes), NT, 0, st>>>(g, planes, nat, split);
}

void launch_to_split_d(cudaStream_t st, const Geo& g, const double* nat, double* split) {
    k_to_split_d<<<grid_for((size_t)g.nx * g.ny * g.nz), NT, 0, st>>>(g, nat, split);
}

void launch_to_natural_d(cudaStream_t st, const Geo& g, const double* split, double* nat) {
    k_to_natural_d<<<grid_for((size_t)g.nx * g.ny * g.nz), NT, 0, st>>>(g, split, nat);
}

// Self-test of the bounded waits: one warp waits on an mbarrier whose phase
// nothing completes (no arrival, no copy), with `limit` polls, through the
// same wait the staged kernels use, and records in *status 1 when the wait
// ran out, 2 if it (wrongly) completed. The kernel then returns normally.
__global__ void k_wait_selftest(unsigned limit, int* status) {
    __shared__ uint64_t bar;
    __shared__ int abort;
    if (threadIdx.x == 0) {
        tma::mbar_init(&bar, 1);
        abort = 0;
        tma::fence_barrier_init();
    }
    __syncwarp();
    const bool got = tma::mbar_wait_or_abort(&bar, 0u, &abort, limit);
    if (threadIdx.x == 0) *status = got ? 2 : (abort ? 1 : 3);
}

cudaError_t launch_wait_selftest(cudaStream_t st, unsigned limit, int* status) {
    k_wait_selftest<<<1, 32, 0, st>>>(limit, status);
    return cudaGetLastError();
}

void launch_faces(cudaStream_t st, const OpView& o, double* dface) {
    k_faces<<<grid_for((size_t)o.g.nx * o.g.ny), NT, 0, st>>>(o, dface);
}

void launch_diag(cudaStream_t st, const OpView& o, const double* dface, double inv_dt, double* diag,
                 double* invd) {
    k_diag<<<grid_for((size_t)o.g.nx * o.g.ny), NT, 0, st>>>(o, dface, inv_dt, diag, invd);
}

void launch_ctl_set(cudaStream_t st, Ctl* ctl, const Ctl& c) { k_ctl_set<<<1, 1, 0, st>>>(ctl, c); }

void launch_zero_if_no_heat(cudaStream_t st, const Ctl* ctl, unsigned n, double* x, float2* xw) {
    // a few blocks striding over x: almost always they read the flag and leave
    k_zero_if_no_heat<<<std::min(grid_for(n), 256u), NT, 0, st>>>(ctl, n, x, xw);
}

void launch_rhs_transient(cudaStream_t st, unsigned n, const float* cap, double inv_dt,
                          const double* P, const double* x, double* b, double* xold) {
    k_rhs_transient<<<grid_for(n), NT, 0, st>>>(n, cap, inv_dt, P, x, b, xold);
}

void launch_true_residual(cudaStream_t st, const OpView& o, const double* P, const double* x,
                          Ctl* ctl, const Red& red) {
    k_true_residual<<<red.blocks, NT, 0, st>>>(o, P, x, ctl, red.part, red.maxb);
}

void launch_step_record(cudaStream_t st, const OpView& o, const double* x, const double* xold,
                        Ctl* ctl, const Red& red) {
    k_step_record<<<red.blocks, NT, 0, st>>>(o, x, xold, ctl, red.part, red.maxb);
}

// A step's record (the step-record sums and the last solve's statistics) into
// entry `slot` of the device table.
__global__ void k_record_keep(const Ctl* ctl, double dt, StepEntry* table, int slot) {
    StepEntry e;
    e.T_max = ctl->aux0;
    e.q_out = ctl->aux1;
    e.q_stored = ctl->aux2 / dt;  // IEEE division, as ct_solver_step_record divides on the host
    e.relres = ctl->relres;
    e.iters = ctl->iter;
    e.converged = ctl->converged;
    e.breakdown = ctl->breakdown;
    e.err = ctl->err;
    table[slot] = e;
}

void launch_record_keep(cudaStream_t st, const Ctl* ctl, double dt, StepEntry* table, int slot) {
    k_record_keep<<<1, 1, 0, st>>>(ctl, dt, table, slot);
}

}  // namespace ct
