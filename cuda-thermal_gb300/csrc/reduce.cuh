// reduce.cuh - deterministic grid reductions for the solver kernels.
//
// Each reducing kernel sums two doubles per thread, then per block (a fixed
// warp-shuffle tree), writes the block's pair to its slot's partials and takes
// a ticket. The block that takes the last ticket adds the partials in block
// order with the same fixed tree and finishes the iteration's scalar work
// (alpha, beta, the convergence test). No floating-point atomics, so the same
// inputs give the same bits on every run and in graph or direct launches.
// The double-word kernels (k_dw.cu, k_batch.cu) run the same trees on float
// pairs instead (block_sum_acc2 / publish_acc2 / gather_acc2 in dw_dev.cuh).
#pragma once
#include "device.h"

namespace ct {

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Block sum of (a, b) over NTH threads (at most 32 warps); the result is
// valid in thread 0.
template <int NTH = NT>
__device__ __forceinline__ void block_sum2(double& a, double& b) {
    constexpr int NW = NTH / 32;
    static_assert(NTH % 32 == 0 && NW <= 32, "whole warps, at most 32");
    __shared__ double sa[NW], sb[NW];
    a = warp_sum(a);
    b = warp_sum(b);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        sa[w] = a;
        sb[w] = b;
    }
    __syncthreads();
    if (w == 0) {
        a = lane < NW ? sa[lane] : 0.0;
        b = lane < NW ? sb[lane] : 0.0;
        a = warp_sum(a);
        b = warp_sum(b);
    }
}

// Publishes the block's sums (valid in thread 0) and returns, in every
// thread, whether this block arrived last.
__device__ __forceinline__ bool publish2(double a, double b, double* part, int maxb,
                                         unsigned* ticket) {
    __shared__ int last;
    if (threadIdx.x == 0) {
        part[blockIdx.x] = a;
        part[maxb + blockIdx.x] = b;
        __threadfence();
        const unsigned t = atomicAdd(ticket, 1u);
        last = (t == gridDim.x - 1) ? 1 : 0;
    }
    __syncthreads();
    return last != 0;
}

// In the last block (NTH threads): the grid totals, valid in thread 0.
// Resets the ticket.
template <int NTH = NT>
__device__ __forceinline__ void gather2(const double* part, int maxb, unsigned* ticket, double& A,
                                        double& B) {
    __threadfence();
    double a = 0.0, b = 0.0;
    for (int k = threadIdx.x; k < (int)gridDim.x; k += NTH) {
        a += __ldcg(part + k);
        b += __ldcg(part + maxb + k);
    }
    block_sum2<NTH>(a, b);
    if (threadIdx.x == 0) {
        A = a;
        B = b;
        *ticket = 0u;
    }
}

// Stops the solve: marks it done and, inside a graph loop, ends the loop
// after the current body. Called by one thread.
__device__ __forceinline__ void stop_loop(Ctl* c, const Cond& cond) {
    c->done = 1;
    if (cond.use) cudaGraphSetConditional(cond.h, 0u);
}

// Entry test of every loop-body kernel: once the solve is done (or, in the
// double-word mode, once its first phase is), the rest of the body is a
// no-op, and (inside a graph loop) the loop is told to end.
// loop_flags loads the two flags it tests (done, phase_end) on their own,
// so that a short kernel can issue its first loads before it waits for them
// and test them before its first store.
__device__ __forceinline__ int2 loop_flags(const Ctl* c) {
    return __ldcv(reinterpret_cast<const int2*>(&c->done));
}
__device__ __forceinline__ bool loop_done(int2 f, const Cond& cond) {
    if (f.x | f.y) {
        if (cond.use && blockIdx.x == 0 && threadIdx.x == 0) cudaGraphSetConditional(cond.h, 0u);
        return true;
    }
    return false;
}
__device__ __forceinline__ bool loop_done(const Ctl* c, const Cond& cond) {
    return loop_done(loop_flags(c), cond);
}

}  // namespace ct
