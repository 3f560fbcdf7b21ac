// batch_dev.cuh - device helpers of the batched kernels (k_batch.cu,
// k_batch64.cu): the convergence mask and the per-instance deterministic
// reductions over a block table (batch.h).
#pragma once
#include "batch.h"
#include "reduce.cuh"

namespace ct {
namespace {

__device__ __forceinline__ bool inst_done(const Ctl* c) { return *(volatile const int*)&c->done != 0; }

// Marks the instance done; the batch's last active instance ends the loop.
__device__ __forceinline__ void inst_stop(Ctl* c, BCtl* bc, const Cond& cond) {
    if (c->done) return;
    c->done = 1;
    if (atomicSub(&bc->active, 1) == 1 && cond.use) cudaGraphSetConditional(cond.h, 0u);
}

// The block's (a, b) go to its slot of the stage; true in the instance's
// last block.
__device__ __forceinline__ bool publish_inst(double a, double b, const BRed& red, int ntasks,
                                             int inst, int count) {
    __shared__ int last;
    if (threadIdx.x == 0) {
        red.part[blockIdx.x] = a;
        red.part[ntasks + blockIdx.x] = b;
        __threadfence();
        const unsigned t = atomicAdd(&red.tickets[inst], 1u);
        last = (t == (unsigned)count - 1u) ? 1 : 0;
    }
    __syncthreads();
    return last != 0;
}

// In the instance's last block: its totals in block-table order (thread 0).
__device__ __forceinline__ void gather_inst(const BRed& red, int ntasks, int inst, int first,
                                            int count, double& A, double& B) {
    __threadfence();
    double a = 0.0, b = 0.0;
    for (int k = threadIdx.x; k < count; k += NT) {
        a += __ldcg(red.part + first + k);
        b += __ldcg(red.part + ntasks + first + k);
    }
    block_sum2(a, b);
    if (threadIdx.x == 0) {
        A = a;
        B = b;
        red.tickets[inst] = 0u;
    }
}

}  // namespace
}  // namespace ct
