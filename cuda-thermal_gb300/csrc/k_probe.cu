// k_probe.cu - a timing probe of this GPU behind one design choice of the
// batched solver: its iteration is a CUDA graph of one launch per stage (all
// instances of a size bucket per launch), not one persistent kernel with a
// grid-wide barrier between stages. The probe times the two ways of
// separating dependent phases on the same grid:
//   * one cooperative (persistent) kernel that runs every phase, with a
//     grid-wide barrier (arrival counter + generation flag, bounded spin)
//     between phases;
//   * one captured graph of one launch per phase, each launched with
//     programmatic dependent launch and waiting on its predecessor
//     (griddepcontrol.wait), as the solver's graphs are.
// Each phase is a real dependency: block b reads what block b + 1 wrote in
// the previous phase (double-buffered), so no phase can run ahead.
#include <cuda_runtime.h>

#include "kernels.h"

namespace ct {

namespace {

// Polls of the generation flag before a barrier wait gives up (about a
// second); a wait that gives up records it and ends the kernel.
constexpr long long kBarrierPolls = 1ll << 21;

struct SyncState {
    unsigned count;  // blocks arrived at the current barrier
    unsigned gen;    // barriers completed
    int err;         // a wait gave up
};

__device__ __forceinline__ void phase_step(unsigned* buf, unsigned nb, int ph) {
    if (threadIdx.x == 0) {
        const unsigned b = blockIdx.x;
        const unsigned* src = buf + (size_t)((ph + 1) & 1) * nb;
        unsigned* dst = buf + (size_t)(ph & 1) * nb;
        dst[b] = __ldcg(&src[(b + 1) % nb]) + 1u;
    }
}

// gen0: barriers completed before this launch (the flag's value at entry).
__global__ void k_sync_persistent(unsigned* buf, SyncState* s, int phases, unsigned gen0) {
    __shared__ int ok;
    const unsigned nb = gridDim.x;
    unsigned gen = gen0;
    if (threadIdx.x == 0) ok = *(volatile int*)&s->err == 0;  // an earlier launch gave up: do nothing
    __syncthreads();
    if (!ok) return;
    for (int ph = 0; ph < phases; ++ph) {
        phase_step(buf, nb, ph);
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            if (atomicAdd(&s->count, 1u) == nb - 1u) {
                atomicExch(&s->count, 0u);
                __threadfence();
                atomicExch(&s->gen, gen + 1u);
            } else {
                long long n = 0;
                while (*(volatile unsigned*)&s->gen == gen) {
                    if (++n > kBarrierPolls || *(volatile int*)&s->err) {
                        atomicExch(&s->err, 1);
                        ok = 0;
                        break;
                    }
                }
                __threadfence();
            }
            gen += 1u;
        }
        __syncthreads();
        if (!ok) return;
    }
}

__global__ void k_sync_phase(unsigned* buf, int ph) {
    pdl_enter();
    phase_step(buf, gridDim.x, ph);
}

}  // namespace

cudaError_t measure_sync_costs(int phases, int blocks_per_sm, double* us_barrier, double* us_launch,
                               int* blocks, int* gave_up) {
    int dev = 0, sms = 0, per = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_sync_persistent, NT, 0);
    if (e != cudaSuccess) return e;
    // every block of the persistent kernel must be resident at once
    const int bps = blocks_per_sm < 1 ? 1 : (blocks_per_sm > per ? per : blocks_per_sm);
    const unsigned nb = (unsigned)(sms * bps);
    *blocks = (int)nb;
    unsigned* buf = nullptr;
    SyncState* s = nullptr;
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaGraph_t g = nullptr;
    cudaGraphExec_t gx = nullptr;
    float ms_bar = 0.0f, ms_launch = 0.0f;
    int herr = 0;
    constexpr int kReps = 3;
    e = cudaMalloc(&buf, 2 * (size_t)nb * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMalloc(&s, sizeof(SyncState));
    if (e == cudaSuccess) e = cudaMemset(buf, 0, 2 * (size_t)nb * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMemset(s, 0, sizeof(SyncState));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    // persistent kernel, phases grid barriers per launch
    unsigned gen0 = 0;
    void* args[4] = {&buf, &s, &phases, &gen0};
    for (int r = 0; e == cudaSuccess && r <= kReps; ++r) {
        if (r == 1) e = cudaEventRecord(e0, st);  // the first launch is a warm-up
        gen0 = (unsigned)(r * phases);             // read when the launch is enqueued
        if (e == cudaSuccess)
            e = cudaLaunchCooperativeKernel((const void*)k_sync_persistent, dim3(nb), dim3(NT), args, 0, st);
    }
    if (e == cudaSuccess) e = cudaEventRecord(e1, st);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms_bar, e0, e1);
    if (e == cudaSuccess) e = cudaMemcpy(&herr, &s->err, sizeof(int), cudaMemcpyDeviceToHost);
    // one graph of phases dependent launches
    if (e == cudaSuccess) e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        for (int ph = 0; ph < phases; ++ph) launch_pdl(k_sync_phase, dim3(nb), dim3(NT), 0, st, buf, ph);
        e = cudaStreamEndCapture(st, &g);
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&gx, g, 0);
    for (int r = 0; e == cudaSuccess && r <= kReps; ++r) {
        if (r == 1) e = cudaEventRecord(e0, st);
        if (e == cudaSuccess) e = cudaGraphLaunch(gx, st);
    }
    if (e == cudaSuccess) e = cudaEventRecord(e1, st);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms_launch, e0, e1);
    if (gx) cudaGraphExecDestroy(gx);
    if (g) cudaGraphDestroy(g);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (st) cudaStreamDestroy(st);
    if (buf) cudaFree(buf);
    if (s) cudaFree(s);
    if (e != cudaSuccess) return e;
    *gave_up = herr;
    *us_barrier = 1e3 * ms_bar / (kReps * (double)phases);
    *us_launch = 1e3 * ms_launch / (kReps * (double)phases);
    return cudaSuccess;
}

}  // namespace ct
