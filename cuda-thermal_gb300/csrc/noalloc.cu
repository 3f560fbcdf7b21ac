// noalloc.cu - ct_true_relres_noalloc: the steady true residual
// ||P - A T|| / ||P|| of a temperature field, for callers that cannot allocate
// device memory.
//
// Who needs it: code that calls the residual check from a place where
// cudaMalloc is not allowed or not safe - a per-frame loop that must not stall
// the device (cudaMalloc can synchronise it), an integration whose host
// framework has reserved the device memory in its own pool (so a fresh
// cudaMalloc can fail), or a plugin that was handed device buffers and no
// allocator. ct_true_relres needs a ct_solver, which owns an allocation; this
// entry point works on the caller's own device arrays and allocates nothing.
//
// Its scratch memory (one pair of partial sums per thread block, a ticket and
// the two totals) lives in the file-scope array g_scratch below, a fixed
// CT_NOALLOC_SCRATCH_BYTES on every GPU that loads the library, held until the
// process exits. One block covers 256 columns, so a model may have at most
// CT_NOALLOC_MAX_COLUMNS = (256 * 8190) columns (nx * ny); larger ones are
// rejected with CT_BAD_ARG. Every call shares the one array and the array
// keeps the last call's contents: each call clears its ticket first, and calls
// whose kernels could overlap on the GPU (other streams, other host threads)
// race on it, so they must be serialised by the caller.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

#include "cthermal.h"
#include "status.h"

namespace {

constexpr int kThreads = 256;
constexpr int kMaxBlocks = 8190;
// Layout of the scratch in doubles: [0, kMaxBlocks) partial ||r||^2,
// [kMaxBlocks, 2 kMaxBlocks) partial ||P||^2, then the ticket (as unsigned).
constexpr int kTicket = 2 * kMaxBlocks;
constexpr int kScratchDoubles = 2 * kMaxBlocks + 4;
static_assert(kScratchDoubles * 8 == CT_NOALLOC_SCRATCH_BYTES, "scratch size");
static_assert((size_t)kThreads * kMaxBlocks == CT_NOALLOC_MAX_COLUMNS, "column limit");

static __device__ __align__(256) double g_scratch[kScratchDoubles];

// The device address of g_scratch, looked up once per device and context.
// In host code the name g_scratch is only a host-side stand-in for the
// symbol, not a device address, so it must never be passed to a kernel. The
// address is cached with the context it was looked up in: after a device
// reset the library's module is loaded again into a new context, where the
// array may sit elsewhere, so a new context means a new lookup.
constexpr int kMaxDevices = 64;
std::mutex g_mu;
struct ScratchAddr {
    void* ctx;
    double* ptr;
};
ScratchAddr g_scratch_addr[kMaxDevices] = {};

using CtxGetCurrentFn = int (*)(void**);
CtxGetCurrentFn ctx_get_current() {
    static CtxGetCurrentFn fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            p = nullptr;
        }
        return reinterpret_cast<CtxGetCurrentFn>(p);
    }();
    return fn;
}

ct_status scratch_for_current_device(double** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return ct::fail(CT_CUDA_ERROR, "cudaGetDevice: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return ct::fail(CT_BAD_ARG, "device %d out of range", dev);
    const CtxGetCurrentFn get = ctx_get_current();
    if (!get) return ct::fail(CT_CUDA_ERROR, "cuCtxGetCurrent not available");
    void* ctx = nullptr;  // null until the runtime has made a context current
    if (get(&ctx) != 0) ctx = nullptr;
    std::lock_guard<std::mutex> lk(g_mu);
    ScratchAddr& a = g_scratch_addr[dev];
    if (!ctx || !a.ptr || a.ctx != ctx) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_scratch);  // also makes the device's context current
        if (e != cudaSuccess || !p)
            return ct::fail(CT_CUDA_ERROR, "cudaGetSymbolAddress(scratch) on device %d: %s", dev,
                            cudaGetErrorString(e));
        if (get(&ctx) != 0 || !ctx)
            return ct::fail(CT_CUDA_ERROR, "no current CUDA context on device %d", dev);
        a.ctx = ctx;
        a.ptr = static_cast<double*>(p);
    }
    *out = a.ptr;
    return CT_OK;
}

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ void block_sum2(double& a, double& b) {
    __shared__ double sa[kThreads / 32], sb[kThreads / 32];
    a = warp_sum(a);
    b = warp_sum(b);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        sa[w] = a;
        sb[w] = b;
    }
    __syncthreads();
    if (w == 0) {
        a = lane < kThreads / 32 ? sa[lane] : 0.0;
        b = lane < kThreads / 32 ? sb[lane] : 0.0;
        a = warp_sum(a);
        b = warp_sum(b);
    }
}

// One thread per column (natural layout), walking up the planes: the steady
// residual P - A T with the diagonal rebuilt from the faces
// (true_relres, src/pcg3d_cpu.cpp:207-220), in FP64. The last block to finish
// adds the per-block partials in block order and writes the ratio.
__global__ void __launch_bounds__(kThreads)
    k_true_relres_nat(ct_model m, const double* __restrict__ T, double* __restrict__ scratch,
                      double* __restrict__ out) {
    const int nx = m.nx, ny = m.ny, nz = m.nz;
    const unsigned ncol = (unsigned)nx * (unsigned)ny;
    const unsigned q = blockIdx.x * kThreads + threadIdx.x;
    double rr = 0.0, bb = 0.0;
    if (q < ncol) {
        const int j = (int)(q / (unsigned)nx), i = (int)(q - (unsigned)j * nx);
        double t_c = T[q], t_b = 0.0;
        float gu_b = 0.0f;
        for (int l = 0; l < nz; ++l) {
            const size_t id = (size_t)l * ncol + q;
            const bool up = l < nz - 1;
            const double t_a = up ? T[id + ncol] : 0.0;
            const float gu = m.gU[id];
            double d = 0.0, off = 0.0;
            if (i > 0) {
                d += (double)m.gE[id - 1];
                off += (double)m.gE[id - 1] * T[id - 1];
            }
            if (i < nx - 1) {
                d += (double)m.gE[id];
                off += (double)m.gE[id] * T[id + 1];
            }
            if (j > 0) {
                d += (double)m.gN[id - nx];
                off += (double)m.gN[id - nx] * T[id - nx];
            }
            if (j < ny - 1) {
                d += (double)m.gN[id];
                off += (double)m.gN[id] * T[id + nx];
            }
            d += (double)gu;
            d += l > 0 ? (double)gu_b : (double)m.gB[q];
            if (l > 0) off += (double)gu_b * t_b;
            if (up) off += (double)gu * t_a;
            const double p = m.P[id];
            const double r = p - (d * t_c - off);
            rr += r * r;
            bb += p * p;
            t_b = t_c;
            t_c = t_a;
            gu_b = gu;
        }
    }
    block_sum2(rr, bb);
    __shared__ int last;
    unsigned* ticket = reinterpret_cast<unsigned*>(scratch + kTicket);
    if (threadIdx.x == 0) {
        scratch[blockIdx.x] = rr;
        scratch[kMaxBlocks + blockIdx.x] = bb;
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1 ? 1 : 0;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double a = 0.0, b = 0.0;
    for (int k = threadIdx.x; k < (int)gridDim.x; k += kThreads) {
        a += __ldcg(scratch + k);
        b += __ldcg(scratch + kMaxBlocks + k);
    }
    block_sum2(a, b);
    if (threadIdx.x == 0) {
        out[0] = sqrt(a / b);
        *ticket = 0u;
    }
}

}  // namespace

extern "C" ct_status ct_true_relres_noalloc(const ct_model* m_dev, const double* T_dev,
                                            double* out_dev, void* stream) {
    if (!m_dev || !T_dev || !out_dev)
        return ct::fail(CT_BAD_ARG, "ct_true_relres_noalloc: null argument");
    const ct_model& m = *m_dev;
    if (m.nx < 1 || m.ny < 1 || m.nz < 1 || m.nz > CT_MAXZ)
        return ct::fail(CT_BAD_ARG, "ct_true_relres_noalloc: bad size %d x %d x %d", m.nx, m.ny, m.nz);
    if (!m.gE || !m.gN || !m.gU || !m.gB || !m.P)
        return ct::fail(CT_BAD_ARG, "ct_true_relres_noalloc: null model array");
    const size_t ncol = (size_t)m.nx * (size_t)m.ny;
    if (ncol > (size_t)CT_NOALLOC_MAX_COLUMNS)
        return ct::fail(CT_BAD_ARG,
                        "ct_true_relres_noalloc: %zu columns (nx * ny) exceed the limit of %d set "
                        "by its fixed %d-byte scratch",
                        ncol, CT_NOALLOC_MAX_COLUMNS, CT_NOALLOC_SCRATCH_BYTES);
    if (ncol * (size_t)m.nz > 0x7fffffffu)
        return ct::fail(CT_BAD_ARG, "ct_true_relres_noalloc: more than 2^31 cells");
    double* scratch = nullptr;
    const ct_status s = scratch_for_current_device(&scratch);
    if (s != CT_OK) return s;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // A call that failed part-way could have left a ticket behind: start at 0.
    cudaError_t e = cudaMemsetAsync(scratch + kTicket, 0, sizeof(double), st);
    if (e != cudaSuccess) return ct::fail(CT_CUDA_ERROR, "cudaMemsetAsync: %s", cudaGetErrorString(e));
    const unsigned blocks = (unsigned)((ncol + kThreads - 1) / kThreads);
    k_true_relres_nat<<<blocks, kThreads, 0, st>>>(m, T_dev, scratch, out_dev);
    e = cudaGetLastError();
    if (e != cudaSuccess) return ct::fail(CT_CUDA_ERROR, "k_true_relres_nat: %s", cudaGetErrorString(e));
    return CT_OK;
}
