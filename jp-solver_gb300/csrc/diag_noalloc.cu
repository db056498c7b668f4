// Energy / enstrophy / mass of a caller-owned macro field without any device allocation.
//
// Some callers cannot allocate device memory at the moment they need the diagnostics: a host
// framework that owns all device memory through its own pool (and forbids cudaMalloc behind its
// back), or a real-time loop that must not allocate after start-up.  jp_diag() keeps its reduction
// partials in memory the solver allocated; this variant keeps them in a fixed array compiled into
// the library instead, so it only needs the caller's input field and output buffer, both in device
// memory of the current device (checked before any work is queued).
//
// The scratch is a file-scope __device__ array of kMaxChunks partial triples (384 KiB).  Every GPU
// that loads this library holds it until the process exits.  Each CTA reduces one chunk of kChunk
// cells into one partial, so a field may have at most kMaxChunks * kChunk = 268,435,456 cells
// (edge n <= 645); larger fields are rejected with JP_ERR_CAPACITY before any work is queued.
// All calls share the array: calls that overlap on the GPU (different streams, or different host
// threads without ordering) race on it and must be serialised by the caller.  Each call overwrites
// every partial it reads, so nothing has to be cleared between calls.
//
// Host code cannot use the array's name as a device address (it names a host-side stand-in); the
// device address is looked up with cudaGetSymbolAddress on the first call made with a device's
// context current, and looked up again when that context has been replaced (cudaDeviceReset tears
// the primary context down and the next one loads the module anew, possibly elsewhere).
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "diag_terms.cuh"
#include "jp.h"
#include "solver.h"

namespace jp {
namespace {

constexpr int kChunk = 16384;      // cells per CTA
constexpr int kMaxChunks = 16384;  // partial triples in the scratch array
constexpr int kThreads = 256;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_partials[kMaxChunks * 3];

// per device: the context the address was looked up in (its process-unique id) and the address
struct ScratchSlot {
    unsigned long long ctx_id;
    double* addr;
};
std::mutex g_setup_mutex;
ScratchSlot g_slots[kMaxDevices] = {};

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// One partial (E, enstrophy, mass sums) per chunk of kChunk cells.  Per cell: 1/2|u|^2,
// 1/2|curl u|^2 from central differences with periodic wrap, rho, in double-float
// (diag_terms.cuh); FP64 accumulation.  float_diff takes each velocity difference in float before
// halving (the uniform solver's convention).
template <bool VEC>
__global__ void __launch_bounds__(kThreads) k_noalloc_partials(const float* __restrict__ F, int n, int float_diff,
                                                              double* __restrict__ partials) {
    const long long cells = (long long)n * n * n;
    const long long begin = (long long)blockIdx.x * kChunk;
    const long long end = begin + kChunk < cells ? begin + kChunk : cells;
    dterm::Acc acc;
    dterm::CellWalk w(begin + threadIdx.x, kThreads, n);
    for (long long c = begin + threadIdx.x; c < end; c += kThreads, w.next()) {
        dterm::FF ce, cens;
        float rho;
        if (float_diff) dterm::cell_terms<true, VEC>(F, n, w.i, w.j, w.k, ce, cens, rho);
        else dterm::cell_terms<false, VEC>(F, n, w.i, w.j, w.k, ce, cens, rho);
        acc.add_cell(ce, cens, rho);
    }
    acc.flush();
    double e = acc.de, ens = acc.dens, mass = acc.dmass;
    __shared__ double sh[3][kThreads / 32];
    e = warp_sum(e);
    ens = warp_sum(ens);
    mass = warp_sum(mass);
    if ((threadIdx.x & 31) == 0) {
        sh[0][threadIdx.x >> 5] = e;
        sh[1][threadIdx.x >> 5] = ens;
        sh[2][threadIdx.x >> 5] = mass;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double t = 0.0;
        for (int wi = 0; wi < kThreads / 32; ++wi) t += sh[threadIdx.x][wi];
        partials[blockIdx.x * 3 + threadIdx.x] = t;
    }
}

// Sum the partials in a fixed order; out = sums / cells.
__global__ void __launch_bounds__(kThreads) k_noalloc_finish(const double* __restrict__ partials, int nparts,
                                                            double inv_cells, double* __restrict__ out) {
    double a[3] = {0.0, 0.0, 0.0};
    for (int p = threadIdx.x; p < nparts; p += kThreads) {
        a[0] += partials[p * 3 + 0];
        a[1] += partials[p * 3 + 1];
        a[2] += partials[p * 3 + 2];
    }
    __shared__ double sh[3][kThreads / 32];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const double t = warp_sum(a[k]);
        if ((threadIdx.x & 31) == 0) sh[k][threadIdx.x >> 5] = t;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double t = 0.0;
        for (int wi = 0; wi < kThreads / 32; ++wi) t += sh[threadIdx.x][wi];
        out[threadIdx.x] = t * inv_cells;
    }
}

// Id of the calling thread's current context (0: none yet).  The two driver calls are reached
// through the runtime's entry-point table, so the library needs no link against the driver.
jp_status current_context_id(unsigned long long* id) {
    if (!g_ctx_get_current || !g_ctx_get_id) {
        void* f0 = nullptr;
        void* f1 = nullptr;
        cudaDriverEntryPointQueryResult q0 = cudaDriverEntryPointSymbolNotFound, q1 = q0;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f0, 12000, cudaEnableDefault, &q0);
        if (e == cudaSuccess) e = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f1, 12000, cudaEnableDefault, &q1);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetDriverEntryPointByVersion");
        if (q0 != cudaDriverEntryPointSuccess || q1 != cudaDriverEntryPointSuccess || !f0 || !f1)
            return fail(JP_ERR_CUDA, "jp_diag_field_noalloc: driver lacks cuCtxGetCurrent / cuCtxGetId");
        g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(f0);
        g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(f1);
    }
    CUcontext ctx = nullptr;
    if (g_ctx_get_current(&ctx) != CUDA_SUCCESS) return fail(JP_ERR_CUDA, "cuCtxGetCurrent failed");
    *id = 0;
    if (ctx && g_ctx_get_id(ctx, id) != CUDA_SUCCESS) return fail(JP_ERR_CUDA, "cuCtxGetId failed");
    return JP_OK;
}

// Device address of the scratch array in the current device's current context: looked up once per
// device and context, again after the context was replaced.
jp_status scratch_address(int dev, double** out) {
    if (dev < 0 || dev >= kMaxDevices) return fail(JP_ERR_INVALID, "device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    unsigned long long id = 0;
    jp_status st = current_context_id(&id);
    if (st != JP_OK) return st;
    ScratchSlot& slot = g_slots[dev];
    if (id == 0 || !slot.addr || slot.ctx_id != id) {
        double* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress((void**)&p, g_noalloc_partials);  // makes the context current
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress");
        st = current_context_id(&id);
        if (st != JP_OK) return st;
        slot.ctx_id = id;
        slot.addr = p;
    }
    *out = slot.addr;
    return JP_OK;
}

// The caller's buffer must be device (or managed) memory reachable on device `dev`: a host pointer
// or another GPU's memory would fault in the kernel, so it is refused here.
jp_status check_on_device(const void* p, int dev, const char* what) {
    cudaPointerAttributes at{};
    cudaError_t e = cudaPointerGetAttributes(&at, p);
    if (e != cudaSuccess) return cuda_fail(e, "cudaPointerGetAttributes");
    if (at.type == cudaMemoryTypeManaged) return JP_OK;
    if (at.type != cudaMemoryTypeDevice)
        return fail(JP_ERR_INVALID, "jp_diag_field_noalloc: %s is not device memory", what);
    if (at.device != dev)
        return fail(JP_ERR_INVALID, "jp_diag_field_noalloc: %s lives on device %d, device %d is current", what,
                    at.device, dev);
    return JP_OK;
}

}  // namespace
}  // namespace jp

extern "C" jp_status jp_diag_field_noalloc(const float* field_dev, int32_t n, int32_t float_diff, double* out_dev,
                                           void* stream) {
    using namespace jp;
    if (!field_dev || !out_dev) return fail(JP_ERR_INVALID, "jp_diag_field_noalloc: null pointer");
    if (n <= 0) return fail(JP_ERR_INVALID, "jp_diag_field_noalloc: n must be positive (got %d)", n);
    const long long cells = (long long)n * n * n;
    const long long chunks = (cells + kChunk - 1) / kChunk;
    if (chunks > kMaxChunks)
        return fail(JP_ERR_CAPACITY,
                    "jp_diag_field_noalloc: %lld cells exceed the fixed scratch (at most %lld cells, n <= 645)", cells,
                    (long long)kMaxChunks * kChunk);
    int dev = 0;
    cudaError_t de = cudaGetDevice(&dev);
    if (de != cudaSuccess) return cuda_fail(de, "cudaGetDevice");
    double* partials = nullptr;
    jp_status st = scratch_address(dev, &partials);
    if (st == JP_OK) st = check_on_device(field_dev, dev, "the field");
    if (st == JP_OK) st = check_on_device(out_dev, dev, "the output");
    if (st != JP_OK) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // a caller's field may start anywhere a float can: 16-byte record loads only where aligned
    if (reinterpret_cast<uintptr_t>(field_dev) % 16 == 0)
        k_noalloc_partials<true><<<(unsigned)chunks, kThreads, 0, s>>>(field_dev, n, float_diff ? 1 : 0, partials);
    else
        k_noalloc_partials<false><<<(unsigned)chunks, kThreads, 0, s>>>(field_dev, n, float_diff ? 1 : 0, partials);
    k_noalloc_finish<<<1, kThreads, 0, s>>>(partials, (int)chunks, 1.0 / double(cells), out_dev);
    note_launch(2);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "jp_diag_field_noalloc launch");
    return JP_OK;
}
