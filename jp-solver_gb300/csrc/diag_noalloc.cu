// Energy / enstrophy / mass of a caller-owned macro field without any device allocation.
//
// Some callers cannot allocate device memory at the moment they need the diagnostics: a host
// framework that owns all device memory through its own pool (and forbids cudaMalloc behind its
// back), a real-time loop that must not allocate after start-up, or code that records work into a
// CUDA graph.  jp_diag() keeps its reduction partials in memory the solver allocated; this variant
// keeps them in a fixed array compiled into the library instead, so it only needs the caller's input
// field and output buffer.
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
// device address is looked up once per device with cudaGetSymbolAddress, on the first call made with
// that device current.  That first call may load the module, so it should come before any stream
// capture.
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

std::mutex g_setup_mutex;
double* g_partials_addr[kMaxDevices] = {};

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

// Device address of the scratch array on the current device, looked up once per device.
jp_status scratch_address(double** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) return fail(JP_ERR_INVALID, "device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_partials_addr[dev]) {
        double* p = nullptr;
        e = cudaGetSymbolAddress((void**)&p, g_noalloc_partials);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress");
        g_partials_addr[dev] = p;
    }
    *out = g_partials_addr[dev];
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
    double* partials = nullptr;
    jp_status st = scratch_address(&partials);
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
