// ORACLE - test infrastructure only.  Runs the reference's own CUDA kernels (compiled from the
// reference checkout into oracle/_ref/*.cubin by oracle/build.py) on host buffers, so tests can pin
// the CPU oracle and the engine against the reference itself.  Host orchestration mirrors the
// reference's main(): src/tgv3d_uniform.cu:157-194.  Built on the GPU host with g++ against the CUDA
// runtime; the cubins are loaded with cudaLibraryLoadFromFile.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

std::string g_err;
cudaLibrary_t g_uni = nullptr;
cudaKernel_t k_init = nullptr, k_step = nullptr, k_macro = nullptr;
const int MB = 8, MB3 = 512, Q = 19;

int seterr(const char* what, cudaError_t e) {
    g_err = std::string(what) + ": " + cudaGetErrorString(e);
    return int(e) ? int(e) : 1;
}
#define RK(call, what)                                  \
    do {                                                \
        cudaError_t e_ = (call);                        \
        if (e_ != cudaSuccess) return seterr(what, e_); \
    } while (0)

int launch(cudaKernel_t k, unsigned grid, unsigned block, void** args) {
    RK(cudaLaunchKernel((const void*)k, dim3(grid), dim3(block), args, 0, 0), "cudaLaunchKernel");
    return 0;
}

}  // namespace

extern "C" {

const char* refrun_last_error(void) { return g_err.c_str(); }

// Load the uniform cubin (reference kernels k_init_tgv3d, k_step, k_macro at MB=8).
int refrun_load_uniform(const char* path) {
    if (g_uni) return 0;
    RK(cudaLibraryLoadFromFile(&g_uni, path, nullptr, nullptr, 0, nullptr, nullptr, 0), "cudaLibraryLoadFromFile");
    RK(cudaLibraryGetKernel(&k_init, g_uni, "_Z12k_init_tgv3dPfiidd"), "k_init_tgv3d");
    RK(cudaLibraryGetKernel(&k_step, g_uni, "_Z6k_stepPKfPfiif"), "k_step");
    RK(cudaLibraryGetKernel(&k_macro, g_uni, "_Z7k_macroPKfiiPf"), "k_macro");
    return 0;
}

// k_init_tgv3d into host_f (19*N^3 floats, reference blocked layout, MB=8).
int ref_uniform_init(float* host_f, int N, double u0) {
    if (!g_uni) { g_err = "uniform cubin not loaded"; return 1; }
    if (N % MB) { g_err = "N%MB"; return 2; }
    int gx = N / MB, nb = gx * gx * gx;
    double kf = 2.0 * M_PI / double(N);
    size_t bytes = (size_t)nb * Q * MB3 * 4;
    float* f = nullptr;
    RK(cudaMalloc(&f, bytes), "cudaMalloc");
    void* args[] = {&f, &gx, &N, &u0, &kf};
    int rc = launch(k_init, nb, MB3, args);
    if (!rc) {
        cudaError_t e = cudaDeviceSynchronize();
        if (e == cudaSuccess) e = cudaMemcpy(host_f, f, bytes, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) rc = seterr("ref_uniform_init", e);
    }
    cudaFree(f);
    return rc;
}

// nsteps reference k_step launches on host_f in place (ping-pong as src/tgv3d_uniform.cu:194).
int ref_uniform_run(float* host_f, int N, float omega, long nsteps) {
    if (!g_uni) { g_err = "uniform cubin not loaded"; return 1; }
    if (N % MB) { g_err = "N%MB"; return 2; }
    int gx = N / MB, nb = gx * gx * gx;
    size_t bytes = (size_t)nb * Q * MB3 * 4;
    float *fa = nullptr, *fb = nullptr;
    RK(cudaMalloc(&fa, bytes), "cudaMalloc");
    cudaError_t e = cudaMalloc(&fb, bytes);
    if (e != cudaSuccess) { cudaFree(fa); return seterr("cudaMalloc", e); }
    int rc = 0;
    e = cudaMemcpy(fa, host_f, bytes, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) rc = seterr("H2D", e);
    for (long s = 0; s < nsteps && !rc; ++s) {
        void* args[] = {&fa, &fb, &gx, &N, &omega};
        rc = launch(k_step, nb, MB3, args);
        std::swap(fa, fb);
    }
    if (!rc) {
        e = cudaDeviceSynchronize();
        if (e == cudaSuccess) e = cudaMemcpy(host_f, fa, bytes, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) rc = seterr("ref_uniform_run", e);
    }
    cudaFree(fa);
    cudaFree(fb);
    return rc;
}

// reference k_macro of host_f into host_field (4*N^3 floats).
int ref_uniform_macro(const float* host_f, int N, float* host_field) {
    if (!g_uni) { g_err = "uniform cubin not loaded"; return 1; }
    int gx = N / MB, nb = gx * gx * gx;
    size_t bytes = (size_t)nb * Q * MB3 * 4, fbytes = (size_t)N * N * N * 16;
    float *f = nullptr, *F = nullptr;
    RK(cudaMalloc(&f, bytes), "cudaMalloc");
    cudaError_t e = cudaMalloc(&F, fbytes);
    if (e != cudaSuccess) { cudaFree(f); return seterr("cudaMalloc", e); }
    int rc = 0;
    e = cudaMemcpy(f, host_f, bytes, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) rc = seterr("H2D", e);
    if (!rc) {
        void* args[] = {&f, &gx, &N, &F};
        rc = launch(k_macro, nb, MB3, args);
    }
    if (!rc) {
        e = cudaDeviceSynchronize();
        if (e == cudaSuccess) e = cudaMemcpy(host_field, F, fbytes, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) rc = seterr("ref_uniform_macro", e);
    }
    cudaFree(f);
    cudaFree(F);
    return rc;
}

// Time `nsteps` reference k_step launches on the TGV state of an N^3 cube (device-resident),
// returning milliseconds from CUDA events: the reference kernel rerun on this GPU.
int ref_uniform_time(int N, double u0, float omega, long warmup, long nsteps, float* ms) {
    if (!g_uni) { g_err = "uniform cubin not loaded"; return 1; }
    int gx = N / MB, nb = gx * gx * gx;
    double kf = 2.0 * M_PI / double(N);
    size_t bytes = (size_t)nb * Q * MB3 * 4;
    float *fa = nullptr, *fb = nullptr;
    RK(cudaMalloc(&fa, bytes), "cudaMalloc");
    cudaError_t e = cudaMalloc(&fb, bytes);
    if (e != cudaSuccess) { cudaFree(fa); return seterr("cudaMalloc", e); }
    int rc = 0;
    {
        void* args[] = {&fa, &gx, &N, &u0, &kf};
        rc = launch(k_init, nb, MB3, args);
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    for (long s = 0; s < warmup + nsteps && !rc; ++s) {
        if (s == warmup) cudaEventRecord(e0, 0);
        void* args[] = {&fa, &fb, &gx, &N, &omega};
        rc = launch(k_step, nb, MB3, args);
        std::swap(fa, fb);
    }
    if (!rc) {
        cudaEventRecord(e1, 0);
        e = cudaEventSynchronize(e1);
        if (e == cudaSuccess) e = cudaEventElapsedTime(ms, e0, e1);
        if (e != cudaSuccess) rc = seterr("ref_uniform_time", e);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(fa);
    cudaFree(fb);
    return rc;
}

}  // extern "C"
