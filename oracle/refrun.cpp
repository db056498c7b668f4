// ORACLE - test infrastructure only.  Runs the reference's own CUDA kernels (compiled from the
// reference checkout into oracle/_ref/*.cubin by oracle/build.py) on host buffers, so tests can pin
// the CPU oracle and the engine against the reference itself.  Host orchestration mirrors the
// reference's main(): src/tgv3d_uniform.cu:157-194 and src/tgv3d_amr.cu:669-837, where the Thrust
// calls (sort, exclusive_scan, copy_if) run on the host instead; their results are uniquely defined
// (order statistic, prefix sum, ordered compaction).  Built on the GPU host with g++ against the
// CUDA runtime; the cubins are loaded with cudaLibraryLoadFromFile.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
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

// =================================================================================================
// AMR: the reference's kernels in the reference's launch order (MB = 8, ghosts (MB+2)^3 per block)
// =================================================================================================
namespace {

cudaLibrary_t g_amr = nullptr;
struct AmrK {
    cudaKernel_t init, step0, prep_list, fill1p, fill2p, step1, step2, restr1, restr2, seed1, seed2, mig1, mig2, sensor,
        mark_thr, mark_ref1, deepmask, scat1, scat2, setall, slab, ref1all, dil0, dil1, composite, diag, qspeed;
} K;
const int EB = 10, EB3 = 1000, HALF = 4;

struct RefAmr {
    int N, cgx, cnb0, l1gx, N1, N2, NG1;
    double frac1, frac2, u0, kf;
    int l1mode, l2mode, develop;
    double tau0, tau1, tau2, nqs01, nqi10, nqs12, nqi21;
    float om0, om1, om2;
    int cap_nref0, cap1, cap_nref1 = INT_MAX, cap2 = 0;
    long hw_nf1 = 0, hw_nf2 = 0;
    double budget;
    size_t PB;
    float *c0a, *c0b, *f1a, *f1b, *gh1, *prep0, *prep1, *f2a = nullptr, *f2b = nullptr, *gh2 = nullptr;
    float *sen0, *sen1, *thr;
    int *ref0, *fof0, *l1pcb, *l1oct, *rl0, *f1pos, *l1grid, *ref1, *fof1, *l2pl1 = nullptr, *l2oct = nullptr, *rl1;
    int *o_ref0, *o_fof0, *o_l1grid, *o_ref1, *o_fof1, *skin0, *skin1, *rank, *deep;
    int nref0 = 0, nf1 = 0, nref1 = 0, nf2 = 0, n_skin0 = 0, n_skin1 = 0, ndeep = 0;
    bool ov = false;
    std::vector<float> ov0, ov1;
    std::vector<void*> allocs;
    int err = 0;
};

template <class T>
int amalloc(RefAmr* a, T** p, size_t n) {
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void**)p, n * sizeof(T));
    if (e != cudaSuccess) return seterr("cudaMalloc", e);
    a->allocs.push_back(*p);
    return 0;
}
#define AK(x)                \
    do {                     \
        int r_ = (x);        \
        if (r_) return r_;   \
    } while (0)

unsigned g256(long n) { return (unsigned)((n + 255) / 256); }

int L(cudaKernel_t k, unsigned grid, unsigned block, std::initializer_list<void*> args) {
    if (grid == 0) return 0;
    std::vector<void*> v(args);
    return launch(k, grid, block, v.data());
}

// exclusive scan of n ints on the device, on the host (thrust::exclusive_scan); returns total
int host_scan(const int* dflags, int n, int* drank, int* total) {
    std::vector<int> f(n), r(n);
    RK(cudaMemcpy(f.data(), dflags, sizeof(int) * n, cudaMemcpyDeviceToHost), "scan D2H");
    int acc = 0;
    for (int i = 0; i < n; ++i) {
        r[i] = acc;
        acc += f[i];
    }
    RK(cudaMemcpy(drank, r.data(), sizeof(int) * n, cudaMemcpyHostToDevice), "scan H2D");
    *total = acc;
    return 0;
}
// threshold value sorted[n - tgt] of the masked sensors (copy_if + thrust::sort), written to d_thr
int host_threshold(const float* dsen, const int* dmask, int n, int tgt_cap, double frac, bool cap_it, float* dthr,
                   int* ncount) {
    std::vector<float> s(n);
    std::vector<int> m(n, 1);
    RK(cudaMemcpy(s.data(), dsen, sizeof(float) * n, cudaMemcpyDeviceToHost), "sensor D2H");
    if (dmask) RK(cudaMemcpy(m.data(), dmask, sizeof(int) * n, cudaMemcpyDeviceToHost), "mask D2H");
    std::vector<float> v;
    for (int i = 0; i < n; ++i)
        if (m[i]) v.push_back(s[i]);
    *ncount = (int)v.size();
    if (v.empty()) return 0;
    int nn = (int)v.size();
    int tgt = std::max(1, (int)(frac * nn));
    if (cap_it) tgt = std::min(tgt_cap, tgt);
    std::sort(v.begin(), v.end());
    float t = v[nn - tgt];
    RK(cudaMemcpy(dthr, &t, 4, cudaMemcpyHostToDevice), "thr H2D");
    return 0;
}
// ordered compaction of the indices with flag != 0 (copy_if over a counting iterator)
int host_compact(const int* dflags, int n, int* dout, int* count) {
    std::vector<int> f(n), o;
    RK(cudaMemcpy(f.data(), dflags, sizeof(int) * n, cudaMemcpyDeviceToHost), "flags D2H");
    for (int i = 0; i < n; ++i)
        if (f[i]) o.push_back(i);
    *count = (int)o.size();
    if (!o.empty()) RK(cudaMemcpy(dout, o.data(), sizeof(int) * o.size(), cudaMemcpyHostToDevice), "compact H2D");
    return 0;
}

int sensor0(RefAmr* a) {
    AK(L(K.sensor, a->cnb0, MB3, {&a->c0a, &a->cnb0, &a->sen0}));
    if (a->ov) RK(cudaMemcpy(a->sen0, a->ov0.data(), sizeof(float) * a->cnb0, cudaMemcpyHostToDevice), "ov");
    return 0;
}
int sensor1(RefAmr* a) {
    AK(L(K.sensor, a->nf1, MB3, {&a->f1a, &a->nf1, &a->sen1}));
    if (a->ov) {
        std::vector<int> pos(a->nf1);
        std::vector<float> v(a->nf1);
        RK(cudaMemcpy(pos.data(), a->f1pos, sizeof(int) * a->nf1, cudaMemcpyDeviceToHost), "f1pos");
        for (int b = 0; b < a->nf1; ++b) v[b] = a->ov1[pos[b]];
        RK(cudaMemcpy(a->sen1, v.data(), sizeof(float) * a->nf1, cudaMemcpyHostToDevice), "ov");
    }
    return 0;
}
int skins(RefAmr* a) {
    AK(L(K.dil0, g256(a->cnb0), 256, {&a->ref0, &a->cnb0, &a->cgx, &a->rank}));
    AK(host_compact(a->rank, a->cnb0, a->skin0, &a->n_skin0));
    if (a->nf1) {
        AK(L(K.dil1, g256(a->nf1), 256, {&a->ref1, &a->f1pos, &a->l1grid, &a->nf1, &a->l1gx, &a->rank}));
        AK(host_compact(a->rank, a->nf1, a->skin1, &a->n_skin1));
    } else {
        a->n_skin1 = 0;
    }
    return 0;
}
bool pool_fits(RefAmr* a, long c1, long c2) { return (double)((size_t)(c1 + c2) * a->PB * 6 / 5) < a->budget; }

// gpurce_init (src/tgv3d_amr.cu:776-815)
int initial_build(RefAmr* a) {
    if (a->l1mode == 0) AK(L(K.setall, g256(a->cnb0), 256, {&a->ref0, &a->cnb0}));
    else if (a->l1mode == 1) AK(L(K.slab, g256(a->cnb0), 256, {&a->ref0, &a->cnb0, &a->cgx}));
    else {
        for (int s = 0; s < a->develop; ++s) {
            AK(L(K.step0, a->cnb0, MB3, {&a->c0a, &a->c0b, &a->cgx, &a->N, &a->om0}));
            std::swap(a->c0a, a->c0b);
        }
        AK(sensor0(a));
        int nn;
        AK(host_threshold(a->sen0, nullptr, a->cnb0, a->cap_nref0, a->frac1, true, a->thr, &nn));
        AK(L(K.mark_thr, g256(a->cnb0), 256, {&a->sen0, &a->thr, &a->ref0, &a->cnb0}));
    }
    int tot;
    AK(host_scan(a->ref0, a->cnb0, a->rank, &tot));
    a->nref0 = tot;
    a->nf1 = 8 * tot;
    a->hw_nf1 = std::max(a->hw_nf1, (long)a->nf1);
    if (a->nf1 > a->cap1) { a->err = 3; g_err = "L1 pool overflow"; return 3; }
    RK(cudaMemset(a->l1grid, 0xFF, sizeof(int) * a->NG1), "memset");
    RK(cudaMemset(a->fof0, 0xFF, sizeof(int) * a->cnb0), "memset");
    if (a->nref0)
        AK(L(K.scat1, g256(a->cnb0), 256, {&a->ref0, &a->rank, &a->cnb0, &a->cgx, &a->l1gx, &a->fof0, &a->rl0, &a->l1pcb,
                                           &a->l1oct, &a->l1grid, &a->f1pos}));
    if (a->nf1) {
        RK(cudaMemset(a->gh1, 0, sizeof(float) * (size_t)a->nf1 * Q * EB3), "memset");
        float nqs = float(a->nqs01);
        AK(L(K.seed1, a->nf1, MB3, {&a->c0a, &a->f1a, &a->l1pcb, &a->l1oct, &a->cgx, &a->N, &nqs}));
    }
    a->nref1 = a->nf2 = 0;
    if (a->nf1) {
        AK(sensor1(a));
        AK(L(K.deepmask, g256(a->nf1), 256, {&a->f1pos, &a->l1grid, &a->l1gx, &a->nf1, &a->deep}));
        RK(cudaMemset(a->ref1, 0, sizeof(int) * a->cap1), "memset");
        if (a->l2mode == 0) AK(L(K.ref1all, g256(a->nf1), 256, {&a->deep, &a->nf1, &a->ref1}));
        else {
            int nd;
            AK(host_threshold(a->sen1, a->deep, a->nf1, 0, a->frac2, false, a->thr, &nd));
            a->ndeep = nd;
            if (nd > 0)
                AK(L(K.mark_ref1, g256(a->nf1), 256, {&a->sen1, &a->thr, &a->f1pos, &a->l1grid, &a->l1gx, &a->nf1, &a->ref1}));
        }
        AK(host_scan(a->ref1, a->nf1, a->rank, &tot));
        a->nref1 = tot;
        a->nf2 = 8 * tot;
        a->hw_nf2 = std::max(a->hw_nf2, (long)a->nf2);
        a->cap_nref1 = std::max(1, (int)std::ceil(a->nref1 * 2.5));
        if (a->l2mode == 0) a->cap_nref1 = std::max(a->cap_nref1, a->nf1);
        a->cap_nref1 = std::min(a->cap_nref1, a->cap1);
        while (a->cap_nref1 > 1 && !pool_fits(a, a->cap1, 8L * a->cap_nref1)) a->cap_nref1--;
        a->cap2 = 8 * a->cap_nref1;
    } else {
        a->cap_nref1 = 1;
        a->cap2 = 8;
    }
    AK(amalloc(a, &a->f2a, (size_t)a->cap2 * Q * MB3));
    AK(amalloc(a, &a->f2b, (size_t)a->cap2 * Q * MB3));
    AK(amalloc(a, &a->gh2, (size_t)a->cap2 * Q * EB3));
    AK(amalloc(a, &a->l2pl1, (size_t)a->cap2));
    AK(amalloc(a, &a->l2oct, (size_t)a->cap2));
    RK(cudaMemset(a->fof1, 0xFF, sizeof(int) * a->cap1), "memset");
    if (a->nf2) {
        AK(L(K.scat2, g256(a->nf1), 256, {&a->ref1, &a->rank, &a->nf1, &a->fof1, &a->rl1, &a->l2pl1, &a->l2oct}));
        RK(cudaMemset(a->gh2, 0, sizeof(float) * (size_t)a->nf2 * Q * EB3), "memset");
        float nqs = float(a->nqs12);
        AK(L(K.seed2, a->nf2, MB3, {&a->f1a, &a->f2a, &a->l2pl1, &a->l2oct, &a->f1pos, &a->l1grid, &a->l1gx, &a->N1, &nqs}));
    }
    AK(skins(a));
    RK(cudaDeviceSynchronize(), "initial build");
    return 0;
}

// gpurce_regrid (src/tgv3d_amr.cu:722-764)
int regrid(RefAmr* a) {
    RK(cudaMemcpy(a->o_ref0, a->ref0, sizeof(int) * a->cnb0, cudaMemcpyDeviceToDevice), "snap");
    RK(cudaMemcpy(a->o_fof0, a->fof0, sizeof(int) * a->cnb0, cudaMemcpyDeviceToDevice), "snap");
    RK(cudaMemcpy(a->o_l1grid, a->l1grid, sizeof(int) * a->NG1, cudaMemcpyDeviceToDevice), "snap");
    RK(cudaMemcpy(a->o_ref1, a->ref1, sizeof(int) * a->cap1, cudaMemcpyDeviceToDevice), "snap");
    RK(cudaMemcpy(a->o_fof1, a->fof1, sizeof(int) * a->cap1, cudaMemcpyDeviceToDevice), "snap");
    AK(sensor0(a));
    int nn, tot;
    AK(host_threshold(a->sen0, nullptr, a->cnb0, a->cap_nref0, a->frac1, true, a->thr, &nn));
    AK(L(K.mark_thr, g256(a->cnb0), 256, {&a->sen0, &a->thr, &a->ref0, &a->cnb0}));
    AK(host_scan(a->ref0, a->cnb0, a->rank, &tot));
    a->nref0 = tot;
    a->nf1 = 8 * tot;
    a->hw_nf1 = std::max(a->hw_nf1, (long)a->nf1);
    if (a->nf1 > a->cap1) { a->err = 3; g_err = "L1 pool overflow"; return 3; }
    RK(cudaMemset(a->l1grid, 0xFF, sizeof(int) * a->NG1), "memset");
    RK(cudaMemset(a->fof0, 0xFF, sizeof(int) * a->cnb0), "memset");
    if (a->nref0)
        AK(L(K.scat1, g256(a->cnb0), 256, {&a->ref0, &a->rank, &a->cnb0, &a->cgx, &a->l1gx, &a->fof0, &a->rl0, &a->l1pcb,
                                           &a->l1oct, &a->l1grid, &a->f1pos}));
    if (a->nf1) {
        float nqs = float(a->nqs01);
        AK(L(K.mig1, a->nf1, MB3, {&a->f1a, &a->f1b, &a->c0a, &a->l1pcb, &a->l1oct, &a->o_ref0, &a->o_fof0, &a->cgx, &a->N, &nqs}));
        std::swap(a->f1a, a->f1b);
    }
    a->nref1 = a->nf2 = 0;
    if (a->nf1) {
        AK(sensor1(a));
        AK(L(K.deepmask, g256(a->nf1), 256, {&a->f1pos, &a->l1grid, &a->l1gx, &a->nf1, &a->deep}));
        int nd;
        RK(cudaMemset(a->ref1, 0, sizeof(int) * a->cap1), "memset");
        AK(host_threshold(a->sen1, a->deep, a->nf1, a->cap_nref1, a->frac2, true, a->thr, &nd));
        a->ndeep = nd;
        if (nd > 0)
            AK(L(K.mark_ref1, g256(a->nf1), 256, {&a->sen1, &a->thr, &a->f1pos, &a->l1grid, &a->l1gx, &a->nf1, &a->ref1}));
        AK(host_scan(a->ref1, a->nf1, a->rank, &tot));
        a->nref1 = tot;
        a->nf2 = 8 * tot;
        a->hw_nf2 = std::max(a->hw_nf2, (long)a->nf2);
        if (a->nf2 > a->cap2) { a->err = 3; g_err = "L2 pool overflow"; return 3; }
        RK(cudaMemset(a->fof1, 0xFF, sizeof(int) * a->cap1), "memset");
        if (a->nref1) AK(L(K.scat2, g256(a->nf1), 256, {&a->ref1, &a->rank, &a->nf1, &a->fof1, &a->rl1, &a->l2pl1, &a->l2oct}));
        if (a->nf2) {
            float nqs = float(a->nqs12);
            AK(L(K.mig2, a->nf2, MB3, {&a->f2a, &a->f2b, &a->f1a, &a->l2pl1, &a->l2oct, &a->f1pos, &a->o_l1grid, &a->o_ref1,
                                       &a->o_fof1, &a->l1grid, &a->l1gx, &a->N1, &nqs}));
            std::swap(a->f2a, a->f2b);
        }
    }
    AK(skins(a));
    RK(cudaDeviceSynchronize(), "regrid");
    return 0;
}

// base_step (src/tgv3d_amr.cu:821-837)
int base_step(RefAmr* a) {
    AK(L(K.step0, a->cnb0, MB3, {&a->c0a, &a->c0b, &a->cgx, &a->N, &a->om0}));
    std::swap(a->c0a, a->c0b);
    if (!a->nf1) return 0;
    float nqs01 = float(a->nqs01), nqs12 = float(a->nqs12), nqi21 = float(a->nqi21), nqi10 = float(a->nqi10);
    AK(L(K.prep_list, a->n_skin0, MB3, {&a->c0a, &a->prep0, &a->skin0, &a->n_skin0, &nqs01}));
    AK(L(K.fill1p, a->nf1, MB3, {&a->prep0, &a->gh1, &a->l1pcb, &a->l1oct, &a->ref0, &a->cgx, &a->N}));
    for (int s1 = 0; s1 < 2; ++s1) {
        if (a->nf2) {
            AK(L(K.prep_list, a->n_skin1, MB3, {&a->f1a, &a->prep1, &a->skin1, &a->n_skin1, &nqs12}));
            AK(L(K.fill2p, a->nf2, MB3, {&a->prep1, &a->gh2, &a->l2pl1, &a->l2oct, &a->f1pos, &a->l1grid, &a->ref1, &a->l1gx, &a->N1}));
            for (int s2 = 0; s2 < 2; ++s2) {
                AK(L(K.step2, a->nf2, MB3, {&a->f2a, &a->f2b, &a->gh2, &a->l2pl1, &a->l2oct, &a->f1pos, &a->l1grid, &a->ref1,
                                            &a->fof1, &a->l1gx, &a->N1, &a->om2}));
                std::swap(a->f2a, a->f2b);
            }
            AK(L(K.restr2, (unsigned)(((long)a->nref1 * MB3 + 127) / 128), 128, {&a->f1a, &a->f2a, &a->rl1, &a->fof1, &a->nref1, &nqi21}));
        }
        AK(L(K.step1, a->nf1, MB3, {&a->f1a, &a->f1b, &a->gh1, &a->l1pcb, &a->l1oct, &a->ref0, &a->fof0, &a->cgx, &a->N, &a->om1}));
        std::swap(a->f1a, a->f1b);
    }
    AK(L(K.restr1, (unsigned)(((long)a->nref0 * MB3 + 127) / 128), 128, {&a->c0a, &a->f1a, &a->rl0, &a->fof0, &a->nref0, &a->cgx, &nqi10}));
    return 0;
}

}  // namespace

extern "C" {

int refrun_load_amr(const char* path) {
    if (g_amr) return 0;
    RK(cudaLibraryLoadFromFile(&g_amr, path, nullptr, nullptr, 0, nullptr, nullptr, 0), "cudaLibraryLoadFromFile");
    struct { cudaKernel_t* k; const char* n; } tab[] = {
        {&K.init, "_Z12k_init_tgv3dPfiidd"}, {&K.step0, "_Z9k_step_L0PKfPfiif"},
        {&K.prep_list, "_Z11k_prep_listPKfPfPKiif"}, {&K.fill1p, "_Z12k_fillcf_L1pPKfPfPKiS3_S3_ii"},
        {&K.fill2p, "_Z12k_fillcf_L2pPKfPfPKiS3_S3_S3_S3_ii"}, {&K.step1, "_Z9k_step_L1PKfPfS0_PKiS3_S3_S3_iif"},
        {&K.step2, "_Z9k_step_L2PKfPfS0_PKiS3_S3_S3_S3_S3_iif"}, {&K.restr1, "_Z13k_restrict_L1PfPKfPKiS3_iif"},
        {&K.restr2, "_Z13k_restrict_L2PfPKfPKiS3_if"}, {&K.seed1, "_Z9k_seed_L1PKfPfPKiS3_iif"},
        {&K.seed2, "_Z9k_seed_L2PKfPfPKiS3_S3_S3_iif"}, {&K.mig1, "_Z12k_migrate_L1PKfPfS0_PKiS3_S3_S3_iif"},
        {&K.mig2, "_Z12k_migrate_L2PKfPfS0_PKiS3_S3_S3_S3_S3_S3_iif"}, {&K.sensor, "_Z8k_sensorPKfiPf"},
        {&K.mark_thr, "_Z10k_mark_thrPKfS0_Pii"}, {&K.mark_ref1, "_Z11k_mark_ref1PKfS0_PKiS2_iiPi"},
        {&K.deepmask, "_Z10k_deepmaskPKiS0_iiPi"}, {&K.scat1, "_Z12k_scatter_L1PKiS0_iiiPiS1_S1_S1_S1_S1_"},
        {&K.scat2, "_Z12k_scatter_L2PKiS0_iPiS1_S1_S1_"}, {&K.setall, "_Z8k_setallPii"},
        {&K.slab, "_Z11k_mark_slabPiii"}, {&K.ref1all, "_Z15k_mark_ref1_allPKiiPi"},
        {&K.dil0, "_Z11k_dilate_L0PKiiiPi"}, {&K.dil1, "_Z11k_dilate_L1PKiS0_S0_iiPi"},
        {&K.composite, "_Z11k_compositePKfS0_S0_PKiS2_S2_iiiPf"}, {&K.diag, "_Z13k_diag_reducePKfiPd"},
        {&K.qspeed, "_Z8k_qspeedPKfiPfS1_S1_i"},
    };
    for (auto& t : tab) RK(cudaLibraryGetKernel(t.k, g_amr, t.n), t.n);
    return 0;
}

void* ref_amr_create(int N, double re, double u0, double tstar, int l1mode, int l2mode, double frac1, double frac2,
                     int develop, double budget_bytes) {
    if (!g_amr || N % MB) { g_err = "amr cubin not loaded or N%MB"; return nullptr; }
    RefAmr* a = new RefAmr();
    a->N = N; a->cgx = N / MB; a->cnb0 = a->cgx * a->cgx * a->cgx; a->l1gx = 2 * a->cgx; a->N1 = 2 * N; a->N2 = 4 * N;
    a->NG1 = a->l1gx * a->l1gx * a->l1gx;
    a->frac1 = frac1; a->frac2 = frac2; a->u0 = u0; a->l1mode = l1mode; a->l2mode = l2mode; a->develop = develop;
    double nu = u0 * double(N) / (2.0 * M_PI * re);
    a->tau0 = 3.0 * nu + 0.5; a->tau1 = 2.0 * a->tau0 - 0.5; a->tau2 = 2.0 * a->tau1 - 0.5;
    a->om0 = float(1.0 / a->tau0); a->om1 = float(1.0 / a->tau1); a->om2 = float(1.0 / a->tau2);
    a->nqs01 = (a->tau1 - 1.0) / (2.0 * (a->tau0 - 1.0)); a->nqi10 = (2.0 * (a->tau0 - 1.0)) / (a->tau1 - 1.0);
    a->nqs12 = (a->tau2 - 1.0) / (2.0 * (a->tau1 - 1.0)); a->nqi21 = (2.0 * (a->tau1 - 1.0)) / (a->tau2 - 1.0);
    a->kf = 2.0 * M_PI / double(N);
    (void)tstar;
    a->budget = budget_bytes;
    a->PB = size_t(Q) * 4 * (2 * MB3 + EB3);
    a->cap_nref0 = (l1mode == 0) ? a->cnb0 : std::min(a->cnb0, std::max(1, (int)std::ceil(frac1 * a->cnb0 * 1.4)));
    while (a->cap_nref0 > 1 && !pool_fits(a, 8L * a->cap_nref0, 0)) a->cap_nref0--;
    a->cap1 = 8 * a->cap_nref0;
    size_t c0 = (size_t)a->cnb0 * Q * MB3, c1 = (size_t)a->cap1 * Q * MB3;
    int rc = 0;
    rc |= amalloc(a, &a->c0a, c0); rc |= amalloc(a, &a->c0b, c0); rc |= amalloc(a, &a->prep0, c0);
    rc |= amalloc(a, &a->f1a, c1); rc |= amalloc(a, &a->f1b, c1); rc |= amalloc(a, &a->prep1, c1);
    rc |= amalloc(a, &a->gh1, (size_t)a->cap1 * Q * EB3);
    rc |= amalloc(a, &a->sen0, a->cnb0); rc |= amalloc(a, &a->sen1, a->cap1); rc |= amalloc(a, &a->thr, 1);
    int** cnb[] = {&a->ref0, &a->fof0, &a->o_ref0, &a->o_fof0, &a->skin0};
    for (int** t : cnb) rc |= amalloc(a, t, a->cnb0);
    int** cap[] = {&a->l1pcb, &a->l1oct, &a->rl0, &a->f1pos, &a->ref1, &a->fof1, &a->o_ref1, &a->o_fof1, &a->rl1, &a->skin1, &a->deep};
    for (int** t : cap) rc |= amalloc(a, t, a->cap1);
    rc |= amalloc(a, &a->l1grid, a->NG1); rc |= amalloc(a, &a->o_l1grid, a->NG1);
    rc |= amalloc(a, &a->rank, std::max(a->cnb0, a->cap1));
    if (rc) { delete a; return nullptr; }
    cudaMemset(a->fof1, 0xFF, sizeof(int) * a->cap1);
    cudaMemset(a->ref1, 0, sizeof(int) * a->cap1);
    cudaMemset(a->l1grid, 0xFF, sizeof(int) * a->NG1);
    cudaMemset(a->ref0, 0, sizeof(int) * a->cnb0);
    int gx = a->cgx;
    if (L(K.init, a->cnb0, MB3, {&a->c0a, &gx, &a->N, &a->u0, &a->kf})) { delete a; return nullptr; }
    cudaDeviceSynchronize();
    return a;
}
void ref_amr_destroy(void* h) {
    RefAmr* a = static_cast<RefAmr*>(h);
    for (void* p : a->allocs) cudaFree(p);
    delete a;
}
void ref_amr_set_sensor_override(void* h, const float* sen0, const float* sen1pos) {
    RefAmr* a = static_cast<RefAmr*>(h);
    if (!sen0 || !sen1pos) { a->ov = false; return; }
    a->ov = true;
    a->ov0.assign(sen0, sen0 + a->cnb0);
    a->ov1.assign(sen1pos, sen1pos + a->NG1);
}
int ref_amr_initial_build(void* h) { return initial_build(static_cast<RefAmr*>(h)); }
int ref_amr_regrid(void* h) { return regrid(static_cast<RefAmr*>(h)); }
int ref_amr_step(void* h, long n) {
    RefAmr* a = static_cast<RefAmr*>(h);
    for (long i = 0; i < n; ++i) AK(base_step(a));
    RK(cudaDeviceSynchronize(), "ref_amr_step");
    return 0;
}
// reference k_composite + k_diag_reduce (double atomics) at 4N0
int ref_amr_diag(void* h, double* out) {
    RefAmr* a = static_cast<RefAmr*>(h);
    long NN = (long)a->N2 * a->N2 * a->N2;
    float* F = nullptr;
    double* acc = nullptr;
    RK(cudaMalloc(&F, sizeof(float) * 4 * NN), "cudaMalloc");
    RK(cudaMalloc(&acc, 3 * sizeof(double)), "cudaMalloc");
    RK(cudaMemset(acc, 0, 3 * sizeof(double)), "memset");
    unsigned g = (unsigned)((NN + 255) / 256);
    int rc = L(K.composite, g, 256, {&a->c0a, &a->f1a, &a->f2a, &a->ref1, &a->fof1, &a->l1grid, &a->cgx, &a->l1gx, &a->N2, &F});
    if (!rc) rc = L(K.diag, g, 256, {&F, &a->N2, &acc});
    double h3[3] = {0, 0, 0};
    if (!rc) {
        cudaError_t e = cudaMemcpy(h3, acc, sizeof h3, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) rc = seterr("diag", e);
    }
    cudaFree(F);
    cudaFree(acc);
    double inv = 1.0 / double(NN);
    for (int i = 0; i < 3; ++i) out[i] = h3[i] * inv;
    return rc;
}
// reference k_composite + k_qspeed (src/tgv3d_amr.cu:523-536,553-564): Q-criterion and speed at 4N0
int ref_amr_qspeed(void* h, float* q_out, float* speed_out) {
    RefAmr* a = static_cast<RefAmr*>(h);
    long NN = (long)a->N2 * a->N2 * a->N2;
    float *F = nullptr, *Qd = nullptr, *Sd = nullptr, *nov = nullptr;
    int zero = 0;
    RK(cudaMalloc(&F, sizeof(float) * 4 * NN), "cudaMalloc");
    cudaError_t e = cudaMalloc(&Qd, sizeof(float) * NN);
    if (e == cudaSuccess) e = cudaMalloc(&Sd, sizeof(float) * NN);
    int rc = e == cudaSuccess ? 0 : seterr("cudaMalloc", e);
    unsigned g = (unsigned)((NN + 255) / 256);
    if (!rc)
        rc = L(K.composite, g, 256, {&a->c0a, &a->f1a, &a->f2a, &a->ref1, &a->fof1, &a->l1grid, &a->cgx, &a->l1gx, &a->N2, &F});
    if (!rc) rc = L(K.qspeed, g, 256, {&F, &a->N2, &Qd, &Sd, &nov, &zero});
    if (!rc) {
        e = cudaMemcpy(q_out, Qd, sizeof(float) * NN, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(speed_out, Sd, sizeof(float) * NN, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) rc = seterr("qspeed", e);
    }
    cudaFree(F);
    cudaFree(Qd);
    cudaFree(Sd);
    return rc;
}
void ref_amr_counts(void* h, long* out) {
    RefAmr* a = static_cast<RefAmr*>(h);
    long v[16] = {a->nref0, a->nf1, a->nref1, a->nf2, a->n_skin0, a->n_skin1, a->cap1, a->cap2, a->cnb0, a->NG1,
                  a->hw_nf1, a->hw_nf2, a->ndeep, a->cap_nref0, a->cap_nref1, 0};
    memcpy(out, v, sizeof v);
}
int ref_amr_get_table(void* h, int id, int* out, long cap) {
    RefAmr* a = static_cast<RefAmr*>(h);
    const int* p = nullptr;
    long n = 0;
    switch (id) {
        case 0: p = a->ref0; n = a->cnb0; break;
        case 1: p = a->fof0; n = a->cnb0; break;
        case 2: p = a->rl0; n = a->nref0; break;
        case 3: p = a->l1pcb; n = a->nf1; break;
        case 4: p = a->l1oct; n = a->nf1; break;
        case 5: p = a->f1pos; n = a->nf1; break;
        case 6: p = a->l1grid; n = a->NG1; break;
        case 7: p = a->ref1; n = a->nf1; break;
        case 8: p = a->fof1; n = a->nf1; break;
        case 9: p = a->rl1; n = a->nref1; break;
        case 10: p = a->l2pl1; n = a->nf2; break;
        case 11: p = a->l2oct; n = a->nf2; break;
        case 12: p = a->skin0; n = a->n_skin0; break;
        case 13: p = a->skin1; n = a->n_skin1; break;
        case 14: p = a->deep; n = a->nf1; break;
        default: return -1;
    }
    if (n > cap) return -2;
    if (n && cudaMemcpy(out, p, sizeof(int) * n, cudaMemcpyDeviceToHost) != cudaSuccess) return -3;
    return (int)n;
}
long ref_amr_get_pops(void* h, int level, float* out, long cap) {
    RefAmr* a = static_cast<RefAmr*>(h);
    const float* p = level == 0 ? a->c0a : (level == 1 ? a->f1a : a->f2a);
    long nb = level == 0 ? a->cnb0 : (level == 1 ? a->nf1 : a->nf2);
    long n = nb * Q * MB3;
    if (n > cap) return -2;
    if (n && cudaMemcpy(out, p, sizeof(float) * n, cudaMemcpyDeviceToHost) != cudaSuccess) return -3;
    return n;
}
long ref_amr_set_pops(void* h, int level, const float* in, long count) {
    RefAmr* a = static_cast<RefAmr*>(h);
    float* p = level == 0 ? a->c0a : (level == 1 ? a->f1a : a->f2a);
    long nb = level == 0 ? a->cnb0 : (level == 1 ? a->nf1 : a->nf2);
    long n = nb * Q * MB3;
    if (count != n) return -2;
    if (n && cudaMemcpy(p, in, sizeof(float) * n, cudaMemcpyHostToDevice) != cudaSuccess) return -3;
    return n;
}
int ref_amr_get_sensor(void* h, int level, float* out, long cap) {
    RefAmr* a = static_cast<RefAmr*>(h);
    long n = level == 0 ? a->cnb0 : a->nf1;
    if (n > cap) return -2;
    if (n && cudaMemcpy(out, level == 0 ? a->sen0 : a->sen1, sizeof(float) * n, cudaMemcpyDeviceToHost) != cudaSuccess) return -3;
    return (int)n;
}
// device time of n reference base_steps (no regrid), after `warmup` untimed ones
int ref_amr_time(void* h, long warmup, long n, float* ms) {
    RefAmr* a = static_cast<RefAmr*>(h);
    for (long i = 0; i < warmup; ++i) AK(base_step(a));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, 0);
    for (long i = 0; i < n; ++i) AK(base_step(a));
    cudaEventRecord(e1, 0);
    cudaError_t e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess) return seterr("ref_amr_time", e);
    return 0;
}

}  // extern "C"
