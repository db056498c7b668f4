// Internal launch interface between the C ABI (capi.cu) and the kernel translation units.
// Nothing here is exported from the shared library.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

namespace jp {

// ---- uniform periodic cube, flat SoA layout [q][z][y][x] ----------------------------------------

// One periodic cube of a batched stream-collide launch.
struct UniSolve {
    const void* src;         // populations at t   (19 * n^3 elements)
    void* dst;               // populations at t+1
    int n;                   // edge
    int nxs;                 // n / V: x segments per row
    float omega;             // 1/tau (FP32 and shifted storages)
    int pad;
    double omega_d;          // 1/tau (FP64 storage)
    long long blk_begin;     // first CUDA block of this cube in the launch
    long long nseg;          // n^3 / V threads
};
constexpr int kMaxBatch = 48;
struct UniBatch {
    int count;
    int pad;
    UniSolve s[kMaxBatch];
};

// Launch one stream-collide over `count` cubes of the same storage format (storage id of jp_storage).
// vec: cells per thread along x (0 = default), tpb: threads per block (0 = default).
// Returns the CUDA error of the launch.
cudaError_t launch_stream_collide(int storage, const UniSolve* solves, int count, int vec, int tpb,
                                  cudaStream_t st);

// In-place (AA) step over `count` cubes, each with src == dst: parity 0 (even step count) runs the
// local step, 1 the stream step (uniform_aa.cu).  vec must be the storage's default; the threads per
// block are the smallest of 128, 256, 512 that hold a whole x-row (tpb is not followed).
cudaError_t launch_stream_collide_inplace(int storage, const UniSolve* solves, int count, int parity, int vec,
                                          int tpb, cudaStream_t st);
// Threads per block the in-place steps use for cubes up to edge max_n (0: not supported).
int inplace_tpb(int storage, int vec, int tpb, int max_n);

// Largest supported vec for a storage; a valid vec divides n and keeps n^3/vec a multiple of 32.
int default_vec(int storage);
bool vec_supported(int storage, int vec);

// TGV initial state (src/tgv3d_uniform.cu:63-77) into flat storage; axis_tab: 3*n doubles of scratch.
// aa: in the in-place layout of step 0 (population q of cell x at [q][x + c_q]).
cudaError_t launch_init_tgv(int storage, void* f, int n, double u0, double kf, double* axis_tab, cudaStream_t st,
                            bool aa = false);

// Macroscopic field (rho, ux, uy, uz) per cell, linear (z*n+y)*n+x.  FP64 storage writes double4,
// every other storage float4 (k_macro, src/tgv3d_uniform.cu:80-90).  layout: 0 flat [q][x]; 1, 2 the
// in-place layouts after an even / odd step count (aa_layout()).
cudaError_t launch_macro(int storage, const void* f, void* field, int n, cudaStream_t st, int layout = 0);

// Energy, enstrophy, mass of a macro field, reduced deterministically to out_dev[3] (device).
// partials_dev holds kDiagBlocks*3 doubles.  float_diff=true takes the velocity differences in
// float before widening (the uniform host loop, src/tgv3d_uniform.cu:103-105); false exactly
// (k_diag_reduce, src/tgv3d_amr.cu:542-546).  A float field is read in 16-byte cell records and must
// be 16-byte aligned (every solver's own field is).
constexpr int kDiagBlocks = 1216;   // 152 SMs x 8
constexpr int kDiagThreads = 256;
constexpr int kDiagPartials = kDiagBlocks * 3 + 1;  // block partials + the error word of launch_diag_pop
inline int* diag_err_word(double* partials) { return reinterpret_cast<int*>(partials + kDiagBlocks * 3); }
cudaError_t launch_diag_field(bool field_is_double, bool float_diff, const void* field, int n,
                              double* partials_dev, double* out_dev, cudaStream_t st);

// Energy, enstrophy, mass of a float-storage cube (storage 0 FP32, 1 FP16, 2 BF16) straight from its
// populations f in layout 0 / 1 / 2 (as launch_macro), with no macro field: the per-cell terms of
// launch_macro + launch_diag_field(float_diff=true), summed another way (double-float partials in a
// fixed order) to ~1e-13 of the result.
// Cubes it takes: even n (pairs of cells), n <= 1600 (32-bit cell indices).  partials_dev holds
// kDiagPartials doubles: the last is the kernel's error word (zero when allocated; set if a bounded
// wait between its warps gave up, cleared by the launch's final sum, which copies it to *flag_out
// when flag_out is given and then writes NaN diagnostics).
cudaError_t launch_diag_pop(int storage, int layout, const void* f, int n, double* partials_dev, double* out_dev,
                            double* flag_out, cudaStream_t st);
inline bool diag_pop_ok(int storage, int n) { return storage >= 0 && storage <= 2 && n % 2 == 0 && n <= 1600; }

// Q-criterion, speed and (vel != nullptr) velocity of a macro field of edge n into device arrays.
cudaError_t launch_qspeed(bool field_is_double, bool float_diff, const void* field, int n, float* Q, float* speed,
                          float* vel, cudaStream_t st);

// Count of kernel launches issued by this library (for the bench's launch accounting).
void note_launch(int k = 1);
long long launch_count();

}  // namespace jp
