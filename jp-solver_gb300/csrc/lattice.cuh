// D3Q19 lattice, BGK equilibrium and population storage formats.
//
// Velocity order, weights and the second-order equilibrium follow the reference
// (src/tgv3d_uniform.cu:28-38, src/tgv3d_amr.cu:41-55): q=0 rest, 1..6 the faces
// (+x,-x,+y,-y,+z,-z), 7..18 the edges in pairs (q, q+1) of opposite velocities.  The order is kept
// so that populations exported through the C ABI index the same way as the reference's arrays.
// Here the tables are compile-time constants: in fully unrolled loops cdot() emits only the non-zero
// terms of every c_q . u.
#pragma once
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cuda_bf16.h>
#include <stdint.h>

namespace jp {

constexpr int Q = 19;

__host__ __device__ constexpr int cx(int q) {
    constexpr int t[Q] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0};
    return t[q];
}
__host__ __device__ constexpr int cy(int q) {
    constexpr int t[Q] = {0, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1};
    return t[q];
}
__host__ __device__ constexpr int cz(int q) {
    constexpr int t[Q] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1};
    return t[q];
}
// opposite direction of q
// (i, j, k) of cell c of an n^3 grid, i fastest: 32-bit division while the grid has fewer than 2^32
// cells (a 64-bit division by a runtime n is a long instruction sequence)
__device__ __forceinline__ void cell_ijk(long long c, int n, int& i, int& j, int& k) {
    if ((long long)n * n * n <= 0xffffffffLL) {
        const unsigned u = unsigned(c), un = unsigned(n);
        i = int(u % un);
        j = int((u / un) % un);
        k = int(u / (un * un));
    } else {
        i = int(c % n);
        j = int((c / n) % n);
        k = int(c / ((long long)n * n));
    }
}

__host__ __device__ constexpr int opp(int q) { return q == 0 ? 0 : ((q & 1) ? q + 1 : q - 1); }

// Weights as the reference rounds them to float (1.f/3, 1.f/18, 1.f/36).
__host__ __device__ constexpr float wf(int q) {
    return q == 0 ? 1.f / 3.f : (q <= 6 ? 1.f / 18.f : 1.f / 36.f);
}
__host__ __device__ constexpr double wd(int q) {
    return q == 0 ? 1.0 / 3.0 : (q <= 6 ? 1.0 / 18.0 : 1.0 / 36.0);
}

// c_q . u with only the non-zero terms (q is a compile-time constant after unrolling).  IEEE
// semantics forbid folding 0*x away, so spelling the zero terms out would cost instructions; the
// value is the same sum in the same order (x + y*0 == x for finite y).
template <class R>
__host__ __device__ __forceinline__ R cdot(int q, R ux, R uy, R uz) {
    R a = R(0);
    bool have = false;
    if (cx(q) != 0) {
        a = cx(q) > 0 ? ux : -ux;
        have = true;
    }
    if (cy(q) != 0) {
        const R t = cy(q) > 0 ? uy : -uy;
        a = have ? a + t : t;
        have = true;
    }
    if (cz(q) != 0) {
        const R t = cz(q) > 0 ? uz : -uz;
        a = have ? a + t : t;
    }
    return a;
}

// Reference-form equilibrium, float: w*rho*(1 + cu + cu^2/2 - 1.5|u|^2), cu = 3 c.u
// (src/tgv3d_uniform.cu:35-38).
__host__ __device__ __forceinline__ float feq_ref(int q, float rho, float ux, float uy, float uz) {
    float cu = 3.f * cdot<float>(q, ux, uy, uz);
    return wf(q) * rho * (1.f + cu + 0.5f * cu * cu - 1.5f * (ux * ux + uy * uy + uz * uz));
}
__host__ __device__ __forceinline__ double feq_ref_d(int q, double rho, double ux, double uy, double uz) {
    double cu = 3.0 * cdot<double>(q, ux, uy, uz);
    return wd(q) * rho * (1.0 + cu + 0.5 * cu * cu - 1.5 * (ux * ux + uy * uy + uz * uz));
}

// ---- storage formats -------------------------------------------------------------------------
// Each format says how a population is held in HBM and how it enters and leaves the FP32 (FP64)
// collision.  Shifted formats hold g = f - w_q so the stored number carries only the deviation from
// rest; the collision then works on deviations too (rho = 1 + sum g), which keeps FP32 round-off at
// the level of the deviation instead of the O(w_q) total.

struct StF32 {
    using raw = float;      // element in memory
    using real = float;     // collision arithmetic
    static constexpr bool shifted = false;
    static constexpr int id = 0;
    __device__ static __forceinline__ float load(raw v) { return v; }
    __device__ static __forceinline__ raw store(float v) { return v; }
};
struct StF16 {
    using raw = uint16_t;
    using real = float;
    static constexpr bool shifted = true;
    static constexpr int id = 1;
    __device__ static __forceinline__ float load(raw v) { return __half2float(__ushort_as_half(v)); }
    __device__ static __forceinline__ raw store(float v) { return __half_as_ushort(__float2half_rn(v)); }
    // two values rounded and packed in one conversion (a in the low half)
    __device__ static __forceinline__ unsigned int store2(float a, float b) {
        const __half2 h = __floats2half2_rn(a, b);
        return *reinterpret_cast<const unsigned int*>(&h);
    }
};
struct StBF16 {
    using raw = uint16_t;
    using real = float;
    static constexpr bool shifted = true;
    static constexpr int id = 2;
    __device__ static __forceinline__ float load(raw v) { return __bfloat162float(__ushort_as_bfloat16(v)); }
    __device__ static __forceinline__ raw store(float v) { return __bfloat16_as_ushort(__float2bfloat16_rn(v)); }
    __device__ static __forceinline__ unsigned int store2(float a, float b) {
        const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
        return *reinterpret_cast<const unsigned int*>(&h);
    }
};
struct StF64 {
    using raw = double;
    using real = double;
    static constexpr bool shifted = false;
    static constexpr int id = 3;
    __device__ static __forceinline__ double load(raw v) { return v; }
    __device__ static __forceinline__ raw store(double v) { return v; }
};

// FP32 arithmetic on one cell (float) or on a pair of cells (float2: Blackwell's packed f32x2 add,
// multiply and FMA, one instruction for both lanes), each lane rounded to nearest like the scalar op.
// Code written once over T issues half the FP32 instructions on pairs and gives every cell the same
// bits either way.
#ifdef __CUDACC__
template <class T> struct Lanes;
template <> struct Lanes<float> {
    static __device__ __forceinline__ float bc(float s) { return s; }
    static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
    static __device__ __forceinline__ float sub(float a, float b) { return __fadd_rn(a, -b); }
    static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
    static __device__ __forceinline__ float fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
    static __device__ __forceinline__ float rcp(float a) { return __frcp_rn(a); }
};
template <> struct Lanes<float2> {
    static __device__ __forceinline__ float2 bc(float s) { return make_float2(s, s); }
    static __device__ __forceinline__ float2 add(float2 a, float2 b) { return __fadd2_rn(a, b); }
    // a - b as a + (-b): an add is never merged with the product before it (an FMA by -1 can be)
    static __device__ __forceinline__ float2 sub(float2 a, float2 b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); }
    static __device__ __forceinline__ float2 mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
    static __device__ __forceinline__ float2 fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
    static __device__ __forceinline__ float2 rcp(float2 a) { return make_float2(__frcp_rn(a.x), __frcp_rn(a.y)); }
};
#endif

template <class R> __host__ __device__ constexpr R wgt(int q);
template <> __host__ __device__ constexpr float wgt<float>(int q) { return wf(q); }
template <> __host__ __device__ constexpr double wgt<double>(int q) { return wd(q); }

}  // namespace jp
