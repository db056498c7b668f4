// D3Q19 lattice, BGK equilibrium and population storage formats.
//
// Velocity order, weights and the second-order equilibrium follow the reference
// (src/tgv3d_uniform.cu:28-38, src/tgv3d_amr.cu:41-55): q=0 rest, 1..6 the faces
// (+x,-x,+y,-y,+z,-z), 7..18 the edges in pairs (q, q+1) of opposite velocities.  The order is kept
// so that populations exported through the C ABI index the same way as the reference's arrays.
// Here the tables are compile-time constants, so fully unrolled loops fold every c_q*u product.
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
__host__ __device__ constexpr int opp(int q) { return q == 0 ? 0 : ((q & 1) ? q + 1 : q - 1); }

// Weights as the reference rounds them to float (1.f/3, 1.f/18, 1.f/36).
__host__ __device__ constexpr float wf(int q) {
    return q == 0 ? 1.f / 3.f : (q <= 6 ? 1.f / 18.f : 1.f / 36.f);
}
__host__ __device__ constexpr double wd(int q) {
    return q == 0 ? 1.0 / 3.0 : (q <= 6 ? 1.0 / 18.0 : 1.0 / 36.0);
}

// Reference-form equilibrium, float: w*rho*(1 + cu + cu^2/2 - 1.5|u|^2), cu = 3 c.u
// (src/tgv3d_uniform.cu:35-38).
__host__ __device__ __forceinline__ float feq_ref(int q, float rho, float ux, float uy, float uz) {
    float cu = 3.f * (cx(q) * ux + cy(q) * uy + cz(q) * uz);
    return wf(q) * rho * (1.f + cu + 0.5f * cu * cu - 1.5f * (ux * ux + uy * uy + uz * uz));
}
__host__ __device__ __forceinline__ double feq_ref_d(int q, double rho, double ux, double uy, double uz) {
    double cu = 3.0 * (cx(q) * ux + cy(q) * uy + cz(q) * uz);
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

template <class R> __host__ __device__ constexpr R wgt(int q);
template <> __host__ __device__ constexpr float wgt<float>(int q) { return wf(q); }
template <> __host__ __device__ constexpr double wgt<double>(int q) { return wd(q); }

// ---- BGK collision of one cell ----------------------------------------------------------------
// In: 19 populations (or shifted deviations) of the cell after streaming.  Out: post-collision values
// in the same representation.  Opposite pairs share the symmetric part of the equilibrium, so the
// 19 equilibria cost 9 velocity projections.  rho, u are the pre-collision moments; collision
// conserves them.
template <class R, bool SHIFT>
__device__ __forceinline__ void bgk_collide(R (&f)[Q], R omega, R& rho_out, R& ux_out, R& uy_out, R& uz_out) {
    R s = f[0];
#pragma unroll
    for (int q = 1; q < Q; ++q) s += f[q];
    // momentum: the sums run in q order over the non-zero terms, as the reference's loops do
    R jx = f[1] - f[2] + f[7] - f[8] + f[9] - f[10] + f[11] - f[12] + f[13] - f[14];
    R jy = f[3] - f[4] + f[7] - f[8] - f[9] + f[10] + f[15] - f[16] + f[17] - f[18];
    R jz = f[5] - f[6] + f[11] - f[12] - f[13] + f[14] + f[15] - f[16] - f[17] + f[18];
    const R rho = SHIFT ? R(1) + s : s;
    const R ux = jx / rho, uy = jy / rho, uz = jz / rho;
    const R usq = R(1.5) * (ux * ux + uy * uy + uz * uz);
    rho_out = rho; ux_out = ux; uy_out = uy; uz_out = uz;
    // rest population
    {
        const R w0 = wgt<R>(0);
        R feq = SHIFT ? w0 * (s - rho * usq) : w0 * rho * (R(1) - usq);
        f[0] = f[0] - omega * (f[0] - feq);
    }
#pragma unroll
    for (int q = 1; q < Q; q += 2) {
        const R w = wgt<R>(q);
        const R cu = R(3) * (R(cx(q)) * ux + R(cy(q)) * uy + R(cz(q)) * uz);
        const R wr = w * rho;
        // symmetric and antisymmetric parts of the pair's equilibria
        const R sym = SHIFT ? w * s + wr * (R(0.5) * cu * cu - usq) : wr * (R(1) + R(0.5) * cu * cu - usq);
        const R asym = wr * cu;
        const R fp = sym + asym, fm = sym - asym;
        f[q] = f[q] - omega * (f[q] - fp);
        f[q + 1] = f[q + 1] - omega * (f[q + 1] - fm);
    }
}

}  // namespace jp
