// Device helpers of the three-level block AMR (reference: src/tgv3d_amr.cu).
//
// Block payloads keep the reference's layout float[blk][19][MB^3] (cell = (k*MB+j)*MB+i), so block
// tables index the same way on both sides.  Ghost layers differ: the reference stores a full
// (MB+2)^3 box per fine block of which only the shell is ever written or read; here a fine block's
// ghosts are the shell's faces and edges only (6*MB^2 + 12*MB cells; D3Q19 never pulls across a
// corner), stored as float[blk][19][SH], so the fill writes and the step reads a dense array.
#pragma once
#include <cmath>

#include "lattice.cuh"

// Loads of population arrays (pools, prolongation sources, ghost shells).  Separate kernel launches
// read them through the read-only path (__ldg).  A kernel that writes these arrays in one phase and
// reads them in a later phase of the same launch (the persistent coarse step, amr_persist.cuh)
// defines JP_COHERENT_POOLS before including this header: its loads are then ordinary weak loads
// (ld.global.ca), which the memory model orders after the acquire of the grid barrier between the
// phases; the read-only path carries no such guarantee for data written during the launch.
#ifdef JP_COHERENT_POOLS
#define JP_LDP(p) __ldca(p)
#else
#define JP_LDP(p) __ldg(p)
#endif

namespace jp {
namespace amr {

template <int MB> struct Geo {
    static constexpr int MB3 = MB * MB * MB;
    static constexpr int HALF = MB / 2;
    static constexpr int SH = 6 * MB * MB + 12 * MB;   // ghost shell cells per fine block
    static constexpr int TPB = MB3 < 512 ? MB3 : 512;  // threads per CTA for per-cell kernels
};

// Shell index of a ghost cell at block-local (i, j, k), each in [-1, MB]; -1 for interior/corner.
template <int MB>
__host__ __device__ __forceinline__ int shell_index(int i, int j, int k) {
    const bool bx = (i < 0) | (i >= MB), by = (j < 0) | (j >= MB), bz = (k < 0) | (k >= MB);
    const int cnt = int(bx) + int(by) + int(bz);
    if (cnt == 1) {
        if (bx) return (i < 0 ? 0 : 1) * MB * MB + k * MB + j;
        if (by) return (j < 0 ? 2 : 3) * MB * MB + k * MB + i;
        return (k < 0 ? 4 : 5) * MB * MB + j * MB + i;
    }
    if (cnt == 2) {
        const int base = 6 * MB * MB;
        if (!bx) return base + ((j < 0 ? 0 : 1) + 2 * (k < 0 ? 0 : 1)) * MB + i;
        if (!by) return base + (4 + (i < 0 ? 0 : 1) + 2 * (k < 0 ? 0 : 1)) * MB + j;
        return base + (8 + (i < 0 ? 0 : 1) + 2 * (j < 0 ? 0 : 1)) * MB + k;
    }
    return -1;
}
// Inverse of shell_index for t in [0, SH).
template <int MB>
__host__ __device__ __forceinline__ void shell_coord(int t, int& i, int& j, int& k) {
    if (t < 6 * MB * MB) {
        const int f = t / (MB * MB), r = t % (MB * MB), a = r % MB, b = r / MB;
        switch (f) {
            case 0: i = -1; j = a; k = b; break;
            case 1: i = MB; j = a; k = b; break;
            case 2: i = a; j = -1; k = b; break;
            case 3: i = a; j = MB; k = b; break;
            case 4: i = a; j = b; k = -1; break;
            default: i = a; j = b; k = MB; break;
        }
        return;
    }
    const int u = t - 6 * MB * MB, e = u / MB, a = u % MB;
    if (e < 4) {
        i = a; j = (e & 1) ? MB : -1; k = (e & 2) ? MB : -1;
    } else if (e < 8) {
        j = a; i = ((e - 4) & 1) ? MB : -1; k = ((e - 4) & 2) ? MB : -1;
    } else {
        k = a; i = ((e - 8) & 1) ? MB : -1; j = ((e - 8) & 2) ? MB : -1;
    }
}

// Neighbour slot of a ghost-shell cell at block-local (i, j, k), each in [-1, MB].
template <int MB>
__host__ __device__ __forceinline__ int shell_slot(int i, int j, int k) {
    return (k < 0 ? 0 : (k >= MB ? 2 : 1)) * 9 + (j < 0 ? 0 : (j >= MB ? 2 : 1)) * 3 + (i < 0 ? 0 : (i >= MB ? 2 : 1));
}

// rho, u of one cell, summed in q order as the reference's loops do
__device__ __forceinline__ void moments(const float (&f)[Q], float& rho, float& ux, float& uy, float& uz) {
    float r = f[0];
#pragma unroll
    for (int q = 1; q < Q; ++q) r += f[q];
    const float jx = f[1] - f[2] + f[7] - f[8] + f[9] - f[10] + f[11] - f[12] + f[13] - f[14];
    const float jy = f[3] - f[4] + f[7] - f[8] - f[9] + f[10] + f[15] - f[16] + f[17] - f[18];
    const float jz = f[5] - f[6] + f[11] - f[12] - f[13] + f[14] + f[15] - f[16] - f[17] + f[18];
    rho = r;
    ux = jx / r;
    uy = jy / r;
    uz = jz / r;
}

// Hermite regularisation of a non-equilibrium vector: project onto the second-order moments
// Pi = sum c c n and rebuild n_q = 4.5 w_q Q_q : Pi, Q_q = c c - I/3 (src/tgv3d_amr.cu:56-67).
__device__ __forceinline__ void regularize(float (&n)[Q]) {
    const float Pxx = n[1] + n[2] + n[7] + n[8] + n[9] + n[10] + n[11] + n[12] + n[13] + n[14];
    const float Pyy = n[3] + n[4] + n[7] + n[8] + n[9] + n[10] + n[15] + n[16] + n[17] + n[18];
    const float Pzz = n[5] + n[6] + n[11] + n[12] + n[13] + n[14] + n[15] + n[16] + n[17] + n[18];
    const float Pxy = n[7] + n[8] - n[9] - n[10];
    const float Pxz = n[11] + n[12] - n[13] - n[14];
    const float Pyz = n[15] + n[16] - n[17] - n[18];
    const float third = 1.f / 3.f;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const float Qxx = float(cx(q) * cx(q)) - third, Qyy = float(cy(q) * cy(q)) - third,
                    Qzz = float(cz(q) * cz(q)) - third;
        const float Qxy = float(cx(q) * cy(q)), Qxz = float(cx(q) * cz(q)), Qyz = float(cy(q) * cz(q));
        n[q] = 4.5f * wf(q) * (Qxx * Pxx + Qyy * Pyy + Qzz * Pzz + 2.f * (Qxy * Pxy + Qxz * Pxz + Qyz * Pyz));
    }
}

// Prolongation source of one parent cell: feq + nqs * regularize(f - feq).
__device__ __forceinline__ void prep_cell(float (&f)[Q], float nqs) {
    float rho, ux, uy, uz;
    moments(f, rho, ux, uy, uz);
    float fe[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        fe[q] = feq_ref(q, rho, ux, uy, uz);
        f[q] = f[q] - fe[q];
    }
    regularize(f);
#pragma unroll
    for (int q = 0; q < Q; ++q) f[q] = fe[q] + nqs * f[q];
}

// BGK collide of one cell in the reference's form out = f - omega (f - feq)
__device__ __forceinline__ void bgk(float (&f)[Q], float om) {
    float rho, ux, uy, uz;
    moments(f, rho, ux, uy, uz);
#pragma unroll
    for (int q = 0; q < Q; ++q) f[q] = f[q] - om * (f[q] - feq_ref(q, rho, ux, uy, uz));
}

// The same BGK collide with the arithmetic of the uniform stream-collide: one reciprocal of rho,
// out = (1 - omega) f + omega feq with omega*w*rho folded per weight class and
// feq_pm = w rho (1 - 1.5|u|^2 + 4.5 a^2) +- 3 w rho a for a = c.u over the non-zero terms only.
// Agrees with bgk() to FP32 round-off (a few ulp per population).  SH: the values are the shifts
// g = f - w_q (every AMR step works on them, PoolIO), rho = 1 + sum g, and the result is shifted too
// (feq_q - w_q = w_q (s + rho (3a + 4.5a^2 - 1.5|u|^2)) with s = sum g), which keeps the round-off at
// the level of the deviations: sum feq - rho then carries no bias of the O(w_q) terms, and mass
// drifts ~1e3 times less.  Written once over the lane type (Lanes): T = float relaxes one cell,
// T = float2 two cells with packed FP32 instructions, every operation spelled out in the same order,
// so a cell gets the same bits either way (the rows kernel relaxes its four cells as two pairs).
#ifdef __CUDACC__
template <class T, bool SH = false>
__device__ __forceinline__ void bgk_lanes(T (&f)[Q], float om) {
    using L = Lanes<T>;
    T sm = f[0];
#pragma unroll
    for (int q = 1; q < Q; ++q) sm = L::add(sm, f[q]);
    // j in q order: a signed sum of the populations with that velocity component
    constexpr int kx[10] = {1, 2, 7, 8, 9, 10, 11, 12, 13, 14}, ky[10] = {3, 4, 7, 8, 9, 10, 15, 16, 17, 18},
                  kz[10] = {5, 6, 11, 12, 13, 14, 15, 16, 17, 18};
    T jx = f[1], jy = f[3], jz = f[5];
#pragma unroll
    for (int i = 1; i < 10; ++i) {
        jx = cx(kx[i]) > 0 ? L::add(jx, f[kx[i]]) : L::sub(jx, f[kx[i]]);
        jy = cy(ky[i]) > 0 ? L::add(jy, f[ky[i]]) : L::sub(jy, f[ky[i]]);
        jz = cz(kz[i]) > 0 ? L::add(jz, f[kz[i]]) : L::sub(jz, f[kz[i]]);
    }
    const T rho = SH ? L::add(L::bc(1.f), sm) : sm;
    const T inv = L::rcp(rho);
    const T ux = L::mul(jx, inv), uy = L::mul(jy, inv), uz = L::mul(jz, inv);
    T t2 = L::mul(ux, ux);
    t2 = L::fma(uy, uy, t2);
    t2 = L::fma(uz, uz, t2);
    const T usq = L::mul(L::bc(1.5f), t2);
    const T base = SH ? L::mul(L::bc(-1.5f), t2) : L::sub(L::bc(1.f), usq);  // -usq exactly when SH
    const float omc = 1.f - om;
    const T orho = L::mul(L::bc(om), rho);
    const T owr1 = L::mul(orho, L::bc(wf(1))), owr2 = L::mul(orho, L::bc(wf(7)));
    const T owr3a = L::mul(L::bc(3.f), owr1), owr3b = L::mul(L::bc(3.f), owr2);
    if constexpr (SH) {  // (omega w0) (s - rho usq)
        f[0] = L::fma(L::bc(omc), f[0], L::mul(L::bc(om * wf(0)), L::fma(rho, base, sm)));
    } else {
        f[0] = L::fma(L::bc(omc), f[0], L::mul(L::mul(orho, L::bc(wf(0))), base));
    }
#pragma unroll
    for (int q = 1; q < Q; q += 2) {  // q odd: the first non-zero component of c_q is positive
        T a = cx(q) != 0 ? ux : (cy(q) != 0 ? uy : uz);
        if (cx(q) != 0 && cy(q) != 0) a = cy(q) > 0 ? L::add(a, uy) : L::sub(a, uy);
        if ((cx(q) != 0 || cy(q) != 0) && cz(q) != 0) a = cz(q) > 0 ? L::add(a, uz) : L::sub(a, uz);
        T t = L::mul(q < 7 ? owr1 : owr2, L::fma(L::mul(L::bc(4.5f), a), a, base));
        // + omega w s, the shifted part, as one FMA: a product by a broadcast constant followed by an add
        // is not compiled alike for one lane and for two, an FMA is
        if constexpr (SH) t = L::fma(L::bc(om * wf(q)), sm, t);
        const T as = L::mul(q < 7 ? owr3a : owr3b, a);
        f[q] = L::fma(L::bc(omc), f[q], L::add(t, as));
        f[q + 1] = L::fma(L::bc(omc), f[q + 1], L::sub(t, as));
    }
}
template <bool SH = false>
__device__ __forceinline__ void bgk_fast(float (&f)[Q], float om) {
    bgk_lanes<float, SH>(f, om);
}
#endif

// Where population q of cell (i, j, k) is pulled from: the neighbour slot e = (dz+1)*9 + (dy+1)*3 +
// (dx+1) of the same-level block at offset (dx, dy, dz) (13: the block itself) and the cell sc inside
// that block.  MB is a power of two, so sc is the pulled coordinate masked by MB-1; with q unrolled,
// which offsets a population can reach is known at compile time.
template <int MB>
__host__ __device__ __forceinline__ void pull_src(int q, int i, int j, int k, int& e, int& sc) {
    constexpr int M = MB - 1;
    static_assert((MB & M) == 0, "MB must be a power of two");
    const int li = i - cx(q), lj = j - cy(q), lk = k - cz(q);
    const int ex = cx(q) > 0 ? (li < 0 ? 0 : 1) : (cx(q) < 0 ? (li > M ? 2 : 1) : 1);
    const int ey = cy(q) > 0 ? (lj < 0 ? 0 : 1) : (cy(q) < 0 ? (lj > M ? 2 : 1) : 1);
    const int ez = cz(q) > 0 ? (lk < 0 ? 0 : 1) : (cz(q) < 0 ? (lk > M ? 2 : 1) : 1);
    e = ez * 9 + ey * 3 + ex;
    sc = ((lk & M) * MB + (lj & M)) * MB + (li & M);
}

#ifdef __CUDACC__
// Element access of the AMR pools, prolongation sources and ghost shells in a storage format of
// lattice.cuh.  f(): the unshifted population, the quantity prolongation, restriction, the sensor
// and the composite work on; n(): the stored number itself, the quantity the collision works on
// (f for FP32; the shift g = f - w_q for the 16-bit formats).
template <class ST>
struct PoolIO {
    using raw = typename ST::raw;
    static constexpr bool SH = ST::shifted;
    // the collision works on shifts g = f - w_q in every format: the 16-bit formats store them, FP32
    // shifts on load and back on store (its mass then drifts at the deviations' round-off instead of
    // the O(w_q) totals' biased round-off)
    static constexpr bool SA = true;
    __device__ static __forceinline__ float n(const raw* p) { return ST::load(JP_LDP(p)); }
    __device__ static __forceinline__ float f(const raw* p, int q) { return SH ? wf(q) + n(p) : n(p); }
    __device__ static __forceinline__ void put_n(raw* p, float v) { *p = ST::store(v); }
    __device__ static __forceinline__ void put_f(raw* p, int q, float v) { *p = ST::store(SH ? v - wf(q) : v); }
    // stored value -> the collision's shift, and back; stored value -> unshifted population
    __device__ static __forceinline__ float g_of(raw x, int q) { return SH ? ST::load(x) : ST::load(x) - wf(q); }
    __device__ static __forceinline__ raw of_g(float g, int q) { return ST::store(SH ? g : g + wf(q)); }
    __device__ static __forceinline__ float f_of(raw x, int q) { return SH ? wf(q) + ST::load(x) : ST::load(x); }
};

// Pull of the 19 populations of cell (i, j, k) of pool block b, as the collision's shifts
// (PoolIO::g_of).  nbrow[e] (global memory, the
// block's row of its level's neighbour table) is the pool index of the same-level neighbour in slot
// e (pull_src), or -1 where that neighbour is not on this level; then the value comes from b's
// ghost shell gh (GHOST = false: every neighbour exists).  Every thread reads the few table entries
// its cell needs itself: the row is shared by the whole CTA and stays in L1, and no barrier stands
// between a thread and its loads.
template <int MB, class ST, bool GHOST>
__device__ __forceinline__ void pull_cell(const typename ST::raw* __restrict__ fa, const typename ST::raw* __restrict__ gh,
                                          const int* __restrict__ nbrow, int b, int i, int j, int k,
                                          float (&f)[Q]) {
    constexpr int MB3 = MB * MB * MB, SH = Geo<MB>::SH;
    // raw values first, conversions after the loop: a conversion inside the branch would wait for
    // its load before the next population's load is issued
    typename ST::raw rv[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        int e, sc;
        pull_src<MB>(q, i, j, k, e, sc);
        const int blk = e == 13 ? b : __ldg(nbrow + e);
        if (!GHOST || blk >= 0) {
            rv[q] = JP_LDP(fa + ((size_t)blk * Q + q) * MB3 + sc);
        } else {
            rv[q] = JP_LDP(gh + ((size_t)b * Q + q) * SH + shell_index<MB>(i - cx(q), j - cy(q), k - cz(q)));
        }
    }
#pragma unroll
    for (int q = 0; q < Q; ++q) f[q] = PoolIO<ST>::g_of(rv[q], q);
}
#endif

// Trilinear weights of the cell-centred 2:1 prolongation: fine index g maps to the parent position
// (g+0.5)/2-0.5 = (2g-1)/4 (src/tgv3d_amr.cu:71-73), so the lower parent is floor((g-1)/2) and the
// weight of the upper one is 0.75 for even g, 0.25 for odd g: the reference's double expression's
// values, exactly, in integer arithmetic (GB300's FP64 rate is a small fraction of its FP32 rate).
__device__ __forceinline__ void tri_axis(int g, int& lo, float& t) {
    lo = (g - 1) >> 1;  // arithmetic shift: floor for g = 0 too
    t = (g & 1) ? 0.25f : 0.75f;
}

// a mod n for a in [-n, 2n): a wrap without a division (the corner and shell coordinates of the
// fills are at most one cell outside the periodic box)
__device__ __forceinline__ int wrap1(int a, int n) { return a < 0 ? a + n : (a >= n ? a - n : a); }

}  // namespace amr
}  // namespace jp
