// Per-cell diagnostic terms of a float macro field (rho, ux, uy, uz per cell) without FP64 arithmetic
// in the per-cell work.
//
// The reference forms 1/2|u|^2, 1/2|curl u|^2 (central differences, periodic) and rho per cell in
// FP64 and sums them in FP64 (src/tgv3d_amr.cu:538-549; the uniform program's host loop,
// src/tgv3d_uniform.cu:172-181).  GB300 issues FP64 at a small fraction of its FP32 rate, so those
// ~45 FP64 instructions per cell made a diagnostic cost more than the steps it reports on (an N=128
// field: ~150 us, against ~50 us for an FP32 step of the cube).
//
// Here each per-cell term is an unevaluated sum of two floats (hi + lo, "double-float") built from
// error-free transformations: TwoProd (hi = a*b, lo = fma(a, b, -hi)) makes the product of two floats
// exact, TwoSum (Knuth) the sum of two floats.  The velocity differences are therefore exact (in FP64
// they are exact for floats of similar magnitude), the squares and sums carry about 2^-47 relative
// error, and the three terms are non-negative, so every sum of them keeps that relative error
// (~1e-14), well below the summation-order differences of FP64 sums (the diagnostics are checked to
// 1e-12 relative).  A thread keeps its running sums in double-float over kFlush cells and then adds
// them to FP64 accumulators: a few FP64 instructions per kFlush cells.  All arithmetic goes through
// the _rn intrinsics, which the compiler never contracts or reorders.
#pragma once
#include <cuda_runtime.h>

namespace jp {
namespace dterm {

struct FF {
    float hi, lo;
};

// a + b exactly (Knuth's TwoSum)
__device__ __forceinline__ FF two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}

// a + b exactly when |a| >= |b| or a == 0 (Dekker's Fast2Sum)
__device__ __forceinline__ FF fast_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

// a * b exactly (barring underflow of the error term)
__device__ __forceinline__ FF two_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    return {p, __fmaf_rn(a, b, -p)};
}

// x + y for x, y of the same sign: relative error below 2^-46
__device__ __forceinline__ FF add_same_sign(FF x, FF y) {
    const FF s = two_sum(x.hi, y.hi);
    return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(x.lo, y.lo)));
}

// x + y of any signs (Joldes, Muller, Popescu 2017, "AccurateDWPlusDW"): relative error below
// 3 * 2^-48 even under cancellation
__device__ __forceinline__ FF add(FF x, FF y) {
    const FF s = two_sum(x.hi, y.hi);
    const FF t = two_sum(x.lo, y.lo);
    const FF v = fast_two_sum(s.hi, __fadd_rn(s.lo, t.hi));
    return fast_two_sum(v.hi, __fadd_rn(t.lo, v.lo));
}

__device__ __forceinline__ FF sq(FF x) {
    const FF p = two_prod(x.hi, x.hi);
    return fast_two_sum(p.hi, __fmaf_rn(__fmul_rn(2.f, x.hi), x.lo, p.lo));
}

__device__ __forceinline__ FF half(FF x) { return {__fmul_rn(x.hi, 0.5f), __fmul_rn(x.lo, 0.5f)}; }

__device__ __forceinline__ double to_double(FF x) { return double(x.hi) + double(x.lo); }

// 1/2|u|^2 and 1/2|curl u|^2 of a cell from its velocity (u, v, w) and its six face neighbours'
// components that the curl uses: v, w at x+1 / x-1, u, w at y+1 / y-1, u, v at z+1 / z-1.
// FLOAT_DIFF takes each velocity difference in float (rounded) before halving, as the uniform
// program's host loop does; otherwise the difference of the two floats is exact, as in the AMR
// diagnostic kernel.
template <bool FLOAT_DIFF>
__device__ __forceinline__ void velocity_terms(float u, float v, float w, float vxp, float vxm, float wxp, float wxm,
                                               float uyp, float uym, float wyp, float wym, float uzp, float uzm,
                                               float vzp, float vzm, FF& e, FF& ens) {
    auto dif = [&](float a, float b) -> FF {
        if (FLOAT_DIFF) return {__fmul_rn(__fsub_rn(a, b), 0.5f), 0.f};
        return half(two_sum(a, -b));
    };
    e = half(add_same_sign(add_same_sign(two_prod(u, u), two_prod(v, v)), two_prod(w, w)));
    const FF dudy = dif(uyp, uym), dudz = dif(uzp, uzm);
    const FF dvdx = dif(vxp, vxm), dvdz = dif(vzp, vzm);
    const FF dwdx = dif(wxp, wxm), dwdy = dif(wyp, wym);
    FF ox, oy, oz;
    if (FLOAT_DIFF) {  // differences of single floats: exact
        ox = two_sum(dwdy.hi, -dvdz.hi);
        oy = two_sum(dudz.hi, -dwdx.hi);
        oz = two_sum(dvdx.hi, -dudy.hi);
    } else {
        ox = add(dwdy, {-dvdz.hi, -dvdz.lo});
        oy = add(dudz, {-dwdx.hi, -dwdx.lo});
        oz = add(dvdx, {-dudy.hi, -dudy.lo});
    }
    ens = half(add_same_sign(add_same_sign(sq(ox), sq(oy)), sq(oz)));
}

// 1/2|u|^2, 1/2|curl u|^2 and rho of cell (i, j, k) of an n^3 field F[cell][4] (rho, ux, uy, uz;
// i fastest), periodic.  VEC reads each cell record with one 16-byte load (F 16-byte aligned), else
// per float.
template <bool FLOAT_DIFF, bool VEC>
__device__ __forceinline__ void cell_terms(const float* __restrict__ F, int n, int i, int j, int k, FF& e, FF& ens,
                                           float& rho) {
    const int ip = i + 1 == n ? 0 : i + 1, im = i == 0 ? n - 1 : i - 1;
    const int jp = j + 1 == n ? 0 : j + 1, jm = j == 0 ? n - 1 : j - 1;
    const int kp = k + 1 == n ? 0 : k + 1, km = k == 0 ? n - 1 : k - 1;
    auto rec = [&](int a, int b, int cc) -> float4 {
        const float* p = F + (((size_t)cc * n + b) * n + a) * 4;
        if (VEC) return __ldg(reinterpret_cast<const float4*>(p));
        return make_float4(__ldg(p), __ldg(p + 1), __ldg(p + 2), __ldg(p + 3));
    };
    const float4 me = rec(i, j, k);
    const float4 xp = rec(ip, j, k), xm = rec(im, j, k), yp = rec(i, jp, k), ym = rec(i, jm, k);
    const float4 zp = rec(i, j, kp), zm = rec(i, j, km);
    rho = me.x;
    velocity_terms<FLOAT_DIFF>(me.y, me.z, me.w, xp.z, xm.z, xp.w, xm.w, yp.y, ym.y, yp.w, ym.w, zp.y, zm.y, zp.z,
                               zm.z, e, ens);
}

// The cells c0, c0 + S, c0 + 2S, ... of an n^3 grid (i fastest) as (i, j, k), advanced by adding the
// stride's own (i, j, k) with carries: no division per cell (a 64-bit division by a runtime n is a
// long instruction sequence).  Valid while k < n.
struct CellWalk {
    int i, j, k, si, sj, sk, n;
    __device__ __forceinline__ CellWalk(long long c0, long long S, int n_) : n(n_) {
        const long long plane = (long long)n * n;
        k = int(c0 / plane);
        j = int((c0 - (long long)k * plane) / n);
        i = int(c0 - (long long)k * plane - (long long)j * n);
        sk = int(S / plane);
        sj = int((S - (long long)sk * plane) / n);
        si = int(S - (long long)sk * plane - (long long)sj * n);
    }
    __device__ __forceinline__ bool valid() const { return k < n; }
    __device__ __forceinline__ void next() {
        i += si;
        if (i >= n) {
            i -= n;
            ++j;
        }
        j += sj;
        if (j >= n) {
            j -= n;
            ++k;
        }
        k += sk;
    }
};

// A thread's sums: double-float over kFlush cells, then into FP64.
struct Acc {
    static constexpr int kFlush = 8;
    FF e{0.f, 0.f}, ens{0.f, 0.f}, mass{0.f, 0.f};
    double de = 0.0, dens = 0.0, dmass = 0.0;
    int k = 0;
    __device__ __forceinline__ void add_cell(FF ce, FF cens, float rho) {
        e = add_same_sign(e, ce);
        ens = add_same_sign(ens, cens);
        mass = add(mass, {rho, 0.f});  // rho of any sign (a field under test need not be physical)
        if (++k == kFlush) flush();
    }
    __device__ __forceinline__ void flush() {
        de += to_double(e);
        dens += to_double(ens);
        dmass += to_double(mass);
        e = ens = mass = FF{0.f, 0.f};
        k = 0;
    }
};

// Running sums for the diagnostic straight from the populations, cheaper per cell than Acc.  A cell
// adds its three energy products u*u, v*v, w*w (exact pairs from two_prod) into a double-float
// partial (hi by TwoSum, the low parts and TwoSum's errors gathered in lo), that partial into the
// energy sum with add_same_sign; the enstrophy likewise from the three exact vorticity components
// (hi^2 + 2 hi lo; lo^2 < 2^-48 of it is dropped); the mass with TwoSum and a renormalisation per
// cell, so any sign of rho keeps it exact to ~2^-47.  The 1/2 of the energy and the enstrophy is
// applied once, in FP64, at the flush (halving is exact).  Error per cell below ~2^-46 of the
// running sum; kFlush cells per FP64 flush keep the sums within ~32 * 2^-46 ~ 5e-13 relative in the
// worst case, ~1e-14 in practice.
struct CellSums {
    static constexpr int kFlush = 32;
    FF e{0.f, 0.f}, ens{0.f, 0.f}, mass{0.f, 0.f};
    double de = 0.0, dens = 0.0, dmass = 0.0;
    int k = 0;

    // the first square of a partial, then the next ones
    __device__ static __forceinline__ FF sq1(float a) {
        const float p = __fmul_rn(a, a);
        return {p, __fmaf_rn(a, a, -p)};
    }
    __device__ static __forceinline__ void sq_add(FF& s, float a) {
        const float p = __fmul_rn(a, a);
        const float lo = __fmaf_rn(a, a, -p);
        const FF t = two_sum(s.hi, p);
        s = {t.hi, __fadd_rn(s.lo, __fadd_rn(t.lo, lo))};
    }
    // x^2 of an exact double-float x, to ~2^-47
    __device__ static __forceinline__ FF dsq1(FF x) {
        const float p = __fmul_rn(x.hi, x.hi);
        return {p, __fmaf_rn(__fadd_rn(x.hi, x.hi), x.lo, __fmaf_rn(x.hi, x.hi, -p))};
    }
    __device__ static __forceinline__ void dsq_add(FF& s, FF x) {
        const FF q = dsq1(x);
        const FF t = two_sum(s.hi, q.hi);
        s = {t.hi, __fadd_rn(s.lo, __fadd_rn(t.lo, q.lo))};
    }

    // the cell with velocity (u, v, w), density rho and the neighbour components velocity_terms takes;
    // velocity differences in float (rounded), as the uniform program's host loop takes them
    __device__ __forceinline__ void add_cell(float u, float v, float w, float rho, float vxp, float vxm, float wxp,
                                             float wxm, float uyp, float uym, float wyp, float wym, float uzp,
                                             float uzm, float vzp, float vzm) {
        FF pe = sq1(u);
        sq_add(pe, v);
        sq_add(pe, w);
        e = add_same_sign(e, pe);
        auto dif = [](float a, float b) { return __fmul_rn(__fsub_rn(a, b), 0.5f); };
        const float dudy = dif(uyp, uym), dudz = dif(uzp, uzm);
        const float dvdx = dif(vxp, vxm), dvdz = dif(vzp, vzm);
        const float dwdx = dif(wxp, wxm), dwdy = dif(wyp, wym);
        FF pz = dsq1(two_sum(dwdy, -dvdz));
        dsq_add(pz, two_sum(dudz, -dwdx));
        dsq_add(pz, two_sum(dvdx, -dudy));
        ens = add_same_sign(ens, pz);
        const FF t = two_sum(mass.hi, rho);
        mass = fast_two_sum(t.hi, __fadd_rn(mass.lo, t.lo));
        if (++k == kFlush) flush();
    }
    __device__ __forceinline__ void flush() {
        de += 0.5 * to_double(e);
        dens += 0.5 * to_double(ens);
        dmass += to_double(mass);
        e = ens = mass = FF{0.f, 0.f};
        k = 0;
    }
};

}  // namespace dterm
}  // namespace jp
