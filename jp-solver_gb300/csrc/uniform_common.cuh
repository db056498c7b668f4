// Pieces shared by the uniform-cube step kernels: 16-byte row vectors, lane exchange, the occupancy
// floor per variant, and the BGK relaxation of V cells held in registers.
//
// The pull step (uniform.cu) and the in-place AA steps (uniform_aa.cu) relax with the same
// CellBgk code, so for the same collision inputs they produce the same bits.
#pragma once

#include <type_traits>

#include "lattice.cuh"

namespace jp {

// ---- vector access helpers ---------------------------------------------------------------------

template <class RAW, int V>
struct Pack {
    static constexpr int bytes = int(sizeof(RAW)) * V;
    using word = typename std::conditional<bytes == 16, uint4,
                 typename std::conditional<bytes == 8, uint2,
                 typename std::conditional<bytes == 4, unsigned int, unsigned short>::type>::type>::type;
    union {
        word w;
        RAW v[V];
        unsigned int u32[(bytes + 3) / 4];
    };
};

// read-only for the kernel's lifetime (the pull step's source array)
template <class RAW, int V>
__device__ __forceinline__ Pack<RAW, V> ld_pack(const RAW* p) {
    Pack<RAW, V> r;
    r.w = __ldg(reinterpret_cast<const typename Pack<RAW, V>::word*>(p));
    return r;
}
// coherent load at L2, for an array the same kernel writes (the in-place steps)
template <class RAW, int V>
__device__ __forceinline__ Pack<RAW, V> ld_pack_cg(const RAW* p) {
    Pack<RAW, V> r;
    r.w = __ldcg(reinterpret_cast<const typename Pack<RAW, V>::word*>(p));
    return r;
}
template <class RAW, int V>
__device__ __forceinline__ void st_pack(RAW* p, const Pack<RAW, V>& r) {
    __stcs(reinterpret_cast<typename Pack<RAW, V>::word*>(p), r.w);
}
template <class RAW, int V>
__device__ __forceinline__ void zero_pack(Pack<RAW, V>& r) {
#pragma unroll
    for (int i = 0; i < (Pack<RAW, V>::bytes + 3) / 4; ++i) r.u32[i] = 0u;
}

template <class RAW> __device__ __forceinline__ RAW ld_one(const RAW* p) { return __ldg(p); }
template <> __device__ __forceinline__ uint16_t ld_one<uint16_t>(const uint16_t* p) {
    return __ldg(reinterpret_cast<const unsigned short*>(p));
}

template <class RAW> __device__ __forceinline__ RAW shfl_up1(RAW v) { return __shfl_up_sync(0xffffffffu, v, 1); }
template <class RAW> __device__ __forceinline__ RAW shfl_dn1(RAW v) { return __shfl_down_sync(0xffffffffu, v, 1); }
template <> __device__ __forceinline__ uint16_t shfl_up1<uint16_t>(uint16_t v) {
    return (uint16_t)__shfl_up_sync(0xffffffffu, (unsigned)v, 1);
}
template <> __device__ __forceinline__ uint16_t shfl_dn1<uint16_t>(uint16_t v) {
    return (uint16_t)__shfl_down_sync(0xffffffffu, (unsigned)v, 1);
}
template <class T> __device__ __forceinline__ T shfl_from(T v, int lane) { return __shfl_sync(0xffffffffu, v, lane); }
template <> __device__ __forceinline__ uint16_t shfl_from<uint16_t>(uint16_t v, int lane) {
    return (uint16_t)__shfl_sync(0xffffffffu, (unsigned)v, lane);
}

// Occupancy floor per SM for a variant: the wide-vector variants need warps (to keep 19 vector
// loads per thread in flight, and for the issue-bound 16-bit collision) more than registers:
// FP32 V=4 and 16-bit V=4 to 128 registers, 16-bit V=8 to 168.
template <class ST, int V, int TPB>
constexpr int min_blocks() {
    return (sizeof(typename ST::raw) * V == 16 && sizeof(typename ST::raw) == 2) ? (384 / TPB > 0 ? 384 / TPB : 1)
         : (sizeof(typename ST::raw) * V >= 8 && sizeof(typename ST::raw) <= 4) ? (512 / TPB > 0 ? 512 / TPB : 1) : 1;
}

// ---- BGK relaxation of V cells ------------------------------------------------------------------
// f[v][q] holds the collision inputs of cell v in the collision type R: the shifts g = f - w_q when SA
// (FP32 shifts on load, the 16-bit formats store shifts), f itself for FP64.  BGK as
// out = (1 - omega) f + omega feq with omega*w*rho folded per weight class: with a = c.u,
// feq_pm = w rho (1 - 1.5|u|^2 + 4.5 a^2) +- 3 w rho a (shifted: the -w part cancels against g).
// PACK: the FP32 relaxation on pairs of cells (CellBgk<float, V, true, true> below), for the 16-bit
// storages, whose steps are issue-bound; FP32 and FP64 storage keep this one.
template <class R, int V, bool SA, bool PACK = false>
struct CellBgk {
    R om, omc;
    R s[V], rho[V], ux[V], uy[V], uz[V], usq[V];
    // per cell: omega*w*rho and (shifted) omega*w*s for the face (1/18) and edge (1/36) classes, and
    // the base term 1 - 1.5|u|^2 (or -1.5|u|^2 shifted)
    R owr1[V], owr2[V], owr3a[V], owr3b[V], ows1[V], ows2[V], base[V];

    __device__ __forceinline__ explicit CellBgk(R omega) : om(omega), omc(R(1) - omega) {}

    // moments per cell (one reciprocal of rho instead of three divisions)
    __device__ __forceinline__ void moments(const R (&f)[V][Q]) {
#pragma unroll
        for (int v = 0; v < V; ++v) {
            const R* g = f[v];
            R sm = g[0];
#pragma unroll
            for (int q = 1; q < Q; ++q) sm += g[q];
            const R jx = g[1] - g[2] + g[7] - g[8] + g[9] - g[10] + g[11] - g[12] + g[13] - g[14];
            const R jy = g[3] - g[4] + g[7] - g[8] - g[9] + g[10] + g[15] - g[16] + g[17] - g[18];
            const R jz = g[5] - g[6] + g[11] - g[12] - g[13] + g[14] + g[15] - g[16] - g[17] + g[18];
            const R rh = SA ? R(1) + sm : sm;
            const R inv = R(1) / rh;
            s[v] = sm;
            rho[v] = rh;
            ux[v] = jx * inv;
            uy[v] = jy * inv;
            uz[v] = jz * inv;
            usq[v] = R(1.5) * (ux[v] * ux[v] + uy[v] * uy[v] + uz[v] * uz[v]);
        }
    }

    // relaxed rest population of cell v; sets cell v's folded terms for pair()
    __device__ __forceinline__ R rest(const R (&f)[V][Q], int v) {
        const R w0 = wgt<R>(0);
        const R feq = SA ? w0 * (s[v] - rho[v] * usq[v]) : w0 * rho[v] * (R(1) - usq[v]);
        const R o = omc * f[v][0] + om * feq;
        const R orho = om * rho[v];
        owr1[v] = orho * wgt<R>(1);
        owr2[v] = orho * wgt<R>(7);
        owr3a[v] = R(3) * owr1[v];
        owr3b[v] = R(3) * owr2[v];
        ows1[v] = SA ? om * wgt<R>(1) * s[v] : R(0);
        ows2[v] = SA ? om * wgt<R>(7) * s[v] : R(0);
        base[v] = SA ? -usq[v] : R(1) - usq[v];
        return o;
    }

    // relaxed populations q and q+1 = opp(q) (q odd) of every cell; rest() must have run for all cells
    __device__ __forceinline__ void pair(const R (&f)[V][Q], int q, R (&oa)[V], R (&ob)[V]) const {
#pragma unroll
        for (int v = 0; v < V; ++v) {
            const R a = cdot<R>(q, ux[v], uy[v], uz[v]);
            const R owr = q < 7 ? owr1[v] : owr2[v];
            const R t = owr * (R(4.5) * a * a + base[v]);
            const R osym = SA ? (q < 7 ? ows1[v] : ows2[v]) + t : t;  // omega * symmetric part
            const R oasym = (q < 7 ? owr3a[v] : owr3b[v]) * a;           // omega * antisymmetric part
            oa[v] = omc * f[v][q] + (osym + oasym);
            ob[v] = omc * f[v][q + 1] + (osym - oasym);
        }
    }
};

// ---- the same relaxation in FP32 on pairs of cells ------------------------------------------------
// Blackwell issues two FP32 adds, multiplies or FMAs in one instruction (f32x2; __fadd2_rn,
// __fmul2_rn, __ffma2_rn, each lane rounded to nearest like its scalar op).  The FP32 steps hold V = 2,
// 4 or 8 cells per thread, so the relaxation runs on pairs of cells and issues half the FP32
// instructions; an odd V runs the same sequence on single floats.  The 16-bit storages use it (their
// steps are issue-bound); FP32 storage, bound by HBM, keeps the scalar code above.  Every operation is spelled out
// (no contraction left to the compiler), so a cell's result does not depend on V, and the pull and
// in-place steps, which share this code, produce the same bits.  The sequence per cell:
//   s = g0 + g1 + ... + g18, j = the signed sums in q order, rho = 1 + s, inv = 1/rho (IEEE), u = j inv
//   t = ux ux + uy uy + uz uz (two FMAs), base = -1.5 t, feq0 = w0 (s + rho base)
//   out0 = (1 - om) g0 + om feq0, and per odd q with a = c_q . u (two terms at most):
//   sym = fma(om w, s, om w rho (4.5 a a + base)), asym = 3 om w rho a, out_q = (1 - om) g_q + (sym + asym),
//   out_opp(q) = (1 - om) g_opp(q) + (sym - asym).
template <int V>
struct CellBgk<float, V, true, true> {
    static constexpr bool PAIR = V % 2 == 0;
    static constexpr int NP = PAIR ? V / 2 : V;  // lanes
    using T = typename std::conditional<PAIR, float2, float>::type;
    using L = Lanes<T>;
    float om, omc;
    T s[NP], rho[NP], ux[NP], uy[NP], uz[NP], base[NP];
    T owr1[NP], owr2[NP], owr3a[NP], owr3b[NP];
    T orest[NP];

    __device__ __forceinline__ explicit CellBgk(float omega) : om(omega), omc(1.f - omega) {}

    static __device__ __forceinline__ T get(const float (&f)[V][Q], int p, int q) {
        if constexpr (PAIR) return make_float2(f[2 * p][q], f[2 * p + 1][q]);
        else return f[p][q];
    }
    static __device__ __forceinline__ void put(float (&o)[V], int p, T v) {
        if constexpr (PAIR) {
            o[2 * p] = v.x;
            o[2 * p + 1] = v.y;
        } else {
            o[p] = v;
        }
    }
    // c_q . u for odd q (its first non-zero component is positive)
    __device__ __forceinline__ T cdot_odd(int q, int p) const {
        T a = cx(q) != 0 ? ux[p] : (cy(q) != 0 ? uy[p] : uz[p]);
        if (cx(q) != 0 && cy(q) != 0) a = cy(q) > 0 ? L::add(a, uy[p]) : L::sub(a, uy[p]);
        if ((cx(q) != 0 || cy(q) != 0) && cz(q) != 0) a = cz(q) > 0 ? L::add(a, uz[p]) : L::sub(a, uz[p]);
        return a;
    }

    __device__ __forceinline__ void moments(const float (&f)[V][Q]) {
#pragma unroll
        for (int p = 0; p < NP; ++p) {
            T g[Q];
#pragma unroll
            for (int q = 0; q < Q; ++q) g[q] = get(f, p, q);
            T sm = g[0];
#pragma unroll
            for (int q = 1; q < Q; ++q) sm = L::add(sm, g[q]);
            // j in q order: a signed sum of the populations with that velocity component
            constexpr int kx[10] = {1, 2, 7, 8, 9, 10, 11, 12, 13, 14}, ky[10] = {3, 4, 7, 8, 9, 10, 15, 16, 17, 18},
                          kz[10] = {5, 6, 11, 12, 13, 14, 15, 16, 17, 18};
            T jx = g[1], jy = g[3], jz = g[5];
#pragma unroll
            for (int i = 1; i < 10; ++i) {
                jx = cx(kx[i]) > 0 ? L::add(jx, g[kx[i]]) : L::sub(jx, g[kx[i]]);
                jy = cy(ky[i]) > 0 ? L::add(jy, g[ky[i]]) : L::sub(jy, g[ky[i]]);
                jz = cz(kz[i]) > 0 ? L::add(jz, g[kz[i]]) : L::sub(jz, g[kz[i]]);
            }
            const T rh = L::add(L::bc(1.f), sm);
            const T inv = L::rcp(rh);
            s[p] = sm;
            rho[p] = rh;
            ux[p] = L::mul(jx, inv);
            uy[p] = L::mul(jy, inv);
            uz[p] = L::mul(jz, inv);
            T t = L::mul(ux[p], ux[p]);
            t = L::fma(uy[p], uy[p], t);
            t = L::fma(uz[p], uz[p], t);
            base[p] = L::mul(L::bc(-1.5f), t);
            // the folded per-class terms and the rest population
            const T feq0 = L::mul(L::bc(wf(0)), L::fma(rh, base[p], sm));
            orest[p] = L::fma(L::bc(omc), g[0], L::mul(L::bc(om), feq0));
            const T orho = L::mul(L::bc(om), rh);
            owr1[p] = L::mul(orho, L::bc(wf(1)));
            owr2[p] = L::mul(orho, L::bc(wf(7)));
            owr3a[p] = L::mul(L::bc(3.f), owr1[p]);
            owr3b[p] = L::mul(L::bc(3.f), owr2[p]);

        }
    }

    // relaxed rest population of cell v (moments() computed it)
    __device__ __forceinline__ float rest(const float (&)[V][Q], int v) const {
        if constexpr (PAIR) return (v & 1) ? orest[v / 2].y : orest[v / 2].x;
        else return orest[v];
    }

    // relaxed populations q and q+1 = opp(q) (q odd) of every cell
    __device__ __forceinline__ void pair(const float (&f)[V][Q], int q, float (&oa)[V], float (&ob)[V]) const {
#pragma unroll
        for (int p = 0; p < NP; ++p) {
            const T a = cdot_odd(q, p);
            const T owr = q < 7 ? owr1[p] : owr2[p];
            const T t = L::mul(owr, L::fma(L::mul(L::bc(4.5f), a), a, base[p]));
            // + omega w s as one FMA (a product by a broadcast constant then an add is not compiled
            // alike in every kernel; an FMA is)
            const T osym = L::fma(L::bc(om * wf(q)), s[p], t);
            const T oasym = L::mul(q < 7 ? owr3a[p] : owr3b[p], a);
            put(oa, p, L::fma(L::bc(omc), get(f, p, q), L::add(osym, oasym)));
            put(ob, p, L::fma(L::bc(omc), get(f, p, q + 1), L::sub(osym, oasym)));
        }
    }
};

// Relaxed values of V cells into a row vector of storage words: 16-bit formats convert two cells per
// instruction; FP32 shifts back by w_q (SA without SH).
template <class ST, int V, bool SA>
__device__ __forceinline__ void put_row(Pack<typename ST::raw, V>& p, const typename ST::real (&o)[V], int q) {
    using R = typename ST::real;
    if constexpr (ST::shifted && V % 2 == 0) {
#pragma unroll
        for (int v = 0; v < V; v += 2) p.u32[v / 2] = ST::store2(o[v], o[v + 1]);
    } else {
#pragma unroll
        for (int v = 0; v < V; ++v) p.v[v] = ST::store((SA && !ST::shifted) ? o[v] + wgt<R>(q) : o[v]);
    }
}

}  // namespace jp
