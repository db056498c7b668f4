// Uniform periodic D3Q19 BGK: Taylor-Green initial state, fused pull stream-collide, macro field and
// the energy / enstrophy / mass reduction.
//
// Reference: src/tgv3d_uniform.cu.  The reference keeps populations as [block][q][8^3 cells] and
// launches one CUDA block per 8^3 block with a modulo per population to find the pulled cell
// (k_step, :40-61).  Here a cube lives in the flat SoA layout [q][z][y][x]: a thread owns V
// consecutive cells of one x-row, reads each of the 19 source rows as one aligned 16-byte vector,
// and gets the one value that a +-x pull needs from outside its vector from the neighbouring lane by
// a warp shuffle (a direct load only at the warp and row edges, which wrap periodically).  Every
// population is therefore read from HBM once and written once per step, with full 128-byte lines
// on both sides: 152 B per lattice update in FP32, 76 B in FP16/BF16, 304 B in FP64.
#include "kernels.h"
#include "lattice.cuh"
#include "diag_terms.cuh"
#include "uniform_common.cuh"

#include <algorithm>
#include <atomic>

namespace jp {

static std::atomic<long long> g_launches{0};
void note_launch(int k) { g_launches.fetch_add(k, std::memory_order_relaxed); }
long long launch_count() { return g_launches.load(std::memory_order_relaxed); }

template <class ST, int V, int TPB>
__global__ void __launch_bounds__(TPB, (min_blocks<ST, V, TPB>())) k_stream_collide(const __grid_constant__ UniBatch b) {
    using raw = typename ST::raw;
    using R = typename ST::real;
    constexpr bool SH = ST::shifted;
    // the collision works on the shifts g = f - w_q: the 16-bit formats store them, FP32 shifts on
    // load and back on store (mass drift at the level of the deviations' round-off, not of the
    // O(w_q) totals' biased round-off); FP64 works on f
    constexpr bool SA = SH || sizeof(raw) == 4;

    // which cube this CUDA block belongs to (uniform over the block)
    int si = 0;
#pragma unroll 1
    for (int i = 1; i < b.count; ++i) si = (b.s[i].blk_begin <= (long long)blockIdx.x) ? i : si;
    const UniSolve& d = b.s[si];
    const long long seg = ((long long)blockIdx.x - d.blk_begin) * TPB + threadIdx.x;
    if (seg >= d.nseg) return;  // whole warps: nseg is a multiple of 32

    const int n = d.n;
    const int nxs = d.nxs;
    const raw* __restrict__ src = static_cast<const raw*>(d.src);
    raw* __restrict__ dst = static_cast<raw*>(d.dst);
    const int xs = int(seg % nxs);
    const long long r = seg / nxs;
    const int y = int(r % n);
    const int z = int(r / n);
    const int x0 = xs * V;
    const int lane = threadIdx.x & 31;
    const size_t qs = (size_t)n * n * n;
    // the nine x-rows around (y, z) (periodic): offsets of their starts within a population plane,
    // 32-bit (n^3 < 2^32, checked at launch); row (dy, dz) at roff[(dz + 1) * 3 + dy + 1]
    unsigned roff[9];
    {
        const int ys[3] = {y == 0 ? n - 1 : y - 1, y, y == n - 1 ? 0 : y + 1};
        const int zs[3] = {z == 0 ? n - 1 : z - 1, z, z == n - 1 ? 0 : z + 1};
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int c = 0; c < 3; ++c) roff[a * 3 + c] = ((unsigned)zs[a] * n + ys[c]) * n;
    }
    const bool prev_direct = (lane == 0) || (x0 == 0);
    const bool next_direct = (lane == 31) || (x0 + V == n);
    const int xprev = x0 == 0 ? n - 1 : x0 - 1;
    const int xnext = (x0 + V == n) ? 0 : x0 + V;

    // 1. issue every load: 19 row vectors + the edge values of the 10 populations with c_x != 0
    Pack<raw, V> L[Q];
    raw E[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const raw* p = src + q * qs + roff[(1 - cz(q)) * 3 + 1 - cy(q)];  // pull from (y, z) - c_(y,z)
        L[q] = ld_pack<raw, V>(p + x0);
        E[q] = raw(0);
        if (cx(q) > 0 && prev_direct) E[q] = ld_one(p + xprev);
        if (cx(q) < 0 && next_direct) E[q] = ld_one(p + xnext);
    }
    // 2. neighbour values across the vector edge from the adjacent lanes
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        if (cx(q) > 0) {
            raw t = shfl_up1(L[q].v[V - 1]);
            if (!prev_direct) E[q] = t;
        } else if (cx(q) < 0) {
            raw t = shfl_dn1(L[q].v[0]);
            if (!next_direct) E[q] = t;
        }
    }
    // 3. the pulled values of every cell, converted to the collision type once
    R f[V][Q];
#pragma unroll
    for (int q = 0; q < Q; ++q)
#pragma unroll
        for (int v = 0; v < V; ++v) {
            raw e;
            if (cx(q) > 0) e = (v == 0) ? E[q] : L[q].v[v - 1];
            else if (cx(q) < 0) e = (v == V - 1) ? E[q] : L[q].v[v + 1];
            else e = L[q].v[v];
            f[v][q] = (SA && !SH) ? ST::load(e) - wgt<R>(q) : ST::load(e);
        }

    // 4. moments, 5. relax and store, one population pair at a time
    const R om = sizeof(R) == 8 ? R(d.omega_d) : R(d.omega);
    CellBgk<R, V, SA, SH> c(om);
    c.moments(f);
    const size_t orow = ((size_t)z * n + y) * n + x0;
    {
        R o[V];
#pragma unroll
        for (int v = 0; v < V; ++v) o[v] = c.rest(f, v);
        Pack<raw, V> p;
        put_row<ST, V, SA>(p, o, 0);
        st_pack<raw, V>(dst + orow, p);
    }
#pragma unroll
    for (int q = 1; q < Q; q += 2) {
        R oa[V], ob[V];
        c.pair(f, q, oa, ob);
        Pack<raw, V> pa, pb;
        put_row<ST, V, SA>(pa, oa, q);
        put_row<ST, V, SA>(pb, ob, q + 1);
        st_pack<raw, V>(dst + q * qs + orow, pa);
        st_pack<raw, V>(dst + (q + 1) * qs + orow, pb);
    }
}

int default_vec(int storage) {
    switch (storage) {
        case 0: return 4;   // float4
        case 1: return 4;   // 4 x half
        case 2: return 4;   // 4 x bf16
        case 3: return 2;   // double2
    }
    return 0;
}
bool vec_supported(int storage, int vec) {
    switch (storage) {
        case 0: return vec == 1 || vec == 2 || vec == 4;
        case 1: case 2: return vec == 2 || vec == 4 || vec == 8;
        case 3: return vec == 1 || vec == 2;
    }
    return false;
}

template <class ST, int V, int TPB>
static cudaError_t launch_sc(const UniSolve* solves, int count, cudaStream_t st) {
    UniBatch b;
    b.count = count;
    b.pad = 0;
    long long blocks = 0;
    for (int i = 0; i < count; ++i) {
        b.s[i] = solves[i];
        b.s[i].nxs = solves[i].n / V;
        b.s[i].nseg = (long long)solves[i].n * solves[i].n * solves[i].n / V;
        b.s[i].blk_begin = blocks;
        blocks += (b.s[i].nseg + TPB - 1) / TPB;
    }
    if (blocks <= 0) return cudaSuccess;
    if (blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
    k_stream_collide<ST, V, TPB><<<(unsigned)blocks, TPB, 0, st>>>(b);
    note_launch();
    return cudaGetLastError();
}

template <class ST, int V>
static cudaError_t launch_sc_tpb(int tpb, const UniSolve* s, int c, cudaStream_t st) {
    switch (tpb) {
        case 64: return launch_sc<ST, V, 64>(s, c, st);
        case 128: return launch_sc<ST, V, 128>(s, c, st);
        case 512: return launch_sc<ST, V, 512>(s, c, st);
        default: return launch_sc<ST, V, 256>(s, c, st);
    }
}

cudaError_t launch_stream_collide(int storage, const UniSolve* solves, int count, int vec, int tpb,
                                  cudaStream_t st) {
    if (count <= 0) return cudaSuccess;
    if (count > kMaxBatch) return cudaErrorInvalidValue;
    if (vec == 0) vec = default_vec(storage);
    if (!vec_supported(storage, vec)) return cudaErrorInvalidValue;
    for (int i = 0; i < count; ++i)
        if (solves[i].n % vec != 0 || ((long long)solves[i].n * solves[i].n * solves[i].n / vec) % 32 != 0 ||
            (long long)solves[i].n * solves[i].n * solves[i].n >= (1LL << 32))
            return cudaErrorInvalidValue;
    switch (storage) {
        case 0:
            if (vec == 4) return launch_sc_tpb<StF32, 4>(tpb, solves, count, st);
            if (vec == 2) return launch_sc_tpb<StF32, 2>(tpb, solves, count, st);
            return launch_sc_tpb<StF32, 1>(tpb, solves, count, st);
        case 1:
            if (vec == 8) return launch_sc_tpb<StF16, 8>(tpb, solves, count, st);
            if (vec == 4) return launch_sc_tpb<StF16, 4>(tpb, solves, count, st);
            return launch_sc_tpb<StF16, 2>(tpb, solves, count, st);
        case 2:
            if (vec == 8) return launch_sc_tpb<StBF16, 8>(tpb, solves, count, st);
            if (vec == 4) return launch_sc_tpb<StBF16, 4>(tpb, solves, count, st);
            return launch_sc_tpb<StBF16, 2>(tpb, solves, count, st);
        case 3:
            if (vec == 2) return launch_sc_tpb<StF64, 2>(tpb, solves, count, st);
            return launch_sc_tpb<StF64, 1>(tpb, solves, count, st);
    }
    return cudaErrorInvalidValue;
}

// ---- Taylor-Green initial state ------------------------------------------------------------------
// u = u0 sin x cos y cos z, v = -u0 cos x sin y cos z, w = 0 at cell centres (i+0.5)kf, pressure folded
// into rho = 1 + 3p, p = u0^2/16 (cos2x + cos2y)(cos2z + 2), equilibrium populations
// (src/tgv3d_uniform.cu:63-77).  FP32 storage rounds rho and u to float and evaluates the float
// equilibrium as the reference does; FP64 keeps double; shifted formats store the double deviation.
// The field is separable: sin, cos and cos(2.) of (i+0.5)kf per axis index, tabulated once with the
// same double expressions, give the same values as evaluating them per cell.
__global__ void k_tgv_axis(double* __restrict__ tab, int n, double kf) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double x = (i + 0.5) * kf;
    tab[i] = sin(x);
    tab[n + i] = cos(x);
    tab[2 * n + i] = cos(2 * x);
}

// aa: write population q of cell x to x + c_q (the in-place layout of an even step count, in which
// every population already sits where the next step reads it)
template <class ST>
__global__ void k_init_tgv(typename ST::raw* __restrict__ f, int n, double u0, const double* __restrict__ tab,
                           bool aa) {
    const long long cells = (long long)n * n * n;
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cells) return;
    int i, j, k;
    cell_ijk(c, n, i, j, k);
    const double sx = tab[i], cxv = tab[n + i], c2x = tab[2 * n + i];
    const double sy = tab[j], cyv = tab[n + j], c2y = tab[2 * n + j];
    const double czv = tab[n + k], c2z = tab[2 * n + k];
    const double ux = u0 * sx * cyv * czv;
    const double uy = -u0 * cxv * sy * czv;
    const double p = (u0 * u0 / 16.0) * (c2x + c2y) * (c2z + 2.0);
    const double rho = 1.0 + 3.0 * p;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        typename ST::raw v;
        if constexpr (ST::id == 0) {
            v = feq_ref(q, float(rho), float(ux), float(uy), 0.f);
        } else if constexpr (ST::id == 3) {
            v = feq_ref_d(q, rho, ux, uy, 0.0);
        } else {
            const double cu = 3.0 * (cx(q) * ux + cy(q) * uy);
            const double g = wd(q) * (3.0 * p + rho * (cu + 0.5 * cu * cu - 1.5 * (ux * ux + uy * uy)));
            v = ST::store(float(g));
        }
        size_t o = c;
        if (aa) {
            const int xi = (i + cx(q) + n) % n, yj = (j + cy(q) + n) % n, zk = (k + cz(q) + n) % n;
            o = ((size_t)zk * n + yj) * n + xi;
        }
        f[(size_t)q * cells + o] = v;
    }
}

cudaError_t launch_init_tgv(int storage, void* f, int n, double u0, double kf, double* axis_tab, cudaStream_t st,
                            bool aa) {
    const long long cells = (long long)n * n * n;
    const unsigned blocks = (unsigned)((cells + 255) / 256);
    k_tgv_axis<<<(n + 255) / 256, 256, 0, st>>>(axis_tab, n, kf);
    switch (storage) {
        case 0: k_init_tgv<StF32><<<blocks, 256, 0, st>>>((float*)f, n, u0, axis_tab, aa); break;
        case 1: k_init_tgv<StF16><<<blocks, 256, 0, st>>>((uint16_t*)f, n, u0, axis_tab, aa); break;
        case 2: k_init_tgv<StBF16><<<blocks, 256, 0, st>>>((uint16_t*)f, n, u0, axis_tab, aa); break;
        case 3: k_init_tgv<StF64><<<blocks, 256, 0, st>>>((double*)f, n, u0, axis_tab, aa); break;
        default: return cudaErrorInvalidValue;
    }
    note_launch(2);
    return cudaGetLastError();
}

// ---- macro field ---------------------------------------------------------------------------------
// layout 0: population q of cell x at [q][x]; the in-place layouts: 1 (even step count) at
// [q][x + c_q], 2 (odd step count) at [opp q][x]
// rho and u = j / rho of one cell from its 19 populations (shifted storage adds the rest density 1)
template <class ST>
__device__ __forceinline__ void cell_macro(const typename ST::real (&v)[Q], typename ST::real& rho,
                                           typename ST::real& ux, typename ST::real& uy, typename ST::real& uz) {
    using R = typename ST::real;
    R sm = v[0];
#pragma unroll
    for (int q = 1; q < Q; ++q) sm += v[q];
    const R jx = v[1] - v[2] + v[7] - v[8] + v[9] - v[10] + v[11] - v[12] + v[13] - v[14];
    const R jy = v[3] - v[4] + v[7] - v[8] - v[9] + v[10] + v[15] - v[16] + v[17] - v[18];
    const R jz = v[5] - v[6] + v[11] - v[12] - v[13] + v[14] + v[15] - v[16] - v[17] + v[18];
    rho = ST::shifted ? R(1) + sm : sm;
    ux = jx / rho;
    uy = jy / rho;
    uz = jz / rho;
}

template <class ST, class FT>
__global__ void k_macro(const typename ST::raw* __restrict__ f, FT* __restrict__ out, int n, int layout) {
    using R = typename ST::real;
    const long long cells = (long long)n * n * n;
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cells) return;
    int i, j, k;
    cell_ijk(c, n, i, j, k);
    R v[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        size_t o = (size_t)q * cells + c;
        if (layout == 1)
            o = (size_t)q * cells + ((size_t)((k + cz(q) + n) % n) * n + (j + cy(q) + n) % n) * n + (i + cx(q) + n) % n;
        else if (layout == 2)
            o = (size_t)opp(q) * cells + c;
        v[q] = ST::load(f[o]);
    }
    R rho, ux, uy, uz;
    cell_macro<ST>(v, rho, ux, uy, uz);
    FT* o = out + 4 * c;
    o[0] = FT(rho);
    o[1] = FT(ux);
    o[2] = FT(uy);
    o[3] = FT(uz);
}

cudaError_t launch_macro(int storage, const void* f, void* field, int n, cudaStream_t st, int layout) {
    const long long cells = (long long)n * n * n;
    const unsigned blocks = (unsigned)((cells + 255) / 256);
    switch (storage) {
        case 0: k_macro<StF32, float><<<blocks, 256, 0, st>>>((const float*)f, (float*)field, n, layout); break;
        case 1: k_macro<StF16, float><<<blocks, 256, 0, st>>>((const uint16_t*)f, (float*)field, n, layout); break;
        case 2: k_macro<StBF16, float><<<blocks, 256, 0, st>>>((const uint16_t*)f, (float*)field, n, layout); break;
        case 3: k_macro<StF64, double><<<blocks, 256, 0, st>>>((const double*)f, (double*)field, n, layout); break;
        default: return cudaErrorInvalidValue;
    }
    note_launch();
    return cudaGetLastError();
}

// ---- energy / enstrophy / mass ---------------------------------------------------------------------
// Per cell: 1/2|u|^2, 1/2|curl u|^2 with central differences (periodic), rho; a float field's terms
// in double-float (diag_terms.cuh), an FP64 field's in FP64; sums in FP64.  Each thread walks a fixed
// grid-stride sequence of cells, blocks reduce in a fixed tree, and one block sums the block partials
// in a fixed order, so the result is the same on every run.

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <class FT, bool FLOAT_DIFF>
__global__ void __launch_bounds__(kDiagThreads) k_diag_field(const FT* __restrict__ F, int n,
                                                             double* __restrict__ partials) {
    const long long cells = (long long)n * n * n;
    double e = 0.0, ens = 0.0, mass = 0.0;
    if constexpr (sizeof(FT) == 4) {  // float fields: per-cell terms in double-float (diag_terms.cuh)
        dterm::Acc acc;
        for (dterm::CellWalk w((long long)blockIdx.x * kDiagThreads + threadIdx.x, (long long)gridDim.x * kDiagThreads, n);
             w.valid(); w.next()) {
            dterm::FF ce, cens;
            float rho;
            dterm::cell_terms<FLOAT_DIFF, true>(F, n, w.i, w.j, w.k, ce, cens, rho);  // fields from cudaMalloc
            acc.add_cell(ce, cens, rho);
        }
        acc.flush();
        e = acc.de;
        ens = acc.dens;
        mass = acc.dmass;
    } else {  // FP64 fields (FP64 storage): per-cell terms in FP64
        for (long long c = (long long)blockIdx.x * kDiagThreads + threadIdx.x; c < cells;
             c += (long long)gridDim.x * kDiagThreads) {
            int i, j, k;
            cell_ijk(c, n, i, j, k);
            const int ip = i + 1 == n ? 0 : i + 1, im = i == 0 ? n - 1 : i - 1;
            const int jp = j + 1 == n ? 0 : j + 1, jm = j == 0 ? n - 1 : j - 1;
            const int kp = k + 1 == n ? 0 : k + 1, km = k == 0 ? n - 1 : k - 1;
            auto at = [&](int a, int b, int cc, int comp) -> double {
                return double(F[(((size_t)cc * n + b) * n + a) * 4 + comp]);
            };
            const double rho = double(F[c * 4 + 0]);
            const double u = double(F[c * 4 + 1]), v = double(F[c * 4 + 2]), w = double(F[c * 4 + 3]);
            const double dudy = (at(i, jp, k, 1) - at(i, jm, k, 1)) * 0.5, dudz = (at(i, j, kp, 1) - at(i, j, km, 1)) * 0.5;
            const double dvdx = (at(ip, j, k, 2) - at(im, j, k, 2)) * 0.5, dvdz = (at(i, j, kp, 2) - at(i, j, km, 2)) * 0.5;
            const double dwdx = (at(ip, j, k, 3) - at(im, j, k, 3)) * 0.5, dwdy = (at(i, jp, k, 3) - at(i, jm, k, 3)) * 0.5;
            const double ox = dwdy - dvdz, oy = dudz - dwdx, oz = dvdx - dudy;
            e += 0.5 * (u * u + v * v + w * w);
            ens += 0.5 * (ox * ox + oy * oy + oz * oz);
            mass += rho;
        }
    }
    __shared__ double sh[3][kDiagThreads / 32];
    e = warp_sum(e);
    ens = warp_sum(ens);
    mass = warp_sum(mass);
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        sh[0][wid] = e;
        sh[1][wid] = ens;
        sh[2][wid] = mass;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double t = 0.0;
        for (int i = 0; i < kDiagThreads / 32; ++i) t += sh[threadIdx.x][i];
        partials[blockIdx.x * 3 + threadIdx.x] = t;
    }
}

// Sum `nparts` partial triples in a fixed order and scale by 1/cells.  err (optional): the error word
// of the kernel that wrote the partials, copied to *flag_out (when given) and cleared for the next one.
__global__ void __launch_bounds__(256) k_diag_finish(const double* __restrict__ partials, int nparts,
                                                     double inv_cells, double* __restrict__ out,
                                                     int* __restrict__ err = nullptr,
                                                     double* __restrict__ flag_out = nullptr) {
    double a[3] = {0.0, 0.0, 0.0};
    for (int p = threadIdx.x; p < nparts; p += 256) {
        a[0] += partials[p * 3 + 0];
        a[1] += partials[p * 3 + 1];
        a[2] += partials[p * 3 + 2];
    }
    __shared__ double sh[3][8];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const double t = warp_sum(a[k]);
        if (lane == 0) sh[k][wid] = t;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double t = 0.0;
        for (int i = 0; i < 8; ++i) t += sh[threadIdx.x][i];
        out[threadIdx.x] = t * inv_cells;
    }
    if (threadIdx.x == 0 && err) {
        if (flag_out) *flag_out = double(*err);
        *err = 0;
    }
}

// ---- energy / enstrophy / mass straight from the populations ---------------------------------------
// The float storages' diagnostic without a macro field in HBM (k_macro writes 16 B per cell that
// k_diag_field reads back with its neighbours).  A CTA takes a tile of kPopTx x kPopTy cells of the
// x-y plane and marches it along z over a chunk of planes, reading each cell's 19 populations once
// per plane.  A thread owns two x-adjacent cells (one 8-byte FP32 or 4-byte 16-bit load per
// population); the tile's one-cell halo in x and y is loaded too (its populations come mostly from
// L2: the neighbouring tiles' CTAs run beside it over the same planes).  The velocities of a plane
// land in a ring of three planes in shared memory, the z neighbours of a thread's own cells stay in
// its registers, and once plane z+1 is in, the tile's cells add the terms of plane z.  The planes
// are handed over by a split barrier: a warp arrives on an mbarrier once its velocities of plane g
// are in the ring and then waits for plane g-1 only, so no warp waits for the slowest warp of the
// plane it has just written; a ring of four planes keeps a slot from being rewritten while a slow
// warp still reads it (a warp writing plane g has seen every warp arrive for plane g-2, after its
// terms of plane g-3, the slot's last reader).  Every wait is bounded: past kPopWaitNs the warp
// sets the CTA's abort flag, every warp leaves at its next wait, the CTA's partials become NaN and
// the error word is set.  rho and u
// come from cell_macro (k_macro's arithmetic) and the velocity differences are taken in float, as in
// the two-pass path, so each cell's terms are the same numbers; dterm::CellSums adds them (to
// ~1e-13 of the sums) in a fixed order: items dealt to CTAs in a fixed order, fixed trees.  The next
// plane's loads are issued before the current plane's terms, so they are in flight across the
// wait.  One 608-thread CTA per SM (96 registers) with this tile measured faster than two 336-thread
// CTAs of 64 x 8 (a quarter of the loads in the halo, spills at 80 registers).
constexpr int kPopTx = 64, kPopTy = 16;
constexpr int kPopCols = kPopTx + 4;                          // x0-2 .. x0+kPopTx+1: whole pairs
constexpr int kPopRows = kPopTy + 2;                          // y0-1 .. y0+kPopTy
constexpr int kPopInner = kPopTx / 2 * kPopTy;                // threads on the tile's own pairs
constexpr int kPopThreads = kPopInner + kPopTx + 2 * kPopTy;  // + the rows y0-1, y0+kPopTy, the x pairs
constexpr int kPopWarps = kPopThreads / 32;
constexpr int kPopSlots = 4;
constexpr size_t kPopRingBytes = sizeof(float) * kPopSlots * 3 * kPopRows * kPopCols;  // 58,752 B, dynamic
constexpr unsigned long long kPopWaitNs = 2000000000ull;  // a plane hand-over takes microseconds

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long* b, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(unsigned long long* b) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(smem_u32(b))
                 : "memory");
}
__device__ __forceinline__ bool mbar_done(unsigned long long* b, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(b)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ unsigned long long pop_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Warp-collective (every lane calls it): true once the phase of parity `parity` of *b has completed;
// false, the same in every lane, when *abort is set or the wait outlives kPopWaitNs (then it sets it).
__device__ __forceinline__ bool pop_wait(unsigned long long* b, unsigned parity, volatile int* abort) {
    unsigned long long t0 = 0;
    for (;;) {
        const bool ok = mbar_done(b, parity);
        if (__all_sync(0xffffffffu, ok)) return true;
        bool bad = *abort != 0;
        if (!bad) {
            const unsigned long long t = pop_ns();
            if (t0 == 0) t0 = t;
            else bad = t - t0 > kPopWaitNs;
        }
        if (__any_sync(0xffffffffu, bad)) {
            *abort = 1;
            return false;
        }
    }
}

// the 19 population arrays of a cube, in the order the kernel reads them (layout 2 permuted here)
template <class RAW>
struct PopPtrs {
    const RAW* q[Q];
};

template <class RAW> struct PopPair;
template <> struct PopPair<float> {
    using word = float2;
    __device__ static __forceinline__ float lo(word w) { return w.x; }
    __device__ static __forceinline__ float hi(word w) { return w.y; }
    __device__ static __forceinline__ word make(float a, float b) { return make_float2(a, b); }
};
template <> struct PopPair<uint16_t> {
    using word = unsigned int;  // the cell at the lower address in the low half
    __device__ static __forceinline__ uint16_t lo(word w) { return (uint16_t)(w & 0xffffu); }
    __device__ static __forceinline__ uint16_t hi(word w) { return (uint16_t)(w >> 16); }
    __device__ static __forceinline__ word make(uint16_t a, uint16_t b) { return (unsigned)a | ((unsigned)b << 16); }
};

// the two cells of a pair word in the collision type: both halves of a 16-bit pair in one conversion
template <class ST>
__device__ __forceinline__ void pop_unpack(typename PopPair<typename ST::raw>::word w, float& a, float& b) {
    if constexpr (ST::id == 1) {
        const float2 t = __half22float2(*reinterpret_cast<const __half2*>(&w));
        a = t.x;
        b = t.y;
    } else if constexpr (ST::id == 2) {
        const float2 t = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&w));
        a = t.x;
        b = t.y;
    } else {
        a = ST::load(PopPair<typename ST::raw>::lo(w));
        b = ST::load(PopPair<typename ST::raw>::hi(w));
    }
}

// SHIFTED: the in-place layout after an even step count (population q of cell x at [q][x + c_q]).
template <class ST, bool SHIFTED>
__global__ void __launch_bounds__(kPopThreads, 1)
    k_diag_pop(const PopPtrs<typename ST::raw> P, int n, int ntx, int ntiles, int zc, int items,
               double* __restrict__ partials, int* __restrict__ err) {
    using RAW = typename ST::raw;
    using PP = PopPair<RAW>;
    using W = typename PP::word;
    extern __shared__ __align__(16) float pop_ring[];
    auto ring = reinterpret_cast<float(*)[3][kPopRows][kPopCols]>(pop_ring);  // [slot][u, v, w][row][col]
    __shared__ unsigned long long mb[2];  // plane g complete: mb[g & 1], phase g >> 1
    __shared__ int abort_flag;
    volatile int* abort = &abort_flag;
    const int t = threadIdx.x, lane = t & 31;
    if (t == 0) {
        mbar_init(&mb[0], kPopWarps);
        mbar_init(&mb[1], kPopWarps);
        abort_flag = 0;
    }
    __syncthreads();
    // this thread's pair (x, x+1) relative to the tile origin: the tile's pairs, the rows y = -1 and
    // y = kPopTy, then the pairs x = -2 and x = kPopTx of the tile's rows
    int ox, oy;
    if (t < kPopInner) {
        ox = 2 * (t % 32);
        oy = t / 32;
    } else if (t < kPopInner + kPopTx) {
        const int l = t - kPopInner;
        ox = 2 * (l % 32);
        oy = l < 32 ? -1 : kPopTy;
    } else {
        const int l = t - kPopInner - kPopTx;
        ox = l < kPopTy ? -2 : kPopTx;
        oy = l < kPopTy ? l : l - kPopTy;
    }
    const int row = oy + 1, col = ox + 2;
    auto wrap = [n](int a) {
        a %= n;
        return a < 0 ? a + n : a;
    };
    dterm::CellSums sums;
    unsigned g = 0;  // planes this CTA has walked, over all its items
    bool ok = true;
    for (int it = blockIdx.x; ok && it < items; it += gridDim.x) {
        const int zci = it / ntiles, tile = it - zci * ntiles;
        const int ty = tile / ntx, tx = tile - ty * ntx;
        const int x0 = tx * kPopTx, y0 = ty * kPopTy;
        const int zs = zci * zc, m = min(n, zs + zc) - zs;
        const int gx = wrap(x0 + ox), gy = wrap(y0 + oy);  // gx even (n is even), gx + 1 < n
        const bool valid = t < kPopInner && x0 + ox < n && y0 + oy < n;
        W a[Q];
        auto load_plane = [&](int z) {
            if (!SHIFTED) {
                const unsigned c = ((unsigned)z * n + gy) * n + gx;
#pragma unroll
                for (int q = 0; q < Q; ++q) a[q] = __ldg(reinterpret_cast<const W*>(P.q[q] + c));
            } else {
                const int zm = z == 0 ? n - 1 : z - 1, zp = z + 1 == n ? 0 : z + 1;
                const int gym = gy == 0 ? n - 1 : gy - 1, gyp = gy + 1 == n ? 0 : gy + 1;
                const int xm = gx == 0 ? n - 1 : gx - 1, xp2 = gx + 2 == n ? 0 : gx + 2;
#pragma unroll
                for (int q = 0; q < Q; ++q) {
                    const int zz = cz(q) > 0 ? zp : cz(q) < 0 ? zm : z;
                    const int yy = cy(q) > 0 ? gyp : cy(q) < 0 ? gym : gy;
                    const unsigned r = ((unsigned)zz * n + yy) * n;
                    const int xa = cx(q) > 0 ? gx + 1 : cx(q) < 0 ? xm : gx;        // cell gx + c_q
                    const int xb = cx(q) > 0 ? xp2 : cx(q) < 0 ? gx : gx + 1;       // cell gx + 1 + c_q
                    a[q] = PP::make(ld_one<RAW>(P.q[q] + r + xa), ld_one<RAW>(P.q[q] + r + xb));
                }
            }
        };
        load_plane(zs == 0 ? n - 1 : zs - 1);
        // the thread's two cells one plane back (u, v, w, rho) and two planes back (u, v)
        float u1a = 0.f, v1a = 0.f, w1a = 0.f, r1a = 0.f, u2a = 0.f, v2a = 0.f;
        float u1b = 0.f, v1b = 0.f, w1b = 0.f, r1b = 0.f, u2b = 0.f, v2b = 0.f;
        for (int r = 0; r <= m + 1; ++r, ++g) {  // plane zs - 1 + r, ring slot g & 3
            float rhoa, ua, va, wa, rhob, ub, vb, wb;
            {
                float fa[Q], fb[Q];
#pragma unroll
                for (int q = 0; q < Q; ++q) pop_unpack<ST>(a[q], fa[q], fb[q]);
                cell_macro<ST>(fa, rhoa, ua, va, wa);
                cell_macro<ST>(fb, rhob, ub, vb, wb);
            }
            if (r <= m) load_plane(zs + r == n ? 0 : zs + r);
            const int cur = g & 3;
            *reinterpret_cast<float2*>(&ring[cur][0][row][col]) = make_float2(ua, ub);
            *reinterpret_cast<float2*>(&ring[cur][1][row][col]) = make_float2(va, vb);
            *reinterpret_cast<float2*>(&ring[cur][2][row][col]) = make_float2(wa, wb);
            __syncwarp();
            if (lane == 0) mbar_arrive(&mb[g & 1]);
            if (g > 0 && !pop_wait(&mb[(g - 1) & 1], ((g - 1) >> 1) & 1, abort)) {
                ok = false;
                break;
            }
            if (r >= 2) {
                if (valid) {  // the terms of plane zs + r - 2, from the slot of plane g - 1
                    const int pv = (g - 1) & 3;
                    auto ld2 = [&](int comp, int rr, int cc) {
                        return *reinterpret_cast<const float2*>(&ring[pv][comp][rr][cc]);
                    };
                    const float2 vl = ld2(1, row, col - 2), vr = ld2(1, row, col + 2), vc = ld2(1, row, col);
                    const float2 wl = ld2(2, row, col - 2), wr = ld2(2, row, col + 2), wc = ld2(2, row, col);
                    const float2 un = ld2(0, row + 1, col), us = ld2(0, row - 1, col);
                    const float2 wn = ld2(2, row + 1, col), ws = ld2(2, row - 1, col);
                    // cell x: x-1 at col-1, x+1 at col+1; cell x+1: x at col, x+2 at col+2
                    sums.add_cell(u1a, v1a, w1a, r1a, vc.y, vl.y, wc.y, wl.y, un.x, us.x, wn.x, ws.x, ua, u2a, va, v2a);
                    sums.add_cell(u1b, v1b, w1b, r1b, vr.x, vc.x, wr.x, wc.x, un.y, us.y, wn.y, ws.y, ub, u2b, vb, v2b);
                }
            }
            u2a = u1a;
            v2a = v1a;
            u1a = ua;
            v1a = va;
            w1a = wa;
            r1a = rhoa;
            u2b = u1b;
            v2b = v1b;
            u1b = ub;
            v1b = vb;
            w1b = wb;
            r1b = rhob;
        }
    }
    sums.flush();
    double e = warp_sum(sums.de), ens = warp_sum(sums.dens), mass = warp_sum(sums.dmass);
    __shared__ double sh[3][kPopThreads / 32];
    const int wid = t >> 5;
    if (lane == 0) {
        sh[0][wid] = e;
        sh[1][wid] = ens;
        sh[2][wid] = mass;
    }
    __syncthreads();
    if (t < 3) {
        double sum = 0.0;
        for (int i = 0; i < kPopThreads / 32; ++i) sum += sh[t][i];
        partials[blockIdx.x * 3 + t] = *abort ? __longlong_as_double(0x7ff8000000000000ll) : sum;
    }
    if (t == 0 && *abort) atomicExch(err, 1);
}

template <class ST>
static cudaError_t launch_diag_pop_t(int layout, const void* f, int n, double* partials_dev, double* out_dev,
                                     int* err_dev, double* flag_out, cudaStream_t st) {
    using RAW = typename ST::raw;
    auto kern = layout == 1 ? k_diag_pop<ST, true> : k_diag_pop<ST, false>;
    PopPtrs<RAW> P;
    const size_t cells = (size_t)n * n * n;
    for (int q = 0; q < Q; ++q) P.q[q] = (const RAW*)f + (size_t)(layout == 2 ? opp(q) : q) * cells;
    int dev = 0, sms = 0, per_sm = 0;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kPopRingBytes);
    if (e == cudaSuccess) e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kPopThreads, kPopRingBytes);
    if (e != cudaSuccess) return e;
    const long long cap = std::min<long long>(kDiagBlocks, std::max(1, sms * std::max(1, per_sm)));
    const int ntx = (n + kPopTx - 1) / kPopTx, nty = (n + kPopTy - 1) / kPopTy, ntiles = ntx * nty;
    // z chunk: a CTA walks rounds x (chunk + 2 halo planes) planes, rounds = items over the resident
    // CTA slots; take the chunk with the fewest (the longest on a tie)
    int best_zc = n;
    long long best = -1;
    for (int zc = n; zc >= 4; --zc) {
        const long long items = (long long)ntiles * ((n + zc - 1) / zc);
        const long long planes = (items + cap - 1) / cap * (zc + 2);
        if (best < 0 || planes < best) {
            best = planes;
            best_zc = zc;
        }
    }
    const long long nzc = (n + best_zc - 1) / best_zc, items = (long long)ntiles * nzc;
    const int grid = (int)std::min(items, cap);
    kern<<<grid, kPopThreads, kPopRingBytes, st>>>(P, n, ntx, ntiles, best_zc, (int)items, partials_dev, err_dev);
    k_diag_finish<<<1, 256, 0, st>>>(partials_dev, grid, 1.0 / double(cells), out_dev, err_dev, flag_out);
    note_launch(2);
    return cudaGetLastError();
}

cudaError_t launch_diag_pop(int storage, int layout, const void* f, int n, double* partials_dev, double* out_dev,
                            double* flag_out, cudaStream_t st) {
    // pairs of cells at even x need an even n; cell indices are 32-bit
    if (n < 2 || n % 2 != 0 || n > 1600 || layout < 0 || layout > 2) return cudaErrorInvalidValue;
    int* err = diag_err_word(partials_dev);
    switch (storage) {
        case 0: return launch_diag_pop_t<StF32>(layout, f, n, partials_dev, out_dev, err, flag_out, st);
        case 1: return launch_diag_pop_t<StF16>(layout, f, n, partials_dev, out_dev, err, flag_out, st);
        case 2: return launch_diag_pop_t<StBF16>(layout, f, n, partials_dev, out_dev, err, flag_out, st);
        default: return cudaErrorInvalidValue;
    }
}

// ---- output fields: Q-criterion, speed, velocity ---------------------------------------------------
// Q = -1/2 sum_ab g_ab g_ba of the central-difference gradient g_cd = d u_c / d x_d (periodic), in FP64;
// FLOAT_DIFF takes each difference in the field's float first, as the uniform reference's host writer
// (src/tgv3d_uniform.cu:98-121); otherwise in double, as k_qspeed (src/tgv3d_amr.cu:553-564).
template <class FT, bool FLOAT_DIFF>
__global__ void __launch_bounds__(256) k_qspeed(const FT* __restrict__ F, int n, float* __restrict__ Qo,
                                               float* __restrict__ spd, float* __restrict__ vel) {
    const long long cells = (long long)n * n * n;
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cells) return;
    int i, j, k;
    cell_ijk(c, n, i, j, k);
    const int ip = i + 1 == n ? 0 : i + 1, im = i == 0 ? n - 1 : i - 1;
    const int jp = j + 1 == n ? 0 : j + 1, jm = j == 0 ? n - 1 : j - 1;
    const int kp = k + 1 == n ? 0 : k + 1, km = k == 0 ? n - 1 : k - 1;
    auto at = [&](int a, int b, int cc, int comp) -> FT { return F[(((size_t)cc * n + b) * n + a) * 4 + 1 + comp]; };
    auto dif = [&](FT a, FT b) -> double {
        if (FLOAT_DIFF) return double(FT(a - b)) * 0.5;
        return (double(a) - double(b)) * 0.5;
    };
    const double u = double(F[c * 4 + 1]), v = double(F[c * 4 + 2]), w = double(F[c * 4 + 3]);
    spd[c] = float(sqrt(u * u + v * v + w * w));
    if (vel) {
        vel[c * 3 + 0] = float(u);
        vel[c * 3 + 1] = float(v);
        vel[c * 3 + 2] = float(w);
    }
    double g[3][3];
#pragma unroll
    for (int cc = 0; cc < 3; ++cc) {
        g[cc][0] = dif(at(ip, j, k, cc), at(im, j, k, cc));
        g[cc][1] = dif(at(i, jp, k, cc), at(i, jm, k, cc));
        g[cc][2] = dif(at(i, j, kp, cc), at(i, j, km, cc));
    }
    double Q = 0.0;
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) Q -= 0.5 * g[a][b] * g[b][a];
    Qo[c] = float(Q);
}

cudaError_t launch_qspeed(bool field_is_double, bool float_diff, const void* field, int n, float* Q, float* speed,
                          float* vel, cudaStream_t st) {
    const long long cells = (long long)n * n * n;
    const unsigned blocks = (unsigned)((cells + 255) / 256);
    if (field_is_double) k_qspeed<double, false><<<blocks, 256, 0, st>>>((const double*)field, n, Q, speed, vel);
    else if (float_diff) k_qspeed<float, true><<<blocks, 256, 0, st>>>((const float*)field, n, Q, speed, vel);
    else k_qspeed<float, false><<<blocks, 256, 0, st>>>((const float*)field, n, Q, speed, vel);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_diag_field(bool field_is_double, bool float_diff, const void* field, int n,
                              double* partials_dev, double* out_dev, cudaStream_t st) {
    const long long cells = (long long)n * n * n;
    const int blocks = (int)std::min<long long>(kDiagBlocks, (cells + kDiagThreads - 1) / kDiagThreads);
    if (field_is_double) {
        k_diag_field<double, false><<<blocks, kDiagThreads, 0, st>>>((const double*)field, n, partials_dev);
    } else if (float_diff) {
        k_diag_field<float, true><<<blocks, kDiagThreads, 0, st>>>((const float*)field, n, partials_dev);
    } else {
        k_diag_field<float, false><<<blocks, kDiagThreads, 0, st>>>((const float*)field, n, partials_dev);
    }
    k_diag_finish<<<1, 256, 0, st>>>(partials_dev, blocks, 1.0 / double(cells), out_dev);
    note_launch(2);
    return cudaGetLastError();
}

}  // namespace jp
