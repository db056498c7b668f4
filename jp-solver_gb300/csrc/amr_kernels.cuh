// AMR level kernels: coarse step, prolongation sources ("prep"), ghost-shell fill, fine steps,
// restriction, seeding and migration, sensor and the composite macro field, for one storage format
// ST of lattice.cuh (pools, prolongation sources and ghost shells all in that format; FP32
// arithmetic).  Instantiated once per format by amr_kernels_<format>.cu.
// Reference: src/tgv3d_amr.cu:69-453, 514-536.  One CTA per block; a thread owns one cell (MB<=8)
// or several (MB=16), and the steps take 128, 256 or 512 threads per CTA at MB = 8 and 16.
// Arithmetic follows the reference's expressions so results agree within round-off; loop orders of
// the trilinear and the 8-child average are the reference's.  Per-block kernels keep their body in
// a d_* device function that takes the block index, shared by the single-solve kernel (k_*) and the
// batched kernels over many solves (kb_*).
#pragma once
#include "amr_common.cuh"
#include "amr_kernels.h"
#include "kernels.h"

namespace jp {
namespace amr {

#define CELL_LOOP(c) for (int c = threadIdx.x; c < G::MB3; c += G::TPB)

// ---- TGV initial state of the coarse grid (src/tgv3d_amr.cu:431-440) ---------------------------
template <int MB, class ST>
__global__ void __launch_bounds__(Geo<MB>::TPB) k_init(typename ST::raw* __restrict__ f, int cgx, double u0, double kf) {
    using G = Geo<MB>;
    const int b = blockIdx.x;
    const int bx = b % cgx, by = (b / cgx) % cgx, bz = b / (cgx * cgx);
    CELL_LOOP(cell) {
        const int i = cell % MB, j = (cell / MB) % MB, k = cell / (MB * MB);
        const double x = (bx * MB + i + 0.5) * kf, y = (by * MB + j + 0.5) * kf, z = (bz * MB + k + 0.5) * kf;
        const double ux = u0 * sin(x) * cos(y) * cos(z), uy = -u0 * cos(x) * sin(y) * cos(z);
        const double p = (u0 * u0 / 16.0) * (cos(2 * x) + cos(2 * y)) * (cos(2 * z) + 2.0), rho = 1.0 + 3.0 * p;
#pragma unroll
        for (int q = 0; q < Q; ++q)
            PoolIO<ST>::put_f(f + ((size_t)b * Q + q) * G::MB3 + cell, q, feq_ref(q, float(rho), float(ux), float(uy), 0.f));
    }
}

// ---- dense periodic coarse step (src/tgv3d_amr.cu:203-220) ---------------------------------------
template <int MB, class ST, int TPB>
__device__ __forceinline__ void d_step_l0(const typename ST::raw* __restrict__ fa,
                                                             typename ST::raw* __restrict__ fb, int cgx, float om, int blk) {
    using G = Geo<MB>;
    const int b = blk;
    const int bx = b % cgx, by = (b / cgx) % cgx, bz = b / (cgx * cgx);
    __shared__ int snb[27];  // periodic neighbour blocks (arithmetic only: no loads wait on the barrier)
    if (threadIdx.x < 27) {
        const int dx = threadIdx.x % 3 - 1, dy = (threadIdx.x / 3) % 3 - 1, dz = threadIdx.x / 9 - 1;
        snb[threadIdx.x] = (((bz + dz + cgx) % cgx) * cgx + (by + dy + cgx) % cgx) * cgx + (bx + dx + cgx) % cgx;
    }
    __syncthreads();
    for (int cell = threadIdx.x; cell < G::MB3; cell += TPB) {
        const int i = cell % MB, j = (cell / MB) % MB, k = cell / (MB * MB);
        float f[Q];
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            int e, sc;
            pull_src<MB>(q, i, j, k, e, sc);
            f[q] = PoolIO<ST>::g_of(JP_LDP(fa + ((size_t)snb[e] * Q + q) * G::MB3 + sc), q);
        }
        bgk_fast<true>(f, om);
#pragma unroll
        for (int q = 0; q < Q; ++q) fb[((size_t)b * Q + q) * G::MB3 + cell] = PoolIO<ST>::of_g(f[q], q);
    }
}
template <int MB, class ST, int TPB>
__global__ void __launch_bounds__(TPB, 1024 / TPB) k_step_l0(const typename ST::raw* __restrict__ fa,
                                                             typename ST::raw* __restrict__ fb, int cgx, float om) {
    d_step_l0<MB, ST, TPB>(fa, fb, cgx, om, (int)blockIdx.x);
}

// ---- prolongation sources on a cell list (src/tgv3d_amr.cu:160-171) ------------------------------
// Only the cells a fill can read are prepared.  A fill interpolates a ghost cell of a fine block
// from the 2x2x2 parent cells around it; the parent cell U holding the ghost is unrefined, the parent
// R of the fine cell next to it is refined, and every one of those corners lies within one cell of
// both (per axis).  So a fill reads only interface cells, whose 3x3x3 neighbourhood holds refined and
// unrefined cells; other cells of a skin block keep stale values nobody reads.  The interface cells
// are listed at each grid change (adapt_prep_list: the skin blocks with a change of refinement among
// their 27 neighbour blocks; adapt_prep_cells: their interface cells), and a thread prepares one
// listed cell; the threads tid, tid + nthreads, ... walk the list, whose length stays on the device.
template <int MB, class ST>
__device__ __forceinline__ void d_prep(const typename ST::raw* __restrict__ fin,
                                                      typename ST::raw* __restrict__ pr,
                                                      const int* __restrict__ cells, float nqs,
                                                      const int* __restrict__ nlim, const int* __restrict__ gate,
                                                      int tid, int nthreads) {
    using G = Geo<MB>;
    if (gate && __ldg(gate) == 0) return;  // no fine block of the next level has a ghost to fill
    const int n = __ldg(nlim);
    for (int idx = tid; idx < n; idx += nthreads) {
        const int v = __ldg(cells + idx);
        const int b = v / G::MB3, cell = v % G::MB3;
        float f[Q];
#pragma unroll
        for (int q = 0; q < Q; ++q) f[q] = PoolIO<ST>::f(fin + ((size_t)b * Q + q) * G::MB3 + cell, q);
        prep_cell(f, nqs);
#pragma unroll
        for (int q = 0; q < Q; ++q) PoolIO<ST>::put_f(pr + ((size_t)b * Q + q) * G::MB3 + cell, q, f[q]);
    }
}
template <int MB, class ST>
__global__ void __launch_bounds__(256) k_prep(const typename ST::raw* __restrict__ fin,
                                              typename ST::raw* __restrict__ pr, const int* __restrict__ cells,
                                              float nqs, const int* __restrict__ nlim, const int* __restrict__ gate) {
    d_prep<MB, ST>(fin, pr, cells, nqs, nlim, gate, (int)(blockIdx.x * blockDim.x + threadIdx.x),
                   (int)(gridDim.x * blockDim.x));
}

// SMs x resident CTAs per SM of `kernel` at `threads` threads and `smem` bytes of dynamic shared
// memory on the current device: the grid of the kernels that walk a list or a level.
template <class K>
static int resident_grid(K kernel, int threads, size_t smem) {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, smem);
    return (sms > 0 ? sms : 1) * (per > 0 ? per : 1);
}

// the prep kernel's grid
template <int MB, class ST>
static int prep_grid_cap() {
    static const int cap = resident_grid(k_prep<MB, ST>, 256, 0);
    return cap;
}

// Trilinear prolongation from a precomputed source (k_prep), one population at a time: the eight
// corners (pointer to the corner cell's population 0, weight) are found once per fine cell, then
// interp() sums q over them in corner order (src/tgv3d_amr.cu:122-144).  On the dense coarse grid
// every corner exists; on the scattered level 1 an absent corner has a null pointer and is dropped,
// and the sum is renormalised by the weights present (wsum < 0.999).
template <int MB, class ST>
__device__ __forceinline__ void corners_l0(const typename ST::raw* __restrict__ pr, int cgx, int N, int gfi, int gfj,
                                           int gfk, const typename ST::raw* (&p)[8], float (&w)[8]) {
    constexpr int MB3 = MB * MB * MB;
    int ib, jb, kb;
    float tx, ty, tz;
    tri_axis(gfi, ib, tx);
    tri_axis(gfj, jb, ty);
    tri_axis(gfk, kb, tz);
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const int di = c & 1, dj = (c >> 1) & 1, dk = c >> 2;
        w[c] = (di ? tx : 1 - tx) * (dj ? ty : 1 - ty) * (dk ? tz : 1 - tz);
        const int ci = wrap1(ib + di, N), cj = wrap1(jb + dj, N), ck = wrap1(kb + dk, N);
        const int cb = ((ck / MB) * cgx + cj / MB) * cgx + ci / MB;
        const int cc = ((ck % MB) * MB + cj % MB) * MB + ci % MB;
        p[c] = pr + (size_t)cb * Q * MB3 + cc;
    }
}
template <int MB, class ST>
__device__ __forceinline__ float corners_l1(const typename ST::raw* __restrict__ pr, const int* __restrict__ l1grid,
                                            int l1gx, int N1, int g2i, int g2j, int g2k,
                                            const typename ST::raw* (&p)[8], float (&w)[8]) {
    constexpr int MB3 = MB * MB * MB;
    int ib, jb, kb;
    float tx, ty, tz, wsum = 0.f;
    tri_axis(g2i, ib, tx);
    tri_axis(g2j, jb, ty);
    tri_axis(g2k, kb, tz);
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const int di = c & 1, dj = (c >> 1) & 1, dk = c >> 2;
        w[c] = (di ? tx : 1 - tx) * (dj ? ty : 1 - ty) * (dk ? tz : 1 - tz);
        const int ci = wrap1(ib + di, N1), cj = wrap1(jb + dj, N1), ck = wrap1(kb + dk, N1);
        const int lb = __ldg(l1grid + ((ck / MB) * l1gx + cj / MB) * l1gx + ci / MB);
        const int cc = ((ck % MB) * MB + cj % MB) * MB + ci % MB;
        p[c] = lb < 0 ? nullptr : pr + (size_t)lb * Q * MB3 + cc;
        if (lb >= 0) wsum += w[c];
    }
    return wsum;
}
// The pulled populations of one ghost cell (ghost_need: 5 on a face, 1 on an edge), interpolated
// together: all their corner loads are issued before any sum, each population summed in corner
// order as one at a time would be.  On an edge the spare slots repeat its one population and are not
// stored.
template <int MB, class ST, bool SPARSE>
__device__ __forceinline__ int interp_needed(const typename ST::raw* const (&p)[8], const float (&w)[8], unsigned need,
                                             int (&qs)[5], float (&v)[5]) {
    constexpr int MB3 = MB * MB * MB;
    const int nq = __popc(need);
#pragma unroll
    for (int s = 0; s < 5; ++s) {
        qs[s] = need ? __ffs(need) - 1 : qs[0];
        need &= need - 1u;
    }
    typename ST::raw r[8][5];
#pragma unroll
    for (int c = 0; c < 8; ++c)
#pragma unroll
        for (int s = 0; s < 5; ++s) r[c][s] = (!SPARSE || p[c]) ? JP_LDP(p[c] + qs[s] * MB3) : typename ST::raw(0);
#pragma unroll
    for (int s = 0; s < 5; ++s) {
        float acc = 0.f;
#pragma unroll
        for (int c = 0; c < 8; ++c)
            if (!SPARSE || p[c]) acc += w[c] * (ST::shifted ? wf(qs[s]) + ST::load(r[c][s]) : ST::load(r[c][s]));
        v[s] = acc;
    }
    return nq;
}

// Populations a fine step pulls from the ghost cell at (i, j, k) just outside the block: those whose
// velocity points from it into the block, c = -d in every direction d in which the cell lies
// outside (5 for a face cell, 1 for an edge cell).  The fills write only these; the other slots of
// the shell are never read.
template <int MB>
__device__ __forceinline__ unsigned ghost_need(int i, int j, int k) {
    const int dx = i < 0 ? -1 : (i >= MB ? 1 : 0), dy = j < 0 ? -1 : (j >= MB ? 1 : 0), dz = k < 0 ? -1 : (k >= MB ? 1 : 0);
    unsigned m = 0;
#pragma unroll
    for (int q = 1; q < Q; ++q)
        if ((dx == 0 || cx(q) == -dx) && (dy == 0 || cy(q) == -dy) && (dz == 0 || cz(q) == -dz)) m |= 1u << q;
    return m;
}

// ---- ghost shells (src/tgv3d_amr.cu:173-202) -------------------------------------------------------
// One thread per cell of the fill list: the shell cells (b * SH + t) of fine blocks whose neighbour
// slot is on another level, listed at each grid change (adapt_fill_list); the threads tid,
// tid + nthreads, ... walk the list, whose length stays on the device.  Shell cells next to a
// same-level block are never listed (the step gathers them from that block).
template <int MB, class ST>
__device__ __forceinline__ void d_fill_l1(const typename ST::raw* __restrict__ pr, typename ST::raw* __restrict__ gh,
                                                const int* __restrict__ pcb, const int* __restrict__ poct, int cgx, int N,
                                                const int* __restrict__ list, const int* __restrict__ nlim, int tid,
                                                int nthreads) {
    using G = Geo<MB>;
    const int n = __ldg(nlim);
    const int N1 = 2 * N;
    for (int idx = tid; idx < n; idx += nthreads) {
        const int v = __ldg(list + idx);
        const int fb = v / G::SH, t = v % G::SH;
        const int cb = __ldg(pcb + fb), oct = __ldg(poct + fb);
        const int cbx = cb % cgx, cby = (cb / cgx) % cgx, cbz = cb / (cgx * cgx);
        const int ox = cbx * 2 * MB + (oct & 1) * MB, oy = cby * 2 * MB + ((oct >> 1) & 1) * MB,
                  oz = cbz * 2 * MB + (oct >> 2) * MB;
        int i, j, k;
        shell_coord<MB>(t, i, j, k);
        const int gfi = wrap1(ox + i, N1), gfj = wrap1(oy + j, N1), gfk = wrap1(oz + k, N1);
        const typename ST::raw* p[8];
        float w[8];
        corners_l0<MB, ST>(pr, cgx, N, gfi, gfj, gfk, p, w);
        // only the populations a step pulls from this cell: five on a face, one on an edge
        int qs[5];
        float val[5];
        const int nq = interp_needed<MB, ST, false>(p, w, ghost_need<MB>(i, j, k), qs, val);
#pragma unroll
        for (int s = 0; s < 5; ++s)
            if (s < nq) PoolIO<ST>::put_f(gh + ((size_t)fb * Q + qs[s]) * G::SH + t, qs[s], val[s]);
    }
}
template <int MB, class ST>
__global__ void __launch_bounds__(256) k_fill_l1(const typename ST::raw* __restrict__ pr, typename ST::raw* __restrict__ gh,
                                                const int* __restrict__ pcb, const int* __restrict__ poct, int cgx, int N,
                                                const int* __restrict__ list, const int* __restrict__ nlim) {
    d_fill_l1<MB, ST>(pr, gh, pcb, poct, cgx, N, list, nlim, (int)(blockIdx.x * blockDim.x + threadIdx.x),
                      (int)(gridDim.x * blockDim.x));
}

template <int MB, class ST>
__device__ __forceinline__ void d_fill_l2(const typename ST::raw* __restrict__ pr, typename ST::raw* __restrict__ gh,
                                                const int* __restrict__ l2pl1, const int* __restrict__ l2oct,
                                                const int* __restrict__ f1pos, const int* __restrict__ l1grid, int l1gx, int N1,
                                                const int* __restrict__ list, const int* __restrict__ nlim, int tid,
                                                int nthreads) {
    using G = Geo<MB>;
    const int n = __ldg(nlim);
    const int N2 = 2 * N1;
    for (int idx = tid; idx < n; idx += nthreads) {
        const int v = __ldg(list + idx);
        const int b = v / G::SH, t = v % G::SH;
        const int pl1 = __ldg(l2pl1 + b), oct = __ldg(l2oct + b);
        const int pp = __ldg(f1pos + pl1), px = pp % l1gx, py = (pp / l1gx) % l1gx, pz = pp / (l1gx * l1gx);
        const int ox = px * 2 * MB + (oct & 1) * MB, oy = py * 2 * MB + ((oct >> 1) & 1) * MB,
                  oz = pz * 2 * MB + (oct >> 2) * MB;
        int i, j, k;
        shell_coord<MB>(t, i, j, k);
        const int g2i = wrap1(ox + i, N2), g2j = wrap1(oy + j, N2), g2k = wrap1(oz + k, N2);
        const typename ST::raw* p[8];
        float w[8];
        const float wsum = corners_l1<MB, ST>(pr, l1grid, l1gx, N1, g2i, g2j, g2k, p, w);
        const bool renorm = wsum > 0.f && wsum < 0.999f;
        const float inv = renorm ? 1.f / wsum : 1.f;
        int qs[5];
        float val[5];
        const int nq = interp_needed<MB, ST, true>(p, w, ghost_need<MB>(i, j, k), qs, val);
#pragma unroll
        for (int s = 0; s < 5; ++s)
            if (s < nq) PoolIO<ST>::put_f(gh + ((size_t)b * Q + qs[s]) * G::SH + t, qs[s], renorm ? val[s] * inv : val[s]);
    }
}
template <int MB, class ST>
__global__ void __launch_bounds__(256) k_fill_l2(const typename ST::raw* __restrict__ pr, typename ST::raw* __restrict__ gh,
                                                const int* __restrict__ l2pl1, const int* __restrict__ l2oct,
                                                const int* __restrict__ f1pos, const int* __restrict__ l1grid, int l1gx, int N1,
                                                const int* __restrict__ list, const int* __restrict__ nlim) {
    d_fill_l2<MB, ST>(pr, gh, l2pl1, l2oct, f1pos, l1grid, l1gx, N1, list, nlim,
                      (int)(blockIdx.x * blockDim.x + threadIdx.x), (int)(gridDim.x * blockDim.x));
}

// the fills' grid
template <int MB, class ST, int LEVEL>
static int fill_grid_cap() {
    static const int cap = LEVEL == 1 ? resident_grid(k_fill_l1<MB, ST>, 256, 0) : resident_grid(k_fill_l2<MB, ST>, 256, 0);
    return cap;
}

// Restriction of one fine block, staged in shared memory as sf[q * MB^3 + cell] after its last
// substep, into the octant `oct` of its parent block: each covered parent cell becomes
// feq + nqi*regularize(avg - feq) of its 8 children, summed in the reference's dk, dj, di order
// (k_restrict_L1/L2, src/tgv3d_amr.cu:275-298, 357-381).
template <int MB, class ST>
__device__ __forceinline__ void restrict_octant(const float* __restrict__ sf, typename ST::raw* __restrict__ parent, int oct,
                                                float nqi) {
    constexpr int H = MB / 2, MB3 = MB * MB * MB;
    for (int t = threadIdx.x; t < H * H * H; t += blockDim.x) {
        const int i = t % H, j = (t / H) % H, k = t / (H * H);
        float a[Q];
#pragma unroll
        for (int q = 0; q < Q; ++q) a[q] = 0.f;
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            const int di = c & 1, dj = (c >> 1) & 1, dk = c >> 2;
            const int sc = ((2 * k + dk) * MB + (2 * j + dj)) * MB + (2 * i + di);
#pragma unroll
            for (int q = 0; q < Q; ++q) a[q] += 0.125f * sf[q * MB3 + sc];
        }
        float rho, ux, uy, uz;
        moments(a, rho, ux, uy, uz);
        float fe[Q];
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            fe[q] = feq_ref(q, rho, ux, uy, uz);
            a[q] = a[q] - fe[q];
        }
        regularize(a);
        const int pc = (((oct >> 2) * H + k) * MB + (((oct >> 1) & 1) * H + j)) * MB + ((oct & 1) * H + i);
#pragma unroll
        for (int q = 0; q < Q; ++q) PoolIO<ST>::put_f(parent + q * MB3 + pc, q, fe[q] + nqi * a[q]);
    }
}

// ---- same-level neighbour tables -----------------------------------------------------------------
// nb[b*27 + e] = pool index of the same-level block at offset slot e (pull_src) of fine block b, or
// -1 where that neighbour is not on the block's level (its cells come from the ghost shell).  Built
// once per grid change, so the steps and fills read one table instead of walking the block tables.
template <class ST>
__global__ void k_nbtab_l1(int* __restrict__ nb, const int* __restrict__ pcb, const int* __restrict__ poct,
                           const int* __restrict__ ref0, const int* __restrict__ fof0, int cgx, int nf1) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 27LL * nf1) return;
    const int b = int(idx / 27), e = int(idx % 27);
    const int cb = pcb[b], oct = poct[b], l1gx = 2 * cgx;
    const int cbx = cb % cgx, cby = (cb / cgx) % cgx, cbz = cb / (cgx * cgx);
    const int dx = e % 3 - 1, dy = (e / 3) % 3 - 1, dz = e / 9 - 1;
    const int nx = (2 * cbx + (oct & 1) + dx + l1gx) % l1gx, ny = (2 * cby + ((oct >> 1) & 1) + dy + l1gx) % l1gx,
              nz = (2 * cbz + (oct >> 2) + dz + l1gx) % l1gx;
    const int ncb = ((nz >> 1) * cgx + (ny >> 1)) * cgx + (nx >> 1);
    nb[idx] = ref0[ncb] ? fof0[ncb] + ((nz & 1) * 4 + (ny & 1) * 2 + (nx & 1)) : -1;
}

template <class ST>
__global__ void k_nbtab_l2(int* __restrict__ nb, const int* __restrict__ l2pl1, const int* __restrict__ l2oct,
                           const int* __restrict__ f1pos, const int* __restrict__ l1grid, const int* __restrict__ ref1,
                           const int* __restrict__ fof1, int l1gx, int nf2) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 27LL * nf2) return;
    const int b = int(idx / 27), e = int(idx % 27);
    const int oct = l2oct[b], p = f1pos[l2pl1[b]], g2 = 2 * l1gx;
    const int px = p % l1gx, py = (p / l1gx) % l1gx, pz = p / (l1gx * l1gx);
    const int dx = e % 3 - 1, dy = (e / 3) % 3 - 1, dz = e / 9 - 1;
    const int nx = (2 * px + (oct & 1) + dx + g2) % g2, ny = (2 * py + ((oct >> 1) & 1) + dy + g2) % g2,
              nz = (2 * pz + (oct >> 2) + dz + g2) % g2;
    const int lb = l1grid[((nz >> 1) * l1gx + (ny >> 1)) * l1gx + (nx >> 1)];
    nb[idx] = (lb >= 0 && ref1[lb]) ? fof1[lb] + ((nz & 1) * 4 + (ny & 1) * 2 + (nx & 1)) : -1;
}

// ---- fine steps (src/tgv3d_amr.cu:241-274, 331-356) -----------------------------------------------
// One kernel for both fine levels: the neighbour table says, per offset, which pool block holds the
// pulled cells or that they come from the ghost shell.  TPB threads share the block's MB^3 cells.
// FUSE: this is the last substep before the restriction into the parent level, so the block also
// restricts itself into its parent octant (`parent`, `poct`), which saves re-reading the level from
// HBM in a separate restriction kernel.
template <int MB, class ST, int TPB, bool FUSE>
__device__ __forceinline__ void d_step_fine(const typename ST::raw* __restrict__ fa,
                                                               typename ST::raw* __restrict__ fbuf,
                                                               const typename ST::raw* __restrict__ gh,
                                                               const int* __restrict__ nbtab,
                                                               const int* __restrict__ parent,
                                                               const int* __restrict__ poct, float om,
                                                               typename ST::raw* __restrict__ parent_pool, float nqi,
                                                               const int* __restrict__ nlim, int blk) {
    static_assert(Geo<MB>::MB3 % TPB == 0, "cells must split evenly over the CTA");
    extern __shared__ float sf[];
    using G = Geo<MB>;
    if (nlim && (int)blk >= __ldg(nlim)) return;  // whole CTA: the barrier below stays uniform
    const int b = blk;
    const int* nbrow = nbtab + (size_t)b * 27;
    for (int cell = threadIdx.x; cell < G::MB3; cell += TPB) {
        const int i = cell % MB, j = (cell / MB) % MB, k = cell / (MB * MB);
        float f[Q];
        pull_cell<MB, ST, true>(fa, gh, nbrow, b, i, j, k, f);
        bgk_fast<true>(f, om);
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            const typename ST::raw o = PoolIO<ST>::of_g(f[q], q);
            fbuf[((size_t)b * Q + q) * G::MB3 + cell] = o;
            if (FUSE) sf[q * G::MB3 + cell] = PoolIO<ST>::f_of(o, q);  // restriction: unshifted, as stored
        }
    }
    if (FUSE) {
        __syncthreads();
        restrict_octant<MB, ST>(sf, parent_pool + (size_t)parent[b] * Q * G::MB3, poct[b], nqi);
    }
}
template <int MB, class ST, int TPB, bool FUSE>
__global__ void __launch_bounds__(TPB, 1024 / TPB) k_step_fine(const typename ST::raw* __restrict__ fa,
                                                               typename ST::raw* __restrict__ fbuf,
                                                               const typename ST::raw* __restrict__ gh,
                                                               const int* __restrict__ nbtab,
                                                               const int* __restrict__ parent,
                                                               const int* __restrict__ poct, float om,
                                                               typename ST::raw* __restrict__ parent_pool, float nqi,
                                                               const int* __restrict__ nlim) {
    d_step_fine<MB, ST, TPB, FUSE>(fa, fbuf, gh, nbtab, parent, poct, om, parent_pool, nqi, nlim, (int)blockIdx.x);
}

// ---- fine step on rows of four cells -----------------------------------------------------------------
// The same step as d_step_fine with a thread on four consecutive cells of a block row (MB = 8: two
// threads per row, 128 per block; MB = 16: four per row, 256 threads looping over the block).  For
// each population the source row (j - c_y, k - c_z) is read as one vector from the block or the
// neighbour block that holds it, or from the ghost shell, whose y/z faces and yz edges are contiguous
// in x.  The value a +-x pull needs from outside the four cells comes from the neighbouring thread of
// the row by a warp shuffle, or, at the block's x faces, from the x-neighbour block (or its ghost
// cells).  Per-cell arithmetic is d_step_fine's, so the results are the same bits.
template <class ST>
struct Vec4 {  // four stored values, one 16-byte (FP32) or 8-byte (16-bit) access
    using raw = typename ST::raw;
    using word = typename std::conditional<sizeof(raw) == 4, uint4, uint2>::type;
    union {
        word w;
        raw v[4];
    };
    __device__ __forceinline__ void load(const raw* p) { w = JP_LDP(reinterpret_cast<const word*>(p)); }
    __device__ __forceinline__ void store(raw* p) const { __stcs(reinterpret_cast<word*>(p), w); }
};
template <class RAW> __device__ __forceinline__ RAW shfl_by(RAW v, int d) {
    return d > 0 ? __shfl_down_sync(0xffffffffu, v, d) : __shfl_up_sync(0xffffffffu, v, -d);
}
template <> __device__ __forceinline__ uint16_t shfl_by<uint16_t>(uint16_t v, int d) {
    const unsigned u = v;
    return (uint16_t)(d > 0 ? __shfl_down_sync(0xffffffffu, u, d) : __shfl_up_sync(0xffffffffu, u, -d));
}

template <int MB>
struct RowGeo {
    static constexpr int SPR = MB / 4;                           // threads (segments) per row
    static constexpr int SEGS = MB * MB * SPR;                   // segments per block
    static constexpr int TPB = SEGS < 256 ? SEGS : 256;          // threads per CTA
};

// LIST: the blocks stepped are blist[0 .. *nlim) (a subset of the level, e.g. its skin blocks) instead
// of 0 .. *nlim.
template <int MB, class ST, bool FUSE, bool WALK, bool LIST = false>
__device__ __forceinline__ void d_step_fine_rows(const typename ST::raw* __restrict__ fa,
                                                 typename ST::raw* __restrict__ fbuf,
                                                 const typename ST::raw* __restrict__ gh,
                                                 const int* __restrict__ nbtab, const int* __restrict__ parent,
                                                 const int* __restrict__ poct, float om,
                                                 typename ST::raw* __restrict__ parent_pool, float nqi,
                                                 const int* __restrict__ nlim, int blk, int stride,
                                                 const int* __restrict__ blist = nullptr) {
    using G = Geo<MB>;
    using RG = RowGeo<MB>;
    using raw = typename ST::raw;
    constexpr int M = MB - 1, MB3 = G::MB3, SH = G::SH;
    static_assert(MB % 4 == 0 && 32 % RG::SPR == 0 && RG::SEGS % RG::TPB == 0, "row mapping");
    extern __shared__ float sf[];
    if (!WALK && blk >= __ldg(nlim)) return;  // whole CTA
    // WALK: blocks blk, blk + gridDim.x, ... (a resident grid walks the level; the loop bound is
    // CTA-uniform, so the barriers of the fused restriction stay uniform); else the one block blk.
    // The count is re-read from L1 and the stride is gridDim.x, so the loop holds one register.
    for (int bi = blk; bi < __ldg(nlim); bi += (WALK ? (int)gridDim.x : stride)) {
    const int b = LIST ? __ldg(blist + bi) : bi;
    const int* nbrow = nbtab + (size_t)b * 27;
    for (int seg = threadIdx.x; seg < RG::SEGS; seg += RG::TPB) {
        const int s = seg % RG::SPR, r = seg / RG::SPR, j = r % MB, k = r / MB, i0 = 4 * s;
        // 1. issue every load: 19 row vectors, and at the block's x faces the one value of each
        //    +-x population from the x-neighbour block or the ghost shell
        Vec4<ST> L[Q];
        raw E[Q];
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            const int lj = j - cy(q), lk = k - cz(q);
            const int ey = cy(q) > 0 ? (lj < 0 ? 0 : 1) : (cy(q) < 0 ? (lj > M ? 2 : 1) : 1);
            const int ez = cz(q) > 0 ? (lk < 0 ? 0 : 1) : (cz(q) < 0 ? (lk > M ? 2 : 1) : 1);
            const int erow = ez * 9 + ey * 3 + 1;
            const int rb = erow == 13 ? b : __ldg(nbrow + erow);
            const int rowc = ((lk & M) * MB + (lj & M)) * MB;  // cell of the row's x = 0 in its block
            if (rb >= 0) {
                L[q].load(fa + ((size_t)rb * Q + q) * MB3 + rowc + i0);
            } else {  // a y/z face or yz edge of the ghost shell: contiguous in x
                const int base = (ey != 1 && ez != 1)
                                     ? 6 * MB * MB + ((lj < 0 ? 0 : 1) + 2 * (lk < 0 ? 0 : 1)) * MB
                                     : (ey != 1 ? (lj < 0 ? 2 : 3) * MB * MB + lk * MB : (lk < 0 ? 4 : 5) * MB * MB + lj * MB);
                L[q].load(gh + ((size_t)b * Q + q) * SH + base + i0);
            }
            E[q] = raw(0);
            if (cx(q) != 0 && (cx(q) > 0 ? s == 0 : s == RG::SPR - 1)) {
                const int eb = __ldg(nbrow + ez * 9 + ey * 3 + (cx(q) > 0 ? 0 : 2));
                const int li = cx(q) > 0 ? -1 : MB;
                E[q] = eb >= 0 ? JP_LDP(fa + ((size_t)eb * Q + q) * MB3 + rowc + (li & M))
                               : JP_LDP(gh + ((size_t)b * Q + q) * SH + shell_index<MB>(li, lj, lk));
            }
        }
        // 2. inside the row the value comes from the neighbouring thread (all lanes shuffle)
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            if (cx(q) == 0) continue;
            const raw nb = cx(q) > 0 ? shfl_by<raw>(L[q].v[3], -1) : shfl_by<raw>(L[q].v[0], 1);
            if (!(cx(q) > 0 ? s == 0 : s == RG::SPR - 1)) E[q] = nb;
        }
        // 3. the pulled values of the four cells, converted once, and relaxed.  FP32: as two pairs of
        // cells (v, v + 1) in packed FP32 instructions (bgk_lanes: each cell gets the per-cell steps'
        // bits), which shortens the latency-bound FP32 rows.  The 16-bit rows, which hold five CTAs per
        // SM in fewer registers, relax cell by cell: in packed pairs they spilled and ran slower (also
        // one pair at a time with 4-byte stores).
        auto pulled = [&](int q, int v) -> raw {
            return cx(q) > 0 ? (v == 0 ? E[q] : L[q].v[v - 1]) : (cx(q) < 0 ? (v == 3 ? E[q] : L[q].v[v + 1]) : L[q].v[v]);
        };
        const int cell0 = (k * MB + j) * MB + i0;
        if constexpr (sizeof(raw) == 4) {
            float2 g[2][Q];
#pragma unroll
            for (int q = 0; q < Q; ++q) {
                g[0][q] = make_float2(PoolIO<ST>::g_of(pulled(q, 0), q), PoolIO<ST>::g_of(pulled(q, 1), q));
                g[1][q] = make_float2(PoolIO<ST>::g_of(pulled(q, 2), q), PoolIO<ST>::g_of(pulled(q, 3), q));
            }
            bgk_lanes<float2, true>(g[0], om);
            bgk_lanes<float2, true>(g[1], om);
#pragma unroll
            for (int q = 0; q < Q; ++q) {
                Vec4<ST> o;
                o.v[0] = PoolIO<ST>::of_g(g[0][q].x, q);
                o.v[1] = PoolIO<ST>::of_g(g[0][q].y, q);
                o.v[2] = PoolIO<ST>::of_g(g[1][q].x, q);
                o.v[3] = PoolIO<ST>::of_g(g[1][q].y, q);
                o.store(fbuf + ((size_t)b * Q + q) * MB3 + cell0);
                if (FUSE) {  // the restriction works on unshifted populations of the values as stored
#pragma unroll
                    for (int v = 0; v < 4; ++v) sf[q * MB3 + cell0 + v] = PoolIO<ST>::f_of(o.v[v], q);
                }
            }
        } else {
            float f[4][Q];
#pragma unroll
            for (int q = 0; q < Q; ++q)
#pragma unroll
                for (int v = 0; v < 4; ++v) f[v][q] = PoolIO<ST>::g_of(pulled(q, v), q);
#pragma unroll
            for (int v = 0; v < 4; ++v) bgk_fast<true>(f[v], om);
#pragma unroll
            for (int q = 0; q < Q; ++q) {
                Vec4<ST> o;
#pragma unroll
                for (int v = 0; v < 4; ++v) o.v[v] = PoolIO<ST>::of_g(f[v][q], q);
                o.store(fbuf + ((size_t)b * Q + q) * MB3 + cell0);
                if (FUSE) {
#pragma unroll
                    for (int v = 0; v < 4; ++v) sf[q * MB3 + cell0 + v] = PoolIO<ST>::f_of(o.v[v], q);
                }
            }
        }
    }
    if (FUSE) {
        __syncthreads();
        restrict_octant<MB, ST>(sf, parent_pool + (size_t)parent[b] * Q * G::MB3, poct[b], nqi);
        if (WALK && bi + (int)gridDim.x < __ldg(nlim)) __syncthreads();  // the next block stages into sf
    }
    if (!WALK) break;
    }
}
// CTAs per SM the rows kernels are built for: 16-bit rows hold half the bytes in flight per thread,
// so they trade registers for a fifth CTA
template <int MB, class ST>
constexpr int rows_min_blocks() { return (sizeof(typename ST::raw) == 2 ? 640 : 512) / RowGeo<MB>::TPB; }

template <int MB, class ST, bool FUSE, bool WALK>
__global__ void __launch_bounds__(RowGeo<MB>::TPB, (rows_min_blocks<MB, ST>())) k_step_fine_rows(
    const typename ST::raw* __restrict__ fa, typename ST::raw* __restrict__ fbuf, const typename ST::raw* __restrict__ gh,
    const int* __restrict__ nbtab, const int* __restrict__ parent, const int* __restrict__ poct, float om,
    typename ST::raw* __restrict__ parent_pool, float nqi, const int* __restrict__ nlim) {
    d_step_fine_rows<MB, ST, FUSE, WALK>(fa, fbuf, gh, nbtab, parent, poct, om, parent_pool, nqi, nlim,
                                         (int)blockIdx.x, (int)gridDim.x);
}

// The non-fused walking rows step over a block list (blist[0 .. *nlim)): part of a level stepped on
// its own, e.g. the level-1 blocks outside the skin beside the level-2 work that only the skin feeds.
template <int MB, class ST>
__global__ void __launch_bounds__(RowGeo<MB>::TPB, (rows_min_blocks<MB, ST>())) k_step_fine_rows_listed(
    const typename ST::raw* __restrict__ fa, typename ST::raw* __restrict__ fbuf, const typename ST::raw* __restrict__ gh,
    const int* __restrict__ nbtab, float om, const int* __restrict__ nlim, const int* __restrict__ blist) {
    d_step_fine_rows<MB, ST, false, true, true>(fa, fbuf, gh, nbtab, nullptr, nullptr, om, nullptr, 0.f, nlim,
                                               (int)blockIdx.x, (int)gridDim.x, blist);
}
template <int MB, class ST>
static int rows_listed_grid_cap() {
    static const int cap = resident_grid(k_step_fine_rows_listed<MB, ST>, RowGeo<MB>::TPB, 0);
    return cap;
}

// The grid of the walking rows kernels (resident CTAs): each CTA walks the level's blocks, so the
// start of a CTA (the block count, the first table reads) is paid once per CTA instead of once per
// block.
template <int MB, class ST, bool FUSE>
static int rows_grid_cap() {
    static const int cap = resident_grid(k_step_fine_rows<MB, ST, FUSE, true>, RowGeo<MB>::TPB,
                                         FUSE ? sizeof(float) * Q * Geo<MB>::MB3 : 0);
    return cap;
}

// ---- restriction (src/tgv3d_amr.cu:275-298, 357-381) -------------------------------------------------
// One CTA per refined parent block; each parent cell becomes feq + nqi*regularize(avg - feq) of the
// average of its 8 children (summed in the reference's dk, dj, di order).
template <int MB, class ST>
__device__ __forceinline__ void d_restrict(typename ST::raw* __restrict__ cf,
                                                          const typename ST::raw* __restrict__ ff,
                                                          const int* __restrict__ rl, const int* __restrict__ fof,
                                                          float nqi, const int* __restrict__ nlim, int blk) {
    using G = Geo<MB>;
    if (nlim && (int)blk >= __ldg(nlim)) return;
    const int cb = rl[blk];
    const int fbase = fof[cb];
    CELL_LOOP(cell) {
        const int lci = cell % MB, lcj = (cell / MB) % MB, lck = cell / (MB * MB);
        const int oct = (lck / G::HALF) * 4 + (lcj / G::HALF) * 2 + lci / G::HALF;
        const int fi0 = 2 * (lci % G::HALF), fj0 = 2 * (lcj % G::HALF), fk0 = 2 * (lck % G::HALF);
        const typename ST::raw* src = ff + (size_t)(fbase + oct) * Q * G::MB3;
        float a[Q];
#pragma unroll
        for (int q = 0; q < Q; ++q) a[q] = 0.f;
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            const int di = c & 1, dj = (c >> 1) & 1, dk = c >> 2;
            const int sc = ((fk0 + dk) * MB + (fj0 + dj)) * MB + (fi0 + di);
#pragma unroll
            for (int q = 0; q < Q; ++q) a[q] += 0.125f * PoolIO<ST>::f(src + q * G::MB3 + sc, q);
        }
        float rho, ux, uy, uz;
        moments(a, rho, ux, uy, uz);
        float fe[Q];
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            fe[q] = feq_ref(q, rho, ux, uy, uz);
            a[q] = a[q] - fe[q];
        }
        regularize(a);
#pragma unroll
        for (int q = 0; q < Q; ++q) PoolIO<ST>::put_f(cf + ((size_t)cb * Q + q) * G::MB3 + cell, q, fe[q] + nqi * a[q]);
    }
}
template <int MB, class ST>
__global__ void __launch_bounds__(Geo<MB>::TPB) k_restrict(typename ST::raw* __restrict__ cf,
                                                          const typename ST::raw* __restrict__ ff,
                                                          const int* __restrict__ rl, const int* __restrict__ fof,
                                                          float nqi, const int* __restrict__ nlim) {
    d_restrict<MB, ST>(cf, ff, rl, fof, nqi, nlim, (int)blockIdx.x);
}

// ---- on-the-fly prolongation for seeding and migration (src/tgv3d_amr.cu:70-118) ----------------
template <int MB, class ST>
__device__ __forceinline__ void prolong_l0(const typename ST::raw* __restrict__ cf, int cgx, int N, int gfi, int gfj, int gfk,
                                           float nqs, float (&out)[Q]) {
    constexpr int MB3 = MB * MB * MB;
    int ib, jb, kb;
    float tx, ty, tz;
    tri_axis(gfi, ib, tx);
    tri_axis(gfj, jb, ty);
    tri_axis(gfk, kb, tz);
#pragma unroll
    for (int q = 0; q < Q; ++q) out[q] = 0.f;
#pragma unroll 1
    for (int c = 0; c < 8; ++c) {
        const int di = c & 1, dj = (c >> 1) & 1, dk = c >> 2;
        const float wgt = (di ? tx : 1 - tx) * (dj ? ty : 1 - ty) * (dk ? tz : 1 - tz);
        const int ci = wrap1(ib + di, N), cj = wrap1(jb + dj, N), ck = wrap1(kb + dk, N);
        const int cb = ((ck / MB) * cgx + cj / MB) * cgx + ci / MB;
        const int cc = ((ck % MB) * MB + cj % MB) * MB + ci % MB;
        float f[Q];
#pragma unroll
        for (int q = 0; q < Q; ++q) f[q] = PoolIO<ST>::f(cf + ((size_t)cb * Q + q) * MB3 + cc, q);
        prep_cell(f, nqs);
#pragma unroll
        for (int q = 0; q < Q; ++q) out[q] += wgt * f[q];
    }
}
template <int MB, class ST>
__device__ __forceinline__ void prolong_l1(const typename ST::raw* __restrict__ f1, const int* __restrict__ l1grid, int l1gx,
                                           int N1, int g2i, int g2j, int g2k, float nqs, float (&out)[Q]) {
    constexpr int MB3 = MB * MB * MB;
    int ib, jb, kb;
    float tx, ty, tz, wsum = 0.f;
    tri_axis(g2i, ib, tx);
    tri_axis(g2j, jb, ty);
    tri_axis(g2k, kb, tz);
#pragma unroll
    for (int q = 0; q < Q; ++q) out[q] = 0.f;
#pragma unroll 1
    for (int c = 0; c < 8; ++c) {
        const int di = c & 1, dj = (c >> 1) & 1, dk = c >> 2;
        const float wgt = (di ? tx : 1 - tx) * (dj ? ty : 1 - ty) * (dk ? tz : 1 - tz);
        const int ci = wrap1(ib + di, N1), cj = wrap1(jb + dj, N1), ck = wrap1(kb + dk, N1);
        const int lb = __ldg(l1grid + ((ck / MB) * l1gx + cj / MB) * l1gx + ci / MB);
        if (lb < 0) continue;
        const int cc = ((ck % MB) * MB + cj % MB) * MB + ci % MB;
        float f[Q];
#pragma unroll
        for (int q = 0; q < Q; ++q) f[q] = PoolIO<ST>::f(f1 + ((size_t)lb * Q + q) * MB3 + cc, q);
        prep_cell(f, nqs);
        wsum += wgt;
#pragma unroll
        for (int q = 0; q < Q; ++q) out[q] += wgt * f[q];
    }
    if (wsum > 0.f && wsum < 0.999f) {
        const float inv = 1.f / wsum;
#pragma unroll
        for (int q = 0; q < Q; ++q) out[q] *= inv;
    }
}

// seed (old_ref == nullptr) or migrate level 1: a block whose parent was refined before copies its old
// payload, a new one is prolonged from the coarse level (src/tgv3d_amr.cu:299-308, 397-411)
template <int MB, class ST>
__global__ void __launch_bounds__(Geo<MB>::TPB) k_seed_l1(const typename ST::raw* __restrict__ oldf,
                                                         typename ST::raw* __restrict__ newf,
                                                         const typename ST::raw* __restrict__ c0, const int* __restrict__ pcb,
                                                         const int* __restrict__ poct, const int* __restrict__ old_ref0,
                                                         const int* __restrict__ old_fof0, int cgx, int N, float nqs) {
    using G = Geo<MB>;
    const int nfb = blockIdx.x;
    const int cb = pcb[nfb], oct = poct[nfb];
    const bool copy = old_ref0 != nullptr && old_ref0[cb];
    const int ofb = copy ? old_fof0[cb] + oct : 0;
    const int cbx = cb % cgx, cby = (cb / cgx) % cgx, cbz = cb / (cgx * cgx);
    CELL_LOOP(cell) {
        if (copy) {
#pragma unroll
            for (int q = 0; q < Q; ++q)
                newf[((size_t)nfb * Q + q) * G::MB3 + cell] = __ldg(oldf + ((size_t)ofb * Q + q) * G::MB3 + cell);
            continue;
        }
        const int i = cell % MB, j = (cell / MB) % MB, k = cell / (MB * MB);
        float out[Q];
        prolong_l0<MB, ST>(c0, cgx, N, cbx * 2 * MB + (oct & 1) * MB + i, cby * 2 * MB + ((oct >> 1) & 1) * MB + j,
                           cbz * 2 * MB + (oct >> 2) * MB + k, nqs, out);
#pragma unroll
        for (int q = 0; q < Q; ++q) PoolIO<ST>::put_f(newf + ((size_t)nfb * Q + q) * G::MB3 + cell, q, out[q]);
    }
}

// seed or migrate level 2, keyed by the level-1 grid position (src/tgv3d_amr.cu:382-393, 414-430)
template <int MB, class ST>
__global__ void __launch_bounds__(Geo<MB>::TPB) k_seed_l2(const typename ST::raw* __restrict__ oldf,
                                                         typename ST::raw* __restrict__ newf,
                                                         const typename ST::raw* __restrict__ f1, const int* __restrict__ l2pl1,
                                                         const int* __restrict__ l2oct, const int* __restrict__ f1pos,
                                                         const int* __restrict__ old_l1grid, const int* __restrict__ old_ref1,
                                                         const int* __restrict__ old_fof1, const int* __restrict__ l1grid,
                                                         int l1gx, int N1, float nqs) {
    using G = Geo<MB>;
    const int nfb = blockIdx.x;
    const int pl1 = l2pl1[nfb], oct = l2oct[nfb], p = f1pos[pl1];
    bool copy = false;
    int of2 = 0;
    if (old_l1grid != nullptr) {
        const int old_l1b = old_l1grid[p];
        copy = old_l1b >= 0 && old_ref1[old_l1b];
        if (copy) of2 = old_fof1[old_l1b] + oct;
    }
    const int px = p % l1gx, py = (p / l1gx) % l1gx, pz = p / (l1gx * l1gx);
    CELL_LOOP(cell) {
        if (copy) {
#pragma unroll
            for (int q = 0; q < Q; ++q)
                newf[((size_t)nfb * Q + q) * G::MB3 + cell] = __ldg(oldf + ((size_t)of2 * Q + q) * G::MB3 + cell);
            continue;
        }
        const int i = cell % MB, j = (cell / MB) % MB, k = cell / (MB * MB);
        float out[Q];
        prolong_l1<MB, ST>(f1, l1grid, l1gx, N1, px * 2 * MB + (oct & 1) * MB + i,
                           py * 2 * MB + ((oct >> 1) & 1) * MB + j, pz * 2 * MB + (oct >> 2) * MB + k, nqs, out);
#pragma unroll
        for (int q = 0; q < Q; ++q) PoolIO<ST>::put_f(newf + ((size_t)nfb * Q + q) * G::MB3 + cell, q, out[q]);
    }
}

// ---- refinement sensor (src/tgv3d_amr.cu:442-453) -----------------------------------------------
// Block max over cells of |f - feq|_2 / rho.  With `override_pos` set, block b takes the supplied
// value of its grid position instead (pos == nullptr: position = block index).
template <int MB, class ST>
__global__ void __launch_bounds__(Geo<MB>::TPB) k_sensor(const typename ST::raw* __restrict__ ff, float* __restrict__ d,
                                                        const float* __restrict__ override_val,
                                                        const int* __restrict__ pos) {
    using G = Geo<MB>;
    const int b = blockIdx.x;
    if (override_val) {
        if (threadIdx.x == 0) d[b] = override_val[pos ? pos[b] : b];
        return;
    }
    float m = -INFINITY;
    CELL_LOOP(cell) {
        float f[Q];
#pragma unroll
        for (int q = 0; q < Q; ++q) f[q] = PoolIO<ST>::f(ff + ((size_t)b * Q + q) * G::MB3 + cell, q);
        float rho, ux, uy, uz;
        moments(f, rho, ux, uy, uz);
        float s = 0.f;
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            const float d2 = f[q] - feq_ref(q, rho, ux, uy, uz);
            s += d2 * d2;
        }
        m = fmaxf(m, sqrtf(s) / rho);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    __shared__ float sm[32];
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        float r = sm[0];
        for (int w = 1; w < (G::TPB + 31) / 32; ++w) r = fmaxf(r, sm[w]);
        d[b] = r;
    }
}

// ---- composite macro field at 4*N0 (src/tgv3d_amr.cu:514-536) ----------------------------------
template <int MB, class ST>
__global__ void __launch_bounds__(256) k_composite(const typename ST::raw* __restrict__ c0,
                                                  const typename ST::raw* __restrict__ f1,
                                                  const typename ST::raw* __restrict__ f2, const int* __restrict__ ref1,
                                                  const int* __restrict__ fof1, const int* __restrict__ l1grid, int cgx,
                                                  int l1gx, int N2, float* __restrict__ F) {
    constexpr int MB3 = MB * MB * MB;
    const long long NN = (long long)N2 * N2 * N2;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= NN) return;
    int gi, gj, gk;
    if (NN <= 0xffffffffLL) {  // 32-bit division: a 64-bit one by a runtime N2 is a long sequence
        const unsigned u = unsigned(idx), n2 = unsigned(N2);
        gi = int(u % n2);
        gj = int((u / n2) % n2);
        gk = int(u / (n2 * n2));
    } else {
        gi = int(idx % N2);
        gj = int((idx / N2) % N2);
        gk = int(idx / ((long long)N2 * N2));
    }
    const int lb = l1grid[((gk / (2 * MB)) * l1gx + gj / (2 * MB)) * l1gx + gi / (2 * MB)];
    const typename ST::raw* src;
    size_t blk;
    int sc;
    if (lb >= 0 && ref1[lb]) {
        blk = fof1[lb] + (((gk % (2 * MB)) / MB) * 4 + ((gj % (2 * MB)) / MB) * 2 + (gi % (2 * MB)) / MB);
        sc = ((gk % MB) * MB + gj % MB) * MB + gi % MB;
        src = f2;
    } else if (lb >= 0) {
        const int g1i = gi / 2, g1j = gj / 2, g1k = gk / 2;
        blk = lb;
        sc = ((g1k % MB) * MB + g1j % MB) * MB + g1i % MB;
        src = f1;
    } else {
        const int c0i = gi / 4, c0j = gj / 4, c0k = gk / 4;
        blk = ((c0k / MB) * cgx + c0j / MB) * cgx + c0i / MB;
        sc = ((c0k % MB) * MB + c0j % MB) * MB + c0i % MB;
        src = c0;
    }
    float f[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) f[q] = PoolIO<ST>::f(src + (blk * Q + q) * MB3 + sc, q);
    float rho, ux, uy, uz;
    moments(f, rho, ux, uy, uz);
    F[idx * 4 + 0] = rho;
    F[idx * 4 + 1] = ux;
    F[idx * 4 + 2] = uy;
    F[idx * 4 + 3] = uz;
}

// ---- launchers ------------------------------------------------------------------------------------
#define POOL(p) reinterpret_cast<typename ST::raw*>(p)
#define CPOOL(p) reinterpret_cast<const typename ST::raw*>(p)

// the steps with TPB threads per CTA (the block's MB^3 cells split evenly)
template <int MB, class ST, int TPB>
static void launch_steps(const AmrLaunch& L, int op) {
    using G = Geo<MB>;
    if (op == OP_STEP_L0) {
        k_step_l0<MB, ST, TPB><<<L.nblocks, TPB, 0, L.st>>>(CPOOL(L.in), POOL(L.out), L.cgx, L.omega);
        return;
    }
    const int* parent = L.t0;  // pcb (level 1) or l2pl1 (level 2)
    if constexpr (MB <= 8) {
        if (L.out2) {
            k_step_fine<MB, ST, TPB, true><<<L.nblocks, TPB, sizeof(float) * Q * G::MB3, L.st>>>(
                CPOOL(L.in), POOL(L.out), CPOOL(L.aux), L.nbt, parent, L.t1, L.omega, POOL(L.out2), L.scale, L.nlim);
            return;
        }
    }
    k_step_fine<MB, ST, TPB, false><<<L.nblocks, TPB, 0, L.st>>>(CPOOL(L.in), POOL(L.out), CPOOL(L.aux), L.nbt,
                                                                 parent, L.t1, L.omega, nullptr, 0.f, L.nlim);
}

// the fine steps on rows of four cells (MB = 8, 16)
template <int MB, class ST>
static void launch_rows(const AmrLaunch& L) {
    using G = Geo<MB>;
    constexpr int T = RowGeo<MB>::TPB;
    // FP32 with the fused restriction walks only levels of up to 16 blocks per resident CTA (by
    // capacity): there the walk saves CTA starts and evens the tail; on longer levels its barrier per
    // block (the shared staging is reused) and its registers cost more than a CTA per block
    constexpr size_t sm = sizeof(float) * Q * G::MB3;
    if (L.out2) {
        const int cap = rows_grid_cap<MB, ST, true>();
        if (sizeof(typename ST::raw) == 4 && L.nblocks > 16 * cap)
            k_step_fine_rows<MB, ST, true, false><<<L.nblocks, T, sm, L.st>>>(
                CPOOL(L.in), POOL(L.out), CPOOL(L.aux), L.nbt, L.t0, L.t1, L.omega, POOL(L.out2), L.scale, L.nlim);
        else
            k_step_fine_rows<MB, ST, true, true><<<std::min(L.nblocks, cap), T, sm, L.st>>>(
                CPOOL(L.in), POOL(L.out), CPOOL(L.aux), L.nbt, L.t0, L.t1, L.omega, POOL(L.out2), L.scale, L.nlim);
    } else if (L.list) {  // the listed blocks only (L.nblocks: the list's capacity)
        k_step_fine_rows_listed<MB, ST><<<std::min(L.nblocks, rows_listed_grid_cap<MB, ST>()), T, 0, L.st>>>(
            CPOOL(L.in), POOL(L.out), CPOOL(L.aux), L.nbt, L.omega, L.nlim, L.list);
    } else {
        k_step_fine_rows<MB, ST, false, true><<<std::min(L.nblocks, rows_grid_cap<MB, ST, false>()), T, 0, L.st>>>(
            CPOOL(L.in), POOL(L.out), CPOOL(L.aux), L.nbt, L.t0, L.t1, L.omega, nullptr, 0.f, L.nlim);
    }
}

template <int MB, class ST>
static cudaError_t dispatch(const AmrLaunch& L, int op) {
    using G = Geo<MB>;
    const dim3 cta(G::TPB);
    const dim3 shl(G::SH < 256 ? ((G::SH + 31) / 32) * 32 : 256);
    switch (op) {
        case OP_INIT:
            k_init<MB, ST><<<L.nblocks, cta, 0, L.st>>>(POOL(L.out), L.cgx, L.u0, L.kf);
            break;
        case OP_STEP_L0:
        case OP_STEP_L1:
        case OP_STEP_L2: {
            const int tpb = L.tpb ? L.tpb : default_step_tpb(MB);
            if constexpr (MB == 4) {
                if (tpb != 64) return cudaErrorInvalidConfiguration;
                launch_steps<MB, ST, 64>(L, op);
            } else if (op != OP_STEP_L0 && (L.vec ? L.vec : default_step_vec(MB)) == 4) {
                // fused restriction with rows: the shared staging is sized for MB <= 8
                if (L.out2 && MB > 8) return cudaErrorInvalidConfiguration;
                if constexpr (MB <= 8) launch_rows<MB, ST>(L);
                else {
                    if (L.out2) return cudaErrorInvalidConfiguration;
                    launch_rows<MB, ST>(L);
                }
            } else {
                if (tpb == 128) launch_steps<MB, ST, 128>(L, op);
                else if (tpb == 256) launch_steps<MB, ST, 256>(L, op);
                else if (tpb == 512) launch_steps<MB, ST, 512>(L, op);
                else return cudaErrorInvalidConfiguration;
            }
            break;
        }
        case OP_NBTAB_L1:
            k_nbtab_l1<ST><<<(unsigned)((27LL * L.nblocks + 255) / 256), 256, 0, L.st>>>(L.iout, L.t0, L.t1, L.t2,
                                                                                      L.t3, L.cgx, L.nblocks);
            break;
        case OP_NBTAB_L2:
            k_nbtab_l2<ST><<<(unsigned)((27LL * L.nblocks + 255) / 256), 256, 0, L.st>>>(
                L.iout, L.t0, L.t1, L.t2, L.t3, L.t4, L.t5, L.l1gx, L.nblocks);
            break;
        case OP_PREP:
            k_prep<MB, ST><<<std::max(1, std::min((L.nblocks + 255) / 256, prep_grid_cap<MB, ST>())), 256, 0, L.st>>>(
                CPOOL(L.in), POOL(L.out), L.list, L.scale, L.nlim, L.t0);
            break;
        case OP_FILL_L1:
            k_fill_l1<MB, ST><<<std::max(1, std::min((L.nblocks + 255) / 256, fill_grid_cap<MB, ST, 1>())), 256, 0,
                                L.st>>>(CPOOL(L.in), POOL(L.out), L.t0, L.t1, L.cgx, L.n, L.list, L.nlim);
            break;
        case OP_FILL_L2:
            k_fill_l2<MB, ST><<<std::max(1, std::min((L.nblocks + 255) / 256, fill_grid_cap<MB, ST, 2>())), 256, 0,
                                L.st>>>(CPOOL(L.in), POOL(L.out), L.t0, L.t1, L.t2, L.t3, L.l1gx, L.n1, L.list, L.nlim);
            break;
        case OP_RESTRICT:
            k_restrict<MB, ST><<<L.nblocks, cta, 0, L.st>>>(POOL(L.out), CPOOL(L.in), L.list, L.t0, L.scale, L.nlim);
            break;
        case OP_SEED_L1:
            k_seed_l1<MB, ST><<<L.nblocks, cta, 0, L.st>>>(CPOOL(L.in), POOL(L.out), CPOOL(L.aux), L.t0, L.t1, L.t2,
                                                           L.t3, L.cgx, L.n, L.scale);
            break;
        case OP_SEED_L2:
            k_seed_l2<MB, ST><<<L.nblocks, cta, 0, L.st>>>(CPOOL(L.in), POOL(L.out), CPOOL(L.aux), L.t0, L.t1, L.t2,
                                                           L.t3, L.t4, L.t5, L.t6, L.l1gx, L.n1, L.scale);
            break;
        case OP_SENSOR:
            k_sensor<MB, ST><<<L.nblocks, cta, 0, L.st>>>(CPOOL(L.in), reinterpret_cast<float*>(L.out),
                                                          reinterpret_cast<const float*>(L.aux), L.t0);
            break;
        case OP_COMPOSITE: {
            const long long NN = (long long)L.n2 * L.n2 * L.n2;
            k_composite<MB, ST><<<(unsigned)((NN + 255) / 256), 256, 0, L.st>>>(
                CPOOL(L.in), CPOOL(L.aux), CPOOL(L.aux2), L.t0, L.t1, L.t2, L.cgx, L.l1gx, L.n2,
                reinterpret_cast<float*>(L.out));
            break;
        }
        case OP_WARM:  // launch shapes of the rows steps, preps and fills, found before any graph capture
            prep_grid_cap<MB, ST>();
            fill_grid_cap<MB, ST, 1>();
            fill_grid_cap<MB, ST, 2>();
            if constexpr (MB >= 8) {
                if constexpr (MB <= 8) rows_grid_cap<MB, ST, true>();
                rows_grid_cap<MB, ST, false>();
                rows_listed_grid_cap<MB, ST>();
            }
            return cudaGetLastError();
        default:
            return cudaErrorInvalidValue;
    }
    note_launch();
    return cudaGetLastError();
}

// ---- batched launches: one grid over the blocks of many solves ------------------------------------
// A CTA finds its member by bisection over the members' first CTAs and runs the stage's body on the
// member's block blockIdx.x - begin.
__device__ __forceinline__ int batch_member(const AmrBatch& B) {
    int lo = 0, hi = B.count - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (B.it[mid].begin <= (int)blockIdx.x) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

template <int MB, class ST, bool FUSE>
__global__ void __launch_bounds__(RowGeo<MB>::TPB, (rows_min_blocks<MB, ST>())) kb_step_rows(const __grid_constant__ AmrBatch B) {
    const AmrItem& it = B.it[batch_member(B)];
    const int blk = (int)blockIdx.x - it.begin;
    using raw = typename ST::raw;
    d_step_fine_rows<MB, ST, FUSE, false>((const raw*)it.in, (raw*)it.out, (const raw*)it.aux, it.nbt, it.t0, it.t1,
                                          it.omega, (raw*)it.out2, it.scale, it.nlim, blk, 0);
}

template <int MB, class ST, int TPB, bool FUSE, bool L0>
__global__ void __launch_bounds__(TPB, 1024 / TPB) kb_step(const __grid_constant__ AmrBatch B) {
    const AmrItem& it = B.it[batch_member(B)];
    const int blk = (int)blockIdx.x - it.begin;
    using raw = typename ST::raw;
    if constexpr (L0) {
        d_step_l0<MB, ST, TPB>((const raw*)it.in, (raw*)it.out, it.cgx, it.omega, blk);
    } else {
        d_step_fine<MB, ST, TPB, FUSE>((const raw*)it.in, (raw*)it.out, (const raw*)it.aux, it.nbt, it.t0, it.t1,
                                       it.omega, (raw*)it.out2, it.scale, it.nlim, blk);
    }
}

template <int MB, class ST, int OP>
__global__ void __launch_bounds__(OP == OP_FILL_L1 || OP == OP_FILL_L2 || OP == OP_PREP ? 256 : Geo<MB>::TPB)
    kb_cells(const __grid_constant__ AmrBatch B) {
    const AmrItem& it = B.it[batch_member(B)];
    const int blk = (int)blockIdx.x - it.begin;
    using raw = typename ST::raw;
    if constexpr (OP == OP_PREP) {
        d_prep<MB, ST>((const raw*)it.in, (raw*)it.out, it.list, it.scale, it.nlim, it.t0,
                       blk * (int)blockDim.x + (int)threadIdx.x, it.nct * (int)blockDim.x);
    } else if constexpr (OP == OP_FILL_L1) {
        d_fill_l1<MB, ST>((const raw*)it.in, (raw*)it.out, it.t0, it.t1, it.cgx, it.n, it.list, it.nlim,
                          blk * (int)blockDim.x + (int)threadIdx.x, it.nct * (int)blockDim.x);
    } else if constexpr (OP == OP_FILL_L2) {
        d_fill_l2<MB, ST>((const raw*)it.in, (raw*)it.out, it.t0, it.t1, it.t2, it.t3, it.l1gx, it.n1, it.list, it.nlim,
                          blk * (int)blockDim.x + (int)threadIdx.x, it.nct * (int)blockDim.x);
    } else {
        d_restrict<MB, ST>((raw*)it.out, (const raw*)it.in, it.list, it.t0, it.scale, it.nlim, blk);
    }
}

template <int MB, class ST, int TPB>
static void batch_steps(int op, bool fuse, const AmrBatch& B, cudaStream_t st) {
    using G = Geo<MB>;
    if (op == OP_STEP_L0) {
        kb_step<MB, ST, TPB, false, true><<<B.total, TPB, 0, st>>>(B);
        return;
    }
    if constexpr (MB <= 8) {
        if (fuse) {
            kb_step<MB, ST, TPB, true, false><<<B.total, TPB, sizeof(float) * Q * G::MB3, st>>>(B);
            return;
        }
    }
    kb_step<MB, ST, TPB, false, false><<<B.total, TPB, 0, st>>>(B);
}

template <int MB, class ST>
static void batch_rows(bool fuse, const AmrBatch& B, cudaStream_t st);

template <int MB, class ST>
static cudaError_t batch_dispatch(int op, int tpb, bool fuse, const AmrBatch& B, cudaStream_t st) {
    using G = Geo<MB>;
    const dim3 cta(G::TPB);
    const dim3 shl(G::SH < 256 ? ((G::SH + 31) / 32) * 32 : 256);
    switch (op) {
        case OP_STEP_L0:
        case OP_STEP_L1:
        case OP_STEP_L2: {
            const int t = tpb ? tpb : default_step_tpb(MB);
            if constexpr (MB == 4) {
                if (t != 64) return cudaErrorInvalidConfiguration;
                batch_steps<MB, ST, 64>(op, fuse, B, st);
            } else if (op != OP_STEP_L0 && (B.vec ? B.vec : default_step_vec(MB)) == 4) {
                if (fuse && MB > 8) return cudaErrorInvalidConfiguration;
                batch_rows<MB, ST>(fuse, B, st);
            } else {
                if (t == 128) batch_steps<MB, ST, 128>(op, fuse, B, st);
                else if (t == 256) batch_steps<MB, ST, 256>(op, fuse, B, st);
                else if (t == 512) batch_steps<MB, ST, 512>(op, fuse, B, st);
                else return cudaErrorInvalidConfiguration;
            }
            break;
        }
        case OP_PREP: kb_cells<MB, ST, OP_PREP><<<B.total, 256, 0, st>>>(B); break;
        case OP_FILL_L1: kb_cells<MB, ST, OP_FILL_L1><<<B.total, 256, 0, st>>>(B); break;
        case OP_FILL_L2: kb_cells<MB, ST, OP_FILL_L2><<<B.total, 256, 0, st>>>(B); break;
        case OP_RESTRICT: kb_cells<MB, ST, OP_RESTRICT><<<B.total, cta, 0, st>>>(B); break;
        default: return cudaErrorInvalidValue;
    }
    note_launch();
    return cudaGetLastError();
}

template <int MB, class ST>
static void batch_rows(bool fuse, const AmrBatch& B, cudaStream_t st) {
    using G = Geo<MB>;
    constexpr int T = RowGeo<MB>::TPB;
    if constexpr (MB <= 8) {
        if (fuse) {
            kb_step_rows<MB, ST, true><<<B.total, T, sizeof(float) * Q * G::MB3, st>>>(B);
            return;
        }
    }
    kb_step_rows<MB, ST, false><<<B.total, T, 0, st>>>(B);
}

template <class ST>
cudaError_t amr_batch_launch_st(int mb, int op, int tpb, bool fuse, const AmrBatch& B, cudaStream_t st) {
    if (B.count <= 0 || B.total <= 0) return cudaSuccess;
    switch (mb) {
        case 4: return batch_dispatch<4, ST>(op, tpb, fuse, B, st);
        case 8: return batch_dispatch<8, ST>(op, tpb, fuse, B, st);
        case 16: return batch_dispatch<16, ST>(op, tpb, fuse, B, st);
    }
    return cudaErrorInvalidValue;
}

// every launch of one storage format (amr_kernels_<format>.cu instantiates it)
template <class ST>
cudaError_t amr_launch_st(int mb, int op, const AmrLaunch& L) {
    switch (mb) {
        case 4: return dispatch<4, ST>(L, op);
        case 8: return dispatch<8, ST>(L, op);
        case 16: return dispatch<16, ST>(L, op);
    }
    return cudaErrorInvalidValue;
}

#undef POOL
#undef CPOOL
#undef CELL_LOOP

}  // namespace amr
}  // namespace jp
