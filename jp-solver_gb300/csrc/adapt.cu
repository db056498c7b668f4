// On-device adaptation pipeline: marking, exact-threshold selection, prefix sums, block-table
// scatter, 2:1 balance (deep mask) and skin lists.
//
// Reference: src/tgv3d_amr.cu:455-513 (kernels) and the Thrust calls of gpurce_init / gpurce_regrid
// (:722-815): an ascending thrust::sort to read the order statistic sorted[n - tgt], exclusive_scan
// for ranks, copy_if for the deep-sensor compaction and the skin lists.  Here the order statistic is
// a four-pass 8-bit radix select (same float-to-key order as a radix sort, so the same element), the
// scans and compactions are single-CTA warp-shuffle scans, and tgt is computed on the device, so a
// regrid needs no host round trip until the new block counts are read.  All results are integers
// or selected elements: bit-exact by construction.
#include "amr_common.cuh"
#include "amr_kernels.h"
#include "kernels.h"

namespace jp {
namespace amr {

constexpr int kScanThreads = 1024;

__device__ __forceinline__ unsigned float_key(float f) {
    const unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float key_float(unsigned k) {
    return __uint_as_float((k & 0x80000000u) ? (k ^ 0x80000000u) : ~k);
}

// Block-wide exclusive scan of one int per thread (kScanThreads threads); returns the prefix and
// the tile total.
__device__ __forceinline__ int block_exclusive_scan(int v, int& total) {
    __shared__ int wsum[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wsum[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int w = wsum[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        wsum[lane] = w;  // inclusive over warps
    }
    __syncthreads();
    const int warp_prefix = wid ? wsum[wid - 1] : 0;
    total = wsum[31];
    __syncthreads();
    return warp_prefix + x - v;
}

// rank[i] = sum_{j<i} flag[j]; returns the total (all threads)
__device__ int scan_into(const int* __restrict__ flag, int n, int* __restrict__ rank) {
    int carry = 0;
    for (int base = 0; base < n; base += kScanThreads) {
        const int i = base + threadIdx.x;
        const int v = i < n ? (flag[i] != 0) : 0;
        int tot;
        const int ex = block_exclusive_scan(v, tot);
        if (i < n) rank[i] = carry + ex;
        carry += tot;
    }
    return carry;
}

// ---- marking --------------------------------------------------------------------------------------
__global__ void k_mark_mode(int mode, int* __restrict__ ref, int cnb0, int cgx) {
    const int cb = blockIdx.x * blockDim.x + threadIdx.x;
    if (cb >= cnb0) return;
    ref[cb] = mode == 0 ? 1 : ((cb / (cgx * cgx) < cgx / 2) ? 1 : 0);  // k_setall / k_mark_slab
}

// Single-CTA exact threshold + mark (k_mark_thr / k_mark_ref1 with the sorted-copy threshold).
__global__ void __launch_bounds__(kScanThreads) k_threshold_mark(const float* __restrict__ sen,
                                                                const int* __restrict__ mask, int n, double frac,
                                                                int cap, int* __restrict__ ref,
                                                                AdaptCounts* __restrict__ counts, int which) {
    __shared__ unsigned hist[256];
    __shared__ unsigned s_prefix, s_pmask;
    __shared__ int s_k;
    int cnt = 0;
    for (int i = threadIdx.x; i < n; i += kScanThreads) cnt += mask ? (mask[i] != 0) : 1;
    int nm;
    block_exclusive_scan(cnt, nm);
    if (mask && threadIdx.x == 0) counts->ndeep = nm;
    if (nm == 0) {
        for (int i = threadIdx.x; i < n; i += kScanThreads) ref[i] = 0;
        return;
    }
    // tgt = min(cap, max(1, int(frac * nm)))  (src/tgv3d_amr.cu:728,746)
    int tgt = (int)(frac * (double)nm);
    tgt = tgt < 1 ? 1 : tgt;
    tgt = tgt < cap ? tgt : cap;
    if (threadIdx.x == 0) {
        s_prefix = 0u;
        s_pmask = 0u;
        s_k = nm - tgt;  // 0-based ascending rank of the threshold
    }
    __syncthreads();
    for (int pass = 0; pass < 4; ++pass) {
        const int shift = 24 - 8 * pass;
        for (int b = threadIdx.x; b < 256; b += kScanThreads) hist[b] = 0u;
        __syncthreads();
        const unsigned prefix = s_prefix, pmask = s_pmask;
        for (int i = threadIdx.x; i < n; i += kScanThreads) {
            if (mask && !mask[i]) continue;
            const unsigned key = float_key(sen[i]);
            if ((key & pmask) == prefix) atomicAdd(&hist[(key >> shift) & 255u], 1u);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            int k = s_k;
            unsigned b = 0;
            for (; b < 255u; ++b) {
                if ((int)hist[b] > k) break;
                k -= (int)hist[b];
            }
            s_k = k;
            s_prefix = prefix | (b << shift);
            s_pmask = pmask | (255u << shift);
        }
        __syncthreads();
    }
    const float thr = key_float(s_prefix);
    if (threadIdx.x == 0) {
        if (which == 0) counts->thr0 = thr;
        else counts->thr1 = thr;
    }
    for (int i = threadIdx.x; i < n; i += kScanThreads) {
        const bool in = mask ? (mask[i] != 0) : true;
        ref[i] = (in && sen[i] >= thr) ? 1 : 0;
    }
}

// k_deepmask (src/tgv3d_amr.cu:468-474): the six face neighbours of the level-1 grid position exist
__global__ void k_deepmask(const int* __restrict__ f1pos, const int* __restrict__ l1grid, int l1gx, int nf1,
                           int* __restrict__ deep) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nf1) return;
    const int p = f1pos[b], px = p % l1gx, py = (p / l1gx) % l1gx, pz = p / (l1gx * l1gx);
    const int xm = (px - 1 + l1gx) % l1gx, xp = (px + 1) % l1gx, ym = (py - 1 + l1gx) % l1gx, yp = (py + 1) % l1gx;
    const int zm = (pz - 1 + l1gx) % l1gx, zp = (pz + 1) % l1gx;
    int ok = l1grid[(pz * l1gx + py) * l1gx + xm] >= 0;
    ok &= l1grid[(pz * l1gx + py) * l1gx + xp] >= 0;
    ok &= l1grid[(pz * l1gx + ym) * l1gx + px] >= 0;
    ok &= l1grid[(pz * l1gx + yp) * l1gx + px] >= 0;
    ok &= l1grid[(zm * l1gx + py) * l1gx + px] >= 0;
    ok &= l1grid[(zp * l1gx + py) * l1gx + px] >= 0;
    deep[b] = ok;
}

// exclusive scan + k_scatter_L1 (src/tgv3d_amr.cu:476-486), one CTA
__global__ void __launch_bounds__(kScanThreads) k_build_l1(const int* __restrict__ ref0, int cnb0, int cgx, int l1gx,
                                                          int ng1, int cap1, int* __restrict__ rank, int* __restrict__ fof0,
                                                          int* __restrict__ rl0, int* __restrict__ pcb,
                                                          int* __restrict__ poct, int* __restrict__ l1grid,
                                                          int* __restrict__ f1pos, AdaptCounts* __restrict__ counts) {
    const int total = scan_into(ref0, cnb0, rank);
    if (threadIdx.x == 0) {
        counts->nref0 = total;
        counts->nf1 = 8 * total;
        if (8 * total > cap1) counts->err |= ADAPT_ERR_CAP1;
    }
    if (8 * total > cap1) return;  // nothing written: the caller keeps the previous tables
    for (int p = threadIdx.x; p < ng1; p += kScanThreads) l1grid[p] = -1;
    __syncthreads();
    for (int cb = threadIdx.x; cb < cnb0; cb += kScanThreads) {
        if (!ref0[cb]) {
            fof0[cb] = -1;
            continue;
        }
        const int r = rank[cb];
        fof0[cb] = 8 * r;
        rl0[r] = cb;
        const int cbx = cb % cgx, cby = (cb / cgx) % cgx, cbz = cb / (cgx * cgx);
        for (int oct = 0; oct < 8; ++oct) {
            const int fb = 8 * r + oct;
            const int pos = ((cbz * 2 + (oct >> 2)) * l1gx + cby * 2 + ((oct >> 1) & 1)) * l1gx + cbx * 2 + (oct & 1);
            pcb[fb] = cb;
            poct[fb] = oct;
            f1pos[fb] = pos;
            l1grid[pos] = fb;
        }
    }
}

__global__ void __launch_bounds__(kScanThreads) k_scan_l2(const int* __restrict__ ref1, int nf1, int* __restrict__ rank,
                                                         AdaptCounts* __restrict__ counts) {
    const int total = scan_into(ref1, nf1, rank);
    if (threadIdx.x == 0) {
        counts->nref1 = total;
        counts->nf2 = 8 * total;
    }
}

// k_scatter_L2 (src/tgv3d_amr.cu:488-494)
__global__ void k_scatter_l2(const int* __restrict__ ref1, const int* __restrict__ rank, int nf1, int cap2,
                             int* __restrict__ fof1, int* __restrict__ rl1, int* __restrict__ l2pl1,
                             int* __restrict__ l2oct, AdaptCounts* __restrict__ counts) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (counts->nf2 > cap2) {
        if (b == 0) counts->err |= ADAPT_ERR_CAP2;
        return;
    }
    if (b >= nf1) return;
    if (!ref1[b]) {
        fof1[b] = -1;
        return;
    }
    const int r = rank[b];
    fof1[b] = 8 * r;
    rl1[r] = b;
    for (int oct = 0; oct < 8; ++oct) {
        l2pl1[8 * r + oct] = b;
        l2oct[8 * r + oct] = oct;
    }
}

// skin flags (k_dilate_L0 / k_dilate_L1, src/tgv3d_amr.cu:502-513): flags[0..cnb0) level 0,
// flags[cnb0..cnb0+nf1) level 1
__global__ void k_dilate(const int* __restrict__ ref0, int cnb0, int cgx, const int* __restrict__ ref1,
                         const int* __restrict__ f1pos, const int* __restrict__ l1grid, int nf1, int l1gx,
                         int* __restrict__ flags) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < cnb0) {
        const int bx = t % cgx, by = (t / cgx) % cgx, bz = t / (cgx * cgx);
        int f = 0;
        for (int c = 0; c < 27 && !f; ++c) {
            const int nx = (bx + c % 3 - 1 + cgx) % cgx, ny = (by + (c / 3) % 3 - 1 + cgx) % cgx,
                      nz = (bz + c / 9 - 1 + cgx) % cgx;
            f = ref0[(nz * cgx + ny) * cgx + nx] != 0;
        }
        flags[t] = f;
    } else if (t < cnb0 + nf1) {
        const int b = t - cnb0;
        const int p = f1pos[b], px = p % l1gx, py = (p / l1gx) % l1gx, pz = p / (l1gx * l1gx);
        int f = 0;
        for (int c = 0; c < 27 && !f; ++c) {
            const int nx = (px + c % 3 - 1 + l1gx) % l1gx, ny = (py + (c / 3) % 3 - 1 + l1gx) % l1gx,
                      nz = (pz + c / 9 - 1 + l1gx) % l1gx;
            const int nb = l1grid[(nz * l1gx + ny) * l1gx + nx];
            f = nb >= 0 && ref1[nb];
        }
        flags[t] = f;
    }
}

// ordered compaction of the two flag ranges into the skin lists (copy_if over a counting iterator)
__global__ void __launch_bounds__(kScanThreads) k_compact_skins(const int* __restrict__ flags, int cnb0, int nf1,
                                                               int* __restrict__ skin0, int* __restrict__ skin1,
                                                               int* __restrict__ rest1, AdaptCounts* __restrict__ counts) {
    for (int part = 0; part < 2; ++part) {
        const int* fl = part == 0 ? flags : flags + cnb0;
        const int n = part == 0 ? cnb0 : nf1;
        int* out = part == 0 ? skin0 : skin1;
        int carry = 0;
        for (int base = 0; base < n; base += kScanThreads) {
            const int i = base + threadIdx.x;
            const int v = i < n ? fl[i] : 0;
            int tot;
            const int ex = block_exclusive_scan(v, tot);
            if (v) out[carry + ex] = i;
            else if (part == 1 && rest1 && i < n) rest1[i - carry - ex] = i;  // i minus the skins before it
            carry += tot;
        }
        if (threadIdx.x == 0) {
            if (part == 0) counts->n_skin0 = carry;
            else {
                counts->n_skin1 = carry;
                counts->n_rest1 = n - carry;
            }
        }
    }
}

__global__ void k_fill_int(int* __restrict__ p, int v, long long n) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        p[i] = v;
}

// Fill list of a fine level: the ghost-shell cells (faces and edges; the D3Q19 pulls never cross a
// corner) whose neighbour slot is on another level, as b * SH + shell cell.  CTA per block, the
// threads over its shell; warp-aggregated append, *count zero on entry, order not fixed.
template <int MB>
__global__ void k_fill_list(const int* __restrict__ nb, int* __restrict__ list, int* __restrict__ count) {
    constexpr int SH = Geo<MB>::SH;
    const int b = blockIdx.x;
    const int* row = nb + (size_t)b * 27;
    for (int base = 0; base < SH; base += blockDim.x) {  // uniform trip count: every lane meets the ballot
        const int t = base + threadIdx.x;
        bool need = false;
        if (t < SH) {
            int i, j, k;
            shell_coord<MB>(t, i, j, k);
            need = __ldg(row + shell_slot<MB>(i, j, k)) < 0;
        }
        const unsigned mask = __ballot_sync(0xffffffffu, need);
        if (!mask) continue;
        const int lane = threadIdx.x & 31;
        int at = 0;
        if (lane == 0) at = atomicAdd(count, __popc(mask));
        at = __shfl_sync(0xffffffffu, at, 0);
        if (need) list[at + __popc(mask & ((1u << lane) - 1u))] = b * SH + t;
    }
}

// Prep list of a level: the skin blocks with a change of refinement among their 27 neighbour blocks
// (periodic), as {block, mask of the refined ones}.  Level 0: blocks are positions of the dense grid
// of edge gx (pos null); level 1: pos[b] in the level-1 grid `grid`, an absent block unrefined.
__global__ void k_prep_list(const int* __restrict__ skin, const int* __restrict__ nskin_dev, const int* __restrict__ ref,
                            const int* __restrict__ pos, const int* __restrict__ grid, int gx,
                            int2* __restrict__ list, int* __restrict__ count) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    const int nskin = __ldg(nskin_dev);  // the skin count as the device holds it (grid: capacity)
    unsigned rm = 0;
    int b = 0;
    if (s < nskin) {
        b = skin[s];
        const int p = pos ? pos[b] : b;
        const int px = p % gx, py = (p / gx) % gx, pz = p / (gx * gx);
#pragma unroll 1
        for (int e = 0; e < 27; ++e) {
            const int nx = (px + e % 3 - 1 + gx) % gx, ny = (py + (e / 3) % 3 - 1 + gx) % gx, nz = (pz + e / 9 - 1 + gx) % gx;
            const int np = (nz * gx + ny) * gx + nx;
            const int nb = pos ? grid[np] : np;
            if (nb >= 0 && ref[nb] != 0) rm |= 1u << e;
        }
    }
    const bool need = rm != 0u && rm != (1u << 27) - 1u;
    const unsigned mask = __ballot_sync(0xffffffffu, need);
    if (!mask) return;
    const int lane = threadIdx.x & 31;
    int base = 0;
    if (lane == 0) base = atomicAdd(count, __popc(mask));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (need) list[base + __popc(mask & ((1u << lane) - 1u))] = make_int2(b, (int)rm);
}

// Interface cells of the blocks of a prep list {block, refined-neighbour mask}: the cells whose 3x3x3
// neighbourhood reaches refined and unrefined blocks, as b * mb^3 + cell.  CTA per entry (CTAs past
// *pcount return); warp-aggregated append, *ncells zero on entry.
__global__ void k_prep_cells(const int2* __restrict__ plist, const int* __restrict__ pcount, int mb,
                             int* __restrict__ cells, int* __restrict__ ncells) {
    if ((int)blockIdx.x >= *pcount) return;
    const int2 e = plist[blockIdx.x];
    const int b = e.x;
    const unsigned rm = (unsigned)e.y;
    const int mb3 = mb * mb * mb;
    for (int base = 0; base < mb3; base += blockDim.x) {  // uniform trip count: every lane meets the ballot
        const int cell = base + threadIdx.x;
        bool need = false;
        if (cell < mb3) {
            const int i = cell % mb, j = (cell / mb) % mb, k = cell / (mb * mb);
            // slots of the blocks the cell's neighbourhood reaches: per axis 0..2 (offset -1..1)
            const unsigned mx = (i == 0 ? 3u : (i == mb - 1 ? 6u : 2u)), my = (j == 0 ? 3u : (j == mb - 1 ? 6u : 2u)),
                           mz = (k == 0 ? 3u : (k == mb - 1 ? 6u : 2u));
            const unsigned plane = ((my & 1u) ? mx : 0u) | ((my & 2u) ? mx << 3 : 0u) | ((my & 4u) ? mx << 6 : 0u);
            const unsigned span = ((mz & 1u) ? plane : 0u) | ((mz & 2u) ? plane << 9 : 0u) | ((mz & 4u) ? plane << 18 : 0u);
            const unsigned sel = rm & span;
            need = sel != 0u && sel != span;
        }
        const unsigned mask = __ballot_sync(0xffffffffu, need);
        if (!mask) continue;
        const int lane = threadIdx.x & 31;
        int at = 0;
        if (lane == 0) at = atomicAdd(ncells, __popc(mask));
        at = __shfl_sync(0xffffffffu, at, 0);
        if (need) cells[at + __popc(mask & ((1u << lane) - 1u))] = b * mb3 + cell;
    }
}

// ---- host launchers --------------------------------------------------------------------------------
static inline unsigned grid_for(long long n, int t) { return (unsigned)((n + t - 1) / t); }

cudaError_t adapt_mark_mode(int mode, int* ref, int cnb0, int cgx, cudaStream_t st) {
    k_mark_mode<<<grid_for(cnb0, 256), 256, 0, st>>>(mode, ref, cnb0, cgx);
    note_launch();
    return cudaGetLastError();
}
cudaError_t adapt_threshold_mark(const float* sen, const int* mask, int n, double frac, int cap, int* ref,
                                 AdaptCounts* counts, int which, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_threshold_mark<<<1, kScanThreads, 0, st>>>(sen, mask, n, frac, cap, ref, counts, which);
    note_launch();
    return cudaGetLastError();
}
cudaError_t adapt_deepmask(const int* f1pos, const int* l1grid, int l1gx, int nf1, int* deep, cudaStream_t st) {
    if (nf1 <= 0) return cudaSuccess;
    k_deepmask<<<grid_for(nf1, 256), 256, 0, st>>>(f1pos, l1grid, l1gx, nf1, deep);
    note_launch();
    return cudaGetLastError();
}
cudaError_t adapt_build_l1(const int* ref0, int cnb0, int cgx, int l1gx, int cap1, int* rank, int* fof0, int* rl0,
                           int* pcb, int* oct, int* l1grid, int* f1pos, AdaptCounts* counts, cudaStream_t st) {
    const int ng1 = l1gx * l1gx * l1gx;
    k_build_l1<<<1, kScanThreads, 0, st>>>(ref0, cnb0, cgx, l1gx, ng1, cap1, rank, fof0, rl0, pcb, oct, l1grid, f1pos,
                                           counts);
    note_launch();
    return cudaGetLastError();
}
cudaError_t adapt_scan_l2(const int* ref1, int nf1, int* rank, AdaptCounts* counts, cudaStream_t st) {
    k_scan_l2<<<1, kScanThreads, 0, st>>>(ref1, nf1, rank, counts);
    note_launch();
    return cudaGetLastError();
}
cudaError_t adapt_scatter_l2(const int* ref1, const int* rank, int nf1, int cap2, int* fof1, int* rl1, int* l2pl1,
                             int* l2oct, AdaptCounts* counts, cudaStream_t st) {
    k_scatter_l2<<<grid_for(nf1 > 0 ? nf1 : 1, 256), 256, 0, st>>>(ref1, rank, nf1, cap2, fof1, rl1, l2pl1, l2oct, counts);
    note_launch();
    return cudaGetLastError();
}
cudaError_t adapt_skins(const int* ref0, int cnb0, int cgx, const int* ref1, const int* f1pos, const int* l1grid,
                        int nf1, int l1gx, int* flags, int* skin0, int* skin1, AdaptCounts* counts, cudaStream_t st,
                        int* rest1) {
    k_dilate<<<grid_for(cnb0 + nf1, 256), 256, 0, st>>>(ref0, cnb0, cgx, ref1, f1pos, l1grid, nf1, l1gx, flags);
    k_compact_skins<<<1, kScanThreads, 0, st>>>(flags, cnb0, nf1, skin0, skin1, rest1, counts);
    note_launch(2);
    return cudaGetLastError();
}
// One layer of refinement-mark dilation (--buffer): out[b] = in[b] or a mark on any of the 26
// neighbours (periodic).  Level 0 (pos == nullptr): the coarse grid of gx^3 blocks.  Level 1: the
// neighbours through the level-1 grid map, and only deep blocks take marks (2:1 balance).
__global__ void k_dilate_marks(const int* __restrict__ in, int* __restrict__ out, int n, int gx,
                               const int* __restrict__ pos, const int* __restrict__ grid,
                               const int* __restrict__ deep) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n) return;
    const int p = pos ? pos[b] : b;
    const int px = p % gx, py = (p / gx) % gx, pz = p / (gx * gx);
    int f = in[b] != 0;
    for (int c = 0; c < 27 && !f; ++c) {
        const int nx = (px + c % 3 - 1 + gx) % gx, ny = (py + (c / 3) % 3 - 1 + gx) % gx, nz = (pz + c / 9 - 1 + gx) % gx;
        const int q = (nz * gx + ny) * gx + nx;
        const int nb = grid ? grid[q] : q;
        f = nb >= 0 && in[nb] != 0;
    }
    out[b] = (deep && !deep[b]) ? 0 : f;
}

cudaError_t adapt_dilate_marks(int* ref, int* tmp, int n, int gx, const int* pos, const int* grid, const int* deep,
                               int layers, cudaStream_t st) {
    if (n <= 0 || layers <= 0) return cudaSuccess;
    for (int l = 0; l < layers; ++l) {
        k_dilate_marks<<<grid_for(n, 256), 256, 0, st>>>(ref, tmp, n, gx, pos, grid, deep);
        cudaError_t e = cudaMemcpyAsync(ref, tmp, sizeof(int) * (size_t)n, cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) return e;
        note_launch();
    }
    return cudaGetLastError();
}

cudaError_t adapt_fill_list(const int* nb, int nf, int mb, int* list, int* count, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(count, 0, sizeof(int), st);
    if (e != cudaSuccess || nf <= 0) return e;
    switch (mb) {
        case 4: k_fill_list<4><<<nf, 160, 0, st>>>(nb, list, count); break;
        case 8: k_fill_list<8><<<nf, 256, 0, st>>>(nb, list, count); break;
        case 16: k_fill_list<16><<<nf, 256, 0, st>>>(nb, list, count); break;
        default: return cudaErrorInvalidValue;
    }
    note_launch();
    return cudaGetLastError();
}

cudaError_t adapt_prep_list(const int* skin, const int* nskin_dev, int cap, const int* ref, const int* pos,
                            const int* grid, int gx, int* list, int* count, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(count, 0, sizeof(int), st);
    if (e != cudaSuccess || cap <= 0) return e;
    k_prep_list<<<grid_for(cap, 256), 256, 0, st>>>(skin, nskin_dev, ref, pos, grid, gx, reinterpret_cast<int2*>(list),
                                                     count);
    note_launch();
    return cudaGetLastError();
}

cudaError_t adapt_prep_cells(const int* plist, const int* pcount, int max_entries, int mb, int* cells, int* ncells,
                             cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(ncells, 0, sizeof(int), st);
    if (e != cudaSuccess || max_entries <= 0) return e;
    const int mb3 = mb * mb * mb;
    k_prep_cells<<<max_entries, mb3 < 256 ? ((mb3 + 31) / 32) * 32 : 256, 0, st>>>(
        reinterpret_cast<const int2*>(plist), pcount, mb, cells, ncells);
    note_launch();
    return cudaGetLastError();
}

cudaError_t adapt_fill(int* p, int v, long long n, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    const unsigned g = (unsigned)std::min<long long>(grid_for(n, 256), 4096);
    k_fill_int<<<g, 256, 0, st>>>(p, v, n);
    note_launch();
    return cudaGetLastError();
}

}  // namespace amr
}  // namespace jp
