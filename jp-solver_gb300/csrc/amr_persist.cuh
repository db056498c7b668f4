// Persistent coarse steps: many AMR solves, several coarse steps each, in one cooperative launch.
//
// The batched path (amr_batch_step) issues base_step's stages as separate launches, each a grid over
// the blocks of all solves: 13 launches per coarse step, most of them fractions of a wave on the
// small grids of a served ensemble.  Here one launch runs the whole sequence (src/tgv3d_amr.cu:821-837)
// for up to kAmrBatchMax solves and `steps` coarse steps each (ragged: a solve with fewer steps drops
// out of the later ones), the CTAs walking the ragged per-level work of every solve stage by stage.
// Stages that share no array run in the same phase (the level-0 chain beside the first level-2 pair,
// as base_step's side branch does), so a coarse step is ten grid-wide phases:
//
//   1 coarse step        | level-1 prep (a)        6 level-1 prep (b)
//   2 level-0 prep       | level-2 fill (a)        7 level-2 fill (b)
//   3 level-1 fill       | level-2 substep         8 level-2 substep
//   4 level-2 substep, restricting into level 1    9 level-2 substep, restricting into level 1
//   5 level-1 substep                              10 level-1 substep, restricting into level 0
//
// Work units: a block for the steps (a CTA of RowGeo<MB>::TPB threads per block, the row mapping), a
// slice of TPB listed cells for the preps and fills; their counts come from the device counts of each
// solve's current grid, read once per launch, so no CTA is launched for capacity it does not use.
// CTA b takes units b, b + grid, ... of each phase (a counter that hands out units measured slower:
// its atomic and barriers per unit cost more than the imbalance they remove).  Every unit runs the
// same device body as the per-stage kernels, so results are the same bits.
//
// Between phases the CTAs meet at a grid barrier (a counter in PersistSync).  The launch is
// cooperative, so every CTA is resident and the barrier cannot wait on a CTA that never starts; each
// wait is still bounded: past limit_ns (globaltimer) the CTA records the error, phase and step in
// PersistSync and returns, and every other CTA returns at its next barrier once it sees the error.
// Population arrays are written in one phase and read in a later one of the same launch, so this
// translation unit reads them with ordinary weak loads (JP_COHERENT_POOLS), ordered after the
// barrier's acquire, not through the read-only path.
#pragma once
#define JP_COHERENT_POOLS 1
#include "amr_kernels.cuh"

namespace jp {
namespace amr {

// stages of one coarse step, in base_step's order
enum PersistStage {
    PS_STEP0 = 0, PS_PREP0, PS_FILL1, PS_PREP1A, PS_FILL2A, PS_STEP2A, PS_STEP2AF, PS_STEP1A,
    PS_PREP1B, PS_FILL2B, PS_STEP2B, PS_STEP2BF, PS_STEP1BF, PS_NONE
};
// unit kinds: the count a stage's work units follow
enum PersistKind { PK_CNB0 = 0, PK_PREP0, PK_FILL1, PK_PREP1, PK_FILL2, PK_NF2, PK_NF1, PK_KINDS };

__host__ __device__ constexpr int persist_kind(int stage) {
    return stage == PS_STEP0 ? PK_CNB0
         : stage == PS_PREP0 ? PK_PREP0
         : stage == PS_FILL1 ? PK_FILL1
         : (stage == PS_PREP1A || stage == PS_PREP1B) ? PK_PREP1
         : (stage == PS_FILL2A || stage == PS_FILL2B) ? PK_FILL2
         : (stage == PS_STEP2A || stage == PS_STEP2AF || stage == PS_STEP2B || stage == PS_STEP2BF) ? PK_NF2
                                                                                                    : PK_NF1;
}
// the stages of each phase (two at most; PS_NONE: none)
__device__ __forceinline__ int persist_stage(int phase, int slot) {
    constexpr int8_t tab[kPersistPhases][2] = {
        {PS_STEP0, PS_PREP1A}, {PS_PREP0, PS_FILL2A}, {PS_FILL1, PS_STEP2A}, {PS_STEP2AF, PS_NONE},
        {PS_STEP1A, PS_NONE},  {PS_PREP1B, PS_NONE},  {PS_FILL2B, PS_NONE},  {PS_STEP2B, PS_NONE},
        {PS_STEP2BF, PS_NONE}, {PS_STEP1BF, PS_NONE}};
    return tab[phase][slot];
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ int ld_relaxed(const int* p) {
    int v;
    asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Grid barrier number `k` (1, 2, ...): every CTA arrives once per barrier, so the k-th completes at
// k * gridDim.x arrivals.  Returns false (whole CTA) when the launch has to stop: this CTA's wait
// ran past limit_ns (it records the error) or another CTA recorded one.
__device__ __forceinline__ bool persist_barrier(PersistSync* sy, unsigned k, long long limit_ns, int phase, int step) {
    __shared__ int go;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();  // this CTA's writes before its arrival
        atomicAdd(&sy->arrived, 1u);
        const unsigned target = k * gridDim.x;
        const unsigned long long t0 = global_ns();
        int ok = 1;
        for (;;) {
            if (ld_acquire(&sy->arrived) >= target) break;
            if (ld_relaxed(&sy->err)) {
                ok = 0;
                break;
            }
            if ((long long)(global_ns() - t0) > limit_ns) {
                if (atomicCAS(&sy->err, 0, 1) == 0) {
                    sy->phase = phase;
                    sy->step = step;
                }
                ok = 0;
                break;
            }
            __nanosleep(64);
        }
        __threadfence();  // the other CTAs' writes before this CTA's next phase
        go = ok;
    }
    __syncthreads();
    return go != 0;
}

// the work units of kind k of one member (the list slices are TPB cells)
template <int TPB>
__device__ __forceinline__ int persist_units(const PersistMember& M, int k) {
    switch (k) {
        case PK_CNB0: return M.cnb0;
        case PK_PREP0: return __ldg(M.n_fill1) == 0 ? 0 : (__ldg(M.n_prep0) + TPB - 1) / TPB;
        case PK_FILL1: return (__ldg(M.n_fill1) + TPB - 1) / TPB;
        case PK_PREP1: return __ldg(M.n_fill2) == 0 ? 0 : (__ldg(M.n_prep1) + TPB - 1) / TPB;
        case PK_FILL2: return (__ldg(M.n_fill2) + TPB - 1) / TPB;
        case PK_NF2: return __ldg(M.n_f2);
        default: return __ldg(M.n_f1);
    }
}

// One work unit u (of `nu`) of a stage of member M in coarse step j of the launch.
template <int MB, class ST>
__device__ __forceinline__ void persist_unit(const PersistMember& M, int stage, int j, int u, int nu) {
    using raw = typename ST::raw;
    constexpr int T = RowGeo<MB>::TPB;
    const raw* c0s = (const raw*)M.c0[j & 1];  // this coarse step's source
    raw* c0d = (raw*)M.c0[(j & 1) ^ 1];        // its result, the coarse state of the fine substeps
    const int tid = u * T + (int)threadIdx.x, nth = nu * T;
    raw *f1a = (raw*)M.f1a, *f1b = (raw*)M.f1b, *f2a = (raw*)M.f2a, *f2b = (raw*)M.f2b;
    raw *prep0 = (raw*)M.prep0, *prep1 = (raw*)M.prep1, *gh1 = (raw*)M.gh1, *gh2 = (raw*)M.gh2;
    switch (stage) {
        case PS_STEP0: d_step_l0<MB, ST, T>(c0s, c0d, M.cgx, M.om0, u); break;
        case PS_PREP0: d_prep<MB, ST>(c0d, prep0, M.pc0, M.nqs01, M.n_prep0, M.n_fill1, tid, nth); break;
        case PS_FILL1: d_fill_l1<MB, ST>(prep0, gh1, M.pcb, M.oct, M.cgx, M.n, M.fl1, M.n_fill1, tid, nth); break;
        case PS_PREP1A: d_prep<MB, ST>(f1a, prep1, M.pc1, M.nqs12, M.n_prep1, M.n_fill2, tid, nth); break;
        case PS_PREP1B: d_prep<MB, ST>(f1b, prep1, M.pc1, M.nqs12, M.n_prep1, M.n_fill2, tid, nth); break;
        case PS_FILL2A:
        case PS_FILL2B:
            d_fill_l2<MB, ST>(prep1, gh2, M.l2pl1, M.l2oct, M.f1pos, M.l1grid, M.l1gx, M.n1, M.fl2, M.n_fill2, tid,
                              nth);
            break;
        case PS_STEP2A:
        case PS_STEP2B:
            d_step_fine_rows<MB, ST, false, false>(f2a, f2b, gh2, M.nb2, M.l2pl1, M.l2oct, M.om2, nullptr, 0.f,
                                                   M.n_f2, u, 0);
            break;
        case PS_STEP2AF:  // the second level-2 substep restricts into level 1 (f1a before its substep)
            d_step_fine_rows<MB, ST, true, false>(f2b, f2a, gh2, M.nb2, M.l2pl1, M.l2oct, M.om2, f1a, M.nqi21, M.n_f2,
                                                  u, 0);
            break;
        case PS_STEP2BF:  // ... and after the first level-1 substep into f1b
            d_step_fine_rows<MB, ST, true, false>(f2b, f2a, gh2, M.nb2, M.l2pl1, M.l2oct, M.om2, f1b, M.nqi21, M.n_f2,
                                                  u, 0);
            break;
        case PS_STEP1A:
            d_step_fine_rows<MB, ST, false, false>(f1a, f1b, gh1, M.nb1, M.pcb, M.oct, M.om1, nullptr, 0.f, M.n_f1, u,
                                                   0);
            break;
        default:  // PS_STEP1BF: the second level-1 substep restricts into this coarse step's result
            d_step_fine_rows<MB, ST, true, false>(f1b, f1a, gh1, M.nb1, M.pcb, M.oct, M.om1, c0d, M.nqi10, M.n_f1, u,
                                                  0);
            break;
    }
}

// four CTAs per SM in every storage format: the kernel holds every stage's body, and at the 16-bit
// rows kernels' five it would spill (~290 bytes per thread)
template <int MB, class ST>
__global__ void __launch_bounds__(RowGeo<MB>::TPB, 4) kp_coarse_steps(const __grid_constant__ AmrPersist P) {
    constexpr int T = RowGeo<MB>::TPB, E = 2 * kAmrBatchMax;
    // units[m][k]: work units of kind k of member m (the grid is fixed during the launch)
    __shared__ int units[kAmrBatchMax][PK_KINDS];
    // first[ph][2m + s]: first unit of member m's stage in slot s of phase ph, members in order
    __shared__ int first[kPersistPhases][E + 1];
    for (int i = threadIdx.x; i < P.count * PK_KINDS; i += blockDim.x)
        units[i / PK_KINDS][i % PK_KINDS] = persist_units<T>(P.m[i / PK_KINDS], i % PK_KINDS);
    __syncthreads();
    if (threadIdx.x < kPersistPhases) {
        const int ph = threadIdx.x;
        int acc = 0;
        for (int e = 0; e < 2 * P.count; ++e) {
            first[ph][e] = acc;
            const int stg = persist_stage(ph, e & 1);
            acc += stg == PS_NONE ? 0 : units[e >> 1][persist_kind(stg)];
        }
        first[ph][2 * P.count] = acc;
    }
    __syncthreads();
    unsigned barrier = 0;
    int active = P.count;  // members still stepping: a prefix, since they are sorted by steps
    for (int j = 0; j < P.maxsteps; ++j) {
        while (active > 0 && P.m[active - 1].steps <= j) --active;
        for (int ph = 0; ph < kPersistPhases; ++ph) {
            const int* fp = first[ph];
            const int total = fp[2 * active];
            for (int u = blockIdx.x; u < total; u += gridDim.x) {
                int lo = 0, hi = 2 * active - 1;  // the entry e with fp[e] <= u < fp[e + 1]
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (fp[mid] <= u) lo = mid;
                    else hi = mid - 1;
                }
                const int stg = persist_stage(ph, lo & 1);
                const int m = lo >> 1;
                persist_unit<MB, ST>(P.m[m], stg, j, u - fp[lo], units[m][persist_kind(stg)]);
                __syncthreads();  // the next unit reuses the bodies' shared memory
            }
            if (j + 1 == P.maxsteps && ph + 1 == kPersistPhases) break;
            if (!persist_barrier(P.sync, ++barrier, P.limit_ns, ph, j)) return;
        }
    }
}

template <int MB, class ST>
static int persist_grid_cap() {
    static const int cap = [] {
        int dev = 0, sms = 0, per = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaFuncSetAttribute(kp_coarse_steps<MB, ST>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(sizeof(float) * Q * Geo<MB>::MB3));
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kp_coarse_steps<MB, ST>, RowGeo<MB>::TPB,
                                                      sizeof(float) * Q * Geo<MB>::MB3);
        return sms * per;
    }();
    return cap;
}

template <class ST>
cudaError_t amr_persist_launch_st(int mb, const AmrPersist& P, int grid, cudaStream_t st, int* grid_used) {
    if (mb != 8) return cudaErrorInvalidValue;
    constexpr int MB = 8;
    const int cap = persist_grid_cap<MB, ST>();
    if (cap <= 0) return cudaErrorLaunchOutOfResources;
    const int g = grid > 0 && grid < cap ? grid : cap;
    if (grid_used) *grid_used = g;
    if (P.count <= 0 || P.maxsteps <= 0) return cudaSuccess;
    void* args[] = {const_cast<AmrPersist*>(&P)};
    cudaError_t e = cudaLaunchCooperativeKernel((const void*)kp_coarse_steps<MB, ST>, dim3(g), dim3(RowGeo<MB>::TPB),
                                                args, sizeof(float) * Q * Geo<MB>::MB3, st);
    note_launch();
    return e;
}

}  // namespace amr
}  // namespace jp
