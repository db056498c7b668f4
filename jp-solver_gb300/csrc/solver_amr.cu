// Three-level block AMR solver: pools, the initial build, regrid, the 1:2:4 subcycled step and the
// composite diagnostics.  Reference: main() of src/tgv3d_amr.cu (pool sizing :675-709, gpurce_regrid
// :722-764, gpurce_init :776-815, base_step :821-837, diagnostics :866-888).  The launch sequence and
// the pool policy are the reference's, so block tables come out identical; the kernels are this
// library's (amr_kernels.cu, adapt.cu).
#include "amr_kernels.h"
#include "jp.h"
#include "kernels.h"
#include "lattice.cuh"
#include "solver.h"

#include <algorithm>
#include <cstddef>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

namespace jp {
using namespace amr;

struct AmrState {
    jp_solver* owner = nullptr;  // allocations go through dev_alloc of the owning solver
    int storage = 0;             // population format of pools, prolongation sources and ghosts
    size_t elem = 4;             // bytes per stored population
    int MB = 8, MB3 = 512, SH = 480, N = 0, cgx = 0, cnb0 = 0, l1gx = 0, N1 = 0, N2 = 0, NG1 = 0;
    double tau0 = 0, tau1 = 0, tau2 = 0, nqs01 = 0, nqi10 = 0, nqs12 = 0, nqi21 = 0;
    float om0 = 0, om1 = 0, om2 = 0;
    int l1mode = 0, l2mode = 0;
    bool dynamic = false;
    int cap_nref0 = 0, cap1 = 0, cap_nref1 = INT_MAX, cap2 = 0;
    long long hw_nf1 = 0, hw_nf2 = 0;
    double budget = 0;
    size_t PB = 0;
    float *c0a = nullptr, *c0b = nullptr, *f1a = nullptr, *f1b = nullptr, *gh1 = nullptr, *prep0 = nullptr,
          *prep1 = nullptr, *f2a = nullptr, *f2b = nullptr, *gh2 = nullptr;
    int *ref0 = nullptr, *fof0 = nullptr, *rl0 = nullptr, *pcb = nullptr, *oct = nullptr, *f1pos = nullptr,
        *l1grid = nullptr, *ref1 = nullptr, *fof1 = nullptr, *rl1 = nullptr, *l2pl1 = nullptr, *l2oct = nullptr,
        *skin0 = nullptr, *skin1 = nullptr;
    int* rest1 = nullptr;  // level-1 blocks outside the skin, ascending (adapt_skins), SC_REST1 of them
    int *o_ref0 = nullptr, *o_fof0 = nullptr, *o_l1grid = nullptr, *o_ref1 = nullptr, *o_fof1 = nullptr;
    int *rank = nullptr, *deep = nullptr, *flags = nullptr;
    int *nb1 = nullptr, *nb2 = nullptr;  // same-level neighbour tables of the fine levels (27 per block)
    int *fl1 = nullptr, *fl2 = nullptr;  // fill lists: ghost cells b * SH + t to fill (adapt_fill_list)
    int *pl0 = nullptr, *pl1 = nullptr;  // prep lists: {skin block, refined neighbours} (adapt_prep_list)
    int *pc0 = nullptr, *pc1 = nullptr;  // their interface cells, b * MB^3 + cell (adapt_prep_cells)
    int tpb = 0;                         // threads per CTA of the per-cell steps (0: default_step_tpb)
    int vec = 0;                         // fine steps: 4 rows of four cells, 1 a cell per thread (0: default)
    float *sen0 = nullptr, *sen1 = nullptr;
    float *ov_sen0 = nullptr, *ov_sen1pos = nullptr;
    AdaptCounts* cnt_dev = nullptr;
    AdaptCounts* cnt_host = nullptr;
    int nref0 = 0, nf1 = 0, nref1 = 0, nf2 = 0, n_skin0 = 0, n_skin1 = 0, ndeep = 0;
    bool skins_pending = false;  // n_skin0/1 arrive with the read-back skins() queued (skins_landed)
    float* field = nullptr;
    std::vector<void*> owned;
    // Block counts the step kernels read on the device ({nf1, nf2, n_skin0, n_skin1, nref0, nref1}):
    // the step launches grids sized for the pool capacities, so one captured step serves every grid
    // a regrid builds within them.
    int* step_cnt = nullptr;
    int* step_cnt_host = nullptr;  // pinned staging of the upload
    // captured base_step graphs, one per combination of the ping-pong parities of the three levels
    // (a coarse step swaps level 0 once and the fine levels an even number of times; a regrid's
    // seeding swaps a fine level once).  Dropped only when buffers move (pool growth, new initial
    // build) or the launch shape changes.
    cudaGraphExec_t graph[8] = {};
    float *c0_home = nullptr, *f1_home = nullptr, *f2_home = nullptr;
    AmrFork fk;  // a coarse step's level-0 chain runs on fk.side, beside the first level-2 pair (base_step)
};
// SC_COUNT entries come from the host (upload_counts); the fill-list lengths are written on the device
// (SC_PREP0/1: interface cells of the prep lists, whose block counts are SC_PBLK0/1)
enum { SC_NF1 = 0, SC_NF2, SC_SKIN0, SC_SKIN1, SC_NREF0, SC_NREF1, SC_COUNT, SC_FILL1 = SC_COUNT, SC_FILL2, SC_PREP0,
       SC_PREP1, SC_PBLK0, SC_PBLK1, SC_REST1, SC_ALL };
// CTAs per member of a batched prep or fill (its threads walk the member's cell list)
constexpr int kBatchPrepCtas = 64;

// drop the captured steps and take the current buffers as the parity reference
static void reset_graphs(AmrState* a) {
    for (auto& g : a->graph)
        if (g) {
            cudaGraphExecDestroy(g);
            g = nullptr;
        }
    a->c0_home = a->c0a;
    a->f1_home = a->f1a;
    a->f2_home = a->f2a;
}

#define ACK(call, what)                                     \
    do {                                                    \
        cudaError_t e_ = (call);                            \
        if (e_ != cudaSuccess) return cuda_fail(e_, what);  \
    } while (0)

template <class T>
static jp_status dalloc(AmrState* a, T** p, size_t count, const char* what) {
    *p = nullptr;
    if (count == 0) count = 1;
    cudaError_t e = dev_alloc(a->owner, (void**)p, count * sizeof(T));
    if (e != cudaSuccess) return cuda_fail(e, what);
    a->owned.push_back(*p);
    return JP_OK;
}
template <class T>
static void dfree(AmrState* a, T*& p) {
    if (!p) return;
    auto it = std::find(a->owned.begin(), a->owned.end(), (void*)p);
    if (it != a->owned.end()) a->owned.erase(it);
    dev_free(a->owner, p);
    p = nullptr;
}

#define TRY(x)                      \
    do {                            \
        jp_status s_ = (x);         \
        if (s_ != JP_OK) return s_; \
    } while (0)

// Floats of allocation that hold n populations in the solver's storage format (the population
// arrays are typed float* and carry 16-bit values for the shifted formats).
static size_t pf(const AmrState* a, size_t n) { return (n * a->elem + 3) / 4; }

static jp_status launch(jp_solver* s, int op, AmrLaunch L, cudaStream_t st = nullptr) {
    L.st = st ? st : s->stream;
    cudaError_t e = amr_launch(s->amr->storage, s->amr->MB, op, L);
    if (e != cudaSuccess) return cuda_fail(e, "AMR kernel launch");
    return JP_OK;
}

static jp_status read_counts(jp_solver* s) {
    AmrState* a = s->amr;
    ACK(cudaMemcpyAsync(a->cnt_host, a->cnt_dev, sizeof(AdaptCounts), cudaMemcpyDeviceToHost, s->stream), "counts D2H");
    ACK(wait_stream(s), "adaptation");
    return JP_OK;
}

static bool pool_fits(const AmrState* a, long long c1, long long c2) {
    return (double)((size_t)(c1 + c2) * a->PB * 6 / 5) < a->budget;
}

// sensor of level 0 (all coarse blocks) or level 1 (active fine blocks), override-aware
static jp_status sensor(jp_solver* s, int level) {
    AmrState* a = s->amr;
    AmrLaunch L;
    if (level == 0) {
        L.nblocks = a->cnb0;
        L.in = a->c0a;
        L.out = a->sen0;
        L.aux = a->ov_sen0;
        L.t0 = nullptr;
    } else {
        L.nblocks = a->nf1;
        L.in = a->f1a;
        L.out = a->sen1;
        L.aux = a->ov_sen1pos;
        L.t0 = a->ov_sen1pos ? a->f1pos : nullptr;
    }
    return launch(s, OP_SENSOR, L);
}

static jp_status step_l0(jp_solver* s, cudaStream_t st = nullptr) {
    AmrState* a = s->amr;
    AmrLaunch L;
    L.nblocks = a->cnb0;
    L.in = a->c0a;
    L.out = a->c0b;
    L.cgx = a->cgx;
    L.n = a->N;
    L.omega = a->om0;
    L.tpb = a->tpb;
    TRY(launch(s, OP_STEP_L0, L, st));
    std::swap(a->c0a, a->c0b);
    return JP_OK;
}

// the host's block counts of the current grid to the device copy the step kernels read
static jp_status upload_counts(jp_solver* s) {
    AmrState* a = s->amr;
    int* h = a->step_cnt_host;
    h[SC_NF1] = a->nf1;
    h[SC_NF2] = a->nf2;
    h[SC_SKIN0] = a->n_skin0;
    h[SC_SKIN1] = a->n_skin1;
    h[SC_NREF0] = a->nref0;
    h[SC_NREF1] = a->nref1;
    ACK(cudaMemcpyAsync(a->step_cnt, h, sizeof(int) * SC_COUNT, cudaMemcpyHostToDevice, s->stream), "counts H2D");
    return JP_OK;
}

// prep lists of both levels from their skin lists and refinement marks, lengths into the device counts;
// the skin counts are read on the device (step_cnt[SC_SKIN0/1]), the grids sized by capacity
static jp_status prep_lists(jp_solver* s) {
    AmrState* a = s->amr;
    ACK(adapt_prep_list(a->skin0, a->step_cnt + SC_SKIN0, a->cnb0, a->ref0, nullptr, nullptr, a->cgx, a->pl0,
                        a->step_cnt + SC_PBLK0, s->stream), "prep list 0");
    ACK(adapt_prep_list(a->skin1, a->step_cnt + SC_SKIN1, a->cap1, a->ref1, a->f1pos, a->l1grid, a->l1gx, a->pl1,
                        a->step_cnt + SC_PBLK1, s->stream), "prep list 1");
    ACK(adapt_prep_cells(a->pl0, a->step_cnt + SC_PBLK0, a->cnb0, a->MB, a->pc0, a->step_cnt + SC_PREP0, s->stream),
        "prep cells 0");
    ACK(adapt_prep_cells(a->pl1, a->step_cnt + SC_PBLK1, a->cap1, a->MB, a->pc1, a->step_cnt + SC_PREP1, s->stream),
        "prep cells 1");
    return JP_OK;
}

static_assert(offsetof(AdaptCounts, n_skin1) == offsetof(AdaptCounts, n_skin0) + sizeof(int) &&
                  SC_SKIN1 == SC_SKIN0 + 1,
              "the two skin counts are copied as one pair");

// Skin lists of the current grid and the prep lists built from them.  Their lengths stay on the
// device: the host's block counts go up first, then the two skin counts are copied over theirs
// from the adaptation counts, and the prep lists read them there.  The host's copy of the skin
// counts arrives with a read-back queued here and is taken after the caller's wait (skins_landed):
// a regrid needs no read-back for its skins.
static jp_status skins(jp_solver* s) {
    AmrState* a = s->amr;
    ACK(adapt_skins(a->ref0, a->cnb0, a->cgx, a->ref1, a->f1pos, a->l1grid, a->nf1, a->l1gx, a->flags, a->skin0,
                    a->skin1, a->cnt_dev, s->stream, a->rest1), "skins");
    TRY(upload_counts(s));
    ACK(cudaMemcpyAsync(a->step_cnt + SC_SKIN0, &a->cnt_dev->n_skin0, 2 * sizeof(int), cudaMemcpyDeviceToDevice,
                        s->stream), "skin counts");
    ACK(cudaMemcpyAsync(a->step_cnt + SC_REST1, &a->cnt_dev->n_rest1, sizeof(int), cudaMemcpyDeviceToDevice,
                        s->stream), "rest count");
    TRY(prep_lists(s));
    ACK(cudaMemcpyAsync(a->cnt_host, a->cnt_dev, sizeof(AdaptCounts), cudaMemcpyDeviceToHost, s->stream), "counts D2H");
    a->skins_pending = true;
    return JP_OK;
}

// the host's skin counts, once the stream has passed the read-back skins() queued
static void skins_landed(AmrState* a) {
    if (!a->skins_pending) return;
    a->n_skin0 = a->cnt_host->n_skin0;
    a->n_skin1 = a->cnt_host->n_skin1;
    a->skins_pending = false;
}

static jp_status check_err(jp_solver* s) {
    const int e = s->amr->cnt_host->err;
    if (e & ADAPT_ERR_CAP1) return fail(JP_ERR_CAPACITY, "level-1 pool overflow: %d blocks > capacity %d", s->amr->cnt_host->nf1, s->amr->cap1);
    if (e & ADAPT_ERR_CAP2) return fail(JP_ERR_CAPACITY, "level-2 pool overflow: %d blocks > capacity %d", s->amr->cnt_host->nf2, s->amr->cap2);
    return JP_OK;
}

static jp_status mark_l0_by_sensor(jp_solver* s) {
    AmrState* a = s->amr;
    TRY(sensor(s, 0));
    ACK(adapt_threshold_mark(a->sen0, nullptr, a->cnb0, s->cfg.frac1, a->cap_nref0, a->ref0, a->cnt_dev, 0, s->stream),
        "threshold L0");
    // --buffer: a margin of refined blocks around the marked ones (compaction for localised features)
    ACK(adapt_dilate_marks(a->ref0, a->flags, a->cnb0, a->cgx, nullptr, nullptr, nullptr, s->cfg.buffer, s->stream),
        "buffer L0");
    return JP_OK;
}

// --buffer on level 1: dilate the level-2 marks over the level-1 grid, deep blocks only
static jp_status buffer_l1(jp_solver* s) {
    AmrState* a = s->amr;
    ACK(adapt_dilate_marks(a->ref1, a->flags, a->nf1, a->l1gx, a->f1pos, a->l1grid, a->deep, s->cfg.buffer, s->stream),
        "buffer L1");
    return JP_OK;
}

// Replace a device array by one of `count` elements that keeps the first `keep` elements.
template <class T>
static jp_status regrow(jp_solver* s, T*& p, size_t count, size_t keep) {
    AmrState* a = s->amr;
    T* q = nullptr;
    TRY(dalloc(a, &q, count, "cudaMalloc (pool growth)"));
    if (keep && p) ACK(cudaMemcpyAsync(q, p, keep * sizeof(T), cudaMemcpyDeviceToDevice, s->stream), "pool growth copy");
    ACK(wait_stream(s), "pool growth");
    dfree(a, p);
    p = q;
    return JP_OK;
}

static void update_bytes(jp_solver* s) {
    const AmrState* a = s->amr;
    s->info.bytes_state = (int64_t)((((size_t)3 * a->cnb0 + 3 * (size_t)a->cap1 + 2 * (size_t)a->cap2) * Q * a->MB3 +
                                     ((size_t)a->cap1 + a->cap2) * Q * a->SH) * a->elem);
}

// Reallocate the arrays sized by the level-1 capacity; keep: the payload the migration reads and
// the snapshots of the previous grid survive (pool growth), else nothing does (state loading).
static jp_status set_cap1(jp_solver* s, int cap, bool keep) {
    AmrState* a = s->amr;
    const size_t blk = (size_t)Q * a->MB3, old = keep ? std::min(a->cap1, cap) : 0;
    TRY(regrow(s, a->f1a, pf(a, cap * blk), pf(a, old * blk)));  // payload the migration reads
    TRY(regrow(s, a->f1b, pf(a, cap * blk), 0));
    TRY(regrow(s, a->gh1, pf(a, (size_t)cap * Q * a->SH), 0));
    TRY(regrow(s, a->prep1, pf(a, cap * blk), 0));
    TRY(regrow(s, a->o_ref1, cap, old));           // snapshots of the previous grid
    TRY(regrow(s, a->o_fof1, cap, old));
    int** scratch[] = {&a->pcb, &a->oct, &a->rl0, &a->f1pos, &a->ref1, &a->fof1, &a->rl1, &a->skin1, &a->rest1,
                       &a->deep};
    for (int** t : scratch) TRY(regrow(s, *t, cap, 0));
    TRY(regrow(s, a->sen1, cap, 0));
    TRY(regrow(s, a->rank, std::max(a->cnb0, cap), 0));
    TRY(regrow(s, a->flags, (size_t)a->cnb0 + cap, 0));
    TRY(regrow(s, a->nb1, (size_t)cap * 27, 0));
    TRY(regrow(s, a->fl1, (size_t)a->SH * cap, 0));
    TRY(regrow(s, a->pl1, 2 * (size_t)cap, 0));
    TRY(regrow(s, a->pc1, (size_t)interface_cells(a->MB) * cap, 0));
    reset_graphs(a);
    ACK(cudaMemsetAsync(a->fof1, 0xFF, sizeof(int) * cap, s->stream), "memset");
    ACK(cudaMemsetAsync(a->ref1, 0, sizeof(int) * cap, s->stream), "memset");
    a->cap1 = cap;
    update_bytes(s);
    return JP_OK;
}

static jp_status set_cap2(jp_solver* s, int cap, bool keep) {
    AmrState* a = s->amr;
    const size_t blk = (size_t)Q * a->MB3, old = keep ? std::min(a->cap2, cap) : 0;
    TRY(regrow(s, a->f2a, pf(a, cap * blk), pf(a, old * blk)));  // payload the migration reads
    TRY(regrow(s, a->f2b, pf(a, cap * blk), 0));
    TRY(regrow(s, a->gh2, pf(a, (size_t)cap * Q * a->SH), 0));
    TRY(regrow(s, a->l2pl1, cap, 0));
    TRY(regrow(s, a->l2oct, cap, 0));
    TRY(regrow(s, a->nb2, (size_t)cap * 27, 0));
    TRY(regrow(s, a->fl2, (size_t)a->SH * cap, 0));
    reset_graphs(a);
    a->cap2 = cap;
    update_bytes(s);
    return JP_OK;
}

// Pools grow on overflow instead of being written past their end (the reference sizes them with
// margins and does not check: ties at the threshold over-admit).  The new capacity is at least
// twice the old one and must fit the HBM budget; payloads and the snapshots of the previous grid
// that a regrid still reads are kept.
static jp_status grow_l1(jp_solver* s, int needed) {
    AmrState* a = s->amr;
    const int cap = ((std::max(needed, 2 * a->cap1) + 7) / 8) * 8;
    if (!pool_fits(a, cap, a->cap2))
        return fail(JP_ERR_CAPACITY, "level-1 pool overflow: %d blocks needed, %d held, budget allows no growth", needed,
                    a->cap1);
    return set_cap1(s, cap, true);
}

static jp_status grow_l2(jp_solver* s, int needed) {
    AmrState* a = s->amr;
    const int cap = ((std::max(needed, 2 * a->cap2) + 7) / 8) * 8;
    if (!pool_fits(a, a->cap1, cap))
        return fail(JP_ERR_CAPACITY, "level-2 pool overflow: %d blocks needed, %d held, budget allows no growth", needed,
                    a->cap2);
    return set_cap2(s, cap, true);
}

// exclusive scan of the marks and the level-1 tables; on overflow of the level-1 pool nothing is
// written, the pool grows and the tables are built again.  If the pool cannot grow the error stands
// and, in a regrid (restore_marks), the previous marks come back: the old grid stays valid.
static jp_status build_l1(jp_solver* s, bool restore_marks) {
    AmrState* a = s->amr;
    ACK(adapt_build_l1(a->ref0, a->cnb0, a->cgx, a->l1gx, a->cap1, a->rank, a->fof0, a->rl0, a->pcb, a->oct, a->l1grid,
                       a->f1pos, a->cnt_dev, s->stream), "build L1");
    TRY(read_counts(s));
    if (a->cnt_host->err & ADAPT_ERR_CAP1) {
        jp_status g = grow_l1(s, a->cnt_host->nf1);
        if (g == JP_OK) {
            a->cnt_host->err = 0;
            ACK(cudaMemsetAsync(&a->cnt_dev->err, 0, sizeof(int), s->stream), "counts");
            ACK(adapt_build_l1(a->ref0, a->cnb0, a->cgx, a->l1gx, a->cap1, a->rank, a->fof0, a->rl0, a->pcb, a->oct,
                               a->l1grid, a->f1pos, a->cnt_dev, s->stream), "build L1");
            TRY(read_counts(s));
        } else if (restore_marks) {
            ACK(cudaMemcpyAsync(a->ref0, a->o_ref0, sizeof(int) * a->cnb0, cudaMemcpyDeviceToDevice, s->stream), "restore");
            ACK(wait_stream(s), "restore");
            return g;
        } else {
            return g;
        }
    }
    TRY(check_err(s));
    a->nref0 = a->cnt_host->nref0;
    a->nf1 = a->cnt_host->nf1;
    a->hw_nf1 = std::max(a->hw_nf1, (long long)a->nf1);
    return JP_OK;
}

// fill lists of both fine levels from their neighbour tables, lengths into the device counts
static jp_status fill_lists(jp_solver* s) {
    AmrState* a = s->amr;
    ACK(adapt_fill_list(a->nb1, a->nf1, a->MB, a->fl1, a->step_cnt + SC_FILL1, s->stream), "fill list 1");
    ACK(adapt_fill_list(a->nb2, a->nf2, a->MB, a->fl2, a->step_cnt + SC_FILL2, s->stream), "fill list 2");
    return JP_OK;
}

// same-level neighbour tables of both fine levels for the current grid
static jp_status neighbour_tables(jp_solver* s) {
    AmrState* a = s->amr;
    AmrLaunch L;
    L.nblocks = a->nf1;
    L.iout = a->nb1;
    L.t0 = a->pcb;
    L.t1 = a->oct;
    L.t2 = a->ref0;
    L.t3 = a->fof0;
    L.cgx = a->cgx;
    TRY(launch(s, OP_NBTAB_L1, L));
    AmrLaunch M;
    M.nblocks = a->nf2;
    M.iout = a->nb2;
    M.t0 = a->l2pl1;
    M.t1 = a->l2oct;
    M.t2 = a->f1pos;
    M.t3 = a->l1grid;
    M.t4 = a->ref1;
    M.t5 = a->fof1;
    M.l1gx = a->l1gx;
    TRY(launch(s, OP_NBTAB_L2, M));
    return fill_lists(s);
}

// gpurce_init (src/tgv3d_amr.cu:776-815)
static jp_status initial_build(jp_solver* s) {
    AmrState* a = s->amr;
    const jp_config& c = s->cfg;
    ACK(cudaMemsetAsync(a->cnt_dev, 0, sizeof(AdaptCounts), s->stream), "counts");
    if (a->l1mode == JP_REFINE_ALL || a->l1mode == JP_REFINE_SLAB) {
        ACK(adapt_mark_mode(a->l1mode == JP_REFINE_ALL ? 0 : 1, a->ref0, a->cnb0, a->cgx, s->stream), "mark L0");
    } else {
        for (int i = 0; i < c.develop_steps; ++i) TRY(step_l0(s));  // uncounted coarse steps (:711,779)
        TRY(mark_l0_by_sensor(s));
    }
    TRY(build_l1(s, false));
    if (a->nf1) {
        ACK(cudaMemsetAsync(a->gh1, 0, a->elem * (size_t)a->nf1 * Q * a->SH, s->stream), "memset gh1");
        AmrLaunch L;
        L.nblocks = a->nf1;
        L.out = a->f1a;
        L.aux = a->c0a;
        L.t0 = a->pcb;
        L.t1 = a->oct;
        L.cgx = a->cgx;
        L.n = a->N;
        L.scale = float(a->nqs01);
        TRY(launch(s, OP_SEED_L1, L));
    }
    a->nref1 = a->nf2 = 0;
    if (a->nf1) {
        TRY(sensor(s, 1));
        ACK(adapt_deepmask(a->f1pos, a->l1grid, a->l1gx, a->nf1, a->deep, s->stream), "deepmask");
        ACK(cudaMemsetAsync(a->ref1, 0, sizeof(int) * a->cap1, s->stream), "memset ref1");
        if (a->l2mode == JP_REFINE_ALL) {
            ACK(cudaMemcpyAsync(a->ref1, a->deep, sizeof(int) * a->nf1, cudaMemcpyDeviceToDevice, s->stream), "ref1=deep");
        } else {
            ACK(adapt_threshold_mark(a->sen1, a->deep, a->nf1, c.frac2, INT_MAX, a->ref1, a->cnt_dev, 1, s->stream),
                "threshold L1");
            TRY(buffer_l1(s));
        }
        ACK(adapt_scan_l2(a->ref1, a->nf1, a->rank, a->cnt_dev, s->stream), "scan L2");
        TRY(read_counts(s));
        a->nref1 = a->cnt_host->nref1;
        a->nf2 = a->cnt_host->nf2;
        a->ndeep = a->cnt_host->ndeep;
        a->hw_nf2 = std::max(a->hw_nf2, (long long)a->nf2);
        a->cap_nref1 = std::max(1, (int)std::ceil(a->nref1 * 2.5));
        if (a->l2mode == JP_REFINE_ALL) a->cap_nref1 = std::max(a->cap_nref1, a->nf1);
        a->cap_nref1 = std::min(a->cap_nref1, a->cap1);
        while (a->cap_nref1 > 1 && !pool_fits(a, a->cap1, 8LL * a->cap_nref1)) a->cap_nref1--;
        a->cap2 = 8 * a->cap_nref1;
    } else {
        a->cap_nref1 = 1;
        a->cap2 = 8;
    }
    if (a->nf2 > a->cap2) return fail(JP_ERR_CAPACITY, "level-2 pool overflow: %d > %d", a->nf2, a->cap2);
    dfree(a, a->f2a);
    dfree(a, a->f2b);
    dfree(a, a->gh2);
    dfree(a, a->l2pl1);
    dfree(a, a->l2oct);
    dfree(a, a->nb2);
    dfree(a, a->fl2);
    const size_t blk = (size_t)Q * a->MB3;
    TRY(dalloc(a, &a->nb2, (size_t)a->cap2 * 27, "cudaMalloc nb2"));
    TRY(dalloc(a, &a->fl2, (size_t)a->SH * a->cap2, "cudaMalloc fl2"));
    TRY(dalloc(a, &a->f2a, pf(a, (size_t)a->cap2 * blk), "cudaMalloc f2"));
    TRY(dalloc(a, &a->f2b, pf(a, (size_t)a->cap2 * blk), "cudaMalloc f2"));
    TRY(dalloc(a, &a->gh2, pf(a, (size_t)a->cap2 * Q * a->SH), "cudaMalloc gh2"));
    TRY(dalloc(a, &a->l2pl1, (size_t)a->cap2, "cudaMalloc l2pl1"));
    TRY(dalloc(a, &a->l2oct, (size_t)a->cap2, "cudaMalloc l2oct"));
    ACK(cudaMemsetAsync(a->fof1, 0xFF, sizeof(int) * a->cap1, s->stream), "memset fof1");
    if (a->nf2) {
        ACK(adapt_scatter_l2(a->ref1, a->rank, a->nf1, a->cap2, a->fof1, a->rl1, a->l2pl1, a->l2oct, a->cnt_dev,
                             s->stream), "scatter L2");
        ACK(cudaMemsetAsync(a->gh2, 0, a->elem * (size_t)a->nf2 * Q * a->SH, s->stream), "memset gh2");
        AmrLaunch L;
        L.nblocks = a->nf2;
        L.out = a->f2a;
        L.aux = a->f1a;
        L.t0 = a->l2pl1;
        L.t1 = a->l2oct;
        L.t2 = a->f1pos;
        L.t6 = a->l1grid;
        L.l1gx = a->l1gx;
        L.n1 = a->N1;
        L.scale = float(a->nqs12);
        TRY(launch(s, OP_SEED_L2, L));
    }
    TRY(neighbour_tables(s));
    TRY(skins(s));
    return JP_OK;
}

// gpurce_regrid (src/tgv3d_amr.cu:722-764)
static jp_status regrid(jp_solver* s) {
    AmrState* a = s->amr;
    const jp_config& c = s->cfg;
    ACK(cudaMemsetAsync(a->cnt_dev, 0, sizeof(AdaptCounts), s->stream), "counts");
    ACK(cudaMemcpyAsync(a->o_ref0, a->ref0, sizeof(int) * a->cnb0, cudaMemcpyDeviceToDevice, s->stream), "snapshot");
    ACK(cudaMemcpyAsync(a->o_fof0, a->fof0, sizeof(int) * a->cnb0, cudaMemcpyDeviceToDevice, s->stream), "snapshot");
    ACK(cudaMemcpyAsync(a->o_l1grid, a->l1grid, sizeof(int) * a->NG1, cudaMemcpyDeviceToDevice, s->stream), "snapshot");
    ACK(cudaMemcpyAsync(a->o_ref1, a->ref1, sizeof(int) * a->cap1, cudaMemcpyDeviceToDevice, s->stream), "snapshot");
    ACK(cudaMemcpyAsync(a->o_fof1, a->fof1, sizeof(int) * a->cap1, cudaMemcpyDeviceToDevice, s->stream), "snapshot");
    TRY(mark_l0_by_sensor(s));
    TRY(build_l1(s, true));
    if (a->nf1) {
        AmrLaunch L;
        L.nblocks = a->nf1;
        L.in = a->f1a;
        L.out = a->f1b;
        L.aux = a->c0a;
        L.t0 = a->pcb;
        L.t1 = a->oct;
        L.t2 = a->o_ref0;
        L.t3 = a->o_fof0;
        L.cgx = a->cgx;
        L.n = a->N;
        L.scale = float(a->nqs01);
        TRY(launch(s, OP_SEED_L1, L));
        std::swap(a->f1a, a->f1b);
    }
    a->nref1 = a->nf2 = 0;
    if (a->nf1) {
        TRY(sensor(s, 1));
        ACK(adapt_deepmask(a->f1pos, a->l1grid, a->l1gx, a->nf1, a->deep, s->stream), "deepmask");
        ACK(cudaMemsetAsync(a->ref1, 0, sizeof(int) * a->cap1, s->stream), "memset ref1");
        ACK(adapt_threshold_mark(a->sen1, a->deep, a->nf1, c.frac2, a->cap_nref1, a->ref1, a->cnt_dev, 1, s->stream),
            "threshold L1");
        TRY(buffer_l1(s));
        ACK(adapt_scan_l2(a->ref1, a->nf1, a->rank, a->cnt_dev, s->stream), "scan L2");
        TRY(read_counts(s));
        a->nref1 = a->cnt_host->nref1;
        a->nf2 = a->cnt_host->nf2;
        a->ndeep = a->cnt_host->ndeep;
        a->hw_nf2 = std::max(a->hw_nf2, (long long)a->nf2);
        if (a->nf2 > a->cap2) TRY(grow_l2(s, a->nf2));  // on failure the solver needs jp_init_tgv
        ACK(cudaMemsetAsync(a->fof1, 0xFF, sizeof(int) * a->cap1, s->stream), "memset fof1");
        if (a->nref1)
            ACK(adapt_scatter_l2(a->ref1, a->rank, a->nf1, a->cap2, a->fof1, a->rl1, a->l2pl1, a->l2oct, a->cnt_dev,
                                 s->stream), "scatter L2");
        if (a->nf2) {
            AmrLaunch L;
            L.nblocks = a->nf2;
            L.in = a->f2a;
            L.out = a->f2b;
            L.aux = a->f1a;
            L.t0 = a->l2pl1;
            L.t1 = a->l2oct;
            L.t2 = a->f1pos;
            L.t3 = a->o_l1grid;
            L.t4 = a->o_ref1;
            L.t5 = a->o_fof1;
            L.t6 = a->l1grid;
            L.l1gx = a->l1gx;
            L.n1 = a->N1;
            L.scale = float(a->nqs12);
            TRY(launch(s, OP_SEED_L2, L));
            std::swap(a->f2a, a->f2b);
        }
    }
    TRY(neighbour_tables(s));
    TRY(skins(s));
    return JP_OK;
}

cudaError_t AmrFork::create(cudaStream_t like) {
    int prio = 0;
    cudaError_t e = cudaStreamGetPriority(like, &prio);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&side, cudaStreamNonBlocking, prio);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&join, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&fork2, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&join2, cudaEventDisableTiming);
    return e;
}

// the side stream's work is always joined into its main stream, so nothing on it outlives that
void AmrFork::destroy() {
    if (side) cudaStreamSynchronize(side);
    if (fork) cudaEventDestroy(fork);
    if (join) cudaEventDestroy(join);
    if (fork2) cudaEventDestroy(fork2);
    if (join2) cudaEventDestroy(join2);
    if (side) cudaStreamDestroy(side);
    side = nullptr;
    fork = join = fork2 = join2 = nullptr;
}

// Takes a side branch back into a stream (or a capture) on every return, errors included.
struct JoinOnExit {
    cudaStream_t st;
    cudaEvent_t ev;
    bool pending = true;
    jp_status now() {
        pending = false;
        ACK(cudaStreamWaitEvent(st, ev, 0), "join");
        return JP_OK;
    }
    ~JoinOnExit() {
        if (pending) cudaStreamWaitEvent(st, ev, 0);
    }
};

// the coarse step and the level-1 ghosts it feeds (prolongation sources of level 0, level-1 fill)
static jp_status level0_chain(jp_solver* s, cudaStream_t st) {
    AmrState* a = s->amr;
    const int* cnt = a->step_cnt;
    TRY(step_l0(s, st));
    if (s->cfg.flags & JP_FLAG_SKIP_PREP) return JP_OK;
    AmrLaunch L;
    L.nblocks = interface_cells(a->MB) * a->cnb0;
    L.nlim = cnt + SC_PREP0;
    L.in = a->c0a;
    L.out = a->prep0;
    L.list = a->pc0;
    L.scale = float(a->nqs01);
    L.t0 = cnt + SC_FILL1;
    TRY(launch(s, OP_PREP, L, st));
    AmrLaunch F;
    F.nblocks = a->SH * a->cap1;
    F.list = a->fl1;
    F.nlim = cnt + SC_FILL1;
    F.in = a->prep0;
    F.out = a->gh1;
    F.t0 = a->pcb;
    F.t1 = a->oct;
    F.cgx = a->cgx;
    F.n = a->N;
    return launch(s, OP_FILL_L1, F, st);
}

// base_step (src/tgv3d_amr.cu:821-837): coarse once, level 1 twice, level 2 four times, restricting
// level 2 into level 1 after each pair and level 1 into level 0 at the end.  Launch shapes depend on
// the pool capacities only; the kernels read the block counts of the current grid on the device.
//
// The level-0 chain (coarse step, its prolongation sources, the level-1 ghost fill) and the first
// level-2 pair (level-1 sources, level-2 fill, two level-2 substeps restricting into level 1) share
// no array: 2:1 balance keeps level 2 away from level 0, so level-2 ghosts come from level 1 alone.
// They meet at the first level-1 substep, which reads the level-1 ghosts and the restricted level 1.
// The level-0 chain therefore runs on a side stream (a branch of the captured graph), and the short
// latency-bound fills and preps of one chain overlap the bandwidth-bound steps of the other.  Every
// kernel sees the same inputs as in one stream: results are unchanged.
static jp_status base_step(jp_solver* s) {
    AmrState* a = s->amr;
    const bool skip_prep = s->cfg.flags & JP_FLAG_SKIP_PREP, skip_restrict = s->cfg.flags & JP_FLAG_SKIP_RESTRICT;
    // restrictions fused into the last substep of each fine level (same values, one pass less)
    const bool fuse = !skip_restrict && can_fuse_restrict(a->MB);
    const int* cnt = a->step_cnt;
    ACK(cudaEventRecord(a->fk.fork, s->stream), "fork");
    ACK(cudaStreamWaitEvent(a->fk.side, a->fk.fork, 0), "fork");
    const jp_status st0 = level0_chain(s, a->fk.side);
    ACK(cudaEventRecord(a->fk.join, a->fk.side), "join");
    JoinOnExit join{s->stream, a->fk.join};
    TRY(st0);
    // The first level-1 substep in two parts: its skin blocks (the only ones the next level-2 pair
    // reads, through the prep cells, and the only ones that pair restricts into), then the others on
    // the side branch, beside the whole second level-2 pair; they join before the last level-1
    // substep.  Each block is stepped as in one launch (rows mapping).
    const bool split = a->MB >= 8 && (a->vec ? a->vec : default_step_vec(a->MB)) == 4;
    JoinOnExit join2{s->stream, a->fk.join2, false};
    for (int s1 = 0; s1 < 2; ++s1) {
        if (!skip_prep) {
            AmrLaunch L;
            L.nblocks = interface_cells(a->MB) * a->cap1;
            L.nlim = cnt + SC_PREP1;
            L.in = a->f1a;
            L.out = a->prep1;
            L.list = a->pc1;
            L.scale = float(a->nqs12);
            L.t0 = cnt + SC_FILL2;
            TRY(launch(s, OP_PREP, L));
            AmrLaunch F;
            F.nblocks = a->SH * a->cap2;
            F.list = a->fl2;
            F.nlim = cnt + SC_FILL2;
            F.in = a->prep1;
            F.out = a->gh2;
            F.t0 = a->l2pl1;
            F.t1 = a->l2oct;
            F.t2 = a->f1pos;
            F.t3 = a->l1grid;
            F.l1gx = a->l1gx;
            F.n1 = a->N1;
            TRY(launch(s, OP_FILL_L2, F));
        }
        for (int s2 = 0; s2 < 2; ++s2) {
            AmrLaunch S;
            S.nblocks = a->cap2;
            S.nlim = cnt + SC_NF2;
            S.in = a->f2a;
            S.out = a->f2b;
            S.aux = a->gh2;
            S.nbt = a->nb2;
            S.t0 = a->l2pl1;
            S.t1 = a->l2oct;
            S.omega = a->om2;
            S.tpb = a->tpb;
            S.vec = a->vec;
            if (s2 == 1 && fuse) {  // last level-2 substep restricts itself into level 1
                S.out2 = a->f1a;
                S.scale = float(a->nqi21);
            }
            TRY(launch(s, OP_STEP_L2, S));
            std::swap(a->f2a, a->f2b);
        }
        if (!skip_restrict && !fuse) {
            AmrLaunch R;
            R.nblocks = (a->cap2 + 7) / 8;
            R.nlim = cnt + SC_NREF1;
            R.out = a->f1a;
            R.in = a->f2a;
            R.list = a->rl1;
            R.t0 = a->fof1;
            R.scale = float(a->nqi21);
            TRY(launch(s, OP_RESTRICT, R));
        }
        if (s1 == 0) TRY(join.now());
        if (s1 == 1 && join2.pending) TRY(join2.now());
        AmrLaunch S;
        S.nblocks = a->cap1;
        S.nlim = cnt + SC_NF1;
        S.in = a->f1a;
        S.out = a->f1b;
        S.aux = a->gh1;
        S.nbt = a->nb1;
        S.t0 = a->pcb;
        S.t1 = a->oct;
        S.omega = a->om1;
        S.tpb = a->tpb;
        S.vec = a->vec;
        if (s1 == 1 && fuse) {  // last level-1 substep restricts itself into the coarse level
            S.out2 = a->c0a;
            S.scale = float(a->nqi10);
        }
        if (s1 == 0 && split) {
            AmrLaunch K = S;  // the skin blocks
            K.list = a->skin1;
            K.nlim = cnt + SC_SKIN1;
            TRY(launch(s, OP_STEP_L1, K));
            ACK(cudaEventRecord(a->fk.fork2, s->stream), "fork");
            ACK(cudaStreamWaitEvent(a->fk.side, a->fk.fork2, 0), "fork");
            AmrLaunch R = S;  // the others, on the side branch
            R.list = a->rest1;
            R.nlim = cnt + SC_REST1;
            const jp_status sr = launch(s, OP_STEP_L1, R, a->fk.side);
            ACK(cudaEventRecord(a->fk.join2, a->fk.side), "join");
            join2.pending = true;
            TRY(sr);
        } else {
            TRY(launch(s, OP_STEP_L1, S));
        }
        std::swap(a->f1a, a->f1b);
    }
    if (skip_restrict || fuse) return JP_OK;
    AmrLaunch R;
    R.nblocks = (a->cap1 + 7) / 8;
    R.nlim = cnt + SC_NREF0;
    R.out = a->c0a;
    R.in = a->f1a;
    R.list = a->rl0;
    R.t0 = a->fof0;
    R.scale = float(a->nqi10);
    return launch(s, OP_RESTRICT, R);
}

// One coarse step of many AMR solves with one launch per stage over all of them (base_step's
// sequence, each launch an AmrBatch of up to kAmrBatchMax members).  The members share block edge,
// storage, step threads and skip flags (amr_batch_compatible).
jp_status amr_batch_step(const std::vector<jp_solver*>& ms, cudaStream_t st, const AmrFork* fk) {
    if (ms.empty()) return JP_OK;
    const AmrState* a0 = ms[0]->amr;
    const int flags = ms[0]->cfg.flags;
    const bool skip_prep = flags & JP_FLAG_SKIP_PREP, skip_restrict = flags & JP_FLAG_SKIP_RESTRICT;
    const bool fuse = !skip_restrict && can_fuse_restrict(a0->MB);
    // one stage over all members on stream `on`: fill() sets a member's item and returns its CTAs
    // (0: nothing)
    auto run_on = [&](cudaStream_t on, int op, bool fused, auto fill) -> jp_status {
        for (size_t i0 = 0; i0 < ms.size(); i0 += kAmrBatchMax) {
            AmrBatch B;
            B.vec = a0->vec;
            for (size_t i = i0; i < ms.size() && i < i0 + kAmrBatchMax; ++i) {
                AmrItem& it = B.it[B.count];
                std::memset(&it, 0, sizeof it);
                const int n = fill(ms[i]->amr, it);
                if (n <= 0) continue;
                it.nct = n;
                it.begin = B.total;
                B.total += n;
                ++B.count;
            }
            cudaError_t e = amr_batch_launch(a0->storage, a0->MB, op, a0->tpb, fused, B, on);
            if (e != cudaSuccess) return cuda_fail(e, "batched AMR launch");
        }
        return JP_OK;
    };
    auto run = [&](int op, bool fused, auto fill) { return run_on(st, op, fused, fill); };
    // the level-0 chain, on the side stream when there is one (base_step: it shares no array with
    // the first level-2 pair and joins before the first level-1 substep)
    const cudaStream_t s0 = fk ? fk->side : st;
    if (fk) {
        ACK(cudaEventRecord(fk->fork, st), "fork");
        ACK(cudaStreamWaitEvent(fk->side, fk->fork, 0), "fork");
    }
    auto level0 = [&]() -> jp_status {
        TRY(run_on(s0, OP_STEP_L0, false, [](AmrState* a, AmrItem& it) {
            it.in = a->c0a;
            it.out = a->c0b;
            it.cgx = a->cgx;
            it.omega = a->om0;
            return a->cnb0;
        }));
        for (jp_solver* m : ms) std::swap(m->amr->c0a, m->amr->c0b);
        if (skip_prep) return JP_OK;
        TRY(run_on(s0, OP_PREP, false, [](AmrState* a, AmrItem& it) {
            it.in = a->c0a;
            it.out = a->prep0;
            it.list = a->pc0;
            it.scale = float(a->nqs01);
            it.nlim = a->step_cnt + SC_PREP0;
            it.t0 = a->step_cnt + SC_FILL1;
            return std::min((interface_cells(a->MB) * a->cnb0 + 255) / 256, kBatchPrepCtas);
        }));
        return run_on(s0, OP_FILL_L1, false, [](AmrState* a, AmrItem& it) {
            it.in = a->prep0;
            it.out = a->gh1;
            it.t0 = a->pcb;
            it.t1 = a->oct;
            it.cgx = a->cgx;
            it.n = a->N;
            it.list = a->fl1;
            it.nlim = a->step_cnt + SC_FILL1;
            return std::min((a->SH * a->cap1 + 255) / 256, kBatchPrepCtas);
        });
    };
    const jp_status st0 = level0();
    if (fk) ACK(cudaEventRecord(fk->join, fk->side), "join");
    JoinOnExit join{st, fk ? fk->join : nullptr, fk != nullptr};
    TRY(st0);
    for (int s1 = 0; s1 < 2; ++s1) {
        if (!skip_prep) {
            TRY(run(OP_PREP, false, [](AmrState* a, AmrItem& it) {
                it.in = a->f1a;
                it.out = a->prep1;
                it.list = a->pc1;
                it.scale = float(a->nqs12);
                it.nlim = a->step_cnt + SC_PREP1;
                it.t0 = a->step_cnt + SC_FILL2;
                return std::min((interface_cells(a->MB) * a->cap1 + 255) / 256, kBatchPrepCtas);
            }));
            TRY(run(OP_FILL_L2, false, [](AmrState* a, AmrItem& it) {
                it.in = a->prep1;
                it.out = a->gh2;
                it.t0 = a->l2pl1;
                it.t1 = a->l2oct;
                it.t2 = a->f1pos;
                it.t3 = a->l1grid;
                it.l1gx = a->l1gx;
                it.n1 = a->N1;
                it.list = a->fl2;
                it.nlim = a->step_cnt + SC_FILL2;
                return std::min((a->SH * a->cap2 + 255) / 256, kBatchPrepCtas);
            }));
        }
        for (int s2 = 0; s2 < 2; ++s2) {
            const bool f = s2 == 1 && fuse;  // last level-2 substep restricts itself into level 1
            TRY(run(OP_STEP_L2, f, [f](AmrState* a, AmrItem& it) {
                it.in = a->f2a;
                it.out = a->f2b;
                it.aux = a->gh2;
                it.nbt = a->nb2;
                it.t0 = a->l2pl1;
                it.t1 = a->l2oct;
                it.omega = a->om2;
                it.nlim = a->step_cnt + SC_NF2;
                if (f) {
                    it.out2 = a->f1a;
                    it.scale = float(a->nqi21);
                }
                return a->cap2;
            }));
            for (jp_solver* m : ms) std::swap(m->amr->f2a, m->amr->f2b);
        }
        if (!skip_restrict && !fuse) {
            TRY(run(OP_RESTRICT, false, [](AmrState* a, AmrItem& it) {
                it.out = a->f1a;
                it.in = a->f2a;
                it.list = a->rl1;
                it.t0 = a->fof1;
                it.scale = float(a->nqi21);
                it.nlim = a->step_cnt + SC_NREF1;
                return (a->cap2 + 7) / 8;
            }));
        }
        if (s1 == 0 && join.pending) TRY(join.now());
        const bool f = s1 == 1 && fuse;  // last level-1 substep restricts itself into the coarse level
        TRY(run(OP_STEP_L1, f, [f](AmrState* a, AmrItem& it) {
            it.in = a->f1a;
            it.out = a->f1b;
            it.aux = a->gh1;
            it.nbt = a->nb1;
            it.t0 = a->pcb;
            it.t1 = a->oct;
            it.omega = a->om1;
            it.nlim = a->step_cnt + SC_NF1;
            if (f) {
                it.out2 = a->c0a;
                it.scale = float(a->nqi10);
            }
            return a->cap1;
        }));
        for (jp_solver* m : ms) std::swap(m->amr->f1a, m->amr->f1b);
    }
    if (!skip_restrict && !fuse) {
        TRY(run(OP_RESTRICT, false, [](AmrState* a, AmrItem& it) {
            it.out = a->c0a;
            it.in = a->f1a;
            it.list = a->rl0;
            it.t0 = a->fof0;
            it.scale = float(a->nqi10);
            it.nlim = a->step_cnt + SC_NREF0;
            return (a->cap1 + 7) / 8;
        }));
    }
    for (jp_solver* m : ms) ++m->step_count;
    return JP_OK;
}

bool amr_persist_ok(const jp_solver* s) {
    const AmrState* a = s->amr;
    const bool skip_restrict = s->cfg.flags & JP_FLAG_SKIP_RESTRICT;
    return amr_persist_supported(a->MB, a->vec, !skip_restrict && can_fuse_restrict(a->MB),
                                 (s->cfg.flags & JP_FLAG_SKIP_PREP) != 0);
}

// base_step's sequence for many solves and several coarse steps each in one cooperative launch per
// kAmrBatchMax solves (amr_persist.cuh): the members' arrays and device counts, ordered by their step
// counts (descending), and afterwards the coarse ping-pong of every member with an odd count swapped.
jp_status amr_persist_steps(const std::vector<jp_solver*>& ms, const std::vector<long long>& steps, cudaStream_t st,
                            PersistSync* sync, int nsync, long long limit_ns, int grid, int* launches) {
    if (ms.size() != steps.size()) return fail(JP_ERR_INVALID, "persistent steps: %zu members, %zu step counts",
                                               ms.size(), steps.size());
    std::vector<size_t> order;
    for (size_t i = 0; i < ms.size(); ++i) {
        if (steps[i] < 0 || steps[i] > (1LL << 20)) return fail(JP_ERR_INVALID, "persistent steps: %lld coarse steps",
                                                              steps[i]);
        if (!amr_persist_ok(ms[i]) || !amr_batch_compatible(ms[0], ms[i]))
            return fail(JP_ERR_UNSUPPORTED, "persistent coarse steps: MB=8, rows, fused restrictions, one storage");
        if (steps[i] > 0) order.push_back(i);
    }
    std::stable_sort(order.begin(), order.end(), [&](size_t x, size_t y) { return steps[x] > steps[y]; });
    const size_t chunks = (order.size() + kAmrBatchMax - 1) / kAmrBatchMax;
    if ((long long)chunks > nsync) return fail(JP_ERR_CAPACITY, "persistent steps: %zu launches, %d barrier slots",
                                              chunks, nsync);
    for (size_t c = 0; c < chunks; ++c) {
        AmrPersist P;
        P.sync = sync + c;
        P.limit_ns = limit_ns;
        for (size_t k = c * kAmrBatchMax; k < order.size() && k < (c + 1) * kAmrBatchMax; ++k) {
            const AmrState* a = ms[order[k]]->amr;
            PersistMember& M = P.m[P.count++];
            std::memset(&M, 0, sizeof M);
            M.c0[0] = a->c0a;
            M.c0[1] = a->c0b;
            M.prep0 = a->prep0;
            M.gh1 = a->gh1;
            M.f1a = a->f1a;
            M.f1b = a->f1b;
            M.prep1 = a->prep1;
            M.gh2 = a->gh2;
            M.f2a = a->f2a;
            M.f2b = a->f2b;
            M.pc0 = a->pc0;
            M.pc1 = a->pc1;
            M.fl1 = a->fl1;
            M.fl2 = a->fl2;
            M.pcb = a->pcb;
            M.oct = a->oct;
            M.l2pl1 = a->l2pl1;
            M.l2oct = a->l2oct;
            M.f1pos = a->f1pos;
            M.l1grid = a->l1grid;
            M.nb1 = a->nb1;
            M.nb2 = a->nb2;
            M.n_prep0 = a->step_cnt + SC_PREP0;
            M.n_fill1 = a->step_cnt + SC_FILL1;
            M.n_prep1 = a->step_cnt + SC_PREP1;
            M.n_fill2 = a->step_cnt + SC_FILL2;
            M.n_f1 = a->step_cnt + SC_NF1;
            M.n_f2 = a->step_cnt + SC_NF2;
            M.cgx = a->cgx;
            M.n = a->N;
            M.l1gx = a->l1gx;
            M.n1 = a->N1;
            M.cnb0 = a->cnb0;
            M.steps = (int)steps[order[k]];
            M.om0 = a->om0;
            M.om1 = a->om1;
            M.om2 = a->om2;
            M.nqs01 = float(a->nqs01);
            M.nqs12 = float(a->nqs12);
            M.nqi21 = float(a->nqi21);
            M.nqi10 = float(a->nqi10);
            P.maxsteps = std::max(P.maxsteps, M.steps);
        }
        ACK(cudaMemsetAsync(P.sync, 0, kPersistResetBytes, st), "persistent barrier reset");
        ACK(amr_persist_launch(ms[0]->amr->storage, ms[0]->amr->MB, P, grid, st, nullptr), "persistent coarse steps");
        if (launches) ++*launches;
    }
    for (size_t i = 0; i < ms.size(); ++i) {
        if (steps[i] & 1) std::swap(ms[i]->amr->c0a, ms[i]->amr->c0b);
        ms[i]->step_count += steps[i];
    }
    return JP_OK;
}

bool amr_batch_compatible(const jp_solver* a, const jp_solver* b) {
    const int skip = JP_FLAG_SKIP_PREP | JP_FLAG_SKIP_RESTRICT;
    return a->amr->MB == b->amr->MB && a->amr->storage == b->amr->storage && a->amr->tpb == b->amr->tpb &&
           a->amr->vec == b->amr->vec && (a->cfg.flags & skip) == (b->cfg.flags & skip);
}

// base_step replayed from a captured graph (captured on first use for each parity combination)
static jp_status graph_step(jp_solver* s, cudaStream_t on = nullptr) {
    AmrState* a = s->amr;
    const int key = (a->c0a == a->c0_home ? 0 : 1) | (a->f1a == a->f1_home ? 0 : 2) | (a->f2a == a->f2_home ? 0 : 4);
    if (!a->graph[key]) {
        float *c0a = a->c0a, *c0b = a->c0b, *f1a = a->f1a, *f1b = a->f1b, *f2a = a->f2a, *f2b = a->f2b;
        ACK(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
        jp_status st = base_step(s);
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(s->stream, &g);
        // the capture only recorded the step; the replay below performs it
        a->c0a = c0a;
        a->c0b = c0b;
        a->f1a = f1a;
        a->f1b = f1b;
        a->f2a = f2a;
        a->f2b = f2b;
        if (st != JP_OK) {
            if (g) cudaGraphDestroy(g);
            return st;
        }
        if (e != cudaSuccess) return cuda_fail(e, "end capture");
        e = cudaGraphInstantiate(&a->graph[key], g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return cuda_fail(e, "graph instantiate");
    }
    ACK(cudaGraphLaunch(a->graph[key], on ? on : s->stream), "graph launch");
    std::swap(a->c0a, a->c0b);  // the fine levels return to their buffers within the step
    return JP_OK;
}

// One coarse step replayed from the solver's captured graph on another stream `st` (ordered there
// like a batched step; the capture itself runs on the solver's idle stream).
jp_status amr_graph_step_on(jp_solver* s, cudaStream_t st) {
    TRY(graph_step(s, st));
    ++s->step_count;
    return JP_OK;
}

// ---- lifecycle -------------------------------------------------------------------------------------

jp_status amr_create(jp_solver* s) {
    TRY(common_setup(s));
    const jp_config& c = s->cfg;
    if (c.storage != JP_FP32 && c.storage != JP_FP16 && c.storage != JP_BF16)
        return fail(JP_ERR_UNSUPPORTED, "AMR solver: FP32, FP16 or BF16 storage (FP64 is uniform only)");
    if (c.flags & JP_FLAG_INPLACE) return fail(JP_ERR_UNSUPPORTED, "in-place streaming is for the uniform cube only");
    if (c.l1_mode < 0 || c.l1_mode > 2 || c.l2_mode < 0 || c.l2_mode > 2) return fail(JP_ERR_INVALID, "bad refine mode");
    if (c.threads_per_block && !step_tpb_supported(c.mb, c.threads_per_block))
        return fail(JP_ERR_INVALID, "threads_per_block %d does not split a block of edge %d (MB=4: 64; 8, 16: 128, 256, 512)",
                    c.threads_per_block, c.mb);
    if (c.vec && !step_vec_supported(c.mb, c.vec))
        return fail(JP_ERR_INVALID, "vec %d: the AMR fine steps take 1 cell per thread, or 4 (rows) at MB >= 8", c.vec);
    AmrState* a = new (std::nothrow) AmrState();
    if (!a) return fail(JP_ERR_NOMEM, "host allocation");
    s->amr = a;
    a->owner = s;
    a->storage = c.storage;
    a->elem = storage_elem(c.storage);
    a->tpb = c.threads_per_block;
    a->vec = c.vec;
    a->MB = c.mb;
    a->MB3 = c.mb * c.mb * c.mb;
    a->SH = shell_cells(c.mb);
    a->N = c.n;
    a->cgx = c.n / c.mb;
    a->cnb0 = a->cgx * a->cgx * a->cgx;
    a->l1gx = 2 * a->cgx;
    a->N1 = 2 * c.n;
    a->N2 = 4 * c.n;
    a->NG1 = a->l1gx * a->l1gx * a->l1gx;
    a->l1mode = c.l1_mode;
    a->l2mode = c.l2_mode;
    a->dynamic = c.l1_mode == JP_REFINE_SENSOR || c.l2_mode == JP_REFINE_SENSOR;
    const double tau0 = s->info.tau;
    a->tau0 = tau0;
    a->tau1 = 2.0 * tau0 - 0.5;
    a->tau2 = 2.0 * a->tau1 - 0.5;
    a->om0 = float(1.0 / a->tau0);
    a->om1 = float(1.0 / a->tau1);
    a->om2 = float(1.0 / a->tau2);
    a->nqs01 = (a->tau1 - 1.0) / (2.0 * (a->tau0 - 1.0));
    a->nqi10 = (2.0 * (a->tau0 - 1.0)) / (a->tau1 - 1.0);
    a->nqs12 = (a->tau2 - 1.0) / (2.0 * (a->tau1 - 1.0));
    a->nqi21 = (2.0 * (a->tau1 - 1.0)) / (a->tau2 - 1.0);
    s->cells = (long long)a->cnb0 * a->MB3;
    s->n = c.n;
    const size_t blk = (size_t)Q * a->MB3;
    TRY(dalloc(a, &a->c0a, pf(a, (size_t)a->cnb0 * blk), "cudaMalloc c0"));
    TRY(dalloc(a, &a->c0b, pf(a, (size_t)a->cnb0 * blk), "cudaMalloc c0"));
    TRY(dalloc(a, &a->sen0, (size_t)a->cnb0, "cudaMalloc sen0"));
    // HBM budget for the fine pools: --maxgb, else 75% of free memory (src/tgv3d_amr.cu:684-688)
    size_t freeB = 0, totB = 0;
    ACK(cudaMemGetInfo(&freeB, &totB), "cudaMemGetInfo");
    a->budget = c.max_gb > 0 ? c.max_gb * double(1ull << 30) : double(freeB) * 0.75;
    a->PB = (size_t)Q * 4 * (2 * a->MB3 + (a->MB + 2) * (a->MB + 2) * (a->MB + 2));
    a->cap_nref0 = (a->l1mode == JP_REFINE_ALL) ? a->cnb0
                                                : std::min(a->cnb0, std::max(1, (int)std::ceil(c.frac1 * a->cnb0 * 1.4)));
    while (a->cap_nref0 > 1 && !pool_fits(a, 8LL * a->cap_nref0, 0)) a->cap_nref0--;
    a->cap1 = 8 * a->cap_nref0;
    TRY(dalloc(a, &a->f1a, pf(a, (size_t)a->cap1 * blk), "cudaMalloc f1"));
    TRY(dalloc(a, &a->f1b, pf(a, (size_t)a->cap1 * blk), "cudaMalloc f1"));
    TRY(dalloc(a, &a->gh1, pf(a, (size_t)a->cap1 * Q * a->SH), "cudaMalloc gh1"));
    TRY(dalloc(a, &a->prep0, pf(a, (size_t)a->cnb0 * blk), "cudaMalloc prep0"));
    TRY(dalloc(a, &a->prep1, pf(a, (size_t)a->cap1 * blk), "cudaMalloc prep1"));
    int** cnb_tabs[] = {&a->ref0, &a->fof0, &a->o_ref0, &a->o_fof0, &a->skin0};
    for (int** t : cnb_tabs) TRY(dalloc(a, t, (size_t)a->cnb0, "cudaMalloc table"));
    int** cap_tabs[] = {&a->pcb, &a->oct, &a->rl0, &a->f1pos, &a->ref1, &a->fof1, &a->o_ref1, &a->o_fof1,
                        &a->rl1, &a->skin1, &a->rest1, &a->deep};
    for (int** t : cap_tabs) TRY(dalloc(a, t, (size_t)a->cap1, "cudaMalloc table"));
    TRY(dalloc(a, &a->l1grid, (size_t)a->NG1, "cudaMalloc l1grid"));
    TRY(dalloc(a, &a->o_l1grid, (size_t)a->NG1, "cudaMalloc l1grid"));
    TRY(dalloc(a, &a->rank, (size_t)std::max(a->cnb0, a->cap1), "cudaMalloc rank"));
    TRY(dalloc(a, &a->flags, (size_t)a->cnb0 + a->cap1, "cudaMalloc flags"));
    TRY(dalloc(a, &a->sen1, (size_t)a->cap1, "cudaMalloc sen1"));
    TRY(dalloc(a, &a->nb1, (size_t)a->cap1 * 27, "cudaMalloc nb1"));
    TRY(dalloc(a, &a->fl1, (size_t)a->SH * a->cap1, "cudaMalloc fl1"));
    TRY(dalloc(a, &a->pl1, 2 * (size_t)a->cap1, "cudaMalloc pl1"));
    TRY(dalloc(a, &a->pl0, 2 * (size_t)a->cnb0, "cudaMalloc pl0"));
    TRY(dalloc(a, &a->pc1, (size_t)interface_cells(a->MB) * a->cap1, "cudaMalloc pc1"));
    TRY(dalloc(a, &a->pc0, (size_t)interface_cells(a->MB) * a->cnb0, "cudaMalloc pc0"));
    TRY(dalloc(a, &a->step_cnt, SC_ALL, "cudaMalloc step counts"));
    a->step_cnt_host = (int*)pinned_slot_alloc();
    if (!a->step_cnt_host) return fail(JP_ERR_NOMEM, "pinned host slot");
    TRY(dalloc(a, &a->cnt_dev, 1, "cudaMalloc counts"));
    static_assert(sizeof(AdaptCounts) <= 256, "counts exceed a pinned slot");
    a->cnt_host = (AdaptCounts*)pinned_slot_alloc();
    s->diag_host = (double*)pinned_slot_alloc();
    if (!a->cnt_host || !s->diag_host) return fail(JP_ERR_NOMEM, "pinned host slot");
    ACK(dev_alloc(s, (void**)&s->partials, sizeof(double) * kDiagPartials), "cudaMalloc partials");
    ACK(dev_alloc(s, (void**)&s->diag_dev, sizeof(double) * 3), "cudaMalloc diag");
    ACK(a->fk.create(s->stream), "side stream");
    ACK(cudaMemsetAsync(a->fof1, 0xFF, sizeof(int) * a->cap1, s->stream), "memset");
    ACK(cudaMemsetAsync(a->ref1, 0, sizeof(int) * a->cap1, s->stream), "memset");
    ACK(cudaMemsetAsync(a->l1grid, 0xFF, sizeof(int) * a->NG1, s->stream), "memset");
    TRY(launch(s, OP_WARM, AmrLaunch()));
    if (s->cfg.flags & JP_FLAG_DEFER_INIT) return JP_OK;
    return amr_init(s);
}

void amr_destroy(jp_solver* s) {
    AmrState* a = s->amr;
    if (!a) return;
    reset_graphs(a);
    for (void* p : a->owned) dev_free(s, p);
    a->fk.destroy();
    pinned_slot_free(a->cnt_host);
    pinned_slot_free(a->step_cnt_host);
    dev_free(s, a->field);
    delete a;
    s->amr = nullptr;
}

// TGV state on the coarse grid and the initial build (with the sensor override, if one is set)
jp_status amr_init(jp_solver* s) {
    AmrState* a = s->amr;
    reset_graphs(a);
    AmrLaunch L;
    L.nblocks = a->cnb0;
    L.out = a->c0a;
    L.cgx = a->cgx;
    L.u0 = s->cfg.u0;
    L.kf = s->info.kf;
    TRY(launch(s, OP_INIT, L));
    a->hw_nf1 = a->hw_nf2 = 0;
    TRY(initial_build(s));
    ACK(wait_stream(s), "initial build");
    skins_landed(a);
    reset_graphs(a);  // the level-2 pool was allocated anew
    s->step_count = 0;
    s->initialized = true;
    update_bytes(s);
    return JP_OK;
}

jp_status amr_step(jp_solver* s, int64_t nsteps) {
    const bool graph = s->cfg.flags & JP_FLAG_GRAPH;
    for (int64_t i = 0; i < nsteps; ++i) {
        TRY(graph ? graph_step(s) : base_step(s));
        ++s->step_count;
    }
    return JP_OK;
}

jp_status amr_set_step_map(jp_solver* s, int vec, int tpb) {
    if (tpb && !step_tpb_supported(s->amr->MB, tpb)) return fail(JP_ERR_INVALID, "threads_per_block %d", tpb);
    if (vec && !step_vec_supported(s->amr->MB, vec)) return fail(JP_ERR_INVALID, "vec %d", vec);
    reset_graphs(s->amr);
    s->amr->tpb = tpb;
    s->amr->vec = vec;
    s->cfg.threads_per_block = tpb;
    s->cfg.vec = vec;
    return JP_OK;
}

jp_status amr_regrid(jp_solver* s) {
    TRY(regrid(s));  // the captured steps stay valid unless a pool grew (grow_l1/grow_l2 drop them)
    ACK(wait_stream(s), "regrid");
    skins_landed(s->amr);
    return JP_OK;
}

static jp_status composite(jp_solver* s, cudaStream_t st = nullptr) {
    AmrState* a = s->amr;
    if (!a->field) ACK(dev_alloc(s, (void**)&a->field, sizeof(float) * 4 * (size_t)a->N2 * a->N2 * a->N2), "cudaMalloc composite");
    AmrLaunch L;
    if (st) {  // on another stream: the launch below overrides the solver's own
        L.in = a->c0a;
        L.aux = a->f1a;
        L.aux2 = a->f2a;
        L.out = a->field;
        L.t0 = a->ref1;
        L.t1 = a->fof1;
        L.t2 = a->l1grid;
        L.cgx = a->cgx;
        L.l1gx = a->l1gx;
        L.n2 = a->N2;
        L.st = st;
        cudaError_t e = amr_launch(a->storage, a->MB, OP_COMPOSITE, L);
        if (e != cudaSuccess) return cuda_fail(e, "AMR kernel launch");
        return JP_OK;
    }
    L.in = a->c0a;
    L.aux = a->f1a;
    L.aux2 = a->f2a;
    L.out = a->field;
    L.t0 = a->ref1;
    L.t1 = a->fof1;
    L.t2 = a->l1grid;
    L.cgx = a->cgx;
    L.l1gx = a->l1gx;
    L.n2 = a->N2;
    return launch(s, OP_COMPOSITE, L);
}

jp_status amr_get_output_fields(jp_solver* s, float* q, float* speed, float* vel, int64_t count) {
    AmrState* a = s->amr;
    if (count != (int64_t)a->N2 * a->N2 * a->N2) return fail(JP_ERR_INVALID, "count %lld != (4 N0)^3", (long long)count);
    TRY(composite(s));
    return output_fields_from(s, a->field, false, false, a->N2, q, speed, vel);
}

// The composite field the diagnostics need, allocated ahead of an amr_diag_async on another stream.
jp_status amr_prepare_diag(jp_solver* s) {
    AmrState* a = s->amr;
    if (!a->field) ACK(dev_alloc(s, (void**)&a->field, sizeof(float) * 4 * (size_t)a->N2 * a->N2 * a->N2), "cudaMalloc composite");
    ACK(wait_stream(s), "composite field");
    return JP_OK;
}

// Diagnostics of the current state launched on `st` (which must be ordered after the solver's last
// step) and copied into host_out (pinned, 3 doubles) when the stream gets there.
jp_status amr_diag_async(jp_solver* s, cudaStream_t st, double* host_out) {
    AmrState* a = s->amr;
    if (!a->field) return fail(JP_ERR_STATE, "amr_diag_async: composite field not prepared");
    TRY(composite(s, st));
    ACK(launch_diag_field(false, false, a->field, a->N2, s->partials, s->diag_dev, st), "diag");
    ACK(cudaMemcpyAsync(host_out, s->diag_dev, 3 * sizeof(double), cudaMemcpyDeviceToHost, st), "diag D2H");
    return JP_OK;
}

jp_status amr_diag(jp_solver* s, double out[3]) {
    AmrState* a = s->amr;
    TRY(composite(s));
    ACK(launch_diag_field(false, false, a->field, a->N2, s->partials, s->diag_dev, s->stream), "diag");
    ACK(cudaMemcpyAsync(s->diag_host, s->diag_dev, 3 * sizeof(double), cudaMemcpyDeviceToHost, s->stream), "diag D2H");
    ACK(wait_stream(s), "diag");
    out[0] = s->diag_host[0];
    out[1] = s->diag_host[1];
    out[2] = s->diag_host[2];
    return JP_OK;
}

static float* level_ptr(AmrState* a, int level, long long* nblk) {
    switch (level) {
        case 0: *nblk = a->cnb0; return a->c0a;
        case 1: *nblk = a->nf1; return a->f1a;
        case 2: *nblk = a->nf2; return a->f2a;
    }
    *nblk = -1;
    return nullptr;
}

jp_status amr_population_count(const jp_solver* s, int level, int64_t* count) {
    long long nb;
    if (!level_ptr(s->amr, level, &nb) && nb < 0) return fail(JP_ERR_INVALID, "AMR level must be 0, 1 or 2");
    *count = (int64_t)nb * Q * s->amr->MB3;
    return JP_OK;
}

// Populations cross the boundary as unshifted values in the blocked layout [blk][q][MB^3]
// (FP32 storage read as float: the stored bits; shifted formats converted, f = w_q + g).
jp_status amr_get_populations(jp_solver* s, int level, int layout, int dtype, void* host, int64_t count) {
    AmrState* a = s->amr;
    long long nb;
    float* p = level_ptr(a, level, &nb);
    if (nb < 0) return fail(JP_ERR_INVALID, "AMR level must be 0, 1 or 2");
    if (layout != JP_LAYOUT_BLOCKED) return fail(JP_ERR_UNSUPPORTED, "AMR populations are exported in the blocked layout");
    if (count != nb * Q * a->MB3) return fail(JP_ERR_INVALID, "count %lld != %lld", (long long)count, nb * Q * a->MB3);
    if (count == 0) return JP_OK;
    if (dtype == JP_F32 && a->storage == JP_FP32) {
        ACK(cudaMemcpyAsync(host, p, sizeof(float) * count, cudaMemcpyDeviceToHost, s->stream), "D2H");
        ACK(cudaStreamSynchronize(s->stream), "D2H");
        return JP_OK;
    }
    std::vector<unsigned char> raw((size_t)count * a->elem);
    ACK(cudaMemcpyAsync(raw.data(), p, raw.size(), cudaMemcpyDeviceToHost, s->stream), "D2H");
    ACK(cudaStreamSynchronize(s->stream), "D2H");
    for (int64_t i = 0; i < count; ++i) {
        const double v = stored_to_double(a->storage, raw.data(), (size_t)i, int((i / a->MB3) % Q));
        if (dtype == JP_F32) static_cast<float*>(host)[i] = float(v);
        else static_cast<double*>(host)[i] = v;
    }
    return JP_OK;
}

jp_status amr_set_populations(jp_solver* s, int level, int layout, int dtype, const void* host, int64_t count) {
    AmrState* a = s->amr;
    long long nb;
    float* p = level_ptr(a, level, &nb);
    if (nb < 0) return fail(JP_ERR_INVALID, "AMR level must be 0, 1 or 2");
    if (layout != JP_LAYOUT_BLOCKED) return fail(JP_ERR_UNSUPPORTED, "AMR populations are imported in the blocked layout");
    if (count != nb * Q * a->MB3) return fail(JP_ERR_INVALID, "count %lld != %lld", (long long)count, nb * Q * a->MB3);
    if (count == 0) return JP_OK;
    if (dtype == JP_F32 && a->storage == JP_FP32) {
        ACK(cudaMemcpyAsync(p, host, sizeof(float) * count, cudaMemcpyHostToDevice, s->stream), "H2D");
        ACK(cudaStreamSynchronize(s->stream), "H2D");
        return JP_OK;
    }
    std::vector<unsigned char> raw((size_t)count * a->elem);
    for (int64_t i = 0; i < count; ++i) {
        const double v = dtype == JP_F32 ? double(static_cast<const float*>(host)[i]) : static_cast<const double*>(host)[i];
        double_to_stored(a->storage, raw.data(), (size_t)i, int((i / a->MB3) % Q), v);
    }
    ACK(cudaMemcpyAsync(p, raw.data(), raw.size(), cudaMemcpyHostToDevice, s->stream), "H2D");
    ACK(cudaStreamSynchronize(s->stream), "H2D");
    return JP_OK;
}

// ---- state files (jp_save_state / jp_load_state) ---------------------------------------------------
// AMR payload: the host counts and capacities, every block table whole (their sizes follow from the
// capacities, which a load restores first), then the populations of the blocks in use, as stored.
// Prolongation sources, ghosts, sensors and regrid snapshots are recomputed before they are read.
namespace {
struct TableRef {
    int* p;
    size_t n;
};
std::vector<TableRef> state_tables(AmrState* a) {
    const size_t c0 = a->cnb0, c1 = a->cap1, c2 = a->cap2;
    return {{a->ref0, c0}, {a->fof0, c0}, {a->skin0, c0}, {a->pcb, c1}, {a->oct, c1}, {a->rl0, c1},
            {a->f1pos, c1}, {a->ref1, c1}, {a->fof1, c1}, {a->rl1, c1}, {a->skin1, c1}, {a->deep, c1},
            {a->l1grid, (size_t)a->NG1}, {a->l2pl1, c2}, {a->l2oct, c2}, {a->nb1, c1 * 27}, {a->nb2, c2 * 27}};
}
bool fwrite_all(std::FILE* f, const void* p, size_t n) { return std::fwrite(p, 1, n, f) == n; }
bool fread_all(std::FILE* f, void* p, size_t n) { return std::fread(p, 1, n, f) == n; }
}  // namespace

jp_status amr_save_state(jp_solver* s, std::FILE* f) {
    AmrState* a = s->amr;
    ACK(wait_stream(s), "save");
    const int64_t h[16] = {a->cap1, a->cap2, a->cap_nref0, a->cap_nref1, a->nref0, a->nf1, a->nref1, a->nf2,
                           a->n_skin0, a->n_skin1, a->ndeep, a->hw_nf1, a->hw_nf2, 0, 0, 0};
    if (!fwrite_all(f, h, sizeof h)) return fail(JP_ERR_INVALID, "write failed");
    std::vector<int> buf;
    for (const TableRef& t : state_tables(a)) {
        buf.resize(t.n);
        ACK(cudaMemcpy(buf.data(), t.p, sizeof(int) * t.n, cudaMemcpyDeviceToHost), "table D2H");
        if (!fwrite_all(f, buf.data(), sizeof(int) * t.n)) return fail(JP_ERR_INVALID, "write failed");
    }
    const size_t blk = (size_t)Q * a->MB3 * a->elem;
    const std::pair<const void*, size_t> pools[3] = {{a->c0a, (size_t)a->cnb0 * blk}, {a->f1a, (size_t)a->nf1 * blk},
                                                     {a->f2a, (size_t)a->nf2 * blk}};
    std::vector<unsigned char> raw;
    for (const auto& pl : pools) {
        raw.resize(pl.second);
        if (pl.second) ACK(cudaMemcpy(raw.data(), pl.first, pl.second, cudaMemcpyDeviceToHost), "pool D2H");
        if (!fwrite_all(f, raw.data(), pl.second)) return fail(JP_ERR_INVALID, "write failed");
    }
    return JP_OK;
}

jp_status amr_load_state(jp_solver* s, std::FILE* f) {
    AmrState* a = s->amr;
    int64_t h[16];
    if (!fread_all(f, h, sizeof h)) return fail(JP_ERR_INVALID, "state file truncated");
    if (h[0] < 8 || h[1] < 8 || h[5] < 0 || h[5] > h[0] || h[7] < 0 || h[7] > h[1] || h[8] > a->cnb0 || h[9] > h[0])
        return fail(JP_ERR_INVALID, "state file: inconsistent block counts");
    ACK(wait_stream(s), "load");
    if (h[0] != a->cap1) TRY(set_cap1(s, (int)h[0], false));
    if (h[1] != a->cap2) TRY(set_cap2(s, (int)h[1], false));
    a->cap_nref0 = (int)h[2];
    a->cap_nref1 = (int)h[3];
    a->nref0 = (int)h[4];
    a->nf1 = (int)h[5];
    a->nref1 = (int)h[6];
    a->nf2 = (int)h[7];
    a->n_skin0 = (int)h[8];
    a->n_skin1 = (int)h[9];
    a->ndeep = (int)h[10];
    a->hw_nf1 = h[11];
    a->hw_nf2 = h[12];
    std::vector<int> buf;
    for (const TableRef& t : state_tables(a)) {
        buf.resize(t.n);
        if (!fread_all(f, buf.data(), sizeof(int) * t.n)) return fail(JP_ERR_INVALID, "state file truncated");
        ACK(cudaMemcpy(t.p, buf.data(), sizeof(int) * t.n, cudaMemcpyHostToDevice), "table H2D");
    }
    const size_t blk = (size_t)Q * a->MB3 * a->elem;
    const std::pair<void*, size_t> pools[3] = {{a->c0a, (size_t)a->cnb0 * blk}, {a->f1a, (size_t)a->nf1 * blk},
                                               {a->f2a, (size_t)a->nf2 * blk}};
    std::vector<unsigned char> raw;
    for (const auto& pl : pools) {
        raw.resize(pl.second);
        if (!fread_all(f, raw.data(), pl.second)) return fail(JP_ERR_INVALID, "state file truncated");
        if (pl.second) ACK(cudaMemcpy(pl.first, raw.data(), pl.second, cudaMemcpyHostToDevice), "pool H2D");
    }
    TRY(fill_lists(s));
    TRY(skins(s));  // the skin lists again (the same as stored) with the level-1 rest list, counts, prep lists
    ACK(wait_stream(s), "load");
    skins_landed(a);
    reset_graphs(a);
    update_bytes(s);
    return JP_OK;
}

jp_status amr_get_counts(jp_solver* s, jp_amr_counts* o) {
    AmrState* a = s->amr;
    std::memset(o, 0, sizeof *o);
    o->nref0 = a->nref0;
    o->nf1 = a->nf1;
    o->nref1 = a->nref1;
    o->nf2 = a->nf2;
    o->n_skin0 = a->n_skin0;
    o->n_skin1 = a->n_skin1;
    o->ndeep = a->ndeep;
    o->cnb0 = a->cnb0;
    o->ng1 = a->NG1;
    o->cap_nref0 = a->cap_nref0;
    o->cap1 = a->cap1;
    o->cap_nref1 = a->cap_nref1;
    o->cap2 = a->cap2;
    o->hw_nf1 = a->hw_nf1;
    o->hw_nf2 = a->hw_nf2;
    return JP_OK;
}

jp_status amr_get_table(jp_solver* s, int table, int32_t* host, int64_t capacity, int64_t* count) {
    AmrState* a = s->amr;
    const int* p = nullptr;
    long long n = 0;
    switch (table) {
        case JP_TABLE_REF0: p = a->ref0; n = a->cnb0; break;
        case JP_TABLE_FOF0: p = a->fof0; n = a->cnb0; break;
        case JP_TABLE_RL0: p = a->rl0; n = a->nref0; break;
        case JP_TABLE_L1PCB: p = a->pcb; n = a->nf1; break;
        case JP_TABLE_L1OCT: p = a->oct; n = a->nf1; break;
        case JP_TABLE_F1POS: p = a->f1pos; n = a->nf1; break;
        case JP_TABLE_L1GRID: p = a->l1grid; n = a->NG1; break;
        case JP_TABLE_REF1: p = a->ref1; n = a->nf1; break;
        case JP_TABLE_FOF1: p = a->fof1; n = a->nf1; break;
        case JP_TABLE_RL1: p = a->rl1; n = a->nref1; break;
        case JP_TABLE_L2PL1: p = a->l2pl1; n = a->nf2; break;
        case JP_TABLE_L2OCT: p = a->l2oct; n = a->nf2; break;
        case JP_TABLE_SKIN0: p = a->skin0; n = a->n_skin0; break;
        case JP_TABLE_SKIN1: p = a->skin1; n = a->n_skin1; break;
        case JP_TABLE_DEEP: p = a->deep; n = a->nf1; break;
        default: return fail(JP_ERR_INVALID, "unknown table %d", table);
    }
    if (count) *count = n;
    if (n > capacity) return fail(JP_ERR_CAPACITY, "table %d has %lld entries, buffer holds %lld", table, n, (long long)capacity);
    if (n == 0) return JP_OK;
    ACK(cudaMemcpyAsync(host, p, sizeof(int) * n, cudaMemcpyDeviceToHost, s->stream), "table D2H");
    ACK(cudaStreamSynchronize(s->stream), "table D2H");
    return JP_OK;
}

jp_status amr_get_sensor(jp_solver* s, int level, float* host, int64_t capacity, int64_t* count) {
    AmrState* a = s->amr;
    if (level != 0 && level != 1) return fail(JP_ERR_INVALID, "sensor level must be 0 or 1");
    const long long n = level == 0 ? a->cnb0 : a->nf1;
    if (count) *count = n;
    if (n > capacity) return fail(JP_ERR_CAPACITY, "sensor has %lld entries", n);
    if (n == 0) return JP_OK;
    ACK(cudaMemcpyAsync(host, level == 0 ? a->sen0 : a->sen1, sizeof(float) * n, cudaMemcpyDeviceToHost, s->stream), "D2H");
    ACK(cudaStreamSynchronize(s->stream), "D2H");
    return JP_OK;
}

jp_status amr_set_sensor_override(jp_solver* s, const float* sen0, const float* sen1_by_pos) {
    AmrState* a = s->amr;
    if (!sen0 || !sen1_by_pos) {
        dfree(a, a->ov_sen0);
        dfree(a, a->ov_sen1pos);
        return JP_OK;
    }
    if (!a->ov_sen0) TRY(dalloc(a, &a->ov_sen0, (size_t)a->cnb0, "cudaMalloc override"));
    if (!a->ov_sen1pos) TRY(dalloc(a, &a->ov_sen1pos, (size_t)a->NG1, "cudaMalloc override"));
    ACK(cudaMemcpyAsync(a->ov_sen0, sen0, sizeof(float) * a->cnb0, cudaMemcpyHostToDevice, s->stream), "H2D");
    ACK(cudaMemcpyAsync(a->ov_sen1pos, sen1_by_pos, sizeof(float) * a->NG1, cudaMemcpyHostToDevice, s->stream), "H2D");
    ACK(cudaStreamSynchronize(s->stream), "H2D");
    return JP_OK;
}

}  // namespace jp
