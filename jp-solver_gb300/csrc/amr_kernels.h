// Launch interface of the AMR kernels (amr_kernels.cu) and the adaptation pipeline (adapt.cu).
#pragma once
#include <cuda_runtime.h>

namespace jp {
namespace amr {

enum AmrOp {
    OP_INIT = 0,       // out = TGV state of the coarse grid
    OP_STEP_L0,        // in -> out, dense periodic coarse step
    OP_PREP,           // out = prolongation source of in at the cells a fill can read: list = interface
                       // cells (b * MB^3 + cell, adapt_prep_cells), nlim = their count, nblocks = the
                       // list's capacity; scale = nqs; t0 = device count of the next level's fill list
                       // (skipped when 0) or null
    OP_FILL_L1,        // in = prep0, out = gh1; t0 pcb, t1 oct, list = fill list (ghost cells b * SH + t),
                       // nlim = its length, nblocks = its capacity
    OP_FILL_L2,        // in = prep1, out = gh2; t0 l2pl1, t1 l2oct, t2 f1pos, t3 l1grid; list, nlim, nblocks as
                       // OP_FILL_L1
    OP_STEP_L1,        // in -> out, aux = gh1, nbt = level-1 table; t0 pcb, t1 oct; out2 = c0 restricts (scale nqi);
                       // list (rows mapping, no out2): only the blocks list[0 .. *nlim), nblocks = its capacity
    OP_STEP_L2,        // in -> out, aux = gh2, nbt = level-2 table; t0 l2pl1, t1 l2oct; out2 = f1 restricts
    OP_RESTRICT,       // out = coarse, in = fine; list = refined coarse blocks, t0 = fof; scale = nqi
    OP_SEED_L1,        // in = old f1 (migrate) , out = new f1, aux = c0; t0 pcb, t1 oct, t2 old ref0|null, t3 old fof0
    OP_SEED_L2,        // in = old f2, out = new f2, aux = f1; t0 l2pl1, t1 l2oct, t2 f1pos, t3 old l1grid|null,
                       // t4 old ref1, t5 old fof1, t6 l1grid
    OP_SENSOR,         // in = level, out = sensor; aux = override values|null, t0 = override position map|null
    OP_COMPOSITE,      // in = c0, aux = f1, aux2 = f2, out = field; t0 ref1, t1 fof1, t2 l1grid
    OP_NBTAB_L1,       // iout = level-1 neighbour table (nblocks = nf1); t0 pcb, t1 oct, t2 ref0, t3 fof0
    OP_NBTAB_L2,       // iout = level-2 neighbour table (nblocks = nf2); t0 l2pl1, t1 l2oct, t2 f1pos,
                       // t3 l1grid, t4 ref1, t5 fof1
    OP_WARM            // no launch: find the resident grid of the row steps (before any graph capture)
};

// Population arrays (pools, prolongation sources, ghost shells) are in the solver's storage format
// (FP32, or shifted FP16/BF16); sensor values and the composite field are float.
struct AmrLaunch {
    cudaStream_t st = nullptr;
    int nblocks = 0;
    const void* in = nullptr;
    void* out = nullptr;
    void* out2 = nullptr;    // fused restriction target of the last fine substep (nullptr: none)
    const void* aux = nullptr;
    const void* aux2 = nullptr;
    const int* list = nullptr;
    const int *t0 = nullptr, *t1 = nullptr, *t2 = nullptr, *t3 = nullptr, *t4 = nullptr, *t5 = nullptr, *t6 = nullptr;
    const int* nbt = nullptr;  // same-level neighbour table of the fine level (27 per block)
    int* iout = nullptr;
    int tpb = 0;               // threads per CTA of the per-cell fine steps (0: default_step_tpb)
    int vec = 0;               // fine steps: 4 = rows of four cells per thread, 1 = a cell per thread
                               // (0: default_step_vec)
    // device count of the blocks to process (prep, fill, fine step, restrict): the grid is sized
    // for the capacity and CTAs past *nlim return, so a captured step stays valid after a regrid
    const int* nlim = nullptr;
    int cgx = 0, n = 0, l1gx = 0, n1 = 0, n2 = 0;
    float omega = 0.f, scale = 0.f;
    double u0 = 0.0, kf = 0.0;
};

// One member of a batched launch: the fields of AmrLaunch a per-block stage reads, and the first
// CTA of the member in the batched grid (members follow each other; a member gets as many CTAs as
// its single launch would).
struct AmrItem {
    const void* in;
    void* out;
    const void* aux;
    void* out2;
    const int *t0, *t1, *t2, *t3, *nbt, *list, *nlim;
    int cgx, n, l1gx, n1;
    float omega, scale;
    int begin;
    int nct;  // CTAs of the member (a stage walking a cell list strides with them)
};
constexpr int kAmrBatchMax = 48;
// Many solves in one launch per stage: OP_STEP_L0/L1/L2, OP_PREP, OP_FILL_L1/L2, OP_RESTRICT over up
// to kAmrBatchMax solves of the same block edge, storage and step threads.  Passed by value in kernel
// parameter space.
struct AmrBatch {
    int count = 0, total = 0;  // members, CTAs
    int vec = 0, pad = 0;      // fine-step mapping as AmrLaunch::vec
    AmrItem it[kAmrBatchMax];
};

// ---- persistent coarse steps: many solves, several coarse steps, one launch ---------------------
// One member of a persistent launch: the arrays and device counts of one solve's coarse step
// (base_step's sequence).  c0[0] holds the coarse state when the launch starts; after `steps`
// coarse steps it is in c0[steps & 1].  The fine levels end in f1a / f2a as they started.
struct PersistMember {
    void* c0[2];
    void *prep0, *gh1, *f1a, *f1b, *prep1, *gh2, *f2a, *f2b;
    const int *pc0, *pc1, *fl1, *fl2;                  // interface-cell and fill lists
    const int *pcb, *oct, *l2pl1, *l2oct, *f1pos, *l1grid, *nb1, *nb2;
    const int *n_prep0, *n_fill1, *n_prep1, *n_fill2;  // list lengths on the device
    const int *n_f1, *n_f2;                            // fine block counts on the device
    int cgx, n, l1gx, n1, cnb0, steps;
    float om0, om1, om2, nqs01, nqs12, nqi21, nqi10;
};
// Grid barrier state of a persistent launch: arrivals (zeroed before each launch), and the first
// error (a barrier wait that ran past the limit: 1), the phase and the coarse step where it happened
// (kept until the owner reads and clears them).
struct PersistSync {
    unsigned int arrived;
    int err, phase, step;
};
constexpr size_t kPersistResetBytes = sizeof(unsigned int);  // arrived
constexpr int kPersistPhases = 10;  // grid-wide phases of one coarse step
// Up to kAmrBatchMax members sorted by `steps`, descending (members with fewer coarse steps drop
// out of the later ones: ragged step counts); passed by value in kernel parameter space.
struct AmrPersist {
    int count = 0, maxsteps = 0;
    long long limit_ns = 0;    // longest wait at one grid barrier before the launch gives up
    PersistSync* sync = nullptr;
    PersistMember m[kAmrBatchMax];
};
// the block edge, fine-step mapping and flags the persistent coarse step implements (MB = 8, rows
// of four cells, restrictions fused into the last substeps, preparations and restrictions on)
bool amr_persist_supported(int mb, int vec, bool fuse, bool skip_prep);
// Cooperative launch of the persistent coarse steps on `st` with `grid` CTAs (0: every CTA that can
// be resident; capped there).  *grid_used (optional) returns the grid.
cudaError_t amr_persist_launch(int storage, int mb, const AmrPersist& P, int grid, cudaStream_t st, int* grid_used);
template <class ST> cudaError_t amr_persist_launch_st(int mb, const AmrPersist& P, int grid, cudaStream_t st,
                                                      int* grid_used);

// storage: 0 FP32, 1 shifted FP16, 2 shifted BF16 (jp_storage)
cudaError_t amr_launch(int storage, int mb, int op, const AmrLaunch& L);
// op as in AmrLaunch; tpb: threads per CTA of the steps (0: default); fuse: the fine steps restrict
// into out2 (every member the same)
cudaError_t amr_batch_launch(int storage, int mb, int op, int tpb, bool fuse, const AmrBatch& B, cudaStream_t st);
template <class ST> cudaError_t amr_batch_launch_st(int mb, int op, int tpb, bool fuse, const AmrBatch& B, cudaStream_t st);
template <class ST> cudaError_t amr_launch_st(int mb, int op, const AmrLaunch& L);
size_t storage_elem(int storage);  // bytes per stored population
int shell_cells(int mb);
// the fused restriction stages a block in shared memory: MB <= 8 (38 KiB at MB = 8)
bool can_fuse_restrict(int mb);
// threads per CTA a step of block edge mb can run with, and the default
bool step_tpb_supported(int mb, int tpb);
int default_step_tpb(int mb);
// cells per thread of the fine steps: 4 (rows, MB = 8 and 16) or 1
bool step_vec_supported(int mb, int vec);
int default_step_vec(int mb);

// ---- adaptation pipeline (adapt.cu) ------------------------------------------------------------
// Device counters shared by the pipeline; the host reads them once per stage.
struct AdaptCounts {
    int nref0, nf1, nref1, nf2, n_skin0, n_skin1, ndeep, err;
    float thr0, thr1;
    int n_rest1;  // level-1 blocks outside the skin (adapt_skins' rest1 list)
    int pad[5];
};
enum { ADAPT_ERR_CAP1 = 1, ADAPT_ERR_CAP2 = 2 };

// ref[i] = 1 for all (mode 0) or the lower half in z (mode 1, k_mark_slab)
cudaError_t adapt_mark_mode(int mode, int* ref, int cnb0, int cgx, cudaStream_t st);
// Exact threshold: thr = the (n - tgt)-th smallest of the sensors (ascending, 0-based) where
// tgt = min(cap, max(1, int(frac * n))), n = count of entries with mask != 0 (all if mask is null);
// then ref[i] = (mask[i] && sen[i] >= thr).  Writes n to counts->ndeep when mask is given and the
// threshold to counts->thr0/thr1.  If n == 0 ref is zeroed.
cudaError_t adapt_threshold_mark(const float* sen, const int* mask, int n, double frac, int cap, int* ref,
                                 AdaptCounts* counts, int which, cudaStream_t st);
// deep[b] = all six face neighbours of block b's level-1 grid position are present
cudaError_t adapt_deepmask(const int* f1pos, const int* l1grid, int l1gx, int nf1, int* deep, cudaStream_t st);
// exclusive scan of ref0 -> level-1 tables (k_scatter_L1, l1grid reset first); nref0/nf1 into counts.
// If nf1 > cap1 the error bit is set and no table is written.
cudaError_t adapt_build_l1(const int* ref0, int cnb0, int cgx, int l1gx, int cap1, int* rank, int* fof0, int* rl0,
                           int* pcb, int* oct, int* l1grid, int* f1pos, AdaptCounts* counts, cudaStream_t st);
// exclusive scan of ref1 into rank (counts only): nref1/nf2 into counts
cudaError_t adapt_scan_l2(const int* ref1, int nf1, int* rank, AdaptCounts* counts, cudaStream_t st);
// k_scatter_L2 from the ranks of adapt_scan_l2; error and no scatter if nf2 > cap2
cudaError_t adapt_scatter_l2(const int* ref1, const int* rank, int nf1, int cap2, int* fof1, int* rl1, int* l2pl1,
                             int* l2oct, AdaptCounts* counts, cudaStream_t st);
// skin lists: blocks that are refined or have a refined 26-neighbour, ascending (k_dilate + copy_if);
// rest1 (optional): the other level-1 blocks, ascending, their count in counts->n_rest1
cudaError_t adapt_skins(const int* ref0, int cnb0, int cgx, const int* ref1, const int* f1pos, const int* l1grid,
                        int nf1, int l1gx, int* flags, int* skin0, int* skin1, AdaptCounts* counts, cudaStream_t st,
                        int* rest1 = nullptr);
// set n ints to v
cudaError_t adapt_fill(int* p, int v, long long n, cudaStream_t st);
// fill list of a fine level: the ghost-shell cells (faces, edges) of the nf blocks whose slot of the
// neighbour table nb (27 per block) is on another level (-1), as b * SH + shell cell (SH = shell
// cells of edge mb; at most SH per block); *count is set.  The list's order is not fixed: each
// cell is filled independently.
cudaError_t adapt_fill_list(const int* nb, int nf, int mb, int* list, int* count, cudaStream_t st);
// prep list of a level: the skin blocks whose 27 neighbour blocks (periodic) mix refined and
// unrefined, as pairs {block, mask of the refined neighbours (bit = slot)}; level 0: pos null and
// gx = cgx; level 1: pos = f1pos, grid = l1grid, gx = l1gx (absent blocks unrefined).  The skin
// count is read on the device (*nskin_dev, at most cap: the grid), so no read-back precedes the
// list.  *count is set.
cudaError_t adapt_prep_list(const int* skin, const int* nskin_dev, int cap, const int* ref, const int* pos,
                            const int* grid, int gx, int* list, int* count, cudaStream_t st);
// interface cells of the (at most max_entries, *pcount) blocks of a prep list: the cells whose 3x3x3
// neighbourhood reaches refined and unrefined blocks, as b * mb^3 + cell (at most
// mb^3 - (mb-2)^3 per block); *ncells is set.  The order is not fixed.
cudaError_t adapt_prep_cells(const int* plist, const int* pcount, int max_entries, int mb, int* cells, int* ncells,
                             cudaStream_t st);
// interface cells a block can hold (its cells within one of a face)
inline int interface_cells(int mb) { return mb * mb * mb - (mb - 2) * (mb - 2) * (mb - 2); }
// dilate refinement marks by `layers` block layers (tmp: n ints of scratch); level 1 with the
// position map pos, the grid map and the deep mask (marks only on deep blocks)
cudaError_t adapt_dilate_marks(int* ref, int* tmp, int n, int gx, const int* pos, const int* grid, const int* deep,
                               int layers, cudaStream_t st);

}  // namespace amr
}  // namespace jp
