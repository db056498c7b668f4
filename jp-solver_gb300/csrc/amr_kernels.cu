// AMR kernels with FP32 storage, the launch entry point for every storage format, and the launch
// shape rules of the AMR kernels.  The kernels themselves are in amr_kernels.cuh.
#include "amr_kernels.cuh"

namespace jp {
namespace amr {

template cudaError_t amr_launch_st<StF32>(int mb, int op, const AmrLaunch& L);
template cudaError_t amr_batch_launch_st<StF32>(int mb, int op, int tpb, bool fuse, const AmrBatch& B, cudaStream_t st);
extern template cudaError_t amr_launch_st<StF16>(int mb, int op, const AmrLaunch& L);
extern template cudaError_t amr_launch_st<StBF16>(int mb, int op, const AmrLaunch& L);
extern template cudaError_t amr_batch_launch_st<StF16>(int mb, int op, int tpb, bool fuse, const AmrBatch& B,
                                                       cudaStream_t st);
extern template cudaError_t amr_batch_launch_st<StBF16>(int mb, int op, int tpb, bool fuse, const AmrBatch& B,
                                                        cudaStream_t st);

cudaError_t amr_launch(int storage, int mb, int op, const AmrLaunch& L) {
    if (L.nblocks <= 0 && op != OP_COMPOSITE) return cudaSuccess;
    switch (storage) {
        case 0: return amr_launch_st<StF32>(mb, op, L);
        case 1: return amr_launch_st<StF16>(mb, op, L);
        case 2: return amr_launch_st<StBF16>(mb, op, L);
    }
    return cudaErrorInvalidValue;
}

cudaError_t amr_batch_launch(int storage, int mb, int op, int tpb, bool fuse, const AmrBatch& B, cudaStream_t st) {
    switch (storage) {
        case 0: return amr_batch_launch_st<StF32>(mb, op, tpb, fuse, B, st);
        case 1: return amr_batch_launch_st<StF16>(mb, op, tpb, fuse, B, st);
        case 2: return amr_batch_launch_st<StBF16>(mb, op, tpb, fuse, B, st);
    }
    return cudaErrorInvalidValue;
}

int shell_cells(int mb) { return 6 * mb * mb + 12 * mb; }
bool can_fuse_restrict(int mb) { return mb <= 8; }
// measured on the GB300 (static gold N0=64, all levels refined): 256 threads (two cells each) are
// the fastest split at MB = 8, 512 at MB = 16
int default_step_tpb(int mb) { return mb == 4 ? 64 : (mb == 8 ? 256 : 512); }
// rows of four cells per thread where the block has them (MB >= 8)
int default_step_vec(int mb) { return mb >= 8 ? 4 : 1; }
bool step_vec_supported(int mb, int vec) { return vec == 1 || (vec == 4 && mb >= 8); }
bool step_tpb_supported(int mb, int tpb) {
    if (mb == 4) return tpb == 64;
    return (mb == 8 || mb == 16) && (tpb == 128 || tpb == 256 || tpb == 512);
}
size_t storage_elem(int storage) { return storage == 0 ? 4 : 2; }

}  // namespace amr
}  // namespace jp
