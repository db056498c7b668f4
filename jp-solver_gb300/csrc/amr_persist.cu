// Persistent coarse steps with FP32 storage, and the entry point for every storage format.  The
// kernel is in amr_persist.cuh.
#include "amr_persist.cuh"

namespace jp {
namespace amr {

template cudaError_t amr_persist_launch_st<StF32>(int mb, const AmrPersist& P, int grid, cudaStream_t st,
                                                  int* grid_used);
extern template cudaError_t amr_persist_launch_st<StF16>(int mb, const AmrPersist& P, int grid, cudaStream_t st,
                                                         int* grid_used);
extern template cudaError_t amr_persist_launch_st<StBF16>(int mb, const AmrPersist& P, int grid, cudaStream_t st,
                                                          int* grid_used);

bool amr_persist_supported(int mb, int vec, bool fuse, bool skip_prep) {
    return mb == 8 && (vec == 0 || vec == 4) && fuse && !skip_prep;
}

cudaError_t amr_persist_launch(int storage, int mb, const AmrPersist& P, int grid, cudaStream_t st, int* grid_used) {
    switch (storage) {
        case 0: return amr_persist_launch_st<StF32>(mb, P, grid, st, grid_used);
        case 1: return amr_persist_launch_st<StF16>(mb, P, grid, st, grid_used);
        case 2: return amr_persist_launch_st<StBF16>(mb, P, grid, st, grid_used);
    }
    return cudaErrorInvalidValue;
}

}  // namespace amr
}  // namespace jp
