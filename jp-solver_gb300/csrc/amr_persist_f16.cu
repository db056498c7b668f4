// Persistent coarse steps with shifted FP16 storage.
#include "amr_persist.cuh"

namespace jp {
namespace amr {

template cudaError_t amr_persist_launch_st<StF16>(int mb, const AmrPersist& P, int grid, cudaStream_t st,
                                                  int* grid_used);

}  // namespace amr
}  // namespace jp
