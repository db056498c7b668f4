// AMR kernels with shifted BF16 storage (f - w_q in bfloat16).
#include "amr_kernels.cuh"

namespace jp {
namespace amr {

template cudaError_t amr_launch_st<StBF16>(int mb, int op, const AmrLaunch& L);
template cudaError_t amr_batch_launch_st<StBF16>(int mb, int op, int tpb, bool fuse, const AmrBatch& B,
                                                 cudaStream_t st);

}  // namespace amr
}  // namespace jp
