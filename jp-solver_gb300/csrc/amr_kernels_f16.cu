// AMR kernels with shifted FP16 storage (f - w_q in IEEE half).
#include "amr_kernels.cuh"

namespace jp {
namespace amr {

template cudaError_t amr_launch_st<StF16>(int mb, int op, const AmrLaunch& L);

}  // namespace amr
}  // namespace jp
