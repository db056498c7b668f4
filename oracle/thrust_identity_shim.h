// ORACLE build shim: CCCL 3 (CUDA 13) removed thrust::identity, which the reference's host code
// uses as a copy_if predicate.  Force-included when compiling the reference's AMR file.
#pragma once
#include <thrust/functional.h>
namespace thrust {
template <class T>
struct identity {
    __host__ __device__ const T& operator()(const T& x) const { return x; }
};
}  // namespace thrust
