/* Include shim for compiling the reference's src/coupling.cu with CCCL 3,
 * which removed thrust::identity (used as the stencil predicate of
 * thrust::copy_if at src/coupling.cu:125,160). */
#pragma once
#include <thrust/functional.h>
namespace thrust {
template <class T>
struct identity {
    __host__ __device__ const T& operator()(const T& x) const { return x; }
};
}  // namespace thrust
