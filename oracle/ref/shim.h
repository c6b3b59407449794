// shim.h - force-included when the reference's CUDA sources are compiled
// host-only with g++ (Thrust's CPP backend).  Project-written; it only
// supplies what a 2012 CUDA/Thrust code base expects from its toolchain and
// that a current C++17 host compiler lacks.  No reference code is copied.
#pragma once
#include <algorithm>
#include <cmath>
#include <iostream>
#include <limits>
#include <unistd.h>

#include <cuda_runtime.h>
#include <vector_types.h>

#include <thrust/device_vector.h>
#include <thrust/functional.h>
#include <thrust/host_vector.h>
#include <thrust/sequence.h>
#include <thrust/transform.h>
#include <thrust/transform_reduce.h>

// thrust::unary_function was removed from CCCL 3.
namespace thrust {
template <class A, class R>
struct unary_function {
    typedef A argument_type;
    typedef R result_type;
};
}  // namespace thrust

using std::max;
using std::min;

// Launch-geometry built-ins referenced by an unused __global__ function body.
static dim3 gridDim, blockDim;
static uint3 blockIdx, threadIdx;
