// shim_full.h - additions to shim.h for compiling the reference's whole host
// path (Model, ModelConst/State, CSR/CSC classes, StochKit reader,
// statistics) with g++ on Thrust's CPP backend.  Project-written.
#pragma once
#include "shim.h"

#include <fstream>
#include <memory>
#include <thrust/tuple.h>
#include <cusparse.h>

// model.cu:172-178 adds two (float, float) tuples with a global operator+,
// which argument-dependent lookup no longer reaches from inside
// thrust::plus; declare the same sum in the tuple's own namespace.
_LIBCUDACXX_BEGIN_NAMESPACE_STD
inline tuple<float, float> operator+(tuple<float, float> const& a, tuple<float, float> const& b) {
    return tuple<float, float>(get<0>(a) + get<0>(b), get<1>(a) + get<1>(b));
}
_LIBCUDACXX_END_NAMESPACE_STD

// CUSPARSE 4 entry points the reference calls; removed from current
// cuSPARSE.  Defined host-side in stubs.cpp (a transpose; an unused SpMV).
cusparseStatus_t cusparseScsr2csc(cusparseHandle_t, int m, int n, const float* csrVal, const int* csrRowPtr,
                                  const int* csrColInd, float* cscVal, int* cscRowInd, int* cscColPtr,
                                  int copyValues, cusparseIndexBase_t base);
cusparseStatus_t cusparseScsrmv(cusparseHandle_t, cusparseOperation_t, int, int, float, cusparseMatDescr_t,
                                const float*, const int*, const int*, const float*, float, float*);

// functions.cpp:102 compares a stream with NULL (valid before C++11).
inline bool operator!=(const std::ifstream& f, long) { return f.is_open(); }

// CSCMatrix.cu:42-51 (unused SpMV) calls atomicAdd inside a functor.
template <class T>
inline T atomicAdd(T* a, T v) {
    const T o = *a;
    *a += v;
    return o;
}
