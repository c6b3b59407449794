// stubs.cpp - host definitions of the CUDA runtime / cuSPARSE calls the
// reference's host path makes, so it runs without a GPU or the libraries.
// Project-written.
#include <cstring>
#include <vector>

#include <cuda_runtime.h>
#include <cusparse.h>

extern "C++" {
cusparseStatus_t cusparseScsr2csc(cusparseHandle_t, int m, int n, const float* val, const int* rp, const int* ci,
                                  float* cval, int* cri, int* ccp, int copy, cusparseIndexBase_t) {
    // stable counting-sort transpose of an m x n CSR matrix
    const int nnz = rp[m];
    std::vector<int> cnt(n + 1, 0);
    for (int q = 0; q < nnz; ++q) cnt[ci[q] + 1]++;
    for (int j = 0; j < n; ++j) cnt[j + 1] += cnt[j];
    for (int j = 0; j <= n; ++j) ccp[j] = cnt[j];
    for (int i = 0; i < m; ++i)
        for (int q = rp[i]; q < rp[i + 1]; ++q) {
            const int d = cnt[ci[q]]++;
            cri[d] = i;
            if (copy) cval[d] = val[q];
        }
    return CUSPARSE_STATUS_SUCCESS;
}
cusparseStatus_t cusparseScsrmv(cusparseHandle_t, cusparseOperation_t, int, int, float, cusparseMatDescr_t,
                                const float*, const int*, const int*, const float*, float, float*) {
    return CUSPARSE_STATUS_NOT_SUPPORTED;
}
}

extern "C" {
cusparseStatus_t cusparseCreate(cusparseHandle_t* h) {
    *h = reinterpret_cast<cusparseHandle_t>(1);
    return CUSPARSE_STATUS_SUCCESS;
}
cusparseStatus_t cusparseCreateMatDescr(cusparseMatDescr_t* d) {
    *d = reinterpret_cast<cusparseMatDescr_t>(1);
    return CUSPARSE_STATUS_SUCCESS;
}
cusparseStatus_t cusparseSetMatType(cusparseMatDescr_t, cusparseMatrixType_t) { return CUSPARSE_STATUS_SUCCESS; }
cusparseStatus_t cusparseSetMatIndexBase(cusparseMatDescr_t, cusparseIndexBase_t) { return CUSPARSE_STATUS_SUCCESS; }
cusparseStatus_t cusparseSetMatDiagType(cusparseMatDescr_t, cusparseDiagType_t) { return CUSPARSE_STATUS_SUCCESS; }
cudaError_t cudaGetLastError(void) { return cudaSuccess; }
const char* cudaGetErrorString(cudaError_t) { return "no error"; }
cudaError_t cudaSetDevice(int) { return cudaSuccess; }
}
