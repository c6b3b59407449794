// harness.cpp - C entry points around the reference's own functors
// (CSSL-UWM/tau_leaping), compiled from the reference's sources where they
// lie (tau_leaping/CSRMatrixPacked.cu is included, not copied).  Test
// infrastructure only: the tests use it to pin the FP64 oracle.
#include "tau_leaping/CSRMatrixPacked.cu"

extern "C" {

// IsCriticalAndPropensity (functions.h:100-123).
int ref_propensity(int type, int x0, int x1, int nc, float k, float* prop) {
    bool crit = false;
    IsCriticalAndPropensity((char)type, x0, x1, nc, k, prop, &crit);
    return crit ? 1 : 0;
}

// pack / split (functions.h:126-146).
int ref_pack(int v, int idx) { return pack((char)v, idx); }
void ref_split(int vci, int* v, int* idx) {
    char c;
    split(vci, c, *idx);
    *v = c;
}

// CSRMatrixPacked::CompTau (CSRMatrixPacked.cu:423-462) on a matrix built by
// the reference's own packing constructor (CSRMatrixPacked.cu:22-31).
float ref_comp_tau(int rows, int cols, int nnz, const float* values, const int* row_ptr, const int* col_ind,
                   const unsigned char* crit, const int* x, const signed char* type, const float* a, float eps) {
    vec_float_t v(values, values + nnz);
    vec_int_t rp(row_ptr, row_ptr + rows + 1), ci(col_ind, col_ind + nnz);
    CSRMatrixPacked m(rows, cols, v, rp, ci);
    std::vector<char> cr(crit, crit + cols);
    static_assert(sizeof(bool) == 1, "bool layout");
    return m.CompTau(reinterpret_cast<const bool*>(cr.data()), x, reinterpret_cast<const char*>(type), a, eps,
                     0.f);
}

// TauFn for one species row (CSRMatrixPacked.cu:311-358).
float ref_tau_row(const int* valcol, const int* row_ptr, const unsigned char* crit, const int* x,
                  const signed char* type, const float* a, float eps, int i) {
    TauFn fn(valcol, row_ptr, reinterpret_cast<const bool*>(crit), x, reinterpret_cast<const char*>(type), a, eps,
             0.f);
    return fn(i);
}

// FireReactionsFn (CSRMatrixPacked.cu:464-492) applied to every species row.
void ref_fire_rows(int rows, int nnz, const int* valcol, const int* row_ptr, int cols, const int* k, int* x) {
    vec_int_t vc(valcol, valcol + nnz), rp(row_ptr, row_ptr + rows + 1), kk(k, k + cols), rc(x, x + rows);
    FireReactionsFn fn(vc, rp, kk, rc);
    for (int i = 0; i < rows; ++i) fn(i);
    std::copy(rc.begin(), rc.end(), x);
}

// CSRMatrixPacked::FireReactions as shipped (loop bound = channel count,
// CSRMatrixPacked.cu:502); only defined behaviour when cols == rows.
void ref_fire_as_shipped(int rows, int cols, int nnz, const float* values, const int* row_ptr, const int* col_ind,
                         const int* k, int* x) {
    vec_float_t v(values, values + nnz);
    vec_int_t rp(row_ptr, row_ptr + rows + 1), ci(col_ind, col_ind + nnz);
    CSRMatrixPacked m(rows, cols, v, rp, ci);
    vec_int_t kk(k, k + cols), rc(x, x + rows);
    m.FireReactions(kk, rc);
    std::copy(rc.begin(), rc.end(), x);
}

}  // extern "C"
