// model.cpp - load-time model tables (host C++).
//
// Replaces the reference's device-side load toolchain
// (tau_leaping/CSCMatrix.cu:147-251, CSRMatrix.cu:415-418,
// CSRMatrixPacked.cu:22-31) with plain host code: the species-row CSR is a
// stable counting-sort transpose of the channel-major entries instead of
// cusparseScsr2csc, and orders / reactant indices are detected on the host.
#include <algorithm>
#include <cmath>
#include <map>
#include <string>

#include "../csrc/tl_internal.h"

namespace tl {

namespace {

bool packable(int v) { return v >= -2 && v <= 5; }
int32_t pack(int idx, int v) { return (int32_t)(((uint32_t)idx << 3) | (uint32_t)((v + 2) & 7)); }

// Stable transpose of channel-major packed-free entries into species rows.
void to_rows(int N, int M, const std::vector<int32_t>& cp, const std::vector<int32_t>& rows,
             const std::vector<int>& vals, std::vector<int32_t>& rp, std::vector<int32_t>& vc) {
    rp.assign((size_t)N + 1, 0);
    for (size_t q = 0; q < rows.size(); ++q) rp[(size_t)rows[q] + 1]++;
    for (int i = 0; i < N; ++i) rp[(size_t)i + 1] += rp[(size_t)i];
    vc.assign(rows.size(), 0);
    std::vector<int32_t> fill(rp.begin(), rp.end() - 1);
    for (int j = 0; j < M; ++j)
        for (int q = cp[(size_t)j]; q < cp[(size_t)j + 1]; ++q) vc[(size_t)fill[(size_t)rows[(size_t)q]]++] = pack(j, vals[(size_t)q]);
}

}  // namespace

void channels_to_raw(const std::vector<Channel>& ch, HostModel& h) {
    // ReadXMLToMatrixStruct (CSCHostMatrixData.cpp:40-106): rows of a column
    // sorted ascending; a species listed as reactant and product appears
    // twice, first with the negative (reactant) stoichiometry.
    h.M = (int)ch.size();
    h.col_ptr.assign((size_t)h.M + 1, 0);
    h.row_ind.clear();
    h.stoich.clear();
    h.rate.resize((size_t)h.M);
    for (int j = 0; j < h.M; ++j) {
        const Channel& c = ch[(size_t)j];
        h.rate[(size_t)j] = c.rate;
        std::vector<int> rind;
        for (auto& r : c.reactants) rind.push_back(r.first);
        for (auto& p : c.products) rind.push_back(p.first);
        std::sort(rind.begin(), rind.end());
        std::map<int, bool> found;
        for (int sp : rind) {
            int v = 0;
            auto rit = std::find_if(c.reactants.begin(), c.reactants.end(),
                                    [&](const std::pair<int, int>& e) { return e.first == sp; });
            if (rit == c.reactants.end() || found[sp]) {
                auto pit = std::find_if(c.products.begin(), c.products.end(),
                                        [&](const std::pair<int, int>& e) { return e.first == sp; });
                v = pit != c.products.end() ? (int8_t)pit->second : 0;
            } else {
                v = -(int)(int8_t)rit->second;
                found[sp] = true;
            }
            h.row_ind.push_back(sp);
            h.stoich.push_back((int8_t)v);
        }
        h.col_ptr[(size_t)j + 1] = (int32_t)h.row_ind.size();
    }
}

tl_status derive_tables(HostModel& h, std::string& err) {
    const int N = h.N, M = h.M;
    if (N <= 0 || M <= 0) {
        err = "model needs at least one species and one channel";
        return TL_ERR_INVALID_MODEL;
    }
    if ((int)h.x0.size() != N || (int)h.rate.size() != M || (int)h.col_ptr.size() != M + 1) {
        err = "array sizes do not match N / M";
        return TL_ERR_INVALID_MODEL;
    }
    if (N >= (1 << 28) || M >= (1 << 28)) {
        err = "N and M must stay below 2^28 (packed index field)";
        return TL_ERR_UNSUPPORTED;
    }
    if (h.col_ptr[0] != 0) {
        err = "col_ptr[0] must be 0";
        return TL_ERR_INVALID_MODEL;
    }
    for (int j = 0; j < M; ++j)
        if (h.col_ptr[(size_t)j + 1] < h.col_ptr[(size_t)j]) {
            err = "col_ptr must be non-decreasing";
            return TL_ERR_INVALID_MODEL;
        }
    const int nnz = h.col_ptr[(size_t)M];
    if ((int)h.row_ind.size() != nnz || (int)h.stoich.size() != nnz) {
        err = "row_ind / stoich length differs from col_ptr[M]";
        return TL_ERR_INVALID_MODEL;
    }
    for (int q = 0; q < nnz; ++q)
        if (h.row_ind[(size_t)q] < 0 || h.row_ind[(size_t)q] >= N) {
            err = "species index out of range in channel entries";
            return TL_ERR_INVALID_MODEL;
        }
    int64_t xmax = 0;
    for (int i = 0; i < N; ++i) {
        if (h.x0[(size_t)i] < 0) {
            err = "negative initial population";
            return TL_ERR_INVALID_MODEL;
        }
        xmax = std::max(xmax, h.x0[(size_t)i]);
    }
    for (int j = 0; j < M; ++j) {
        const double c = h.rate[(size_t)j];
        if (!std::isfinite(c) || c < 0.0) {
            err = "rate constants must be finite and >= 0";
            return TL_ERR_NUMERIC;
        }
    }
    if (h.pop_bits == 0) h.pop_bits = xmax > (int64_t)1 << 30 ? 64 : 32;
    if (h.pop_bits != 32 && h.pop_bits != 64) {
        err = "pop_bits must be 0, 32 or 64";
        return TL_ERR_INVALID_ARGUMENT;
    }
    if (h.pop_bits == 32 && xmax > 2147483647LL) {
        err = "initial population exceeds int32; use pop_bits = 64";
        return TL_ERR_OVERFLOW;
    }

    // reaction orders and reactant indices
    h.order.assign((size_t)M, 0);
    h.ref_order.assign((size_t)M, -1);
    h.s0.assign((size_t)M, 0);
    h.s1.assign((size_t)M, 0);
    h.max_order = 0;
    std::vector<std::pair<int, int>> re;  // reused: no allocation per channel
    for (int j = 0; j < M; ++j) {
        // the reference's detector (CSCMatrix.cu:204-231)
        int first = 0, second = 0;
        re.clear();
        for (int q = h.col_ptr[(size_t)j]; q < h.col_ptr[(size_t)j + 1]; ++q) {
            const int v = h.stoich[(size_t)q];
            if (v >= 0) continue;
            if (first == 0) first = v;
            else second = v;
            re.push_back({h.row_ind[(size_t)q], -v});
        }
        int ro = -1;
        if (first == -2) ro = 3;
        else if (first == -1 && second == -1) ro = 2;
        else if (first == -1) ro = 1;
        h.ref_order[(size_t)j] = (int8_t)ro;
        // mass-action order of the reactant multiset
        int ord;
        if (re.empty()) {
            ord = 0;
        } else if (re.size() == 1 && re[0].second == 1) {
            ord = 1;
            h.s0[(size_t)j] = h.s1[(size_t)j] = re[0].first;
        } else if (re.size() == 1 && re[0].second == 2) {
            ord = 3;
            h.s0[(size_t)j] = h.s1[(size_t)j] = re[0].first;
        } else if (re.size() == 2 && re[0].second == 1 && re[1].second == 1) {
            ord = 2;
            h.s0[(size_t)j] = re[0].first;
            h.s1[(size_t)j] = re[1].first;
        } else {
            err = "channel " + std::to_string(j + 1) +
                  ": only reactions of order <= 2 (S, S+S', 2S, or no reactant) are supported";
            return TL_ERR_UNSUPPORTED;
        }
        h.order[(size_t)j] = (int8_t)ord;
        h.max_order = std::max(h.max_order, ord == 3 ? 2 : ord);
    }
    // highest-order-reaction kind per species (CGP 2006, eq. 27)
    h.gkind.assign((size_t)N, 0);
    for (int j = 0; j < M; ++j) {
        const int o = h.order[(size_t)j];
        if (o == 0) continue;
        auto bump = [&](int sp, int k) { h.gkind[(size_t)sp] = (int8_t)std::max<int>(h.gkind[(size_t)sp], k); };
        if (o == 1) bump(h.s0[(size_t)j], 1);
        else if (o == 2) {
            bump(h.s0[(size_t)j], 2);
            bump(h.s1[(size_t)j], 2);
        } else bump(h.s0[(size_t)j], 3);
    }
    // raw species-row CSR (reference packing; CSRMatrixPacked.cu:22-31)
    std::vector<int> raw_v((size_t)nnz);
    for (int q = 0; q < nnz; ++q) {
        raw_v[(size_t)q] = h.stoich[(size_t)q];
        if (!packable(raw_v[(size_t)q])) {
            err = "stoichiometry outside [-2, 5] cannot be packed (functions.h:126-130)";
            return TL_ERR_UNSUPPORTED;
        }
    }
    to_rows(N, M, h.col_ptr, h.row_ind, raw_v, h.raw_rp, h.raw_vc);
    // net stoichiometry (duplicates merged, zeros dropped)
    h.net_cp.assign((size_t)M + 1, 0);
    std::vector<int32_t> nrows;
    std::vector<int> nvals;
    nrows.reserve((size_t)nnz);
    nvals.reserve((size_t)nnz);
    std::vector<std::pair<int, int>> col;  // one column's (species, v), reused
    for (int j = 0; j < M; ++j) {
        // the column's entries by species (columns hold a handful of
        // entries: insertion sort), duplicates summed, zeros dropped
        col.clear();
        for (int q = h.col_ptr[(size_t)j]; q < h.col_ptr[(size_t)j + 1]; ++q) {
            std::pair<int, int> e{h.row_ind[(size_t)q], (int)h.stoich[(size_t)q]};
            size_t k = col.size();
            col.push_back(e);
            while (k > 0 && col[k - 1].first > e.first) {
                col[k] = col[k - 1];
                --k;
            }
            col[k] = e;
        }
        for (size_t a = 0; a < col.size();) {
            const int sp = col[a].first;
            int v = 0;
            for (; a < col.size() && col[a].first == sp; ++a) v += col[a].second;
            if (v == 0) continue;
            if (!packable(v)) {
                err = "net stoichiometry outside [-2, 5] cannot be packed";
                return TL_ERR_UNSUPPORTED;
            }
            nrows.push_back(sp);
            nvals.push_back(v);
        }
        h.net_cp[(size_t)j + 1] = (int32_t)nrows.size();
    }
    h.net_rv.resize(nrows.size());
    for (size_t q = 0; q < nrows.size(); ++q) h.net_rv[q] = pack(nrows[q], nvals[q]);
    to_rows(N, M, h.net_cp, nrows, nvals, h.net_rp, h.net_vc);
    h.max_row = 0;
    for (int i = 0; i < N; ++i) h.max_row = std::max(h.max_row, h.net_rp[(size_t)i + 1] - h.net_rp[(size_t)i]);
    // processing order of species rows: longest first, so the rows a warp
    // walks side by side have similar lengths
    h.rowperm.resize((size_t)N);
    for (int i = 0; i < N; ++i) h.rowperm[(size_t)i] = i;
    std::stable_sort(h.rowperm.begin(), h.rowperm.end(), [&](int a, int b) {
        return h.net_rp[(size_t)a + 1] - h.net_rp[(size_t)a] > h.net_rp[(size_t)b + 1] - h.net_rp[(size_t)b];
    });
    if ((int)h.names.size() != N) {
        h.names.resize((size_t)N);
        for (int i = 0; i < N; ++i) h.names[(size_t)i] = "S" + std::to_string(i + 1);
    }
    return TL_OK;
}

}  // namespace tl
