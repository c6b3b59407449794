// tl_internal.h - host-side structures shared by the C ABI, the model
// builder, the StochKit reader and the kernel launchers.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/tl.h"

namespace tl {

// One channel as written in a StochKit file: reactant / product species with
// stoichiometries (ReactionProp, tau_leaping/StochKitReader.h:18-23).
struct Channel {
    double rate = 0.0;
    std::vector<std::pair<int, int>> reactants;  // (species, stoich), XML order
    std::vector<std::pair<int, int>> products;
};

struct HostModel {
    int N = 0, M = 0;
    int pop_bits = 32;
    std::vector<int64_t> x0;
    std::vector<double> rate;
    // raw channel-major entries (reference layout, duplicates allowed)
    std::vector<int32_t> col_ptr, row_ind;
    std::vector<int8_t> stoich;
    // derived
    std::vector<int8_t> order;      // 0 none, 1 S, 2 S+S', 3 2S
    std::vector<int8_t> ref_order;  // the reference's detector (-1,1,2,3)
    std::vector<int32_t> s0, s1;
    std::vector<int8_t> gkind;      // per species, see g_of()
    std::vector<int32_t> raw_rp, raw_vc;   // species-row CSR of raw entries (packed)
    std::vector<int32_t> net_rp, net_vc;   // species-row CSR of net stoichiometry
    std::vector<int32_t> net_cp, net_rv;   // channel-column CSC of net stoichiometry
    std::vector<int32_t> rowperm;          // species rows by net length, longest first
    std::vector<std::string> names;
    int max_order = 0;
    int max_row = 0;  // longest net species row
};

// Build every derived table from the raw channel-major entries in `h`
// (col_ptr/row_ind/stoich/x0/rate/N/M filled).  Returns TL_OK or an error
// with a message.
tl_status derive_tables(HostModel& h, std::string& err);

// Raw entries for channel lists the way ReadXMLToMatrixStruct builds them
// (tau_leaping/CSCHostMatrixData.cpp:19-107).
void channels_to_raw(const std::vector<Channel>& ch, HostModel& h);

tl_status parse_stochkit_file(const char* path, HostModel& h, std::vector<Channel>& ch,
                              std::string& err);
tl_status write_stochkit_file(const char* path, const HostModel& h, const std::vector<Channel>& ch,
                              const char* description, std::string& err);

tl_status generate_model(const tl_gen_params& g, HostModel& h, std::vector<Channel>& ch, std::string& err);

void set_last_error(const std::string& s);

// ---------------------------------------------------------------------------
// Device side of a model.
// ---------------------------------------------------------------------------
struct DevModel {
    int device = 0;
    unsigned char* blob = nullptr;  // staged constants (net) followed by raw CSR
    size_t blob_bytes = 0;
    int stage_bytes = 0;            // bytes of the net part (what a CTA stages)
    int off_chan = 0, off_rord = 0, off_gkind = 0, off_perm = 0, off_rp = 0, off_vc = 0, off_cp = 0, off_rv = 0;
    int off_raw_rp = 0, off_raw_vc = 0;
    void* x0 = nullptr;             // Pop[N]
    float* rate = nullptr;          // [M]
    int nnz_net = 0, nnz_raw = 0;
};

}  // namespace tl

struct tl_model {
    tl::HostModel h;
    std::vector<tl::Channel> channels;
    tl::DevModel d;
    // scratch (grow-only)
    void* scratch = nullptr;
    size_t scratch_bytes = 0;
    // measured autotuner cache (TL_FLAG_AUTOTUNE_MEASURE)
    int tuned_variant = 0, tuned_block = 0, tuned_nostage = 0;
    unsigned tuned_key = 0;
};
