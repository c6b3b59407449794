// tl_api.cu - the C ABI (include/tl.h): model upload, run configuration,
// the autotuner, kernel launches and result reduction.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "tl_device.cuh"
#include "tl_internal.h"
#include "tl_launch.h"

namespace tl {

static thread_local std::string g_last_error;
static thread_local int g_device = 0;

void set_last_error(const std::string& s) { g_last_error = s; }

static tl_status cuda_fail(cudaError_t e, const char* what) {
    set_last_error(std::string(what) + ": " + cudaGetErrorString(e));
    cudaGetLastError();  // clear a non-sticky error
    return e == cudaErrorMemoryAllocation ? TL_ERR_OUT_OF_MEMORY
           : e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver ? TL_ERR_NO_DEVICE
                                                                          : TL_ERR_CUDA;
}

#define TLC(expr)                                          \
    do {                                                   \
        cudaError_t _e = (expr);                           \
        if (_e != cudaSuccess) return cuda_fail(_e, #expr); \
    } while (0)

static size_t al16(size_t b) { return (b + 15) & ~(size_t)15; }

// Grow-only device scratch owned by the model.
static tl_status scratch_get(tl_model* m, size_t bytes, void** out) {
    if (bytes > m->scratch_bytes) {
        if (m->scratch) cudaFree(m->scratch);
        m->scratch = nullptr;
        m->scratch_bytes = 0;
        TLC(cudaMalloc(&m->scratch, bytes));
        m->scratch_bytes = bytes;
    }
    *out = m->scratch;
    return TL_OK;
}

struct Carver {
    size_t off = 0;
    size_t take(size_t b) {
        const size_t o = off;
        off = (off + b + 255) & ~(size_t)255;
        return o;
    }
};

static tl_status upload(tl_model* m) {
    HostModel& h = m->h;
    DevModel& d = m->d;
    const int N = h.N, M = h.M;
    d.nnz_net = (int)h.net_vc.size();
    d.nnz_raw = (int)h.raw_vc.size();
    // blob: [chan][ref order][gkind][perm][net rp][net vc][net cp][net rv] | [raw rp][raw vc]
    size_t off = 0;
    auto sect = [&](size_t bytes) {
        const size_t o = off;
        off += al16(bytes);
        return (int)o;
    };
    d.off_chan = sect((size_t)M * 8);
    d.off_rord = sect((size_t)M);
    d.off_gkind = sect((size_t)N);
    d.off_perm = sect((size_t)N * 4);
    d.off_rp = sect((size_t)(N + 1) * 4);
    d.off_vc = sect((size_t)d.nnz_net * 4);
    d.off_cp = sect((size_t)(M + 1) * 4);
    d.off_rv = sect((size_t)d.nnz_net * 4);
    d.stage_bytes = (int)off;
    d.off_raw_rp = sect((size_t)(N + 1) * 4);
    d.off_raw_vc = sect((size_t)d.nnz_raw * 4);
    d.blob_bytes = off;
    std::vector<unsigned char> hb(off, 0);
    // channel record: {s0, s1 | order << 28} (species indices < 2^28)
    int2* chan = reinterpret_cast<int2*>(hb.data() + d.off_chan);
    for (int j = 0; j < M; ++j)
        chan[j] = make_int2(h.s0[(size_t)j], h.s1[(size_t)j] | ((int)h.order[(size_t)j] << 28));
    memcpy(hb.data() + d.off_rord, h.ref_order.data(), (size_t)M);
    memcpy(hb.data() + d.off_gkind, h.gkind.data(), (size_t)N);
    memcpy(hb.data() + d.off_perm, h.rowperm.data(), (size_t)N * 4);
    memcpy(hb.data() + d.off_rp, h.net_rp.data(), (size_t)(N + 1) * 4);
    if (d.nnz_net) memcpy(hb.data() + d.off_vc, h.net_vc.data(), (size_t)d.nnz_net * 4);
    memcpy(hb.data() + d.off_cp, h.net_cp.data(), (size_t)(M + 1) * 4);
    if (d.nnz_net) memcpy(hb.data() + d.off_rv, h.net_rv.data(), (size_t)d.nnz_net * 4);
    memcpy(hb.data() + d.off_raw_rp, h.raw_rp.data(), (size_t)(N + 1) * 4);
    if (d.nnz_raw) memcpy(hb.data() + d.off_raw_vc, h.raw_vc.data(), (size_t)d.nnz_raw * 4);
    TLC(cudaMalloc(&d.blob, off));
    TLC(cudaMemcpy(d.blob, hb.data(), off, cudaMemcpyHostToDevice));
    const size_t w = h.pop_bits == 64 ? 8 : 4;
    TLC(cudaMalloc(&d.x0, (size_t)N * w));
    if (w == 8) {
        std::vector<long long> x(h.x0.begin(), h.x0.end());
        TLC(cudaMemcpy(d.x0, x.data(), (size_t)N * 8, cudaMemcpyHostToDevice));
    } else {
        std::vector<int> x(h.x0.begin(), h.x0.end());
        TLC(cudaMemcpy(d.x0, x.data(), (size_t)N * 4, cudaMemcpyHostToDevice));
    }
    std::vector<float> r(h.rate.begin(), h.rate.end());
    TLC(cudaMalloc(&d.rate, (size_t)M * 4));
    TLC(cudaMemcpy(d.rate, r.data(), (size_t)M * 4, cudaMemcpyHostToDevice));
    return TL_OK;
}

static tl_status finish_model(tl_model* m, tl_model** out) {
    std::string err;
    tl_status s = derive_tables(m->h, err);
    if (s != TL_OK) {
        set_last_error(err);
        delete m;
        return s;
    }
    m->d.device = g_device;  // device tables are uploaded on first use
    *out = m;
    return TL_OK;
}

static tl_status ensure_device(tl_model* m) {
    if (m->d.blob) return TL_OK;
    TLC(cudaSetDevice(m->d.device));
    return upload(m);
}

static MView global_view(const tl_model* m, bool raw_mu, bool raw_update) {
    const DevModel& d = m->d;
    const unsigned char* b = d.blob;
    MView v;
    v.chan = reinterpret_cast<const int2*>(b + d.off_chan);
    v.rord = reinterpret_cast<const signed char*>(b + d.off_rord);
    v.gkind = reinterpret_cast<const signed char*>(b + d.off_gkind);
    v.perm = reinterpret_cast<const int*>(b + d.off_perm);
    const int* nrp = reinterpret_cast<const int*>(b + d.off_rp);
    const int* nvc = reinterpret_cast<const int*>(b + d.off_vc);
    const int* rrp = reinterpret_cast<const int*>(b + d.off_raw_rp);
    const int* rvc = reinterpret_cast<const int*>(b + d.off_raw_vc);
    v.rp = raw_mu ? rrp : nrp;
    v.vc = raw_mu ? rvc : nvc;
    v.urp = raw_update ? rrp : nrp;
    v.uvc = raw_update ? rvc : nvc;
    v.cp = reinterpret_cast<const int*>(b + d.off_cp);
    v.rv = reinterpret_cast<const int*>(b + d.off_rv);
    return v;
}

// One group's slot: x, x' and a[]; scored runs add the firing counts.
static size_t slot_bytes(const tl_model* m, bool sens = false) {
    const size_t w = m->h.pop_bits == 64 ? 8 : 4;
    return al16((size_t)m->h.N * w) * 2 + al16((size_t)m->h.M * 4) * (sens ? 2 : 1);
}

static int max_smem_optin() {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    return v > 0 ? v : 48 * 1024;
}

static int sm_count() {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    return v > 0 ? v : 1;
}

// Launch plan for the fused kernel.
struct Plan {
    int kind = 32;      // 1, 32, 0
    int block = 256;
    int grid = 1;
    size_t smem = 0;
    int stage = 0;      // staged bytes (0 = constants read through L1/L2)
    int variant = TL_VARIANT_WARP;
    bool row_warp = false;
    bool gslot = false;  // CTA groups: the slot lives in global memory
};

// The kernel a plan launches (CTA groups with global slots are their own build).
static int launch_kind(const Plan& pl) { return pl.gslot ? kKindCtaGlobal : pl.kind; }

// Autotuner, heuristic part: the group width follows the model size.
//  * a handful of channels: one realization per thread (all lanes busy on
//    independent realizations); small ensembles use small blocks so that
//    every SM gets work;
//  * per-realization state up to 8 KB: a group of W lanes of a warp per
//    realization, 256-thread blocks, model tables staged in shared memory.
//    W is the smallest of 8, 16 and 32 that leaves each lane at most 16
//    channels and 8 species rows, provided the ensemble fills the GPU's
//    warp-group slots at least 8 times over (smaller ensembles keep whole
//    warps, whose realizations finish sooner); scored runs keep whole warps
//    (the sub-warp kinds have no scores-only build).  Measured on GB300 over
//    eight model sizes: 32-channel chain 8 lanes 9.8e8 against a warp 4.3e8,
//    32 x 64 network 8 lanes 9.6e8 against 6.9e8, the 128 x 256 toy network
//    16 lanes 3.64e8 against 3.50e8, 128-channel chain 16 lanes = warp,
//    256 x 512 network and the 40-species colloid a warp;
//  * up to 64 KB: one 128-thread (up to 1024 channels) or 256-thread CTA per
//    realization, tables through L1/L2 (chain-sized models: 1024 species
//    and channels);
//  * larger: one 1024-thread CTA per realization (propensities of ~30k
//    channels fill most of the 227 KB of shared memory).
// The choices follow sweeps of the (variant, block, staging) plans on GB300.
static int heuristic_variant(const tl_model* m, size_t sb, long long total, int mode, int nsm) {
    const int M = m->h.M, N = m->h.N;
    if (M <= 16 && N <= 16) return TL_VARIANT_THREAD;
    if (sb > 8 * 1024) return TL_VARIANT_CTA;
    // warp groups: 256-thread CTAs, 5 per SM
    constexpr long long kWarpGroupsPerSm = 40;
    if (mode != kModeScores && total >= 8 * kWarpGroupsPerSm * (long long)nsm) {
        if (M <= 16 * 8 && N <= 8 * 8) return TL_VARIANT_LANES8;
        if (M <= 16 * 16 && N <= 8 * 16) return TL_VARIANT_LANES16;
    }
    return TL_VARIANT_WARP;
}

static tl_status make_plan(const tl_model* m, int variant, int block_req, int mode, bool compat_stoich,
                           bool no_stage, long long total, Plan& pl, bool force_gslot = false) {
    const size_t sb = slot_bytes(m, mode != kModeFast);
    const int smax = max_smem_optin() - 2048;
    const int stage = (compat_stoich || no_stage) ? 0 : m->d.stage_bytes;
    const bool autov = variant == TL_VARIANT_AUTO;
    const int nsm = sm_count();
    if (autov) variant = heuristic_variant(m, sb, total, mode, nsm);
    pl.variant = variant;
    int groups_per_block = 1;
    if (variant == TL_VARIANT_THREAD) {
        pl.kind = 1;
        int b = block_req;
        if (b <= 0) {
            // spread small ensembles over every SM
            const long long per_sm = (total + nsm - 1) / nsm;
            b = (int)std::min<long long>(128, std::max<long long>(32, (per_sm + 31) / 32 * 32));
        }
        pl.block = b;
        groups_per_block = pl.block;
    } else if (variant == TL_VARIANT_WARP) {
        pl.kind = 32;
        pl.block = block_req > 0 ? block_req : 256;
        groups_per_block = pl.block / 32;
    } else if (variant >= TL_VARIANT_LANES2 && variant <= TL_VARIANT_LANES16) {
        pl.kind = 2 << (variant - TL_VARIANT_LANES2);
        pl.block = block_req > 0 ? block_req : 256;
        groups_per_block = pl.block / pl.kind;
    } else if (variant == TL_VARIANT_CTA) {
        pl.kind = 0;
        // chain-sized models (up to 1024 channels): 128 threads, 8 channels
        // each (cyclic chain 1024: 3.67e7 realization-steps/s against 3.41e7
        // at 256); up to 64 KB of state: 256; larger: 1024
        pl.block = block_req > 0 ? block_req : (sb <= 64 * 1024 ? (m->h.M <= 1024 ? 128 : 256) : 1024);
        groups_per_block = 1;
    } else {
        set_last_error("unknown variant");
        return TL_ERR_INVALID_ARGUMENT;
    }
    if (pl.block % 32 || pl.block < 32 || pl.block > (pl.kind == 0 ? 1024 : 256)) {
        set_last_error("block_threads must be a multiple of 32 in [32, 256] (thread / warp groups) "
                       "or [32, 1024] (CTA groups)");
        return TL_ERR_INVALID_ARGUMENT;
    }
    // shrink the block until the slots fit
    while ((size_t)groups_per_block * sb > (size_t)smax && pl.kind != 0 && pl.block > 32) {
        pl.block -= 32;
        groups_per_block = pl.block / pl.kind;
    }
    if (force_gslot && pl.kind == 0) pl.gslot = true;
    if ((size_t)groups_per_block * sb > (size_t)smax) {
        if (pl.kind != 0) {
            set_last_error("model too large for the shared-memory slot of this variant");
            return TL_ERR_UNSUPPORTED;
        }
        // one realization's state exceeds shared memory: CTA groups keep it
        // in global memory (one slot per CTA, served from L2)
        pl.gslot = true;
    }
    // chain-sized CTA groups leave the tables in L1/L2 (staging them would
    // cost more shared memory than the realization itself)
    const bool stage_ok = !(autov && pl.kind == 0 && sb <= 64 * 1024);
    const size_t slot_smem = pl.gslot ? 0 : (size_t)groups_per_block * sb;
    pl.stage = (stage_ok && slot_smem + (size_t)stage <= (size_t)smax) ? stage : 0;
    pl.smem = (size_t)pl.stage + slot_smem;
    pl.row_warp = pl.kind == 0 && m->h.max_row > 32;
    int bps = 0;
    const int lk = pl.gslot ? kKindCtaGlobal : pl.kind;
    cudaError_t e = m->h.pop_bits == 64 ? fused_occupancy<long long>(lk, mode, pl.block, pl.smem, &bps)
                                        : fused_occupancy<int>(lk, mode, pl.block, pl.smem, &bps);
    if (e != cudaSuccess) return cuda_fail(e, "occupancy");
    if (bps < 1) {
        set_last_error("the launch does not fit an SM");
        return TL_ERR_UNSUPPORTED;
    }
    const long long need = (total + groups_per_block - 1) / groups_per_block;
    pl.grid = (int)std::min<long long>((long long)nsm * bps, std::max<long long>(need, 1));
    return TL_OK;
}

struct RunBuffers {
    float* rates = nullptr;
    double* tfin = nullptr;
    double* grid = nullptr;
    int* tracked = nullptr;
    void* samples = nullptr;
    float* scores = nullptr;
    unsigned long long* ctr = nullptr;
    double* mean = nullptr;
    double* sd = nullptr;
    double* grad = nullptr;
    double* gse = nullptr;
    double* gmean = nullptr;
    void* pstate = nullptr;
    void* pslots = nullptr;
    float* a_all = nullptr;
};

// One (model, configuration) pair of a call: validation, scratch layout,
// device parameters, reduction and result.
struct Job {
    tl_model* m = nullptr;
    const tl_run_cfg* cfg = nullptr;
    tl_result* res = nullptr;
    tl_grad_result* grad = nullptr;
    int S = 1, P = 2, K = 0;
    long long R = 1, total = 1;
    bool sens = false, keep = false, plain = false, compat_stoich = false;
    int mode = kModeFast;  // the kernel build: scores and / or compatibility switches
    size_t w = 4;
    std::vector<float> hrates;
    std::vector<double> htf;
    std::vector<double> hgrid;  // [S][P] grid times
    Plan pl;
    size_t o_rates = 0, o_tf = 0, o_grid = 0, o_tr = 0, o_samp = 0, o_sc = 0, o_ctr = 0, o_mean = 0, o_sd = 0, o_grad = 0,
           o_gse = 0, o_gm = 0, o_ps = 0, o_pslot = 0, o_aall = 0, o_gslot = 0;
    RunBuffers rb;
    SimParams p{};
    std::vector<unsigned char> hs;
    unsigned long long hc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
};

static tl_status job_prepare(Job& J) {
    tl_model* m = J.m;
    const tl_run_cfg* cfg = J.cfg;
    if (!m || !cfg) {
        set_last_error("null model or config");
        return TL_ERR_INVALID_ARGUMENT;
    }
    const HostModel& h = m->h;
    const int N = h.N, M = h.M;
    if (!(cfg->t_final > 0.0) || !std::isfinite(cfg->t_final) || !(cfg->eps > 0.0) || cfg->n_realizations < 1 ||
        cfg->n_intervals < 1 || cfg->n_tracked < 0 || cfg->n_rate_sets < 0 || cfg->max_steps < 0) {
        set_last_error("invalid run configuration (t_final > 0, eps > 0, n >= 1, intervals >= 1)");
        return TL_ERR_INVALID_ARGUMENT;
    }
    if (cfg->n_realizations + cfg->realization_offset > 0xFFFFFFFFLL || cfg->realization_offset < 0 ||
        cfg->n_rate_sets >= (1 << 24)) {
        set_last_error("at most 2^32 realizations per set and 2^24 rate sets");
        return TL_ERR_INVALID_ARGUMENT;
    }
    if (cfg->n_tracked > 0 && !cfg->tracked) {
        set_last_error("tracked is NULL");
        return TL_ERR_INVALID_ARGUMENT;
    }
    for (int q = 0; q < cfg->n_tracked; ++q)
        if (cfg->tracked[q] < 0 || cfg->tracked[q] >= N) {
            set_last_error("tracked species index out of range");
            return TL_ERR_INVALID_ARGUMENT;
        }
    if (cfg->n_rate_sets > 0 && !cfg->rate_sets) {
        set_last_error("rate_sets is NULL");
        return TL_ERR_INVALID_ARGUMENT;
    }
    J.S = std::max(1, cfg->n_rate_sets);
    J.R = cfg->n_realizations;
    J.P = cfg->n_intervals + 1;
    J.K = cfg->n_tracked;
    J.total = J.R * J.S;
    J.sens = J.grad != nullptr;
    J.mode = (cfg->flags & TL_FLAG_COMPAT_REFERENCE) ? kModeGeneral : J.sens ? kModeScores : kModeFast;
    J.keep = (cfg->flags & TL_FLAG_KEEP_SAMPLES) != 0;
    J.plain = cfg->variant == TL_VARIANT_PLAIN;
    J.compat_stoich = (cfg->flags & TL_FLAG_COMPAT_STOICH) != 0;
    J.w = h.pop_bits == 64 ? 8 : 4;
    if (J.plain && J.sens) {
        set_last_error("the plain form has no sensitivity pass");
        return TL_ERR_UNSUPPORTED;
    }
    if (J.sens && J.K < 1) {
        set_last_error("sensitivity needs at least one tracked species");
        return TL_ERR_INVALID_ARGUMENT;
    }
    J.hrates.assign((size_t)J.S * M, 0.f);
    J.htf.assign((size_t)J.S, cfg->t_final);
    for (int s = 0; s < J.S; ++s)
        for (int j = 0; j < M; ++j) {
            const double c = cfg->n_rate_sets > 0 ? cfg->rate_sets[(size_t)s * M + j] : h.rate[(size_t)j];
            if (!std::isfinite(c) || c < 0.0) {
                set_last_error("rate constants must be finite and >= 0");
                return TL_ERR_NUMERIC;
            }
            J.hrates[(size_t)s * M + j] = (float)c;
        }
    if (cfg->n_rate_sets > 0 && cfg->t_final_sets)
        for (int s = 0; s < J.S; ++s) {
            J.htf[(size_t)s] = cfg->t_final_sets[s];
            if (!(J.htf[(size_t)s] > 0.0) || !std::isfinite(J.htf[(size_t)s])) {
                set_last_error("t_final_sets must be > 0");
                return TL_ERR_INVALID_ARGUMENT;
            }
        }
    // grid t_k = T*k/n_int (FP64, the last point T itself)
    J.hgrid.resize((size_t)J.S * J.P);
    for (int s = 0; s < J.S; ++s)
        for (int k = 0; k < J.P; ++k)
            J.hgrid[(size_t)s * J.P + k] = k >= cfg->n_intervals
                                               ? J.htf[(size_t)s]
                                               : J.htf[(size_t)s] * (double)k / (double)cfg->n_intervals;
    return ensure_device(m);
}

static void job_layout(Job& J, Carver& c) {
    const int M = J.m->h.M, N = J.m->h.N, K1 = std::max(J.K, 1);
    J.o_rates = c.take((size_t)J.S * M * 4);
    J.o_tf = c.take((size_t)J.S * 8);
    J.o_grid = c.take((size_t)J.S * J.P * 8);
    J.o_tr = c.take((size_t)K1 * 4);
    J.o_samp = c.take((size_t)J.total * J.P * K1 * J.w);
    J.o_sc = J.sens ? c.take((size_t)J.total * M * 4) : 0;
    J.o_ctr = c.take(8 * 8);
    J.o_mean = c.take((size_t)J.S * J.P * K1 * 8);
    J.o_sd = c.take((size_t)J.S * J.P * K1 * 8);
    J.o_grad = J.sens ? c.take((size_t)J.S * J.K * M * 8) : 0;
    J.o_gse = J.sens ? c.take((size_t)J.S * J.K * M * 8) : 0;
    J.o_gm = J.sens ? c.take((size_t)J.S * J.K * 8) : 0;
    J.o_ps = J.plain ? c.take((size_t)J.total * 64) : 0;
    J.o_pslot = J.plain ? c.take((size_t)J.total * 2 * al16((size_t)N * J.w)) : 0;
    J.o_aall = J.plain ? c.take((size_t)J.total * M * 4) : 0;
    J.o_gslot = (!J.plain && J.pl.gslot) ? c.take((size_t)J.pl.grid * slot_bytes(J.m, J.mode != kModeFast)) : 0;
}

static tl_status job_bind(Job& J, unsigned char* B, cudaStream_t st) {
    tl_model* m = J.m;
    const tl_run_cfg* cfg = J.cfg;
    RunBuffers& rb = J.rb;
    rb.rates = reinterpret_cast<float*>(B + J.o_rates);
    rb.tfin = reinterpret_cast<double*>(B + J.o_tf);
    rb.grid = reinterpret_cast<double*>(B + J.o_grid);
    rb.tracked = reinterpret_cast<int*>(B + J.o_tr);
    rb.samples = B + J.o_samp;
    rb.scores = J.sens ? reinterpret_cast<float*>(B + J.o_sc) : nullptr;
    rb.ctr = reinterpret_cast<unsigned long long*>(B + J.o_ctr);
    rb.mean = reinterpret_cast<double*>(B + J.o_mean);
    rb.sd = reinterpret_cast<double*>(B + J.o_sd);
    if (J.sens) {
        rb.grad = reinterpret_cast<double*>(B + J.o_grad);
        rb.gse = reinterpret_cast<double*>(B + J.o_gse);
        rb.gmean = reinterpret_cast<double*>(B + J.o_gm);
    }
    if (J.plain) {
        rb.pstate = B + J.o_ps;
        rb.pslots = B + J.o_pslot;
        rb.a_all = reinterpret_cast<float*>(B + J.o_aall);
    }
    TLC(cudaMemcpyAsync(rb.rates, J.hrates.data(), J.hrates.size() * 4, cudaMemcpyHostToDevice, st));
    TLC(cudaMemcpyAsync(rb.tfin, J.htf.data(), J.htf.size() * 8, cudaMemcpyHostToDevice, st));
    TLC(cudaMemcpyAsync(rb.grid, J.hgrid.data(), J.hgrid.size() * 8, cudaMemcpyHostToDevice, st));
    if (J.K > 0) TLC(cudaMemcpyAsync(rb.tracked, cfg->tracked, (size_t)J.K * 4, cudaMemcpyHostToDevice, st));
    TLC(cudaMemsetAsync(rb.ctr, 0, 64, st));
    SimParams& p = J.p;
    p = SimParams{};
    p.N = m->h.N;
    p.M = m->h.M;
    p.g = global_view(m, J.compat_stoich, false);
    p.x0 = m->d.x0;
    p.rates = rb.rates;
    p.t_final = rb.tfin;
    p.grid = rb.grid;
    p.R = J.R;
    p.r_off = cfg->realization_offset;
    p.S = J.S;
    p.k0 = (uint32_t)(cfg->seed & 0xFFFFFFFFu);
    p.k1 = (uint32_t)(cfg->seed >> 32);
    round_keys(p.k0, p.k1, p.rk);
    p.eps = (float)cfg->eps;
    p.nc = cfg->n_critical > 0 ? cfg->n_critical : 5;
    p.ssa_factor = (float)(cfg->ssa_factor > 0 ? cfg->ssa_factor : 10);
    p.ssa_block = cfg->ssa_block > 0 ? cfg->ssa_block : 100;
    p.n_int = cfg->n_intervals;
    p.K = J.K;
    p.tracked = rb.tracked;
    p.samples = rb.samples;
    p.scores = rb.scores;
    p.max_steps = cfg->max_steps;
    p.flags = cfg->flags;
    p.max_halv = cfg->max_halvings > 0 ? cfg->max_halvings : 64;
    p.wait_polls = cfg->stage_wait_polls == 0 ? (1 << 22) : std::max(cfg->stage_wait_polls, 0);
    p.blob = m->d.blob;
    p.stage_bytes = J.pl.stage;
    p.off_chan = m->d.off_chan;
    p.off_rord = m->d.off_rord;
    p.off_gkind = m->d.off_gkind;
    p.off_perm = m->d.off_perm;
    p.off_rp = m->d.off_rp;
    p.off_vc = m->d.off_vc;
    p.off_cp = m->d.off_cp;
    p.off_rv = m->d.off_rv;
    p.slot_bytes = (int)slot_bytes(m, J.mode != kModeFast);
    p.row_warp = J.pl.row_warp ? 1 : 0;
    p.gslots = J.pl.gslot ? B + J.o_gslot : nullptr;
    p.ctr = rb.ctr;
    p.pstate = rb.pstate;
    p.pslots = rb.pslots;
    return TL_OK;
}

// Statistics / gradient reductions and the device-to-host copies.
static tl_status job_reduce(Job& J, cudaStream_t st) {
    const int M = J.m->h.M;
    RunBuffers& rb = J.rb;
    cudaError_t le;
    if (J.K > 0) {
        le = J.w == 8 ? launch_stats<long long>(rb.samples, J.R, J.P, J.K, J.S, rb.mean, rb.sd, st)
                      : launch_stats<int>(rb.samples, J.R, J.P, J.K, J.S, rb.mean, rb.sd, st);
        if (le != cudaSuccess) return cuda_fail(le, "statistics launch");
    }
    if (J.sens) {
        le = J.w == 8 ? launch_grad<long long>(rb.samples, rb.scores, J.R, J.P, J.K, M, J.S, rb.grad, rb.gse, rb.gmean, st)
                      : launch_grad<int>(rb.samples, rb.scores, J.R, J.P, J.K, M, J.S, rb.grad, rb.gse, rb.gmean, st);
        if (le != cudaSuccess) return cuda_fail(le, "gradient launch");
    }
    TLC(cudaMemcpyAsync(J.hc, rb.ctr, 64, cudaMemcpyDeviceToHost, st));
    const size_t SPK = (size_t)J.S * J.P * J.K;
    if (J.res) {
        if (J.res->mean && J.K > 0) TLC(cudaMemcpyAsync(J.res->mean, rb.mean, SPK * 8, cudaMemcpyDeviceToHost, st));
        if (J.res->stddev && J.K > 0) TLC(cudaMemcpyAsync(J.res->stddev, rb.sd, SPK * 8, cudaMemcpyDeviceToHost, st));
        if (J.res->samples && J.keep && J.K > 0) {
            J.hs.resize((size_t)J.total * J.P * J.K * J.w);
            TLC(cudaMemcpyAsync(J.hs.data(), rb.samples, J.hs.size(), cudaMemcpyDeviceToHost, st));
        }
    }
    if (J.sens) {
        tl_grad_result* g = J.grad;
        const size_t SKM = (size_t)J.S * J.K * M;
        if (g->grad) TLC(cudaMemcpyAsync(g->grad, rb.grad, SKM * 8, cudaMemcpyDeviceToHost, st));
        if (g->grad_stderr) TLC(cudaMemcpyAsync(g->grad_stderr, rb.gse, SKM * 8, cudaMemcpyDeviceToHost, st));
        if (g->mean_final)
            TLC(cudaMemcpyAsync(g->mean_final, rb.gmean, (size_t)J.S * J.K * 8, cudaMemcpyDeviceToHost, st));
    }
    return TL_OK;
}

// After the stream is synchronised: fill the result, map error bits.
static tl_status job_finish(Job& J, double kernel_ms, int launches, double total_ms) {
    tl_result* res = J.res;
    if (!J.hs.empty()) {
        const size_t n = (size_t)J.total * J.P * J.K;
        if (J.w == 8) memcpy(res->samples, J.hs.data(), n * 8);
        else {
            const int* src = reinterpret_cast<const int*>(J.hs.data());
            for (size_t q = 0; q < n; ++q) res->samples[q] = src[q];
        }
    }
    if (res) {
        if (res->times) std::copy(J.hgrid.begin(), J.hgrid.end(), res->times);
        res->leaps = (int64_t)J.hc[1];
        res->ssa_steps = (int64_t)J.hc[2];
        res->rejections = (int64_t)J.hc[3];
        res->truncated = (int64_t)J.hc[4];
        res->kernel_ms = kernel_ms;
        res->variant_used = J.pl.variant;
        res->block_threads_used = J.pl.block;
        res->grid_used = J.pl.grid;
        res->launches = launches;
        res->total_ms = total_ms;
    }
    const unsigned eb = (unsigned)J.hc[5];
    if (eb & kErrWaitTimeout) {
        set_last_error("shared-memory staging wait timed out");
        return TL_ERR_WAIT_TIMEOUT;
    }
    if (eb & kErrOverflow) {
        set_last_error("a population left the range of the population type");
        return TL_ERR_OVERFLOW;
    }
    if (eb & (kErrHalving | kErrNumeric)) {
        set_last_error("a leap could not be made non-negative by halving tau " +
                       std::to_string(J.p.max_halv) + " times (max_halvings)");
        return TL_ERR_NUMERIC;
    }
    if (J.hc[4] > 0) {
        set_last_error("max_steps reached; truncated realizations hold their last state");
        return TL_ERR_STEP_CAP;
    }
    return TL_OK;
}

static double ms_since(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

// Autotuner, measured part (TL_FLAG_AUTOTUNE_MEASURE): time every plan that
// fits on the first realizations of this very ensemble (identical streams,
// so identical work per candidate), keep the fastest in the model handle,
// keyed by the flags that change the kernel.  The trial writes only the
// prefix of the sample buffer, which the real run then overwrites.
static tl_status autotune_measure(Job& J, cudaStream_t st) {
    tl_model* m = J.m;
    const bool planned_gslot = J.pl.gslot;
    const int planned_grid = J.pl.grid;
    unsigned char* const planned_gslots = J.p.gslots;
    // the best plan depends on how many realizations fill the GPU: key the
    // cache by the ensemble size (power-of-two bucket) as well
    int bucket = 0;
    while (bucket < 40 && (1LL << bucket) < J.total) ++bucket;
    const unsigned key = 0x80000000u | (J.sens ? 1u : 0u) | (J.compat_stoich ? 2u : 0u) | ((unsigned)bucket << 2) |
                         (unsigned)(J.cfg->flags & ~(TL_FLAG_KEEP_SAMPLES | TL_FLAG_AUTOTUNE_MEASURE)) << 8;
    if (m->tuned_key != key) {
        struct Cand {
            int variant, block;
            bool nostage;
        };
        std::vector<Cand> cands;
        if (m->h.M <= 64 && m->h.N <= 64)
            for (int b : {32, 64, 128}) cands.push_back({TL_VARIANT_THREAD, b, false});
        if (m->h.M <= 1024)
            for (int v = TL_VARIANT_LANES2; v <= TL_VARIANT_LANES16; ++v)
                for (int b : {128, 256}) cands.push_back({v, b, false});
        for (int b : {64, 128, 256})
            for (bool ns : {false, true}) cands.push_back({TL_VARIANT_WARP, b, ns});
        for (int b : {64, 128, 256, 512, 1024})
            for (bool ns : {false, true}) cands.push_back({TL_VARIANT_CTA, b, ns});
        // a prefix large enough to fill the GPU under every candidate
        const long long trial = std::min<long long>(J.total, 16384);
        SimParams tp = J.p;
        tp.R = trial;
        tp.S = 1;
        cudaEvent_t e0, e1;
        TLC(cudaEventCreate(&e0));
        TLC(cudaEventCreate(&e1));
        float best = 3.4e38f;
        Cand win{0, 0, false};
        for (const Cand& c : cands) {
            Plan pl;
            if (make_plan(m, c.variant, c.block, J.mode, J.compat_stoich, c.nostage, trial, pl) != TL_OK) continue;
            if (c.variant == TL_VARIANT_THREAD && c.block != pl.block) continue;
            // global slots exist for the launch the heuristic planned
            if (pl.gslot && (!planned_gslot || pl.grid > planned_grid)) continue;
            tp.stage_bytes = pl.stage;
            tp.row_warp = pl.row_warp ? 1 : 0;
            tp.gslots = pl.gslot ? planned_gslots : nullptr;
            if (cudaMemsetAsync(tp.ctr, 0, 64, st) != cudaSuccess) break;
            cudaEventRecord(e0, st);
            cudaError_t le = J.w == 8 ? launch_fused<long long>(tp, launch_kind(pl), J.mode, pl.block, pl.grid, pl.smem, st)
                                      : launch_fused<int>(tp, launch_kind(pl), J.mode, pl.block, pl.grid, pl.smem, st);
            cudaEventRecord(e1, st);
            if (le != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess) {
                cudaGetLastError();
                continue;
            }
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (ms < best) {
                best = ms;
                win = c;
            }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        TLC(cudaMemsetAsync(J.p.ctr, 0, 64, st));
        if (win.variant == 0) {
            set_last_error("autotuner found no plan that fits");
            return TL_ERR_UNSUPPORTED;
        }
        m->tuned_key = key;
        m->tuned_variant = win.variant;
        m->tuned_block = win.block;
        m->tuned_nostage = win.nostage ? 1 : 0;
    }
    tl_status ps = make_plan(m, m->tuned_variant, m->tuned_block, J.mode, J.compat_stoich, m->tuned_nostage != 0,
                             J.total, J.pl);
    if (ps != TL_OK) return ps;
    if (J.pl.gslot && (!planned_gslot || J.pl.grid > planned_grid)) {
        // a cached global-slot plan that needs more slots than were laid out:
        // keep the planned launch
        ps = make_plan(m, TL_VARIANT_AUTO, 0, J.mode, J.compat_stoich, (J.cfg->flags & TL_FLAG_NO_STAGE) != 0,
                       J.total, J.pl);
        if (ps != TL_OK) return ps;
    }
    J.p.stage_bytes = J.pl.stage;
    J.p.row_warp = J.pl.row_warp ? 1 : 0;
    J.p.gslots = J.pl.gslot ? planned_gslots : nullptr;
    return TL_OK;
}

static tl_status run(tl_model* m, const tl_run_cfg* cfg, tl_result* res, tl_grad_result* grad) {
    const auto t0 = std::chrono::steady_clock::now();
    Job J;
    J.m = m;
    J.cfg = cfg;
    J.res = res;
    J.grad = grad;
    tl_status ps = job_prepare(J);
    if (ps != TL_OK) return ps;
    TLC(cudaSetDevice(m->d.device));
    cudaStream_t st = (cudaStream_t)cfg->stream;
    const bool no_stage = (cfg->flags & TL_FLAG_NO_STAGE) != 0;
    const bool measure = !J.plain && cfg->variant == TL_VARIANT_AUTO && (cfg->flags & TL_FLAG_AUTOTUNE_MEASURE);
    if (!J.plain) {
        ps = make_plan(m, cfg->variant, cfg->block_threads, J.mode, J.compat_stoich, no_stage, J.total, J.pl,
                       (cfg->flags & TL_FLAG_GLOBAL_SLOTS) != 0);
        if (ps != TL_OK) return ps;
    } else {
        J.pl.variant = TL_VARIANT_PLAIN;
        J.pl.kind = 1;
        J.pl.block = 128;
        J.pl.grid = (int)((J.total + 127) / 128);
    }
    Carver c;
    job_layout(J, c);
    void* base = nullptr;
    ps = scratch_get(m, c.off, &base);
    if (ps != TL_OK) return ps;
    ps = job_bind(J, reinterpret_cast<unsigned char*>(base), st);
    if (ps != TL_OK) return ps;
    if (measure) {
        ps = autotune_measure(J, st);
        if (ps != TL_OK) return ps;
    }
    const SimParams& p = J.p;
    const size_t w = J.w;

    cudaEvent_t e0, e1;
    TLC(cudaEventCreate(&e0));
    TLC(cudaEventCreate(&e1));
    int launches = 0;
    cudaError_t le = cudaEventRecord(e0, st);
    if (le == cudaSuccess) {
        if (!J.plain) {
            le = w == 8 ? launch_fused<long long>(p, launch_kind(J.pl), J.mode, J.pl.block, J.pl.grid, J.pl.smem, st)
                        : launch_fused<int>(p, launch_kind(J.pl), J.mode, J.pl.block, J.pl.grid, J.pl.smem, st);
            launches = 1;
        } else {
            le = w == 8 ? launch_plain_init<long long>(p, st) : launch_plain_init<int>(p, st);
            launches = 1;
            // With TL_FLAG_GRAPH the 16 step launches between two polls are
            // captured once (on a private stream) and replayed as one graph.
            cudaGraphExec_t gexec = nullptr;
            if (le == cudaSuccess && (cfg->flags & TL_FLAG_GRAPH)) {
                cudaStream_t cs = nullptr;
                le = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
                if (le == cudaSuccess) {
                    cudaGraph_t g = nullptr;
                    le = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
                    for (int q = 0; q < 16 && le == cudaSuccess; ++q)
                        le = w == 8 ? launch_plain_step<long long>(p, J.rb.a_all, cs)
                                    : launch_plain_step<int>(p, J.rb.a_all, cs);
                    const cudaError_t ec = cudaStreamEndCapture(cs, &g);
                    if (le == cudaSuccess) le = ec;
                    if (le == cudaSuccess) le = cudaGraphInstantiate(&gexec, g, 0);
                    if (g) cudaGraphDestroy(g);
                    cudaStreamDestroy(cs);
                }
            }
            unsigned long long* hdone = nullptr;
            if (le == cudaSuccess) le = cudaMallocHost(&hdone, 8);
            while (le == cudaSuccess) {
                if (gexec) {
                    le = cudaGraphLaunch(gexec, st);
                    launches += 16;
                } else {
                    for (int q = 0; q < 16 && le == cudaSuccess; ++q) {
                        le = w == 8 ? launch_plain_step<long long>(p, J.rb.a_all, st)
                                    : launch_plain_step<int>(p, J.rb.a_all, st);
                        ++launches;
                    }
                }
                if (le != cudaSuccess) break;
                le = cudaMemcpyAsync(hdone, J.rb.ctr + 6, 8, cudaMemcpyDeviceToHost, st);
                if (le == cudaSuccess) le = cudaStreamSynchronize(st);
                if (le == cudaSuccess && *hdone >= (unsigned long long)J.total) break;
                if (launches > (1 << 26)) {  // a realization that never ends
                    if (gexec) cudaGraphExecDestroy(gexec);
                    cudaFreeHost(hdone);
                    cudaEventDestroy(e0);
                    cudaEventDestroy(e1);
                    set_last_error("plain form exceeded 2^26 launches; set max_steps");
                    return TL_ERR_STEP_CAP;
                }
            }
            if (gexec) cudaGraphExecDestroy(gexec);
            if (hdone) cudaFreeHost(hdone);
            if (le == cudaSuccess) le = launch_plain_tally(p, st);
            ++launches;
        }
    }
    if (le == cudaSuccess) le = cudaEventRecord(e1, st);
    if (le != cudaSuccess) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        return cuda_fail(le, "simulation launch");
    }
    ps = job_reduce(J, st);
    if (ps != TL_OK) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        return ps;
    }
    TLC(cudaStreamSynchronize(st));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return job_finish(J, ms, launches, ms_since(t0));
}

// One launch over several (model, configuration) items.  Items of small
// models run as lane units (32 realizations per warp, one per lane), the
// others as warp units (one realization per warp); a warp takes units from
// one global counter, so uneven step counts and uneven t_final balance out.
static tl_status run_batch(tl_batch_item* items, int n, cudaStream_t st) {
    const auto t0 = std::chrono::steady_clock::now();
    if (!items || n < 1) {
        set_last_error("empty batch");
        return TL_ERR_INVALID_ARGUMENT;
    }
    std::vector<Job> jobs((size_t)n);
    int device = -1, pop = 0;
    for (int i = 0; i < n; ++i) {
        Job& J = jobs[(size_t)i];
        J.m = items[i].model;
        J.cfg = items[i].cfg;
        J.res = items[i].result;
        J.grad = items[i].grad;
        tl_status ps = job_prepare(J);
        if (ps != TL_OK) return ps;
        if (J.plain) {
            set_last_error("the plain form cannot be batched");
            return TL_ERR_UNSUPPORTED;
        }
        if (device < 0) {
            device = J.m->d.device;
            pop = J.m->h.pop_bits;
        } else if (device != J.m->d.device || pop != J.m->h.pop_bits) {
            set_last_error("batched models must share device and population width");
            return TL_ERR_INVALID_ARGUMENT;
        }
    }
    TLC(cudaSetDevice(device));
    const int smax = max_smem_optin() - 2048;
    // unit kind per item; the warp slot is the largest need
    std::vector<int> lane(n);
    size_t wslot = 0;
    for (int i = 0; i < n; ++i) {
        const tl_model* m = jobs[(size_t)i].m;
        lane[(size_t)i] = (m->h.M <= 16 && m->h.N <= 16) ? 1 : 0;
        const size_t sbi = slot_bytes(m, jobs[(size_t)i].mode != kModeFast);
        const size_t need = lane[(size_t)i] ? 32 * sbi : sbi;
        wslot = std::max(wslot, need);
        Plan& pl = jobs[(size_t)i].pl;
        pl.variant = lane[(size_t)i] ? TL_VARIANT_THREAD : TL_VARIANT_WARP;
    }
    wslot = al16(wslot);
    const size_t spb = al16(sizeof(SimParams));
    // stage every model's tables when they fit next to 4 warps' slots
    std::vector<tl_model*> uniq;
    for (auto& J : jobs)
        if (std::find(uniq.begin(), uniq.end(), J.m) == uniq.end()) uniq.push_back(J.m);
    size_t stage = 0;
    std::vector<size_t> stage_off(uniq.size());
    for (size_t u = 0; u < uniq.size(); ++u) {
        stage_off[u] = stage;
        stage += (size_t)uniq[u]->d.stage_bytes;
    }
    bool staged = true;
    for (auto& J : jobs) staged &= !J.compat_stoich;
    if (stage + 4 * (wslot + spb) > (size_t)smax) staged = false;
    if (!staged) stage = 0;
    int warps = 8;
    while (warps > 1 && stage + (size_t)warps * (wslot + spb) > (size_t)smax) --warps;
    if (stage + (size_t)warps * (wslot + spb) > (size_t)smax) {
        set_last_error("a batched model is too large for a warp unit; run it with tl_simulate");
        return TL_ERR_UNSUPPORTED;
    }
    // scratch: every job's buffers, the item table, the staged tables, a counter
    Carver c;
    for (auto& J : jobs) job_layout(J, c);
    const size_t o_items = c.take(sizeof(BatchItem) * (size_t)n);
    const size_t o_stage = c.take(std::max<size_t>(stage, 16));
    const size_t o_wctr = c.take(16);
    tl_model* owner = jobs[0].m;
    void* base = nullptr;
    tl_status ps = scratch_get(owner, c.off, &base);
    if (ps != TL_OK) return ps;
    unsigned char* B = reinterpret_cast<unsigned char*>(base);
    for (auto& J : jobs) {
        ps = job_bind(J, B, st);
        if (ps != TL_OK) return ps;
    }
    if (staged)
        for (size_t u = 0; u < uniq.size(); ++u)
            TLC(cudaMemcpyAsync(B + o_stage + stage_off[u], uniq[u]->d.blob, (size_t)uniq[u]->d.stage_bytes,
                                cudaMemcpyDeviceToDevice, st));
    // unit table: warp-unit items first (longer realizations), then lane units
    std::vector<int> order;
    for (int i = 0; i < n; ++i)
        if (!lane[(size_t)i]) order.push_back(i);
    for (int i = 0; i < n; ++i)
        if (lane[(size_t)i]) order.push_back(i);
    std::vector<BatchItem> hb((size_t)n);
    long long units = 0;
    for (int k = 0; k < n; ++k) {
        const int i = order[(size_t)k];
        Job& J = jobs[(size_t)i];
        BatchItem& b = hb[(size_t)k];
        b.p = J.p;
        b.p.stage_bytes = 0;
        b.lane_mode = lane[(size_t)i];
        b.unit_begin = units;
        b.units = lane[(size_t)i] ? (J.total + 31) / 32 : J.total;
        units += b.units;
        b.stage_off = -1;
        if (staged) {
            const size_t u = (size_t)(std::find(uniq.begin(), uniq.end(), J.m) - uniq.begin());
            b.stage_off = (int)stage_off[u];
        }
        J.pl.block = 32 * warps;
    }
    TLC(cudaMemcpyAsync(B + o_items, hb.data(), sizeof(BatchItem) * (size_t)n, cudaMemcpyHostToDevice, st));
    TLC(cudaMemsetAsync(B + o_wctr, 0, 16, st));
    BatchParams bp{};
    bp.items = reinterpret_cast<const BatchItem*>(B + o_items);
    bp.n_items = n;
    bp.total_units = units;
    bp.stage_src = B + o_stage;
    bp.stage_bytes = (int)stage;
    bp.warp_slot_bytes = (int)wslot;
    bp.params_bytes = (int)spb;
    bp.wctr = reinterpret_cast<unsigned long long*>(B + o_wctr);
    int bmode = kModeFast;  // the build every item can run on
    for (auto& J : jobs) bmode = std::max(bmode, J.mode);
    const size_t smem = stage + (size_t)warps * (wslot + spb);
    int bps = 0;
    cudaError_t le = pop == 64 ? batch_occupancy<long long>(bmode, 32 * warps, smem, &bps)
                               : batch_occupancy<int>(bmode, 32 * warps, smem, &bps);
    if (le != cudaSuccess) return cuda_fail(le, "batch occupancy");
    const int grid = (int)std::min<long long>((long long)sm_count() * std::max(bps, 1),
                                              (units + warps - 1) / warps);
    for (auto& J : jobs) J.pl.grid = grid;
    cudaEvent_t e0, e1;
    TLC(cudaEventCreate(&e0));
    TLC(cudaEventCreate(&e1));
    le = cudaEventRecord(e0, st);
    if (le == cudaSuccess)
        le = pop == 64 ? launch_batch<long long>(bp, bmode, 32 * warps, grid, smem, st)
                       : launch_batch<int>(bp, bmode, 32 * warps, grid, smem, st);
    if (le == cudaSuccess) le = cudaEventRecord(e1, st);
    if (le != cudaSuccess) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        return cuda_fail(le, "batch launch");
    }
    for (auto& J : jobs) {
        ps = job_reduce(J, st);
        if (ps != TL_OK) {
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            return ps;
        }
    }
    TLC(cudaStreamSynchronize(st));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    tl_status worst = TL_OK;
    for (auto& J : jobs) {
        const tl_status s2 = job_finish(J, ms, 1, ms_since(t0));
        if (s2 != TL_OK && (worst == TL_OK || worst == TL_ERR_STEP_CAP)) worst = s2;
    }
    return worst;
}

}  // namespace tl

using namespace tl;

extern "C" {

const char* tl_status_str(tl_status s) {
    switch (s) {
    case TL_OK: return "ok";
    case TL_ERR_INVALID_ARGUMENT: return "invalid argument";
    case TL_ERR_INVALID_MODEL: return "invalid model";
    case TL_ERR_UNSUPPORTED: return "unsupported";
    case TL_ERR_OVERFLOW: return "population overflow";
    case TL_ERR_STEP_CAP: return "step cap reached";
    case TL_ERR_CUDA: return "CUDA error";
    case TL_ERR_WAIT_TIMEOUT: return "device wait timeout";
    case TL_ERR_NO_DEVICE: return "no CUDA device";
    case TL_ERR_OUT_OF_MEMORY: return "out of memory";
    case TL_ERR_IO: return "I/O error";
    case TL_ERR_PARSE: return "parse error";
    case TL_ERR_NUMERIC: return "numeric error";
    }
    return "unknown status";
}

const char* tl_last_error(void) { return g_last_error.c_str(); }
int32_t tl_abi_version(void) { return TL_ABI_VERSION; }

tl_status tl_set_device(int32_t device) {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDeviceCount");
    if (device < 0 || device >= n) {
        set_last_error("device index out of range");
        return TL_ERR_INVALID_ARGUMENT;
    }
    g_device = device;
    TLC(cudaSetDevice(device));
    return TL_OK;
}

tl_status tl_model_create(const tl_model_desc* d, tl_model** out) {
    if (!d || !out || !d->x0 || !d->rate || !d->col_ptr || (d->nnz > 0 && (!d->row_ind || !d->stoich)) ||
        d->n_species <= 0 || d->n_channels <= 0 || d->nnz < 0) {
        set_last_error("incomplete model description");
        return TL_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    tl_model* m = new tl_model();
    HostModel& h = m->h;
    h.N = d->n_species;
    h.M = d->n_channels;
    h.pop_bits = d->pop_bits;
    h.x0.assign(d->x0, d->x0 + h.N);
    h.rate.assign(d->rate, d->rate + h.M);
    h.col_ptr.assign(d->col_ptr, d->col_ptr + h.M + 1);
    if (h.col_ptr[(size_t)h.M] != d->nnz) {
        set_last_error("col_ptr[M] != nnz");
        delete m;
        return TL_ERR_INVALID_MODEL;
    }
    h.row_ind.assign(d->row_ind, d->row_ind + d->nnz);
    h.stoich.assign(d->stoich, d->stoich + d->nnz);
    return finish_model(m, out);
}

tl_status tl_model_from_stochkit(const char* path, int32_t pop_bits, tl_model** out) {
    if (!path || !out) {
        set_last_error("null path");
        return TL_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    tl_model* m = new tl_model();
    std::string err;
    tl_status s = parse_stochkit_file(path, m->h, m->channels, err);
    if (s != TL_OK) {
        set_last_error(err);
        delete m;
        return s;
    }
    m->h.pop_bits = pop_bits;
    return finish_model(m, out);
}

void tl_gen_params_init(tl_gen_params* g, int32_t family) {
    if (!g) return;
    memset(g, 0, sizeof *g);
    g->family = family;
    switch (family) {
    case TL_GEN_DIMER:  // dimerisation decay with S1 = 100000
        g->n_species = 3;
        g->n_channels = 4;
        g->x0_min = g->x0_max = 100000;
        g->seed = 1;
        break;
    case TL_GEN_TOY:  // 128 species, 256 channels, x0 U[0,10000], c logU[1e-3,1]
        g->n_species = 128;
        g->n_channels = 256;
        g->x0_min = 0;
        g->x0_max = 10000;
        g->rate_min = 1e-3;
        g->rate_max = 1.0;
        g->seed = 7;
        break;
    case TL_GEN_CHAIN:  // 1024 species, rate 1, x0 U[1000,2000]
        g->n_species = 1024;
        g->n_channels = 1024;
        g->x0_min = 1000;
        g->x0_max = 2000;
        g->rate_min = g->rate_max = 1.0;
        g->seed = 11;
        break;
    case TL_GEN_COLLOID:  // 250 species, 31250 channels, x0 U[1000,2000], int64
        g->n_species = 250;
        g->n_channels = 31250;
        g->x0_min = 1000;
        g->x0_max = 2000;
        g->rate_assoc = 1e-4;
        g->rate_dissoc = 0.1;
        g->pop_bits = 64;
        g->seed = 13;
        break;
    default:
        break;
    }
}

tl_status tl_model_generate(const tl_gen_params* g, tl_model** out) {
    if (!g || !out) {
        set_last_error("null argument");
        return TL_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    tl_model* m = new tl_model();
    std::string err;
    tl_status s = generate_model(*g, m->h, m->channels, err);
    if (s != TL_OK) {
        set_last_error(err);
        delete m;
        return s;
    }
    return finish_model(m, out);
}

void tl_model_destroy(tl_model* m) {
    if (!m) return;
    if (m->d.blob || m->d.x0 || m->d.rate || m->scratch) {
        int cur = 0;
        cudaGetDevice(&cur);
        cudaSetDevice(m->d.device);
        if (m->d.blob) cudaFree(m->d.blob);
        if (m->d.x0) cudaFree(m->d.x0);
        if (m->d.rate) cudaFree(m->d.rate);
        if (m->scratch) cudaFree(m->scratch);
        cudaSetDevice(cur);
    }
    delete m;
}

tl_status tl_model_get_info(const tl_model* m, tl_model_info* info) {
    if (!m || !info) return TL_ERR_INVALID_ARGUMENT;
    info->n_species = m->h.N;
    info->n_channels = m->h.M;
    info->nnz_raw = (int32_t)m->h.raw_vc.size();
    info->nnz_net = (int32_t)m->h.net_vc.size();
    info->pop_bits = m->h.pop_bits;
    info->max_order = m->h.max_order;
    return TL_OK;
}

const char* tl_model_species_name(const tl_model* m, int32_t i) {
    if (!m || i < 0 || i >= m->h.N) return nullptr;
    return m->h.names[(size_t)i].c_str();
}

int32_t tl_model_species_index(const tl_model* m, const char* name) {
    if (!m || !name) return -1;
    for (int i = 0; i < m->h.N; ++i)
        if (m->h.names[(size_t)i] == name) return i;
    return -1;
}

tl_status tl_model_get_desc(const tl_model* m, int64_t* x0, double* rate, int32_t* col_ptr, int32_t* row_ind,
                            int8_t* stoich) {
    if (!m) return TL_ERR_INVALID_ARGUMENT;
    const HostModel& h = m->h;
    if (x0) std::copy(h.x0.begin(), h.x0.end(), x0);
    if (rate) std::copy(h.rate.begin(), h.rate.end(), rate);
    if (col_ptr) std::copy(h.col_ptr.begin(), h.col_ptr.end(), col_ptr);
    if (row_ind) std::copy(h.row_ind.begin(), h.row_ind.end(), row_ind);
    if (stoich) std::copy(h.stoich.begin(), h.stoich.end(), stoich);
    return TL_OK;
}

tl_status tl_model_get_tables(const tl_model* m, int8_t* order, int32_t* s0, int32_t* s1, int32_t* rp,
                              int32_t* vc) {
    if (!m) return TL_ERR_INVALID_ARGUMENT;
    const HostModel& h = m->h;
    if (order) std::copy(h.order.begin(), h.order.end(), order);
    if (s0) std::copy(h.s0.begin(), h.s0.end(), s0);
    if (s1) std::copy(h.s1.begin(), h.s1.end(), s1);
    if (rp) std::copy(h.raw_rp.begin(), h.raw_rp.end(), rp);
    if (vc) std::copy(h.raw_vc.begin(), h.raw_vc.end(), vc);
    return TL_OK;
}

tl_status tl_model_write_stochkit(const tl_model* m, const char* path) {
    if (!m || !path) return TL_ERR_INVALID_ARGUMENT;
    std::vector<Channel> ch = m->channels;
    if (ch.empty()) {
        // models built from a descriptor: rebuild channels from the raw entries
        const HostModel& h = m->h;
        ch.resize((size_t)h.M);
        for (int j = 0; j < h.M; ++j) {
            ch[(size_t)j].rate = h.rate[(size_t)j];
            for (int q = h.col_ptr[(size_t)j]; q < h.col_ptr[(size_t)j + 1]; ++q) {
                const int v = h.stoich[(size_t)q];
                if (v < 0) ch[(size_t)j].reactants.push_back({h.row_ind[(size_t)q], -v});
                else if (v > 0) ch[(size_t)j].products.push_back({h.row_ind[(size_t)q], v});
            }
        }
    }
    std::string err;
    tl_status s = write_stochkit_file(path, m->h, ch, "generated by tau_leaping_gb300", err);
    if (s != TL_OK) set_last_error(err);
    return s;
}

void tl_run_cfg_init(tl_run_cfg* cfg) {
    if (!cfg) return;
    memset(cfg, 0, sizeof *cfg);
    cfg->t_final = 1.0;
    cfg->eps = 0.03;  // cl_parser.cpp:22
    cfg->n_realizations = 1;
    cfg->seed = 1;
    cfg->n_intervals = 1;
    cfg->variant = TL_VARIANT_AUTO;
}

tl_status tl_simulate(tl_model* m, const tl_run_cfg* cfg, tl_result* res) { return run(m, cfg, res, nullptr); }

tl_status tl_simulate_batch(tl_batch_item* items, int32_t n_items, void* stream) {
    return run_batch(items, n_items, (cudaStream_t)stream);
}

tl_status tl_sensitivity(tl_model* m, const tl_run_cfg* cfg, tl_result* res, tl_grad_result* grad) {
    if (!grad) {
        set_last_error("grad result is NULL");
        return TL_ERR_INVALID_ARGUMENT;
    }
    return run(m, cfg, res, grad);
}

tl_status tl_eval_leap(tl_model* m, const int64_t* x, int32_t n, double eps, uint32_t flags, int32_t nc, float* a,
                       uint8_t* crit, float* mu, float* sigma2, float* tau1, double* a0) {
    if (!m || !x || n <= 0) {
        set_last_error("bad arguments to tl_eval_leap");
        return TL_ERR_INVALID_ARGUMENT;
    }
    const HostModel& h = m->h;
    const int N = h.N, M = h.M;
    {
        tl_status ds = ensure_device(m);
        if (ds != TL_OK) return ds;
    }
    TLC(cudaSetDevice(m->d.device));
    const size_t smem = slot_bytes(m);
    if (smem > (size_t)max_smem_optin()) {
        set_last_error("model too large for tl_eval_leap");
        return TL_ERR_UNSUPPORTED;
    }
    Carver c;
    const size_t ox = c.take((size_t)n * N * 8), oa = c.take((size_t)n * M * 4), oc = c.take((size_t)n * M),
                 om = c.take((size_t)n * N * 4), os = c.take((size_t)n * N * 4), ot = c.take((size_t)n * 4),
                 o0 = c.take((size_t)n * 8);
    void* base = nullptr;
    tl_status s = scratch_get(m, c.off, &base);
    if (s != TL_OK) return s;
    unsigned char* B = reinterpret_cast<unsigned char*>(base);
    TLC(cudaMemcpy(B + ox, x, (size_t)n * N * 8, cudaMemcpyHostToDevice));
    SimParams p{};
    p.N = N;
    p.M = M;
    p.g = global_view(m, (flags & TL_FLAG_COMPAT_STOICH) != 0, false);
    p.rates = m->d.rate;
    p.eps = (float)eps;
    p.nc = nc > 0 ? nc : 5;
    p.flags = flags;
    cudaError_t e = h.pop_bits == 64
                        ? launch_eval<long long>(p, reinterpret_cast<long long*>(B + ox), n,
                                                 reinterpret_cast<float*>(B + oa), B + oc, reinterpret_cast<float*>(B + om),
                                                 reinterpret_cast<float*>(B + os), reinterpret_cast<float*>(B + ot),
                                                 reinterpret_cast<double*>(B + o0), smem, 0)
                        : launch_eval<int>(p, reinterpret_cast<long long*>(B + ox), n, reinterpret_cast<float*>(B + oa),
                                           B + oc, reinterpret_cast<float*>(B + om), reinterpret_cast<float*>(B + os),
                                           reinterpret_cast<float*>(B + ot), reinterpret_cast<double*>(B + o0), smem, 0);
    if (e != cudaSuccess) return cuda_fail(e, "eval launch");
    TLC(cudaDeviceSynchronize());
    if (a) TLC(cudaMemcpy(a, B + oa, (size_t)n * M * 4, cudaMemcpyDeviceToHost));
    if (crit) TLC(cudaMemcpy(crit, B + oc, (size_t)n * M, cudaMemcpyDeviceToHost));
    if (mu) TLC(cudaMemcpy(mu, B + om, (size_t)n * N * 4, cudaMemcpyDeviceToHost));
    if (sigma2) TLC(cudaMemcpy(sigma2, B + os, (size_t)n * N * 4, cudaMemcpyDeviceToHost));
    if (tau1) TLC(cudaMemcpy(tau1, B + ot, (size_t)n * 4, cudaMemcpyDeviceToHost));
    if (a0) TLC(cudaMemcpy(a0, B + o0, (size_t)n * 8, cudaMemcpyDeviceToHost));
    return TL_OK;
}

tl_status tl_replay(tl_model* m, const int64_t* x0, const int32_t* k, int32_t n_leaps, int32_t raw, int64_t* x_out) {
    if (!m || !x0 || !k || n_leaps <= 0 || !x_out) {
        set_last_error("bad arguments to tl_replay");
        return TL_ERR_INVALID_ARGUMENT;
    }
    const HostModel& h = m->h;
    const int N = h.N, M = h.M;
    for (int i = 0; i < N; ++i)
        if (h.pop_bits == 32 && (x0[i] > 2147483647LL || x0[i] < -2147483647LL)) {
            set_last_error("x0 exceeds int32 for a 32-bit model");
            return TL_ERR_OVERFLOW;
        }
    {
        tl_status ds = ensure_device(m);
        if (ds != TL_OK) return ds;
    }
    TLC(cudaSetDevice(m->d.device));
    const size_t w = h.pop_bits == 64 ? 8 : 4;
    const size_t smem = al16((size_t)N * w) * 2 + 16;
    if (smem > (size_t)max_smem_optin()) {
        set_last_error("model too large for tl_replay");
        return TL_ERR_UNSUPPORTED;
    }
    Carver c;
    const size_t ox = c.take((size_t)N * 8), ok = c.take((size_t)n_leaps * M * 4),
                 oo = c.take((size_t)n_leaps * N * 8), ost = c.take(16);
    void* base = nullptr;
    tl_status s = scratch_get(m, c.off, &base);
    if (s != TL_OK) return s;
    unsigned char* B = reinterpret_cast<unsigned char*>(base);
    TLC(cudaMemcpy(B + ox, x0, (size_t)N * 8, cudaMemcpyHostToDevice));
    TLC(cudaMemcpy(B + ok, k, (size_t)n_leaps * M * 4, cudaMemcpyHostToDevice));
    TLC(cudaMemset(B + ost, 0, 16));
    SimParams p{};
    p.N = N;
    p.M = M;
    p.g = global_view(m, false, raw != 0);
    cudaError_t e = w == 8 ? launch_replay<long long>(p, reinterpret_cast<long long*>(B + ox),
                                                      reinterpret_cast<int*>(B + ok), n_leaps,
                                                      reinterpret_cast<long long*>(B + oo), reinterpret_cast<int*>(B + ost),
                                                      smem, 0)
                           : launch_replay<int>(p, reinterpret_cast<long long*>(B + ox), reinterpret_cast<int*>(B + ok),
                                                n_leaps, reinterpret_cast<long long*>(B + oo),
                                                reinterpret_cast<int*>(B + ost), smem, 0);
    if (e != cudaSuccess) return cuda_fail(e, "replay launch");
    TLC(cudaDeviceSynchronize());
    int stt = 0;
    TLC(cudaMemcpy(&stt, B + ost, 4, cudaMemcpyDeviceToHost));
    TLC(cudaMemcpy(x_out, B + oo, (size_t)n_leaps * N * 8, cudaMemcpyDeviceToHost));
    if (stt) {
        set_last_error("replay left the int32 range");
        return TL_ERR_OVERFLOW;
    }
    return TL_OK;
}

tl_status tl_philox(const uint32_t* ctr, const uint32_t* key, int32_t n, uint32_t* out) {
    if (!ctr || !key || !out || n <= 0) return TL_ERR_INVALID_ARGUMENT;
    TLC(cudaSetDevice(g_device));
    void *dc = nullptr, *dk = nullptr, *dout = nullptr;
    TLC(cudaMalloc(&dc, (size_t)n * 16));
    TLC(cudaMalloc(&dk, (size_t)n * 8));
    TLC(cudaMalloc(&dout, (size_t)n * 16));
    cudaMemcpy(dc, ctr, (size_t)n * 16, cudaMemcpyHostToDevice);
    cudaMemcpy(dk, key, (size_t)n * 8, cudaMemcpyHostToDevice);
    cudaError_t e = launch_philox(dc, dk, n, dout, 0);
    if (e == cudaSuccess) e = cudaMemcpy(out, dout, (size_t)n * 16, cudaMemcpyDeviceToHost);
    cudaFree(dc);
    cudaFree(dk);
    cudaFree(dout);
    if (e != cudaSuccess) return cuda_fail(e, "philox");
    return TL_OK;
}

tl_status tl_poisson(const float* mean, int32_t n, uint64_t seed, uint32_t step, int32_t compat, int32_t* out) {
    if (!mean || !out || n <= 0) return TL_ERR_INVALID_ARGUMENT;
    for (int i = 0; i < n; ++i)
        if (!(mean[i] >= 0.f) || mean[i] > 1e9f) {
            set_last_error("Poisson means must be in [0, 1e9]");
            return TL_ERR_INVALID_ARGUMENT;
        }
    TLC(cudaSetDevice(g_device));
    float* dm = nullptr;
    int* dout = nullptr;
    TLC(cudaMalloc(&dm, (size_t)n * 4));
    TLC(cudaMalloc(&dout, (size_t)n * 4));
    cudaMemcpy(dm, mean, (size_t)n * 4, cudaMemcpyHostToDevice);
    cudaError_t e = launch_poisson(dm, n, (unsigned)(seed & 0xFFFFFFFFu), (unsigned)(seed >> 32), step, compat, dout, 0);
    if (e == cudaSuccess) e = cudaMemcpy(out, dout, (size_t)n * 4, cudaMemcpyDeviceToHost);
    cudaFree(dm);
    cudaFree(dout);
    if (e != cudaSuccess) return cuda_fail(e, "poisson");
    return TL_OK;
}

tl_status tl_merge_moments(int32_t n_parts, int32_t L, const int64_t* counts, const double* means,
                           const double* stddevs, int64_t* count_out, double* mean_out, double* stddev_out) {
    if (n_parts < 1 || L < 1 || !counts || !means || !stddevs || !count_out || !mean_out || !stddev_out) {
        set_last_error("bad arguments to tl_merge_moments");
        return TL_ERR_INVALID_ARGUMENT;
    }
    for (int l = 0; l < L; ++l) {
        double n = 0.0, mean = 0.0, m2 = 0.0;
        for (int p = 0; p < n_parts; ++p) {
            const double nb = (double)counts[p];
            if (nb <= 0) continue;
            const double mb = means[(size_t)p * L + l];
            const double sb = stddevs[(size_t)p * L + l];
            const double m2b = nb > 1 ? sb * sb * (nb - 1.0) : 0.0;
            const double nn = n + nb;
            const double d = mb - mean;
            mean += d * nb / nn;
            m2 += m2b + d * d * n * nb / nn;
            n = nn;
        }
        mean_out[l] = mean;
        stddev_out[l] = n > 1 ? sqrt(m2 / (n - 1.0)) : 0.0;
    }
    int64_t tot = 0;
    for (int p = 0; p < n_parts; ++p) tot += counts[p] > 0 ? counts[p] : 0;
    *count_out = tot;
    return TL_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// tl_simulate_static: tl_simulate's run with its device scratch in one
// file-scope array instead of cudaMalloc'ed memory (see include/tl.h for
// who needs this and the limits).
// ---------------------------------------------------------------------------
namespace tl {

// Held by every GPU that loads the library, until the process exits.
static __device__ __align__(256) unsigned char g_static_scratch[TL_STATIC_SCRATCH_BYTES];

// Device address of g_static_scratch per device ordinal.  In host code the
// array's name is only a host-side stand-in, never a device address: the
// address is looked up once per device, with that device current, and kept
// for the life of the process (so the library must not be used across a
// cudaDeviceReset, which would unmap it).
static std::mutex g_static_mu;
static void* g_static_addr[256];

static tl_status static_scratch_address(int device, void** out) {
    if (device < 0 || device >= 256) {
        set_last_error("device ordinal out of range for the static scratch table");
        return TL_ERR_INVALID_ARGUMENT;
    }
    std::lock_guard<std::mutex> lock(g_static_mu);
    if (!g_static_addr[device]) {
        void* ptr = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&ptr, g_static_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(static scratch)");
        g_static_addr[device] = ptr;
    }
    *out = g_static_addr[device];
    return TL_OK;
}

}  // namespace tl

extern "C" tl_status tl_simulate_static(tl_model* m, const tl_run_cfg* cfg, tl_result* res) {
    const auto t0 = std::chrono::steady_clock::now();
    if (!m || !cfg) {
        set_last_error("null model or config");
        return TL_ERR_INVALID_ARGUMENT;
    }
    if (!m->d.blob) {
        set_last_error("the model's tables are not on the device yet; tl_simulate_static never allocates, so run "
                       "tl_simulate (or tl_eval_leap / tl_replay) on this model once first");
        return TL_ERR_INVALID_ARGUMENT;
    }
    if (cfg->variant == TL_VARIANT_PLAIN) {
        set_last_error("tl_simulate_static runs the fused variants only");
        return TL_ERR_UNSUPPORTED;
    }
    Job J;
    J.m = m;
    J.cfg = cfg;
    J.res = res;
    tl_status ps = job_prepare(J);  // the tables are resident: no upload happens
    if (ps != TL_OK) return ps;
    TLC(cudaSetDevice(m->d.device));
    cudaStream_t st = (cudaStream_t)cfg->stream;
    ps = make_plan(m, cfg->variant, cfg->block_threads, J.mode, J.compat_stoich,
                   (cfg->flags & TL_FLAG_NO_STAGE) != 0, J.total, J.pl, (cfg->flags & TL_FLAG_GLOBAL_SLOTS) != 0);
    if (ps != TL_OK) return ps;
    Carver c;
    job_layout(J, c);
    if (c.off > (size_t)TL_STATIC_SCRATCH_BYTES) {
        set_last_error("this run needs " + std::to_string(c.off) + " bytes of device scratch; tl_simulate_static has " +
                       std::to_string((size_t)TL_STATIC_SCRATCH_BYTES) +
                       " (fewer realizations, tracked species or grid points, or use tl_simulate)");
        return TL_ERR_INVALID_ARGUMENT;
    }
    void* base = nullptr;
    ps = static_scratch_address(m->d.device, &base);
    if (ps != TL_OK) return ps;
    ps = job_bind(J, reinterpret_cast<unsigned char*>(base), st);  // clears the counters
    if (ps != TL_OK) return ps;
    const auto tk = std::chrono::steady_clock::now();
    cudaError_t le = J.w == 8 ? launch_fused<long long>(J.p, launch_kind(J.pl), J.mode, J.pl.block, J.pl.grid, J.pl.smem, st)
                              : launch_fused<int>(J.p, launch_kind(J.pl), J.mode, J.pl.block, J.pl.grid, J.pl.smem, st);
    if (le != cudaSuccess) return cuda_fail(le, "simulation launch");
    ps = job_reduce(J, st);
    if (ps != TL_OK) return ps;
    TLC(cudaStreamSynchronize(st));
    return job_finish(J, ms_since(tk), 1, ms_since(t0));
}
