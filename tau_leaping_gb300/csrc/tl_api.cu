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
    // blob: [chan][gkind][net rp][net vc][net cp][net rv] | [raw rp][raw vc]
    size_t off = 0;
    auto sect = [&](size_t bytes) {
        const size_t o = off;
        off += al16(bytes);
        return (int)o;
    };
    d.off_chan = sect((size_t)M * 16);
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
    int4* chan = reinterpret_cast<int4*>(hb.data() + d.off_chan);
    for (int j = 0; j < M; ++j)
        chan[j] = make_int4(h.s0[(size_t)j], h.s1[(size_t)j], h.order[(size_t)j], h.ref_order[(size_t)j]);
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
    v.chan = reinterpret_cast<const int4*>(b + d.off_chan);
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

static size_t slot_bytes(const tl_model* m) {
    const size_t w = m->h.pop_bits == 64 ? 8 : 4;
    return al16((size_t)m->h.N * w) * 2 + al16((size_t)m->h.M * 4);
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
};

// Autotuner, heuristic part: the group width follows the model size.
//  * a handful of channels: one realization per thread (all lanes busy on
//    independent realizations);
//  * up to a few thousand channels: one warp per realization, per-warp state
//    and propensities in shared memory;
//  * larger: one CTA per realization (propensities of ~30k channels fill
//    most of the 227 KB of shared memory).
static tl_status make_plan(const tl_model* m, int variant, int block_req, bool sens, bool compat_stoich,
                           long long total, Plan& pl) {
    const size_t sb = slot_bytes(m);
    const int smax = max_smem_optin() - 2048;
    const int stage = compat_stoich ? 0 : m->d.stage_bytes;
    if (variant == TL_VARIANT_AUTO) {
        if (m->h.M <= 16 && m->h.N <= 16) variant = TL_VARIANT_THREAD;
        else if (sb * 4 + (size_t)stage <= (size_t)smax || sb * 4 <= (size_t)smax) variant = TL_VARIANT_WARP;
        else variant = TL_VARIANT_CTA;
    }
    pl.variant = variant;
    int groups_per_block = 1;
    if (variant == TL_VARIANT_THREAD) {
        pl.kind = 1;
        pl.block = block_req > 0 ? block_req : 128;
        groups_per_block = pl.block;
    } else if (variant == TL_VARIANT_WARP) {
        pl.kind = 32;
        pl.block = block_req > 0 ? block_req : 256;
        groups_per_block = pl.block / 32;
    } else if (variant == TL_VARIANT_CTA) {
        pl.kind = 0;
        pl.block = block_req > 0 ? block_req : 512;
        groups_per_block = 1;
    } else {
        set_last_error("unknown variant");
        return TL_ERR_INVALID_ARGUMENT;
    }
    if (pl.block % 32 || pl.block < 32 || pl.block > 1024) {
        set_last_error("block_threads must be a multiple of 32 in [32, 1024]");
        return TL_ERR_INVALID_ARGUMENT;
    }
    // shrink the block until the slots fit
    while ((size_t)groups_per_block * sb > (size_t)smax && pl.kind != 0 && pl.block > 32) {
        pl.block -= 32;
        groups_per_block = pl.kind == 1 ? pl.block : pl.block / 32;
    }
    if ((size_t)groups_per_block * sb > (size_t)smax) {
        set_last_error("model too large for the shared-memory slot of this variant");
        return TL_ERR_UNSUPPORTED;
    }
    pl.stage = ((size_t)groups_per_block * sb + (size_t)stage <= (size_t)smax) ? stage : 0;
    pl.smem = (size_t)pl.stage + (size_t)groups_per_block * sb;
    int bps = 0;
    cudaError_t e = m->h.pop_bits == 64 ? fused_occupancy<long long>(pl.kind, sens, pl.block, pl.smem, &bps)
                                        : fused_occupancy<int>(pl.kind, sens, pl.block, pl.smem, &bps);
    if (e != cudaSuccess) return cuda_fail(e, "occupancy");
    if (bps < 1) bps = 1;
    const long long need = (total + groups_per_block - 1) / groups_per_block;
    pl.grid = (int)std::min<long long>((long long)sm_count() * bps, std::max<long long>(need, 1));
    return TL_OK;
}

struct RunBuffers {
    float* rates = nullptr;
    double* tfin = nullptr;
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

static tl_status run(tl_model* m, const tl_run_cfg* cfg, tl_result* res, tl_grad_result* grad) {
    const auto t0 = std::chrono::steady_clock::now();
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
    const int S = std::max(1, cfg->n_rate_sets);
    const long long R = cfg->n_realizations;
    const int P = cfg->n_intervals + 1;
    const int K = cfg->n_tracked;
    const long long total = R * S;
    const bool sens = grad != nullptr;
    const bool keep = (cfg->flags & TL_FLAG_KEEP_SAMPLES) != 0;
    const bool plain = cfg->variant == TL_VARIANT_PLAIN;
    if (plain && sens) {
        set_last_error("the plain form has no sensitivity pass");
        return TL_ERR_UNSUPPORTED;
    }
    if (sens && K < 1) {
        set_last_error("sensitivity needs at least one tracked species");
        return TL_ERR_INVALID_ARGUMENT;
    }
    std::vector<float> hrates((size_t)S * M);
    std::vector<double> htf((size_t)S, cfg->t_final);
    for (int s = 0; s < S; ++s)
        for (int j = 0; j < M; ++j) {
            const double c = cfg->n_rate_sets > 0 ? cfg->rate_sets[(size_t)s * M + j] : h.rate[(size_t)j];
            if (!std::isfinite(c) || c < 0.0) {
                set_last_error("rate constants must be finite and >= 0");
                return TL_ERR_NUMERIC;
            }
            hrates[(size_t)s * M + j] = (float)c;
        }
    if (cfg->n_rate_sets > 0 && cfg->t_final_sets)
        for (int s = 0; s < S; ++s) {
            htf[(size_t)s] = cfg->t_final_sets[s];
            if (!(htf[(size_t)s] > 0.0) || !std::isfinite(htf[(size_t)s])) {
                set_last_error("t_final_sets must be > 0");
                return TL_ERR_INVALID_ARGUMENT;
            }
        }
    {
        tl_status ds = ensure_device(m);
        if (ds != TL_OK) return ds;
    }
    TLC(cudaSetDevice(m->d.device));
    cudaStream_t st = (cudaStream_t)cfg->stream;
    const size_t w = h.pop_bits == 64 ? 8 : 4;
    const bool compat_stoich = (cfg->flags & TL_FLAG_COMPAT_STOICH) != 0;

    Plan pl;
    if (!plain) {
        tl_status ps = make_plan(m, cfg->variant, cfg->block_threads, sens, compat_stoich, total, pl);
        if (ps != TL_OK) return ps;
    } else {
        pl.variant = TL_VARIANT_PLAIN;
        pl.kind = 1;
        pl.block = 128;
        pl.grid = (int)((total + 127) / 128);
    }

    // scratch layout
    Carver c;
    const size_t o_rates = c.take((size_t)S * M * 4);
    const size_t o_tf = c.take((size_t)S * 8);
    const size_t o_tr = c.take((size_t)std::max(K, 1) * 4);
    const size_t o_samp = c.take((size_t)total * P * std::max(K, 1) * w);
    const size_t o_sc = sens ? c.take((size_t)total * M * 4) : 0;
    const size_t o_ctr = c.take(8 * 8);
    const size_t o_mean = c.take((size_t)S * P * std::max(K, 1) * 8);
    const size_t o_sd = c.take((size_t)S * P * std::max(K, 1) * 8);
    const size_t o_grad = sens ? c.take((size_t)S * K * M * 8) : 0;
    const size_t o_gse = sens ? c.take((size_t)S * K * M * 8) : 0;
    const size_t o_gm = sens ? c.take((size_t)S * K * 8) : 0;
    const size_t o_ps = plain ? c.take((size_t)total * 64) : 0;
    const size_t o_pslot = plain ? c.take((size_t)total * 2 * N * w) : 0;
    const size_t o_aall = plain ? c.take((size_t)total * M * 4) : 0;
    void* base = nullptr;
    tl_status ss = scratch_get(m, c.off, &base);
    if (ss != TL_OK) return ss;
    unsigned char* B = reinterpret_cast<unsigned char*>(base);
    RunBuffers rb;
    rb.rates = reinterpret_cast<float*>(B + o_rates);
    rb.tfin = reinterpret_cast<double*>(B + o_tf);
    rb.tracked = reinterpret_cast<int*>(B + o_tr);
    rb.samples = B + o_samp;
    rb.scores = sens ? reinterpret_cast<float*>(B + o_sc) : nullptr;
    rb.ctr = reinterpret_cast<unsigned long long*>(B + o_ctr);
    rb.mean = reinterpret_cast<double*>(B + o_mean);
    rb.sd = reinterpret_cast<double*>(B + o_sd);
    if (sens) {
        rb.grad = reinterpret_cast<double*>(B + o_grad);
        rb.gse = reinterpret_cast<double*>(B + o_gse);
        rb.gmean = reinterpret_cast<double*>(B + o_gm);
    }
    if (plain) {
        rb.pstate = B + o_ps;
        rb.pslots = B + o_pslot;
        rb.a_all = reinterpret_cast<float*>(B + o_aall);
    }
    TLC(cudaMemcpyAsync(rb.rates, hrates.data(), hrates.size() * 4, cudaMemcpyHostToDevice, st));
    TLC(cudaMemcpyAsync(rb.tfin, htf.data(), htf.size() * 8, cudaMemcpyHostToDevice, st));
    if (K > 0) TLC(cudaMemcpyAsync(rb.tracked, cfg->tracked, (size_t)K * 4, cudaMemcpyHostToDevice, st));
    TLC(cudaMemsetAsync(rb.ctr, 0, 64, st));

    SimParams p{};
    p.N = N;
    p.M = M;
    p.g = global_view(m, compat_stoich, false);
    p.x0 = m->d.x0;
    p.rates = rb.rates;
    p.t_final = rb.tfin;
    p.R = R;
    p.r_off = cfg->realization_offset;
    p.S = S;
    p.k0 = (uint32_t)(cfg->seed & 0xFFFFFFFFu);
    p.k1 = (uint32_t)(cfg->seed >> 32);
    p.eps = (float)cfg->eps;
    p.nc = cfg->n_critical > 0 ? cfg->n_critical : 5;
    p.ssa_factor = (float)(cfg->ssa_factor > 0 ? cfg->ssa_factor : 10);
    p.ssa_block = cfg->ssa_block > 0 ? cfg->ssa_block : 100;
    p.n_int = cfg->n_intervals;
    p.K = K;
    p.tracked = rb.tracked;
    p.samples = rb.samples;
    p.scores = rb.scores;
    p.max_steps = cfg->max_steps;
    p.flags = cfg->flags;
    p.blob = m->d.blob;
    p.stage_bytes = pl.stage;
    p.off_chan = m->d.off_chan;
    p.off_gkind = m->d.off_gkind;
    p.off_perm = m->d.off_perm;
    p.off_rp = m->d.off_rp;
    p.off_vc = m->d.off_vc;
    p.off_cp = m->d.off_cp;
    p.off_rv = m->d.off_rv;
    p.slot_bytes = (int)slot_bytes(m);
    p.ctr = rb.ctr;
    p.pstate = rb.pstate;
    p.pslots = rb.pslots;

    cudaEvent_t e0, e1;
    TLC(cudaEventCreate(&e0));
    TLC(cudaEventCreate(&e1));
    int launches = 0;
    cudaError_t le = cudaEventRecord(e0, st);
    if (le == cudaSuccess) {
        if (!plain) {
            le = w == 8 ? launch_fused<long long>(p, pl.kind, sens, pl.block, pl.grid, pl.smem, st)
                        : launch_fused<int>(p, pl.kind, sens, pl.block, pl.grid, pl.smem, st);
            launches = 1;
        } else {
            le = w == 8 ? launch_plain_init<long long>(p, st) : launch_plain_init<int>(p, st);
            launches = 1;
            unsigned long long* hdone = nullptr;
            cudaMallocHost(&hdone, 8);
            while (le == cudaSuccess) {
                for (int q = 0; q < 16 && le == cudaSuccess; ++q) {
                    le = w == 8 ? launch_plain_step<long long>(p, rb.a_all, st) : launch_plain_step<int>(p, rb.a_all, st);
                    ++launches;
                }
                if (le != cudaSuccess) break;
                le = cudaMemcpyAsync(hdone, rb.ctr + 6, 8, cudaMemcpyDeviceToHost, st);
                if (le == cudaSuccess) le = cudaStreamSynchronize(st);
                if (le == cudaSuccess && *hdone >= (unsigned long long)total) break;
                if (launches > (1 << 26)) {  // a realization that never ends
                    cudaFreeHost(hdone);
                    cudaEventDestroy(e0);
                    cudaEventDestroy(e1);
                    set_last_error("plain form exceeded 2^26 launches; set max_steps");
                    return TL_ERR_STEP_CAP;
                }
            }
            cudaFreeHost(hdone);
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
    // statistics
    if (K > 0) {
        le = w == 8 ? launch_stats<long long>(rb.samples, R, P, K, S, rb.mean, rb.sd, st)
                    : launch_stats<int>(rb.samples, R, P, K, S, rb.mean, rb.sd, st);
        if (le != cudaSuccess) return cuda_fail(le, "statistics launch");
    }
    if (sens) {
        le = w == 8 ? launch_grad<long long>(rb.samples, rb.scores, R, P, K, M, S, rb.grad, rb.gse, rb.gmean, st)
                    : launch_grad<int>(rb.samples, rb.scores, R, P, K, M, S, rb.grad, rb.gse, rb.gmean, st);
        if (le != cudaSuccess) return cuda_fail(le, "gradient launch");
    }
    unsigned long long hc[8];
    TLC(cudaMemcpyAsync(hc, rb.ctr, 64, cudaMemcpyDeviceToHost, st));
    if (res) {
        if (res->mean && K > 0)
            TLC(cudaMemcpyAsync(res->mean, rb.mean, (size_t)S * P * K * 8, cudaMemcpyDeviceToHost, st));
        if (res->stddev && K > 0)
            TLC(cudaMemcpyAsync(res->stddev, rb.sd, (size_t)S * P * K * 8, cudaMemcpyDeviceToHost, st));
    }
    std::vector<unsigned char> hs;
    if (res && res->samples && keep && K > 0) {
        hs.resize((size_t)total * P * K * w);
        TLC(cudaMemcpyAsync(hs.data(), rb.samples, hs.size(), cudaMemcpyDeviceToHost, st));
    }
    if (sens) {
        if (grad->grad) TLC(cudaMemcpyAsync(grad->grad, rb.grad, (size_t)S * K * M * 8, cudaMemcpyDeviceToHost, st));
        if (grad->grad_stderr)
            TLC(cudaMemcpyAsync(grad->grad_stderr, rb.gse, (size_t)S * K * M * 8, cudaMemcpyDeviceToHost, st));
        if (grad->mean_final)
            TLC(cudaMemcpyAsync(grad->mean_final, rb.gmean, (size_t)S * K * 8, cudaMemcpyDeviceToHost, st));
    }
    TLC(cudaStreamSynchronize(st));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (!hs.empty()) {
        const size_t n = (size_t)total * P * K;
        if (w == 8) memcpy(res->samples, hs.data(), n * 8);
        else {
            const int* src = reinterpret_cast<const int*>(hs.data());
            for (size_t q = 0; q < n; ++q) res->samples[q] = src[q];
        }
    }
    if (res) {
        if (res->times)
            for (int s = 0; s < S; ++s)
                for (int k = 0; k < P; ++k)
                    res->times[(size_t)s * P + k] =
                        k == cfg->n_intervals ? htf[(size_t)s] : htf[(size_t)s] * (double)k / (double)cfg->n_intervals;
        res->leaps = (int64_t)hc[1];
        res->ssa_steps = (int64_t)hc[2];
        res->rejections = (int64_t)hc[3];
        res->truncated = (int64_t)hc[4];
        res->kernel_ms = ms;
        res->variant_used = pl.variant;
        res->block_threads_used = pl.block;
        res->grid_used = pl.grid;
        res->launches = launches;
        res->total_ms =
            std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
    const unsigned eb = (unsigned)hc[5];
    if (eb & kErrWaitTimeout) {
        set_last_error("shared-memory staging wait timed out");
        return TL_ERR_WAIT_TIMEOUT;
    }
    if (eb & kErrOverflow) {
        set_last_error("a population left the range of the population type");
        return TL_ERR_OVERFLOW;
    }
    if (eb & (kErrHalving | kErrNumeric)) {
        set_last_error("a leap could not be made non-negative by halving tau");
        return TL_ERR_NUMERIC;
    }
    if (hc[4] > 0) {
        set_last_error("max_steps reached; truncated realizations hold their last state");
        return TL_ERR_STEP_CAP;
    }
    return TL_OK;
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

}  // extern "C"
