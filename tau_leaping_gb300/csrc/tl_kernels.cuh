// tl_kernels.cuh - kernels of the engine (instantiated per population type
// in tl_kernels_i32.cu / tl_kernels_i64.cu).
//
//  k_fused   persistent, work-stealing: each group (thread / warp / CTA)
//            takes realizations from a global counter and runs do_step()
//            until t_final.  The model constants are staged once per CTA
//            into shared memory with a TMA bulk copy.
//  k_plain_* the unfused baseline: FP32 time, one realization per thread,
//            state in global memory, one launch per step.
//  k_stats   deterministic two-pass mean / sample-stddev per grid column.
//  k_grad    likelihood-ratio covariance per (set, species, channel).
//  k_eval / k_replay / k_philox / k_poisson  parity entry points.
#pragma once

#include "tl_device.cuh"
#include "tl_launch.h"

namespace tl {

// ---------------------------------------------------------------------------
// TMA bulk copy (cp.async.bulk) + mbarrier helpers.
// ---------------------------------------------------------------------------
TL_D uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

TL_D void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
TL_D void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
TL_D void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
TL_D void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
        "l"(src), "r"(bytes), "r"(bar)
        : "memory");
}
TL_D bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// Stage `bytes` of the constant blob into dst with a bounded wait of
// `polls` mbarrier polls.  Returns false (CTA-uniform) if the copy did not
// complete within them; the copies still in flight into this CTA's shared
// memory are then drained (again bounded) before the caller lets the CTA
// exit.
TL_D bool stage_blob(unsigned char* dst, const unsigned char* src, int bytes, int polls, unsigned long long* bar) {
    const uint32_t ba = smem_u32(bar), da = smem_u32(dst);
    if (threadIdx.x == 0) {
        mbar_init(ba, 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        mbar_expect_tx(ba, (uint32_t)bytes);
        constexpr int kChunk = 32768;
        for (int off = 0; off < bytes; off += kChunk) {
            const int n = bytes - off < kChunk ? bytes - off : kChunk;
            bulk_g2s(da + off, src + off, (uint32_t)n, ba);
        }
    }
    bool ok = false;
    for (int it = 0; it < polls; ++it) {
        if (mbar_try_wait(ba, 0)) {
            ok = true;
            break;
        }
    }
    if (!ok) {
        // gave up: drain the copies before anything else reuses or releases
        // this shared memory
        for (int it = 0; it < (1 << 22); ++it)
            if (mbar_try_wait(ba, 0)) break;
    }
    return __syncthreads_and(ok ? 1 : 0) != 0;
}

TL_D MView staged_view(const unsigned char* s, const SimParams& p) {
    MView v;
    v.chan = reinterpret_cast<const int2*>(s + p.off_chan);
    v.rord = reinterpret_cast<const signed char*>(s + p.off_rord);
    v.gkind = reinterpret_cast<const signed char*>(s + p.off_gkind);
    v.perm = reinterpret_cast<const int*>(s + p.off_perm);
    v.rp = reinterpret_cast<const int*>(s + p.off_rp);
    v.vc = reinterpret_cast<const int*>(s + p.off_vc);
    v.urp = v.rp;
    v.uvc = v.vc;
    v.cp = reinterpret_cast<const int*>(s + p.off_cp);
    v.rv = reinterpret_cast<const int*>(s + p.off_rv);
    return v;
}

template <class Pop>
TL_D Slot<Pop> carve_slot(unsigned char* base, const SimParams& p) {
    Slot<Pop> s;
    const size_t xb = ((size_t)p.N * sizeof(Pop) + 15) & ~(size_t)15;
    s.x = reinterpret_cast<Pop*>(base);
    s.xn = reinterpret_cast<Pop*>(base + xb);
    s.a = reinterpret_cast<float*>(base + 2 * xb);
    // scored runs keep the counts apart (their slots hold M more ints)
    s.k = p.scores ? reinterpret_cast<int*>(base + 2 * xb + (((size_t)p.M * 4 + 15) & ~(size_t)15))
                   : reinterpret_cast<int*>(s.a);
    return s;
}

// KIND: 1 = thread, 32 = warp, 0 = CTA, 2/4/8/16 = that many lanes of a warp.
template <int KIND>
struct GroupOf {
    using type = GSub<KIND>;
    static TL_D GSub<KIND> make(double*) { return GSub<KIND>::make(); }
    static TL_D int index() { return threadIdx.x / KIND; }
};
template <>
struct GroupOf<1> {
    using type = G1;
    static TL_D G1 make(double*) { return G1{}; }
    static TL_D int index() { return threadIdx.x; }
};
template <>
struct GroupOf<32> {
    using type = GWarp;
    static TL_D GWarp make(double*) { return GWarp{(int)(threadIdx.x & 31)}; }
    static TL_D int index() { return threadIdx.x >> 5; }
};
template <>
struct GroupOf<0> {
    using type = GCta;
    static TL_D GCta make(double* red) {
        GCta g;
        g.tid = threadIdx.x;
        g.n = blockDim.x;
        g.lane = threadIdx.x & 31;
        g.warp = threadIdx.x >> 5;
        g.nwarps = blockDim.x >> 5;
        g.red = red;
        return g;
    }
    static TL_D int index() { return 0; }
};

// One realization from x0 to t_final (the body of the persistent loop).
// The realization's step counts go straight to the run's counters (one
// atomic each per realization), so no totals stay live across the loop.
template <class Grp, class Pop, bool SENS, bool COMPAT = true>
TL_D void run_realization(const Grp& g, const SimParams& p, const MView& mv, Slot<Pop>& s, long long w) {
    const int P = p.n_int + 1;
    const int set = (int)(w / p.R);
    const uint32_t r = (uint32_t)(p.r_off + w - (long long)set * p.R);
    Pop* samp = reinterpret_cast<Pop*>(p.samples) + (size_t)w * P * p.K;
    float* score = (SENS && p.scores) ? p.scores + (size_t)w * p.M : nullptr;
    const Pop* x0 = reinterpret_cast<const Pop*>(p.x0);
    for (int i = g.rank(); i < p.N; i += g.size()) s.x[i] = x0[i];
    if (SENS && score)
        for (int j = g.rank(); j < p.M; j += g.size()) score[j] = 0.f;
    g.sync();
    RState<double> st{0.0, 1, 0u, 0, 0, 0u};
    record_point<Grp, Pop>(g, p, s.x, samp, 0);
    bool trunc = false;
    while (!st.done) {
        do_step<Grp, Pop, double, SENS, COMPAT>(g, p, mv, s, set, r, samp, score, st);
        if (!st.done && p.max_steps > 0 && st.nsteps >= p.max_steps) {
            while (st.kpt <= p.n_int) record_point<Grp, Pop>(g, p, s.x, samp, st.kpt++);
            st.done = 1;
            trunc = true;
        }
    }
    if (g.leader()) {
        const long long leaps = st.nsteps - (long long)st.ssa, rej = (long long)st.step - st.nsteps;
        if (leaps) atomicAdd(p.ctr + 1, (unsigned long long)leaps);
        if (st.ssa) atomicAdd(p.ctr + 2, (unsigned long long)st.ssa);
        if (rej) atomicAdd(p.ctr + 3, (unsigned long long)rej);
        if (trunc) atomicAdd(p.ctr + 4, 1ull);
    }
    g.sync();
}

// ---------------------------------------------------------------------------
// Fused persistent kernel.
// ---------------------------------------------------------------------------
// Thread, sub-warp and warp groups launch at most 256 threads per CTA and
// ask the compiler for a number of resident CTAs per SM, which sets the
// register budget 65536 / (256 * n) per thread: TL_THREAD_MINB for thread
// groups, TL_WARP_MINB for the others.  CTA groups use up to 1024 threads.
// Defaults from sweeps on GB300: warp groups run best at 5 CTAs (51
// registers; 4 and 6 were 9 % slower on the toy network), thread groups
// at 3 (85 registers; 8 % faster than 4 on the dimer).
#ifndef TL_WARP_MINB
#define TL_WARP_MINB 5
#endif
#ifndef TL_THREAD_MINB
#define TL_THREAD_MINB 3
#endif
// The batch kernel (thread and warp units, scores on) at 2 CTAs per SM
// (128 registers): 1 gives 160 registers and one CTA per SM (-37 %), 4 and
// 5 spill (-24 %, -22 %).
#ifndef TL_BATCH_MINB
#define TL_BATCH_MINB 2
#endif
// MODE: kModeFast has neither likelihood-ratio scores nor the
// reference-compatibility switches; kModeScores has the scores;
// kModeGeneral has both.  Smaller builds spill fewer registers: the fast
// one is ~6 % faster than the general one, and the scores-only batch 15 %.
// GSLOT (CTA groups only): each CTA's slot lives in global memory, for
// realizations whose state exceeds shared memory.  A separate build, so
// that the shared-memory kernels keep shared-memory addressing.
template <int KIND, class Pop, int MODE, bool GSLOT = false>
__global__ void __launch_bounds__(KIND == 0 ? 1024 : 256, KIND == 0 ? 1 : KIND == 1 ? TL_THREAD_MINB : TL_WARP_MINB)
    k_fused(const __grid_constant__ SimParams p) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ __align__(8) unsigned long long mbar;
    __shared__ double red[34];
    using Grp = typename GroupOf<KIND>::type;

    MView mv = p.g;
    unsigned char* slots = smem;
    if (p.stage_bytes > 0) {
        if (!stage_blob(smem, p.blob, p.stage_bytes, p.wait_polls, &mbar)) {
            if (threadIdx.x == 0) atomicOr((unsigned*)(p.ctr + 5), kErrWaitTimeout | kErrStage);
            return;
        }
        mv = staged_view(smem, p);
        slots = smem + p.stage_bytes;
    }
    const Grp g = GroupOf<KIND>::make(red);
    if constexpr (GSLOT) slots = p.gslots + (size_t)blockIdx.x * (size_t)p.slot_bytes;
    Slot<Pop> s = carve_slot<Pop>(slots + (size_t)GroupOf<KIND>::index() * p.slot_bytes, p);
    const long long total = p.R * (long long)p.S;

    for (;;) {
        long long w = 0;
        if (g.leader()) w = (long long)atomicAdd(p.ctr + 0, 1ull);
        w = g.bcast(w, 0);
        if (w >= total) break;
        run_realization<Grp, Pop, (MODE >= kModeScores), (MODE == kModeGeneral)>(g, p, mv, s, w);
    }
}

// ---------------------------------------------------------------------------
// Batched persistent kernel: items of several models / configurations.
// ---------------------------------------------------------------------------
template <class Pop, int MODE>
__global__ void __launch_bounds__(256, TL_BATCH_MINB) k_batch(BatchParams bp) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ __align__(8) unsigned long long mbar;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (bp.stage_bytes > 0) {
        if (!stage_blob(smem, bp.stage_src, bp.stage_bytes, bp.items[0].p.wait_polls, &mbar)) {
            if (threadIdx.x == 0) atomicOr((unsigned*)(bp.items[0].p.ctr + 5), kErrWaitTimeout | kErrStage);
            return;
        }
    }
    unsigned char* wslot = smem + bp.stage_bytes + (size_t)warp * bp.warp_slot_bytes;
    SimParams* sp = reinterpret_cast<SimParams*>(smem + bp.stage_bytes + (size_t)nw * bp.warp_slot_bytes +
                                                 (size_t)warp * bp.params_bytes);
    int cur = -1;
    for (;;) {
        long long u = 0;
        if (lane == 0) u = (long long)atomicAdd(bp.wctr, 1ull);
        u = __shfl_sync(0xffffffffu, u, 0);
        if (u >= bp.total_units) break;
        int it = 0;
        while (it + 1 < bp.n_items && u >= bp.items[it + 1].unit_begin) ++it;
        if (it != cur) {
            __syncwarp();
            const int* src = reinterpret_cast<const int*>(&bp.items[it].p);
            int* dst = reinterpret_cast<int*>(sp);
            for (int k = lane; k < (int)(sizeof(SimParams) / 4); k += 32) dst[k] = src[k];
            __syncwarp();
            cur = it;
        }
        const SimParams& p = *sp;
        const int soff = bp.items[it].stage_off;
        const MView mv = soff >= 0 ? staged_view(smem + soff, p) : p.g;
        const long long local = u - bp.items[it].unit_begin;
        if (!bp.items[it].lane_mode) {
            const GWarp g{lane};
            Slot<Pop> s = carve_slot<Pop>(wslot, p);
            run_realization<GWarp, Pop, (MODE >= kModeScores), (MODE == kModeGeneral)>(g, p, mv, s, local);
        } else {
            const long long wi = local * 32 + lane;
            if (wi < p.R * (long long)p.S) {
                const G1 g{};
                Slot<Pop> s = carve_slot<Pop>(wslot + (size_t)lane * p.slot_bytes, p);
                run_realization<G1, Pop, (MODE >= kModeScores), (MODE == kModeGeneral)>(g, p, mv, s, wi);
            }
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// Plain form: one thread per realization, one launch per step, FP32 time.
// ---------------------------------------------------------------------------
// Bytes of one plain-form realization's two state buffers in HBM.
template <class Pop>
TL_HD size_t plain_slot_bytes(const SimParams& p) {
    return 2 * (((size_t)p.N * sizeof(Pop) + 15) & ~(size_t)15);
}

struct PlainState {
    float t;
    int kpt;
    uint32_t step;
    int done;
    int par;  // which half of the x buffer holds the current state
    int pad;
    long long nsteps, leaps, ssa, rej, trunc;
};

template <class Pop>
__global__ void k_plain_init(const __grid_constant__ SimParams p) {
    const long long total = p.R * (long long)p.S;
    const long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= total) return;
    PlainState* ps = reinterpret_cast<PlainState*>(p.pstate) + w;
    Pop* xs = carve_slot<Pop>(reinterpret_cast<unsigned char*>(p.pslots) + (size_t)w * plain_slot_bytes<Pop>(p), p).x;
    const Pop* x0 = reinterpret_cast<const Pop*>(p.x0);
    for (int i = 0; i < p.N; ++i) xs[i] = x0[i];
    PlainState z{};
    z.kpt = 1;
    *ps = z;
    const int P = p.n_int + 1;
    Pop* samp = reinterpret_cast<Pop*>(p.samples) + (size_t)w * P * p.K;
    record_point<G1, Pop>(G1{}, p, xs, samp, 0);
}

template <class Pop>
__global__ void k_plain_step(const __grid_constant__ SimParams p, float* a_all) {
    const long long total = p.R * (long long)p.S;
    const long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= total) return;
    PlainState* ps = reinterpret_cast<PlainState*>(p.pstate) + w;
    PlainState q = *ps;
    if (q.done) return;
    // both state buffers in HBM; q.par says which holds the current state
    Slot<Pop> s = carve_slot<Pop>(reinterpret_cast<unsigned char*>(p.pslots) + (size_t)w * plain_slot_bytes<Pop>(p), p);
    if (q.par) {
        Pop* t = s.x;
        s.x = s.xn;
        s.xn = t;
    }
    s.a = a_all + (size_t)w * p.M;
    s.k = reinterpret_cast<int*>(s.a);
    Pop* const x_before = s.x;
    const int set = (int)(w / p.R);
    const uint32_t r = (uint32_t)(p.r_off + w - (long long)set * p.R);
    const int P = p.n_int + 1;
    Pop* samp = reinterpret_cast<Pop*>(p.samples) + (size_t)w * P * p.K;
    RState<float> st{q.t, q.kpt, q.step, 0, q.nsteps, 0u};
    const G1 g{};
    do_step<G1, Pop, float, false>(g, p, p.g, s, set, r, samp, nullptr, st);
    if (!st.done && p.max_steps > 0 && st.nsteps >= p.max_steps) {
        while (st.kpt <= p.n_int) record_point<G1, Pop>(g, p, s.x, samp, st.kpt++);
        st.done = 1;
        q.trunc++;
    }
    // this launch's counts from the step counters (see RState)
    const long long acc = st.nsteps - q.nsteps;
    q.leaps += acc - (long long)st.ssa;
    q.ssa += st.ssa;
    q.rej += (long long)(st.step - q.step) - acc;
    q.t = st.t;
    q.kpt = st.kpt;
    q.step = st.step;
    q.nsteps = st.nsteps;
    if (s.x != x_before) q.par ^= 1;
    q.done = st.done;
    *ps = q;
    if (st.done) atomicAdd(p.ctr + 6, 1ull);
}

#ifdef TL_COMMON_KERNELS
__global__ void k_plain_tally(SimParams p) {
    const long long total = p.R * (long long)p.S;
    long long nl = 0, ns = 0, nr = 0, nt = 0;
    for (long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x; w < total;
         w += (long long)gridDim.x * blockDim.x) {
        const PlainState q = reinterpret_cast<const PlainState*>(p.pstate)[w];
        nl += q.leaps;
        ns += q.ssa;
        nr += q.rej;
        nt += q.trunc;
    }
    if (nl) atomicAdd(p.ctr + 1, (unsigned long long)nl);
    if (ns) atomicAdd(p.ctr + 2, (unsigned long long)ns);
    if (nr) atomicAdd(p.ctr + 3, (unsigned long long)nr);
    if (nt) atomicAdd(p.ctr + 4, (unsigned long long)nt);
}
#endif

// ---------------------------------------------------------------------------
// Deterministic statistics: one CTA per (set, grid point, tracked species).
// ---------------------------------------------------------------------------
template <class T>
TL_D T block_sum(T v, T* sh) {
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    __syncthreads();
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    T x = (threadIdx.x < (unsigned)nw) ? sh[threadIdx.x] : (T)0;
    if (warp == 0) {
#pragma unroll
        for (int o = 16; o; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if (lane == 0) sh[32] = x;
    }
    __syncthreads();
    return sh[32];
}

template <class Pop>
__global__ void k_stats(const Pop* samp, long long R, int P, int K, double* mean, double* sd) {
    __shared__ double sh[33];
    const int col = blockIdx.x;  // s*P*K + pk
    const int PK = P * K;
    const int s = col / PK, pk = col - s * PK;
    const Pop* base = samp + (size_t)s * R * PK + pk;
    double acc = 0.0;
    for (long long r = threadIdx.x; r < R; r += blockDim.x) acc += (double)base[(size_t)r * PK];
    const double m = block_sum(acc, sh) / (double)R;
    double ss = 0.0;
    for (long long r = threadIdx.x; r < R; r += blockDim.x) {
        const double d = (double)base[(size_t)r * PK] - m;
        ss += d * d;
    }
    const double tot = block_sum(ss, sh);
    if (threadIdx.x == 0) {
        mean[col] = m;
        sd[col] = R > 1 ? sqrt(tot / (double)(R - 1)) : 0.0;
    }
}

// Likelihood-ratio estimator: grad[s][k][j] = Cov_r(X_k(T), score_j),
// stderr from the spread of the per-realization products.
template <class Pop>
__global__ void k_grad(const Pop* samp, const float* scores, long long R, int P, int K, int M, double* grad,
                       double* se, double* meanf) {
    __shared__ double sh[33];
    const int col = blockIdx.x;  // (s*K + k)*M + j
    const int j = col % M;
    const int sk = col / M;
    const int k = sk % K, s = sk / K;
    const size_t PK = (size_t)P * K;
    const Pop* xb = samp + (size_t)s * R * PK + (size_t)(P - 1) * K + k;
    const float* sb = scores + (size_t)s * R * M + j;
    double ax = 0.0, asc = 0.0;
    for (long long r = threadIdx.x; r < R; r += blockDim.x) {
        ax += (double)xb[(size_t)r * PK];
        asc += (double)sb[(size_t)r * M];
    }
    const double mx = block_sum(ax, sh) / (double)R;
    const double ms = block_sum(asc, sh) / (double)R;
    double s1 = 0.0, s2 = 0.0;
    for (long long r = threadIdx.x; r < R; r += blockDim.x) {
        const double d = ((double)xb[(size_t)r * PK] - mx) * ((double)sb[(size_t)r * M] - ms);
        s1 += d;
        s2 += d * d;
    }
    const double t1 = block_sum(s1, sh);
    const double t2 = block_sum(s2, sh);
    if (threadIdx.x == 0) {
        const double n = (double)R;
        grad[col] = R > 1 ? t1 / (n - 1.0) : 0.0;
        const double var = R > 1 ? (t2 - t1 * t1 / n) / (n - 1.0) : 0.0;
        se[col] = sqrt(fmax(var, 0.0) / n);
        if (j == 0) meanf[sk] = mx;
    }
}

// ---------------------------------------------------------------------------
// Parity kernels.
// ---------------------------------------------------------------------------
// One warp per state: the same passes the fused warp variant runs.
template <class Pop>
__global__ void k_eval(SimParams p, const long long* xin, float* a_out, unsigned char* crit_out, float* mu_out,
                       float* s2_out, float* tau_out, double* a0_out) {
    extern __shared__ __align__(16) unsigned char smem[];
    Slot<Pop> s = carve_slot<Pop>(smem, p);
    const GWarp g{(int)(threadIdx.x & 31)};
    const int st = blockIdx.x;
    for (int i = g.lane; i < p.N; i += 32) s.x[i] = (Pop)xin[(size_t)st * p.N + i];
    g.sync();
    float pa, pac;
    pass_props<GWarp, Pop>(g, p, p.g, p.rates, s.x, s.a, pa, pac);
    g.sync();
    const double a0 = g.sumd((double)pa);
    float* mu = mu_out ? mu_out + (size_t)st * p.N : reinterpret_cast<float*>(s.xn);
    float* s2 = s2_out ? s2_out + (size_t)st * p.N : reinterpret_cast<float*>(s.xn);
    const float t1 = pass_tau<true, GWarp, Pop>(g, p, p.g, s.x, s.a, mu, s2);
    for (int j = g.lane; j < p.M; j += 32) {
        const float v = s.a[j];
        if (a_out) a_out[(size_t)st * p.M + j] = fabsf(v);
        if (crit_out) crit_out[(size_t)st * p.M + j] = is_crit(v) ? 1 : 0;
    }
    if (g.lane == 0) {
        if (tau_out) tau_out[st] = t1;
        if (a0_out) a0_out[st] = a0;
    }
}

template <class Pop>
__global__ void k_replay(SimParams p, const long long* x0, const int* k, int n_leaps, long long* x_out,
                         int* status) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ double red[34];
    const GCta g = GroupOf<0>::make(red);
    Slot<Pop> s = carve_slot<Pop>(smem, p);
    for (int i = g.rank(); i < p.N; i += g.size()) s.x[i] = (Pop)x0[i];
    g.sync();
    for (int l = 0; l < n_leaps; ++l) {
        bool ovf = false;
        pass_update<GCta, Pop>(g, p, p.g, s.x, k + (size_t)l * p.M, s.xn, ovf);
        if (ovf && g.leader()) *status = 1;
        g.sync();
        for (int i = g.rank(); i < p.N; i += g.size()) {
            x_out[(size_t)l * p.N + i] = (long long)s.xn[i];
            s.x[i] = s.xn[i];
        }
        g.sync();
    }
}

#ifdef TL_COMMON_KERNELS
__global__ void k_philox(const uint4* ctr, const uint2* key, int n, uint4* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint4 c = ctr[i];
    const uint2 k = key[i];
    const U4 r = philox10(U4{c.x, c.y, c.z, c.w}, k.x, k.y);
    out[i] = make_uint4(r.x, r.y, r.z, r.w);
}

__global__ void k_poisson(const float* mean, int n, uint32_t k0, uint32_t k1, uint32_t step, int compat, int* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t rk[20];
    round_keys(k0, k1, rk);
    ChanRng rng;
    rng.init((uint32_t)i, step, 0u, 0u, rk);
    if (compat) {
        out[i] = poisson_reference(mean[i], rng);
    } else {
        // exactly the hot path's draw for channel i of realization 0, set 0
        const U4 gw = group_words(rk, (uint32_t)i >> 2, step, 0u, 0u);
        out[i] = poisson_first(mean[i], word_of(gw, i & 3), rng);
    }
}
#endif

}  // namespace tl
