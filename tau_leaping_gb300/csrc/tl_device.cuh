// tl_device.cuh - device building blocks of the tau-leaping engine.
//
// Everything a realization does in one step lives here, written once and
// instantiated for three cooperation widths (the "group" owning one
// realization): one thread (G1), one warp (GWarp) or one CTA (GCta).  The
// fused persistent kernel loops do_step() until a realization reaches
// t_final; the plain form calls it once per launch.
//
// Reference semantics followed (CSSL-UWM/tau_leaping):
//   propensity / criticality  tau_leaping/functions.h:100-123, model.cu:180-209
//   CGP tau bound             tau_leaping/CSRMatrixPacked.cu:294-358
//   leap / SSA branch         tau_leaping/model.cu:301-413
//   critical channel draw     tau_leaping/model.cu:555-598
//   Poisson firing            tau_leaping/model.cu:458-521
//   integer state update      tau_leaping/CSRMatrixPacked.cu:464-503
//   direct-method step        tau_leaping/model.cu:427-451
// with the Cao-Gillespie-Petzold (J. Chem. Phys. 124, 044109, 2006) rules the
// reference departs from switched by TL_FLAG_COMPAT_* bits.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/tl.h"

namespace tl {

#define TL_HD __host__ __device__ __forceinline__
#define TL_D __device__ __forceinline__

constexpr uint32_t kScalarChannel = 0xFFFFFFFFu;  // counter word 0 of step scalars
constexpr float kInfF = __builtin_huge_valf();

// Error bits written to the run's error word.
enum : unsigned {
    kErrOverflow = 1u << 0,
    kErrWaitTimeout = 1u << 1,
    kErrHalving = 1u << 2,    // leap still rejected after max_halv halvings
    kErrNumeric = 1u << 3,
    kErrStage = 1u << 4,
};

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
// as 1, 2, 3", SC'11).  Round: (c0,c1,c2,c3) -> (hi(B*c2)^c1^k0, lo(B*c2),
// hi(A*c0)^c3^k1, lo(A*c0)) with A=0xD2511F53, B=0xCD9E8D57; the key is
// bumped by the Weyl constants between rounds.
// ---------------------------------------------------------------------------
struct U4 {
    uint32_t x, y, z, w;
};

TL_HD uint32_t mulhi32(uint32_t a, uint32_t b) {
#ifdef __CUDA_ARCH__
    return __umulhi(a, b);
#else
    return (uint32_t)(((uint64_t)a * (uint64_t)b) >> 32);
#endif
}

TL_HD U4 philox10(U4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        const uint32_t hi0 = mulhi32(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
        const uint32_t hi1 = mulhi32(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
        c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
    }
    return c;
}

// The same Philox4x32-10 with the ten rounds' keys precomputed:
// rk[2r] = k0 + r*0x9E3779B9, rk[2r+1] = k1 + r*0xBB67AE85.  The engine's
// kernels read rk from their launch parameters (constant bank), so the key
// schedule costs no instruction; the words are those of philox10.
TL_HD U4 philox10rk(U4 c, const uint32_t* rk) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint32_t hi0 = mulhi32(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
        const uint32_t hi1 = mulhi32(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
        c = U4{hi1 ^ c.y ^ rk[2 * r], lo1, hi0 ^ c.w ^ rk[2 * r + 1], lo0};
    }
    return c;
}

TL_HD void round_keys(uint32_t k0, uint32_t k1, uint32_t* rk) {
    for (int r = 0; r < 10; ++r) {
        rk[2 * r] = k0 + (uint32_t)r * 0x9E3779B9u;
        rk[2 * r + 1] = k1 + (uint32_t)r * 0xBB67AE85u;
    }
}

// Uniform in (0,1): 23 random bits at odd multiples of 2^-24 (exact in FP32).
TL_HD float u01f(uint32_t w) { return ((float)(w >> 9) + 0.5f) * 1.1920928955078125e-07f; }
// Uniform in (0,1) with 52 random bits, exact in FP64.
TL_HD double u01d(uint32_t hi, uint32_t lo) {
    const uint64_t k = ((uint64_t)(hi >> 6) << 26) | (uint64_t)(lo >> 6);
    return ((double)k + 0.5) * 2.220446049250313e-16;
}

// Step scalars of (realization r, set s, step): 4 words.
TL_HD U4 step_words(const uint32_t* rk, uint32_t step, uint32_t r, uint32_t set) {
    return philox10rk(U4{kScalarChannel, step, r, set << 8}, rk);
}

// Per-channel uniform stream: blocks (j, step, r, set<<8 | b), b = 0, 1, ...
struct ChanRng {
    U4 buf;
    uint32_t j, step, r, c3;
    const uint32_t* rk;  // round keys (philox10rk)
    int left;
    TL_D void init(uint32_t j_, uint32_t step_, uint32_t r_, uint32_t set, const uint32_t* rk_) {
        j = j_;
        step = step_;
        r = r_;
        c3 = set << 8;
        rk = rk_;
        left = 0;
    }
    TL_D float next() {
        if (left == 0) {
            buf = philox10rk(U4{j, step, r, c3}, rk);
            c3 += 1;  // next block; 256 blocks per (j, step) before wrapping into set+1
            left = 4;
        }
        const uint32_t w = buf.x;
        buf.x = buf.y;
        buf.y = buf.z;
        buf.z = buf.w;
        --left;
        return u01f(w);
    }
};

// ---------------------------------------------------------------------------
// Poisson samplers (FP32).
// ---------------------------------------------------------------------------
__device__ __constant__ const float kLogFact[10] = {
    0.0f, 0.0f, 0.693147180559945f, 1.7917594692280554f, 3.178053830347945f,
    4.787491742782047f, 6.579251212010102f, 8.525161361065415f, 10.604602902745249f,
    12.801827480081467f};

// log P(K = k) for K ~ Poisson(mu), mu >= 10, written so that FP32 keeps its
// accuracy for large mu: with d = k - mu, r = d/mu and Stirling's series for
// log k!,  log p = -(k*(log1p(r) - r) + d*r) - 0.5*log(2*pi*k) - delta(k),
// delta(k) = 1/(12k) - 1/(360k^3) + 1/(1260k^5).
TL_D float log_poisson_pmf(float kf, float mu, float lmu) {
    if (kf < 10.f) return kf * lmu - mu - kLogFact[(int)kf];
    const float d = kf - mu;
    const float r = __fdividef(d, mu);
    float l1mr;  // log1p(r) - r
    if (fabsf(r) <= 0.01f) {
        // -r^2/2 + r^3/3 - r^4/4 + r^5/5 - r^6/6
        l1mr = r * r * (-0.5f + r * (1.f / 3.f + r * (-0.25f + r * (0.2f - r * (1.f / 6.f)))));
    } else {
        l1mr = log1pf(r) - r;
    }
    const float t = kf * l1mr + d * r;
    const float ik = __fdividef(1.f, kf), ik2 = ik * ik;
    const float delta = ik * (1.f / 12.f - ik2 * (1.f / 360.f - ik2 * (1.f / 1260.f)));
    return -t - 0.5f * logf(6.283185307179586f * kf) - delta;
}

// Hormann's PTRS transformed rejection (Insurance: Mathematics and Economics
// 12, 39-45, 1993), valid for mu >= 10.  Its divisions are __fdividef (2
// ulp; every divisor here lies far inside [2^-126, 2^126]): the acceptance
// boundaries move by ~1e-7 relative, the size of FP32 rounding, and the
// sampler runs 8-14 % faster on the chain and dimer models.
template <class Rng>
TL_D int poisson_ptrs(float mu, Rng& rng) {
    const float smu = sqrtf(mu);
    const float lmu = logf(mu);
    const float b = 0.931f + 2.53f * smu;
    const float a = -0.059f + 0.02483f * b;
    const float inv_alpha = 1.1239f + __fdividef(1.1328f, b - 3.4f);
    const float vr = 0.9277f - __fdividef(3.6224f, b - 2.f);
    for (int it = 0; it < 512; ++it) {
        const float U = rng.next() - 0.5f;
        const float V = rng.next();
        const float us = 0.5f - fabsf(U);
        const float kf = floorf((__fdividef(2.f * a, us) + b) * U + mu + 0.43f);
        if (us >= 0.07f && V <= vr) return (int)kf;
        if (kf < 0.f || (us < 0.013f && V > us)) continue;
        const float lhs = logf(__fdividef(V * inv_alpha, __fdividef(a, us * us) + b));
        if (lhs <= log_poisson_pmf(kf, mu, lmu)) return (int)kf;
    }
    return (int)(mu + 0.5f);  // unreachable in practice (acceptance > 0.89)
}

// Sequential-search inversion for mu < 10 with one uniform per attempt.  If
// the FP32 CDF stops growing before it passes u (u above the representable
// mass) the uniform is discarded and a fresh one drawn, so no tail value is
// ever produced by rounding.
template <class Rng>
TL_D int poisson_inversion(float mu, Rng& rng) {
    const float emu = expf(-mu);
    for (int attempt = 0; attempt < 16; ++attempt) {
        const float u = rng.next();
        float p = emu, F = emu;
        int k = 0;
        bool ok = true;
        while (u > F) {
            ++k;
            p = p * __fdividef(mu, (float)k);
            const float Fn = F + p;
            if (Fn == F) {
                ok = false;
                break;
            }
            F = Fn;
        }
        if (ok) return k;
    }
    return (int)mu;
}

template <class Rng>
TL_D int poisson_cgp(float mu, Rng& rng) {
    if (!(mu > 0.f)) return 0;
    if (mu < 10.f) return poisson_inversion(mu, rng);
    return poisson_ptrs(mu, rng);
}

// Shared first words: channels 4g..4g+3 of one step take their first 32-bit
// word from one Philox block (g, step, r, set<<8 | 0xFF); the private
// stream (j, step, r, set<<8 | b), b < 0xFF, supplies any further uniforms.
TL_HD U4 group_words(const uint32_t* rk, uint32_t g, uint32_t step, uint32_t r, uint32_t set) {
    return philox10rk(U4{g, step, r, (set << 8) | 0xFFu}, rk);
}

// P(K >= 1) = 1 - exp(-mu) for 0 < mu: below 0.1 the Taylor series to
// mu^6 (truncation < mu^7/5040, relative 2e-10), above it 1 - expf(-mu)
// (relative error < 1.2e-6: expf is within 2 ulp and exp(-mu) < 0.905).
TL_D float poisson_p1(float mu) {
    if (mu < 0.1f)
        return mu * (1.f - mu * (0.5f - mu * (1.f / 6.f - mu * (1.f / 24.f - mu * (1.f / 120.f - mu * (1.f / 720.f))))));
    return 1.f - expf(-mu);
}

// P(K >= 2) = 1 - exp(-mu)(1 + mu) for 0 < mu < 10: below 0.5 the series
// sum_{n>=2} (-1)^n (n-1) mu^n / n! to n = 9 (relative error < 3e-8), above
// it directly (exp(-mu)(1 + mu) < 0.91 there: relative error < 1.3e-6).
TL_D float poisson_p2(float mu) {
    if (mu < 0.5f) {
        const float c = 0.5f + mu * (-1.f / 3.f + mu * (1.f / 8.f + mu * (-1.f / 30.f + mu * (1.f / 144.f +
                        mu * (-1.f / 840.f + mu * (1.f / 5760.f - mu * (1.f / 45360.f)))))));
        return mu * mu * c;
    }
    return 1.f - expf(-mu) * (1.f + mu);
}

// Poisson(mu) for mu < 10 from one 32-bit word w by inversion with
// q = (w + 1/2) 2^-32, which is uniform on (0,1) with full relative precision
// near 0: k = 0 iff q >= P(K >= 1), k = 1 iff P(K >= 2) <= q < P(K >= 1).
// Both tests are exact for the tiny means that dominate (a 23-bit uniform
// would quantise them); k >= 2 continues the sequential inversion on
// u = 1 - q.  mu >= 10 uses PTRS on the private stream.
template <class Rng>
TL_D int poisson_tail2(float mu, float q, Rng& rng) {
    if (mu >= 10.f) return poisson_ptrs(mu, rng);
    const float u = 1.f - q;
    const float e = expf(-mu);
    float p = e * mu, F = e + p;
    for (int k = 2; k < 64; ++k) {
        p = p * __fdividef(mu, (float)k);
        const float Fn = F + p;
        if (u <= Fn) return k;
        if (Fn == F) break;  // u above the representable mass: draw afresh
        F = Fn;
    }
    return poisson_inversion(mu, rng);
}

template <class Rng>
TL_D int poisson_first(float mu, uint32_t w, Rng& rng) {
    if (!(mu > 0.f)) return 0;
    if (mu >= 10.f) return poisson_ptrs(mu, rng);
    const float q = ((float)w + 0.5f) * 2.3283064365386963e-10f;
    const float s0 = poisson_p1(mu);
    if (q >= s0) return 0;
    if (q >= poisson_p2(mu)) return 1;
    return poisson_tail2(mu, q, rng);
}

TL_D uint32_t word_of(const U4& w, int e) { return e == 0 ? w.x : e == 1 ? w.y : e == 2 ? w.z : w.w; }

// The reference's sampler (model.cu:477-520, functions.h:37-54): Knuth's
// product method below mean 80 capped at 300 firings, |Normal(mean, mean)|
// from the polar Box-Muller draw above, truncated toward zero.
template <class Rng>
TL_D int poisson_reference(float mu, Rng& rng) {
    if (mu < 80.f) {
        const float lam = 1.f / expf(mu);
        float val = 1.f;
        for (int n = 1; n < 300; ++n) {
            val *= rng.next();
            if (val < lam) return n - 1;
        }
        return 300;
    }
    float u, v, s;
    int it = 0;
    do {
        u = 2.f * rng.next() - 1.f;
        v = 2.f * rng.next() - 1.f;
        s = u * u + v * v;
    } while (s >= 1.f && ++it < 64);
    const float z = u * sqrtf(-2.f * logf(s) / s);
    return (int)fabsf(mu + sqrtf(mu) * z);
}

// The draw of one channel once its k <= 1 tests have failed (or its mean is
// >= 10, or the reference's sampler is asked for).  Warp and CTA groups run
// it from one call site after the unrolled channel loop (pass_fire), so one
// copy of it sits in the loop.
// REFS: the reference's sampler can be asked for (compatibility builds).
template <bool REFS>
TL_D int poisson_rare_inline(float mu, float q, uint32_t j, uint32_t step, uint32_t r, uint32_t set,
                             const uint32_t* rk, int refs) {
    ChanRng rng;
    rng.init(j, step, r, set, rk);
    if (REFS && refs) return poisson_reference(mu, rng);
    return poisson_tail2(mu, q, rng);
}
// Inlined there by default (TL_RARE_INLINE 1): a call would save the
// registers live across it, and those saves were most of the warp kernel's
// spills.  Measured on GB300 against the out-of-line call: toy network +3 %,
// chain +4 %, colloid +1 %, batch +2 %.
#ifndef TL_RARE_INLINE
#define TL_RARE_INLINE 1
#endif
#if TL_RARE_INLINE
#define TL_RARE_ATTR __forceinline__
#else
#define TL_RARE_ATTR __noinline__
#endif
template <bool REFS>
static __device__ TL_RARE_ATTR int poisson_rare(float mu, float q, uint32_t j, uint32_t step, uint32_t r,
                                                uint32_t set, const uint32_t* rk, int refs) {
    return poisson_rare_inline<REFS>(mu, q, j, step, r, set, rk, refs);
}

// ---------------------------------------------------------------------------
// Propensity and criticality of one channel (functions.h:100-123).
// chan = {s0, s1 | order << 28}; order 0 = no reactant (a = c).
// ---------------------------------------------------------------------------
// Population to FP32.  int64 -> float runs at the reduced FP64 rate; an
// int64 population that fits in int32 (the usual case) takes the 32-bit
// conversion, which rounds to the same float.
TL_D float popf(int x) { return (float)x; }
static __device__ __noinline__ float popf_wide(long long x) { return (float)x; }
TL_D float popf(long long x) { return (long long)(int)x == x ? (float)(int)x : popf_wide(x); }

template <class Pop>
TL_D void propensity(const int2 ch, float c, const Pop* x, int nc, bool compat_crit, float& a,
                     bool& crit) {
    // Branch-free over the order so that a warp's mixed-order channels do
    // not diverge.  For order 1/3 the table holds s1 = s0 (order 0: s0 = s1
    // = 0), so both loads are always in bounds.  The products keep the
    // reference's evaluation order: (c*x0)*x1, and (c*x0)*(x0-1)/2 with the
    // halving exact.
    const int order = (int)((unsigned)ch.y >> 28);
    const Pop x0 = x[ch.x], x1 = x[ch.y & 0x0FFFFFFF];
    // second factor picked as an integer first: two conversions per channel
    const Pop y = order == 2 ? x1 : order == 3 ? x0 - 1 : (Pop)1;
    const float f0 = order == 0 ? 1.f : popf(x0);
    const float f1 = popf(y) * (order == 3 ? 0.5f : 1.f);
    a = c * f0 * f1;
    const Pop t0 = order == 3 ? (compat_crit ? (Pop)((nc + 1) / 2) : (Pop)(2 * nc)) : (Pop)nc;
    crit = order != 0 && (x0 < t0 || (order == 2 && x1 < (Pop)nc));
}

// g_i of the CGP bound.  kind: 0 not a reactant, 1 HOR 1, 2 HOR 2 (S_i+S_k),
// 3 HOR 2 with 2S_i (g = 2 + 1/(x-1)).  The reference's GetG
// (CSRMatrixPacked.cu:294-309) maps channel orders 1,2,3 the same way.
TL_D float g_of(int kind, float x) {
    if (kind == 1) return 1.f;
    if (kind == 2) return 2.f;
    if (kind == 3) return x >= 2.f ? 2.f + 1.f / (x - 1.f) : 3.f;
    return 0.f;
}

TL_D bool is_crit(float a) { return __float_as_uint(a) >> 31; }

// ---------------------------------------------------------------------------
// Groups: the threads that own one realization.
// ---------------------------------------------------------------------------
struct G1 {
    static constexpr int kWidth = 1;
    TL_D int rank() const { return 0; }
    TL_D int size() const { return 1; }
    TL_D void sync() const {}
    TL_D bool leader() const { return true; }
    TL_D float sumf(float v) const { return v; }
    TL_D double sumd(double v) const { return v; }
    TL_D float minf(float v) const { return v; }
    TL_D bool any(bool p) const { return p; }
    TL_D double excl_scan(double) const { return 0.0; }
    TL_D int first(bool p) const { return p ? 0 : -1; }
    TL_D int last(bool p) const { return p ? 0 : -1; }
    template <class T>
    TL_D T bcast(T v, int) const {
        return v;
    }
};

struct GWarp {
    static constexpr int kWidth = 32;
    int lane;
    TL_D int rank() const { return lane; }
    TL_D int size() const { return 32; }
    TL_D void sync() const { __syncwarp(); }
    TL_D bool leader() const { return lane == 0; }
    TL_D float sumf(float v) const {
#pragma unroll
        for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        return v;
    }
    TL_D double sumd(double v) const {
#pragma unroll
        for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        return v;
    }
    TL_D float minf(float v) const {
#pragma unroll
        for (int o = 16; o; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
        return v;
    }
    TL_D bool any(bool p) const { return __any_sync(0xffffffffu, p); }
    TL_D double excl_scan(double v) const {
        double s = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const double n = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += n;
        }
        const double e = __shfl_up_sync(0xffffffffu, s, 1);
        return lane ? e : 0.0;
    }
    TL_D int first(bool p) const {
        const unsigned b = __ballot_sync(0xffffffffu, p);
        return b ? __ffs(b) - 1 : -1;
    }
    TL_D int last(bool p) const {
        const unsigned b = __ballot_sync(0xffffffffu, p);
        return b ? 31 - __clz(b) : -1;
    }
    template <class T>
    TL_D T bcast(T v, int src) const {
        return __shfl_sync(0xffffffffu, v, src);
    }
};

// W lanes of one warp (W = 2, 4, 8, 16): lanes [base, base + W).  Shuffles
// run on W-lane segments with the group's own mask, so the groups of a warp
// advance independently (different realizations take different paths).
template <int W>
struct GSub {
    static_assert(W >= 2 && W <= 16 && (W & (W - 1)) == 0, "sub-warp width");
    static constexpr int kWidth = W;
    int lane;       // rank in the group
    int base;       // first lane of the group in its warp
    unsigned mask;  // the group's lanes
    static TL_D GSub make() {
        GSub g;
        const int l = (int)(threadIdx.x & 31);
        g.lane = l & (W - 1);
        g.base = l & ~(W - 1);
        g.mask = (W == 32 ? 0xffffffffu : ((1u << W) - 1u)) << g.base;
        return g;
    }
    TL_D int rank() const { return lane; }
    TL_D int size() const { return W; }
    TL_D void sync() const { __syncwarp(mask); }
    TL_D bool leader() const { return lane == 0; }
    TL_D float sumf(float v) const {
#pragma unroll
        for (int o = W / 2; o; o >>= 1) v += __shfl_xor_sync(mask, v, o, W);
        return v;
    }
    TL_D double sumd(double v) const {
#pragma unroll
        for (int o = W / 2; o; o >>= 1) v += __shfl_xor_sync(mask, v, o, W);
        return v;
    }
    TL_D float minf(float v) const {
#pragma unroll
        for (int o = W / 2; o; o >>= 1) v = fminf(v, __shfl_xor_sync(mask, v, o, W));
        return v;
    }
    TL_D bool any(bool p) const { return (__ballot_sync(mask, p) & mask) != 0u; }
    TL_D double excl_scan(double v) const {
        double s = v;
#pragma unroll
        for (int o = 1; o < W; o <<= 1) {
            const double n = __shfl_up_sync(mask, s, o, W);
            if (lane >= o) s += n;
        }
        const double e = __shfl_up_sync(mask, s, 1, W);
        return lane ? e : 0.0;
    }
    TL_D int first(bool p) const {
        const unsigned b = (__ballot_sync(mask, p) & mask) >> base;
        return b ? __ffs(b) - 1 : -1;
    }
    TL_D int last(bool p) const {
        const unsigned b = (__ballot_sync(mask, p) & mask) >> base;
        return b ? 31 - __clz(b) : -1;
    }
    template <class T>
    TL_D T bcast(T v, int src) const {
        return __shfl_sync(mask, v, src, W);
    }
};

// Whole CTA; needs a shared scratch of 34 doubles.  Every member is a
// CTA-wide collective (call from all threads, uniform control flow).  The
// scratch holds each value in its own type (FP32 reductions stay FP32).
struct GCta {
    static constexpr int kWidth = 0;
    int tid, n, lane, warp, nwarps;
    double* red;
    TL_D int rank() const { return tid; }
    TL_D int size() const { return n; }
    TL_D void sync() const { __syncthreads(); }
    TL_D bool leader() const { return tid == 0; }
    TL_D float sumf(float v) const { return reduce_sum<float>(v); }
    template <class T>
    TL_D T reduce_sum(T v) const {
        T* rt = reinterpret_cast<T*>(red);
#pragma unroll
        for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        __syncthreads();
        if (lane == 0) rt[warp] = v;
        __syncthreads();
        if (warp == 0) {
            T x = lane < nwarps ? rt[lane] : (T)0;
#pragma unroll
            for (int o = 16; o; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
            if (lane == 0) *reinterpret_cast<T*>(red + 33) = x;
        }
        __syncthreads();
        return *reinterpret_cast<const T*>(red + 33);
    }
    TL_D double sumd(double v) const { return reduce_sum<double>(v); }
    TL_D float minf(float v) const {
        float* rf = reinterpret_cast<float*>(red);
#pragma unroll
        for (int o = 16; o; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
        __syncthreads();
        if (lane == 0) rf[warp] = v;
        __syncthreads();
        if (warp == 0) {
            float x = lane < nwarps ? rf[lane] : kInfF;
#pragma unroll
            for (int o = 16; o; o >>= 1) x = fminf(x, __shfl_xor_sync(0xffffffffu, x, o));
            if (lane == 0) rf[66] = x;
        }
        __syncthreads();
        return rf[66];
    }
    TL_D bool any(bool p) const { return __syncthreads_or(p ? 1 : 0) != 0; }
    TL_D double excl_scan(double v) const {
        double s = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const double t = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += t;
        }
        const double e_in = __shfl_up_sync(0xffffffffu, s, 1);
        __syncthreads();
        if (lane == 31) red[warp] = s;
        __syncthreads();
        if (warp == 0) {
            double y = lane < nwarps ? red[lane] : 0.0;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const double t = __shfl_up_sync(0xffffffffu, y, o);
                if (lane >= o) y += t;
            }
            const double ex = __shfl_up_sync(0xffffffffu, y, 1);
            if (lane < nwarps) red[lane] = lane ? ex : 0.0;  // exclusive warp offsets
        }
        __syncthreads();
        const double off = red[warp];
        __syncthreads();
        return (lane ? e_in : 0.0) + off;
    }
    TL_D int first(bool p) const {
        const unsigned b = __ballot_sync(0xffffffffu, p);
        __syncthreads();
        if (lane == 0) red[warp] = b ? (double)(warp * 32 + __ffs(b) - 1) : 1e9;
        __syncthreads();
        if (warp == 0) {
            double x = lane < nwarps ? red[lane] : 1e9;
#pragma unroll
            for (int o = 16; o; o >>= 1) x = fmin(x, __shfl_xor_sync(0xffffffffu, x, o));
            if (lane == 0) red[33] = x;
        }
        __syncthreads();
        const double r = red[33];
        return r > 1e8 ? -1 : (int)r;
    }
    TL_D int last(bool p) const {
        const unsigned b = __ballot_sync(0xffffffffu, p);
        __syncthreads();
        if (lane == 0) red[warp] = b ? (double)(warp * 32 + 31 - __clz(b)) : -1.0;
        __syncthreads();
        if (warp == 0) {
            double x = lane < nwarps ? red[lane] : -1.0;
#pragma unroll
            for (int o = 16; o; o >>= 1) x = fmax(x, __shfl_xor_sync(0xffffffffu, x, o));
            if (lane == 0) red[33] = x;
        }
        __syncthreads();
        return (int)red[33];
    }
    template <class T>
    TL_D T bcast(T v, int src) const {
        static_assert(sizeof(T) <= 8, "bcast of a value wider than 8 bytes");
        __syncthreads();
        if (tid == src) *reinterpret_cast<T*>(red + 32) = v;
        __syncthreads();
        const T r = *reinterpret_cast<const T*>(red + 32);
        __syncthreads();
        return r;
    }
};

// ---------------------------------------------------------------------------
// Model view (global or staged copy in shared memory).
// ---------------------------------------------------------------------------
struct MView {
    const int2* chan;         // [M] {s0, s1 | order << 28}
    const signed char* rord;  // [M] the reference's order detector (-1, 1, 2, 3)
    const signed char* gkind; // [N]
    const int* perm;          // [N] row processing order (longest rows first)
    const int* rp;            // [N+1] CSR used for mu/sigma^2
    const int* vc;            // [nnz] packed (col<<3)|((v+2)&7)
    const int* urp;           // [N+1] CSR used for the update (net entries)
    const int* uvc;
    const int* cp;            // [M+1] CSC net (direct-method firing)
    const int* rv;            // [nnz] packed (row<<3)|((v+2)&7)
};

TL_HD int unpack_idx(int p) { return p >> 3; }
TL_HD int unpack_v(int p) { return (p & 7) - 2; }
// v as a float without an int-to-float conversion: 2^23 + (p & 7) is exact
// in FP32 and subtracting 2^23 + 2 leaves (p & 7) - 2.
TL_D float unpack_vf(int p) { return __int_as_float(0x4B000000 | (p & 7)) - 8388610.f; }

struct SimParams {
    int N, M;
    MView g;            // global view
    const void* x0;     // Pop[N]
    const float* rates; // [S][M]
    const double* t_final; // [S]
    const double* grid;    // [S][n_int+1] grid times
    long long R;        // realizations per set in this call
    long long r_off;    // id of the first realization (sharding)
    int S;
    uint32_t k0, k1;    // Philox key (seed)
    uint32_t rk[20];    // its round keys (round_keys)
    float eps;
    int nc;
    float ssa_factor;
    int ssa_block;
    int n_int;          // grid intervals (points = n_int + 1)
    int K;
    const int* tracked; // [K]
    void* samples;      // Pop[S*R][n_int+1][K]
    float* scores;      // [S*R][M] when sensitivity is on
    long long max_steps;
    unsigned flags;
    int max_halv;       // tau halvings allowed per leap before the realization stops
    int wait_polls;     // polls of the bounded staging wait (0: give up at once)
    // staging of the constant blob into shared memory
    const unsigned char* blob;
    int stage_bytes;    // 0 = no staging
    int off_chan, off_rord, off_gkind, off_perm, off_rp, off_vc, off_cp, off_rv;  // byte offsets (net)
    int slot_bytes;     // per group
    int row_warp;       // CTA groups: one warp per species row (long rows)
    unsigned char* gslots;  // CTA groups whose slot exceeds shared memory:
                            // one slot per CTA in global memory (else null)
    unsigned long long* ctr; // [0] work, [1] leaps, [2] ssa, [3] rejections,
                             // [4] truncated, [5] error bits, [6] done count
    // plain form state
    void* pstate;
    void* pslots;       // global slots for the plain form
};

// One item of a batched launch (tl_simulate_batch).
struct BatchItem {
    SimParams p;
    long long unit_begin, units;
    int lane_mode;  // 1: a unit is 32 realizations, one per lane
    int stage_off;  // byte offset of the model's tables in the staged region, -1: global
};

struct BatchParams {
    const BatchItem* items;
    int n_items;
    long long total_units;
    const unsigned char* stage_src;
    int stage_bytes;
    int warp_slot_bytes;
    int params_bytes;
    unsigned long long* wctr;
};

template <class Pop>
struct Slot {
    Pop* x;
    Pop* xn;   // next state of the update
    float* a;  // propensity (sign bit = critical)
    int* k;    // firing counts of the leap: over a[] unless the run keeps
               // likelihood-ratio scores, which read a[] after the leap
};

// Per-realization progress.  Every leap attempt and every direct-method
// step advances the Philox step counter once, so the counts need no
// registers of their own: accepted steps nsteps = leaps + ssa, and
// step = nsteps + rejections.
template <class TimeT>
struct RState {
    TimeT t;
    int kpt;           // next grid point to record
    uint32_t step;     // Philox step counter
    int done;
    long long nsteps;  // accepted steps (cap)
    uint32_t ssa;      // direct-method steps
};

TL_HD bool flag(unsigned f, unsigned b) { return (f & b) != 0; }
// A reference-compatibility switch: compiled out of the kernels built
// without them (COMPAT = false), read at run time otherwise.
template <bool COMPAT>
TL_D bool cflag(unsigned f, unsigned b) {
    return COMPAT && (f & b) != 0;
}

// Grid time k of rate set `set`: T*k/n_int (T itself for k = n_int), from
// the table the host fills with exactly that FP64 expression, so that a leap
// loads one double instead of dividing on the reduced-rate FP64 pipe.
template <class TimeT>
TL_D TimeT grid_time(const SimParams& p, int set, int k) {
    return (TimeT)__ldg(p.grid + (size_t)set * (p.n_int + 1) + k);
}

// ---------------------------------------------------------------------------
// Passes.
// ---------------------------------------------------------------------------

// Propensities of all channels into a[] (sign = critical); lane partial sums.
template <class Grp, class Pop, bool COMPAT = true>
TL_D void pass_props(const Grp& g, const SimParams& p, const MView& mv, const float* rate,
                     const Pop* x, float* a, float& pa, float& pac) {
    const bool cc = cflag<COMPAT>(p.flags, TL_FLAG_COMPAT_CRIT);
    float s = 0.f, sc = 0.f;
    for (int j = g.rank(); j < p.M; j += g.size()) {
        float aj;
        bool crit;
        propensity<Pop>(mv.chan[j], __ldg(rate + j), x, p.nc, cc, aj, crit);
        aj = fabsf(aj);  // 2S-> at x=0 gives -0.0; the sign bit carries criticality
        a[j] = crit ? -aj : aj;
        s += aj;
        sc += crit ? aj : 0.f;
    }
    pa = s;
    pac = sc;
}

// CGP bound of species i from its CSR row; optional moments out.
template <class Pop, bool COMPAT = true>
TL_D float species_bound(const SimParams& p, const MView& mv, const Pop* x, const float* a, int i,
                         float mu, float s2) {
    const bool cg = cflag<COMPAT>(p.flags, TL_FLAG_COMPAT_G);
    const float xi = popf(x[i]);
    float gi;
    if (cg) {
        const int ord = i < p.M ? mv.rord[i] : 0;
        gi = (ord >= 1 && ord <= 3) ? (ord == 3 ? 2.f + 1.f / (xi - 1.f) : (float)ord) : 0.f;
    } else {
        gi = g_of(mv.gkind[i], xi);
    }
    // __fdividef (2 ulp); a zero moment gives an infinite bound as with IEEE
    const float num = fmaxf(p.eps * __fdividef(xi, gi), 1.f);
    const float b1 = mu != 0.f ? __fdividef(num, fabsf(mu)) : kInfF;
    const float b2 = s2 != 0.f ? __fdividef(num * num, fabsf(s2)) : kInfF;
    return fminf(b1, b2);
}

template <bool OUT, class Grp, class Pop, bool COMPAT = true>
TL_D float pass_tau(const Grp& g, const SimParams& p, const MView& mv, const Pop* x, const float* a,
                    float* mu_out, float* s2_out) {
    const bool all_rows = cflag<COMPAT>(p.flags, TL_FLAG_COMPAT_STOICH);
    float tmin = kInfF;
    bool done = false;
    if constexpr (Grp::kWidth == 0) {
      if (p.row_warp) {
        // one warp per species row, lanes stride the row's entries
        const GCta& gc = g;
        done = true;
        for (int i = gc.warp; i < p.N; i += gc.nwarps) {
            if (!all_rows && mv.gkind[i] == 0 && !OUT) continue;
            float mu = 0.f, s2 = 0.f;
            const int e = mv.rp[i + 1];
            for (int q = mv.rp[i] + gc.lane; q < e; q += 32) {
                const int pk = mv.vc[q];
                const float aj = fmaxf(a[unpack_idx(pk)], 0.f);
                const float v = unpack_vf(pk);
                const float t = v * aj;
                mu += t;
                s2 += v * t;
            }
#pragma unroll
            for (int o = 16; o; o >>= 1) {
                mu += __shfl_xor_sync(0xffffffffu, mu, o);
                s2 += __shfl_xor_sync(0xffffffffu, s2, o);
            }
            if (gc.lane == 0) {
                if (OUT) {
                    mu_out[i] = mu;
                    s2_out[i] = s2;
                }
                if (all_rows || mv.gkind[i] != 0) tmin = fminf(tmin, species_bound<Pop, COMPAT>(p, mv, x, a, i, mu, s2));
            }
        }
      }
    }
    if (!done) {
        for (int ii = g.rank(); ii < p.N; ii += g.size()) {
            const int i = mv.perm[ii];
            if (!all_rows && mv.gkind[i] == 0 && !OUT) continue;
            float mu = 0.f, s2 = 0.f;
            const int e = mv.rp[i + 1];
#pragma unroll 4
            for (int q = mv.rp[i]; q < e; ++q) {
                const int pk = mv.vc[q];
                // critical channels are stored negative: max(a, 0) drops them
                const float aj = fmaxf(a[unpack_idx(pk)], 0.f);
                const float v = unpack_vf(pk);
                const float t = v * aj;
                mu += t;
                s2 += v * t;
            }
            if (OUT) {
                mu_out[i] = mu;
                s2_out[i] = s2;
            }
            if (all_rows || mv.gkind[i] != 0) tmin = fminf(tmin, species_bound<Pop, COMPAT>(p, mv, x, a, i, mu, s2));
        }
    }
    return g.minf(tmin);
}

// xn = x + V k (k stored as int in a[]); returns true if any xn < 0 (or the
// population type overflows, which also sets *ovf).
template <class Grp, class Pop>
TL_D bool pass_update(const Grp& g, const SimParams& p, const MView& mv, const Pop* x, const int* k,
                      Pop* xn, bool& ovf) {
    bool neg = false, of = false;
    bool done = false;
    if constexpr (Grp::kWidth == 0) {
      if (p.row_warp) {
        const GCta& gc = g;
        done = true;
        for (int i = gc.warp; i < p.N; i += gc.nwarps) {
            long long d = 0;
            const int e = mv.urp[i + 1];
            for (int q = mv.urp[i] + gc.lane; q < e; q += 32) {
                const int pk = mv.uvc[q];
                d += (long long)unpack_v(pk) * (long long)k[unpack_idx(pk)];
            }
#pragma unroll
            for (int o = 16; o; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
            if (gc.lane == 0) {
                const long long nx = (long long)x[i] + d;
                if (sizeof(Pop) == 4 && nx > 2147483647LL) of = true;
                xn[i] = (Pop)nx;
                neg |= nx < 0;
            }
        }
      }
    }
    if (!done) {
        for (int ii = g.rank(); ii < p.N; ii += g.size()) {
            const int i = mv.perm[ii];
            long long d = 0;
            const int e = mv.urp[i + 1];
#pragma unroll 4
            for (int q = mv.urp[i]; q < e; ++q) {
                const int pk = mv.uvc[q];
                d += (long long)unpack_v(pk) * (long long)k[unpack_idx(pk)];
            }
            const long long nx = (long long)x[i] + d;
            if (sizeof(Pop) == 4 && nx > 2147483647LL) of = true;
            xn[i] = (Pop)nx;
            neg |= nx < 0;
        }
    }
    ovf = g.any(of);
    return g.any(neg || of);
}

// Draw a channel with probability a_j / total among channels whose
// criticality matches `want` (want: 0 = all channels, 1 = critical only).
// Channels are taken in lane-major order: lane l owns j = l, l+G, ... .  The
// cumulative sums across lanes are FP64; inside a lane the FP32 partial sum
// is replayed in the same order it was accumulated, so the lane intervals
// tile [0, total) exactly as the totals were formed.
// Out of line: it runs only when a critical channel fires and in
// direct-method steps, and one copy keeps the leap loop small.
template <class Grp, class AccT>
__device__ __noinline__ int select_channel_impl(const Grp g, const int M, const float* a, float lane_part,
                                                AccT target, int want_crit) {
    const AccT part = (AccT)lane_part;
    AccT excl;
    if constexpr (Grp::kWidth == 1) {
        excl = 0;
    } else {
        excl = (AccT)g.excl_scan((double)part);
    }
    const bool mine = (part > (AccT)0) && (target < excl + part);
    int L = g.first(mine);
    if (L < 0) L = g.last(part > (AccT)0);
    int sel = -1;
    if (g.rank() == L) {
        float acc = 0.f;
        int lastpos = -1;
        // Inside the lane the search runs on the lane's FP32 running sum:
        // the offset into the lane, target - excl (FP64), rounded toward
        // -inf, so that for a float acc  rd(t) < acc  <=>  t < acc exactly.
        const AccT trem = target - excl;
        const float tf = sizeof(AccT) == 8 ? __double2float_rd((double)trem) : (float)trem;
        for (int j = g.rank(); j < M; j += g.size()) {
            const float aj = a[j];
            const bool c = is_crit(aj);
            if (want_crit && !c) continue;
            const float v = fabsf(aj);
            if (!(v > 0.f)) continue;
            acc += v;
            lastpos = j;
            if (tf < acc) {
                sel = j;
                break;
            }
        }
        if (sel < 0) sel = lastpos;
    }
    if constexpr (Grp::kWidth == 1) {
        return sel;
    } else {
        return g.bcast(sel, L < 0 ? 0 : L);
    }
}

template <class Grp, class AccT>
TL_D int select_channel(const Grp& g, const SimParams& p, const float* a, float lane_part, AccT target,
                        int want_crit) {
    return select_channel_impl<Grp, AccT>(g, p.M, a, lane_part, target, want_crit);
}

// Lane partial sum of critical propensities in the same order select uses.
// (pass_props already returns it as pac.)

template <class Grp, class Pop>
TL_D void record_point(const Grp& g, const SimParams& p, const Pop* x, Pop* samp, int kpt) {
    Pop* dst = samp + (size_t)kpt * p.K;
    for (int q = g.rank(); q < p.K; q += g.size()) dst[q] = x[p.tracked[q]];
}

// Poisson firing counts of one leap (model.cu:458-549), written over a[] as
// ints.  A thread takes four consecutive channels at a time so that they
// share one Philox block for their first uniforms.
template <class Grp, bool COMPAT = true>
TL_D void pass_fire(const Grp& g, const SimParams& p, const float* a, int* kk, float tauf, int jc, uint32_t step,
                    uint32_t r, uint32_t set) {
    const bool refs = cflag<COMPAT>(p.flags, TL_FLAG_COMPAT_POISSON);
    const bool vec = (reinterpret_cast<uintptr_t>(a) & 15) == 0 && (reinterpret_cast<uintptr_t>(kk) & 15) == 0;
    for (int g4 = g.rank(); 4 * g4 < p.M; g4 += g.size()) {
        const int j0 = 4 * g4;
        const bool full = vec && j0 + 3 < p.M;
        float av[4];
        if (full) {
            const float4 v = *reinterpret_cast<const float4*>(a + j0);
            av[0] = v.x;
            av[1] = v.y;
            av[2] = v.z;
            av[3] = v.w;
        } else {
#pragma unroll
            for (int e = 0; e < 4; ++e) av[e] = j0 + e < p.M ? a[j0 + e] : -0.f;
        }
        // the shared block feeds only the k = 0 tests of means in (0, 10)
        bool need = false;
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const float m = av[e] * tauf;
            need |= !is_crit(av[e]) && m > 0.f && m < 10.f;
        }
        U4 gw{0u, 0u, 0u, 0u};
        if (need && !refs) gw = group_words(p.rk, (uint32_t)g4, step, r, set);
        // hot path: criticals, zero means, and the k = 0 / k = 1 tests of
        // poisson_first on the shared word; the draws that go on (k >= 2,
        // means >= 10, the reference's sampler) are marked in `rare`
        // Thread groups (one realization per thread, latency-bound) finish
        // each long draw in place; warp and CTA groups mark them in `rare`.
        // k = 0 iff q >= P(K >= 1), and P(K >= 1) as poisson_p1 computes it
        // never exceeds mu (below 0.1 the series factor rounds to <= 1;
        // above, 1 - exp(-mu) < 0.96 mu), so q >= mu settles k = 0 with one
        // compare.  Thread groups skip the exact tests that way; sub-warp
        // and warp groups mark the channels with q < mu in `slow` and run
        // the exact tests on those alone after the unrolled loop, so that
        // the tests' branches do not diverge across the warp once per
        // channel.  CTA groups (large models, whose means are seldom far
        // below 1) keep the tests in the loop: deferred, they measured
        // 3 % slower on the colloid model.
        int kv[4];
        unsigned rare = 0, slow = 0;
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            int k = 0;
            if (is_crit(av[e])) {
                k = (j0 + e == jc) ? 1 : 0;
            } else {
                const float mu = av[e] * tauf;
                if (mu > 0.f) {
                    bool more = refs || mu >= 10.f;
                    float q = 0.f;
                    if (!more) {
                        q = ((float)word_of(gw, e) + 0.5f) * 2.3283064365386963e-10f;
                        if constexpr (Grp::kWidth >= 2) {
                            if (q < mu) slow |= 1u << e;
                        } else if (Grp::kWidth == 0 || q < mu) {
                            if (q < poisson_p1(mu)) {
                                if (q >= poisson_p2(mu)) k = 1;
                                else more = true;
                            }
                        }
                    }
                    if (more) {
                        if constexpr (Grp::kWidth == 1)
                            k = poisson_rare_inline<COMPAT>(mu, q, (uint32_t)(j0 + e), step, r, set, p.rk,
                                                            refs ? 1 : 0);
                        else
                            rare |= 1u << e;
                    }
                }
            }
            kv[e] = k;
        }
        // the exact k <= 1 tests of the channels with q < mu
        while (slow) {
            const int e = __ffs(slow) - 1;
            slow &= slow - 1;
            const float mu = (e == 0 ? av[0] : e == 1 ? av[1] : e == 2 ? av[2] : av[3]) * tauf;
            const float q = ((float)word_of(gw, e) + 0.5f) * 2.3283064365386963e-10f;
            if (q < poisson_p1(mu)) {
                if (q >= poisson_p2(mu)) {
                    kv[0] = e == 0 ? 1 : kv[0];
                    kv[1] = e == 1 ? 1 : kv[1];
                    kv[2] = e == 2 ? 1 : kv[2];
                    kv[3] = e == 3 ? 1 : kv[3];
                } else {
                    rare |= 1u << e;
                }
            }
        }
        // the marked draws, from one call site (one copy of the long draw in
        // the loop rather than one per unrolled channel)
        while (rare) {
            const int e = __ffs(rare) - 1;
            rare &= rare - 1;
            const float mu = (e == 0 ? av[0] : e == 1 ? av[1] : e == 2 ? av[2] : av[3]) * tauf;
            const float q = refs ? 0.f : ((float)word_of(gw, e) + 0.5f) * 2.3283064365386963e-10f;
            const uint32_t j = (uint32_t)(j0 + e);
            // out of line unless TL_RARE_INLINE
            const int k = poisson_rare<COMPAT>(mu, q, j, step, r, set, p.rk, refs ? 1 : 0);
            kv[0] = e == 0 ? k : kv[0];
            kv[1] = e == 1 ? k : kv[1];
            kv[2] = e == 2 ? k : kv[2];
            kv[3] = e == 3 ? k : kv[3];
        }
        if (full) {
            *reinterpret_cast<int4*>(kk + j0) = make_int4(kv[0], kv[1], kv[2], kv[3]);
        } else {
#pragma unroll
            for (int e = 0; e < 4; ++e)
                if (j0 + e < p.M) kk[j0 + e] = kv[e];
        }
    }
}

// ---------------------------------------------------------------------------
// One step of one realization: a tau-leap (with rejection + halving) or a
// block of direct-method steps (model.cu:301-413).
// ---------------------------------------------------------------------------
template <class Grp, class Pop, class TimeT, bool SENS, bool COMPAT = true>
TL_D void do_step(const Grp& g, const SimParams& p, const MView& mv, Slot<Pop>& s, int set, uint32_t r,
                  Pop* samp, float* score, RState<TimeT>& st) {
    const float* rate = p.rates + (size_t)set * p.M;
    const double T = p.t_final[set];
    const unsigned f = p.flags;

    float pa, pac;
    pass_props<Grp, Pop, COMPAT>(g, p, mv, rate, s.x, s.a, pa, pac);
    g.sync();
    const float a0f = g.sumf(pa);  // FP32: only the branch test and tau2 use it
    if (!(a0f > 0.f)) {
        // nothing can fire: the state holds to t_final
        while (st.kpt <= p.n_int) record_point<Grp, Pop>(g, p, s.x, samp, st.kpt++);
        st.t = (TimeT)T;
        st.done = 1;
        return;
    }
    float tau1 = pass_tau<false, Grp, Pop, COMPAT>(g, p, mv, s.x, s.a, nullptr, nullptr);

    if (tau1 * a0f < p.ssa_factor) {
        // ---- direct-method block (CGP 2006 step 2; model.cu:334-345) ----
        for (int q = 0; q < p.ssa_block; ++q) {
            if (q > 0) {
                pass_props<Grp, Pop, COMPAT>(g, p, mv, rate, s.x, s.a, pa, pac);
                g.sync();
            }
            // total for the cumulative search: FP64 over the lane partials
            const TimeT a0 = (TimeT)g.sumd((double)pa);
            {
                if (!(a0 > (TimeT)0)) {
                    while (st.kpt <= p.n_int) record_point<Grp, Pop>(g, p, s.x, samp, st.kpt++);
                    if (SENS) {
                        // no channel can fire: the survival term is zero
                    }
                    st.t = (TimeT)T;
                    st.done = 1;
                    return;
                }
            }
            const U4 w = step_words(p.rk, st.step, r, (uint32_t)set);
            const TimeT target = (TimeT)u01d(w.z, w.w) * a0;
            const int j = select_channel<Grp, TimeT>(g, p, s.a, pa, target, 0);
            // the waiting time in FP32 (FP64 keeps only the time sum)
            const float ex = -logf(u01f(w.x));
            const TimeT dt = (TimeT)(cflag<COMPAT>(f, TL_FLAG_COMPAT_TAU2) ? ex / fabsf(s.a[j]) : ex / (float)a0);
            while (st.kpt <= p.n_int && st.t + dt >= grid_time<TimeT>(p, set, st.kpt))
                record_point<Grp, Pop>(g, p, s.x, samp, st.kpt++);
            if (st.kpt > p.n_int) {
                if (SENS && score) {
                    const float rem = (float)((TimeT)T - st.t);
                    for (int m = g.rank(); m < p.M; m += g.size()) {
                        const float c = __ldg(rate + m);
                        if (c > 0.f) score[m] -= fabsf(s.a[m]) * rem / c;
                    }
                }
                st.t = (TimeT)T;
                st.done = 1;
                g.sync();
                return;
            }
            if (SENS && score) {
                const float dtf = (float)dt;
                for (int m = g.rank(); m < p.M; m += g.size()) {
                    const float c = __ldg(rate + m);
                    if (c > 0.f) score[m] += ((m == j ? 1.f : 0.f) - fabsf(s.a[m]) * dtf) / c;
                }
            }
            g.sync();
            if (!cflag<COMPAT>(f, TL_FLAG_COMPAT_SSA) && j >= 0) {
                const int e = mv.cp[j + 1];
                for (int q2 = mv.cp[j] + g.rank(); q2 < e; q2 += g.size()) {
                    const int pk = mv.rv[q2];
                    s.x[unpack_idx(pk)] += (Pop)unpack_v(pk);
                }
            }
            g.sync();
            st.t += dt;
            st.step++;
            st.ssa++;
            st.nsteps++;
            if (p.max_steps > 0 && st.nsteps >= p.max_steps) return;
        }
        return;
    }

    // ---- tau-leap with negative-population rejection (CGP 2006 steps 3-5) ----
    const TimeT t_next = grid_time<TimeT>(p, set, st.kpt);
    TimeT t_new;      // time after the leap (unless clamped to t_next)
    float tau_used;   // the leap's tau
    bool clamp;
    for (int attempt = 0;; ++attempt) {
        const float a0cf = g.sumf(pac);
        // the step's scalar words are needed only when a channel is critical
        const U4 w = a0cf > 0.f ? step_words(p.rk, st.step, r, (uint32_t)set) : U4{0u, 0u, 0u, 0u};
        int jc = -1;
        float tau2 = kInfF;
        if (a0cf > 0.f) {
            if (cflag<COMPAT>(f, TL_FLAG_COMPAT_TAU2)) {
                const TimeT a0c = (TimeT)g.sumd((double)pac);
                jc = select_channel<Grp, TimeT>(g, p, s.a, pac, (TimeT)u01d(w.z, w.w) * a0c, 1);
                tau2 = -logf(u01f(w.x)) / fabsf(s.a[jc]);
            } else {
                tau2 = -logf(u01f(w.x)) / a0cf;
            }
        }
        float tauf = fminf(tau1, tau2);
        bool fire = tau2 < tau1;
        t_new = st.t + (TimeT)tauf;
        clamp = t_new >= t_next;
        if (clamp) {
            tauf = (float)(t_next - st.t);
            fire = false;
        }
        tau_used = tauf;
        if (fire && jc < 0) {
            const TimeT a0c = (TimeT)g.sumd((double)pac);
            jc = select_channel<Grp, TimeT>(g, p, s.a, pac, (TimeT)u01d(w.z, w.w) * a0c, 1);
        }
        if (!fire) jc = -1;
        pass_fire<Grp, COMPAT>(g, p, s.a, s.k, tauf, jc, st.step, r, (uint32_t)set);
        g.sync();
        bool ovf = false;
        const bool bad = pass_update<Grp, Pop>(g, p, mv, s.x, s.k, s.xn, ovf);
        if (ovf) {
            if (g.leader()) atomicOr((unsigned*)(p.ctr + 5), kErrOverflow);
            st.done = 1;
            while (st.kpt <= p.n_int) record_point<Grp, Pop>(g, p, s.x, samp, st.kpt++);
            return;
        }
        if (!bad) break;
        // reject: halve tau1, fresh counters, same state
        st.step++;
        tau1 *= 0.5f;
        g.sync();
        pass_props<Grp, Pop, COMPAT>(g, p, mv, rate, s.x, s.a, pa, pac);
        g.sync();
        if (attempt + 1 > p.max_halv) {
            if (g.leader()) atomicOr((unsigned*)(p.ctr + 5), kErrHalving);
            st.done = 1;
            while (st.kpt <= p.n_int) record_point<Grp, Pop>(g, p, s.x, samp, st.kpt++);
            return;
        }
    }
    if (SENS && score) {
        // score_j += (k_j - a_j*tau)/c_j with a_j of the pre-leap state, kept
        // in a[] (the counts went to their own array in scored runs)
        const float tauf = tau_used;
        const int* kk = s.k;
        for (int m = g.rank(); m < p.M; m += g.size()) {
            const float c = __ldg(rate + m);
            if (c > 0.f) score[m] += ((float)kk[m] - fabsf(s.a[m]) * tauf) / c;
        }
    }
    g.sync();
    {
        Pop* t = s.x;
        s.x = s.xn;
        s.xn = t;
    }
    st.t = clamp ? t_next : t_new;
    st.step++;
    st.nsteps++;
    if (clamp) {
        record_point<Grp, Pop>(g, p, s.x, samp, st.kpt);
        st.kpt++;
        if (st.kpt > p.n_int) st.done = 1;
    }
    g.sync();
}

}  // namespace tl
