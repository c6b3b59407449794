// tl_oracle.cpp - FP64 host oracle of the tau-leaping hot path.
//
// TEST INFRASTRUCTURE ONLY.  Nothing in the engine links or calls this code;
// only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
// it (liboracle.so), as the checker the CUDA path is compared against.
//
// It restates, in double precision and in plain loops, the algorithm of the
// reference (CSSL-UWM/tau_leaping) with the Cao-Gillespie-Petzold rules the
// engine's default mode uses, each function citing what it follows:
//   reaction order / reactant indices   tau_leaping/CSCMatrix.cu:185-251
//   propensity + criticality            tau_leaping/functions.h:100-123
//   g, mu, sigma^2, tau1                tau_leaping/CSRMatrixPacked.cu:294-358
//   leap / direct-method branch         tau_leaping/model.cu:301-413
//   critical channel, tau2              tau_leaping/model.cu:555-598
//   Poisson firing                      tau_leaping/model.cu:458-521
//   integer update                      tau_leaping/CSRMatrixPacked.cu:464-492
//   direct-method step                  tau_leaping/model.cu:427-451
// plus an exact direct-method SSA (Gillespie 1977) for statistical checks.
// Random numbers come from its own Philox4x32-10 (Salmon et al. SC'11) with
// the engine's counter layout: step scalars (0xFFFFFFFF, step, r, set<<8),
// first Poisson words of channels 4g..4g+3 (g, step, r, set<<8|0xFF), and
// further per-channel uniforms (j, step, r, set<<8|b), so both sides draw
// from the same streams.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

namespace {

struct W4 {
    uint32_t x, y, z, w;
};

W4 philox(W4 c, uint32_t k0, uint32_t k1) {
    for (int r = 0; r < 10; ++r) {
        if (r) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        const uint64_t p0 = (uint64_t)0xD2511F53u * c.x;
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c.z;
        c = W4{(uint32_t)(p1 >> 32) ^ c.y ^ k0, (uint32_t)p1, (uint32_t)(p0 >> 32) ^ c.w ^ k1, (uint32_t)p0};
    }
    return c;
}

double uni23(uint32_t w) { return ((double)(w >> 9) + 0.5) / 8388608.0; }
double uni52(uint32_t hi, uint32_t lo) {
    const uint64_t k = ((uint64_t)(hi >> 6) << 26) | (uint64_t)(lo >> 6);
    return ((double)k + 0.5) / 4503599627370496.0;
}

struct Stream {
    uint32_t j, step, r, c3, k0, k1;
    W4 b{};
    int left = 0;
    double next() {
        if (!left) {
            b = philox(W4{j, step, r, c3}, k0, k1);
            c3++;
            left = 4;
        }
        const uint32_t w = b.x;
        b.x = b.y;
        b.y = b.z;
        b.z = b.w;
        --left;
        return uni23(w);
    }
};

// Poisson(mu): inversion below 10, Hormann's PTRS (1993) above.  For mu <
// 10 the first uniform is q = (w + 1/2) 2^-32 from the channel's word of the
// shared block: K = 0 iff q >= 1 - exp(-mu); otherwise the inversion goes on
// with u = 1 - q from k = 1.  Further uniforms come from the private stream.
int64_t poisson_inv(double mu, Stream& s);
int64_t poisson(double mu, uint32_t w, Stream& s) {
    if (!(mu > 0.0)) return 0;
    if (mu < 10.0) {
        const double q = ((double)w + 0.5) / 4294967296.0;
        if (q >= -std::expm1(-mu)) return 0;
        const double u = 1.0 - q;
        double p = std::exp(-mu), F = p;
        for (int k = 1; k < 200; ++k) {
            p *= mu / (double)k;
            const double Fn = F + p;
            if (u <= Fn) return k;
            if (Fn == F) break;
            F = Fn;
        }
        return poisson_inv(mu, s);
    }
    return poisson_inv(mu, s);
}

int64_t poisson_inv(double mu, Stream& s) {
    if (!(mu > 0.0)) return 0;
    if (mu < 10.0) {
        for (;;) {
            const double u = s.next();
            double p = std::exp(-mu), F = p;
            int64_t k = 0;
            bool ok = true;
            while (u > F) {
                ++k;
                p *= mu / (double)k;
                const double Fn = F + p;
                if (Fn == F) {
                    ok = false;
                    break;
                }
                F = Fn;
            }
            if (ok) return k;
        }
    }
    const double smu = std::sqrt(mu), lmu = std::log(mu);
    const double b = 0.931 + 2.53 * smu, a = -0.059 + 0.02483 * b;
    const double ia = 1.1239 + 1.1328 / (b - 3.4), vr = 0.9277 - 3.6224 / (b - 2.0);
    for (;;) {
        const double U = s.next() - 0.5, V = s.next();
        const double us = 0.5 - std::fabs(U);
        const double k = std::floor((2.0 * a / us + b) * U + mu + 0.43);
        if (us >= 0.07 && V <= vr) return (int64_t)k;
        if (k < 0.0 || (us < 0.013 && V > us)) continue;
        if (std::log(V * ia / (a / (us * us) + b)) <= -mu + k * lmu - std::lgamma(k + 1.0)) return (int64_t)k;
    }
}

// The reference's sampler, model.cu:477-520 (Knuth below 80, |Normal| above).
int64_t poisson_ref(double mu, Stream& s) {
    if (mu < 80.0) {
        const double lam = std::exp(-mu);
        double val = 1.0;
        for (int n = 1; n < 300; ++n) {
            val *= s.next();
            if (val < lam) return n - 1;
        }
        return 300;
    }
    double u, v, q;
    do {
        u = 2.0 * s.next() - 1.0;
        v = 2.0 * s.next() - 1.0;
        q = u * u + v * v;
    } while (q >= 1.0);
    return (int64_t)std::fabs(mu + std::sqrt(mu) * u * std::sqrt(-2.0 * std::log(q) / q));
}

enum : unsigned {
    F_COMPAT_G = 1u << 8,
    F_COMPAT_CRIT = 1u << 9,
    F_COMPAT_STOICH = 1u << 10,
    F_COMPAT_TAU2 = 1u << 11,
    F_COMPAT_SSA = 1u << 12,
    F_COMPAT_POISSON = 1u << 13,
};

}  // namespace

struct ora_model {
    int N = 0, M = 0;
    std::vector<int64_t> x0;
    std::vector<double> rate;
    std::vector<int> order, ref_order, s0, s1, gkind;
    // species-row lists: raw entries and net stoichiometry
    std::vector<std::vector<std::pair<int, int>>> raw_rows, net_rows;
    // channel-column net stoichiometry
    std::vector<std::vector<std::pair<int, int>>> net_cols;
};

extern "C" {

ora_model* ora_model_new(int N, int M, const int64_t* x0, const double* rate, const int32_t* cp, const int32_t* ri,
                         const int8_t* st) {
    ora_model* m = new ora_model();
    m->N = N;
    m->M = M;
    m->x0.assign(x0, x0 + N);
    m->rate.assign(rate, rate + M);
    m->order.assign(M, 0);
    m->ref_order.assign(M, -1);
    m->s0.assign(M, 0);
    m->s1.assign(M, 0);
    m->gkind.assign(N, 0);
    m->raw_rows.assign(N, {});
    m->net_rows.assign(N, {});
    m->net_cols.assign(M, {});
    for (int j = 0; j < M; ++j) {
        // reference order detector (CSCMatrix.cu:204-231)
        int first = 0, second = 0;
        std::vector<std::pair<int, int>> re;
        std::vector<std::pair<int, int>> net;
        for (int q = cp[j]; q < cp[j + 1]; ++q) {
            const int v = st[q];
            m->raw_rows[ri[q]].push_back({j, v});
            bool merged = false;
            for (auto& e : net)
                if (e.first == ri[q]) {
                    e.second += v;
                    merged = true;
                }
            if (!merged) net.push_back({ri[q], v});
            if (v >= 0) continue;
            if (!first) first = v;
            else second = v;
            re.push_back({ri[q], -v});
        }
        m->ref_order[j] = first == -2 ? 3 : (first == -1 && second == -1) ? 2 : first == -1 ? 1 : -1;
        if (re.empty()) m->order[j] = 0;
        else if (re.size() == 1) {
            m->order[j] = re[0].second == 2 ? 3 : 1;
            m->s0[j] = m->s1[j] = re[0].first;
        } else {
            m->order[j] = 2;
            m->s0[j] = re[0].first;
            m->s1[j] = re[1].first;
        }
        for (auto& e : net)
            if (e.second) {
                m->net_cols[j].push_back(e);
                m->net_rows[e.first].push_back({j, e.second});
            }
        const int o = m->order[j];
        if (o == 1) m->gkind[m->s0[j]] = std::max(m->gkind[m->s0[j]], 1);
        if (o == 2) {
            m->gkind[m->s0[j]] = std::max(m->gkind[m->s0[j]], 2);
            m->gkind[m->s1[j]] = std::max(m->gkind[m->s1[j]], 2);
        }
        if (o == 3) m->gkind[m->s0[j]] = 3;
    }
    for (auto& row : m->net_rows) std::sort(row.begin(), row.end());
    return m;
}

void ora_model_free(ora_model* m) { delete m; }

}  // extern "C"

namespace {

// functions.h:100-123 (+ order 0: constant propensity, never critical)
void propensity(const ora_model& m, int j, double c, const int64_t* x, int nc, bool compat_crit, double& a,
                bool& crit) {
    const int o = m.order[j];
    const int64_t x0 = x[m.s0[j]], x1 = x[m.s1[j]];
    if (o == 1) {
        a = c * (double)x0;
        crit = x0 < nc;
    } else if (o == 2) {
        a = c * (double)x0 * (double)x1;
        crit = x0 < nc || x1 < nc;
    } else if (o == 3) {
        a = c * (double)x0 * (double)(x0 - 1) / 2.0;
        crit = compat_crit ? 2 * x0 < nc : x0 < 2 * (int64_t)nc;
    } else {
        a = c;
        crit = false;
    }
}

// CSRMatrixPacked.cu:294-358: per species mu, sigma^2 over non-critical
// channels, tau1 = min_i min(max(eps x_i/g_i,1)/|mu_i|, max(..)^2/sigma_i^2).
double tau_bound(const ora_model& m, const int64_t* x, const std::vector<double>& a, const std::vector<char>& crit,
                 double eps, unsigned flags, double* mu_out, double* s2_out) {
    const bool raw = flags & F_COMPAT_STOICH;
    double tmin = INFINITY;
    for (int i = 0; i < m.N; ++i) {
        const auto& row = raw ? m.raw_rows[i] : m.net_rows[i];
        double mu = 0.0, s2 = 0.0;
        for (auto& e : row) {
            if (crit[e.first]) continue;
            mu += e.second * a[e.first];
            s2 += (double)e.second * e.second * a[e.first];
        }
        if (mu_out) mu_out[i] = mu;
        if (s2_out) s2_out[i] = s2;
        if (!raw && m.gkind[i] == 0) continue;
        const double xi = (double)x[i];
        double g;
        if (flags & F_COMPAT_G) {
            const int o = i < m.M ? m.ref_order[i] : 0;
            g = o == 1 ? 1.0 : o == 2 ? 2.0 : o == 3 ? 2.0 + 1.0 / (xi - 1.0) : 0.0;
        } else {
            const int k = m.gkind[i];
            g = k == 1 ? 1.0 : k == 2 ? 2.0 : (xi >= 2.0 ? 2.0 + 1.0 / (xi - 1.0) : 3.0);
        }
        double num = eps * xi / g;
        if (!(num > 1.0)) num = 1.0;
        const double b = std::min(num / std::fabs(mu), num * num / std::fabs(s2));
        tmin = std::min(tmin, b);
    }
    return tmin;
}

}  // namespace

extern "C" {

int ora_eval(const ora_model* m, const int64_t* x, int n, double eps, unsigned flags, int nc, double* a_out,
             uint8_t* crit_out, double* mu_out, double* s2_out, double* tau_out, double* a0_out) {
    std::vector<double> a(m->M);
    std::vector<char> crit(m->M);
    for (int s = 0; s < n; ++s) {
        const int64_t* xs = x + (size_t)s * m->N;
        double a0 = 0.0;
        for (int j = 0; j < m->M; ++j) {
            bool c;
            propensity(*m, j, m->rate[j], xs, nc > 0 ? nc : 5, flags & F_COMPAT_CRIT, a[j], c);
            crit[j] = c;
            a0 += a[j];
            if (a_out) a_out[(size_t)s * m->M + j] = a[j];
            if (crit_out) crit_out[(size_t)s * m->M + j] = c;
        }
        const double t = tau_bound(*m, xs, a, crit, eps, flags, mu_out ? mu_out + (size_t)s * m->N : nullptr,
                                   s2_out ? s2_out + (size_t)s * m->N : nullptr);
        if (tau_out) tau_out[s] = t;
        if (a0_out) a0_out[s] = a0;
    }
    return 0;
}

// CSRMatrixPacked.cu:464-492 with the loop over species rows (not channels).
int ora_replay(const ora_model* m, const int64_t* x0, const int32_t* k, int n_leaps, int raw, int64_t* x_out) {
    std::vector<int64_t> x(x0, x0 + m->N);
    for (int l = 0; l < n_leaps; ++l) {
        const int32_t* kl = k + (size_t)l * m->M;
        std::vector<int64_t> xn(x);
        for (int i = 0; i < m->N; ++i) {
            const auto& row = raw ? m->raw_rows[i] : m->net_rows[i];
            for (auto& e : row) xn[i] += (int64_t)e.second * kl[e.first];
        }
        x = xn;
        std::copy(x.begin(), x.end(), x_out + (size_t)l * m->N);
    }
    return 0;
}

void ora_philox(const uint32_t* ctr, const uint32_t* key, int n, uint32_t* out) {
    for (int i = 0; i < n; ++i) {
        const W4 r = philox(W4{ctr[4 * i], ctr[4 * i + 1], ctr[4 * i + 2], ctr[4 * i + 3]}, key[2 * i], key[2 * i + 1]);
        out[4 * i] = r.x;
        out[4 * i + 1] = r.y;
        out[4 * i + 2] = r.z;
        out[4 * i + 3] = r.w;
    }
}

int ora_poisson(const double* mean, int n, uint64_t seed, uint32_t step, int compat, int64_t* out) {
    for (int i = 0; i < n; ++i) {
        Stream s{(uint32_t)i, step, 0u, 0u, (uint32_t)seed, (uint32_t)(seed >> 32)};
        const W4 gw = philox(W4{(uint32_t)i >> 2, step, 0u, 0xFFu}, (uint32_t)seed, (uint32_t)(seed >> 32));
        const uint32_t w0 = (i & 3) == 0 ? gw.x : (i & 3) == 1 ? gw.y : (i & 3) == 2 ? gw.z : gw.w;
        out[i] = compat ? poisson_ref(mean[i], s) : poisson(mean[i], w0, s);
    }
    return 0;
}

typedef struct ora_cfg {
    double t_final, eps;
    int64_t R;          // realizations per set
    uint64_t seed;
    int32_t n_int, K;
    const int32_t* tracked;
    int32_t S;          // sets (>= 1)
    const double* rate_sets;    // [S][M] or NULL
    const double* t_final_sets; // [S] or NULL
    uint32_t flags;
    int32_t nc, ssa_factor, ssa_block;
    int64_t max_steps;
    int32_t method;     // 0 = CGP tau-leaping, 1 = exact SSA
    int32_t threads;
    int64_t r_begin, r_end;  // realizations r_begin..r_end-1 of each set
    int32_t sens;       // accumulate likelihood-ratio scores
} ora_cfg;

}  // extern "C"

namespace {

struct Counters {
    int64_t leaps = 0, ssa = 0, rej = 0, trunc = 0;
};

// One realization.  samp: [P][K]; score: [M] or null.
void run_one(const ora_model& m, const ora_cfg& c, int set, uint32_t r, int64_t* samp, double* score, Counters& cnt) {
    const int N = m.N, M = m.M, P = c.n_int + 1, K = c.K;
    const double* rate = c.rate_sets ? c.rate_sets + (size_t)set * M : m.rate.data();
    const double T = c.t_final_sets ? c.t_final_sets[set] : c.t_final;
    const uint32_t k0 = (uint32_t)c.seed, k1 = (uint32_t)(c.seed >> 32);
    const int nc = c.nc > 0 ? c.nc : 5;
    const double nssa = c.ssa_factor > 0 ? c.ssa_factor : 10;
    const int blk = c.ssa_block > 0 ? c.ssa_block : 100;
    const unsigned f = c.flags;
    std::vector<int64_t> x(m.x0), xn(N);
    std::vector<double> a(M);
    std::vector<char> crit(M);
    std::vector<int64_t> kk(M);
    auto grid = [&](int k) { return k >= c.n_int ? T : T * (double)k / (double)c.n_int; };
    auto rec = [&](int k) {
        for (int q = 0; q < K; ++q) samp[(size_t)k * K + q] = x[c.tracked[q]];
    };
    auto props = [&](double& a0, double& a0c) {
        a0 = a0c = 0.0;
        for (int j = 0; j < M; ++j) {
            bool cr;
            propensity(m, j, rate[j], x.data(), nc, f & F_COMPAT_CRIT, a[j], cr);
            crit[j] = cr;
            a0 += a[j];
            if (cr) a0c += a[j];
        }
    };
    auto pick = [&](double target, bool crit_only) {
        double acc = 0.0;
        int last = -1;
        for (int j = 0; j < M; ++j) {
            if (crit_only && !crit[j]) continue;
            if (!(a[j] > 0.0)) continue;
            acc += a[j];
            last = j;
            if (target < acc) return j;
        }
        return last;
    };
    if (score) std::fill(score, score + M, 0.0);
    double t = 0.0;
    int kpt = 1;
    uint32_t step = 0;
    int64_t nsteps = 0;
    rec(0);
    auto finish = [&]() {
        while (kpt <= c.n_int) rec(kpt++);
    };
    while (kpt <= c.n_int) {
        if (c.max_steps > 0 && nsteps >= c.max_steps) {
            finish();
            cnt.trunc++;
            break;
        }
        double a0, a0c;
        props(a0, a0c);
        if (!(a0 > 0.0)) {
            finish();
            break;
        }
        if (c.method == 1) {
            // exact direct method (Gillespie 1977)
            const W4 w = philox(W4{0xFFFFFFFFu, step, r, (uint32_t)set << 8}, k0, k1);
            const double dt = -std::log(uni23(w.x)) / a0;
            const int j = pick(uni52(w.z, w.w) * a0, false);
            while (kpt <= c.n_int && t + dt >= grid(kpt)) rec(kpt++);
            if (kpt > c.n_int) break;
            for (auto& e : m.net_cols[j]) x[e.first] += e.second;
            t += dt;
            step++;
            nsteps++;
            cnt.ssa++;
            continue;
        }
        const double tau1 = tau_bound(m, x.data(), a, crit, c.eps, f, nullptr, nullptr);
        if (tau1 * a0 < nssa) {
            // block of direct-method steps (model.cu:334-345)
            for (int q = 0; q < blk && kpt <= c.n_int; ++q) {
                if (q > 0) {
                    props(a0, a0c);
                    if (!(a0 > 0.0)) {
                        finish();
                        break;
                    }
                }
                const W4 w = philox(W4{0xFFFFFFFFu, step, r, (uint32_t)set << 8}, k0, k1);
                const int j = pick(uni52(w.z, w.w) * a0, false);
                const double dt = (f & F_COMPAT_TAU2) ? -std::log(uni23(w.x)) / a[j] : -std::log(uni23(w.x)) / a0;
                while (kpt <= c.n_int && t + dt >= grid(kpt)) rec(kpt++);
                if (kpt > c.n_int) {
                    if (score)
                        for (int mm = 0; mm < M; ++mm)
                            if (rate[mm] > 0.0) score[mm] -= a[mm] * (T - t) / rate[mm];
                    break;
                }
                if (score)
                    for (int mm = 0; mm < M; ++mm)
                        if (rate[mm] > 0.0) score[mm] += ((mm == j ? 1.0 : 0.0) - a[mm] * dt) / rate[mm];
                if (!(f & F_COMPAT_SSA))
                    for (auto& e : m.net_cols[j]) x[e.first] += e.second;
                t += dt;
                step++;
                nsteps++;
                cnt.ssa++;
                if (c.max_steps > 0 && nsteps >= c.max_steps) break;
            }
            continue;
        }
        // tau-leap with rejection and halving (CGP 2006 steps 3-5)
        const double tnext = grid(kpt);
        double tt = tau1, tau = 0.0;
        bool clamp = false;
        for (int attempt = 0;; ++attempt) {
            const W4 w = philox(W4{0xFFFFFFFFu, step, r, (uint32_t)set << 8}, k0, k1);
            int jc = -1;
            double tau2 = INFINITY;
            if (a0c > 0.0) {
                if (f & F_COMPAT_TAU2) {
                    jc = pick(uni52(w.z, w.w) * a0c, true);
                    tau2 = -std::log(uni23(w.x)) / a[jc];
                } else {
                    tau2 = -std::log(uni23(w.x)) / a0c;
                }
            }
            tau = std::min(tt, tau2);
            bool fire = tau2 < tt;
            clamp = false;
            if (t + tau >= tnext) {
                tau = tnext - t;
                clamp = true;
                fire = false;
            }
            if (fire && jc < 0) jc = pick(uni52(w.z, w.w) * a0c, true);
            if (!fire) jc = -1;
            W4 gw{0, 0, 0, 0};
            for (int j = 0; j < M; ++j) {
                if ((j & 3) == 0)
                    gw = philox(W4{(uint32_t)j >> 2, step, r, ((uint32_t)set << 8) | 0xFFu}, k0, k1);
                if (crit[j]) {
                    kk[j] = j == jc;
                } else {
                    Stream s{(uint32_t)j, step, r, (uint32_t)set << 8, k0, k1};
                    const uint32_t w0 = (j & 3) == 0 ? gw.x : (j & 3) == 1 ? gw.y : (j & 3) == 2 ? gw.z : gw.w;
                    kk[j] = (f & F_COMPAT_POISSON) ? poisson_ref(a[j] * tau, s) : poisson(a[j] * tau, w0, s);
                }
            }
            bool neg = false;
            for (int i = 0; i < N; ++i) {
                int64_t v = x[i];
                for (auto& e : m.net_rows[i]) v += (int64_t)e.second * kk[e.first];
                xn[i] = v;
                neg |= v < 0;
            }
            if (!neg) break;
            step++;
            cnt.rej++;
            tt *= 0.5;
            if (attempt >= 64) {
                finish();
                return;
            }
        }
        if (score)
            for (int j = 0; j < M; ++j)
                if (rate[j] > 0.0) score[j] += ((double)kk[j] - a[j] * tau) / rate[j];
        x.swap(xn);
        t = clamp ? tnext : t + tau;
        step++;
        nsteps++;
        cnt.leaps++;
        if (clamp) rec(kpt++);
    }
}

}  // namespace

extern "C" {

// Runs realizations r_begin..r_end-1 of every set; samples [S][R'][P][K],
// scores [S][R'][M] (R' = r_end - r_begin).  counters: leaps, ssa, rej, trunc.
int ora_simulate(const ora_model* m, const ora_cfg* c, int64_t* samples, double* scores, int64_t* counters) {
    const int S = std::max(1, c->S);
    const int64_t rb = c->r_begin, re = c->r_end > 0 ? c->r_end : c->R;
    const int64_t Rn = re - rb;
    const int P = c->n_int + 1;
    const int64_t total = Rn * S;
    const int nt = std::max(1, c->threads);
    std::atomic<int64_t> next{0};
    std::vector<Counters> cnt(nt);
    auto worker = [&](int tid) {
        for (;;) {
            const int64_t wi = next.fetch_add(1);
            if (wi >= total) break;
            const int set = (int)(wi / Rn);
            const int64_t rr = wi - (int64_t)set * Rn;
            run_one(*m, *c, set, (uint32_t)(rb + rr), samples + (size_t)wi * P * c->K,
                    scores ? scores + (size_t)wi * m->M : nullptr, cnt[tid]);
        }
    };
    std::vector<std::thread> th;
    for (int i = 1; i < nt; ++i) th.emplace_back(worker, i);
    worker(0);
    for (auto& x : th) x.join();
    if (counters) {
        counters[0] = counters[1] = counters[2] = counters[3] = 0;
        for (auto& k : cnt) {
            counters[0] += k.leaps;
            counters[1] += k.ssa;
            counters[2] += k.rej;
            counters[3] += k.trunc;
        }
    }
    return 0;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Workload models without the engine: the four seeded families of the
// benchmark configurations, built here so that a CPU-only caller (the
// reference arm of the benchmark) never loads the engine library.  The
// draws follow the engine's generator's documented order and mappings
// (std::mt19937_64; integers by 128-bit multiply-shift; reals from the top
// 53 bits; rates rounded to 9 significant digits; channel structures, then
// rates, then x0); tests check the two produce identical descriptions.
// Channel structures: the dimerisation decay of the reference's
// examples/dimer_decay.xml, the random toy network, the cyclic chain, and
// colloidal aggregation in the channel order of
// toy_system_gen/main.cpp:712-756.
// ---------------------------------------------------------------------------
#include <cstdio>
#include <cstdlib>
#include <map>
#include <random>

struct ora_gen {
    std::vector<int64_t> x0;
    std::vector<double> rate;
    std::vector<int32_t> col_ptr{0}, row_ind;
    std::vector<int8_t> stoich;
};

namespace {

struct GenDraw {
    std::mt19937_64 e;
    int64_t in(int64_t lo, int64_t hi) {  // uniform integer in [lo, hi]
        const unsigned __int128 n = (unsigned __int128)(uint64_t)(hi - lo) + 1u;
        return lo + (int64_t)(uint64_t)(((unsigned __int128)e() * n) >> 64);
    }
    double unit() { return (double)(e() >> 11) / 9007199254740992.0; }
};

double sig9(double v) {
    char s[48];
    std::snprintf(s, sizeof s, "%.9g", v);
    return std::strtod(s, nullptr);
}

// one channel: reactant and product species are distinct in every family,
// so the column is the species sorted ascending, reactants negative
void add_channel(ora_gen& g, const std::map<int, int>& entries) {
    for (const auto& e : entries) {
        g.row_ind.push_back(e.first);
        g.stoich.push_back((int8_t)e.second);
    }
    g.col_ptr.push_back((int32_t)g.row_ind.size());
}

}  // namespace

extern "C" {

// family: 1 dimer, 2 toy, 3 chain, 4 colloid (the engine's numbering).
// Returns nullptr for an unknown family or sizes the family rejects.
ora_gen* ora_gen_new(int family, int N, int M, int64_t x0_min, int64_t x0_max, double rate_min, double rate_max,
                     double rate_assoc, double rate_dissoc, uint64_t seed) {
    ora_gen* g = new ora_gen();
    GenDraw d{std::mt19937_64(seed)};
    if (family == 1) {
        const double c[4] = {1.0, 0.002, 0.5, 0.04};
        add_channel(*g, {{0, -1}});
        add_channel(*g, {{0, -2}, {1, 1}});
        add_channel(*g, {{0, 2}, {1, -1}});
        add_channel(*g, {{1, -1}, {2, 1}});
        g->rate.assign(c, c + 4);
        g->x0 = {x0_max, 0, 0};
    } else if (family == 2) {
        if (N < 4 || M < 1) {
            delete g;
            return nullptr;
        }
        std::vector<int> pool(N);
        for (int i = 0; i < N; ++i) pool[i] = i;
        // species from the not-yet-used pool first, then uniformly
        auto take = [&]() {
            if (pool.empty()) return (int)d.in(0, N - 1);
            const size_t k = (size_t)d.in(0, (int64_t)pool.size() - 1);
            std::swap(pool[k], pool.back());
            const int s = pool.back();
            pool.pop_back();
            return s;
        };
        auto take_new = [&](const std::map<int, int>& have) {
            for (int t = 0; t < 1000; ++t) {
                const int s = take();
                if (!have.count(s)) return s;
            }
            for (int s = 0; s < N; ++s)
                if (!have.count(s)) return s;
            return 0;
        };
        for (int j = 0; j < M; ++j) {
            std::map<int, int> col;
            const bool two = d.in(0, 1) == 1;
            const int a = take();
            if (!two) {
                col[a] = -(1 + (int)d.in(0, 1));
            } else {
                col[a] = -1;
                const int b = take_new(col);
                col[b] = -1;
            }
            const int np = 1 + (int)d.in(0, 1);
            for (int q = 0; q < np; ++q) {
                const int p = take_new(col);
                col[p] = 1 + (int)d.in(0, 1);
            }
            add_channel(*g, col);
        }
        const double l0 = std::log10(rate_min), l1 = std::log10(rate_max);
        for (int j = 0; j < M; ++j) g->rate.push_back(sig9(std::pow(10.0, l0 + (l1 - l0) * d.unit())));
        for (int i = 0; i < N; ++i) g->x0.push_back(d.in(x0_min, x0_max));
    } else if (family == 3) {
        if (N < 2) {
            delete g;
            return nullptr;
        }
        for (int i = 0; i < N; ++i) {
            add_channel(*g, {{i, -1}, {(i + 1) % N, 1}});
            g->rate.push_back(sig9(rate_min));
        }
        for (int i = 0; i < N; ++i) g->x0.push_back(d.in(x0_min, x0_max));
    } else if (family == 4) {
        if (N < 2) {
            delete g;
            return nullptr;
        }
        // S_k is index k-1: association n + m -> n + m (m >= n), then
        // dissociation p -> q + (p - q), q <= p / 2
        for (int n = 1; 2 * n <= N; ++n)
            for (int m = n; m <= N - n; ++m) {
                if (m == n) add_channel(*g, {{n - 1, -2}, {2 * n - 1, 1}});
                else add_channel(*g, {{n - 1, -1}, {m - 1, -1}, {n + m - 1, 1}});
                g->rate.push_back(sig9(rate_assoc));
            }
        for (int p = 1; p <= N; ++p)
            for (int q = 1; 2 * q <= p; ++q) {
                if (2 * q == p) add_channel(*g, {{p - 1, -1}, {q - 1, 2}});
                else add_channel(*g, {{p - 1, -1}, {q - 1, 1}, {p - q - 1, 1}});
                g->rate.push_back(sig9(rate_dissoc));
            }
        for (int i = 0; i < N; ++i) g->x0.push_back(d.in(x0_min, x0_max));
    } else {
        delete g;
        return nullptr;
    }
    return g;
}

void ora_gen_sizes(const ora_gen* g, int* N, int* M, int* nnz) {
    *N = (int)g->x0.size();
    *M = (int)g->rate.size();
    *nnz = (int)g->row_ind.size();
}

void ora_gen_copy(const ora_gen* g, int64_t* x0, double* rate, int32_t* col_ptr, int32_t* row_ind, int8_t* stoich) {
    std::copy(g->x0.begin(), g->x0.end(), x0);
    std::copy(g->rate.begin(), g->rate.end(), rate);
    std::copy(g->col_ptr.begin(), g->col_ptr.end(), col_ptr);
    std::copy(g->row_ind.begin(), g->row_ind.end(), row_ind);
    std::copy(g->stoich.begin(), g->stoich.end(), stoich);
}

void ora_gen_free(ora_gen* g) { delete g; }

}  // extern "C"
