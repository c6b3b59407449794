// generator.cpp - seeded model generator (host C++).
//
// The reference's toy_system_gen (toy_system_gen/main.cpp) seeds its RNG from
// time() (:836-840) and emits channels from an unordered_set, so its models
// cannot be regenerated.  This generator is deterministic: std::mt19937_64
// (bit-exact by the C++ standard) with integer / real mappings written out
// here, and every rate rounded to 9 significant digits, so the same seed
// gives the same model on every host.
//
// Families:
//   dimer   : S1->0 (c1), 2S1->S2 (c2), S2->2S1 (c3), S2->S3 (c4)
//             (examples/dimer_decay.xml of the reference)
//   toy     : random network; each channel has 1-2 distinct reactants (one
//             reactant may have stoichiometry 2; two reactants have 1 each,
//             keeping order <= 2) and 1-2 distinct products (stoichiometry 1
//             or 2) different from the reactants.  Species are drawn from the
//             not-yet-used pool first, like GetNextInd (main.cpp:544-558).
//             Rates log-uniform in [rate_min, rate_max].
//   chain   : S_i -> S_(i+1 mod N), rate rate_min (main.cpp:694-710).
//   colloid : 2S_n -> S_2n and S_n + S_m -> S_(n+m) at rate_assoc,
//             S_p -> S_q + S_(p-q) (2S_q when q = p-q) at rate_dissoc, in the
//             order of GenColloidalAggregationReactionsList (main.cpp:712-756).
// Draw order: all channel structures, then all rates, then all x0.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>

#include "../csrc/tl_internal.h"

namespace tl {

namespace {

struct Rng {
    std::mt19937_64 e;
    explicit Rng(uint64_t s) : e(s) {}
    uint64_t bits() { return e(); }
    // integer uniform on [lo, hi] by multiply-shift
    int64_t uint(int64_t lo, int64_t hi) {
        const unsigned __int128 span = (unsigned __int128)(uint64_t)(hi - lo) + 1;
        return lo + (int64_t)(uint64_t)(((unsigned __int128)bits() * span) >> 64);
    }
    double real() { return (double)(bits() >> 11) * 1.1102230246251565e-16; }
};

double round9(double v) {
    char buf[64];
    snprintf(buf, sizeof buf, "%.9g", v);
    return strtod(buf, nullptr);
}

}  // namespace

tl_status generate_model(const tl_gen_params& g, HostModel& h, std::vector<Channel>& ch, std::string& err) {
    Rng rng(g.seed);
    ch.clear();
    int N = g.n_species;
    switch (g.family) {
    case TL_GEN_DIMER: {
        N = 3;
        const double c[4] = {1.0, 0.002, 0.5, 0.04};
        Channel a, b, d, e;
        a.reactants = {{0, 1}};
        b.reactants = {{0, 2}};
        b.products = {{1, 1}};
        d.reactants = {{1, 1}};
        d.products = {{0, 2}};
        e.reactants = {{1, 1}};
        e.products = {{2, 1}};
        a.rate = c[0];
        b.rate = c[1];
        d.rate = c[2];
        e.rate = c[3];
        ch = {a, b, d, e};
        h.N = N;
        h.x0 = {g.x0_max, 0, 0};
        break;
    }
    case TL_GEN_TOY: {
        const int M = g.n_channels;
        if (N < 4 || M < 1) {
            err = "toy family needs n_species >= 4 and n_channels >= 1";
            return TL_ERR_INVALID_ARGUMENT;
        }
        std::vector<int> unused((size_t)N);
        for (int i = 0; i < N; ++i) unused[(size_t)i] = i;
        auto next = [&]() -> int {
            if (unused.empty()) return (int)rng.uint(0, N - 1);
            const size_t k = (size_t)rng.uint(0, (int64_t)unused.size() - 1);
            std::swap(unused[k], unused.back());
            const int s = unused.back();
            unused.pop_back();
            return s;
        };
        auto distinct = [&](const std::vector<int>& avoid) -> int {
            for (int t = 0; t < 1000; ++t) {
                const int s = next();
                bool clash = false;
                for (int a : avoid) clash |= (a == s);
                if (!clash) return s;
            }
            for (int s = 0; s < N; ++s) {
                bool clash = false;
                for (int a : avoid) clash |= (a == s);
                if (!clash) return s;
            }
            return 0;
        };
        ch.resize((size_t)M);
        for (int j = 0; j < M; ++j) {
            Channel& c = ch[(size_t)j];
            std::vector<int> used;
            const int nr = 1 + (int)rng.uint(0, 1);
            const int r1 = next();
            used.push_back(r1);
            if (nr == 1) {
                c.reactants.push_back({r1, 1 + (int)rng.uint(0, 1)});
            } else {
                const int r2 = distinct(used);
                used.push_back(r2);
                c.reactants.push_back({r1, 1});
                c.reactants.push_back({r2, 1});
            }
            const int np = 1 + (int)rng.uint(0, 1);
            for (int q = 0; q < np; ++q) {
                const int pr = distinct(used);
                used.push_back(pr);
                c.products.push_back({pr, 1 + (int)rng.uint(0, 1)});
            }
        }
        const double lo = std::log10(g.rate_min), hi = std::log10(g.rate_max);
        for (int j = 0; j < M; ++j) ch[(size_t)j].rate = round9(std::pow(10.0, lo + (hi - lo) * rng.real()));
        h.N = N;
        h.x0.resize((size_t)N);
        for (int i = 0; i < N; ++i) h.x0[(size_t)i] = rng.uint(g.x0_min, g.x0_max);
        break;
    }
    case TL_GEN_CHAIN: {
        if (N < 2) {
            err = "chain family needs n_species >= 2";
            return TL_ERR_INVALID_ARGUMENT;
        }
        ch.resize((size_t)N);
        for (int i = 0; i < N; ++i) {
            ch[(size_t)i].reactants = {{i, 1}};
            ch[(size_t)i].products = {{(i + 1) % N, 1}};
            ch[(size_t)i].rate = round9(g.rate_min);
        }
        h.N = N;
        h.x0.resize((size_t)N);
        for (int i = 0; i < N; ++i) h.x0[(size_t)i] = rng.uint(g.x0_min, g.x0_max);
        break;
    }
    case TL_GEN_COLLOID: {
        if (N < 2) {
            err = "colloid family needs n_species >= 2";
            return TL_ERR_INVALID_ARGUMENT;
        }
        // species S1..SN are indices 0..N-1
        for (int n = 1; n <= N / 2; ++n) {
            Channel c;
            c.reactants = {{n - 1, 2}};
            c.products = {{2 * n - 1, 1}};
            c.rate = round9(g.rate_assoc);
            ch.push_back(c);
            for (int m = n + 1; m <= N - n; ++m) {
                Channel d;
                d.reactants = {{n - 1, 1}, {m - 1, 1}};
                d.products = {{m + n - 1, 1}};
                d.rate = round9(g.rate_assoc);
                ch.push_back(d);
            }
        }
        for (int p = 1; p <= N; ++p)
            for (int q = 1; q <= p / 2; ++q) {
                Channel c;
                c.reactants = {{p - 1, 1}};
                if (q == p - q) c.products = {{q - 1, 2}};
                else c.products = {{q - 1, 1}, {p - q - 1, 1}};
                c.rate = round9(g.rate_dissoc);
                ch.push_back(c);
            }
        h.N = N;
        h.x0.resize((size_t)N);
        for (int i = 0; i < N; ++i) h.x0[(size_t)i] = rng.uint(g.x0_min, g.x0_max);
        break;
    }
    default:
        err = "unknown generator family";
        return TL_ERR_INVALID_ARGUMENT;
    }
    h.names.resize((size_t)h.N);
    for (int i = 0; i < h.N; ++i) h.names[(size_t)i] = "S" + std::to_string(i + 1);
    h.pop_bits = g.pop_bits;
    channels_to_raw(ch, h);
    return TL_OK;
}

}  // namespace tl
