// tl_cli.cpp - drop-in replacement of the reference's tau_leaping executable
// (tau_leaping/tau_leaping.cpp:40-190, cl_parser.cpp:19-130), written
// against the C ABI only.
//
//   tl_cli -f model.xml -t T -n R -r S1 S5 [-e eps] [-i intervals]
//          [-a max_steps] [-b name] [-d device]
//          [--seed S] [--compat] [--variant auto|thread|lanes2|lanes4|lanes8|lanes16|warp|cta|plain]
//          [--autotune] [--pop64] [--samples file]
//
// Writes mean_<name>.txt and stddev_<name>.txt, one line per grid time
// "t v1 v2 ..." for the tracked species in species order, like StatToFile
// (tau_leaping/statistics.cpp:89-111).  Differences from the reference,
// each deliberate: -d selects the device (tau_leaping.cpp:48 ignores it),
// the t_final row is written (statistics.cpp:41-44 drops it), the state on
// the grid is the simulated state at the grid time (no interpolation), and
// runs are reproducible from --seed.
#include <cerrno>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <set>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/tl.h"

namespace {

struct Args {
    std::string file;
    double t_final = 0.0;
    double eps = 0.03;
    long long n = 1;
    std::vector<std::string> track;
    std::string log_name;  // -b: ".txt" appended like cl_parser.cpp:63
    int intervals = 1;
    long long max_steps = 0;
    int device = 0;
    unsigned long long seed = 1;
    bool compat = false;
    bool autotune = false;
    int variant = TL_VARIANT_AUTO;
    int pop_bits = 0;
    std::string samples_file;
};

void usage() {
    std::cerr << "usage: tl_cli -f <model.xml> -t <t_final> -n <realizations> -r <species ...|all>\n"
                 "              [-e eps] [-i intervals] [-a max_steps] [-b name] [-d device]\n"
                 "              [--seed S] [--compat] [--variant auto|thread|lanes2|lanes4|lanes8|lanes16|warp|cta|plain]\n"
                 "              [--autotune] [--pop64] [--samples file]\n";
}

bool parse(int argc, char** argv, Args& a) {
    for (int i = 1; i < argc; ++i) {
        const std::string k = argv[i];
        auto need = [&](const char* what) -> const char* {
            if (i + 1 >= argc) {
                std::cerr << "missing value for " << what << "\n";
                return nullptr;
            }
            return argv[++i];
        };
        const char* v = nullptr;
        if (k == "-f") {
            if (!(v = need("-f"))) return false;
            a.file = v;
        } else if (k == "-t") {
            if (!(v = need("-t"))) return false;
            a.t_final = atof(v);
        } else if (k == "-n") {
            if (!(v = need("-n"))) return false;
            a.n = atoll(v);
        } else if (k == "-e") {
            if (!(v = need("-e"))) return false;
            a.eps = atof(v);
        } else if (k == "-i") {
            if (!(v = need("-i"))) return false;
            a.intervals = atoi(v);
        } else if (k == "-a") {
            if (!(v = need("-a"))) return false;
            a.max_steps = atoll(v);
        } else if (k == "-d") {
            if (!(v = need("-d"))) return false;
            a.device = atoi(v);
        } else if (k == "-b") {
            if (!(v = need("-b"))) return false;
            a.log_name = std::string(v) + ".txt";
        } else if (k == "-r") {
            // names up to the next option, split on blanks and commas
            while (i + 1 < argc && (argv[i + 1][0] != '-' || strcmp(argv[i + 1], "-1") == 0)) {
                std::string s = argv[++i];
                for (char& c : s)
                    if (c == ',') c = ' ';
                std::istringstream is(s);
                std::string t;
                while (is >> t) a.track.push_back(t);
            }
        } else if (k == "--seed") {
            if (!(v = need("--seed"))) return false;
            a.seed = strtoull(v, nullptr, 10);
        } else if (k == "--compat") {
            a.compat = true;
        } else if (k == "--autotune") {
            a.autotune = true;
        } else if (k == "--pop64") {
            a.pop_bits = 64;
        } else if (k == "--samples") {
            if (!(v = need("--samples"))) return false;
            a.samples_file = v;
        } else if (k == "--variant") {
            if (!(v = need("--variant"))) return false;
            const std::string s = v;
            a.variant = s == "thread" ? TL_VARIANT_THREAD : s == "warp" ? TL_VARIANT_WARP
                      : s == "cta" ? TL_VARIANT_CTA : s == "plain" ? TL_VARIANT_PLAIN
                      : s == "lanes2" ? TL_VARIANT_LANES2 : s == "lanes4" ? TL_VARIANT_LANES4
                      : s == "lanes8" ? TL_VARIANT_LANES8 : s == "lanes16" ? TL_VARIANT_LANES16 : TL_VARIANT_AUTO;
        } else if (k == "-h" || k == "--help") {
            usage();
            exit(0);
        } else {
            std::cerr << "unknown option " << k << "\n";
            return false;
        }
    }
    if (a.file.empty() || !(a.t_final > 0.0) || a.n < 1) {
        std::cerr << "need -f <file>, -t <t_final> > 0 and -n >= 1\n";
        return false;
    }
    return true;
}

int fail(const char* what, tl_status s) {
    std::cerr << what << ": " << tl_status_str(s) << " (" << tl_last_error() << ")\n";
    return 1;
}

}  // namespace

int main(int argc, char** argv) {
    Args a;
    if (!parse(argc, argv, a)) {
        usage();
        return 2;
    }
    std::cout << "Processing file " << a.file << "\nFinish time: " << a.t_final << "\nRunning " << a.n
              << " system(s) in parallel\nLogging intervals: " << a.intervals << "\nIterations limit: "
              << (a.max_steps ? std::to_string(a.max_steps) : std::string("none")) << "\n";
    tl_model* m = nullptr;
    tl_status s = tl_model_from_stochkit(a.file.c_str(), a.pop_bits, &m);
    if (s != TL_OK) return fail("reading model", s);
    tl_model_info info;
    tl_model_get_info(m, &info);
    std::vector<int32_t> tracked;
    const bool all = a.track.size() == 1 && (a.track[0] == "all" || a.track[0] == "-1");
    std::set<std::string> want(a.track.begin(), a.track.end());
    for (int i = 0; i < info.n_species; ++i)
        if (all || want.count(tl_model_species_name(m, i))) tracked.push_back(i);
    for (const auto& t : a.track)
        if (!all && tl_model_species_index(m, t.c_str()) < 0)
            std::cerr << "warning: species " << t << " not in the model\n";
    if (tracked.empty()) {
        std::cerr << "no species to track (-r)\n";
        tl_model_destroy(m);
        return 2;
    }
    std::cout << "Tracking reactants:\n";
    for (int i : tracked) std::cout << tl_model_species_name(m, i) << "\n";
    s = tl_set_device(a.device);
    if (s != TL_OK) return fail("selecting device", s);

    tl_run_cfg cfg;
    tl_run_cfg_init(&cfg);
    cfg.t_final = a.t_final;
    cfg.eps = a.eps;
    cfg.n_realizations = a.n;
    cfg.seed = a.seed;
    cfg.n_intervals = a.intervals;
    cfg.n_tracked = (int32_t)tracked.size();
    cfg.tracked = tracked.data();
    cfg.variant = a.variant;
    cfg.max_steps = a.max_steps;
    if (a.compat) cfg.flags |= TL_FLAG_COMPAT_REFERENCE;
    if (a.autotune) cfg.flags |= TL_FLAG_AUTOTUNE_MEASURE;
    const size_t P = (size_t)a.intervals + 1, K = tracked.size();
    std::vector<double> times(P), mean(P * K), sd(P * K);
    std::vector<int64_t> samples;
    tl_result res{};
    res.times = times.data();
    res.mean = mean.data();
    res.stddev = sd.data();
    if (!a.samples_file.empty()) {
        cfg.flags |= TL_FLAG_KEEP_SAMPLES;
        samples.resize((size_t)a.n * P * K);
        res.samples = samples.data();
    }
    const auto t0 = std::chrono::steady_clock::now();
    s = tl_simulate(m, &cfg, &res);
    const double took = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (s == TL_ERR_STEP_CAP) std::cerr << "warning: " << res.truncated << " realization(s) hit the -a limit\n";
    else if (s != TL_OK) return fail("simulation", s);
    std::cout << "It took " << took << " s to complete calculations\n"
              << "Device time, s: " << res.kernel_ms / 1e3 << "\n"
              << "Tau-leaps: " << res.leaps << "  direct-method steps: " << res.ssa_steps
              << "  rejected leaps: " << res.rejections << "\n";
    std::ofstream fm("mean_" + a.log_name), fs("stddev_" + a.log_name);
    if (!fm || !fs) {
        std::cerr << "can not write mean_/stddev_ files\n";
        return 1;
    }
    for (size_t k = 0; k < P; ++k) {
        fm << times[k] << " ";
        fs << times[k] << " ";
        for (size_t q = 0; q < K; ++q) {
            fm << mean[k * K + q] << " ";
            fs << sd[k * K + q] << " ";
        }
        fm << "\n";
        fs << "\n";
    }
    if (!a.samples_file.empty()) {
        std::ofstream f(a.samples_file);
        for (long long r = 0; r < a.n; ++r) {
            for (size_t q = 0; q < K; ++q) f << samples[((size_t)r * P + (P - 1)) * K + q] << (q + 1 < K ? " " : "\n");
        }
    }
    std::cout << "Statistics written to mean_" << a.log_name << " and stddev_" << a.log_name << "\n";
    tl_model_destroy(m);
    return 0;
}
