// driver.cpp - runs the reference's own Model API (tau_leaping/model.h:20-98)
// host-only and prints per-realization samples on the statistics grid, as
// built by the reference's AllStat2StepStat (statistics.cpp:15-64).
// Project-written test infrastructure; replaces tau_leaping.cpp's main so
// that logging is on (the shipped main hard-codes it off, tau_leaping.cpp:30).
//
//   ref_driver <model.xml> <t_final> <realizations> <intervals> <eps> <seed> <species...>
// prints: "#time <seconds> steps <logged steps>" then per grid time
//         "t <t>" followed by one line per realization with the tracked values.
#include <cstdio>
#include <cstdlib>
#include <sys/time.h>

#include "model.h"
#include "statistics.h"

std::string g_logFN = "stat.txt";
bool g_doLogging = true;
cusparseHandle_t g_handle;

int main(int argc, char** argv) {
    if (argc < 8) {
        fprintf(stderr, "usage: ref_driver model.xml t_final n intervals eps seed species...\n");
        return 2;
    }
    const float T = (float)atof(argv[2]);
    const int n = atoi(argv[3]);
    const int intervals = atoi(argv[4]);
    const float eps = (float)atof(argv[5]);
    srand((unsigned)atoi(argv[6]));
    std::vector<std::string> names;
    Model* m0 = Model::ReadXML(argv[1], names);
    std::vector<char> track(m0->ReactantsCount(), 0);
    for (int a = 7; a < argc; ++a)
        for (size_t i = 0; i < names.size(); ++i)
            if (names[i] == argv[a]) track[i] = 1;
    std::vector<stat_t> stats(n);
    timeval t0, t1;
    gettimeofday(&t0, nullptr);
    long steps = 0;
    // like tau_leaping.cpp:127-150: clone every realization first, then run
    std::vector<Model*> ms(1, m0);
    for (int r = 1; r < n; ++r) ms.push_back(m0->Clone());
    for (int r = 0; r < n; ++r) ms[r]->InitSeeds();
    for (int r = 0; r < n; ++r) {
        ms[r]->PerformCalc(T, eps, track, stats[r], 1 << 30);
        steps += (long)stats[r].size();
        if (r) delete ms[r];
    }
    gettimeofday(&t1, nullptr);
    const double secs = (t1.tv_sec - t0.tv_sec) + 1e-6 * (t1.tv_usec - t0.tv_usec);
    printf("#time %.6f steps %ld\n", secs, steps);
    // Per realization, the value at grid time t is interpolated between the
    // logged states around t with the formula of AllStat2StepStat
    // (statistics.cpp:40-56); past the last logged state (the final step is
    // never logged) the last state is held.  Unlike AllStat2StepStat this
    // does not stop the whole grid when one realization ends early.
    const double dt = (double)T / intervals;
    for (int k = 0; k < intervals; ++k) {
        const double t = dt * k;
        printf("t %.9g\n", t);
        for (int r = 0; r < n; ++r) {
            const stat_t& st = stats[r];
            auto it = st.upper_bound(t);
            std::vector<double> v;
            if (it == st.end()) {
                for (int x : st.rbegin()->second) v.push_back(x);
            } else {
                auto pv = it;
                --pv;
                const double sh = (t - pv->first) / (it->first - pv->first);
                for (size_t q = 0; q < it->second.size(); ++q)
                    v.push_back(pv->second[q] + (it->second[q] - pv->second[q]) * sh);
            }
            for (size_t q = 0; q < v.size(); ++q) printf("%.6f%c", v[q], q + 1 < v.size() ? ' ' : '\n');
        }
    }
    delete m0;
    return 0;
}
