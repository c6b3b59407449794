// gpu_model.h - a drop-in `Model` for the reference's tau_leaping.cpp over the
// C ABI of libtl.so (include/tl.h).  The binding a maintainer of the reference
// (CSSL-UWM/tau_leaping) adds in place of tau_leaping/model.h:20-98: same
// names, argument meanings and error behaviour (a failing ReadXML throws
// std::runtime_error, StochKitReader.cpp:29).  Header-only; link with -ltl.
#pragma once
#include <stdexcept>
#include <string>
#include <vector>
#include "tl.h"

class Model {
  public:
    static Model* ReadXML(const char* fn, std::vector<std::string>& names) {
        tl_model* h = nullptr;
        tl_status s = tl_model_from_stochkit(fn, 0, &h);
        if (s != TL_OK) throw std::runtime_error(std::string("Model::ReadXML: ") + tl_last_error());
        tl_model_info info;
        tl_model_get_info(h, &info);
        names.clear();
        for (int i = 0; i < info.n_species; ++i) names.push_back(tl_model_species_name(h, i));
        return new Model(h, info);
    }
    ~Model() { tl_model_destroy(h_); }
    int ChannelsCount() const { return info_.n_channels; }
    int ReactantsCount() const { return info_.n_species; }
    // Runs all n realizations at once (the reference loops PerformCalc per
    // realization).  Fills mean/stddev [intervals+1][tracked].
    void PerformCalcAll(float endTau, float eps, const std::vector<char>& r2Track, int n, int intervals,
                        int maxIterations, unsigned long long seed, std::vector<double>& mean,
                        std::vector<double>& stddev, std::vector<double>& times) {
        std::vector<int32_t> tracked;
        for (int i = 0; i < (int)r2Track.size(); ++i)
            if (r2Track[i]) tracked.push_back(i);
        tl_run_cfg c;
        tl_run_cfg_init(&c);
        c.t_final = endTau;
        c.eps = eps;
        c.n_realizations = n;
        c.seed = seed;
        c.n_intervals = intervals;
        c.n_tracked = (int32_t)tracked.size();
        c.tracked = tracked.data();
        c.max_steps = maxIterations == 0x7fffffff ? 0 : maxIterations;
        const size_t P = (size_t)intervals + 1;
        mean.resize(P * tracked.size());
        stddev.resize(P * tracked.size());
        times.resize(P);
        tl_result r{};
        r.mean = mean.data();
        r.stddev = stddev.data();
        r.times = times.data();
        tl_status s = tl_simulate(h_, &c, &r);
        if (s != TL_OK && s != TL_ERR_STEP_CAP) throw std::runtime_error(tl_last_error());
    }
  private:
    Model(tl_model* h, tl_model_info i) : h_(h), info_(i) {}
    tl_model* h_;
    tl_model_info info_;
};
