// tl_gen.cpp - seeded model generator CLI (replaces toy_system_gen, whose
// models depend on time(); toy_system_gen/main.cpp:240-407 for the flags).
//
//   tl_gen [-r species] [-c channels] [-mnp min_pop] [-mxp max_pop]
//          [-w | -s | --dimer] [--seed S] [-o file.xml]
//
//   default : random toy network (-r 128 -c 256 -mnp 0 -mxp 10000, seed 7)
//   -w      : weakly coupled cyclic chain (seed 11)
//   -s      : strongly coupled colloidal aggregation, N^2/2 channels (seed 13)
//   --dimer : dimerisation decay with S1 = -mxp
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>

#include "../../include/tl.h"

int main(int argc, char** argv) {
    int family = TL_GEN_TOY;
    for (int i = 1; i < argc; ++i) {
        if (!strcmp(argv[i], "-w")) family = TL_GEN_CHAIN;
        if (!strcmp(argv[i], "-s")) family = TL_GEN_COLLOID;
        if (!strcmp(argv[i], "--dimer")) family = TL_GEN_DIMER;
    }
    tl_gen_params g;
    tl_gen_params_init(&g, family);
    std::string out = "/dev/stdout";
    for (int i = 1; i < argc; ++i) {
        const std::string k = argv[i];
        const bool has = i + 1 < argc;
        if (k == "-r" && has) g.n_species = atoi(argv[++i]);
        else if (k == "-c" && has) g.n_channels = atoi(argv[++i]);
        else if (k == "-mnp" && has) g.x0_min = atoll(argv[++i]);
        else if (k == "-mxp" && has) g.x0_max = atoll(argv[++i]);
        else if (k == "--seed" && has) g.seed = strtoull(argv[++i], nullptr, 10);
        else if (k == "-o" && has) out = argv[++i];
        else if (k == "-w" || k == "-s" || k == "--dimer") continue;
        else {
            std::cerr << "usage: tl_gen [-r N] [-c M] [-mnp min] [-mxp max] [-w|-s|--dimer] [--seed S] [-o file]\n";
            return 2;
        }
    }
    if (family == TL_GEN_DIMER) g.x0_min = g.x0_max;
    tl_model* m = nullptr;
    tl_status s = tl_model_generate(&g, &m);
    if (s == TL_OK) s = tl_model_write_stochkit(m, out.c_str());
    if (s != TL_OK) {
        std::cerr << "tl_gen: " << tl_status_str(s) << " (" << tl_last_error() << ")\n";
        return 1;
    }
    tl_model_destroy(m);
    return 0;
}
