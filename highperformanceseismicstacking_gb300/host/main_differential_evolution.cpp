// single_host_differential_evolution: CLI of the GB300 engine with the reference's flags
// (cuda/main/single_host/differential_evolution.cpp).
#include "hpss_host.hpp"

int main(int argc, char *argv[]) {
    hpsshost::DifferentialEvolutionParser parser;
    hpsshost::SingleHostRunner runner(&parser);
    return runner.main(argc, const_cast<const char **>(argv));
}
