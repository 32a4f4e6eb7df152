// single_host_linear_search: CLI of the GB300 engine with the reference's flags
// (cuda/main/single_host/linear_search.cpp).
#include "hpss_host.hpp"

int main(int argc, char *argv[]) {
    hpsshost::LinearSearchParser parser;
    hpsshost::SingleHostRunner runner(&parser);
    return runner.main(argc, const_cast<const char **>(argv));
}
