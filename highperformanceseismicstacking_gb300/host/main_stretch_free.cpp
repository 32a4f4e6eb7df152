// single_host_stretch_free: CLI of the GB300 engine with the reference's flags
// (cuda/main/single_host/stretch_free.cpp).
#include "hpss_host.hpp"

int main(int argc, char *argv[]) {
    hpsshost::StretchFreeParser parser;
    hpsshost::SingleHostRunner runner(&parser);
    return runner.main(argc, const_cast<const char **>(argv));
}
