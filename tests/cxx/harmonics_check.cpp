// The drop-in solidfmm::harmonics::R/S/dR/dS (solidfmm_gb300/cxx/harmonics.cpp)
// evaluated through the public C++ API, for comparison with the reference's
// own values (solidfmm/harmonics.cpp:32-349, kept as golden vectors).
//
// usage: harmonics_check P x y z [x y z ...]
// writes, per point, R (P(P+1) doubles), S, dR (3 P(P+1)), dS as raw binary
// doubles to stdout, in that order.
#include <cstdio>
#include <cstdlib>

#include <solidfmm/harmonics.hpp>
#include <solidfmm/solid.hpp>

using namespace solidfmm;

static void put(const solid<double> &s)
{
    const size_t cnt = s.order() * (s.order() + 1) * s.dimension();
    std::fwrite(s.memptr(), sizeof(double), cnt, stdout);
}

int main(int argc, char **argv)
{
    if (argc < 5 || (argc - 2) % 3) {
        std::fprintf(stderr, "usage: %s P x y z [x y z ...]\n", argv[0]);
        return 2;
    }
    const size_t P = std::strtoul(argv[1], nullptr, 10);
    for (int a = 2; a + 2 < argc; a += 3) {
        const double x = std::strtod(argv[a], nullptr), y = std::strtod(argv[a + 1], nullptr),
                     z = std::strtod(argv[a + 2], nullptr);
        put(harmonics::R<double>(P, x, y, z));
        put(harmonics::S<double>(P, x, y, z));
        put(harmonics::dR<double>(P, x, y, z));
        put(harmonics::dS<double>(P, x, y, z));
    }
    return 0;
}
