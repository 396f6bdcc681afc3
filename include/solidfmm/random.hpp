// Deterministic uniform random reals in [min, max) with the interface of the
// reference's random_real<real> (solidfmm/random.hpp:28-50): default-seeded
// engine, so every instance yields the same sequence.
#ifndef SOLIDFMM_RANDOM_HPP
#define SOLIDFMM_RANDOM_HPP

#include <memory>
#include <random>

namespace solidfmm
{

template <typename real>
class random_real
{
public:
    random_real(real min, real max) : st(std::make_shared<state>(min, max)) {}
    real operator()() const { return st->dist(st->engine); }

private:
    struct state {
        state(real lo, real hi) : dist(lo, hi) {}
        std::default_random_engine engine;
        std::uniform_real_distribution<double> dist;
    };
    std::shared_ptr<state> st;
};

}  // namespace solidfmm

#endif
