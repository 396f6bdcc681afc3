// Wall-clock timer with the interface of the reference's stopwatch<real>
// (solidfmm/stopwatch.hpp:28-56), used by benchmark programs.
#ifndef SOLIDFMM_STOPWATCH_HPP
#define SOLIDFMM_STOPWATCH_HPP

#include <chrono>

namespace solidfmm
{

template <typename real>
class stopwatch
{
public:
    void reset() noexcept { start = std::chrono::steady_clock::now(); }
    real elapsed() const noexcept
    {
        return std::chrono::duration<real>(std::chrono::steady_clock::now() - start).count();
    }

private:
    std::chrono::steady_clock::time_point start{std::chrono::steady_clock::now()};
};

}  // namespace solidfmm

#endif
