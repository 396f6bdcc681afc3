// solidfmm-gb300 drop-in: minimal bounding spheres.
//
// Same interface as the reference's solidfmm/sphere.hpp:29-42: a sphere is a
// centre and a radius; bounding_sphere returns the smallest sphere that
// contains n points, or a range of spheres.  Used by FMM codes to size boxes
// for adaptive acceptance criteria; host code (no GPU work).
// Errors: an empty input throws std::logic_error; a degenerate configuration
// the algorithm cannot resolve in floating point throws std::runtime_error.
#ifndef SOLIDFMM_SPHERE_HPP
#define SOLIDFMM_SPHERE_HPP

#include <cstddef>

namespace solidfmm
{

template <typename real>
struct sphere
{
    real x{0}, y{0}, z{0};  // centre
    real r{0};              // radius
};

extern template struct sphere<float>;
extern template struct sphere<double>;

sphere<float> bounding_sphere(size_t n, const float *x, const float *y, const float *z);
sphere<double> bounding_sphere(size_t n, const double *x, const double *y, const double *z);

sphere<float> bounding_sphere(const sphere<float> *begin, const sphere<float> *end);
sphere<double> bounding_sphere(const sphere<double> *begin, const sphere<double> *end);

}  // namespace solidfmm

#endif
