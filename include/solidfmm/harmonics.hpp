// solidfmm-gb300 drop-in: regular (R) and singular (S) solid harmonics and
// their gradients (dR, dS, three components), same interface as the
// reference's solidfmm/harmonics.hpp:33-46.
#ifndef SOLIDFMM_HARMONICS_HPP
#define SOLIDFMM_HARMONICS_HPP

#include <cstddef>

namespace solidfmm
{

template <typename real> class solid;

namespace harmonics
{

template <typename real> solid<real> R(size_t P, real x, real y, real z);
template <typename real> solid<real> S(size_t P, real x, real y, real z);
template <typename real> solid<real> dR(size_t P, real x, real y, real z);
template <typename real> solid<real> dS(size_t P, real x, real y, real z);

template <> solid<float> R(size_t P, float x, float y, float z);
template <> solid<float> S(size_t P, float x, float y, float z);
template <> solid<float> dR(size_t P, float x, float y, float z);
template <> solid<float> dS(size_t P, float x, float y, float z);

template <> solid<double> R(size_t P, double x, double y, double z);
template <> solid<double> S(size_t P, double x, double y, double z);
template <> solid<double> dR(size_t P, double x, double y, double z);
template <> solid<double> dS(size_t P, double x, double y, double z);

}  // namespace harmonics

}  // namespace solidfmm

#endif
