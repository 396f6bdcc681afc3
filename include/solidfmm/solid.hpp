// solidfmm-gb300 drop-in: solid-harmonic expansions.
//
// Same interface and memory layout as the reference's solid<real>
// (solidfmm/solid.hpp:29-77): an expansion of order P with dim components owns
// dim*P*(P+1) reals from malloc; component d, degree n: real parts
// re(n,0..n) at d*P(P+1) + n(n+1), imaginary parts at d*P(P+1) + (n+1)^2.
// Negative m is implicit, C_n^{-m} = (-1)^m conj(C_n^m).
#ifndef SOLIDFMM_SOLID_HPP
#define SOLIDFMM_SOLID_HPP

#include <cstddef>

namespace solidfmm
{

template <typename real>
class solid
{
public:
    solid() = default;
    solid(size_t P, size_t dim = 1);
    solid(const solid &rhs);
    solid(solid &&rhs) noexcept;
    solid &operator=(const solid &rhs);
    solid &operator=(solid &&rhs) noexcept;
    ~solid();

    void resize(size_t P, size_t dim = 1);
    void reinit(size_t P, size_t dim = 1);
    void zeros() noexcept;

    const real &re(size_t n, size_t m, size_t d = 0) const noexcept { return data[ridx(n, m, d)]; }
    real &re(size_t n, size_t m, size_t d = 0) noexcept { return data[ridx(n, m, d)]; }
    const real &im(size_t n, size_t m, size_t d = 0) const noexcept { return data[iidx(n, m, d)]; }
    real &im(size_t n, size_t m, size_t d = 0) noexcept { return data[iidx(n, m, d)]; }

    size_t order() const noexcept { return P; }
    size_t dimension() const noexcept { return dim; }

    const real *memptr() const noexcept { return data; }
    real *memptr() noexcept { return data; }

private:
    size_t num_reals() const noexcept { return dim * P * (P + 1); }
    size_t ridx(size_t n, size_t m, size_t d) const noexcept { return d * P * (P + 1) + n * (n + 1) + m; }
    size_t iidx(size_t n, size_t m, size_t d) const noexcept { return d * P * (P + 1) + (n + 1) * (n + 1) + m; }

    size_t P{0};
    size_t dim{1};
    real *data{nullptr};
};

extern template class solid<float>;
extern template class solid<double>;

// result[da*B.dimension()+db] = sum_n sum_{m=-n..n} A_n^m conj(B_n^m) over the common degrees
void dot(const solid<float> &A, const solid<float> &B, float *result) noexcept;
void dot(const solid<double> &A, const solid<double> &B, double *result) noexcept;

// B += fac * A (fac per component for the pointer overloads); orders and dimensions must match
void fmadd(const float fac, const solid<float> &A, solid<float> &B);
void fmadd(const float *fac, const solid<float> &A, solid<float> &B);
void fmadd(const double fac, const solid<double> &A, solid<double> &B);
void fmadd(const double *fac, const solid<double> &A, solid<double> &B);

}  // namespace solidfmm

#endif
