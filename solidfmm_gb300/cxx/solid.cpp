// solid<real>, dot and fmadd for the drop-in API (semantics of the
// reference's solidfmm/solid.cpp:41-238).
#include <solidfmm/solid.hpp>

#include <cstdlib>
#include <cstring>
#include <new>
#include <stdexcept>
#include <utility>

namespace solidfmm
{

template <typename real>
solid<real>::solid(size_t P_, size_t dim_)
{
    resize(P_, dim_);
    zeros();
}

template <typename real>
solid<real>::solid(const solid &rhs)
{
    resize(rhs.P, rhs.dim);
    if (num_reals()) std::memcpy(data, rhs.data, sizeof(real) * num_reals());
}

template <typename real>
solid<real>::solid(solid &&rhs) noexcept : P{rhs.P}, dim{rhs.dim}, data{rhs.data}
{
    rhs.P = 0;
    rhs.dim = 1;
    rhs.data = nullptr;
}

template <typename real>
solid<real> &solid<real>::operator=(const solid &rhs)
{
    if (this != &rhs) {
        resize(rhs.P, rhs.dim);
        if (num_reals()) std::memcpy(data, rhs.data, sizeof(real) * num_reals());
    }
    return *this;
}

template <typename real>
solid<real> &solid<real>::operator=(solid &&rhs) noexcept
{
    std::swap(P, rhs.P);
    std::swap(dim, rhs.dim);
    std::swap(data, rhs.data);
    return *this;
}

template <typename real>
solid<real>::~solid()
{
    std::free(data);
}

template <typename real>
void solid<real>::resize(size_t P_, size_t dim_)
{
    size_t want = sizeof(real) * P_ * (P_ + 1) * dim_;
    if (want != sizeof(real) * num_reals()) {
        if (want == 0) {
            std::free(data);
            data = nullptr;
        } else {
            void *p = std::realloc(data, want);
            if (!p) throw std::bad_alloc{};
            data = static_cast<real *>(p);
        }
    }
    P = P_;
    dim = dim_;
}

template <typename real>
void solid<real>::reinit(size_t P_, size_t dim_)
{
    resize(P_, dim_);
    zeros();
}

template <typename real>
void solid<real>::zeros() noexcept
{
    if (num_reals()) std::memset(data, 0, sizeof(real) * num_reals());
}

template class solid<float>;
template class solid<double>;

namespace
{

template <typename real>
void dot_t(const solid<real> &A, const solid<real> &B, real *result) noexcept
{
    const size_t PA = A.order(), PB = B.order(), P = PA < PB ? PA : PB;
    const size_t SA = PA * (PA + 1), SB = PB * (PB + 1);
    for (size_t da = 0; da < A.dimension(); ++da)
        for (size_t db = 0; db < B.dimension(); ++db) {
            const real *a = A.memptr() + da * SA;
            const real *b = B.memptr() + db * SB;
            real all = 0, m0 = 0;
            for (size_t k = 0; k < P * (P + 1); ++k) all += a[k] * b[k];
            for (size_t n = 0; n < P; ++n) m0 += a[n * (n + 1)] * b[n * (n + 1)];
            // m and -m contribute equally; m = 0 once
            *result++ = real(2) * all - m0;
        }
}

template <typename real>
void fmadd_t(const real *fac, bool per_dim, const solid<real> &A, solid<real> &B)
{
    if (A.dimension() != B.dimension()) throw std::logic_error{"solidfmm::fmadd(): dimension mismatch."};
    if (A.order() != B.order()) throw std::logic_error{"solidfmm::fmadd(): order mismatch."};
    const size_t S = A.order() * (A.order() + 1);
    for (size_t d = 0; d < A.dimension(); ++d) {
        const real f = per_dim ? fac[d] : fac[0];
        const real *a = A.memptr() + d * S;
        real *b = B.memptr() + d * S;
        for (size_t k = 0; k < S; ++k) b[k] += f * a[k];
    }
}

}  // namespace

void dot(const solid<float> &A, const solid<float> &B, float *result) noexcept { dot_t(A, B, result); }
void dot(const solid<double> &A, const solid<double> &B, double *result) noexcept { dot_t(A, B, result); }
void fmadd(const float fac, const solid<float> &A, solid<float> &B) { fmadd_t(&fac, false, A, B); }
void fmadd(const float *fac, const solid<float> &A, solid<float> &B) { fmadd_t(fac, true, A, B); }
void fmadd(const double fac, const solid<double> &A, solid<double> &B) { fmadd_t(&fac, false, A, B); }
void fmadd(const double *fac, const solid<double> &A, solid<double> &B) { fmadd_t(fac, true, A, B); }

}  // namespace solidfmm
