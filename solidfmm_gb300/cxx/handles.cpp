// operator_data, operator_handle and buffer_handle for the drop-in API
// (semantics of the reference's solidfmm/handles.cpp:30-115 and
// operator_data.cpp:151-164).
#include <solidfmm/handles.hpp>
#include <solidfmm/operator_data.hpp>
#include <solidfmm/threadlocal_buffer.hpp>

#include <cuda_runtime.h>

#include <stdexcept>
#include <string>

#include "sfmm.h"

namespace solidfmm
{

namespace
{
template <typename real> constexpr int dtype_of();
template <> constexpr int dtype_of<float>() { return SFMM_F32; }
template <> constexpr int dtype_of<double>() { return SFMM_F64; }
template <typename real> constexpr size_t default_order();
template <> constexpr size_t default_order<float>() { return 18; }
template <> constexpr size_t default_order<double>() { return 30; }
}  // namespace

template <typename real>
operator_data<real>::operator_data(size_t P_) : P{P_}, ctx{nullptr}
{
    if (P == 0) throw std::logic_error{"solidfmm::operator_data(): Requested order P = 0."};
    if (P > (dtype_of<real>() == SFMM_F32 ? 18u : 86u))
        throw std::overflow_error{
            "solidfmm::operator_data(): Requested order is too large for the chosen floating point type."};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) dev = 0;
    int rc = sfmm_create(&ctx, dtype_of<real>(), P, dev);
    if (rc == SFMM_OOM) throw std::bad_alloc{};
    if (rc != SFMM_OK)
        throw std::runtime_error{std::string{"solidfmm::operator_data(): GPU context creation failed: "} +
                                 sfmm_status_string(rc)};
}

template <typename real>
operator_data<real>::~operator_data()
{
    sfmm_destroy(ctx);
}

template class operator_data<float>;
template class operator_data<double>;

template <typename real>
operator_handle<real>::operator_handle() : p{new operator_data<real>(default_order<real>())}
{
}

template <typename real>
operator_handle<real>::operator_handle(size_t P) : p{new operator_data<real>(P)}
{
}

template <typename real>
operator_handle<real>::~operator_handle()
{
    delete p;
}

template <typename real>
operator_handle<real>::operator_handle(const operator_handle &rhs) : p{new operator_data<real>(rhs.p->order())}
{
}

template <typename real>
operator_handle<real> &operator_handle<real>::operator=(const operator_handle &rhs)
{
    if (&rhs != this) {
        pointer tmp = new operator_data<real>(rhs.p->order());
        delete p;
        p = tmp;
    }
    return *this;
}

template <typename real>
buffer_handle<real> operator_handle<real>::make_buffer() const
{
    return buffer_handle<real>{*p};
}

template <typename real>
buffer_handle<real>::buffer_handle() : p{new threadlocal_buffer<real>{}}
{
}

template <typename real>
buffer_handle<real>::buffer_handle(const operator_data<real> &op) : p{new threadlocal_buffer<real>{op}}
{
}

template <typename real>
buffer_handle<real>::buffer_handle(const buffer_handle &rhs) : p{new threadlocal_buffer<real>{*rhs.p}}
{
}

template <typename real>
buffer_handle<real>::~buffer_handle()
{
    delete p;
}

template <typename real>
buffer_handle<real> &buffer_handle<real>::operator=(const buffer_handle &rhs)
{
    *p = *rhs.p;
    return *this;
}

template class operator_handle<float>;
template class buffer_handle<float>;
template class operator_handle<double>;
template class buffer_handle<double>;

}  // namespace solidfmm
