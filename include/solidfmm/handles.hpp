// solidfmm-gb300 drop-in: owning handles for operator data and work buffers,
// same interface as the reference's solidfmm/handles.hpp:33-116 (default
// orders 18 for float and 30 for double; copies re-create the object;
// implicit conversions to operator_data& / threadlocal_buffer&).
#ifndef SOLIDFMM_HANDLES_HPP
#define SOLIDFMM_HANDLES_HPP

#include <cstddef>

namespace solidfmm
{

template <typename real> class operator_data;
template <typename real> class operator_handle;
template <typename real> class threadlocal_buffer;
template <typename real> class buffer_handle;

template <typename real>
class operator_handle
{
public:
    operator_handle();
    operator_handle(size_t P);
    ~operator_handle();
    operator_handle(const operator_handle &rhs);
    operator_handle &operator=(const operator_handle &rhs);

    operator_handle(operator_handle &&rhs) noexcept : p{rhs.p} { rhs.p = nullptr; }
    operator_handle &operator=(operator_handle &&rhs) noexcept
    {
        pointer tmp = p;
        p = rhs.p;
        rhs.p = tmp;
        return *this;
    }

    buffer_handle<real> make_buffer() const;

    using reference = operator_data<real> &;
    using const_reference = const operator_data<real> &;
    using pointer = operator_data<real> *;
    using const_pointer = const operator_data<real> *;

    operator reference() noexcept { return *p; }
    operator const_reference() const noexcept { return *p; }
    operator pointer() noexcept { return p; }
    operator const_pointer() const noexcept { return p; }

private:
    pointer p;
};

template <typename real>
class buffer_handle
{
public:
    buffer_handle();
    buffer_handle(const operator_data<real> &op);
    buffer_handle(const buffer_handle &rhs);
    ~buffer_handle();
    buffer_handle &operator=(const buffer_handle &rhs);

    buffer_handle(buffer_handle &&rhs) noexcept : p{rhs.p} { rhs.p = nullptr; }
    buffer_handle &operator=(buffer_handle &&rhs) noexcept
    {
        pointer tmp = p;
        p = rhs.p;
        rhs.p = tmp;
        return *this;
    }

    using reference = threadlocal_buffer<real> &;
    using const_reference = const threadlocal_buffer<real> &;
    using pointer = threadlocal_buffer<real> *;
    using const_pointer = const threadlocal_buffer<real> *;

    operator reference() noexcept { return *p; }
    operator const_reference() const noexcept { return *p; }
    operator pointer() noexcept { return p; }
    operator const_pointer() const noexcept { return p; }

private:
    pointer p;
};

extern template class operator_handle<float>;
extern template class buffer_handle<float>;
extern template class operator_handle<double>;
extern template class buffer_handle<double>;

}  // namespace solidfmm

#endif
