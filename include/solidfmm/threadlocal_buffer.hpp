// solidfmm-gb300 drop-in: per-thread work buffer (the reference's
// threadlocal_buffer<real>, solidfmm/threadlocal_buffer.hpp:29-52).  The
// GPU kernels keep their working expansions in shared memory, so the
// buffer only records the order it was made for; compatible() is true for
// operators of that order, as in the reference.
#ifndef SOLIDFMM_TRHEADLOCAL_BUFFER_HPP
#define SOLIDFMM_TRHEADLOCAL_BUFFER_HPP

#include <cstddef>

namespace solidfmm
{

template <typename real> class operator_data;

template <typename real>
class threadlocal_buffer
{
public:
    threadlocal_buffer() noexcept = default;
    explicit threadlocal_buffer(const operator_data<real> &op) : P(op.order()) {}
    threadlocal_buffer(const threadlocal_buffer &) = default;
    threadlocal_buffer(threadlocal_buffer &&) noexcept = default;
    threadlocal_buffer &operator=(const threadlocal_buffer &) = default;
    threadlocal_buffer &operator=(threadlocal_buffer &&) noexcept = default;
    ~threadlocal_buffer() = default;

    void swap(threadlocal_buffer &rhs) noexcept
    {
        size_t t = P;
        P = rhs.P;
        rhs.P = t;
    }
    void initialise(const operator_data<real> &op) { P = op.order(); }
    bool compatible(const operator_data<real> &op) const noexcept { return P != 0 && P == op.order(); }

private:
    size_t P{0};
};

}  // namespace solidfmm

#endif
