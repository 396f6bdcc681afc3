// solidfmm-gb300 drop-in: per-order operator data (the reference's
// operator_data<real>, solidfmm/operator_data.hpp:31-68).  Here it owns a
// GPU operator context (sfmm_context, include/sfmm.h) holding the swap,
// rotation and z-translation tables on the device.
#ifndef SOLIDFMM_OPERATOR_DATA_HPP
#define SOLIDFMM_OPERATOR_DATA_HPP

#include <cstddef>

struct sfmm_context;

namespace solidfmm
{

template <typename real>
class operator_data
{
public:
    operator_data() = delete;
    // std::logic_error if P == 0, std::overflow_error if P exceeds the
    // type's limit (18 for float, 86 for double), std::runtime_error if no
    // CUDA device is usable.
    explicit operator_data(size_t P);
    operator_data(const operator_data &) = delete;
    operator_data(operator_data &&) = delete;
    operator_data &operator=(const operator_data &) = delete;
    operator_data &operator=(operator_data &&) = delete;
    ~operator_data();

    size_t order() const noexcept { return P; }
    sfmm_context *context() const noexcept { return ctx; }

private:
    size_t P;
    sfmm_context *ctx;
};

extern template class operator_data<float>;
extern template class operator_data<double>;

}  // namespace solidfmm

#endif
