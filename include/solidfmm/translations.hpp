// solidfmm-gb300 drop-in: the translation operators M2M, M2L and L2L.
//
// Same declarations as the reference's solidfmm/translations.hpp:39-170:
// the batch interface multithreaded_translator<real> with translation_info
// items, and the single-thread overloads (classic pointer arrays and
// translation_info ranges, checked and unchecked).  Every call translates the
// whole batch on the GPU (gather to device memory, one fused kernel launch,
// scatter-add back) and returns when the targets are updated.
//
// Checked variants validate everything before touching any target and
// throw the reference's exception types: std::logic_error (incompatible
// buffer, dimension mismatch), std::out_of_range (orders above the operator
// order), std::runtime_error (CUDA failure).  Unchecked variants skip the
// validation; a CUDA failure there terminates the program.
#ifndef SOLIDFMM_TRANSLATIONS_HPP
#define SOLIDFMM_TRANSLATIONS_HPP

#include <cstddef>

extern "C" {
struct hwloc_topology;
struct hwloc_bitmap_s;
}

namespace solidfmm
{

template <typename real> class solid;

//////////////////////////////
// Multithreaded interface. //
//////////////////////////////

template <typename real>
struct translation_info
{
    const solid<real> *source;
    solid<real> *target;
    real x, y, z;
};

template <typename real>
class multithreaded_translator
{
public:
    using item = translation_info<real>;
    using cpuset_t = hwloc_bitmap_s *;

    multithreaded_translator() = delete;
    multithreaded_translator(const multithreaded_translator &rhs) = delete;
    multithreaded_translator(multithreaded_translator &&rhs) noexcept;
    ~multithreaded_translator();
    multithreaded_translator &operator=(const multithreaded_translator &rhs) = delete;
    multithreaded_translator &operator=(multithreaded_translator &&rhs) noexcept;

    // One GPU batch translator for expansions up to max_expansion_order.
    multithreaded_translator(size_t max_expansion_order);

    // The topology/cpuset form of the reference: the cpusets chose the host
    // cores of the worker threads; here the work runs on the current CUDA
    // device and the host side needs no pinned workers, so the sets are only
    // checked (a null topology throws std::runtime_error, as in the reference).
    multithreaded_translator(size_t max_expansion_order, hwloc_topology *topology, cpuset_t *begin, cpuset_t *end);

    // Scheduling policies of the reference's host threads; a single GPU batch
    // needs neither, both are accepted and keep the default.
    void schedule_equally_among_threads() noexcept;
    void schedule_by_measuring_throughput();

    void m2m(const item *begin, const item *end) const;
    void m2l(const item *begin, const item *end) const;
    void l2l(const item *begin, const item *end) const;

    void m2m_unchecked(const item *begin, const item *end) const noexcept;
    void m2l_unchecked(const item *begin, const item *end) const noexcept;
    void l2l_unchecked(const item *begin, const item *end) const noexcept;

private:
    class impl;
    impl *p;
};

extern template class multithreaded_translator<float>;
extern template class multithreaded_translator<double>;

////////////////////////////////
// Single threaded functions. //
////////////////////////////////

template <typename real> class operator_data;
template <typename real> class threadlocal_buffer;

void m2l(const operator_data<float> &op, threadlocal_buffer<float> &buf, size_t howmany,
         const solid<float> *const *const M, solid<float> *const *const L, const float *x, const float *y,
         const float *z);
void m2l(const operator_data<double> &op, threadlocal_buffer<double> &buf, size_t howmany,
         const solid<double> *const *const M, solid<double> *const *const L, const double *x, const double *y,
         const double *z);
void m2l(const operator_data<float> &op, threadlocal_buffer<float> &buf, const translation_info<float> *begin,
         const translation_info<float> *end);
void m2l(const operator_data<double> &op, threadlocal_buffer<double> &buf, const translation_info<double> *begin,
         const translation_info<double> *end);

void m2m(const operator_data<float> &op, threadlocal_buffer<float> &buf, size_t howmany,
         const solid<float> *const *const Min, solid<float> *const *const Mout, const float *x, const float *y,
         const float *z);
void m2m(const operator_data<double> &op, threadlocal_buffer<double> &buf, size_t howmany,
         const solid<double> *const *const Min, solid<double> *const *const Mout, const double *x, const double *y,
         const double *z);
void m2m(const operator_data<float> &op, threadlocal_buffer<float> &buf, const translation_info<float> *begin,
         const translation_info<float> *end);
void m2m(const operator_data<double> &op, threadlocal_buffer<double> &buf, const translation_info<double> *begin,
         const translation_info<double> *end);

void l2l(const operator_data<float> &op, threadlocal_buffer<float> &buf, size_t howmany,
         const solid<float> *const *const Min, solid<float> *const *const Mout, const float *x, const float *y,
         const float *z);
void l2l(const operator_data<double> &op, threadlocal_buffer<double> &buf, size_t howmany,
         const solid<double> *const *const Lin, solid<double> *const *const Lout, const double *x, const double *y,
         const double *z);
void l2l(const operator_data<float> &op, threadlocal_buffer<float> &buf, const translation_info<float> *begin,
         const translation_info<float> *end);
void l2l(const operator_data<double> &op, threadlocal_buffer<double> &buf, const translation_info<double> *begin,
         const translation_info<double> *end);

void m2l_unchecked(const operator_data<float> &op, threadlocal_buffer<float> &buf,
                   const translation_info<float> *begin, const translation_info<float> *end) noexcept;
void m2l_unchecked(const operator_data<double> &op, threadlocal_buffer<double> &buf,
                   const translation_info<double> *begin, const translation_info<double> *end) noexcept;
void m2m_unchecked(const operator_data<float> &op, threadlocal_buffer<float> &buf,
                   const translation_info<float> *begin, const translation_info<float> *end) noexcept;
void m2m_unchecked(const operator_data<double> &op, threadlocal_buffer<double> &buf,
                   const translation_info<double> *begin, const translation_info<double> *end) noexcept;
void l2l_unchecked(const operator_data<float> &op, threadlocal_buffer<float> &buf,
                   const translation_info<float> *begin, const translation_info<float> *end) noexcept;
void l2l_unchecked(const operator_data<double> &op, threadlocal_buffer<double> &buf,
                   const translation_info<double> *begin, const translation_info<double> *end) noexcept;

// GB300 extension (no counterpart in the reference): arithmetic of the
// double-precision calls in this thread.  false (default) = plain FP64;
// true = split precision (include/sfmm.h, SFMM_SPLIT): FP64 expansions and
// accumulation, the translation on the FP32 and integer pipes with relative
// error <= 1e-7 in the orthonormal basis.
void set_split_precision(bool enable) noexcept;
bool split_precision() noexcept;

}  // namespace solidfmm

#endif
