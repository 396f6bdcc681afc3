/* Force-included only when compiling the reference's microkernel.cpp for the
 * portable-dispatch checker build: pull in the system headers first, then
 * hide the x86-64 macro so get_microkernel() takes its generic branch. */
#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <cmath>
#include <stdexcept>
#include <new>
#include <memory>
#undef __x86_64__
