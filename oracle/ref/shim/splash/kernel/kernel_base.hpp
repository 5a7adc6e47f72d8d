// Minimal stand-in for the splash kernel base classes (the splash submodule
// is absent from the MCPNet snapshot).  Written from how MCPNet's hot-path
// headers use them: functors derive from these templates, read no members
// from them except `processed` (a mutable counter used by mask/threshold),
// and are driven by the oracle's own loops in ref_driver.cpp.
// Test infrastructure only: the checker, never the product.
#pragma once
#include <cstddef>
#include <cmath>
#include <cassert>
#include <chrono>
#include <cstring>

// Logging and timing used by the evaluation kernels (aupr.hpp, auroc.hpp):
// printing is dropped, timing is a steady clock.
#ifndef FMT_ROOT_PRINT
#define FMT_ROOT_PRINT(...) do {} while (0)
#endif
#ifndef FMT_PRINT_RT
#define FMT_PRINT_RT(...) do {} while (0)
#endif
inline std::chrono::steady_clock::time_point getSysTime() { return std::chrono::steady_clock::now(); }
inline double get_duration_s(std::chrono::steady_clock::time_point a, std::chrono::steady_clock::time_point b) {
    return std::chrono::duration<double>(b - a).count();
}

namespace splash { namespace kernel {

enum class DEGREE : int { SCALAR = 0, VECTOR = 1, MATRIX = 2 };

struct kernel_counter {
    mutable size_t processed = 0;
    virtual ~kernel_counter() {}
};

template <typename IT, typename OT, DEGREE IN = DEGREE::VECTOR, DEGREE OUT = DEGREE::VECTOR>
class transform : public kernel_counter {};

template <typename IT, typename OT, DEGREE IN = DEGREE::VECTOR, DEGREE OUT = DEGREE::SCALAR>
class inner_product : public kernel_counter {};

template <typename IT, typename OT, DEGREE IN = DEGREE::VECTOR, DEGREE OUT = DEGREE::SCALAR>
class inner_product_pos : public kernel_counter {};

template <typename IT, typename IT2, typename OT, DEGREE D = DEGREE::VECTOR>
class binary_op : public kernel_counter {};

template <typename IT, typename IT2, typename IT3, typename OT, DEGREE D = DEGREE::VECTOR>
class ternary_op : public kernel_counter {};

template <typename IT, typename LABEL, typename OT, DEGREE D = DEGREE::VECTOR>
class masked_reduce : public kernel_counter {};

}}
