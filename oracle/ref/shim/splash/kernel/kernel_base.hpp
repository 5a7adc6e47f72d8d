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

}}
