// Stand-in for splash::ds::aligned_vector (included, not used, by the
// MCPNet headers the oracle compiles).  Test infrastructure only.
#pragma once
#include <vector>
namespace splash { namespace ds {
template <typename T> using aligned_vector = std::vector<T>;
}}
