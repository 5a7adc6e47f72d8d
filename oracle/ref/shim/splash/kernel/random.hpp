// Stand-in for the splash random-number and partition helpers that
// AdaptivePartitioningMI.hpp names in its add_noise functor (declared so the
// header parses; the oracle never instantiates add_noise).  Test
// infrastructure only.
#pragma once
#include <cstddef>
#include <random>

#ifndef PARTITION_EQUAL
#define PARTITION_EQUAL 0
#endif

namespace splash {
namespace utils {
template <typename T>
struct partition {
    T offset = 0, size = 0, id = 0;
    partition() {}
    partition(T o, T s, T i) : offset(o), size(s), id(i) {}
};
template <int P>
struct partitioner1D {
    template <typename T>
    partition<T> get_partition(partition<T> const& p, size_t, size_t) const { return p; }
};
}  // namespace utils
namespace kernel {
template <typename G = std::default_random_engine>
class random_number_generator {
    G g_;
  public:
    G& get_generator(size_t) { return g_; }
};
}  // namespace kernel
}  // namespace splash
