// Stand-in for splash::ds::buffer: a growable array with a public `data`
// pointer.  resize() zero-fills, which AdaptivePartitionRankMIKernel2 relies
// on (its per-pair `temp` offsets are accumulated from zero after resize).
// Test infrastructure only.
#pragma once
#include <cstddef>
#include <cstring>
#include <vector>

namespace splash { namespace ds {

template <typename T>
class buffer {
    std::vector<T> store_;
  public:
    T* data = nullptr;
    size_t size = 0;
    buffer() {}
    buffer(buffer const& o) : store_(o.store_), data(store_.data()), size(o.size) {}
    buffer& operator=(buffer const& o) {
        store_ = o.store_;
        data = store_.data();
        size = o.size;
        return *this;
    }
    void resize(size_t n) {
        store_.assign(n, T());
        data = store_.data();
        size = n;
    }
};

}}
