// Stand-in for splash::ds::aligned_matrix: a row-major matrix view with the
// accessors MCPNet's hot-path and evaluation headers call (rows, columns,
// data(row), data(row, col), at).
// Test infrastructure only.
#pragma once
#include <cstddef>

namespace splash { namespace ds {

template <typename T>
class aligned_matrix {
    T* ptr_ = nullptr;
    size_t rows_ = 0, cols_ = 0, ld_ = 0;
  public:
    aligned_matrix() {}
    aligned_matrix(T* p, size_t r, size_t c, size_t ld) : ptr_(p), rows_(r), cols_(c), ld_(ld) {}
    size_t rows() const { return rows_; }
    size_t columns() const { return cols_; }
    T* data(size_t r) { return ptr_ + r * ld_; }
    T const* data(size_t r) const { return ptr_ + r * ld_; }
    T* data(size_t r, size_t c) { return ptr_ + r * ld_ + c; }
    T const* data(size_t r, size_t c) const { return ptr_ + r * ld_ + c; }
    T& at(size_t r, size_t c) { return ptr_[r * ld_ + c]; }
};

}}
