// Stand-in for splash::utils::aalloc (aligned allocation), test infrastructure only.
#pragma once
#include <cstdlib>
#include <cstddef>

namespace splash { namespace utils {

template <typename T>
T* aalloc(size_t count) {
    void* p = nullptr;
    size_t bytes = ((count * sizeof(T) + 63) / 64) * 64;
    if (posix_memalign(&p, 64, bytes ? bytes : 64) != 0) return nullptr;
    return static_cast<T*>(p);
}
inline void afree(void* p) { free(p); }

}}
