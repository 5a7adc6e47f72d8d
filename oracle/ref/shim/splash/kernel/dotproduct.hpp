// Stand-in for splash::kernel::dotp_{scalar,sse,avx,avx512}.  The real splash
// implementations are not in the MCPNet snapshot, so their summation order is
// unknown; every variant here is a plain sequential accumulation in T.  MI
// parity against this stand-in is therefore a tolerance check, not bit-exact.
// Test infrastructure only.
#pragma once
#include <cstddef>

namespace splash { namespace kernel {

template <typename T>
inline T dotp_scalar(T const* a, T const* b, size_t const& count) {
    T s = 0;
    for (size_t i = 0; i < count; ++i) s += a[i] * b[i];
    return s;
}
template <typename T>
inline T dotp_sse(T const* a, T const* b, size_t const& count) { return dotp_scalar(a, b, count); }
template <typename T>
inline T dotp_avx(T const* a, T const* b, size_t const& count) { return dotp_scalar(a, b, count); }
template <typename T>
inline T dotp_avx512(T const* a, T const* b, size_t const& count) { return dotp_scalar(a, b, count); }

}}
