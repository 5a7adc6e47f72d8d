// The entry shuffle of MCPNet's semi-supervised evaluation (shuffle_truth,
// apps/pipeline/eval_mcpnet.cpp:214-224: a std::mt19937 seeded with the
// iteration number drives std::shuffle over the (row, col, label) mask).
// TEST INFRASTRUCTURE ONLY: part of the CPU oracle library.
//
//   orc_shuffle_u32     shuffles the positions 0..n-1 the same way;
//   orc_shuffle_tuples  shuffles the reference's own element type, tuples of
//                       (size_t, size_t, int) holding (k, k, k), and returns the
//                       order of k -- equal to orc_shuffle_u32's, because
//                       std::shuffle's swaps depend only on the length and the
//                       generator.
#include <algorithm>
#include <cstdint>
#include <numeric>
#include <random>
#include <tuple>
#include <vector>

extern "C" {

void orc_shuffle_u32(uint32_t* a, int64_t n, uint32_t seed) {
    std::iota(a, a + n, 0u);
    std::mt19937 g(seed);
    std::shuffle(a, a + n, g);
}

void orc_shuffle_tuples(int64_t n, uint32_t seed, int64_t* order) {
    std::vector<std::tuple<size_t, size_t, int>> v;
    v.reserve((size_t)n);
    for (int64_t k = 0; k < n; ++k) v.emplace_back((size_t)k, (size_t)k, (int)k);
    std::mt19937 g(seed);
    std::shuffle(v.begin(), v.end(), g);
    for (int64_t k = 0; k < n; ++k) order[k] = (int64_t)std::get<0>(v[(size_t)k]);
}

}  // extern "C"
