// Seeded synthetic gene-regulatory-network expression data (host only), built
// as its own library (libmcpsynth.so) so that the CPU-only timing of the
// reference path and the tests can make inputs without loading libmcpgpu.so.
//
// Stands in for MCPNet's GNW / DREAM inputs (absent from the reference
// snapshot) with the generator the benchmark configurations name:
//   - a random DAG over a random topological order: each gene draws an
//     in-degree ~ Poisson(2) (capped by the number of earlier genes) and that
//     many distinct parents uniformly among the genes earlier in the order;
//   - edge weights +-U(0.5, 1.5), sign + or - with probability 1/2;
//   - roots ~ N(0, 1); x_g = tanh(sum_p w_pg x_p) + N(0, 0.3^2);
//   - every gene min-max rescaled to [0, 1] (in double from the float
//     values), stored as float.
// The graph comes from std::mt19937_64(seed).  Sample noise comes from a
// counter-based stream (splitmix64 of seed+1, gene, sample) so that samples
// are generated in parallel and independently of the thread count.  Normals
// use Box-Muller.  Results are identical on every run and thread count on one
// machine; libm differences between machines (tanh, log, cos) can move the
// last bits.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <random>
#include <vector>

#include "../include/mcpsynth.h"

namespace {

inline uint64_t splitmix64(uint64_t x) {
    x += 0x9e3779b97f4a7c15ull;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}

inline double u01(uint64_t r) { return (double)(r >> 11) * (1.0 / 9007199254740992.0); }  // [0, 1)

// Standard normal for (stream, gene, sample) by Box-Muller.
inline double normal_at(uint64_t seed, uint64_t g, uint64_t s) {
    const uint64_t base = splitmix64(seed ^ splitmix64(g * 0x100000001b3ull + 0x51ed27ull)) ^ (s * 0x9e3779b97f4a7c15ull);
    const uint64_t r1 = splitmix64(base), r2 = splitmix64(base ^ 0xd1b54a32d192ed03ull);
    const double u1 = 1.0 - u01(r1);  // (0, 1]
    const double u2 = u01(r2);
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
}

int poisson2(std::mt19937_64& rng) {
    // Knuth's multiplication method for lambda = 2.
    const double L = std::exp(-2.0);
    int k = 0;
    double p = 1.0;
    do {
        ++k;
        p *= u01(rng());
    } while (p > L);
    return k - 1;
}

}  // namespace

extern "C" int mcps_synth_grn(int64_t n, int64_t m, uint64_t seed, float* X, int64_t ldx, int32_t* edges,
                              int64_t max_edges, int64_t* n_edges) {
    if (n < 0 || m < 0 || (n > 0 && m > 0 && (!X || ldx < m))) return MCPS_ERR_ARG;
    if (n > INT32_MAX) return MCPS_ERR_ARG;
    if (n_edges) *n_edges = 0;
    if (n == 0) return MCPS_OK;

    std::mt19937_64 rng(seed);
    std::vector<int32_t> order((size_t)n);
    for (int64_t i = 0; i < n; ++i) order[(size_t)i] = (int32_t)i;
    for (int64_t i = n - 1; i > 0; --i) {  // Fisher-Yates
        const int64_t j = (int64_t)(rng() % (uint64_t)(i + 1));
        std::swap(order[(size_t)i], order[(size_t)j]);
    }
    // parents of the gene at topological position t (CSR)
    std::vector<int64_t> start((size_t)n + 1, 0);
    std::vector<int32_t> par;
    std::vector<double> wt;
    par.reserve((size_t)n * 2);
    wt.reserve((size_t)n * 2);
    std::vector<int32_t> pick;
    for (int64_t t = 0; t < n; ++t) {
        int d = poisson2(rng);
        if (d > t) d = (int)t;
        pick.clear();
        while ((int)pick.size() < d) {
            const int32_t c = (int32_t)(rng() % (uint64_t)t);  // position among earlier genes
            if (std::find(pick.begin(), pick.end(), c) == pick.end()) pick.push_back(c);
        }
        for (int32_t c : pick) {
            const double mag = 0.5 + u01(rng());
            const double sgn = (u01(rng()) < 0.5) ? -1.0 : 1.0;
            par.push_back(order[(size_t)c]);
            wt.push_back(sgn * mag);
        }
        start[(size_t)t + 1] = (int64_t)par.size();
    }
    const int64_t ne = (int64_t)par.size();
    if (n_edges) *n_edges = ne;
    if (edges) {
        int64_t e = 0;
        for (int64_t t = 0; t < n && e < max_edges; ++t)
            for (int64_t q = start[(size_t)t]; q < start[(size_t)t + 1] && e < max_edges; ++q, ++e) {
                edges[2 * e] = par[(size_t)q];
                edges[2 * e + 1] = order[(size_t)t];
            }
    }
    if (m == 0) return MCPS_OK;

    // samples: columns are independent given the graph
    const uint64_t sseed = seed + 1;
#pragma omp parallel
    {
        std::vector<double> xs((size_t)n);
#pragma omp for schedule(static)
        for (int64_t s = 0; s < m; ++s) {
            for (int64_t t = 0; t < n; ++t) {
                const int32_t g = order[(size_t)t];
                const int64_t b = start[(size_t)t], e = start[(size_t)t + 1];
                double v;
                if (b == e) {
                    v = normal_at(sseed, (uint64_t)g, (uint64_t)s);
                } else {
                    double acc = 0.0;
                    for (int64_t q = b; q < e; ++q) acc += wt[(size_t)q] * xs[(size_t)par[(size_t)q]];
                    v = std::tanh(acc) + 0.3 * normal_at(sseed, (uint64_t)g, (uint64_t)s);
                }
                xs[(size_t)g] = v;
                X[g * ldx + s] = (float)v;  // raw value for now; rescaled below
            }
        }
    }
    // per-gene min-max rescale of the stored values to [0, 1], in double
#pragma omp parallel for schedule(static)
    for (int64_t g = 0; g < n; ++g) {
        float* row = X + g * ldx;
        double mn = row[0], mx = row[0];
        for (int64_t s = 1; s < m; ++s) {
            mn = std::min(mn, (double)row[s]);
            mx = std::max(mx, (double)row[s]);
        }
        const double span = mx - mn;
        for (int64_t s = 0; s < m; ++s) row[s] = span > 0 ? (float)(((double)row[s] - mn) / span) : 0.0f;
    }
    return MCPS_OK;
}
