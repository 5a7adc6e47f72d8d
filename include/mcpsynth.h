/* mcpsynth -- seeded synthetic gene-regulatory-network expression (host only).
 *
 * The inputs of the benchmark configurations: MCPNet's own GNW / DREAM inputs
 * are not part of the reference, so every configuration runs on this seeded
 * generator.  It is a separate library from libmcpgpu.so (no device code, no
 * CUDA dependency), so that a CPU-only run of the reference path can make the
 * same inputs without loading the GPU library.
 *
 * Model: random DAG over a random topological order, in-degree ~ Poisson(2)
 * from earlier genes, weights +-U(0.5,1.5); x_g = tanh(sum w x_parent) +
 * N(0, 0.3^2), roots ~ N(0,1); each gene min-max rescaled to [0,1].
 */
#ifndef MCPSYNTH_H
#define MCPSYNTH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define MCPS_API __attribute__((visibility("default")))
#else
#define MCPS_API
#endif

#define MCPS_OK 0
#define MCPS_ERR_ARG (-1) /* negative size, null X with n, m > 0, ldx < m, n >= 2^31 */

/* X: n x m row-major floats (ldx >= m), nullable when m == 0.  edges (nullable,
 * capacity max_edges pairs of int32 parent, child) receives the ground-truth
 * DAG; n_edges (nullable) gets the edge count.  Deterministic for a seed: the
 * graph from std::mt19937_64(seed), samples from a counter-based stream of
 * seed + 1, identical for any thread count. */
MCPS_API int mcps_synth_grn(int64_t n, int64_t m, uint64_t seed, float* X, int64_t ldx, int32_t* edges,
                            int64_t max_edges, int64_t* n_edges);

#ifdef __cplusplus
}
#endif

#endif /* MCPSYNTH_H */
