/* CPU oracle for the MCPNet compute core: a C restatement of the reference's
 * B-spline MI, max-min (MCP), ratio, DPI and closure arithmetic.
 *
 * TEST INFRASTRUCTURE ONLY -- the checker, never the thing measured or
 * shipped.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg load it (through oracle/oracle.py).  Its fidelity to the reference is
 * pinned by tests/test_oracle_golden.py against fixtures produced by MCPNet's
 * own kernels (oracle/ref/ref_driver.cpp, tests/golden/make_golden.py).
 *
 * Build: oracle/Makefile -> oracle/_build/libmcporacle.so
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <float.h>

#define REAL float
#define SFX f32
#include "mcp_oracle_impl.h"
#undef REAL
#undef SFX

#define REAL double
#define SFX f64
#include "mcp_oracle_impl.h"
#undef REAL
#undef SFX

int orc_num_threads(void) {
#ifdef _OPENMP
    extern int omp_get_max_threads(void);
    return omp_get_max_threads();
#else
    return 1;
#endif
}
