/*
 * ps_oracle.c -- CPU oracle for the GB300 stencil library. TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C + OpenMP restatement of the arithmetic of ParallelStencil.jl's
 * FiniteDifferences macros and of the example / miniapp kernels built from them. It is the
 * checker for libps_b200.so (tests, smoke check, the benchmark's timed CPU baseline) and
 * never part of the product path.
 *
 * Semantics restated (file:line refer to the reference project):
 *   - FD macros: src/FiniteDifferences.jl:54-61 (1-D), :160-185 (2-D), :328-394 (3-D); the
 *     operation order of every macro is kept (left-to-right sums, `*0.5`, `1.0/(...)*2.0`).
 *   - Masks: `@within` (src/FiniteDifferences.jl:397-408) applied per statement
 *     (src/parallel.jl:654-680); inner index ixi = ix+1 (src/ParallelKernel/parallel.jl:498-504).
 *   - Thread grid: max extents over all array arguments (src/ParallelKernel/parallel.jl:795-798).
 *   - CPU loop: `Threads.@threads for iz; for iy; for ix` (src/ParallelKernel/parallel.jl:755-765),
 *     here `#pragma omp parallel for schedule(static)` over z.
 *   - Literals are cast to the number type (src/ParallelKernel/parallel.jl:400-418): the
 *     FP32 instantiation uses float literals. `1/x` -> `inv(x)` (:477-485) is IEEE 1/x.
 *   - Julia does not contract a*b+c into an FMA; this file is compiled with
 *     -ffp-contract=off for the same reason.
 *
 * Parity pin: the reference cannot run here (it is Julia; no Julia toolchain exists on
 * these machines). The oracle is pinned against known-answer fixtures restated from the
 * reference's own tests (tests/golden/make_golden.py), which compare each kernel to Julia
 * broadcasting with exact equality.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_OK 0
#define ORC_ERR_ARG -1
#define ORC_ERR_SHAPE -3

int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_num_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

#define REAL double
#define SFX(name) name##_f64
#include "ps_oracle_body.h"
#undef REAL
#undef SFX

#define REAL float
#define SFX(name) name##_f32
#include "ps_oracle_body.h"
#undef REAL
#undef SFX
