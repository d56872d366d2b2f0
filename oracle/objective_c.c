/*
 * FP64 pixel term of the D2IC global objective, in C for speed.
 *
 * Test infrastructure only: called by the oracle (oracle/fast.py) to run the
 * reference's nonlinear CG at full benchmark sizes.  Never linked into the
 * product library.
 *
 * Restates residuals_pixelwise_core / J_pixelwise_core and their gradient
 * (d2ic/solver_global_cg.py:205-258) with the oracle's cubic definition: the
 * interpolating cubic B-spline with edge-replicating boundary, evaluated on a
 * coefficient array that carries a `pad`-wide halo (oracle/cubic.py).
 *
 * Two instantiations of objective_body.h: oracle_pixel_terms (double, the
 * oracle) and oracle_pixel_terms_f32 (float: the same arithmetic in the
 * reference's default x32 precision, used only to time an x32-equivalent CPU
 * baseline).
 *
 * Build: see oracle/Makefile (gcc -O2 -fopenmp -ffp-contract=off).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

#define REAL double
#define FN(name) name
#include "objective_body.h"
#undef REAL
#undef FN

#define REAL float
#define FN(name) name##_f32
#include "objective_body.h"
#undef REAL
#undef FN
