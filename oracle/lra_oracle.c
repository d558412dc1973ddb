/*
 * CPU oracle for the sketch-then-factor path -- TEST INFRASTRUCTURE ONLY.
 *
 * Only the tests, the smoke check and the benchmark's CPU-baseline leg load
 * this library, and only as the checker.  The product (liblra) never links
 * or calls it.  Type-generic code lives in lra_oracle_impl.h.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>

#define REAL double
#define SFX d
#define REAL_MAX DBL_MAX
#define REAL_EPS (DBL_EPSILON * 0.5) /* LAPACK xLAMCH('E') */
#define REAL_SAFMIN DBL_MIN          /* LAPACK xLAMCH('S') */
#include "lra_oracle_impl.h"
#undef REAL
#undef SFX
#undef REAL_MAX
#undef REAL_EPS
#undef REAL_SAFMIN

#define REAL float
#define SFX s
#define REAL_MAX FLT_MAX
#define REAL_EPS (FLT_EPSILON * 0.5f)
#define REAL_SAFMIN FLT_MIN
#include "lra_oracle_impl.h"
