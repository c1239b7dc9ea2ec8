/*
 * CPU oracle — TEST INFRASTRUCTURE ONLY (see oracle_impl.h).
 * Builds the float64 and float32 variants of every oracle routine.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>

#define REAL double
#define SFX _f64
#define IS_F64 1
#define EXP exp
#define FABS fabs
#include "oracle_impl.h"
#undef REAL
#undef SFX
#undef IS_F64
#undef EXP
#undef FABS

#define REAL float
#define SFX _f32
#define IS_F64 0
#define EXP expf
#define FABS fabsf
#include "oracle_impl.h"

int orc_num_threads(void) {
#ifdef _OPENMP
  extern int omp_get_max_threads(void);
  return omp_get_max_threads();
#else
  return 1;
#endif
}
