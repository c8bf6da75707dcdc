/*
 * CPU restatement of the reference DUGKS step -- the oracle.
 *
 * TEST INFRASTRUCTURE ONLY: built into oracle/liboracle.so, called by tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline legs as the checker and
 * the timed CPU port.  The product library never links it.
 *
 * Compiled with -ffp-contract=off so that the x86 container and the Arm GPU
 * host give identical results for the same inputs.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>

#include "dugks_oracle.h"

/* D3Q19 velocity set in the reference's population order, src/lbm_d3q19.cu:12-15. */
static const int CIX[19] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0};
static const int CIY[19] = {0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1};
static const int CIZ[19] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1};

int oracle_max_threads(void) { return omp_get_max_threads(); }

#define REAL double
#define SFX _f64
#include "dugks_oracle_impl.h"
#undef REAL
#undef SFX
#undef IDX
#undef SIDX

#define REAL float
#define SFX _f32
#include "dugks_oracle_impl.h"
#undef REAL
#undef SFX
