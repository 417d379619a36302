/*
 * CPU oracle for the batched HDBSCAN path (test infrastructure only).
 *
 * Compiled by oracle/Makefile (and by __graft_entry__.build()) into
 * oracle/libhdb_oracle.so.  Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py load it, as the checker; the product library
 * (hdbscan_gb300/) never links or calls it.
 *
 * Parity pin: tests/test_oracle.py checks this restatement against golden
 * vectors generated from scikit-learn and from the reference's own kernel
 * sources compiled for the CPU (tests/golden/make_golden.py).
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define REAL float
#define SUF f32
#define SQRT sqrtf
#define FMAX fmaxf
#define REAL_MAX_VALUE 3.4028234663852886e+38F
#include "hdb_oracle_body.h"
#undef REAL
#undef SUF
#undef SQRT
#undef FMAX
#undef REAL_MAX_VALUE

#define REAL double
#define SUF f64
#define SQRT sqrt
#define FMAX fmax
#define REAL_MAX_VALUE 1.7976931348623157e+308
#include "hdb_oracle_body.h"
#undef REAL
#undef SUF
#undef SQRT
#undef FMAX
#undef REAL_MAX_VALUE

int hdb_oracle_version(void) { return 1; }
