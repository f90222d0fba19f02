/* Oracle for the CMP/CRS semblance search: a CPU restatement of the reference's
 * OpenMP programs (CMP/OpenMP/src/main.cpp, CRS/OpenMP/src/main.cpp).
 *
 * TEST INFRASTRUCTURE ONLY: used by tests/ as the checker of the CUDA path and by
 * bench.py as the timed CPU baseline.  It is never linked into the product.
 *
 * Parity pinning: tests/test_oracle_pins.py runs the reference's own programs
 * (built from their sources by this directory's Makefile into _ref/) on seeded
 * synthetic inputs and requires this restatement to reproduce their SU outputs
 * bit for bit; tests/golden/ holds those reference outputs so the pin also holds
 * where the reference tree is absent.
 *
 * Constants follow the reference: EPSILON 1e-13 and FACTOR 1e6 (both files'
 * :41-43), MAX_W 16 for CMP (CMP/OpenMP/src/main.cpp:39) and 5 for CRS
 * (CRS/OpenMP/src/main.cpp:39; the reference never checks it, here a larger
 * window is an error). */
#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define EPSILON 1e-13
#define FACTOR 1e6
#define MAX_W_CMP 16
#define MAX_W_CRS 5

/* CRS midpoint displacement switch, read by the restatement (semb_oracle_set_dm) */
static int semb_oracle_dm_signed = 0;
static double semb_oracle_dm_cos = 1.0, semb_oracle_dm_sin = 0.0;

/* Sampling of the checker (semb_oracle_set_t0, semb_oracle_set_top2): the searches
 * evaluate only output samples t0 in [t0_lo, t0_hi) (the other rows are left as the
 * caller initialised them), and, when top2 is set, write per (CDP, t0) the gap
 * between the best and the second-best candidate semblance (double).  Neither
 * changes the arithmetic of an evaluated item. */
static int semb_oracle_t0_lo = 0, semb_oracle_t0_hi = 0x7fffffff;
static double* semb_oracle_top2 = 0;

#define REAL float
#define SQRTR sqrtf
#define SFX _f32
#include "semb_oracle_body.h"
#undef REAL
#undef SQRTR
#undef SFX

#define REAL double
#define SQRTR sqrt
#define SFX _f64
#include "semb_oracle_body.h"
#undef REAL
#undef SQRTR
#undef SFX

int semb_oracle_max_threads(void) { return omp_get_max_threads(); }
void semb_oracle_set_threads(int n) { if (n > 0) omp_set_num_threads(n); }

/* CRS midpoint displacement of the next searches: 0 = |dm| (the reference), 1 =
 * dm projected on the azimuth direction (cos, sin), signed, with dm^2 = dm * dm.
 * The signed operator is this build's extension (SEMB_DM_SIGNED); the reference
 * has no counterpart, so this branch restates the library's definition. */
void semb_oracle_set_dm(int signed_dm, double azimuth_deg) {
  const double az = azimuth_deg * 3.14159265358979323846 / 180.0;
  semb_oracle_dm_signed = signed_dm ? 1 : 0;
  semb_oracle_dm_cos = cos(az);
  semb_oracle_dm_sin = sin(az);
}

/* Evaluate only t0 in [lo, hi) in the next searches (hi <= lo: every t0). */
void semb_oracle_set_t0(int lo, int hi) {
  if (hi <= lo) { lo = 0; hi = 0x7fffffff; }
  semb_oracle_t0_lo = lo < 0 ? 0 : lo;
  semb_oracle_t0_hi = hi;
}

/* Per (CDP, t0) gap best - second best of the next searches into out[ncdps * ns]
 * (NULL: off). */
void semb_oracle_set_top2(double* out) { semb_oracle_top2 = out; }
