/* Precision shim for building the reference OpenMP programs in double precision.
 *
 * Test infrastructure only (the oracle).  Force-included ahead of the reference
 * sources so that the reference's include/utils.hpp (guard UTILS_HPP) is skipped
 * and `real` is double (as CRS/OpenMP/include/utils.hpp:35-41 ships it). */
#ifndef UTILS_HPP
#define UTILS_HPP
#define DOUBLE
#include <string>
#include <cstdlib>
#include <sstream>
#include <cmath>
#include <sys/time.h>
#define real double
#define SQRT(x) sqrt(x)
#endif
