/*
 * Distances between numeric vectors (drop-in for the distance helpers of the
 * reference's src/util.h:12-24).  The reference's HDF5 file helpers
 * (src/util.h:27-35) are not part of this library.
 */
#pragma once

#include <math.h>
#include "config.h"

static inline double reldist(numeric x, numeric y, double eps)
{
	return _abs(x - y) / fmax(_abs(x) + _abs(y), eps);
}

double uniform_distance_real(long n, const double* x, const double* y);

double uniform_distance(long n, const numeric* x, const numeric* y);

double relative_distance(long n, const numeric* x, const numeric* y, double eps);
