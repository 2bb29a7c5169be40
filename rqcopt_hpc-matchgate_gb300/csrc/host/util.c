/* Distances between vectors (reference src/util.c:8-49). */
#include "util.h"

double uniform_distance_real(long n, const double* x, const double* y)
{
	double d = 0;
	for (long i = 0; i < n; i++) d = fmax(d, fabs(x[i] - y[i]));
	return d;
}

double uniform_distance(long n, const numeric* x, const numeric* y)
{
	double d = 0;
	for (long i = 0; i < n; i++) d = fmax(d, _abs(x[i] - y[i]));
	return d;
}

double relative_distance(long n, const numeric* x, const numeric* y, double eps)
{
	double d = 0;
	for (long i = 0; i < n; i++) d = fmax(d, reldist(x[i], y[i], eps));
	return d;
}
