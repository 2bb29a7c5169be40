/*
 * Library-wide state of the host layer: the error message of the last failing call,
 * the API lock, and the precision / tuning settings of mg_gb300.h.
 */
#define _GNU_SOURCE
#include <pthread.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include "mg_gb300.h"
#include "../mg_internal.h"

static __thread char g_err[512];

void mg_set_error(const char* fmt, ...)
{
	va_list ap;
	va_start(ap, fmt);
	vsnprintf(g_err, sizeof(g_err), fmt, ap);
	va_end(ap);
	fprintf(stderr, "matchgate-gb300: %s\n", g_err);
}

const char* mg_last_error(void) { return g_err; }

/* one recursive lock serialises the library's GPU work (one stream per process) */
static pthread_mutex_t g_lock = PTHREAD_RECURSIVE_MUTEX_INITIALIZER_NP;
void mgcu_lock(void) { pthread_mutex_lock(&g_lock); }
void mgcu_unlock(void) { pthread_mutex_unlock(&g_lock); }

static int g_precision = MG_PREC_FP64;
static long g_options[MG_NOPTIONS + 1];

int mg_set_precision(int precision)
{
	if (precision != MG_PREC_FP64 && precision != MG_PREC_MIXED && precision != MG_PREC_FP32)
	{
		mg_set_error("unknown precision %d", precision);
		return MG_ERR_ARG;
	}
	mgcu_lock();
	g_precision = precision;
	mgcu_unlock();
	return 0;
}

int mg_get_precision(void) { return g_precision; }
int mgcu_precision(void) { return g_precision; }

int mg_set_option(int option, long value)
{
	if (option < 1 || option > MG_NOPTIONS || value < 0)
	{
		mg_set_error("invalid option %d = %ld", option, value);
		return MG_ERR_ARG;
	}
	mgcu_lock();
	g_options[option] = value;
	mgcu_unlock();
	return 0;
}

long mg_get_option(int option) { return (option >= 1 && option <= MG_NOPTIONS) ? g_options[option] : -1; }
long mgcu_option(int option) { return mg_get_option(option); }

long mg_launch_count(void) { return mgcu_launch_count(); }

double mg_measure_fp32_peak_gflops(void)
{
	mgcu_lock();
	double r = mgcu_fp32_peak_gflops();
	mgcu_unlock();
	return r;
}

double mg_measure_fp64_peak_gflops(void)
{
	mgcu_lock();
	double r = mgcu_fp64_peak_gflops();
	mgcu_unlock();
	return r;
}
