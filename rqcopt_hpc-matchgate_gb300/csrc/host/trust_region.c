/*
 * Riemannian trust-region optimisation (reference src/trust_region.c; Absil, Mahony,
 * Sepulchre, "Optimization Algorithms on Matrix Manifolds", Alg. 10 and 11).  The
 * subproblem on an explicit Hessian (Steihaug truncated CG) and the model decrease
 * H eta run on the GPU in FP64; the outer loop drives the caller's callbacks.
 */
#include <assert.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include "trust_region.h"
#include "../mg_internal.h"

static double dot(const double* a, const double* b, int n)
{
	double s = 0;
	for (int i = 0; i < n; i++) s += a[i] * b[i];
	return s;
}

bool truncated_cg_hmat(const double* grad, const double* hess, int n, double radius, const struct truncated_cg_params* params, double* z)
{
	mgcu_lock();
	const int r = mgcu_truncated_cg(grad, hess, n, radius, params->maxiter, params->abstol, params->reltol, z);
	mgcu_unlock();
	if (r < 0)
	{
		fprintf(stderr, "truncated_cg_hmat failed on the GPU: %s\n", mg_last_error());
		memset(z, 0, sizeof(double) * n);
		return false;
	}
	return r == 1;
}

/* t > 0 with ||b + t d|| = radius (reference src/trust_region.c:17-74) */
static double to_boundary(const double* b, const double* d, int n, double radius)
{
	const double dd = dot(d, d, n);
	if (dd == 0) { fprintf(stderr, "input vector 'd' is zero\n"); return 0; }
	const double p = dot(b, d, n) / dd;
	const double q = (dot(b, b, n) - radius * radius) / dd;
	if (p == 0) return sqrt(-q);
	const double a = -(p + copysign(1.0, p) * sqrt(p * p - q));
	const double c = q / a;
	return a <= c ? c : a;
}

/* truncated CG with a caller-supplied Hessian-vector product (reference
 * src/trust_region.c:163-221); the products are the caller's, the O(n) vector
 * updates between them are negligible. */
bool truncated_cg_hvp(const double* restrict x, const double* restrict grad, const hessian_vector_product_func f_hvp, void* fdata, const int n, const double radius, const struct truncated_cg_params* params, double* restrict z)
{
	double* r = malloc(sizeof(double) * n);
	double* d = malloc(sizeof(double) * n);
	double* hd = malloc(sizeof(double) * n);
	if (!r || !d || !hd) { free(r); free(d); free(hd); return false; }
	memcpy(r, grad, sizeof(double) * n);
	double rsq = dot(r, r, n);
	const double stoptol = fmax(params->abstol, params->reltol * sqrt(rsq));
	memset(z, 0, sizeof(double) * n);
	for (int i = 0; i < n; i++) d[i] = -r[i];
	bool boundary = false;
	for (int it = 0; it < params->maxiter; it++)
	{
		f_hvp(x, fdata, d, hd);
		const double dhd = dot(d, hd, n);
		const double tb = to_boundary(z, d, n, radius);
		const double alpha = rsq / dhd;
		if (dhd <= 0 || alpha > tb)
		{
			for (int i = 0; i < n; i++) z[i] += tb * d[i];
			boundary = true;
			break;
		}
		for (int i = 0; i < n; i++) { r[i] += alpha * hd[i]; z[i] += alpha * d[i]; }
		const double rsq1 = dot(r, r, n);
		if (sqrt(rsq1) <= stoptol) break;
		const double beta = rsq1 / rsq;
		for (int i = 0; i < n; i++) d[i] = beta * d[i] - r[i];
		rsq = rsq1;
	}
	free(hd); free(d); free(r);
	return boundary;
}

static void matvec(const double* H, const double* x, int n, double* y)
{
	mgcu_lock();
	const int r = mgcu_matvec(H, x, n, y);
	mgcu_unlock();
	if (r) fprintf(stderr, "Hessian-vector product failed on the GPU: %s\n", mg_last_error());
}

/* reference src/trust_region.c:235-306 */
void riemannian_trust_region_optimize_hmat(target_func f, target_gradient_hessian_func f_deriv_hess, void* fdata, retract_func retract, void* rdata,
	const int n, const double* x_init, const int m, const struct rtr_params* params, const int niter, double* f_iter, numeric* f_citer, double* x_final)
{
	assert(0 <= params->rho_trust && params->rho_trust < 0.25);
	double* x = malloc(sizeof(double) * m);
	double* x_next = malloc(sizeof(double) * m);
	double* grad = malloc(sizeof(double) * n);
	double* hess = malloc(sizeof(double) * (size_t)n * n);
	double* eta = malloc(sizeof(double) * n);
	double* heta = malloc(sizeof(double) * n);
	if (!x || !x_next || !grad || !hess || !eta || !heta)
	{
		fprintf(stderr, "riemannian_trust_region_optimize_hmat: out of memory\n");
		free(x); free(x_next); free(grad); free(hess); free(eta); free(heta);
		return;
	}
	memcpy(x, x_init, sizeof(double) * m);
	double radius = params->radius_init;
	if (params->g_func != NULL)
	{
		numeric g;
		params->g_iter[0] = params->g_func(x, params->g_data, &g);
	}
	for (int k = 0; k < niter; k++)
	{
		numeric fc;
		const double fx = f_deriv_hess(x, fdata, &fc, grad, hess);
		const bool on_boundary = truncated_cg_hmat(grad, hess, n, radius, &params->tcg_params, eta);
		retract(x, eta, rdata, x_next);
		f_iter[k] = fx;
		f_citer[k] = fc;
		matvec(hess, eta, n, heta);
		const double rho = (f(x_next, fdata, &fc) - fx) / (dot(grad, eta, n) + 0.5 * dot(eta, heta, n));
		if (rho < 0.25) radius *= 0.25;
		else if (rho > 0.75 && on_boundary) radius = fmin(2 * radius, params->maxradius);
		if (rho > params->rho_trust) { double* y = x; x = x_next; x_next = y; }
		if (params->g_func != NULL)
		{
			numeric g;
			params->g_iter[k + 1] = params->g_func(x, params->g_data, &g);
		}
	}
	memcpy(x_final, x, sizeof(double) * m);
	numeric fc;
	f_iter[niter] = f(x_final, fdata, &fc);
	f_citer[niter] = fc;
	free(heta); free(eta); free(hess); free(grad); free(x_next); free(x);
}

/* The reference declares this variant (src/trust_region.h:84-86) without a body; here
 * it is the loop above with the gradient from f_deriv and the subproblem solved by
 * truncated_cg_hvp. */
void riemannian_trust_region_optimize_hvp(const target_func f, const target_gradient_func f_deriv, const hessian_vector_product_func f_hvp, void* fdata,
	retract_func retract, void* rdata,
	const int n, const double* x_init, const int m, const struct rtr_params* params, const int niter, double* f_iter, double* x_final)
{
	assert(0 <= params->rho_trust && params->rho_trust < 0.25);
	double* x = malloc(sizeof(double) * m);
	double* x_next = malloc(sizeof(double) * m);
	double* grad = malloc(sizeof(double) * n);
	double* eta = malloc(sizeof(double) * n);
	double* heta = malloc(sizeof(double) * n);
	if (!x || !x_next || !grad || !eta || !heta)
	{
		fprintf(stderr, "riemannian_trust_region_optimize_hvp: out of memory\n");
		free(x); free(x_next); free(grad); free(eta); free(heta);
		return;
	}
	memcpy(x, x_init, sizeof(double) * m);
	double radius = params->radius_init;
	if (params->g_func != NULL)
	{
		numeric g;
		params->g_iter[0] = params->g_func(x, params->g_data, &g);
	}
	for (int k = 0; k < niter; k++)
	{
		const double fx = f_deriv(x, fdata, grad);
		const bool on_boundary = truncated_cg_hvp(x, grad, f_hvp, fdata, n, radius, &params->tcg_params, eta);
		retract(x, eta, rdata, x_next);
		f_iter[k] = fx;
		f_hvp(x, fdata, eta, heta);
		numeric fc;
		const double rho = (f(x_next, fdata, &fc) - fx) / (dot(grad, eta, n) + 0.5 * dot(eta, heta, n));
		if (rho < 0.25) radius *= 0.25;
		else if (rho > 0.75 && on_boundary) radius = fmin(2 * radius, params->maxradius);
		if (rho > params->rho_trust) { double* y = x; x = x_next; x_next = y; }
		if (params->g_func != NULL)
		{
			numeric g;
			params->g_iter[k + 1] = params->g_func(x, params->g_data, &g);
		}
	}
	memcpy(x_final, x, sizeof(double) * m);
	numeric fc;
	f_iter[niter] = f(x_final, fdata, &fc);
	free(heta); free(eta); free(grad); free(x_next); free(x);
}
