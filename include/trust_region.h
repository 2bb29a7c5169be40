/*
 * Riemannian trust-region optimisation with a truncated-CG subproblem solver
 * (drop-in for the reference's src/trust_region.h:1-90; the MPI variant is not
 * provided).  The subproblem is solved on the GPU in FP64.
 */
#pragma once

#include <stdbool.h>
#include "config.h"

/* src/trust_region.h:11-18 */
struct truncated_cg_params
{
	int maxiter;
	double abstol;
	double reltol;
};

/* src/trust_region.h:24-29 */
static inline void set_truncated_cg_default_params(int n, struct truncated_cg_params* params)
{
	params->maxiter = 2 * n;
	params->abstol  = 1e-8;
	params->reltol  = 1e-6;
}

/* src/trust_region.c:88 -- returns true when the step ends on the boundary */
bool truncated_cg_hmat(const double* grad, const double* hess, int n, double radius, const struct truncated_cg_params* params, double* z);

typedef void (*hessian_vector_product_func)(const double* restrict x, void* fdata, double* restrict vec, double* restrict hvp);

/* src/trust_region.c:164 */
bool truncated_cg_hvp(const double* restrict x, const double* restrict grad, const hessian_vector_product_func f_hvp, void* fdata, const int n, const double radius, const struct truncated_cg_params* params, double* restrict z);

typedef double (*target_func)(const double* x, void* fdata, numeric* f_complex);

typedef double (*target_gradient_func)(const double* restrict x, void* fdata, double* restrict grad);

typedef double (*target_gradient_hessian_func)(const double* restrict x, void* fdata, numeric* complex_f, double* restrict grad, double* restrict hess);

typedef void (*retract_func)(const double* restrict x, const double* restrict eta, void* rdata, double* restrict xs);

/* src/trust_region.h:53-63 */
struct rtr_params
{
	struct truncated_cg_params tcg_params;
	double rho_trust;
	double radius_init;
	double maxradius;
	target_func g_func;
	void*       g_data;
	double*     g_iter;
};

/* src/trust_region.h:69-78 */
static inline void set_rtr_default_params(int n, struct rtr_params* params)
{
	set_truncated_cg_default_params(n, &params->tcg_params);
	params->rho_trust   = 0.125;
	params->radius_init = 0.01;
	params->maxradius   = 0.1;
	params->g_func      = NULL;
	params->g_data      = NULL;
	params->g_iter      = NULL;
}

/* src/trust_region.c:235 */
void riemannian_trust_region_optimize_hmat(target_func f, target_gradient_hessian_func f_deriv_hess, void* fdata, retract_func retract, void* rdata,
	const int n, const double* x_init, const int m, const struct rtr_params* params, const int niter, double* f_iter, numeric* f_citer, double* x_final);

/* declared by the reference (src/trust_region.h:84-86) without a definition; here it
 * runs the same loop with truncated_cg_hvp as the subproblem solver */
void riemannian_trust_region_optimize_hvp(const target_func f, const target_gradient_func f_deriv, const hessian_vector_product_func f_hvp, void* fdata,
	retract_func retract, void* rdata,
	const int n, const double* x_init, const int m, const struct rtr_params* params, const int niter, double* f_iter, double* x_final);
