/*
 * Native trust-region fit of a brickwall circuit against a GPU target, with the
 * evaluations on device-resident plans and a switch from float-float to complex128
 * evaluations near convergence.
 *
 * The loop is the reference's riemannian_trust_region_optimize_hmat
 * (src/trust_region.c:235-306) driven as optimize_matchgate_brickwall_circuit_hmat drives it
 * (src/mg_brickwall_opt.c:99-122): target Re f, Riemannian gradient and Hessian
 * (src/matchgate_target.c:877-973), Steihaug tCG, retraction per layer, the rho test
 * (rho < 1/4 shrinks the radius by 4, rho > 3/4 on the boundary doubles it up to maxradius,
 * the step is taken when rho > rho_trust).  mg_optimize_circuit runs the same loop on a
 * general circuit with one parameter block per gate.  The last f_iter entry, f at the final
 * iterate, reuses the evaluation of the accepted trial point that became that iterate (the
 * reference evaluates the same point once more; the value is the same, bit for bit).
 *
 * The target does not change during a fit, so (MG_OPT_FIT_RESIDENT 0, the default) its
 * conjugated columns stay on the GPU after the first evaluation when they take at most a
 * quarter of the free device memory, and every later evaluation skips the target sweep; the
 * columns are the same the sweep would produce (same program, same bits), and they are
 * released when the fit ends unless the caller had made the target resident itself.
 */
#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "matchgate_target.h"
#include "trust_region.h"
#include "mg_gb300.h"
#include "../mg_internal.h"

/* the circuit the fit optimises: a brickwall (one gate per layer, perms) or a general
 * circuit (one parameter block per gate, wires) */
typedef struct
{
	int L, nblocks;
	const int** perms;    /* brickwall: [nblocks][L] */
	const int* wires;     /* circuit: [2 nblocks] */
} fit_t;

typedef struct { mg_plan* h; mg_plan* f; int prec; } plans_t;

static void plans_free(plans_t* p)
{
	if (p->h) mg_plan_free(p->h);
	if (p->f) mg_plan_free(p->f);
	p->h = p->f = NULL;
}

static int plans_make(plans_t* p, void* target, const struct matchgate* v, const fit_t* fit, int prec)
{
	plans_free(p);
	const int old = mg_get_precision();
	mg_set_precision(prec);
	const int nl = fit->nblocks, L = fit->L;
	if (fit->perms)
	{
		const int ti = mgcu_option(MG_OPT_TRANSLATIONAL_INVARIANCE_ID) != 0;
		p->h = mg_plan_brickwall(mg_target_apply, target, v, nl, L, fit->perms, MG_EVAL_HESSIAN | (ti ? MG_EVAL_TI : 0));
		p->f = p->h ? mg_plan_brickwall(mg_target_apply, target, v, nl, L, fit->perms, MG_EVAL_TARGET) : NULL;
	}
	else
	{
		p->h = mg_plan_circuit(mg_target_apply, target, v, nl, fit->wires, L, MG_EVAL_HESSIAN);
		p->f = p->h ? mg_plan_circuit(mg_target_apply, target, v, nl, fit->wires, L, MG_EVAL_TARGET) : NULL;
	}
	mg_set_precision(old);
	p->prec = prec;
	return (p->h && p->f) ? 0 : MG_ERR_DEVICE;
}

static int eval_hess(plans_t* p, const struct matchgate* v, double* f, double* grad, double* H)
{
	int rc = mg_plan_set_gates(p->h, v);
	if (!rc) rc = mg_plan_run(p->h);
	numeric fc = 0;
	if (!rc) rc = mg_plan_results(p->h, &fc, NULL, NULL, grad, H);
	if (!rc) *f = creal(fc);
	return rc;
}

static int eval_f(plans_t* p, const struct matchgate* v, double* f)
{
	int rc = mg_plan_set_gates(p->f, v);
	if (!rc) rc = mg_plan_run(p->f);
	numeric fc = 0;
	if (!rc) rc = mg_plan_results(p->f, &fc, NULL, NULL, NULL, NULL);
	if (!rc) *f = creal(fc);
	return rc;
}

static int optimize(void* target, const struct matchgate vlist0[], const fit_t* fit, const struct rtr_params* params, int niter,
	double refine_gnorm, double f_iter[], int prec_iter[], struct matchgate vlist_out[])
{
	const int nlayers = fit->nblocks;
	const int n = 8 * nlayers;
	struct matchgate* x = malloc(sizeof(struct matchgate) * nlayers);
	struct matchgate* xn = malloc(sizeof(struct matchgate) * nlayers);
	double* grad = malloc(sizeof(double) * n);
	double* H = malloc(sizeof(double) * (size_t)n * n);
	double* eta = malloc(sizeof(double) * n);
	if (!x || !xn || !grad || !H || !eta) { free(x); free(xn); free(grad); free(H); free(eta); return MG_ERR_ALLOC; }
	memcpy(x, vlist0, sizeof(struct matchgate) * nlayers);
	plans_t pl = { 0 };
	int prec = refine_gnorm > 0 ? MG_PREC_MIXED : MG_PREC_FP64;
	int made_resident = 0;
	if (mgcu_option(MG_OPT_FIT_RESIDENT_ID) != 1 && mgh_target_resident(target) == 0)
	{
		const double bytes = ldexp(1.0, 2 * fit->L - 1) * 16.0;   /* float-float and complex128 columns */
		if (bytes <= 0.25 * mgcu_device_free_bytes() && mg_target_set_resident(target, 1) == 0) made_resident = 1;
	}
	int rc = plans_make(&pl, target, x, fit, prec);
	double radius = params->radius_init;
	/* f of the current iterate from a target-only evaluation at the current precision, when
	 * one was made (the trial point of an accepted step): the final f_iter entry reuses it
	 * instead of evaluating the same point again, with the same plan and the same bits */
	double fcur = 0;
	int fcur_ok = 0;
	for (int k = 0; k < niter && !rc; k++)
	{
		double fx;
		rc = eval_hess(&pl, x, &fx, grad, H);
		if (rc) break;
		if (prec == MG_PREC_MIXED)
		{
			double g2 = 0;
			for (int i = 0; i < n; i++) g2 += grad[i] * grad[i];
			if (sqrt(g2) < refine_gnorm)
			{
				/* near convergence: complex128 from here on, this iterate re-evaluated */
				prec = MG_PREC_FP64;
				fcur_ok = 0;
				rc = plans_make(&pl, target, x, fit, prec);
				if (!rc) rc = eval_hess(&pl, x, &fx, grad, H);
				if (rc) break;
			}
		}
		f_iter[k] = fx;
		if (prec_iter) prec_iter[k] = prec;
		const bool on_boundary = truncated_cg_hmat(grad, H, n, radius, &params->tcg_params, eta);
		for (int l = 0; l < nlayers; l++) retract_matchgate(&x[l], eta + 8 * l, &xn[l]);
		double fn;
		rc = eval_f(&pl, xn, &fn);
		if (rc) break;
		double ge = 0, eHe = 0;
		for (int i = 0; i < n; i++)
		{
			double s = 0;
			for (int j = 0; j < n; j++) s += H[(size_t)i * n + j] * eta[j];
			ge += grad[i] * eta[i];
			eHe += eta[i] * s;
		}
		const double rho = (fn - fx) / (ge + 0.5 * eHe);
		if (rho < 0.25) radius *= 0.25;
		else if (rho > 0.75 && on_boundary) radius = fmin(2 * radius, params->maxradius);
		if (rho > params->rho_trust)
		{
			memcpy(x, xn, sizeof(struct matchgate) * nlayers);
			fcur = fn;
			fcur_ok = 1;
		}
	}
	if (!rc)
	{
		if (fcur_ok) f_iter[niter] = fcur;
		else rc = eval_f(&pl, x, &f_iter[niter]);
		if (prec_iter) prec_iter[niter] = prec;
		memcpy(vlist_out, x, sizeof(struct matchgate) * nlayers);
	}
	plans_free(&pl);
	if (made_resident) mg_target_set_resident(target, 0);
	free(x); free(xn); free(grad); free(H); free(eta);
	return rc;
}

int mg_optimize_brickwall(void* target, const struct matchgate vlist0[], int nlayers, int nqubits, const int* perms[],
	const struct rtr_params* params, int niter, double refine_gnorm, double f_iter[], int prec_iter[],
	struct matchgate vlist_out[])
{
	if (!target || !vlist0 || nlayers < 1 || !perms || !params || niter < 0 || !f_iter || !vlist_out)
	{
		mg_set_error("mg_optimize_brickwall: bad arguments");
		return MG_ERR_ARG;
	}
	const fit_t fit = { nqubits, nlayers, perms, NULL };
	return optimize(target, vlist0, &fit, params, niter, refine_gnorm, f_iter, prec_iter, vlist_out);
}

/* the same loop with one parameter block per gate of a general circuit: the per-gate
 * Riemannian gradient and Hessian (8 ngates real parameters), retraction per gate */
int mg_optimize_circuit(void* target, const struct matchgate gates0[], int ngates, const int wires[], int nqubits,
	const struct rtr_params* params, int niter, double refine_gnorm, double f_iter[], int prec_iter[],
	struct matchgate gates_out[])
{
	if (!target || !gates0 || ngates < 1 || !wires || !params || niter < 0 || !f_iter || !gates_out)
	{
		mg_set_error("mg_optimize_circuit: bad arguments");
		return MG_ERR_ARG;
	}
	const fit_t fit = { nqubits, ngates, NULL, wires };
	return optimize(target, gates0, &fit, params, niter, refine_gnorm, f_iter, prec_iter, gates_out);
}
