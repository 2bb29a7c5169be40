/*
 * A C caller of the drop-in library, built against include/ and linked to libmgcu.so the
 * way an unchanged reference driver is: the trust-region fit of a brickwall circuit with the
 * reference's glue structure (src/mg_brickwall_opt.c:99-122 -- f and f_deriv_hess callbacks
 * over the layer gates viewed as 16 nlayers doubles, a per-layer retraction, default TR
 * parameters for 16 nlayers unknowns), written here as test code.  The parity test runs it
 * on the GPU against the oracle's restatement of the same optimiser.
 */
#include <complex.h>

#include "matchgate.h"
#include "matchgate_target.h"
#include "trust_region.h"

struct mgt_fit
{
	linear_func ufunc;
	void* udata;
	int nlayers, nqubits;
	const int** perms;
};

static double mgt_f(const double* x, void* fdata, numeric* fc)
{
	const struct mgt_fit* d = fdata;
	numeric f;
	if (matchgate_brickwall_unitary_target(d->ufunc, d->udata, (const struct matchgate*)x, d->nlayers, d->nqubits, d->perms, &f) < 0)
		return -1;
	*fc = f;
	return creal(f);
}

static double mgt_f_deriv_hess(const double* restrict x, void* fdata, numeric* fc, double* restrict grad, double* restrict hess)
{
	const struct mgt_fit* d = fdata;
	numeric f;
	if (matchgate_brickwall_unitary_target_gradient_vector_hessian_matrix(d->ufunc, d->udata, (const struct matchgate*)x,
			d->nlayers, d->nqubits, d->perms, &f, grad, hess) < 0)
		return -1;
	*fc = f;
	return creal(f);
}

static void mgt_retract(const double* restrict x, const double* restrict eta, void* rdata, double* restrict xs)
{
	const int nl = *(const int*)rdata;
	for (int i = 0; i < nl; i++)
		retract_matchgate((const struct matchgate*)x + i, eta + 8 * i, (struct matchgate*)xs + i);
}

/* niter trust-region iterations from vlist0; f_iter[niter + 1], f_citer[niter + 1] and
 * vlist_opt[nlayers] as the reference's optimize_matchgate_brickwall_circuit_hmat fills them */
int mgt_optimize_brickwall_hmat(linear_func ufunc, void* udata, const struct matchgate vlist0[], int nlayers, int nqubits,
	const int* perms[], int niter, double* f_iter, numeric* f_citer, struct matchgate vlist_opt[])
{
	struct mgt_fit d = { ufunc, udata, nlayers, nqubits, perms };
	struct rtr_params params;
	set_rtr_default_params(16 * nlayers, &params);
	int nl = nlayers;
	riemannian_trust_region_optimize_hmat(mgt_f, mgt_f_deriv_hess, &d, mgt_retract, &nl, 8 * nlayers, (const double*)vlist0,
		16 * nlayers, &params, niter, f_iter, f_citer, (double*)vlist_opt);
	return 0;
}
