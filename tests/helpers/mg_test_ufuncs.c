/*
 * Test-side target maps with the reference's `linear_func` signature
 * (src/matchgate_target.h:10).  They are the caller's code in the parity tests:
 * the same C function is handed to the library under test and to the reference
 * build, exactly as the reference's own tests hand their `ufunc` to it.
 *
 *  - mgt_hash_ufunc: the fixed non-unitary index-hash map of
 *    test/test_matchgate_target.c:20-34 (complex variant);
 *  - mgt_dense_ufunc: psi_out = U psi for a row-major 2^L x 2^L matrix passed as
 *    udata (test/test_matchgate_target.c:38-47).
 */
#include <complex.h>

struct mgt_statevector { double complex* data; int nqubits; };

int mgt_hash_ufunc(const struct mgt_statevector* psi, void* udata, struct mgt_statevector* out)
{
	(void)udata;
	const long n = 1L << psi->nqubits;
	for (long i = 0; i < n; i++)
		out->data[i] = (-1.1 + 0.8 * I) * psi->data[((i + 3) * 113) % n] + (0.4 - 0.7 * I) * psi->data[((i + 9) * 173) % n]
		             + (0.5 + 0.1 * I) * psi->data[i] + (-0.3 + 0.2 * I) * psi->data[((i + 4) * 199) % n];
	return 0;
}

int mgt_dense_ufunc(const struct mgt_statevector* psi, void* udata, struct mgt_statevector* out)
{
	const double complex* U = (const double complex*)udata;
	const long n = 1L << psi->nqubits;
	for (long i = 0; i < n; i++)
	{
		double complex s = 0;
		for (long j = 0; j < n; j++) s += U[i * n + j] * psi->data[j];
		out->data[i] = s;
	}
	return 0;
}

/* a ufunc that always fails, for the error-path tests (reference code -2) */
int mgt_failing_ufunc(const struct mgt_statevector* psi, void* udata, struct mgt_statevector* out)
{
	(void)psi; (void)udata; (void)out;
	return -7;
}
