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

/* A brickwall of matchgates applied on the host, the caller-side map of the reference's
 * benchmark drivers (benchmark_hpc/benchmark_threads.c:24-33 hand
 * apply_matchgate_brickwall_unitary to the library as `ufunc`).  udata points to
 * struct mgt_brickwall: nlayers gates of 8 entries (center block row-major, then corner
 * block), each applied to all L/2 pairs (perms[2p], perms[2p+1]) of its layer; qubit 0 is
 * the most significant bit of the index.  Re-entrant: it may be called from many threads. */
struct mgt_brickwall { const double complex* gates; const int* perms; int nlayers; };

int mgt_brickwall_ufunc(const struct mgt_statevector* psi, void* udata, struct mgt_statevector* out)
{
	const struct mgt_brickwall* bw = (const struct mgt_brickwall*)udata;
	const int L = psi->nqubits;
	const long n = 1L << L;
	for (long i = 0; i < n; i++) out->data[i] = psi->data[i];
	for (int l = 0; l < bw->nlayers; l++)
	{
		const double complex* g = bw->gates + 8 * l;
		for (int p = 0; p < L / 2; p++)
		{
			const int qi = bw->perms[l * L + 2 * p], qj = bw->perms[l * L + 2 * p + 1];
			const long mi = 1L << (L - 1 - qi), mj = 1L << (L - 1 - qj);
			for (long a = 0; a < n; a++)
			{
				if (a & (mi | mj)) continue;
				const long x = a, y = a | mj, z = a | mi, w = a | mi | mj;   /* local 00, 01, 10, 11 */
				const double complex X = out->data[x], Y = out->data[y], Z = out->data[z], W = out->data[w];
				out->data[y] = g[0] * Y + g[1] * Z;
				out->data[z] = g[2] * Y + g[3] * Z;
				out->data[x] = g[4] * X + g[5] * W;
				out->data[w] = g[6] * X + g[7] * W;
			}
		}
	}
	return 0;
}
