/*
 * Brickwall sweeps on one host vector (reference src/matchgate_brickwall.c), run on
 * the GPU.  Layer l applies vlist[l] to the pairs (perms[l][2p], perms[l][2p+1]).
 */
#include <assert.h>
#include <stdio.h>
#include <string.h>

#include "matchgate_brickwall.h"
#include "../mg_internal.h"

int mg_circuit_forward_host(const struct matchgate gates[], const int ngates, const int wires[], int L,
	const numeric* psi, struct quantum_circuit_cache* cache, numeric* out);
int mg_circuit_backward_host(const struct matchgate gates[], const int ngates, const int wires[], int L,
	const struct quantum_circuit_cache* cache, const numeric* dpsi_out, numeric* dpsi, struct matchgate dgates[]);

/* the equivalent sequential circuit (reference src/matchgate_target.c:308-324) */
static int expand(const struct matchgate vlist[], int nlayers, const int* perms[], int L, struct matchgate** gates, int** wires)
{
	const int half = L / 2, ng = nlayers * half;
	*gates = malloc(sizeof(struct matchgate) * (ng > 0 ? ng : 1));
	*wires = malloc(sizeof(int) * 2 * (ng > 0 ? ng : 1));
	if (!*gates || !*wires) { free(*gates); free(*wires); return -1; }
	for (int i = 0; i < nlayers; i++)
		for (int p = 0; p < half; p++)
		{
			(*gates)[i * half + p] = vlist[i];
			(*wires)[2 * (i * half + p)] = perms[i][2 * p];
			(*wires)[2 * (i * half + p) + 1] = perms[i][2 * p + 1];
		}
	return 0;
}

int apply_matchgate_brickwall_unitary(const struct matchgate vlist[], const int nlayers, const int* perms[],
	const struct statevector* restrict psi, struct statevector* restrict psi_out)
{
	assert(nlayers >= 1 && psi->nqubits == psi_out->nqubits);
	struct matchgate* g; int* w;
	if (expand(vlist, nlayers, perms, psi->nqubits, &g, &w)) return -1;
	int r = mg_circuit_forward_host(g, nlayers * (psi->nqubits / 2), w, psi->nqubits, psi->data, NULL, psi_out->data);
	free(g); free(w);
	return r ? -1 : 0;
}

int matchgate_brickwall_unitary_forward(const struct matchgate vlist[], int nlayers, const int* perms[],
	const struct statevector* restrict psi, struct quantum_circuit_cache* cache, struct statevector* restrict psi_out)
{
	assert(nlayers >= 1 && psi->nqubits % 2 == 0);
	assert(cache->ngates == nlayers * (psi->nqubits / 2) && cache->nqubits == psi->nqubits);
	struct matchgate* g; int* w;
	if (expand(vlist, nlayers, perms, psi->nqubits, &g, &w)) return -1;
	int r = mg_circuit_forward_host(g, cache->ngates, w, psi->nqubits, psi->data, cache, psi_out->data);
	free(g); free(w);
	return r ? -1 : 0;
}

int matchgate_brickwall_unitary_backward(const struct matchgate vlist[], int nlayers, const int* perms[], const struct quantum_circuit_cache* cache,
	const struct statevector* restrict dpsi_out, struct statevector* restrict dpsi, struct matchgate dvlist[])
{
	const int L = dpsi->nqubits, half = L / 2, ng = nlayers * half;
	assert(nlayers >= 1 && L % 2 == 0 && cache->ngates == ng && cache->nqubits == L);
	struct matchgate* g; int* w;
	if (expand(vlist, nlayers, perms, L, &g, &w)) return -1;
	struct matchgate* dg = malloc(sizeof(struct matchgate) * ng);
	if (!dg) { free(g); free(w); return -1; }
	int r = mg_circuit_backward_host(g, ng, w, L, cache, dpsi_out->data, dpsi->data, dg);
	if (!r)
		/* per-layer sums, last pair first as in src/matchgate_brickwall.c:102-123 */
		for (int i = nlayers - 1; i >= 0; i--)
		{
			zero_matchgate(&dvlist[i]);
			for (int p = half - 1; p >= 0; p--) add_matchgate(&dvlist[i], &dg[i * half + p]);
		}
	free(dg); free(g); free(w);
	return r ? -1 : 0;
}

static int backward_hessian(const struct matchgate vlist[], int nlayers, const int* perms[], const struct quantum_circuit_cache* cache,
	const struct statevector* restrict dpsi_out, struct statevector* restrict dpsi, struct matchgate dvlist[], numeric* hess, int ti)
{
	const int L = dpsi->nqubits, ng = nlayers * (L / 2);
	assert(nlayers >= 1 && L % 2 == 0 && cache->ngates == ng && cache->nqubits == L);
	const size_t n = (size_t)1 << L;
	numeric* flat = malloc(n * ng * sizeof(numeric));
	int* pf = malloc(sizeof(int) * nlayers * L);
	if (!flat || !pf) { free(flat); free(pf); return -1; }
	for (int k = 0; k < ng; k++) memcpy(flat + (size_t)k * n, cache->psi_list[k].data, n * sizeof(numeric));
	for (int i = 0; i < nlayers; i++) memcpy(pf + i * L, perms[i], sizeof(int) * L);
	mgcu_lock();
	int r = mgcu_brickwall_backward_hessian((const mgg*)vlist, nlayers, pf, L, ti, (const mgc*)flat, (const mgc*)dpsi_out->data,
		(mgc*)dpsi->data, (mgg*)dvlist, (mgc*)hess);
	mgcu_unlock();
	free(pf); free(flat);
	return r ? -1 : 0;
}

int matchgate_brickwall_unitary_backward_hessian(const struct matchgate vlist[], int nlayers, const int* perms[], const struct quantum_circuit_cache* cache,
	const struct statevector* restrict dpsi_out, struct statevector* restrict dpsi, struct matchgate dvlist[], numeric* hess)
{
	return backward_hessian(vlist, nlayers, perms, cache, dpsi_out, dpsi, dvlist, hess, 0);
}

int matchgate_ti_brickwall_unitary_backward_hessian(const struct matchgate vlist[], int nlayers, const int* perms[], const struct quantum_circuit_cache* cache,
	const struct statevector* restrict dpsi_out, struct statevector* restrict dpsi, struct matchgate dvlist[], numeric* hess)
{
	return backward_hessian(vlist, nlayers, perms, cache, dpsi_out, dpsi, dvlist, hess, 1);
}
