/*
 * General matchgate circuits on one host vector (reference src/quantum_circuit.c).
 * The sweeps run on the GPU; the cache of intermediate states is copied back into
 * the caller's host cache.
 */
#include <assert.h>
#include <stdio.h>
#include <string.h>

#include "quantum_circuit.h"
#include "../mg_internal.h"

int allocate_quantum_circuit_cache(const int nqubits, const int ngates, struct quantum_circuit_cache* cache)
{
	assert(ngates >= 1);
	cache->nqubits = nqubits;
	cache->ngates = ngates;
	cache->psi_list = aligned_alloc(MEM_DATA_ALIGN, ((ngates * sizeof(struct statevector) + MEM_DATA_ALIGN - 1) / MEM_DATA_ALIGN) * MEM_DATA_ALIGN);
	if (cache->psi_list == NULL)
	{
		fprintf(stderr, "allocating memory for statevector array failed\n");
		return -1;
	}
	for (int i = 0; i < ngates; i++)
	{
		cache->psi_list[i].data = NULL;
		int ret = allocate_statevector(nqubits, &cache->psi_list[i]);
		if (ret < 0) return ret;
	}
	return 0;
}

void free_quantum_circuit_cache(struct quantum_circuit_cache* cache)
{
	for (int i = 0; i < cache->ngates; i++) free_statevector(&cache->psi_list[i]);
	aligned_free(cache->psi_list);
	cache->psi_list = NULL;
	cache->nqubits = 0;
	cache->ngates = 0;
}

/* run the forward sweep on the GPU; cache (optional) receives each gate's input */
int mg_circuit_forward_host(const struct matchgate gates[], const int ngates, const int wires[], int L,
	const numeric* psi, struct quantum_circuit_cache* cache, numeric* out)
{
	const size_t n = (size_t)1 << L;
	numeric* flat = NULL;
	if (cache)
	{
		flat = malloc(n * (size_t)(ngates > 0 ? ngates : 1) * sizeof(numeric));
		if (!flat) return -1;
	}
	mgcu_lock();
	int r = mgcu_circuit_forward((const mgg*)gates, wires, ngates, L, (const mgc*)psi, (mgc*)flat, (mgc*)out);
	mgcu_unlock();
	if (!r && cache)
		for (int g = 0; g < ngates; g++) memcpy(cache->psi_list[g].data, flat + (size_t)g * n, n * sizeof(numeric));
	free(flat);
	return r;
}

int mg_circuit_backward_host(const struct matchgate gates[], const int ngates, const int wires[], int L,
	const struct quantum_circuit_cache* cache, const numeric* dpsi_out, numeric* dpsi, struct matchgate dgates[])
{
	const size_t n = (size_t)1 << L;
	numeric* flat = malloc(n * (size_t)(ngates > 0 ? ngates : 1) * sizeof(numeric));
	if (!flat) return -1;
	for (int g = 0; g < ngates; g++) memcpy(flat + (size_t)g * n, cache->psi_list[g].data, n * sizeof(numeric));
	mgcu_lock();
	int r = mgcu_circuit_backward((const mgg*)gates, wires, ngates, L, (const mgc*)flat, (const mgc*)dpsi_out, (mgc*)dpsi, (mgg*)dgates);
	mgcu_unlock();
	free(flat);
	return r;
}

int apply_quantum_matchgate_circuit(const struct matchgate gates[], const int ngates, const int wires[],
	const struct statevector* restrict psi, struct statevector* restrict psi_out)
{
	assert(psi->nqubits == psi_out->nqubits);
	return mg_circuit_forward_host(gates, ngates, wires, psi->nqubits, psi->data, NULL, psi_out->data) ? -1 : 0;
}

int quantum_matchgate_circuit_forward(const struct matchgate gates[], const int ngates, const int wires[],
	const struct statevector* restrict psi, struct quantum_circuit_cache* cache, struct statevector* restrict psi_out)
{
	assert(cache->ngates == ngates && cache->nqubits == psi->nqubits);
	return mg_circuit_forward_host(gates, ngates, wires, psi->nqubits, psi->data, cache, psi_out->data) ? -1 : 0;
}

int quantum_matchgate_circuit_backward(const struct matchgate gates[], const int ngates, const int wires[], const struct quantum_circuit_cache* cache,
	const struct statevector* restrict dpsi_out, struct statevector* restrict dpsi, struct matchgate dgates[])
{
	assert(cache->ngates == ngates && cache->nqubits == dpsi->nqubits);
	return mg_circuit_backward_host(gates, ngates, wires, dpsi->nqubits, cache, dpsi_out->data, dpsi->data, dgates) ? -1 : 0;
}
