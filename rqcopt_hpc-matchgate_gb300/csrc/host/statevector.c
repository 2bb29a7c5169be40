/*
 * Host state vectors (reference src/statevector.c).  Host memory management for the
 * ABI structs; all state-vector arithmetic of the library runs on the GPU.
 */
#include <assert.h>
#include <stdio.h>
#include <string.h>

#include "statevector.h"

static void* alloc_aligned(size_t bytes)
{
	/* aligned_alloc wants a multiple of the alignment */
	size_t size = (bytes + MEM_DATA_ALIGN - 1) / MEM_DATA_ALIGN * MEM_DATA_ALIGN;
	if (size == 0) size = MEM_DATA_ALIGN;
	return aligned_alloc(MEM_DATA_ALIGN, size);
}

int allocate_statevector(int nqubits, struct statevector* psi)
{
	const size_t bytes = ((size_t)1 << nqubits) * sizeof(numeric);
	psi->nqubits = nqubits;
	psi->data = alloc_aligned(bytes);
	if (psi->data == NULL)
	{
		fprintf(stderr, "allocating statevector memory (%zu bytes) failed\n", bytes);
		return -1;
	}
	return 0;
}

void free_statevector(struct statevector* psi)
{
	if (psi->data != NULL) { aligned_free(psi->data); psi->data = NULL; }
	psi->nqubits = 0;
}

/* psi_trans[j] = psi[k] where bit i of j selects wire perm[nqubits-1-i]
 * (reference src/statevector.c:49-72) */
void transpose_statevector(const struct statevector* restrict psi, const int* perm, struct statevector* restrict psi_trans)
{
	const int L = psi->nqubits;
	assert(L == psi_trans->nqubits);
	intqs strides[64];
	for (int i = 0; i < L; i++)
	{
		assert(0 <= perm[i] && perm[i] < L);
		strides[L - 1 - i] = (intqs)1 << (L - 1 - perm[i]);
	}
	const intqs n = (intqs)1 << L;
	for (intqs j = 0; j < n; j++)
	{
		intqs k = 0;
		for (int i = 0; i < L; i++) k += ((j >> i) & 1) * strides[i];
		psi_trans->data[j] = psi->data[k];
	}
}

void add_statevectors(const struct statevector* restrict psi1, const struct statevector* restrict psi2, struct statevector* restrict psi_sum)
{
	assert(psi1->nqubits == psi2->nqubits && psi1->nqubits == psi_sum->nqubits);
	const intqs n = (intqs)1 << psi1->nqubits;
	for (intqs j = 0; j < n; j++) psi_sum->data[j] = psi1->data[j] + psi2->data[j];
}

int allocate_statevector_array(int nqubits, int nstates, struct statevector_array* psi_array)
{
	const size_t bytes = ((size_t)1 << nqubits) * nstates * sizeof(numeric);
	psi_array->nqubits = nqubits;
	psi_array->nstates = nstates;
	psi_array->data = alloc_aligned(bytes);
	if (psi_array->data == NULL)
	{
		fprintf(stderr, "allocating statevector array memory (%zu bytes) failed\n", bytes);
		return -1;
	}
	return 0;
}

void free_statevector_array(struct statevector_array* psi_array)
{
	if (psi_array->data != NULL) { aligned_free(psi_array->data); psi_array->data = NULL; }
	psi_array->nqubits = 0;
	psi_array->nstates = 0;
}
