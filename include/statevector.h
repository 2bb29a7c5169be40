/*
 * Host state vectors (drop-in for the reference's src/statevector.h:10-42).
 * Layouts are part of the ABI: a statevector holds 2^nqubits amplitudes with qubit 0
 * as the most significant index bit; a statevector_array interleaves nstates vectors
 * as data[index * nstates + state].
 */
#pragma once

#include "config.h"

struct statevector
{
	numeric* data;  /* 2^nqubits entries */
	int nqubits;
};

int allocate_statevector(int nqubits, struct statevector* psi);

void free_statevector(struct statevector* psi);

void transpose_statevector(const struct statevector* restrict psi, const int* perm, struct statevector* restrict psi_trans);

void add_statevectors(const struct statevector* restrict psi1, const struct statevector* restrict psi2, struct statevector* restrict psi_sum);

struct statevector_array
{
	numeric* data;  /* 2^nqubits x nstates entries, interleaved */
	int nqubits;
	int nstates;
};

int allocate_statevector_array(int nqubits, int nstates, struct statevector_array* psi_list);

void free_statevector_array(struct statevector_array* psi_list);
