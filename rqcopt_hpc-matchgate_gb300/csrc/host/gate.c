/*
 * Single-gate operations on host vectors (reference src/gate.c), each run as one
 * FP64 kernel on the GPU (copy in, kernel, copy out).
 */
#include <assert.h>
#include <stdio.h>

#include "gate.h"
#include "../mg_internal.h"

#define CG(p) ((const mgg*)(p))
#define V(p) ((mgc*)(p))
#define CV(p) ((const mgc*)(p))

static void report(int r, const char* what)
{
	if (r) fprintf(stderr, "%s failed on the GPU (code %d): %s\n", what, r, mg_last_error());
}

static void check_wires(int i, int j, int L)
{
	assert(0 <= i && i < L);
	assert(0 <= j && j < L);
	assert(i != j);
	(void)i; (void)j; (void)L;
}

void apply_matchgate(const struct matchgate* gate, const int i, const int j, const struct statevector* restrict psi, struct statevector* restrict psi_out)
{
	assert(psi->nqubits == psi_out->nqubits);
	check_wires(i, j, psi->nqubits);
	mgcu_lock();
	report(mgcu_prim_apply(CG(gate), i, j, psi->nqubits, 1, CV(psi->data), V(psi_out->data)), "apply_matchgate");
	mgcu_unlock();
}

void apply_matchgate_backward(const struct matchgate* gate, const int i, const int j, const struct statevector* restrict psi,
	const struct statevector* restrict dpsi_out, struct statevector* restrict dpsi, struct matchgate* dgate)
{
	assert(psi->nqubits == dpsi_out->nqubits && psi->nqubits == dpsi->nqubits);
	check_wires(i, j, psi->nqubits);
	mgcu_lock();
	report(mgcu_prim_backward(CG(gate), i, j, psi->nqubits, CV(psi->data), CV(dpsi_out->data), V(dpsi->data), (mgg*)dgate), "apply_matchgate_backward");
	mgcu_unlock();
}

void apply_matchgate_to_array(const struct matchgate* gate, const int i, const int j, const struct statevector_array* restrict psi, struct statevector_array* restrict psi_out)
{
	assert(psi->nqubits == psi_out->nqubits && psi->nstates == psi_out->nstates);
	check_wires(i, j, psi->nqubits);
	mgcu_lock();
	report(mgcu_prim_apply(CG(gate), i, j, psi->nqubits, psi->nstates, CV(psi->data), V(psi_out->data)), "apply_matchgate_to_array");
	mgcu_unlock();
}

void apply_matchgate_backward_array(const struct matchgate* gate, const int i, const int j, const struct statevector_array* restrict psi,
	const struct statevector* restrict dpsi_out, struct matchgate* dgates)
{
	assert(psi->nqubits == dpsi_out->nqubits);
	check_wires(i, j, psi->nqubits);
	mgcu_lock();
	report(mgcu_prim_backward_array(CG(gate), i, j, psi->nqubits, psi->nstates, CV(psi->data), CV(dpsi_out->data), (mgg*)dgates), "apply_matchgate_backward_array");
	mgcu_unlock();
}

void apply_matchgate_placeholder(const int i, const int j, const struct statevector* psi, struct statevector_array* psi_out)
{
	assert(psi->nqubits == psi_out->nqubits && psi_out->nstates == 8);
	check_wires(i, j, psi->nqubits);
	mgcu_lock();
	report(mgcu_prim_placeholder(i, j, psi->nqubits, 8, CV(psi->data), V(psi_out->data)), "apply_matchgate_placeholder");
	mgcu_unlock();
}

void apply_gate_placeholder(const int i, const int j, const struct statevector* psi, struct statevector_array* psi_out)
{
	assert(psi->nqubits == psi_out->nqubits && psi_out->nstates == 16);
	check_wires(i, j, psi->nqubits);
	mgcu_lock();
	report(mgcu_prim_placeholder(i, j, psi->nqubits, 16, CV(psi->data), V(psi_out->data)), "apply_gate_placeholder");
	mgcu_unlock();
}
