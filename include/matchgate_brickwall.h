/*
 * Brickwall circuits: layer l applies the one gate vlist[l] to the qubit pairs
 * (perms[l][2p], perms[l][2p+1]), p = 0 .. nqubits/2-1 (drop-in for the reference's
 * src/matchgate_brickwall.h:8-21).  These act on single host vectors.
 */
#pragma once

#include "matchgate.h"
#include "quantum_circuit.h"
#include "statevector.h"

/* src/matchgate_brickwall.c:14 */
int apply_matchgate_brickwall_unitary(const struct matchgate vlist[], const int nlayers, const int* perms[],
	const struct statevector* restrict psi, struct statevector* restrict psi_out);

/* src/matchgate_brickwall.c:52 -- cache must hold nlayers*nqubits/2 vectors */
int matchgate_brickwall_unitary_forward(const struct matchgate vlist[], int nlayers, const int* perms[],
	const struct statevector* restrict psi, struct quantum_circuit_cache* cache, struct statevector* restrict psi_out);

/* src/matchgate_brickwall.c:87 */
int matchgate_brickwall_unitary_backward(const struct matchgate vlist[], int nlayers, const int* perms[], const struct quantum_circuit_cache* cache,
	const struct statevector* restrict dpsi_out, struct statevector* restrict dpsi, struct matchgate dvlist[]);

/* src/matchgate_brickwall.c:137 -- hess is (8*nlayers)^2 */
int matchgate_brickwall_unitary_backward_hessian(const struct matchgate vlist[], int nlayers, const int* perms[], const struct quantum_circuit_cache* cache,
	const struct statevector* restrict dpsi_out, struct statevector* restrict dpsi, struct matchgate dvlist[], numeric* hess);

/* src/matchgate_brickwall.c:308 -- translation-invariant variant */
int matchgate_ti_brickwall_unitary_backward_hessian(const struct matchgate vlist[], int nlayers, const int* perms[], const struct quantum_circuit_cache* cache,
	const struct statevector* restrict dpsi_out, struct statevector* restrict dpsi, struct matchgate dvlist[], numeric* hess);
