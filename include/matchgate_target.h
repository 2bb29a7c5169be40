/*
 * Target function f = -tr(U^dagger W), its gate gradients and Hessian, as a trace
 * over the 2^L basis columns (drop-in for the reference's src/matchgate_target.h:10-51).
 * The reference's column split over OpenMP threads and MPI ranks is replaced by
 * batching all columns on one GPU; the MPI entry points (src/matchgate_target.h:54-77)
 * are not provided.
 *
 * Return codes follow the reference (src/matchgate_target.c:24-53,257-284):
 * 0 success, -1 allocation, -2 the target map returned < 0, -3/-4 forward/backward
 * failure; this library adds -5 for a GPU error (message on stderr).
 *
 * The target map U is the caller's `linear_func`.  A map created by one of the
 * mg_target_* constructors of mg_gb300.h is applied on the GPU; any other function
 * is called on the host once per basis column and its columns are uploaded.
 */
#pragma once

#include "matchgate.h"
#include "quantum_circuit.h"
#include "statevector.h"

typedef int (*linear_func)(const struct statevector* restrict psi, void* fdata, struct statevector* restrict psi_out);

/* src/matchgate_target.c:20 */
int matchgate_circuit_unitary_target(linear_func ufunc, void* udata,
	const struct matchgate gates[], const int ngates, const int wires[], const int nqubits, numeric* fval);

/* src/matchgate_target.c:83 (same result as the serial form here) */
int parallel_matchgate_circuit_unitary_target(linear_func ufunc, void* udata,
	const struct matchgate gates[], const int ngates, const int wires[], const int nqubits, numeric* fval);

/* src/matchgate_target.c:212 -- per-gate holomorphic gradients dgates[ngates] */
int matchgate_circuit_unitary_target_and_gradient(linear_func ufunc, void* udata,
	const struct matchgate gates[], const int ngates, const int wires[], const int nqubits,
	numeric* fval, struct matchgate dgates[]);

/* src/matchgate_target.c:333 */
int matchgate_brickwall_unitary_target(linear_func ufunc, void* udata,
	const struct matchgate vlist[], const int nlayers, const int nqubits, const int* perms[],
	numeric* fval);

/* src/matchgate_target.c:359 -- gradients summed per layer */
int matchgate_brickwall_unitary_target_and_gradient(linear_func ufunc, void* udata,
	const struct matchgate vlist[], const int nlayers, const int nqubits, const int* perms[],
	numeric* fval, struct matchgate dvlist[]);

/* src/matchgate_target.c:397 -- hess is (8*nlayers)^2, hess[((i*8+x)*nlayers+j)*8+y] */
int matchgate_brickwall_unitary_target_gradient_hessian(linear_func ufunc, void* udata,
	const struct matchgate vlist[], const int nlayers, const int nqubits, const int* perms[],
	numeric* fval, struct matchgate dvlist[], numeric* hess);

/* src/matchgate_target.c:515 -- translation-invariant Hessian */
int matchgate_ti_brickwall_unitary_target_gradient_hessian(linear_func ufunc, void* udata,
	const struct matchgate vlist[], const int nlayers, const int nqubits, const int* perms[],
	numeric* fval, struct matchgate dvlist[], numeric* hess);

/* src/matchgate_target.c:877 -- Riemannian gradient vector and real Hessian matrix */
int matchgate_brickwall_unitary_target_gradient_vector_hessian_matrix(linear_func ufunc, void* udata,
	const struct matchgate vlist[], const int nlayers, const int nqubits, const int* perms[],
	numeric* fval, double* grad_vec, double* H);

/* src/matchgate_target.c:626 (same result as the serial form here) */
int parallel_matchgate_brickwall_unitary_target_gradient_hessian(linear_func ufunc, void* udata,
	const struct matchgate vlist[], const int nlayers, const int nqubits, const int* perms[],
	numeric* fval, struct matchgate dvlist[], numeric* hess);
