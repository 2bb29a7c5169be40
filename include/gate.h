/*
 * Single-gate operations on host state vectors (drop-in for the reference's
 * src/gate.h:7-22).  Each call copies its vectors to the GPU, runs one kernel and
 * copies the result back; they serve per-vector callers and tests, while the
 * batched evaluations of matchgate_target.h are the throughput path.
 */
#pragma once

#include "matchgate.h"
#include "statevector.h"

/* src/gate.c:581 */
void apply_matchgate(const struct matchgate* gate, const int i, const int j, const struct statevector* restrict psi, struct statevector* restrict psi_out);

/* src/gate.c:659 -- dpsi = gate^T dpsi_out and dgate = sum dpsi_out (x) psi */
void apply_matchgate_backward(const struct matchgate* gate, const int i, const int j, const struct statevector* restrict psi,
	const struct statevector* restrict dpsi_out, struct statevector* restrict dpsi, struct matchgate* dgate);

/* src/gate.c:779 */
void apply_matchgate_to_array(const struct matchgate* gate, const int i, const int j, const struct statevector_array* restrict psi, struct statevector_array* restrict psi_out);

/* src/gate.c:858 */
void apply_matchgate_backward_array(const struct matchgate* gate, const int i, const int j, const struct statevector_array* restrict psi,
	const struct statevector* restrict dpsi_out, struct matchgate* dgates);

/* src/gate.c:982 -- 8 states d(G psi)/dG_e, e = 0..3 center, 4..7 corner */
void apply_matchgate_placeholder(const int i, const int j, const struct statevector* psi, struct statevector_array* psi_out);

/* src/gate.c:1066 -- 16 states for a general 4x4 gate */
void apply_gate_placeholder(const int i, const int j, const struct statevector* psi, struct statevector_array* psi_out);
